"""Chombo-layout level output on the CPU: the oracle's restatement of the
reference's packing loop against a literal cell loop, and the container
round trip."""
import numpy as np

from oracle import chombo_pack
from rhyme_gb300 import chombo, ic


def _literal_pack(boxes, ncmp):
    """rhyme_chombo_write_level_data.f90:51-70 written as explicit loops."""
    out = []
    for cells in boxes:
        nd = cells.ndim - 1
        dims = [s - 4 for s in cells.shape[1:]][::-1]  # (N1, N2, N3)
        dims += [1] * (3 - nd)
        for var in range(ncmp):
            for k in range(dims[2]):
                for j in range(dims[1]):
                    for i in range(dims[0]):
                        idx = (var,) + ((k + 2,) if nd > 2 else ()) + ((j + 2,) if nd > 1 else ()) + (i + 2,)
                        out.append(np.float32(cells[idx]))
    return np.asarray(out, dtype=np.float32)


def test_pack_matches_literal_loops():
    rng = np.random.default_rng(0)
    for nd, dims_list in ((1, [[9], [4]]), (2, [[5, 3], [2, 6]]), (3, [[3, 4, 2], [2, 2, 5]])):
        boxes = []
        for dims in dims_list:
            c = np.zeros((7,) + tuple(d + 4 for d in dims[::-1]))
            c[:] = rng.normal(size=c.shape) * 10.0 ** rng.integers(-3, 4)
            boxes.append(c)
        got = chombo_pack.pack_level(boxes)
        assert np.array_equal(got, _literal_pack(boxes, 7))
        assert got.size == chombo.level_length([d for d in dims_list], 7)


def test_boxes_table_pads_and_shifts():
    t = chombo_pack.boxes_table([[1, 1], [17, 1]], [[16, 32], [32, 32]])
    assert t.tolist() == [[0, 0, 0, 15, 31, 0], [16, 0, 0, 31, 31, 0]]


def test_container_round_trip(tmp_path):
    cells, dx, p = ic.riemann_1d(n=64, seed=3)
    data = chombo_pack.pack_level([cells])
    attrs = chombo.header_attrs(1, [64], ["rho", "rho_u", "e_tot"], 100, 0.25)
    lv = {"dx": [dx[0], 0, 0], "ref_ratio": 2, "prob_domain": [0, 0, 0, 63, 0, 0],
          "boxes": chombo_pack.boxes_table([[1]], [[64]]), "data": data}
    path = tmp_path / "snap.rhyme"
    chombo.write(str(path), [lv], attrs)
    a2, levels = chombo.read(str(path))
    assert a2 == attrs
    assert np.array_equal(levels[0]["data"], data)
    assert levels[0]["boxes"].tolist() == [[0, 0, 0, 63, 0, 0]]
