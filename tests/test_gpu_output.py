"""Level output drain on the GPU (rhyme_gpu_output_level) against the
oracle's restatement of the reference's packing loop: bit for bit (the same
doubles converted to FP32 with round to nearest), components beyond the
hydro ones left untouched."""
import numpy as np
import pytest

from oracle import chombo_pack
from rhyme_gb300 import gpu, ic
from rhyme_gb300.params import OUTFLOW, PERIODIC, REFLECTIVE, hydro_params

pytestmark = pytest.mark.gpu


def _boxes(nd, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        dims = [int(x) for x in rng.integers(3, {1: 300, 2: 40, 3: 20}[nd], nd)]
        c = ic.empty_box(nd, dims)
        shp = tuple(dims[::-1])
        c[ic.interior(nd, dims)] = ic.prim_to_cons(1 + rng.uniform(size=shp),
                                                   [0.2 * rng.uniform(-1, 1, shp) for _ in range(nd)],
                                                   1 + rng.uniform(size=shp), 5.0 / 3.0)
        out.append(c)
    return out


@pytest.mark.parametrize("nd", [1, 2, 3])
@pytest.mark.parametrize("precision", [0, 1])
def test_output_level_matches_oracle(nd, precision):
    boxes = _boxes(nd, 5, seed=nd)
    p = hydro_params(nd, bc=[PERIODIC, OUTFLOW, REFLECTIVE, OUTFLOW, PERIODIC, PERIODIC],
                     courant={1: 0.8, 2: 0.5, 3: 0.3}[nd], precision=precision)
    with gpu.Context(p) as ctx:
        hs = [ctx.register_box(c) for c in boxes]
        for h, c in zip(hs, boxes):
            ctx.run(h, [1.0 / max(c.shape[1:])] * nd, 3)
        out = ctx.output_level(hs)
        ctx.output_wait()
        for h in hs:
            ctx.sync_to_host(h)
    assert np.array_equal(out, chombo_pack.pack_level(boxes))


def test_output_level_leaves_other_components():
    nd, ncmp = 3, 7
    boxes = _boxes(nd, 4, seed=11)
    with gpu.Context(hydro_params(nd, courant=0.3)) as ctx:
        hs = [ctx.register_box(c) for c in boxes]
        with ctx.batch(hs, [[1 / 16.0] * 3] * len(hs)) as bt:
            bt.run(2)
        n = sum(int(np.prod(h.dims)) for h in hs) * ncmp
        out = np.full(n, -7.0, dtype=np.float32)
        ctx.output_level(hs, ncmp=ncmp, out=out)
        ctx.output_wait()
        first = out.copy()
        ctx.output_level(hs, ncmp=ncmp, out=out)  # a second output reuses the staging buffers
        ctx.output_wait()
        for h in hs:
            ctx.sync_to_host(h)
    full = [np.concatenate([c, np.zeros((ncmp - 5,) + c.shape[1:])]) for c in boxes]
    ref = chombo_pack.pack_level(full, ncmp)
    off = 0
    for c in boxes:
        cells = int(np.prod([s - 4 for s in c.shape[1:]]))
        hyd = slice(off, off + 5 * cells)
        rest = slice(off + 5 * cells, off + ncmp * cells)
        assert np.array_equal(out[hyd], ref[hyd])
        assert (out[rest] == -7.0).all()
        off += ncmp * cells
    assert np.array_equal(first, out)


def test_output_level_errors():
    boxes = _boxes(2, 2, seed=3)
    with gpu.Context(hydro_params(2)) as ctx:
        hs = [ctx.register_box(c) for c in boxes]
        n = sum(int(np.prod(h.dims)) for h in hs) * 4
        with pytest.raises(gpu.RhymeGpuError) as e:
            ctx.output_level(hs, out=np.zeros(n - 1, dtype=np.float32))
        assert e.value.code == gpu.EINVAL
        with pytest.raises(gpu.RhymeGpuError) as e:
            ctx.output_level(hs, ncmp=3)
        assert e.value.code == gpu.EINVAL
        ctx.output_wait()  # nothing pending: returns at once
