"""Test infrastructure (the checker, never the product): numpy restatement
of the level-data packing of the reference's Chombo writer.

rhyme_chombo_write_level_data.f90:36-70: for each box b of the level in
order, for each component var = 1..NCMP, the interior cells
cells(1:dims(1), 1:dims(2), 1:dims(3), var) reshaped in Fortran (column-major)
order and converted with real() (FP64 -> default real, round to nearest) are
stored at chws%data(offset + (var-1)*prod(dims) : ...), offset advancing by
NCMP*prod(dims) per box; the boxes table holds left_edge-1 and right_edge-1
padded to 3 entries with 0 (:53-54).
"""
import numpy as np


def pack_level(boxes_cells, ncmp=None):
    """boxes_cells: list of arrays in the reference layout (NCMP, [N3+4,]
    [N2+4,] N1+4) (numpy C order = Fortran order of cells(i, j, k, var)
    reversed). Returns the float32 dataset."""
    out = []
    for cells in boxes_cells:
        nd = cells.ndim - 1
        k = cells.shape[0] if ncmp is None else ncmp
        inner = cells[(slice(0, k),) + (slice(2, -2),) * nd]
        for var in range(k):
            # numpy C order over (k, j, i) is the Fortran order over (i, j, k)
            out.append(inner[var].reshape(-1).astype(np.float32))
    return np.concatenate(out) if out else np.zeros(0, np.float32)


def boxes_table(left_edges, right_edges):
    """(n, 6) int32 rows: left_edge - 1, right_edge - 1, padded with 0."""
    rows = []
    for le, re in zip(left_edges, right_edges):
        lo = [int(x) - 1 for x in le] + [0] * (3 - len(le))
        hi = [int(x) - 1 for x in re] + [0] * (3 - len(re))
        rows.append(lo + hi)
    return np.asarray(rows, dtype=np.int32).reshape(-1, 6)
