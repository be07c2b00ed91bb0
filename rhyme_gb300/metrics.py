"""Error metrics between two states of the same box.

Per conserved field f over the box interior:
    relative L1   = sum|f - f_ref| / sum|f_ref|
    relative Linf = max|f - f_ref| / max|f_ref|
"""
import numpy as np


def interior(cells, ndim):
    return cells[(slice(None),) + (slice(2, -2),) * ndim]


def field_errors(cells, ref_cells, ndim):
    """[(L1, Linf)] per conserved field (rho, momenta, total energy)."""
    a = interior(cells, ndim)
    b = interior(ref_cells, ndim)
    out = []
    for c in range(ndim + 2):
        d = np.abs(a[c] - b[c])
        s1 = np.abs(b[c]).sum()
        sm = np.abs(b[c]).max()
        l1 = d.sum() / s1 if s1 > 0 else d.sum()
        li = d.max() / sm if sm > 0 else d.max()
        out.append((float(l1), float(li)))
    return out
