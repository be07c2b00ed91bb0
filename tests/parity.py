"""Parity metrics between a GPU result and the CPU oracle.

Per conserved field f over the box interior:
    relative L1   = sum|f_gpu - f_ref| / sum|f_ref|
    relative Linf = max|f_gpu - f_ref| / max|f_ref|
The plain FP64 bar is 1e-12 for both, and 1e-14 relative for each dt.
"""
import numpy as np

from rhyme_gb300.metrics import field_errors, interior  # noqa: F401

FP64_FIELD_TOL = 1e-12
FP64_DT_TOL = 1e-14


def assert_fp64_parity(gpu_cells, ref_cells, ndim, dts_gpu=None, dts_ref=None,
                       tol=FP64_FIELD_TOL, dt_tol=FP64_DT_TOL):
    errs = field_errors(gpu_cells, ref_cells, ndim)
    for c, (l1, li) in enumerate(errs):
        assert l1 <= tol and li <= tol, "field %d: L1 %.3e Linf %.3e" % (c, l1, li)
    if dts_gpu is not None:
        rel = np.abs(np.asarray(dts_gpu) - np.asarray(dts_ref)) / np.abs(dts_ref)
        assert rel.max() <= dt_tol, "dt rel diff %.3e at step %d" % (rel.max(), int(rel.argmax()))
    return errs
