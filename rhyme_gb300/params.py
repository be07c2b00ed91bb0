"""Hot-path parameters with the reference's ids and defaults.

Ids and defaults follow the Fortran modules the C-ABI replaces:
  slope limiter ids   rhyme_slope_limiter.f90:6-15   (slid, slope_limiter_t)
  boundary ids        rhyme_samr_bc.f90:9-28          (bcid, samr_bc_t)
  solver ids          rhyme_muscl_hancock.f90:10-19   (mhid, muscl_hancock_t)
  Riemann defaults    rhyme_riemann_problem.f90:24-31 (riemann_problem_t)
  courant default     rhyme_cfl.f90:7-9               (cfl_t)
  gamma table         rhyme_thermo_base.f90:21-22     (ig_gamma)
"""
import numpy as np

# slid
VAN_LEER, MINMOD, VAN_ALBADA, SUPERBEE = 1, 2, 3, 4
LIMITERS = {"van_leer": VAN_LEER, "minmod": MINMOD, "van_albada": VAN_ALBADA,
            "superbee": SUPERBEE}
# bcid
REFLECTIVE, OUTFLOW, PERIODIC, INFLOW = 1, 2, 3, 4
# a face whose ghost rows the caller fills (a slab of a decomposed box)
HALO = 5
BCS = {"reflective": REFLECTIVE, "outflow": OUTFLOW, "periodic": PERIODIC,
       "inflow": INFLOW}
# mhid
CPU_INTENSIVE, MEMORY_INTENSIVE = 1, 2
# precision modes of this library
FP64, MIXED = 0, 1

GAMMA = {"monatomic": 5.0 / 3.0, "diatomic": 7.0 / 5.0, "polyatomic": 4.0 / 3.0}

# kB / amu with the reference's single-precision SI literals
# (rhyme_units.f90:25,29): only its bits enter, since it cancels in cs.
KB_AMU_SI = float(np.float64(np.float32(1.38064852e-23)) /
                  np.float64(np.float32(1.6605e-27)))


def hydro_params(ndim, limiter=MINMOD, bc=(OUTFLOW,) * 6, gamma=GAMMA["monatomic"],
                 courant=0.8, omega=0.0, vac_rho=0.0, vac_p=0.0, tol=1e-6,
                 n_iter=100, solver_type=MEMORY_INTENSIVE, kb_amu=KB_AMU_SI,
                 precision=FP64, inflow=None, sweep_tuning=0):
    """The values Rhyme's modules hold for one run, as one mapping."""
    bc = list(bc) + [OUTFLOW] * (6 - len(bc))
    return dict(ndim=int(ndim), gamma=float(gamma), kb_amu=float(kb_amu),
                courant=float(courant), limiter=int(limiter), omega=float(omega),
                vac_rho=float(vac_rho), vac_p=float(vac_p), tol=float(tol),
                n_iter=int(n_iter), bc=[int(b) for b in bc[:6]],
                solver_type=int(solver_type), precision=int(precision),
                inflow=inflow, sweep_tuning=int(sweep_tuning))
