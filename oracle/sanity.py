"""Test infrastructure (the checker, never the product): restatement of the
reference's sanity checks and conservation totals as plain loops.

rhyme_samr_calc_total_mass.f90 / _total_energy.f90: sum(cells(:, ..., rho),
mask = rho > 0) over the whole ghosted box (sequential sum here, exact sum
via math.fsum as well). rhyme_sanity_check_perform.f90:34-90: NaN per
field, minval/minloc of rho and e_tot. rhyme_sanity_check_fill.f90:75-185
with update_info (:155-182): per property, in Fortran loop order (i fastest),
count values below / above the range and keep the running extreme and the
one before it. Mach uses the cell's own state (|v| / cs).
"""
import math

import numpy as np

HUGE = np.finfo(np.float64).max


def totals(cells):
    """(sequential masked sums, exact masked sums) of rho and e_tot."""
    nd = cells.ndim - 1
    rho = cells[0].reshape(-1)
    et = cells[nd + 1].reshape(-1)
    seq = [0.0, 0.0]
    for x in rho:
        if x > 0.0:
            seq[0] += float(x)
    for x in et:
        if x > 0.0:
            seq[1] += float(x)
    exact = (math.fsum(float(x) for x in rho if x > 0.0), math.fsum(float(x) for x in et if x > 0.0))
    return tuple(seq), exact


def _values(u, nd, gamma, kb_amu):
    rho = u[0]
    v = {"rho": rho, "vx": u[1] / rho, "e_tot": u[nd + 1]}
    if nd > 1:
        v["vy"] = u[2] / rho
    if nd > 2:
        v["vz"] = u[3] / rho
    ss = 0.0
    for a in range(nd):
        ss = ss + u[1 + a] * u[1 + a]
    absv = math.sqrt(ss) / rho
    v["abs_v"] = absv
    # cs as rhyme_ideal_gas_speed_of_sound.f90:9 with _temperature_per_mu.f90:9-10
    sk = (0.5 * ss) / (rho * rho)
    t_mu = (u[nd + 1] / rho - sk) * (gamma - 1.0) / kb_amu
    x = (gamma * kb_amu) * t_mu
    v["mach"] = absv / math.sqrt(x) if x >= 0 else float("nan")
    return v


def sanity(cells, ranges, gamma=5.0 / 3.0, kb_amu=1.0):
    """Loop-order restatement; returns (properties, general) like
    rhyme_gb300.gpu.Context.sanity_check."""
    nd = cells.ndim - 1
    inner = cells[(slice(None),) + (slice(2, -2),) * nd]
    dims = inner.shape[1:][::-1]
    info = {k: dict(nbelow=0, nabove=0, vbelow=HUGE, vbelow_prev=HUGE, vabove=-HUGE, vabove_prev=-HUGE,
                    cbelow=(0, 0, 0), cabove=(0, 0, 0)) for k in ranges}
    nan = [False] * (nd + 2)
    rho_min = e_min = math.inf
    rho_at = e_at = (0, 0, 0)
    nk = dims[2] if nd > 2 else 1
    nj = dims[1] if nd > 1 else 1
    for k in range(nk):
        for j in range(nj):
            for i in range(dims[0]):
                idx = tuple(x for x, keep in ((k, nd > 2), (j, nd > 1)) if keep) + (i,)
                u = [float(inner[(c,) + idx]) for c in range(nd + 2)]
                pos = (i + 1, j + 1 if nd > 1 else 0, k + 1 if nd > 2 else 0)
                for c in range(nd + 2):
                    if math.isnan(u[c]):
                        nan[c] = True
                if u[0] < rho_min:
                    rho_min, rho_at = u[0], pos
                if u[nd + 1] < e_min:
                    e_min, e_at = u[nd + 1], pos
                vals = _values(u, nd, gamma, kb_amu)
                for name, (lo, hi) in ranges.items():
                    val = vals[name]
                    s = info[name]
                    if val < lo:
                        s["nbelow"] += 1
                        if val < s["vbelow"]:
                            s["vbelow_prev"], s["vbelow"], s["cbelow"] = s["vbelow"], val, pos
                    if val > hi:
                        s["nabove"] += 1
                        if val > s["vabove"]:
                            s["vabove_prev"], s["vabove"], s["cabove"] = s["vabove"], val, pos
    general = dict(nan=nan, rho_min=rho_min, e_tot_min=e_min, rho_min_at=rho_at, e_tot_min_at=e_at)
    return info, general
