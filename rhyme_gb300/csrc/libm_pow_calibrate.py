"""Finds the CALIBRATION offsets of libm_pow_tables.py: the polynomial
coefficients at which the restatement in libm_pow.h returns this machine's C
library pow bit for bit.

    python rhyme_gb300/csrc/libm_pow_calibrate.py [--from-fit] [--bases N] [--exps M]

Needs g++ (with libquadmath), numpy and scipy; takes a few minutes on 8
cores. --from-fit starts from the plain fits (offsets zero) instead of the
committed offsets. Prints the offsets to put into CALIBRATION.

Log polynomial (A3..A6; A1 and A2 are exact from the fit): for each base x of
a sample, libm_pow_calibrate.cpp finds by how many ulps the library's low
part of log x differs from the restatement's (from pow(x, y) over exponents
that make |y log x| 300..500). The library's low part lo* = RN(ar3 q* + s),
with ar3 = -r^3/2 and s the exactly reproduced head terms, so it bounds the
library's q*, a double; q* = RN(p12 + ar2 I) with p12 = RN(A1 + r A2) and
I = A3 + r A4 + ar2 (A5 + r A6) up to roundings far below ulp(q) / |ar2|,
so every base gives an interval for the linear form I(r) in (A3..A6). The
offsets are the point of the polytope of those intervals whose smallest
distance to the bounds of I(r), over all bases, is largest (a linear
program).

Exp polynomial (C4, C5; C2 and C3 are exact from the fit): for arguments
whose result lies within a small fraction of an ulp of a rounding boundary,
the library's result bounds tmp = RN(r^4 (C4 + r C5) + u), with every other
term reproduced exactly, hence C4 + r C5; solved the same way (the point
farthest from the bounds of C4 + r C5).
"""
import argparse
import math
import os
import struct
import subprocess
import sys
import tempfile
from fractions import Fraction as Fr

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import libm_pow_tables as T  # noqa: E402


def _bits(d):
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def _dbl(b):
    return struct.unpack("<d", struct.pack("<Q", b & 0xFFFFFFFFFFFFFFFF))[0]


def _fma(a, b, c):
    return float(Fr(a) * Fr(b) + Fr(c))


def coefficients(calibration):
    a = [T.calibrated("A%d" % (k + 1), v, calibration) for k, v in enumerate(T.log_poly())]
    c = [T.calibrated("C%d" % (k + 2), v, calibration) for k, v in enumerate(T.exp_poly())]
    return a, c


def build_probe(calibration, tmp):
    hdr = os.path.join(tmp, "candidate_tables.h")
    T.main(hdr, calibration)
    exe = os.path.join(tmp, "probe")
    cmd = ["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-std=c++17", '-DLIBM_POW_TABLES_FILE="%s"' % hdr,
           "-I", HERE, os.path.join(HERE, "libm_pow_calibrate.cpp"), "-lquadmath", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def _lp_centre(G, lo, hi):
    """The point of {d : lo <= G d <= hi} farthest from every bound, in the
    units of the bounds (maximise t with lo + t <= G d <= hi - t), and the
    range of each variable over the set (linear programs)."""
    from scipy.optimize import linprog
    n = G.shape[1]
    A = np.vstack([G, -G])
    b = np.concatenate([hi, -lo])
    lo_, hi_ = [], []
    for j in range(n):
        for sgn in (1.0, -1.0):
            c = np.zeros(n)
            c[j] = sgn
            r = linprog(c, A_ub=A, b_ub=b, bounds=[(None, None)] * n, method="highs")
            if r.status != 0:
                raise RuntimeError("calibration data are inconsistent: %s" % r.message)
            (lo_ if sgn > 0 else hi_).append(r.x[j])
    ones = np.ones((A.shape[0], 1))
    c = np.zeros(n + 1)
    c[n] = -1.0
    r = linprog(c, A_ub=np.hstack([A, ones]), b_ub=b, bounds=[(None, None)] * n + [(0, None)], method="highs")
    if r.status != 0:
        raise RuntimeError("no centre: %s" % r.message)
    return r.x[:n], np.array(lo_), np.array(hi_)


def log_rows(x, k, A, table):
    """The interval of I(r) = A3 + r A4 + ar2 (A5 + r A6) for base x whose
    library low part is the restatement's moved by k ulps (None if empty)."""
    ln2 = T.mpmath.log(2)
    ln2_hi = T._round_sig(ln2, 42)
    ln2_lo = float(ln2 - T.mpmath.mpf(ln2_hi))
    ix = _bits(x)
    t = (ix - T.OFF_BITS) & 0xFFFFFFFFFFFFFFFF
    i = (t >> 45) & 127
    kk = t >> 52
    if kk >= 2048:
        kk -= 4096
    z = _dbl(ix - (t & (0xFFF << 52)))
    invc, logc, logctail = table[i]
    kd = float(kk)
    r = _fma(z, invc, -1.0)
    t1 = _fma(kd, ln2_hi, logc)
    t2 = t1 + r
    lo1 = _fma(kd, ln2_lo, logctail)
    lo2 = t1 - t2 + r
    ar = -0.5 * r
    ar2 = r * ar
    ar3 = r * ar2
    hi = t2 + ar2
    lo3 = _fma(ar, r, -ar2)
    lo4 = t2 - hi + ar2
    s = ((lo1 + lo2) + lo3) + lo4
    if ar3 == 0.0:
        return None
    q = _fma(ar2, _fma(ar2, _fma(r, A[5], A[4]), _fma(r, A[3], A[2])), _fma(r, A[1], A[0]))
    lo = _fma(ar3, q, s)
    lot = _dbl(_bits(lo) + k * (1 if lo > 0 else -1))
    up = Fr(math.nextafter(lot, math.inf) - lot)
    dn = Fr(lot - math.nextafter(lot, -math.inf))
    qa, qb = (Fr(lot) - dn / 2 - Fr(s)) / Fr(ar3), (Fr(lot) + up / 2 - Fr(s)) / Fr(ar3)
    if qa > qb:
        qa, qb = qb, qa
    qmin = float(qa)
    if Fr(qmin) < qa:
        qmin = math.nextafter(qmin, math.inf)
    qmax = float(qb)
    if Fr(qmax) > qb:
        qmax = math.nextafter(qmax, -math.inf)
    if qmin > qmax:
        return None
    pa = Fr(qmin) - Fr(qmin - math.nextafter(qmin, -math.inf)) / 2
    pb = Fr(qmax) + Fr(math.nextafter(qmax, math.inf) - qmax) / 2
    p12 = _fma(r, A[1], A[0])
    ia, ib = (pa - Fr(p12)) / Fr(ar2), (pb - Fr(p12)) / Fr(ar2)
    if ia > ib:
        ia, ib = ib, ia
    base = Fr(A[2]) + Fr(r) * Fr(A[3]) + Fr(ar2) * Fr(A[4]) + Fr(r) * Fr(ar2) * Fr(A[5])
    return r, ar2, float(ia - base), float(ib - base)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--from-fit", action="store_true")
    ap.add_argument("--bases", type=int, default=60000)
    ap.add_argument("--exps", type=int, default=30000)
    ap.add_argument("--exp-args", type=int, default=1200000000)
    args = ap.parse_args()
    cal = {} if args.from_fit else dict(T.CALIBRATION)
    table = T.log_table()
    with tempfile.TemporaryDirectory() as tmp:
        # log polynomial
        exe = build_probe(cal, tmp)
        out = subprocess.run([exe, "log", str(args.bases), str(args.exps), "1"], check=True,
                             capture_output=True, text=True).stdout
        A, _ = coefficients(cal)
        rows = [log_rows(float.fromhex(l.split()[0]), int(l.split()[1]), A, table) for l in out.splitlines()]
        rows = [x for x in rows if x is not None]
        r = np.array([x[0] for x in rows])
        ar2 = np.array([x[1] for x in rows])
        slack = 2.5e-16  # inner roundings of I(r)
        lo = np.array([x[2] for x in rows]) - slack
        hi = np.array([x[3] for x in rows]) + slack
        u = [math.ulp(a) for a in A]
        G = np.stack([np.full_like(r, u[2]), r * u[3], ar2 * u[4], r * ar2 * u[5]], 1) / u[2]
        d, dmin, dmax = _lp_centre(G, lo / u[2], hi / u[2])
        for j, name in enumerate(("A3", "A4", "A5", "A6")):
            cal[name] = cal.get(name, 0) + int(round(d[j]))
            print("%s: %d bases; offset range [%.0f, %.0f] ulps, centre %+d" % (
                name, len(rows), dmin[j], dmax[j], int(round(d[j]))), file=sys.stderr)
        # exp polynomial, with the log set
        exe = build_probe(cal, tmp)
        out = subprocess.run([exe, "exp", str(args.exp_args), "0.0005", "2"], check=True,
                             capture_output=True, text=True).stdout
        data = np.array([[float.fromhex(v) for v in l.split()] for l in out.splitlines()])
        _, C = coefficients(cal)
        r, lo, hi = data[:, 0], data[:, 1], data[:, 2]
        keep = np.isfinite(lo) & np.isfinite(hi) & ((np.abs(lo) < 3e-9) | (np.abs(hi) < 3e-9))
        u4, u5 = math.ulp(C[2]), math.ulp(C[3])
        G = np.stack([np.full(keep.sum(), 1.0), r[keep] * u5 / u4], 1)
        d, dmin, dmax = _lp_centre(G, lo[keep] / u4, hi[keep] / u4)
        for j, name in enumerate(("C4", "C5")):
            cal[name] = cal.get(name, 0) + int(round(d[j]))
            print("%s: %d arguments; offset range [%.0f, %.0f] ulps, centre %+d" % (
                name, int(keep.sum()), dmin[j], dmax[j], int(round(d[j]))), file=sys.stderr)
    print("CALIBRATION = %r" % {k: v for k, v in sorted(cal.items()) if v})


if __name__ == "__main__":
    main()
