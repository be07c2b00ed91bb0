"""Writes libm_pow_tables.h: the tables and constants of libm_pow.h.

    python rhyme_gb300/csrc/libm_pow_tables.py        # rewrites libm_pow_tables.h
    python rhyme_gb300/csrc/libm_pow_tables.py OUT    # writes OUT instead

libm_pow.h restates the double-precision pow of the GNU C Library (glibc
2.28 and later, sysdeps/ieee754/dbl-64/e_pow.c; the algorithm is Szabolcs
Nagy's, from Arm's optimized-routines). Every value below is derived here
from its published definition, with mpmath at 240 bits:

log(x), x = 2^k z with z in [OFF, 2 OFF), OFF = 0x1.69555p-1. The range of z
is cut into 128 pieces of equal width in the bit pattern (piece i holds the
z whose bits minus OFF's have i in bits 45..51). For piece i, with centre c
(the double halfway through the piece's bit patterns):
    INVC   = round(128/c)/128 if c < 1, else round(256/c)/256,
             an exact double with few bits, so z*INVC - 1 is exact;
    LOGC   = -log(INVC) rounded to a multiple of 2^-43,
             so k*LN2_HI + LOGC is exact;
    LOGCTAIL = -log(INVC) - LOGC, rounded to double.
The two pieces around 1 get INVC = 1, LOGC = 0.
    LN2_HI = ln 2 rounded to 42 significant bits, LN2_LO = ln 2 - LN2_HI.
log1p(r) - r + r^2/2 = -r^3/2 (A1 + A2 r - r^2/2 (A3 + A4 r - r^2/2 (A5 + A6 r)))
    for |r| <= 0x1.6bp-8: the minimax fit of degree 8 in relative error
    (Remez exchange), each coefficient then rounded to double.

exp(x) = 2^(k/128) exp(r), x = k ln2/128 + r, |r| <= ln2/256:
    EXP_TAIL[j], EXP_SBITS[j] for j = 0..127: with s = 2^(j/128) rounded to
    double, EXP_SBITS[j] = bits(s) - j 2^45 (the exponent of 2^(k/128) is
    added by integer arithmetic) and EXP_TAIL[j] = 2^(j/128)/s - 1 rounded;
    INV_LN2_N = 128/ln 2; NEG_LN2_HI_N = -(ln 2/128 rounded to 36 significant
    bits), NEG_LN2_LO_N = -(ln 2/128 + NEG_LN2_HI_N), both rounded to double;
exp(r) - 1 - r = C2 r^2 + C3 r^3 + C4 r^4 + C5 r^5
    for |r| <= ln2/256: the minimax fit in absolute error, rounded to double.

Calibration. The two minimax fits above are this script's own; the C
library's coefficients came from another fitting procedure and differ from
them by thousands of ulps in the higher terms (which matters only for the
last bit of rare arguments). CALIBRATION moves each fitted coefficient by a
whole number of its ulps, to a point inside the set of coefficients for
which this restatement reproduces the library on every argument of the
calibration data. libm_pow_calibrate.py finds that set: for the log, it
recovers the library's low part log(x) - hi for 10^5 bases x (from the
results of pow(x, y) over many y) and solves a linear program for A3..A6;
for the exp, it keeps 10^6 arguments whose result lies within 5e-4 ulp of a
rounding boundary and solves one for C4..C5. The offsets are the centres of
those sets. With them the restatement is bit-identical to the library on
1.4e9 arguments (the solver's exponents, and random exponents up to 30 in
magnitude); tests/test_oracle_golden.py checks a smaller set on every run.
"""
import math
import os
import struct
import sys

import mpmath

mpmath.mp.prec = 240
N = 128
OFF_BITS = 0x3fe6955500000000
LOG_POLY_HALF_WIDTH = mpmath.mpf(0x16b) / 2 ** 16  # 0x1.6bp-8
# Whole ulps added to each fitted coefficient (see the module docstring).
CALIBRATION = {"A3": -11352, "A4": -79160, "A5": -318993240, "A6": -1985533046, "C4": -236500}


def _bits(d):
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def _dbl(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def _round_sig(v, nbits):
    """v rounded to nbits significant bits (an exact double for nbits <= 53)."""
    e = int(mpmath.floor(mpmath.log(abs(v), 2)))
    return float(mpmath.nint(v * mpmath.mpf(2) ** (nbits - 1 - e)) * mpmath.mpf(2) ** (e - nbits + 1))


def log_table():
    rows = []
    two43 = mpmath.mpf(2) ** 43
    for i in range(N):
        c = mpmath.mpf(_dbl(OFF_BITS + (i << 45) + (1 << 44)))
        invc = mpmath.nint(N / c) / N if c < 1 else mpmath.nint(2 * N / c) / (2 * N)
        lc = -mpmath.log(invc)
        logc = mpmath.nint(lc * two43) / two43
        rows.append((float(invc), float(logc), float(lc - logc)))
    return rows


def exp_table():
    rows = []
    for j in range(N):
        v = mpmath.mpf(2) ** (mpmath.mpf(j) / N)
        s = float(v)
        tail = float(v / mpmath.mpf(s) - 1)
        rows.append((_bits(tail), (_bits(s) - (j << 45)) & 0xFFFFFFFFFFFFFFFF))
    return rows


def remez(f, powers, weight, a, b, npts=3000, iters=40):
    """Minimax coefficients of sum c_k r^k (k in powers) for f on [a, b] with
    the error weighted by weight(r); Remez exchange on a grid, extrema refined
    by golden-section search."""
    n = len(powers)
    xs = [a + (b - a) * (mpmath.mpf(j) + mpmath.mpf("0.3")) / (n + mpmath.mpf("0.8")) for j in range(n + 1)]
    c = None
    for _ in range(iters):
        A = mpmath.matrix(n + 1, n + 1)
        rhs = mpmath.matrix(n + 1, 1)
        for j, x in enumerate(xs):
            for k, p in enumerate(powers):
                A[j, k] = x ** p
            A[j, n] = (-1) ** j / weight(x)
            rhs[j] = f(x)
        sol = mpmath.lu_solve(A, rhs)
        c = [sol[k] for k in range(n)]
        E = sol[n]

        def err(x):
            return weight(x) * (f(x) - sum(ck * x ** p for ck, p in zip(c, powers)))

        grid = [a + (b - a) * mpmath.mpf(j) / npts for j in range(npts + 1)]
        grid = [x for x in grid if x != 0]
        ev = [err(x) for x in grid]
        ext = []
        for j, v in enumerate(ev):
            if (j == 0 or abs(v) >= abs(ev[j - 1])) and (j + 1 == len(ev) or abs(v) >= abs(ev[j + 1])):
                ext.append((grid[j], v))
        alt = []
        for x, v in ext:
            if alt and mpmath.sign(alt[-1][1]) == mpmath.sign(v):
                if abs(v) > abs(alt[-1][1]):
                    alt[-1] = (x, v)
            else:
                alt.append((x, v))
        while len(alt) > n + 1:
            alt.pop(0 if abs(alt[0][1]) < abs(alt[-1][1]) else -1)
        h = (b - a) / npts
        new = []
        for x, v in alt:
            lo, hi = max(a, x - h), min(b, x + h)
            s = mpmath.sign(v)
            for _ in range(80):
                m1 = lo + (hi - lo) * mpmath.mpf("0.381966011250105")
                m2 = lo + (hi - lo) * mpmath.mpf("0.618033988749895")
                if s * err(m1) > s * err(m2):
                    hi = m2
                else:
                    lo = m1
            new.append((lo + hi) / 2)
        worst = max(abs(err(x)) for x in new)
        xs = new
        if abs(worst - abs(E)) <= abs(E) * mpmath.mpf("1e-15"):
            break
    return c


def log_poly():
    w = LOG_POLY_HALF_WIDTH
    c = remez(lambda r: mpmath.log1p(r) - r + r * r / 2, [3, 4, 5, 6, 7, 8],
              lambda r: 1 / abs(mpmath.log1p(r)), -w, w)
    # log1p(r) - r + r^2/2 = -r^3/2 (A1 + A2 r) + r^5/4 (A3 + A4 r) - r^7/8 (A5 + A6 r)
    scale = [-2, -2, 4, 4, -8, -8]
    return [float(s * v) for s, v in zip(scale, c)]


def exp_poly():
    a = mpmath.log(2) / (2 * N)
    c = remez(lambda r: mpmath.exp(r) - 1 - r, [2, 3, 4, 5], lambda r: 1, -a, a)
    return [float(v) for v in c]


def calibrated(name, v, calibration=None):
    """v moved by calibration[name] (default CALIBRATION) of its ulps (exact:
    stays in v's binade)."""
    k = (CALIBRATION if calibration is None else calibration).get(name, 0)
    if not k:
        return v
    out = v + k * math.ulp(v)
    assert math.ulp(out) == math.ulp(v)
    return out


def _hex(v):
    return float.hex(float(v))


def main(out=None, calibration=None):
    ln2 = mpmath.log(2)
    ln2_hi = _round_sig(ln2, 42)
    ln2_n = ln2 / N
    ln2_hi_n = _round_sig(ln2_n, 36)
    lines = [
        "// libm_pow_tables.h -- tables and constants of libm_pow.h, written by",
        "// libm_pow_tables.py (mpmath, 240 bits); do not edit by hand.",
        "#pragma once",
        "",
        "// log pieces: (INVC, LOGC, LOGCTAIL, 0) for i = 0..127.",
        "#define LIBM_POW_LOG_TABLE {",
    ]
    for invc, logc, tail in log_table():
        lines.append("    %s, %s, %s, 0.0," % (_hex(invc), _hex(logc), _hex(tail)))
    lines.append("}")
    lines.append("// exp pieces: (bits of EXP_TAIL, EXP_SBITS) for j = 0..127.")
    lines.append("#define LIBM_POW_EXP_TABLE {")
    for tail, sbits in exp_table():
        lines.append("    0x%016xULL, 0x%016xULL," % (tail, sbits))
    lines.append("}")
    lines.append("")
    a = log_poly()
    cc = exp_poly()
    consts = [
        ("LN2_HI", ln2_hi), ("LN2_LO", float(ln2 - mpmath.mpf(ln2_hi))),
        ("INV_LN2_N", float(N / ln2)), ("NEG_LN2_HI_N", -ln2_hi_n),
        ("NEG_LN2_LO_N", -float(ln2_n - mpmath.mpf(ln2_hi_n))),
    ]
    consts += [("A%d" % (k + 1), v) for k, v in enumerate(a)]
    consts += [("C%d" % (k + 2), v) for k, v in enumerate(cc)]
    consts = [(name, calibrated(name, v, calibration)) for name, v in consts]
    for name, v in consts:
        lines.append("constexpr double LIBM_POW_%s = %s;" % (name, _hex(v)))
    lines.append("")
    for k in range(len(lines)):
        if lines[k].startswith("#define LIBM_POW_") or lines[k].startswith("    "):
            lines[k] += " \\"
    if out is None:
        out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libm_pow_tables.h")
    with open(out, "w") as f:
        f.write("\n".join(lines))
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
