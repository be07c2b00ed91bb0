"""Writes detmath_tables.h: the constants of the table-driven det_pow
(detmath.h), computed with mpmath at 200 bits.

    python rhyme_gb300/csrc/detmath_tables.py   # rewrites detmath_tables.h
    python rhyme_gb300/csrc/detmath_tables.py OUT  # writes OUT instead

log: for m in [1, 2) the interval i = floor((m - 1) 128) has centre
c_i = 1 + (i + 1/2)/128; INVC[i] = RN(1/c_i) and LOGC[i] = -log(INVC[i]) as a
double-double (the exact logarithm of the double INVC[i], so that
log m = LOGC[i] + log1p(m INVC[i] - 1) holds to the table's precision).
exp: EXP2[j] = 2^(j/64), j = 0..63, as double-doubles.
LN2_64 = ln 2 / 64 split into a head with 36 significant bits (n LN2_64_HI
exact for |n| < 2^17) and a tail.
"""
import os

import mpmath

mpmath.mp.prec = 200


def dd(v):
    hi = float(v)
    lo = float(v - mpmath.mpf(hi))
    return hi, lo


def fmt(x):
    return repr(float(x)) if x != 0 else "0.0"


def main(out=None):
    lines = ["// detmath_tables.h -- constants of det_pow (detmath.h), written by",
             "// detmath_tables.py (mpmath, 200 bits); do not edit by hand.",
             "#pragma once", "",
             "// log: INVC[i] = RN(1/c_i), c_i = 1 + (i + 1/2)/128; LOGC[i] = -log(INVC[i])",
             "// as (hi, lo).", "#define DETMATH_INVC_TABLE {"]
    inv, logc = [], []
    for i in range(128):
        c = 1 + (mpmath.mpf(i) + mpmath.mpf(0.5)) / 128
        ic = float(1 / c)
        inv.append(ic)
        logc.append(dd(-mpmath.log(mpmath.mpf(ic))))
    for k in range(0, 128, 4):
        lines.append("    " + ", ".join(fmt(v) for v in inv[k:k + 4]) + ",")
    lines.append("}")
    lines.append("#define DETMATH_LOGC_TABLE {")
    for k in range(0, 128, 2):
        lines.append("    " + ", ".join("%s, %s" % (fmt(h), fmt(l)) for h, l in logc[k:k + 2]) + ",")
    lines.append("}")
    lines.append("")
    lines.append("// exp: EXP2[j] = 2^(j/64) as (hi, lo).")
    lines.append("#define DETMATH_EXP2_TABLE {")
    e2 = [dd(mpmath.power(2, mpmath.mpf(j) / 64)) for j in range(64)]
    for k in range(0, 64, 2):
        lines.append("    " + ", ".join("%s, %s" % (fmt(h), fmt(l)) for h, l in e2[k:k + 2]) + ",")
    lines.append("}")
    ln2_64 = mpmath.log(2) / 64
    # head with 36 significant bits: round ln2/64 * 2^(36 - e) to an integer
    e = int(mpmath.floor(mpmath.log(ln2_64, 2))) + 1
    hi = float(mpmath.nint(ln2_64 * mpmath.power(2, 36 - e)) * mpmath.power(2, e - 36))
    lo = float(ln2_64 - mpmath.mpf(hi))
    lines.append("")
    lines.append("constexpr double DETMATH_LN2_64_HI = %s;" % fmt(hi))
    lines.append("constexpr double DETMATH_LN2_64_LO = %s;" % fmt(lo))
    lines.append("constexpr double DETMATH_INV_LN2_64 = %s;" % fmt(64 / mpmath.log(2)))
    lines.append("")
    # continue the table macros over their lines
    for k in range(len(lines)):
        if lines[k].startswith("#define DETMATH_") or (lines[k].startswith("    ") and k + 1 < len(lines)):
            lines[k] += " \\"
    if out is None:
        out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "detmath_tables.h")
    with open(out, "w") as f:
        f.write("\n".join(lines))
    print("wrote", out)


if __name__ == "__main__":
    import sys
    main(sys.argv[1] if len(sys.argv) > 1 else None)
