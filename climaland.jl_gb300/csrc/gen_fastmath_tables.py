"""Generate clm_fastmath_tables.h: the tables of the table-driven FP64 exp
and log in clm_fastmath.cuh (P. T. P. Tang, "Table-driven implementation of
the exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
1989; "Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990).

Values are computed with the decimal module at 60 digits and rounded to
double, so the header is the same on every machine.

  exp:  EXP2J[j]  = 2^(j/64), j = 0..63
  log:  for m in [1 + j/64, 1 + (j+1)/64), j = 0..63, a centre c_j whose
        reciprocal INVC[j] has at most 21 significant bits; c_0 = 1 and
        c_63 = 2 (so x near 1 from either side has no table term).
        For j >= 32 the table stores log(c_j / 2) and the caller adds one to
        the exponent, which keeps results near 1 free of cancellation.
        LOGC_HI[j] + LOGC_LO[j] = log(c_j) or log(c_j / 2).
"""
from decimal import Decimal, getcontext
from pathlib import Path
import struct

getcontext().prec = 60

N = 64


def dbl(x: Decimal) -> float:
    return float(x)  # correctly rounded conversion (decimal -> binary64)


def exp_dec(x: Decimal) -> Decimal:
    return x.exp()


def ln_dec(x: Decimal) -> Decimal:
    return x.ln()


def round_bits(x: float, bits: int) -> float:
    """Round x to `bits` significant bits."""
    m, e = __import__("math").frexp(x)
    scale = 2 ** bits
    return __import__("math").ldexp(round(m * scale) / scale, e)


def hexd(x: float) -> str:
    return float.hex(x)


def main():
    ln2 = Decimal(2).ln()
    exp2j = [dbl(exp_dec(ln2 * Decimal(j) / Decimal(N))) for j in range(N)]
    invc, lhi, llo = [], [], []
    for j in range(N):
        if j == 0:
            c = 1.0
            ic = 1.0
        elif j == N - 1:
            c = 2.0
            ic = 0.5
        else:
            centre = 1.0 + (j + 0.5) / N
            ic = round_bits(1.0 / centre, 21)
            c = None
        cd = Decimal(1) / Decimal(ic)  # the exact centre the table encodes
        if j >= N // 2:
            cd = cd / 2
        lv = ln_dec(cd)
        hi = dbl(lv)
        lo = dbl(lv - Decimal(hi))
        invc.append(ic)
        lhi.append(hi)
        llo.append(lo)
    # ln2 split: hi with 32 significant bits so e * LN2_HI is exact for |e| < 2^20
    l2hi = round_bits(dbl(ln2), 32)
    l2lo = dbl(ln2 - Decimal(l2hi))
    # exp reduction constant ln2 / 64 split the same way
    lnN = ln2 / N
    lnNhi = round_bits(dbl(lnN), 32)
    lnNlo = dbl(lnN - Decimal(lnNhi))
    invlnN = dbl(Decimal(N) / ln2)

    allv = exp2j + invc + lhi + llo
    body = ", \\\n".join("    " + ", ".join(hexd(v) for v in allv[i:i + 4]) for i in range(0, len(allv), 4))
    table_macro = "// EXP2J[0..63], INVC[64..127], LOGC_HI[128..191], LOGC_LO[192..255]\n" \
                  f"#define CLM_FM_TABLE_INIT {{ \\\n{body} }}\n"

    out = [
        "// Generated by gen_fastmath_tables.py; do not edit.",
        "// Tables of the table-driven FP64 exp/log (Tang 1989, 1990).",
        "#pragma once",
        "namespace clm { namespace fm {",
        f"constexpr double LN2_HI = {hexd(l2hi)};",
        f"constexpr double LN2_LO = {hexd(l2lo)};",
        f"constexpr double LNN_HI = {hexd(lnNhi)};  // ln2 / 64",
        f"constexpr double LNN_LO = {hexd(lnNlo)};",
        f"constexpr double INV_LNN = {hexd(invlnN)};  // 64 / ln2",
        "constexpr int TABLE_SIZE = 256;",
        table_macro,
        "} }  // namespace clm::fm",
        "",
    ]
    p = Path(__file__).with_name("clm_fastmath_tables.h")
    p.write_text("\n".join(out))
    print(p)


if __name__ == "__main__":
    main()
