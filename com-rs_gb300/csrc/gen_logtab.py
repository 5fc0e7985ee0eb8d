"""Generate ``logtab.inc``: the logarithm table of the f64 2 atanh of the sum-product rule
(atanh2.cuh) and of the fast correctly rounded log (crmath_fast.cuh).

The logarithm follows Tang's table-driven method (P. T. P. Tang, "Table-driven
implementation of the logarithm function in IEEE floating-point arithmetic", ACM TOMS
16(4), 1990): for x = 2^e m, m in [1, 2), j = round(256 (m - 1)) picks F_j = 1 + j/256
and c_j, 1/F_j rounded to 9 significant bits.  Then |r| = |m c_j - 1| < 2^-8 and r, a
multiple of 2^-61, fits 53 bits: one fused multiply-add computes it exactly.  Finally
log x = e ln 2 - ln c_j + log1p(r).

Written here, each computed exactly (fractions) or to 60 digits (decimal module):
  * LOGTAB_LN2_HI: ln 2 rounded to a multiple of 2^-43, so that e * LN2_HI + L_hi is exact
    for 0 <= e < 64; LOGTAB_LN2_LO = RN(ln 2 - LN2_HI);
  * LOGTAB[j] = {c_j, L_hi_j, L_lo_j}, j = 0..256: L_hi_j = -ln c_j rounded to a multiple
    of 2^-43, L_lo_j = RN(-ln c_j - L_hi_j);
  * LOGTAB_Q: the Taylor coefficients (-1)^(k+1) / (k + 2), k = 0..5, of
    (log1p(r) - r) / r^2.
Usage: ``python gen_logtab.py > logtab.inc``
"""

from decimal import Decimal, getcontext
from fractions import Fraction

getcontext().prec = 60

N_TAB = 256  # intervals of m in [1, 2); entries j = 0..N_TAB
C_BITS = 9  # significant bits of c_j
Q_TERMS = 6


def ln(fr):
    """ln of a positive Fraction, to the context precision."""
    return Decimal(fr.numerator).ln() - Decimal(fr.denominator).ln()


def to_grid(v, ulp_exp):
    """Decimal v rounded to the nearest multiple of 2^ulp_exp, as an exact Fraction."""
    scaled = Fraction(str(v)) / Fraction(2) ** ulp_exp
    return Fraction(round(scaled)) * Fraction(2) ** ulp_exp


def c_of(j):
    """1 / (1 + j / N_TAB) rounded to C_BITS significant bits (c in (1/2, 1])."""
    inv = Fraction(N_TAB, N_TAB + j)
    if inv == 1:
        return Fraction(1)
    # inv in (1/2, 1): the leading bit is 2^-1, so C_BITS bits end at 2^-C_BITS
    return Fraction(round(inv * 2 ** C_BITS), 2 ** C_BITS)


def main():
    ln2 = Decimal(2).ln()
    ln2_hi = to_grid(ln2, -43)
    ln2_lo = float(Fraction(str(ln2)) - ln2_hi)
    print("/* Tang's table-driven logarithm: the table of atanh2.cuh and crmath_fast.cuh.")
    print("   Generated by gen_logtab.py (exact fractions / 60-digit decimals). */")
    print("#pragma once")
    print("#if defined(__CUDA_ARCH__)\n#define LOGTAB_CONST __device__ static const\n#else\n#define LOGTAB_CONST static const\n#endif")
    print(f"#define LOGTAB_LN2_HI {float(ln2_hi).hex()}")
    print(f"#define LOGTAB_LN2_LO {ln2_lo.hex()}")
    print(f"#define LOGTAB_N {N_TAB + 1}")
    print("LOGTAB_CONST double LOGTAB[LOGTAB_N][3] = {")
    for j in range(N_TAB + 1):
        c = c_of(j)
        L = -ln(c)
        hi = to_grid(L, -43)
        lo = float(Fraction(str(L)) - hi)
        assert float(c) == c and float(hi) == hi
        print(f"  {{{float(c).hex()}, {float(hi).hex()}, {lo.hex()}}},")
    print("};")
    print(f"#define LOGTAB_Q_TERMS {Q_TERMS}")
    print("LOGTAB_CONST double LOGTAB_Q[LOGTAB_Q_TERMS] = {")
    for k in range(Q_TERMS):
        print(f"  {float(Fraction((-1) ** (k + 1), k + 2)).hex()},")
    print("};")


if __name__ == "__main__":
    main()
