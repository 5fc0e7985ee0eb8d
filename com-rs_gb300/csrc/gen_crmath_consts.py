"""Generate ``crmath_consts.inc``: double-double constants of the correctly-rounded
f64 logarithm and sine/cosine used by the f64 noise kernels, and the tables of the fast
sine/cosine (crmath_fast.cuh): sin and cos of j pi/128, j = 0..32, as double-doubles, and
pi/128 as H1 + H2 + H3 with H1 a multiple of 2^-45 (j H1 exact for |j| <= 32).

Constants are computed exactly (fractions) or to 60 decimal digits (decimal module):
ln 2, pi/2 as three doubles, 1/(2k+1) for the atanh series of the logarithm and 1/n!
for the Taylor series of sine and cosine, each split as hi + lo with hi = RN(value),
lo = RN(value - hi).  Usage: ``python gen_crmath_consts.py > crmath_consts.inc``
"""

from decimal import Decimal, getcontext
from fractions import Fraction

getcontext().prec = 80


def atan_inv(n):
    """atan(1/n) by its Taylor series, to the context precision."""
    x = Decimal(1) / n
    x2 = x * x
    term, total, k = x, Decimal(0), 0
    while abs(term) > Decimal(10) ** -75:
        total += term / (2 * k + 1) * (1 if k % 2 == 0 else -1)
        term *= x2
        k += 1
    return total


def split(v, parts=2):
    """v (Decimal or Fraction) as `parts` doubles, each the rounding of the rest."""
    out = []
    rest = Fraction(v) if isinstance(v, Fraction) else Fraction(str(v))
    for _ in range(parts):
        d = float(rest)  # Fraction -> float is correctly rounded
        out.append(d)
        rest -= Fraction(d)
    return out


def h(d):
    return d.hex()


def main():
    pi = 16 * atan_inv(5) - 4 * atan_inv(239)
    ln2 = Decimal(2).ln()
    print("/* Double-double constants of the correctly-rounded f64 log and sin/cos.")
    print("   Generated by gen_crmath_consts.py (exact fractions / 80-digit decimals). */")
    hi, lo = split(ln2)
    print(f"#define CR_LN2_HI {h(hi)}\n#define CR_LN2_LO {h(lo)}")
    p1, p2, p3 = split(pi / 2, 3)
    print(f"#define CR_PIO2_1 {h(p1)}\n#define CR_PIO2_2 {h(p2)}\n#define CR_PIO2_3 {h(p3)}")
    # 2/pi to pick the quadrant
    print(f"#define CR_TWO_OVER_PI {h(float(2 / pi))}")
    # atanh series: 1/(2k+1), k = 0..CR_LOG_TERMS-1
    n_log = 23
    print(f"#define CR_LOG_TERMS {n_log}")
    print("CR_CONST double CR_LOG_COEF[CR_LOG_TERMS][2] = {")
    for k in range(n_log):
        a, b = split(Fraction(1, 2 * k + 1))
        print(f"  {{{h(a)}, {h(b)}}},")
    print("};")
    # sin: (-1)^k / (2k+1)!, cos: (-1)^k / (2k)!
    n_trig = 16
    print(f"#define CR_TRIG_TERMS {n_trig}")
    for name, off in (("CR_SIN_COEF", 1), ("CR_COS_COEF", 0)):
        print(f"CR_CONST double {name}[CR_TRIG_TERMS][2] = {{")
        for k in range(n_trig):
            fact = 1
            for t in range(1, 2 * k + off + 1):
                fact *= t
            a, b = split(Fraction((-1) ** k, fact))
            print(f"  {{{h(a)}, {h(b)}}},")
        print("};")
    main_fast(pi)


def sin_cos(x):
    """sin and cos of the Decimal x by their Taylor series, to the context precision."""
    s, c, term, k = Decimal(0), Decimal(0), Decimal(1), 0
    while True:
        if k % 4 == 0:
            c += term
        elif k % 4 == 1:
            s += term
        elif k % 4 == 2:
            c -= term
        else:
            s -= term
        k += 1
        term = term * x / k
        if abs(term) < Decimal(10) ** -75:
            return s, c


def main_fast(pi):
    hh = pi / 128
    h1 = Fraction(round(Fraction(str(hh)) * 2 ** 45), 2 ** 45)
    assert float(h1) == h1
    h2, h3 = split(Fraction(str(hh)) - h1)
    print(f"#define CR_SC_H1 {h(float(h1))}")
    print(f"#define CR_SC_H2 {h(h2)}")
    print(f"#define CR_SC_H3 {h(h3)}")
    print(f"#define CR_SC_INV_H {h(float(128 / pi))}")
    print("#define CR_SC_N 33")
    print("CR_CONST double CR_SC_TAB[CR_SC_N][4] = {  /* sin hi, sin lo, cos hi, cos lo of j pi/128 */")
    for j in range(33):
        sv, cv = sin_cos(hh * j)
        a, b = split(sv)
        c, d = split(cv)
        print(f"  {{{h(a)}, {h(b)}, {h(c)}, {h(d)}}},")
    print("};")


if __name__ == "__main__":
    main()
