// Fast paths of the correctly rounded f64 log and sin/cos of crmath.cuh, by Ziv's strategy
// (A. Ziv, "Fast evaluation of elementary mathematical functions with correctly rounded
// last bit", ACM TOMS 17(3), 1991): a quick evaluation S + T with a proven absolute error
// bound eps, then a rounding test.  If S + (T - eps) and S + (T + eps) round to the same
// double, that double is the correctly rounded value; otherwise (about one call in 10^4)
// the double-double routine of crmath.cuh decides.  The results are therefore the same
// bits as crmath.cuh's, at a few percent of its FP64 work.
//
// log: Tang's table-driven method (P. T. P. Tang, ACM TOMS 16(4), 1990) on the table of
// logtab.inc: x = 2^e m, m in [1, 2); j = round(256 (m - 1)); r = m c_j - 1, exact,
// |r| < 2^-8.41; log x = e ln 2 - ln c_j + r - r^2/2 + r^3 (1/3 - r/4 + ... - r^5/8), with
// the exact part e LN2_HI + L_hi_j and the leading terms summed by error-free
// transformations.  Error (absolute): below 2^-75 + 2^-103 |log x| when the exact part is
// not zero, else below |r|^3 2^-48 + 2^-103 |log x|.
//
// sin/cos of a in [0, 8): t = a - k pi/2 with pi/2 in three parts (error-free products and
// sums: t stays accurate when a is close to a multiple of pi/2); then t = j pi/128 + s,
// |s| <= pi/256, with the double-double table of sin and cos of j pi/128
// (crmath_consts.inc): sin t = S_j (1 + cm) + C_j sin s and cos t = C_j (1 + cm) - S_j sin s,
// cm = cos s - 1, the products with the table's leading parts exact and summed by
// Fast2Sum.  Error (absolute): below 2^-70 + 2^-100 |result| for j != 0 and for cos,
// |s|^3 2^-50 + 2^-100 |sin t| for sin with j = 0.
#pragma once
#include <cstdint>

#include "crmath.cuh"
#include "logtab.inc"

namespace crm {

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ double logtab(int j, int k) { return __ldg(&LOGTAB[j][k]); }
#else
inline double logtab(int j, int k) { return LOGTAB[j][k]; }
#endif

// Ziv's rounding test: S + T with |error| <= eps.  Widening eps by 2^-50 |T| covers the
// rounding of T +- eps, so both sums bracket the exact value's rounding.
CR_HD bool round_test(double S, double T, double eps, double* out) {
  const double w = fma_rn(std::fabs(T), 8.8817841970012523e-16, add_rn(eps, eps));
  const double up = add_rn(S, add_rn(T, w)), dn = add_rn(S, sub_rn(T, w));
  *out = up;
  return up == dn;
}

// log(x) correctly rounded: the fast path for normal x, crmath.cuh's cr_log otherwise
CR_HD double cr_log_fast(double x) {
  const uint64_t b = (uint64_t)d2ll(x);
  if (b - 0x0010000000000000ull >= 0x7fe0000000000000ull) return cr_log(x);  // not normal positive
  const int e = (int)(b >> 52) - 1023;
  const double m = ll2d((int64_t)((b & 0x000fffffffffffffull) | 0x3ff0000000000000ull));
  const int j = (int)((((b >> 43) & 511u) + 1u) >> 1);
  const double c = logtab(j, 0), lh = logtab(j, 1), ll = logtab(j, 2);
  const double r = fma_rn(m, c, -1.0);  // exact
  const double rh = mul_rn(r, r), rl = fma_rn(r, r, -rh);
  double q = -0.125;
  q = fma_rn(q, r, 0.14285714285714285);
  q = fma_rn(q, r, -0.16666666666666666);
  q = fma_rn(q, r, 0.2);
  q = fma_rn(q, r, -0.25);
  q = fma_rn(q, r, 0.33333333333333331);
  const double r3 = mul_rn(rh, r);
  const double t3 = mul_rn(r3, q);
  const double ed = (double)e;
  const double hi = fma_rn(ed, LOGTAB_LN2_HI, lh);  // exact: both on the 2^-43 grid
  const double lo0 = fma_rn(ed, LOGTAB_LN2_LO, ll);
  // hi + r (TwoSum: near x = 1 from below |hi| can be smaller than |r|), then - rh/2
  // (Fast2Sum: |S1| >= 2^-10 > rh/2 unless hi = 0, when S1 = r)
  const dd s1 = two_sum(hi, r);
  const dd s2 = quick_two_sum(s1.hi, mul_rn(-0.5, rh));
  const double T = add_rn(add_rn(s1.lo, s2.lo), add_rn(lo0, fma_rn(-0.5, rl, t3)));
  const double rel = mul_rn(std::fabs(s2.hi), 9.8607613152626476e-32);  // 2^-103 |S|
  const double eps = hi != 0.0 ? add_rn(2.6469779601696886e-23, rel)     // 2^-75
                               : fma_rn(std::fabs(r3), 3.5527136788005009e-15, rel);  // 2^-48 |r^3|
  double y;
  if (round_test(s2.hi, T, eps, &y)) return y;
  return cr_log(x);
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ double sctab(int j, int k) { return __ldg(&CR_SC_TAB[j][k]); }
#else
inline double sctab(int j, int k) { return CR_SC_TAB[j][k]; }
#endif

// sin(a) and cos(a) correctly rounded for 0 <= a < 8: the fast path, crmath.cuh's
// cr_sincos when a rounding test fails
CR_HD void cr_sincos_fast(double a, double* s_out, double* c_out) {
  if (!(a >= 0.0 && a < 8.0)) return cr_sincos(a, s_out, c_out);
  const double kd = std::floor(add_rn(mul_rn(a, CR_TWO_OVER_PI), 0.5));
  const int k = (int)kd;
  // t = th + tl = a - k pi/2
  double th = a, tl = 0.0;
  if (k != 0) {
    const dd p1 = two_prod(kd, CR_PIO2_1);
    const dd p2 = two_prod(kd, CR_PIO2_2);
    const dd u = two_sum(sub_rn(a, p1.hi), -p1.lo);  // a - p1.hi is exact (Sterbenz)
    const dd v = two_sum(u.hi, -p2.hi);
    const double w = add_rn(add_rn(u.lo, v.lo), sub_rn(-p2.lo, mul_rn(kd, CR_PIO2_3)));
    const dd t = quick_two_sum(v.hi, w);
    th = t.hi;
    tl = t.lo;
  }
  // s = sh + sl = t - j pi/128; j H1 and th - j H1 are exact
  const double jd = std::rint(mul_rn(th, CR_SC_INV_H));
  const int j = (int)jd, aj = j < 0 ? -j : j;
  const dd jh2 = two_prod(jd, CR_SC_H2);
  const dd s1 = two_sum(fma_rn(-jd, CR_SC_H1, th), -jh2.hi);
  const double sh = s1.hi;
  const double sl = add_rn(s1.lo, sub_rn(sub_rn(tl, jh2.lo), mul_rn(jd, CR_SC_H3)));
  const double sg = j < 0 ? -1.0 : 1.0;
  const double Sh = mul_rn(sg, sctab(aj, 0)), Sl = mul_rn(sg, sctab(aj, 1));
  const double Ch = sctab(aj, 2), Cl = sctab(aj, 3);
  // z = sh^2; sin s = sh + sl + sh z P(z); cos s - 1 = cm_hi + cm_lo
  const dd z = two_prod(sh, sh);
  double P = 2.7557319223985893e-06;
  P = fma_rn(P, z.hi, -1.9841269841269841e-04);
  P = fma_rn(P, z.hi, 8.3333333333333332e-03);
  P = fma_rn(P, z.hi, -0.16666666666666666);
  double Q = -2.7557319223985888e-07;
  Q = fma_rn(Q, z.hi, 2.4801587301587302e-05);
  Q = fma_rn(Q, z.hi, -1.3888888888888889e-03);
  Q = fma_rn(Q, z.hi, 4.1666666666666664e-02);
  const double s3p = mul_rn(mul_rn(sh, z.hi), P);
  const double cm_hi = mul_rn(-0.5, z.hi);
  const double cm_lo = fma_rn(mul_rn(z.hi, z.hi), Q, fma_rn(-sh, sl, mul_rn(-0.5, z.lo)));
  const double sls = add_rn(sl, s3p);  // sin s - sh
  // sin t
  const dd ps = two_prod(Ch, sh);
  const dd as = quick_two_sum(Sh, ps.hi);
  const dd ms = two_prod(Sh, cm_hi);
  const dd bs = quick_two_sum(as.hi, ms.hi);
  double rs = add_rn(add_rn(as.lo, bs.lo), add_rn(ps.lo, ms.lo));
  rs = add_rn(rs, fma_rn(Sh, cm_lo, fma_rn(Sl, cm_hi, fma_rn(Cl, sh, Sl))));
  rs = fma_rn(Ch, sls, rs);
  // cos t
  const dd pc = two_prod(-Sh, sh);
  const dd ac = quick_two_sum(Ch, pc.hi);
  const dd mc = two_prod(Ch, cm_hi);
  const dd bc = quick_two_sum(ac.hi, mc.hi);
  double rc = add_rn(add_rn(ac.lo, bc.lo), add_rn(pc.lo, mc.lo));
  rc = add_rn(rc, fma_rn(Ch, cm_lo, fma_rn(Cl, cm_hi, fma_rn(-Sl, sh, Cl))));
  rc = fma_rn(-Sh, sls, rc);
  const double es = j != 0 ? fma_rn(std::fabs(bs.hi), 7.8886090522101181e-31, 8.4703294725430034e-22)  // 2^-100, 2^-70
                           : fma_rn(std::fabs(bs.hi), 7.8886090522101181e-31,
                                    mul_rn(std::fabs(mul_rn(sh, z.hi)), 8.8817841970012523e-16));  // 2^-50 |s|^3
  const double ec = fma_rn(std::fabs(bc.hi), 7.8886090522101181e-31, 8.4703294725430034e-22);
  double sv, cv;
  if (!round_test(bs.hi, rs, es, &sv) || !round_test(bc.hi, rc, ec, &cv)) return cr_sincos(a, s_out, c_out);
  switch (k & 3) {
    case 0: *s_out = sv; *c_out = cv; break;
    case 1: *s_out = cv; *c_out = -sv; break;
    case 2: *s_out = -sv; *c_out = -cv; break;
    default: *s_out = -cv; *c_out = sv; break;
  }
}

}  // namespace crm
