// Correctly-rounded f64 natural logarithm and sine/cosine for the noise draws.
//
// The reference draws its Gaussian noise with the platform libm (Rust std:
// `ln`, `sin_cos`, crates/com-core/src/rng.rs:161-167), whose last bit depends on the
// platform.  The GPU path computes the correctly-rounded value instead, so that a
// frame's noise is a pure function of its stream on every machine.
//
// Method: double-double arithmetic (the error-free transformations of Knuth's TwoSum
// and Dekker's product with FMA, as in Hida, Li & Bailey, "Algorithms for quad-double
// precision floating point arithmetic", ARITH-15, 2001), evaluated to about 2^-104
// relative and rounded once:
//   * log: x = 2^e m, m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(f), f = (m-1)/(m+1),
//     with the atanh Taylor series in f^2;
//   * sin/cos: Cody-Waite reduction a = k pi/2 + t with pi/2 as three doubles, then the
//     Taylor series of sin t and cos t for |t| <= pi/4, and the quadrant.
// Every operation is an explicitly rounded one (no contraction), so the host copy
// compiled with -ffp-contract=off returns the same bits as the device.
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define CR_HD __host__ __device__ __forceinline__
#else
#define CR_HD inline
#endif

#if defined(__CUDA_ARCH__)
#define CR_CONST __device__ static const
#else
#define CR_CONST static const
#endif

#include <cmath>
#include <cstring>

#include "crmath_consts.inc"

namespace crm {

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ int64_t d2ll(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double ll2d(int64_t x) { return __longlong_as_double(x); }
#else
inline double add_rn(double a, double b) { return a + b; }
inline double mul_rn(double a, double b) { return a * b; }
inline double fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline double div_rn(double a, double b) { return a / b; }
inline int64_t d2ll(double x) { int64_t r; std::memcpy(&r, &x, 8); return r; }
inline double ll2d(int64_t x) { double r; std::memcpy(&r, &x, 8); return r; }
#endif
CR_HD double sub_rn(double a, double b) { return add_rn(a, -b); }

struct dd {
  double hi, lo;
};

CR_HD dd two_sum(double a, double b) {
  double s = add_rn(a, b);
  double bb = sub_rn(s, a);
  double e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
  return {s, e};
}
CR_HD dd quick_two_sum(double a, double b) {
  double s = add_rn(a, b);
  return {s, sub_rn(b, sub_rn(s, a))};
}
CR_HD dd two_prod(double a, double b) {
  double p = mul_rn(a, b);
  return {p, fma_rn(a, b, -p)};
}
CR_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  double e = add_rn(s.lo, t.hi);
  dd u = quick_two_sum(s.hi, e);
  e = add_rn(u.lo, t.lo);
  return quick_two_sum(u.hi, e);
}
CR_HD dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  double e = add_rn(p.lo, add_rn(mul_rn(a.hi, b.lo), mul_rn(a.lo, b.hi)));
  return quick_two_sum(p.hi, e);
}
CR_HD dd dd_mul_d(dd a, double b) {
  dd p = two_prod(a.hi, b);
  double e = add_rn(p.lo, mul_rn(a.lo, b));
  return quick_two_sum(p.hi, e);
}
// a / b for double-doubles: two Newton-style correction steps
CR_HD dd dd_div(dd a, dd b) {
  double q1 = div_rn(a.hi, b.hi);
  dd r = dd_add(a, dd_mul_d(b, -q1));
  double q2 = div_rn(r.hi, b.hi);
  r = dd_add(r, dd_mul_d(b, -q2));
  double q3 = div_rn(r.hi, b.hi);
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}

// log(x) correctly rounded, x positive and finite (subnormals included)
CR_HD double cr_log(double x) {
  if (x == 1.0) return 0.0;
  int64_t bits = d2ll(x);
  int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) {  // subnormal: scale by 2^54
    x = mul_rn(x, 18014398509481984.0);
    bits = d2ll(x);
    e = (int)((bits >> 52) & 0x7ff) - 54;
  }
  e -= 1023;
  double m = ll2d((bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll);  // [1, 2)
  if (m > 1.4142135623730951) {
    m = mul_rn(m, 0.5);
    e += 1;
  }
  // f = (m - 1)/(m + 1): m - 1 is exact (Sterbenz), m + 1 as an exact pair
  dd num = {sub_rn(m, 1.0), 0.0};
  dd den = two_sum(m, 1.0);
  dd f = dd_div(num, den);
  dd s = dd_mul(f, f);
  dd p = {CR_LOG_COEF[CR_LOG_TERMS - 1][0], CR_LOG_COEF[CR_LOG_TERMS - 1][1]};
  for (int k = CR_LOG_TERMS - 2; k >= 0; k--) {
    p = dd_mul(p, s);
    p = dd_add(p, dd{CR_LOG_COEF[k][0], CR_LOG_COEF[k][1]});
  }
  dd lm = dd_mul(f, p);
  lm.hi = mul_rn(lm.hi, 2.0);
  lm.lo = mul_rn(lm.lo, 2.0);
  if (e != 0) {
    double ed = (double)e;
    dd el = two_prod(ed, CR_LN2_HI);
    el = dd_add(el, two_prod(ed, CR_LN2_LO));
    lm = dd_add(el, lm);
  }
  return add_rn(lm.hi, lm.lo);
}

// sin(a) and cos(a) correctly rounded for 0 <= a < 8 (the angles 2 pi u, u in [0, 1))
CR_HD void cr_sincos(double a, double* s_out, double* c_out) {
  double kd = std::floor(add_rn(mul_rn(a, CR_TWO_OVER_PI), 0.5));
  int k = (int)kd;
  // t = a - k pi/2 in double-double; a - k*P1 is exact by Sterbenz once split exactly
  dd kp1 = two_prod(kd, CR_PIO2_1);
  dd t = two_sum(sub_rn(a, kp1.hi), -kp1.lo);
  t = dd_add(t, dd_mul_d(dd{-CR_PIO2_2, 0.0}, kd));
  t = dd_add(t, dd{mul_rn(-CR_PIO2_3, kd), 0.0});
  dd t2 = dd_mul(t, t);
  dd ps = {CR_SIN_COEF[CR_TRIG_TERMS - 1][0], CR_SIN_COEF[CR_TRIG_TERMS - 1][1]};
  dd pc = {CR_COS_COEF[CR_TRIG_TERMS - 1][0], CR_COS_COEF[CR_TRIG_TERMS - 1][1]};
  for (int i = CR_TRIG_TERMS - 2; i >= 0; i--) {
    ps = dd_add(dd_mul(ps, t2), dd{CR_SIN_COEF[i][0], CR_SIN_COEF[i][1]});
    pc = dd_add(dd_mul(pc, t2), dd{CR_COS_COEF[i][0], CR_COS_COEF[i][1]});
  }
  dd sn = dd_mul(ps, t);
  double sv = add_rn(sn.hi, sn.lo), cv = add_rn(pc.hi, pc.lo);
  switch (k & 3) {
    case 0: *s_out = sv; *c_out = cv; break;
    case 1: *s_out = cv; *c_out = -sv; break;
    case 2: *s_out = -sv; *c_out = -cv; break;
    default: *s_out = -cv; *c_out = sv; break;
  }
}

}  // namespace crm
