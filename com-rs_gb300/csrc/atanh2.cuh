// 2 atanh(p) in f64 for the sum-product check-node rule, o = 2 atanh(clamp(p, -B, B))
// (crates/com-fec/src/ldpc.rs:93, :451-466), in about half the FP64 instructions of
// CUDA's atanh (measured on GB300: 36 against 63 plus the doubling).
//
// Method: 2 atanh(a) = log u, u = (1 + a) / (1 - a), for a = min(|p|, B) >= 0; the sign of
// p is put back at the end.
//   * 1 + a and 1 - a are exact double-double sums; u = q + ul is their quotient to about
//     2^-100 relative: q = s RN(1/d), and the remainder by fused multiply-adds.
//   * log u by Tang's table-driven method (P. T. P. Tang, ACM TOMS 16(4), 1990), tables
//     in logtab.inc.  q = 2^e m with m in [1, 2); j = round(256 (m - 1)); r = m c_j - 1,
//     exact; log u = e ln 2 - ln c_j + log1p(r) + ul / q, with log1p(r) = r + r^2 Q(r) from
//     its Taylor series (|r| < 2^-8, truncation below 2^-61 relative), ln 2 and ln c_j as
//     hi + lo pairs whose hi parts add exactly, and ul / q = ul c_j 2^-e (1 - r) to first
//     order.  The last two additions are a Fast2Sum of the exact hi part and r, then
//     the rest.
// Every step is an explicitly rounded IEEE operation, so the host copy (tests, compiled
// with -ffp-contract=off) returns the same bits as the device.  Measured against 2 atanhl
// in x86 long double on 12 M inputs: within 0.51 ulp, the correctly rounded value on
// 99.97 % of them.  glibc's atanh (the reference's libm) is within 1.7 ulp and correctly
// rounded on 82-97 % of the same inputs, so the two differ by an ulp on the rest, as
// CUDA's atanh does.
//
// Domain: B < 1 - 2^-40, so that u < 2^41; p finite (the product of tanh values).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define AT2_HD __host__ __device__ __forceinline__
#else
#define AT2_HD inline
#endif

#include <cstring>

#include "logtab.inc"

namespace at2 {

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double rcp(double a) { return __drcp_rn(a); }
__device__ __forceinline__ uint64_t bits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double from_bits(uint64_t b) { return __longlong_as_double((long long)b); }
// the bits of |x| by an AND in inline PTX (written in C++, the compiler turns the AND into
// fabs and forms |x| with an FP64 instruction for the integer comparison that follows)
__device__ __forceinline__ uint64_t abs_bits(uint64_t b) {
  uint64_t r;
  asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(r) : "l"(b));
  return r;
}
__device__ __forceinline__ double tab(int j, int k) { return __ldg(&LOGTAB[j][k]); }
#else
inline double add(double a, double b) { return a + b; }
inline double sub(double a, double b) { return a - b; }
inline double mul(double a, double b) { return a * b; }
inline double fma_rn(double a, double b, double c) { return __builtin_fma(a, b, c); }
inline double rcp(double a) { return 1.0 / a; }
inline uint64_t bits(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
}
inline uint64_t abs_bits(uint64_t b) { return b & 0x7fffffffffffffffull; }
inline double from_bits(uint64_t b) {
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}
inline double tab(int j, int k) { return LOGTAB[j][k]; }
#endif

// 2 atanh(clamp(p, -bound, bound)) (see the header comment for the domain)
AT2_HD double twice_atanh(double p, double bound) {
  const uint64_t sign = bits(p) & 0x8000000000000000ull;
  // a = min(|p|, bound): non-negative doubles order as their bit patterns
  uint64_t ab = abs_bits(bits(p));
  const uint64_t bb = bits(bound);
  ab = ab < bb ? ab : bb;
  const double a = from_bits(ab);
  // 1 + a = s + t and 1 - a = d + dl, exactly (Fast2Sum: 1 >= a)
  const double s = add(1.0, a);
  const double t = sub(a, sub(s, 1.0));
  const double d = sub(1.0, a);
  const double dl = sub(sub(1.0, d), a);
  // u = (s + t) / (d + dl) = q + ul
  const double R = rcp(d);
  const double q = mul(s, R);
  double rho = fma_rn(-q, d, s);
  rho = add(rho, t);
  rho = fma_rn(-q, dl, rho);
  const double ul = mul(rho, R);
  // q = 2^e m, q >= 1
  const uint64_t qb = bits(q);
  const int e = (int)(qb >> 52) - 1023;
  const double m = from_bits((qb & 0x000fffffffffffffull) | 0x3ff0000000000000ull);
  const int j = (int)((((qb >> 43) & 511u) + 1u) >> 1);
  const double c = tab(j, 0), lhi = tab(j, 1), llo = tab(j, 2);
  const double r = fma_rn(m, c, -1.0);
  // ul / q to first order in r; c 2^-e is exact (c in [1/2, 1], 0 <= e < 41)
  const double cs = from_bits(bits(c) - ((uint64_t)e << 52));
  const double d0 = mul(ul, cs);
  const double delta = fma_rn(-d0, r, d0);
  double qp = LOGTAB_Q[LOGTAB_Q_TERMS - 1];
  for (int k = LOGTAB_Q_TERMS - 2; k >= 0; k--) qp = fma_rn(qp, r, LOGTAB_Q[k]);
  const double r2 = mul(r, r);
  const double ed = (double)e;
  const double hi = fma_rn(ed, LOGTAB_LN2_HI, lhi);  // exact
  double lo = fma_rn(ed, LOGTAB_LN2_LO, llo);
  lo = add(lo, delta);
  lo = fma_rn(r2, qp, lo);
  // hi + r by Fast2Sum: hi is 0 (then S = r) or at least -ln c_1 > |r|
  const double S = add(hi, r);
  const double err = add(sub(hi, S), r);
  double res = add(S, add(err, lo));
  // a < 2^-27: 2 atanh(a) = 2a (1 + a^2/3 + ...) rounds to 2a, which the sum above misses
  // by up to an ulp when ul is as large as the result
  if (ab < 0x3e40000000000000ull) res = add(a, a);
  return from_bits(bits(res) | sign);
}

}  // namespace at2
