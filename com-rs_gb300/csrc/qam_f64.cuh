// The f64 channel of the frame generators: one complex Gaussian sample of the
// reference's generator and the LLRs of one received QAM symbol.
#pragma once
#include <cuda_runtime.h>

#include "crmath_fast.cuh"
#include "device_common.cuh"

namespace cbk {

// Rng::complex_gaussian (crates/com-core/src/rng.rs:161-167): two uniforms u1, u2;
// r = sqrt(-2 ln(1 - u1)) / sqrt(2); (r cos 2 pi u2, r sin 2 pi u2), with the correctly
// rounded log, sin and cos (the fast paths of crmath_fast.cuh, the same bits as
// crmath.cuh's)
__device__ __forceinline__ void complex_gaussian_f64(cbd::Xoshiro& r, double& nre, double& nim) {
  const double u1 = (double)(cbd::xoshiro_next(r) >> 11) * (1.0 / 9007199254740992.0);
  const double u2 = (double)(cbd::xoshiro_next(r) >> 11) * (1.0 / 9007199254740992.0);
  const double l = crm::cr_log_fast(__dsub_rn(1.0, u1));
  const double rad = __dmul_rn(__dsqrt_rn(__dmul_rn(-2.0, l)), 0.70710678118654752440);
  double sn, cs;
  crm::cr_sincos_fast(__dmul_rn(6.283185307179586, u2), &sn, &cs);
  nre = __dmul_rn(rad, cs);
  nim = __dmul_rn(rad, sn);
}

// -ns / s2 correctly rounded, from y = RN(1/s2): q = RN(-ns y) is within an ulp of the
// quotient, the remainder r = -ns - s2 q is exact as one fused multiply-add, and
// RN(q + r y) is then the correctly rounded quotient (Markstein's theorem: P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000 processor", IBM J.
// Res. Develop. 34(1), 1990; Muller et al., Handbook of Floating-Point Arithmetic, 2018,
// ch. 4).  Three FP64 instructions instead of a division's dozen; the theorem needs no
// intermediate under- or overflow, so operands whose exponents leave [2^-800, 2^800]
// take the division.  A zero ns gives -0, as the division does.
__device__ __forceinline__ double neg_div_by(double ns, double s2, double y) {
  const double a = -ns;
  const double q = __dmul_rn(a, y);
  const unsigned ea = (unsigned)(__double2hiint(a) >> 20) & 0x7ffu, eq = (unsigned)(__double2hiint(q) >> 20) & 0x7ffu;
  if (ea == 0u) return ns == 0.0 ? q : __ddiv_rn(a, s2);
  if (ea - 223u > 1600u || eq - 223u > 1600u) return __ddiv_rn(a, s2);
  const double r = __fma_rn(-s2, q, a);
  return __fma_rn(r, y, q);
}

// max(a, b) of two negative doubles (or -inf), neither NaN: the larger has the smaller
// magnitude, so its bit pattern is the smaller unsigned integer (integer pipes, where
// fmax takes the FP64 pipe)
__device__ __forceinline__ double max_neg(double a, double b) {
  const unsigned long long x = (unsigned long long)__double_as_longlong(a);
  const unsigned long long z = (unsigned long long)__double_as_longlong(b);
  return __longlong_as_double((long long)(x < z ? x : z));
}

// demap_f64 (below) for a constellation of M points known at compile time: the M
// metrics once per symbol in registers, and exp(metric - max) once per symbol for the
// halves whose maximum is the symbol's largest metric.  Every value is computed by the
// same operations from the same operands as in demap_f64, so the LLRs are identical.
template <int M, typename Put>
__device__ __forceinline__ void demap_f64_fixed(const double* pts, double log_m, bool exact, double yre, double yim,
                                                double sigma2, double inv_s2, int n_bits, Put&& put) {
  constexpr int MB = M == 4 ? 2 : (M == 16 ? 4 : (M == 64 ? 6 : 8));
  const double uniform = -log_m;
  double met[M];
  double top = -INFINITY;
#pragma unroll
  for (int i = 0; i < M; i++) {
    const double dr = __dsub_rn(yre, pts[2 * i]), di = __dsub_rn(yim, pts[2 * i + 1]);
    const double ns = __dadd_rn(__dmul_rn(dr, dr), __dmul_rn(di, di));
    met[i] = __dadd_rn(neg_div_by(ns, sigma2, inv_s2), uniform);
    top = max_neg(top, met[i]);
  }
  double ex[M];
  if (exact && isfinite(top)) {
#pragma unroll
    for (int i = 0; i < M; i++) ex[i] = exp(__dsub_rn(met[i], top));
  }
#pragma unroll
  for (int o = 0; o < MB; o++) {
    if (o >= n_bits) break;
    const int shift = MB - 1 - o;
    double m0 = -INFINITY, m1 = -INFINITY;
#pragma unroll
    for (int i = 0; i < M; i++) {
      if ((i >> shift) & 1) m1 = max_neg(m1, met[i]);
      else m0 = max_neg(m0, met[i]);
    }
    if (exact && isfinite(m0) && isfinite(m1)) {
      double s0 = 0.0, s1 = 0.0;
#pragma unroll
      for (int i = 0; i < M; i++) {
        if ((i >> shift) & 1) s1 = __dadd_rn(s1, m1 == top ? ex[i] : exp(__dsub_rn(met[i], m1)));
        else s0 = __dadd_rn(s0, m0 == top ? ex[i] : exp(__dsub_rn(met[i], m0)));
      }
      put(o, __dsub_rn(__dsub_rn(__dadd_rn(m0, log(s0)), m1), log(s1)));
    } else {
      put(o, __dsub_rn(m0, m1));
    }
  }
}

// The LLRs of the mbits bits of one symbol y, most significant first
// (crates/com-mapping/src/demapper.rs:82-146, :270-297): metric_i = -|y - x_i|^2 /
// sigma^2 - ln M; max-log L = max_{b=0} - max_{b=1}; exact (LabelHalves) the sums of
// exp(metric - max) in label order, L = m0 + ln s0 - m1 - ln s1, with CUDA's exp and
// log where the reference calls libm.  put(o, L) receives bit o's LLR; bits at o >=
// n_bits are skipped.
// QPSK and 16-QAM take demap_f64_fixed.  Every metric is negative (-ns / sigma^2 - ln M
// with ln M > 0), so the maxima take max_neg; inv_s2 is RN(1 / sigma2) for neg_div_by.
template <typename Put>
__device__ __forceinline__ void demap_f64(const double* pts, int m, int mbits, double log_m, bool exact, double yre,
                                          double yim, double sigma2, double inv_s2, int n_bits, Put&& put) {
  if (m == 4) return demap_f64_fixed<4>(pts, log_m, exact, yre, yim, sigma2, inv_s2, n_bits, put);
  if (m == 16) return demap_f64_fixed<16>(pts, log_m, exact, yre, yim, sigma2, inv_s2, n_bits, put);
  const double uniform = -log_m;
  for (int o = 0; o < mbits && o < n_bits; o++) {
    const int shift = mbits - 1 - o;
    double m0 = -INFINITY, m1 = -INFINITY;
    for (int i = 0; i < m; i++) {
      const double dr = __dsub_rn(yre, pts[2 * i]), di = __dsub_rn(yim, pts[2 * i + 1]);
      const double ns = __dadd_rn(__dmul_rn(dr, dr), __dmul_rn(di, di));
      const double met = __dadd_rn(neg_div_by(ns, sigma2, inv_s2), uniform);
      if ((i >> shift) & 1) m1 = max_neg(m1, met);
      else m0 = max_neg(m0, met);
    }
    if (exact && isfinite(m0) && isfinite(m1)) {
      double s0 = 0.0, s1 = 0.0;
      for (int i = 0; i < m; i++) {
        const double dr = __dsub_rn(yre, pts[2 * i]), di = __dsub_rn(yim, pts[2 * i + 1]);
        const double ns = __dadd_rn(__dmul_rn(dr, dr), __dmul_rn(di, di));
        const double met = __dadd_rn(neg_div_by(ns, sigma2, inv_s2), uniform);
        if ((i >> shift) & 1) s1 = __dadd_rn(s1, exp(__dsub_rn(met, m1)));
        else s0 = __dadd_rn(s0, exp(__dsub_rn(met, m0)));
      }
      put(o, __dsub_rn(__dsub_rn(__dadd_rn(m0, log(s0)), m1), log(s1)));
    } else {
      put(o, __dsub_rn(m0, m1));
    }
  }
}

}  // namespace cbk
