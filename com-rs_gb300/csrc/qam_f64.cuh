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

// The measured power's sum of |x|^2 over a frame's symbols (com-math lib.rs:146-148), in
// symbol order as the reference adds it, each term RN(RN(re^2) + RN(im^2)).  A term only
// depends on the symbol's label, so the block computes the M labels' energies once
// (label_energies, into shared memory; a barrier follows) and one thread adds them up
// (energy_sum): the sequential chain is then one FP64 addition per symbol instead of two
// multiplications and two additions.  The chain runs on one lane, and a one-lane FP64
// instruction holds the FP64 pipe as long as a full warp's.
__device__ __forceinline__ void label_energies(const double* pts, int m, double* en, int tid, int nt) {
  for (int i = tid; i < m; i += nt) {
    const double re = pts[2 * i], im = pts[2 * i + 1];
    en[i] = __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
  }
}
__device__ __forceinline__ double energy_sum(const uint8_t* lab, int n_sym, const double* en) {
  double e = 0.0;
#pragma unroll 8
  for (int s = 0; s < n_sym; s++) e = __dadd_rn(e, en[lab[s]]);
  return e;
}

// the reflected binary Gray code, at compile time
__host__ __device__ constexpr int gray_code(int i) { return i ^ (i >> 1); }

// The max-log LLRs of demap_f64 (below), bit for bit, for the Gray square QAM of
// qam_points (code_host.cpp) with M points known at compile time.  That constellation's
// label is gray(r) side + gray(a): its first H = log2(side) bits depend on the imaginary
// level b = side - 1 - r only, its last H bits on the real level a only; the real part
// of a point with real level a is pts[2 gray(a)] and the imaginary part of one with
// imaginary level b is pts[2 gray(side - 1 - b) side + 1], the same doubles for every
// point of that level.
// The metric of point i, RN(RN(-ns_i / sigma^2) - ln M) with ns_i = RN(dr_i^2 + di_i^2)
// (each square rounded), does not increase with ns_i, and RN(x + y) does not decrease
// with x or with y.  So the largest metric of a half (the points whose bit o is 0, or 1)
// is the metric of RN(min dr^2 + min di^2), the minima over the half's levels: those of
// bit o's dimension whose Gray code has that bit, and all levels of the other dimension.
// The 2 side squared distances, the half minima of each bit on their bit patterns
// (non-negative doubles order as their bits) and two metrics per bit take 4 side +
// 11 log2 M FP64 instructions per symbol instead of 9 per point (16-QAM: 60 against 148).
template <int M, typename Put>
__device__ __forceinline__ void demap_f64_maxlog(const double* pts, double log_m, double yre, double yim,
                                                 double sigma2, double inv_s2, int n_bits, Put&& put) {
  constexpr int MB = M == 4 ? 2 : (M == 16 ? 4 : (M == 64 ? 6 : 8));
  constexpr int H = MB / 2, SIDE = 1 << H;
  const double uniform = -log_m;
  // hr[2 j + v]: the least squared real distance over the real levels whose Gray code
  // has bit j equal to v; hi[] the same for the imaginary levels (bit patterns)
  unsigned long long hr[2 * H], hi[2 * H];
#pragma unroll
  for (int t = 0; t < 2 * H; t++) hr[t] = hi[t] = ~0ull;
#pragma unroll
  for (int q = 0; q < SIDE; q++) {
    const double dr = __dsub_rn(yre, pts[2 * gray_code(q)]);
    const double di = __dsub_rn(yim, pts[2 * (gray_code(SIDE - 1 - q) * SIDE) + 1]);
    const unsigned long long vr = (unsigned long long)__double_as_longlong(__dmul_rn(dr, dr));
    const unsigned long long vi = (unsigned long long)__double_as_longlong(__dmul_rn(di, di));
#pragma unroll
    for (int j = 0; j < H; j++) {
      const int br = 2 * j + ((gray_code(q) >> j) & 1), bi = 2 * j + ((gray_code(SIDE - 1 - q) >> j) & 1);
      hr[br] = vr < hr[br] ? vr : hr[br];
      hi[bi] = vi < hi[bi] ? vi : hi[bi];
    }
  }
  // the least over all levels of a dimension: either half of any bit
  const unsigned long long gre = hr[0] < hr[1] ? hr[0] : hr[1], gim = hi[0] < hi[1] ? hi[0] : hi[1];
#pragma unroll
  for (int o = 0; o < MB; o++) {
    if (o >= n_bits) break;
    const bool im_bit = o < H;
    const int j = im_bit ? H - 1 - o : MB - 1 - o;  // the bit of gray(r), or of gray(a)
    const unsigned long long h0 = im_bit ? hi[2 * j] : hr[2 * j], h1 = im_bit ? hi[2 * j + 1] : hr[2 * j + 1];
    const double other = __longlong_as_double((long long)(im_bit ? gre : gim));
    const double ns0 = __dadd_rn(__longlong_as_double((long long)h0), other);
    const double ns1 = __dadd_rn(__longlong_as_double((long long)h1), other);
    const double m0 = __dadd_rn(neg_div_by(ns0, sigma2, inv_s2), uniform);
    const double m1 = __dadd_rn(neg_div_by(ns1, sigma2, inv_s2), uniform);
    put(o, __dsub_rn(m0, m1));
  }
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
// Max-log takes demap_f64_maxlog; exact, QPSK and 16-QAM take demap_f64_fixed.  Every
// metric is negative (-ns / sigma^2 - ln M
// with ln M > 0), so the maxima take max_neg; inv_s2 is RN(1 / sigma2) for neg_div_by.
template <typename Put>
__device__ __forceinline__ void demap_f64(const double* pts, int m, int mbits, double log_m, bool exact, double yre,
                                          double yim, double sigma2, double inv_s2, int n_bits, Put&& put) {
  if (!exact) {
    if (m == 4) return demap_f64_maxlog<4>(pts, log_m, yre, yim, sigma2, inv_s2, n_bits, put);
    if (m == 16) return demap_f64_maxlog<16>(pts, log_m, yre, yim, sigma2, inv_s2, n_bits, put);
    if (m == 64) return demap_f64_maxlog<64>(pts, log_m, yre, yim, sigma2, inv_s2, n_bits, put);
    if (m == 256) return demap_f64_maxlog<256>(pts, log_m, yre, yim, sigma2, inv_s2, n_bits, put);
  }
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
