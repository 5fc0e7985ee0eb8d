// Device helpers shared by every decoder, also compiled at run time by NVRTC for the
// graph-specialised decoder (layered_nr.cuh): explicitly rounded arithmetic, the min
// helpers of the row updates, the L2 policy of the check-node state and the block-wide
// syndrome test on packed hard decisions.  No includes but <cstdint> under nvcc.
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#else
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef int int32_t;
typedef unsigned long long uint64_t;
typedef long long int64_t;
typedef unsigned long long uintptr_t;
#endif

namespace cbk {
namespace {

template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b);
template <>
__device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }
template <>
__device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }

// The bit pattern of |x| from that of a double x: the AND as inline PTX, opaque to the
// compiler's recognition of `bits & 0x7fff...` as fabs, whose result it then forms on the
// FP64 pipe when the consumer is an integer comparison
__device__ __forceinline__ long long abs_bits(long long b) {
  long long r;
  asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(r) : "l"(b));
  return r;
}

template <typename T>
__device__ __forceinline__ T infinity();
template <>
__device__ __forceinline__ double infinity<double>() { return __longlong_as_double(0x7ff0000000000000ll); }
template <>
__device__ __forceinline__ float infinity<float>() { return __int_as_float(0x7f800000); }

// ---- syndrome test on packed hard decisions
// post < 0 for the hard decision: in f64 the sign bit (an integer test), since the
// posteriors are never -0.0 or NaN
__device__ __forceinline__ uint32_t is_negative(double v) {
  return (uint32_t)((unsigned long long)__double_as_longlong(v) >> 63);
}
__device__ __forceinline__ uint32_t is_negative(float v) { return (uint32_t)(v < 0.0f); }

// hd holds, per base column j, the hard decisions of its Z bits packed 32 per word
// (ceil(Z/32) words, then one zero word).  The parity of the 32 lifted rows
// [32g, 32g + 32) of layer L is the XOR over the layer's entries (j, s) of the
// Z-bit circular window of column j starting at (32g + s) mod Z.
template <typename T>
__device__ __forceinline__ void build_hard_decisions(const T* post, uint32_t* hd, int ncol, int z, int tid, int nt) {
  const int wz = (z + 31) >> 5, ws = wz + 1;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int task = warp; task < ncol * wz; task += nw) {
    const int j = task / wz, w = task - j * wz;
    const int r = w * 32 + lane;
    const uint32_t word = __ballot_sync(0xffffffffu, r < z && is_negative(post[j * z + r]));
    if (lane == 0) {
      hd[j * ws + w] = word;
      if (w == wz - 1) hd[j * ws + wz] = 0u;
    }
  }
}

// 32 bits of a packed column from bit o (bits at or beyond Z read as 0)
__device__ __forceinline__ uint32_t window32(const uint32_t* col, int o) {
  return __funnelshift_r(col[o >> 5], col[(o >> 5) + 1], o & 31);
}

// Stage 2 of the syndrome test: every row on packed hard decisions.  Block-wide.
template <typename T>
__device__ __forceinline__ bool some_packed_check_fails(const T* post, uint32_t* hd, const uint32_t* ent,
                                                        const uint16_t* lstart, int rows_n, int ncol, int z, int tid,
                                                        int nt) {
  int bad = 0;
  build_hard_decisions(post, hd, ncol, z, tid, nt);
  __syncthreads();
  const int wz = (z + 31) >> 5, ws = wz + 1;
  for (int task = tid; task < rows_n * wz && !bad; task += nt) {
    const int L = task / wz, g = task - L * wz;
    const int r0 = g * 32, nrows = min(32, z - r0);
    uint32_t par = 0;
    for (int t = lstart[L]; t < lstart[L + 1]; t++) {
      const uint32_t en = ent[t];
      const uint32_t* col = hd + (en >> 16) * ws;
      int o = r0 + (int)(en & 0xffffu);
      o -= (o >= z) ? z : 0;
      uint32_t win = window32(col, o);
      if (o + nrows > z) win |= window32(col, 0) << (z - o);
      par ^= win;
    }
    const uint32_t mask = nrows == 32 ? 0xffffffffu : ((1u << nrows) - 1u);
    bad = (par & mask) != 0u;
  }
  return __syncthreads_or(bad) != 0;
}

// Whether some check fails on the hard decisions of post (hard_decisions_are_a_codeword,
// ldpc.rs:555-557).  Block-wide.  Stage 1 reads the rows of the first two layers
// directly (each thread its own row, stopping at the first failure): while the
// decoder has not converged this almost always finds a failing check.  Only when every
// one of those rows is satisfied does stage 2 test all rows on packed hard decisions.
// Either way the answer is exactly "H c != 0".
template <typename T>
__device__ __forceinline__ bool some_check_fails(const T* post, uint32_t* hd, const uint32_t* ent,
                                                 const uint16_t* lstart, int rows_n, int ncol, int z, int tid,
                                                 int nt) {
  int bad = 0;
  if (tid < z) {
    for (int L = 0; L < 2 && !bad; L++) {
      uint32_t par = 0;
      for (int t = lstart[L]; t < lstart[L + 1]; t++) {
        const uint32_t en = ent[t];
        int cc = tid + (int)(en & 0xffffu);
        cc -= (cc >= z) ? z : 0;
        par ^= is_negative(post[(int)(en >> 16) * z + cc]);
      }
      bad = (int)par;
    }
  }
  if (__syncthreads_or(bad)) return true;
  return some_packed_check_fails(post, hd, ent, lstart, rows_n, ncol, z, tid, nt);
}

__device__ __forceinline__ float ld_post(const float* post, int off) {
  return *reinterpret_cast<const float*>(reinterpret_cast<const char*>(post) + off);
}
__device__ __forceinline__ void st_post(float* post, int off, float v) {
  *reinterpret_cast<float*>(reinterpret_cast<char*>(post) + off) = v;
}
// |d| = min(|a|, |b|), sign(d) = sign(a) xor sign(b)
__device__ __forceinline__ float min_xorsign_abs(float a, float b) {
  float d;
  asm("min.xorsign.abs.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// The state records of all resident CTAs (64 MB at BG1 Z = 384) fit in L2, but the LLR
// stream of a launch (830 MB for 8192 codewords) would evict them: the records are read
// and written with an L2 evict-last policy, the LLRs with streaming loads.
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

}  // namespace
}  // namespace cbk
