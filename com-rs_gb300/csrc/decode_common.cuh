// Device helpers shared by the decoders (decode.cu, nms_learned.cu): explicitly rounded
// arithmetic, and the block-wide syndrome test on packed hard decisions.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

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

template <typename T>
__device__ __forceinline__ T infinity();
template <>
__device__ __forceinline__ double infinity<double>() { return __longlong_as_double(0x7ff0000000000000ll); }
template <>
__device__ __forceinline__ float infinity<float>() { return __int_as_float(0x7f800000); }

__device__ __forceinline__ int lifted_col(uint32_t entry, int r, int z) {
  int c = r + (int)(entry & 0xffffu);
  c -= (c >= z) ? z : 0;
  return (int)(entry >> 16) * z + c;
}

// ---- syndrome test on packed hard decisions
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
    const uint32_t word = __ballot_sync(0xffffffffu, r < z && post[j * z + r] < (T)0);
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
        par ^= (uint32_t)(post[(int)(en >> 16) * z + cc] < (T)0);
      }
      bad = (int)par;
    }
  }
  if (__syncthreads_or(bad)) return true;
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

}  // namespace
}  // namespace cbk
