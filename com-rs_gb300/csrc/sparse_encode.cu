// Systematic encoders of generic sparse LDPC codes: LdpcCode::encode_block
// (crates/com-fec/src/ldpc.rs:753-791) for the Sums encoder of LdpcCode::from_rows and
// the Accumulate encoder of LdpcCode::accumulate.  One CTA per frame (grid-stride over
// the frames); the frame's information bits are packed 32 to a word in shared memory.
#include <algorithm>

#include "kernels.h"

namespace cbk {
namespace {

constexpr int kSumsThreads = 256;
constexpr int kAccThreads = 512;
constexpr int kMaxGrid = 4096;

// bit i % 32 of word i / 32 = bit 0 of u[i], by one ballot per warp and word
__device__ __forceinline__ void pack_info(const uint8_t* u, int k, uint32_t* s_u) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int words = (k + 31) / 32;
  for (int w = warp; w < words; w += nw) {
    const int i = w * 32 + lane;
    const uint32_t b = __ballot_sync(0xffffffffu, i < k && (u[i] & 1));
    if (lane == 0) s_u[w] = b;
  }
}

// the information bits at their positions; parity bit t = the parity of the AND of its
// row of the reduced H with the packed information word
__global__ void __launch_bounds__(kSumsThreads) sums_encode_kernel(SumsEncodeArgs a) {
  extern __shared__ uint32_t s_u[];
  for (int64_t f = blockIdx.x; f < a.n_frames; f += gridDim.x) {
    const uint8_t* u = a.info + f * a.k;
    uint8_t* c = a.coded + f * a.n;
    pack_info(u, a.k, s_u);
    __syncthreads();
    for (int i = threadIdx.x; i < a.k; i += blockDim.x) c[a.info_pos[i]] = (s_u[i >> 5] >> (i & 31)) & 1;
    for (int t = threadIdx.x; t < a.rank; t += blockDim.x) {
      uint32_t acc = 0;
      for (int w = 0; w < a.words; w++) acc ^= __ldg(a.pmat + (size_t)w * a.rank + t) & s_u[w];
      c[a.pivots[t]] = (uint8_t)(__popc(acc) & 1);
    }
    __syncthreads();
  }
}

// s_r = the sum of the information bits of check r; parity bit k + r = s_0 + ... + s_r,
// a prefix XOR: every thread sums a run of consecutive checks, the runs' sums are
// scanned across the CTA, then every thread writes its run
__global__ void __launch_bounds__(kAccThreads) accumulate_encode_kernel(AccumulateEncodeArgs a) {
  extern __shared__ uint32_t s_mem[];
  __shared__ uint32_t s_warp[kAccThreads / 32];
  const int words = (a.k + 31) / 32;
  uint32_t* s_u = s_mem;
  uint8_t* s_s = reinterpret_cast<uint8_t*>(s_mem + words);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int run = (a.m + blockDim.x - 1) / blockDim.x;
  const int r0 = min(a.m, (int)threadIdx.x * run), r1 = min(a.m, r0 + run);
  for (int64_t f = blockIdx.x; f < a.n_frames; f += gridDim.x) {
    const uint8_t* u = a.info + f * a.k;
    uint8_t* c = a.coded + f * a.n;
    pack_info(u, a.k, s_u);
    for (int i = threadIdx.x; i < a.k; i += blockDim.x) c[i] = u[i] & 1;
    __syncthreads();
    for (int r = threadIdx.x; r < a.m; r += blockDim.x) {
      uint32_t s = 0;
      for (int e = a.row_start[r]; e < a.row_start[r + 1]; e++) {
        const int v = a.vars[e];
        if (v < a.k) s ^= s_u[v >> 5] >> (v & 31);
      }
      s_s[r] = (uint8_t)(s & 1);
    }
    __syncthreads();
    uint32_t x = 0;
    for (int r = r0; r < r1; r++) x ^= s_s[r];
    uint32_t incl = x;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl ^= y;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t v = lane < nw ? s_warp[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v ^= y;
      }
      if (lane < nw) s_warp[lane] = v;
    }
    __syncthreads();
    uint32_t p = (incl ^ x) ^ (warp > 0 ? s_warp[warp - 1] : 0u);
    for (int r = r0; r < r1; r++) {
      p ^= s_s[r];
      c[a.k + r] = (uint8_t)p;
    }
    __syncthreads();
  }
}

int grid_for(int64_t n_frames) { return (int)std::min<int64_t>(n_frames, kMaxGrid); }

}  // namespace

size_t sums_encode_smem(int words) { return (size_t)words * 4; }

size_t accumulate_encode_smem(int k, int m) { return (size_t)(k + 31) / 32 * 4 + (size_t)m; }

cudaError_t launch_sums_encode(const SumsEncodeArgs& a, cudaStream_t stream) {
  if (a.n_frames <= 0) return cudaSuccess;
  const size_t smem = sums_encode_smem(a.words);
  cudaError_t e = cudaFuncSetAttribute(sums_encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  sums_encode_kernel<<<grid_for(a.n_frames), kSumsThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_accumulate_encode(const AccumulateEncodeArgs& a, cudaStream_t stream) {
  if (a.n_frames <= 0) return cudaSuccess;
  const size_t smem = accumulate_encode_smem(a.k, a.m);
  cudaError_t e =
      cudaFuncSetAttribute(accumulate_encode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  accumulate_encode_kernel<<<grid_for(a.n_frames), kAccThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace cbk
