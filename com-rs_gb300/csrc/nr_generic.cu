// The NR code through the generic sparse decoder (the sum-product rule and the flooding
// schedule, which the layered min-sum kernel of decode.cu does not run): the E received
// LLRs become the n_full LLRs of the full word (NrLdpc::full_llr,
// crates/com-fec/src/nr/ldpc.rs:191-197), sparse.cu decodes them, and an epilogue
// writes what decode.cu writes: hard decisions of the K' information bits
// (signal.rs:47-49), their a posteriori LLRs, the iterations and the error counts
// (errors.rs:39-42).
#include <cuda_runtime.h>

#include "decode_common.cuh"
#include "kernels.h"

namespace cbk {
namespace {

constexpr int kThreads = 256;

// one CTA per frame; the same steps as decode.cu's prologue
template <typename T>
__global__ void __launch_bounds__(kThreads) full_llr_kernel(const __grid_constant__ cbd::DevCode c, const T* llr,
                                                            int64_t n_frames, T* full) {
  const int64_t f = blockIdx.x;
  if (f >= n_frames) return;
  const T* in = llr + (size_t)f * c.e;
  T* out = full + (size_t)f * c.n_full;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int v = tid; v < c.n_full; v += nt) out[v] = (T)0;
  __syncthreads();
  if (c.map_is_offset) {
    for (int t = tid; t < c.e; t += nt) out[2 * c.z + t] = add_rn((T)0, in[t]);
  } else if (!c.has_repeats) {
    for (int t = tid; t < c.e; t += nt) out[c.map[t]] = add_rn((T)0, in[t]);
  } else {
    for (int v = tid; v < c.n_full; v += nt) {
      const int b0 = c.inv_start[v], b1 = c.inv_start[v + 1];
      if (b0 == b1) continue;
      T s = (T)0;
      for (int i = b0; i < b1; i++) s = add_rn(s, in[c.inv_t[i]]);
      out[v] = s;
    }
  }
  __syncthreads();
  for (int v = c.k_info + tid; v < c.k; v += nt) out[v] = (T)cbd::kKnownBitLlr;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) nr_epilogue_kernel(const __grid_constant__ NrEpilogueArgs<T> a) {
  const int64_t f = blockIdx.x;
  if (f >= a.n_frames) return;
  const T* post = a.post + (size_t)f * a.n_full;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int wpf = (a.k_info + 31) >> 5;
  __shared__ unsigned int s_err;
  if (tid == 0) s_err = 0;
  __syncthreads();
  unsigned int be = 0;
  for (int b0 = warp * 32; b0 < a.k_info; b0 += nw * 32) {
    const int v = b0 + lane;
    const uint32_t word = __ballot_sync(0xffffffffu, v < a.k_info && post[v] < (T)0);
    if (lane == 0) {
      const size_t w = (size_t)f * wpf + (b0 >> 5);
      if (a.bits_out) a.bits_out[w] = word;
      if (a.ref_bits) be += __popc(word ^ a.ref_bits[w]);
    }
  }
  if (a.app_out)
    for (int v = tid; v < a.k_info; v += blockDim.x) a.app_out[(size_t)f * a.k_info + v] = post[v];
  if (be) atomicAdd(&s_err, be);
  __syncthreads();
  if (tid == 0) {
    const int it = a.iters_in[f];
    if (a.iters_out) a.iters_out[f] = it;
    if (a.results) {
      cbd::FrameResult r;
      r.bit_errors = s_err;
      r.frame_error = s_err > 0;
      r.iterations = (uint8_t)it;
      r.reserved = 0;
      a.results[f] = r;
    }
  }
}

}  // namespace

template <typename T>
cudaError_t launch_full_llr(const cbd::DevCode& c, const T* llr, int64_t n_frames, T* full, cudaStream_t s) {
  if (n_frames <= 0) return cudaSuccess;
  full_llr_kernel<T><<<(unsigned)n_frames, kThreads, 0, s>>>(c, llr, n_frames, full);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_nr_epilogue(const NrEpilogueArgs<T>& a, cudaStream_t s) {
  if (a.n_frames <= 0) return cudaSuccess;
  nr_epilogue_kernel<T><<<(unsigned)a.n_frames, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_full_llr<double>(const cbd::DevCode&, const double*, int64_t, double*, cudaStream_t);
template cudaError_t launch_full_llr<float>(const cbd::DevCode&, const float*, int64_t, float*, cudaStream_t);
template cudaError_t launch_nr_epilogue<double>(const NrEpilogueArgs<double>&, cudaStream_t);
template cudaError_t launch_nr_epilogue<float>(const NrEpilogueArgs<float>&, cudaStream_t);

}  // namespace cbk
