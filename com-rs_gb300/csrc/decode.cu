// Layered normalised/offset min-sum decoding of 5G NR LDPC codewords on the GPU.
//
// Restates LdpcCode::propagate and check_message (crates/com-fec/src/ldpc.rs:449-557)
// for the lifted NR graphs of crates/com-fec/src/nr/ldpc.rs:124-134, with the LLR
// placement of NrLdpc::full_llr (nr/ldpc.rs:191-197).
//
// Parallel form: a layer is one base-graph row; its Z lifted rows touch disjoint
// variables (each base entry is a Z x Z circulant permutation and a base row holds each
// column once), so processing the Z rows of a layer at once performs exactly the
// reference's sequential row order.  Thread r of a CTA owns lifted row (layer, r);
// the rows of the next layer start after a barrier.
//
// Data layout per codeword:
//   * posteriors post[n_full] in shared memory (T = double or float);
//   * check-to-variable messages compressed per lifted row: the two output
//     magnitudes (scale or offset already applied), the index of the minimum and the
//     sign bit of every outgoing message.  The min-sum output of a row is a function of
//     these alone (ldpc.rs:468-490), so the compression is exact, -0.0 included.  The
//     state of a CTA lives in its own global slot, reused across its codewords (a
//     persistent, work-stealing grid), so it stays resident in L2.
//
// Exactness: every arithmetic step is an explicitly rounded IEEE operation in the
// reference's order (incoming = post - c2v, o = s * (alpha * mag), post = incoming + o),
// the sign tests are `x < 0` (so -0.0 counts as positive), min/argmin use strict `<`.
// In f64 the posteriors, hard decisions and iteration counts are those of the
// reference bit for bit; in f32 they are those of the same algorithm in f32.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "kernels.h"

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

// Whether some check of the codeword fails on the hard decisions of post
// (hard_decisions_are_a_codeword, ldpc.rs:555-557).  Block-wide.
template <typename T>
__device__ __forceinline__ bool some_check_fails(const cbd::DevCode& c, const T* post, int tid) {
  int bad = 0;
  if (tid < c.z) {
    for (int L = 0; L < c.rows_n && !bad; L++) {
      int par = 0;
      for (int t = c.layer_start[L]; t < c.layer_start[L + 1]; t++)
        par ^= (int)(post[lifted_col(c.entry[t], tid, c.z)] < (T)0);
      bad = par;
    }
  }
  return __syncthreads_or(bad) != 0;
}

// One lifted row of a layer: thread r, degree D known at compile time.
// old state (a1, a2, mt) -> new state (n1, n2, nm); post updated in place.
template <typename T, int D>
__device__ __forceinline__ void row_update(T* __restrict__ post, const uint32_t* __restrict__ ent, int r, int z,
                                           T a1, T a2, uint32_t mt, int rule, T alpha, T& n1, T& n2,
                                           uint32_t& nm) {
  int off[D];
  T x[D];
  const int old_i1 = (int)(mt & 31u);
#pragma unroll
  for (int e = 0; e < D; e++) {
    const uint32_t en = ent[e];
    // (r + shift) mod Z with one unsigned min: r + shift < 2Z
    unsigned c = (unsigned)r + (en & 0xffffu);
    unsigned cm = c - (unsigned)z;
    off[e] = (int)(en >> 16) * z + (int)min(c, cm);
    T mag = (e == old_i1) ? a2 : a1;
    T old = ((mt >> (8 + e)) & 1u) ? -mag : mag;
    x[e] = sub_rn(post[off[e]], old);
  }
  // check_message, min-sum branch (ldpc.rs:468-491): sign product with `l < 0`, strict
  // `<` for the minimum and its index, min(m2, a) for the second (equal for non-NaN,
  // and a NaN is skipped by both)
  uint32_t par = (uint32_t)(x[0] < (T)0);
  T m1 = fmin(fabs(x[0]), infinity<T>()), m2 = infinity<T>();
  int i1 = 0;
#pragma unroll
  for (int e = 1; e < D; e++) {
    par ^= (uint32_t)(x[e] < (T)0);
    T av = fabs(x[e]);
    bool lt = av < m1;
    m2 = lt ? m1 : fmin(m2, av);
    m1 = lt ? av : m1;
    i1 = lt ? e : i1;
  }
  if (rule == cbd::RULE_NMS) {
    n1 = mul_rn(alpha, m1);
    n2 = mul_rn(alpha, m2);
  } else {
    n1 = fmax(sub_rn(m1, alpha), (T)0);
    n2 = fmax(sub_rn(m2, alpha), (T)0);
  }
  nm = (uint32_t)i1;
#pragma unroll
  for (int e = 0; e < D; e++) {
    uint32_t ng = par ^ (uint32_t)(x[e] < (T)0);
    T mag = (e == i1) ? n2 : n1;
    T o = ng ? -mag : mag;
    post[off[e]] = add_rn(x[e], o);
    nm |= ng << (8 + e);
  }
}

template <typename T>
__device__ __forceinline__ void row_dispatch(int d, T* post, const uint32_t* ent, int r, int z, T a1, T a2,
                                             uint32_t mt, int rule, T alpha, T& n1, T& n2, uint32_t& nm) {
  switch (d) {
    case 3: row_update<T, 3>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 4: row_update<T, 4>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 5: row_update<T, 5>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 6: row_update<T, 6>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 7: row_update<T, 7>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 8: row_update<T, 8>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 9: row_update<T, 9>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    case 10: row_update<T, 10>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    default: row_update<T, 19>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
  }
}

template <typename T>
__global__ void __launch_bounds__(384) layered_kernel(const __grid_constant__ DecodeArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* post = reinterpret_cast<T*>(smem);
  __shared__ long long s_cw;
  __shared__ unsigned int s_err;
  const cbd::DevCode& c = a.code;
  const int z = c.z, nt = blockDim.x, tid = threadIdx.x;
  const int rows = c.rows_n * z;
  const size_t slot = ((size_t)rows * (2 * sizeof(T) + 4) + 255) & ~(size_t)255;
  unsigned char* base = reinterpret_cast<unsigned char*>(a.state) + (size_t)blockIdx.x * slot;
  T* A1 = reinterpret_cast<T*>(base);
  T* A2 = A1 + rows;
  uint32_t* meta = reinterpret_cast<uint32_t*>(A2 + rows);
  const T alpha = (T)a.cfg.alpha;
  const int rule = a.cfg.rule;
  const int max_it = a.cfg.max_iterations;
  const int wpf = (c.k_info + 31) >> 5;
  const bool active = tid < z;

  for (;;) {
    if (tid == 0) {
      s_cw = (long long)atomicAdd(reinterpret_cast<unsigned long long*>(a.work_counter), 1ull);
      s_err = 0;
    }
    __syncthreads();
    const long long cw = s_cw;
    if (cw >= a.n_frames) break;

    // ---- channel LLRs of the full word (NrLdpc::full_llr)
    const T* llr = a.llr + (size_t)cw * c.e;
    for (int v = tid; v < c.n_full; v += nt) post[v] = (T)0;
    __syncthreads();
    if (c.map_is_offset) {
      for (int t = tid; t < c.e; t += nt) post[2 * z + t] = add_rn((T)0, llr[t]);
    } else if (!c.has_repeats) {
      for (int t = tid; t < c.e; t += nt) post[c.map[t]] = add_rn((T)0, llr[t]);
    } else {
      for (int v = tid; v < c.n_full; v += nt) {
        int b0 = c.inv_start[v], b1 = c.inv_start[v + 1];
        if (b0 == b1) continue;
        T s = (T)0;
        for (int i = b0; i < b1; i++) s = add_rn(s, llr[c.inv_t[i]]);
        post[v] = s;
      }
    }
    __syncthreads();
    for (int v = c.k_info + tid; v < c.k; v += nt) post[v] = (T)cbd::kKnownBitLlr;
    __syncthreads();

    // ---- propagate (ldpc.rs:509-551), layered schedule
    int it = 0;
    if (some_check_fails(c, post, tid)) {
      it = max_it;
      for (int iter = 1; iter <= max_it; iter++) {
        // the state of a layer is prefetched one layer ahead
        T a1 = (T)0, a2 = (T)0;
        uint32_t mt = 0;
        if (iter > 1 && active) {
          a1 = A1[tid];
          a2 = A2[tid];
          mt = meta[tid];
        }
        for (int L = 0; L < c.rows_n; L++) {
          T p1 = (T)0, p2 = (T)0;
          uint32_t pm = 0;
          if (iter > 1 && active && L + 1 < c.rows_n) {
            const int nrow = (L + 1) * z + tid;
            p1 = A1[nrow];
            p2 = A2[nrow];
            pm = meta[nrow];
          }
          if (active) {
            const int s0 = c.layer_start[L];
            const int d = c.layer_start[L + 1] - s0;
            T n1, n2;
            uint32_t nm;
            row_dispatch<T>(d, post, c.entry + s0, tid, z, a1, a2, mt, rule, alpha, n1, n2, nm);
            const int row = L * z + tid;
            A1[row] = n1;
            A2[row] = n2;
            meta[row] = nm;
          }
          a1 = p1;
          a2 = p2;
          mt = pm;
          __syncthreads();
        }
        if (!some_check_fails(c, post, tid)) {
          it = iter;
          break;
        }
      }
    }

    // ---- outputs: hard decisions (signal.rs:47-49), counts (errors.rs:39-42)
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    unsigned int be = 0;
    for (int b0 = warp * 32; b0 < c.k_info; b0 += nw * 32) {
      int v = b0 + lane;
      bool bit = v < c.k_info && post[v] < (T)0;
      uint32_t word = __ballot_sync(0xffffffffu, bit);
      if (lane == 0) {
        size_t w = (size_t)cw * wpf + (b0 >> 5);
        if (a.bits_out) a.bits_out[w] = word;
        if (a.ref_bits) be += __popc(word ^ a.ref_bits[w]);
      }
    }
    if (a.app_out)
      for (int v = tid; v < c.k_info; v += nt) a.app_out[(size_t)cw * c.k_info + v] = post[v];
    if (a.post_out)
      for (int v = tid; v < c.n_full; v += nt) a.post_out[(size_t)cw * c.n_full + v] = post[v];
    if (be) atomicAdd(&s_err, be);
    __syncthreads();
    if (tid == 0) {
      if (a.iters_out) a.iters_out[cw] = it;
      if (a.results) {
        cbd::FrameResult r;
        r.bit_errors = s_err;
        r.frame_error = s_err > 0;
        r.iterations = (uint8_t)it;
        r.reserved = 0;
        a.results[cw] = r;
      }
    }
    __syncthreads();
  }
}

template <typename T>
void* kernel_for(int max_degree) {
  (void)max_degree;
  return (void*)layered_kernel<T>;
}

int block_threads(int z) { return ((z + 31) / 32) * 32; }

size_t smem_bytes(const cbd::DevCode& c, int precision) {
  return (size_t)c.n_full * (precision == 0 ? sizeof(double) : sizeof(float));
}

}  // namespace

size_t decode_state_bytes_per_slot(const cbd::DevCode& c, int precision) {
  size_t t = precision == 0 ? sizeof(double) : sizeof(float);
  return (((size_t)c.rows_n * c.z * (2 * t + 4)) + 255) & ~(size_t)255;
}

int decode_grid_size(const cbd::DevCode& c, int precision, int device) {
  void* k = precision == 0 ? kernel_for<double>(c.max_degree) : kernel_for<float>(c.max_degree);
  size_t smem = smem_bytes(c, precision);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block_threads(c.z), smem);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return per_sm * sms;
}

template <typename T>
cudaError_t launch_decode(const DecodeArgs<T>& a, int grid, cudaStream_t stream) {
  const int precision = sizeof(T) == 8 ? 0 : 1;
  void* k = kernel_for<T>(a.code.max_degree);
  size_t smem = smem_bytes(a.code, precision);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3(grid), dim3(block_threads(a.code.z)), args, smem, stream);
}

template cudaError_t launch_decode<double>(const DecodeArgs<double>&, int, cudaStream_t);
template cudaError_t launch_decode<float>(const DecodeArgs<float>&, int, cudaStream_t);

}  // namespace cbk
