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

#include "decode_common.cuh"
#include "kernels.h"

namespace cbk {
namespace {

template <typename T>
__host__ __device__ __forceinline__ size_t slot_bytes(int rows) {
  return (StateSlot<T>::bytes(rows) + 255) & ~(size_t)255;
}

template <typename T>
__host__ __device__ __forceinline__ size_t decode_smem_bytes(int n_full, int z, int rows_n, int n_entries) {
  const int ws = (z + 31) / 32 + 1;
  size_t b = (size_t)n_full * sizeof(T);
  b += (size_t)(n_full / z) * ws * 4;    // packed hard decisions
  b += (size_t)n_entries * 4;             // entries
  b += (size_t)(rows_n + 1) * 2 + 16;     // layer starts
  return (b + 15) & ~(size_t)15;
}

// Weights of the learned min-sum (f32 only): none (the plain decoder), in global memory,
// in the launch parameters, or each iteration's staged in shared memory
enum LearnedWeights { kPlain = 0, kWeightsGlobal = 1, kWeightsParam = 2, kWeightsShared = 3 };

// One layered iteration of decode_body: the rows in schedule order, each row's state from
// the previous iteration (L2-resident: loaded where it is used), a barrier after each level.
template <typename T, int LW, int RULE>
__device__ __forceinline__ void decode_layers(const cbd::DevCode& c, T* post, const StateSlot<T>& st,
                                              const LearnedRowW& lw, int iter, int tid, int z, bool active,
                                              T alpha) {
  for (int q = 0; q < c.rows_n; q++) {
    const int L = c.layer_order[q];
    T a1 = (T)0, a2 = (T)0;
    uint32_t mt = 0;
    if (iter > 1 && active) st.load(L * z + tid, a1, a2, mt);
    if (active) {
      const int s0 = c.layer_start[L];
      const int d = c.layer_start[L + 1] - s0;
      T n1, n2;
      uint32_t nm;
      if constexpr (LW != kPlain)
        row_dispatch_learned(d, post, EdgeAddrTable{c.eaddr + s0, tid, 4 * tid, 4 * z},
                             LearnedRowW{lw.a_prev, lw.b_prev, lw.a_cur, lw.b_cur, s0, lw.stride, lw.roff}, iter - 1,
                             iter == 1, a1, a2, mt, n1, n2, nm);
      else if constexpr (sizeof(T) == 4)
        row_dispatch_lean<RULE>(d, post, EdgeAddrTable{c.eaddr + s0, tid, 4 * tid, 4 * z}, a1, a2, mt, alpha, n1, n2,
                                nm);
      else
        row_dispatch<T, RULE>(d, post, c.entry + s0, tid, z, a1, a2, mt, alpha, n1, n2, nm);
      st.store(L * z + tid, n1, n2, nm);
    }
    if (c.level_end[q]) __syncthreads();
  }
}

template <typename T, int LW>
__device__ __forceinline__ void decode_body(const DecodeArgs<T>& a, const float* la, const float* lb) {
  constexpr bool LEARNED = LW != kPlain;
  extern __shared__ __align__(16) unsigned char smem[];
  const cbd::DevCode& c = a.code;
  const int z = c.z, nt = blockDim.x, tid = threadIdx.x;
  const int ncol = c.n_full / z;
  const int ws = (z + 31) / 32 + 1;
  T* post = reinterpret_cast<T*>(smem);
  uint32_t* hd = reinterpret_cast<uint32_t*>(post + c.n_full);
  uint32_t* s_ent = hd + ncol * ws;
  uint16_t* s_lstart = reinterpret_cast<uint16_t*>(s_ent + c.n_entries);
  __shared__ long long s_cw;
  __shared__ unsigned int s_err;
  const int rows = c.rows_n * z;
  const StateSlot<T> st(reinterpret_cast<unsigned char*>(a.state) + (size_t)blockIdx.x * slot_bytes<T>(rows), rows);
  const T alpha = (T)a.cfg.alpha;
  const int rule = a.cfg.rule;
  const int max_it = a.cfg.max_iterations;
  const int wpf = (c.k_info + 31) >> 5;
  const bool active = tid < z;
  for (int i = tid; i < c.n_entries; i += nt) s_ent[i] = c.entry[i];
  for (int i = tid; i <= c.rows_n; i += nt) s_lstart[i] = c.layer_start[i];

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
      if (sizeof(T) == 4 && (c.e & 3) == 0 && (reinterpret_cast<uintptr_t>(a.llr) & 15) == 0) {
        // 128-bit streaming loads: a 16-byte aligned buffer with E % 4 == 0 keeps every
        // frame's row 16-byte aligned (any other buffer takes the 32-bit loads below)
        const float4* l4 = reinterpret_cast<const float4*>(llr);
        for (int q = tid; q < (c.e >> 2); q += nt) {
          const float4 v = __ldcs(l4 + q);
          T* d = post + 2 * z + 4 * q;
          d[0] = add_rn((T)0, (T)v.x);
          d[1] = add_rn((T)0, (T)v.y);
          d[2] = add_rn((T)0, (T)v.z);
          d[3] = add_rn((T)0, (T)v.w);
        }
      } else {
        for (int t = tid; t < c.e; t += nt) post[2 * z + t] = add_rn((T)0, __ldcs(llr + t));
      }
    } else if (!c.has_repeats) {
      for (int t = tid; t < c.e; t += nt) post[c.map[t]] = add_rn((T)0, __ldcs(llr + t));
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
    if (some_check_fails(post, hd, s_ent, s_lstart, c.rows_n, ncol, z, tid, nt)) {
      it = max_it;
      for (int iter = 1; iter <= max_it; iter++) {
        // learned weights of iterations iter - 2 (old messages) and iter - 1
        const float *w_ap = nullptr, *w_bp = nullptr, *w_ac = nullptr, *w_bc = nullptr;
        int w_stride = 1, w_roff = 0;
        if constexpr (LEARNED) {
          const int t = iter - 1, ne = c.n_entries;
          if constexpr (LW == kWeightsShared) {
            float* sw = reinterpret_cast<float*>(smem + decode_smem_bytes<T>(c.n_full, z, c.rows_n, c.n_entries));
            float* cur = sw + (t & 1) * 2 * ne;
            for (int i = tid; i < ne; i += nt) {
              cur[i] = la[(size_t)t * ne + i];
              cur[ne + i] = lb[(size_t)t * ne + i];
            }
            __syncthreads();
            w_ac = cur;
            w_bc = cur + ne;
            w_ap = sw + ((t + 1) & 1) * 2 * ne;
            w_bp = w_ap + ne;
          } else {
            const size_t per = a.l_shared ? (size_t)ne : (size_t)ne * z;
            w_ac = la + (size_t)t * per;
            w_bc = lb + (size_t)t * per;
            w_ap = t > 0 ? w_ac - per : w_ac;
            w_bp = t > 0 ? w_bc - per : w_bc;
            if (!a.l_shared) {
              w_stride = z;
              w_roff = tid;
            }
          }
        }
        // the rows of one iteration, the rule a template parameter (one branch around the
        // whole iteration, none in the rows)
        const LearnedRowW lw{w_ap, w_bp, w_ac, w_bc, 0, w_stride, w_roff};
        if (LEARNED || rule == cbd::RULE_NMS)
          decode_layers<T, LW, cbd::RULE_NMS>(c, post, st, lw, iter, tid, z, active, alpha);
        else
          decode_layers<T, LW, cbd::RULE_OMS>(c, post, st, lw, iter, tid, z, active, alpha);
        if (!some_check_fails(post, hd, s_ent, s_lstart, c.rows_n, ncol, z, tid, nt)) {
          it = iter;
          break;
        }
      }
    }

    // ---- outputs: hard decisions (signal.rs:47-49), counts (errors.rs:39-42).  The words
    // of decisions are staged in hd (free after the syndrome test) and written 16 bytes at
    // a time when the row of words allows it.
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    // the sent words, one per thread, loaded before the ballots so that their latency
    // overlaps them
    const uint32_t* ref = a.ref_bits ? a.ref_bits + (size_t)cw * wpf : nullptr;
    const uint32_t ref_w = (ref && tid < wpf) ? ref[tid] : 0u;
    for (int b0 = warp * 32; b0 < c.k_info; b0 += nw * 32) {
      int v = b0 + lane;
      bool bit = v < c.k_info && post[v] < (T)0;
      uint32_t word = __ballot_sync(0xffffffffu, bit);
      if (lane == 0) hd[b0 >> 5] = word;
    }
    __syncthreads();
    unsigned int be = 0;
    if (ref) {
      if (tid < wpf) be = __popc(hd[tid] ^ ref_w);
      for (int w = tid + nt; w < wpf; w += nt) be += __popc(hd[w] ^ ref[w]);
    }
    if (a.bits_out) {
      uint32_t* dst = a.bits_out + (size_t)cw * wpf;
      if ((wpf & 3) == 0 && (reinterpret_cast<uintptr_t>(a.bits_out) & 15) == 0) {
        for (int q = tid; q < (wpf >> 2); q += nt) reinterpret_cast<uint4*>(dst)[q] = reinterpret_cast<const uint4*>(hd)[q];
      } else {
        for (int w = tid; w < wpf; w += nt) dst[w] = hd[w];
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

template <typename T, int LW>
__global__ void __launch_bounds__(384, sizeof(T) == 4 ? 2 : 1) layered_kernel(const __grid_constant__ DecodeArgs<T> a) {
  decode_body<T, LW>(a, a.l_alpha, a.l_beta);
}

__global__ void __launch_bounds__(384, 2) layered_learned_param_kernel(const __grid_constant__ LearnedParamArgs a) {
  decode_body<float, kWeightsParam>(a.d, a.alpha, a.beta);
}

template <typename T>
void* kernel_for(const DecodeArgs<T>& a) {
  if constexpr (sizeof(T) == 4) {
    if (a.l_alpha) return a.l_smem ? (void*)layered_kernel<T, kWeightsShared> : (void*)layered_kernel<T, kWeightsGlobal>;
  }
  return (void*)layered_kernel<T, kPlain>;
}

int block_threads(int z) { return ((z + 31) / 32) * 32; }

size_t smem_bytes(const cbd::DevCode& c, int precision) {
  return precision == 0 ? decode_smem_bytes<double>(c.n_full, c.z, c.rows_n, c.n_entries)
                        : decode_smem_bytes<float>(c.n_full, c.z, c.rows_n, c.n_entries);
}

}  // namespace

size_t decode_state_bytes_per_slot(const cbd::DevCode& c, int precision) {
  const int rows = c.rows_n * c.z;
  return precision == 0 ? slot_bytes<double>(rows) : slot_bytes<float>(rows);
}

int decode_grid_size(const cbd::DevCode& c, int precision, int device) {
  void* k = precision == 0 ? (void*)layered_kernel<double, kPlain> : (void*)layered_kernel<float, kPlain>;
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
  void* k = kernel_for<T>(a);
  size_t smem = smem_bytes(a.code, precision) + (a.l_smem ? (size_t)4 * 4 * a.code.n_entries : 0);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3(grid), dim3(block_threads(a.code.z)), args, smem, stream);
}

cudaError_t launch_decode_learned_param(const LearnedParamArgs& a, int grid, cudaStream_t stream) {
  void* k = (void*)layered_learned_param_kernel;
  size_t smem = smem_bytes(a.d.code, 1);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3(grid), dim3(block_threads(a.d.code.z)), args, smem, stream);
}

template cudaError_t launch_decode<double>(const DecodeArgs<double>&, int, cudaStream_t);
template cudaError_t launch_decode<float>(const DecodeArgs<float>&, int, cudaStream_t);

}  // namespace cbk
