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

// f32 row update with fewer integer-pipe operations (same results as row_update for
// finite LLRs):
//   * min and second min with min/max only; the edges that receive the second minimum
//     are those whose magnitude equals the minimum (if several do, the two minima are
//     equal, so every edge gets the same magnitude, as in the reference);
//   * the sign test `x < 0` is the sign bit of x: the posteriors never hold -0.0 (they
//     start as 0.0 + LLR or 30.0, and a difference or sum is -0.0 only when an operand
//     already is), so no message input x = post - c2v is -0.0 either;
//   * outgoing signs are applied and collected with bit operations.
// State word: bits 0-4 an edge holding the second minimum, bits 8.. the outgoing sign of
// edge e at bit 8 + (D - 1 - e).
template <int D>
__device__ __forceinline__ void row_update_lean(float* __restrict__ post, const uint32_t* __restrict__ ent, int r,
                                                int z, float a1, float a2, uint32_t mt, int rule, float alpha,
                                                float& n1, float& n2, uint32_t& nm) {
  int off[D];
  float x[D];
  const int old_i1 = (int)(mt & 31u);
  const uint32_t t0 = mt << (24 - D);  // the old sign of edge 0 at bit 31
#pragma unroll
  for (int e = 0; e < D; e++) {
    const uint32_t en = ent[e];
    unsigned c = (unsigned)r + (en & 0xffffu);
    unsigned cm = c - (unsigned)z;
    off[e] = (int)(en >> 16) * z + (int)min(c, cm);
    float mag = (e == old_i1) ? a2 : a1;
    uint32_t ob = __float_as_uint(mag) | ((t0 << e) & 0x80000000u);
    x[e] = __fsub_rn(post[off[e]], __uint_as_float(ob));
  }
  uint32_t par = 0;
  float m1 = infinity<float>(), m2 = infinity<float>();
#pragma unroll
  for (int e = 0; e < D; e++) {
    par ^= __float_as_uint(x[e]);
    float av = fabsf(x[e]);
    m2 = fminf(m2, fmaxf(m1, av));
    m1 = fminf(m1, av);
  }
  if (rule == cbd::RULE_NMS) {
    n1 = __fmul_rn(alpha, m1);
    n2 = __fmul_rn(alpha, m2);
  } else {
    n1 = fmaxf(__fsub_rn(m1, alpha), 0.0f);
    n2 = fmaxf(__fsub_rn(m2, alpha), 0.0f);
  }
  const uint32_t ps = par & 0x80000000u;
  const uint32_t n1p = __float_as_uint(n1) | ps, n2p = __float_as_uint(n2) | ps;
  uint32_t sm = 0;
  int i1 = 0;
#pragma unroll
  for (int e = 0; e < D; e++) {
    bool eq = fabsf(x[e]) == m1;
    uint32_t magp = eq ? n2p : n1p;
    i1 = eq ? e : i1;
    uint32_t ob = magp ^ (__float_as_uint(x[e]) & 0x80000000u);
    post[off[e]] = __fadd_rn(x[e], __uint_as_float(ob));
    sm = (sm << 1) | (ob >> 31);
  }
  nm = (sm << 8) | (uint32_t)i1;
}

template <typename T>
__device__ __forceinline__ void row_dispatch(int d, T* post, const uint32_t* ent, int r, int z, T a1, T a2,
                                             uint32_t mt, int rule, T alpha, T& n1, T& n2, uint32_t& nm) {
#ifndef CB_F32_CLASSIC_ROWS
  if constexpr (sizeof(T) == 4) {
    switch (d) {
      case 3: row_update_lean<3>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 4: row_update_lean<4>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 5: row_update_lean<5>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 6: row_update_lean<6>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 7: row_update_lean<7>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 8: row_update_lean<8>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 9: row_update_lean<9>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      case 10: row_update_lean<10>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
      default: row_update_lean<19>(post, ent, r, z, a1, a2, mt, rule, alpha, n1, n2, nm); break;
    }
    return;
  }
#endif
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

// check-node state of one lifted row: f32 as one 16-byte record {n1, n2, meta, 0};
// f64 as a 16-byte {n1, n2} record plus a separate plane of meta words
template <typename T>
struct StateSlot;
// The state records of all resident CTAs (86 MB at BG1 Z = 384) fit in L2, but the LLR
// stream of a launch (830 MB for 8192 codewords) would evict them: the records are read
// and written with an L2 evict-last policy, the LLRs with streaming loads.
__device__ __forceinline__ uint64_t l2_evict_last_policy() {
  uint64_t pol;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}

template <>
struct StateSlot<float> {
  uint4* rec;
  uint64_t pol;
  __device__ __forceinline__ StateSlot(unsigned char* base, int rows)
      : rec(reinterpret_cast<uint4*>(base)), pol(l2_evict_last_policy()) {
    (void)rows;
  }
  __device__ __forceinline__ void load(int row, float& a1, float& a2, uint32_t& mt) const {
    uint32_t x, y, zz, w;
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(x), "=r"(y), "=r"(zz), "=r"(w)
                 : "l"(rec + row), "l"(pol));
    (void)w;
    a1 = __uint_as_float(x);
    a2 = __uint_as_float(y);
    mt = zz;
  }
  __device__ __forceinline__ void store(int row, float n1, float n2, uint32_t nm) const {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(rec + row),
                 "r"(__float_as_uint(n1)), "r"(__float_as_uint(n2)), "r"(nm), "r"(0u), "l"(pol)
                 : "memory");
  }
  static __host__ __device__ size_t bytes(int rows) { return (size_t)rows * 16; }
};
template <>
struct StateSlot<double> {
  double2* rec;
  uint32_t* meta;
  __device__ __forceinline__ StateSlot(unsigned char* base, int rows)
      : rec(reinterpret_cast<double2*>(base)), meta(reinterpret_cast<uint32_t*>(base + (size_t)rows * 16)) {}
  __device__ __forceinline__ void load(int row, double& a1, double& a2, uint32_t& mt) const {
    double2 v = rec[row];
    a1 = v.x;
    a2 = v.y;
    mt = meta[row];
  }
  __device__ __forceinline__ void store(int row, double n1, double n2, uint32_t nm) const {
    rec[row] = make_double2(n1, n2);
    meta[row] = nm;
  }
  static __host__ __device__ size_t bytes(int rows) { return (size_t)rows * 20; }
};

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

template <typename T>
__global__ void __launch_bounds__(384, sizeof(T) == 4 ? 2 : 1) layered_kernel(const __grid_constant__ DecodeArgs<T> a) {
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
      for (int t = tid; t < c.e; t += nt) post[2 * z + t] = add_rn((T)0, __ldcs(llr + t));
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
        // the state of a layer is prefetched one layer ahead
        T a1 = (T)0, a2 = (T)0;
        uint32_t mt = 0;
        if (iter > 1 && active) st.load(tid, a1, a2, mt);
        for (int L = 0; L < c.rows_n; L++) {
          T p1 = (T)0, p2 = (T)0;
          uint32_t pm = 0;
          if (iter > 1 && active && L + 1 < c.rows_n) st.load((L + 1) * z + tid, p1, p2, pm);
          if (active) {
            const int s0 = c.layer_start[L];
            const int d = c.layer_start[L + 1] - s0;
            T n1, n2;
            uint32_t nm;
            row_dispatch<T>(d, post, c.entry + s0, tid, z, a1, a2, mt, rule, alpha, n1, n2, nm);
            st.store(L * z + tid, n1, n2, nm);
          }
          a1 = p1;
          a2 = p2;
          mt = pm;
          __syncthreads();
        }
        if (!some_check_fails(post, hd, s_ent, s_lstart, c.rows_n, ncol, z, tid, nt)) {
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
  return precision == 0 ? decode_smem_bytes<double>(c.n_full, c.z, c.rows_n, c.n_entries)
                        : decode_smem_bytes<float>(c.n_full, c.z, c.rows_n, c.n_entries);
}

}  // namespace

size_t decode_state_bytes_per_slot(const cbd::DevCode& c, int precision) {
  const int rows = c.rows_n * c.z;
  return precision == 0 ? slot_bytes<double>(rows) : slot_bytes<float>(rows);
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
