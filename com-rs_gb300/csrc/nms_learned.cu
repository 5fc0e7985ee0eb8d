// Learned (neural) min-sum: the layered min-sum of decode.cu with a scale and an offset
// per iteration and per edge, trained by hand-written reverse-mode differentiation of
// the unrolled iterations.  No counterpart in the reference; the plain normalised
// min-sum is its special case alpha = 0.75, beta = 0 and remains its fallback.
//
// Check message at iteration t, edge e of a row (the row's other edges k != e):
//   y_e = s_e * max(alpha[t, e] * m_e - beta[t, e], 0)  (the product and the difference
//   rounded once, as one fused multiply-add),
//   s_e = prod sign(x_k), m_e = min |x_k|, x_k = post[v_k] - c2v_k (ldpc.rs:468-491),
// then post[v_e] = x_e + y_e and c2v_e = y_e.  Weights are indexed [t][entry][r] (one per
// lifted edge) or [t][entry] (one per base-graph edge, shared across Z); the edge
// storage is [entry][r], so a layer's Z threads touch consecutive words.
//
// Training loss: the mean over frames and over the codeword bits [0, loss_bits) (all n_full
// bits, or the K' information bits) of softplus(-(1 - 2 c_v) post_v), the binary
// cross-entropy of the soft output: of the
// last iteration, or (multi-loss) a weighted mean over the outputs of all T iterations,
// whose posteriors the forward then saves: weights 1/T, or a ramp 2(t+1)/(T(T+1)).
// Backward: for t = T-1..0 and the layers in reverse, each row recomputes its forward
// quantities from the saved inputs x and propagates
//   g_y = g_post[v] + g_c2v, g_a = g_y s [a > 0], dL/dalpha += g_a m, dL/dbeta -= g_a,
//   g_m = g_a alpha flows to |x| of the argmin (or of the second argmin for the argmin),
//   g_x = g_post[v] + sign(x) g_|x|, then g_post[v] = g_x and g_c2v = -g_x.
#include <cuda_runtime.h>

#include <cmath>

#include "decode_common.cuh"
#include "kernels.h"

namespace cbk {
namespace {

__device__ __forceinline__ size_t weight_index(const LearnedArgs& a, int t, int entry, int r) {
  return a.shared ? (size_t)t * a.code.n_entries + entry
                  : ((size_t)t * a.code.n_entries + entry) * a.code.z + r;
}

// weight of iteration t's output in the multi-loss: 1/T each (mode 1), or a linear ramp
// 2 (t + 1) / (T (T + 1)) that leans on the last iterations (mode 2)
__device__ __forceinline__ float iter_loss_weight(int mode, int t, int T) {
  return mode == 2 ? 2.f * (float)(t + 1) / ((float)T * (float)(T + 1)) : 1.f / (float)T;
}

__device__ __forceinline__ float softplus_f(float x) { return x > 0.f ? x + log1pf(__expf(-x)) : log1pf(__expf(x)); }
__device__ __forceinline__ float sigmoid_f(float x) { return 1.f / (1.f + __expf(-x)); }

// forward of one lifted row, degree D
template <int D>
__device__ __forceinline__ void learned_row_fwd(const LearnedArgs& a, float* post, float* c2v, float* X, int t,
                                                int s0, int r, int z) {
  int off[D];
  float x[D];
#pragma unroll
  for (int e = 0; e < D; e++) {
    const uint32_t en = a.code.entry[s0 + e];
    unsigned cc = (unsigned)r + (en & 0xffffu);
    unsigned cm = cc - (unsigned)z;
    off[e] = (int)(en >> 16) * z + (int)min(cc, cm);
    const size_t ed = (size_t)(s0 + e) * z + r;
    float old = t > 0 ? c2v[ed] : 0.f;
    x[e] = __fsub_rn(post[off[e]], old);
    if (X) X[(size_t)t * a.code.n_entries * z + ed] = x[e];
  }
  uint32_t par = 0;
  float m1 = INFINITY, m2 = INFINITY;
  int i1 = 0;
#pragma unroll
  for (int e = 0; e < D; e++) {
    par ^= (uint32_t)(x[e] < 0.f);
    float av = fabsf(x[e]);
    bool lt = av < m1;
    m2 = lt ? m1 : fminf(m2, av);
    m1 = lt ? av : m1;
    i1 = lt ? e : i1;
  }
#pragma unroll
  for (int e = 0; e < D; e++) {
    const size_t w = weight_index(a, t, s0 + e, r);
    float m = e == i1 ? m2 : m1;
    float am = __fmaf_rn(a.alpha[w], m, -a.beta[w]);
    float mag = am > 0.f ? am : 0.f;
    bool neg = (par ^ (uint32_t)(x[e] < 0.f)) & 1u;
    float y = neg ? -mag : mag;
    c2v[(size_t)(s0 + e) * z + r] = y;
    post[off[e]] = __fadd_rn(x[e], y);
  }
}

template <int D>
__device__ __forceinline__ void learned_row_bwd(const LearnedArgs& a, float* gp, float* gc, const float* X, int t,
                                                int s0, int r, int z, float* sga, float* sgb) {
  int off[D];
  float x[D];
#pragma unroll
  for (int e = 0; e < D; e++) {
    const uint32_t en = a.code.entry[s0 + e];
    unsigned cc = (unsigned)r + (en & 0xffffu);
    unsigned cm = cc - (unsigned)z;
    off[e] = (int)(en >> 16) * z + (int)min(cc, cm);
    x[e] = X[(size_t)t * a.code.n_entries * z + (size_t)(s0 + e) * z + r];
  }
  uint32_t par = 0;
  float m1 = INFINITY, m2 = INFINITY;
  int i1 = 0, i2 = 0;
#pragma unroll
  for (int e = 0; e < D; e++) {
    par ^= (uint32_t)(x[e] < 0.f);
    float av = fabsf(x[e]);
    if (av < m1) {
      m2 = m1;
      i2 = i1;
      m1 = av;
      i1 = e;
    } else if (av < m2) {
      m2 = av;
      i2 = e;
    }
  }
  float g1 = 0.f, g2 = 0.f;  // gradients of |x_i1| and |x_i2|
#pragma unroll
  for (int e = 0; e < D; e++) {
    const size_t w = weight_index(a, t, s0 + e, r);
    const size_t ed = (size_t)(s0 + e) * z + r;
    float m = e == i1 ? m2 : m1;
    float al = a.alpha[w];
    float am = __fmaf_rn(al, m, -a.beta[w]);
    bool neg = (par ^ (uint32_t)(x[e] < 0.f)) & 1u;
    float gy = gp[off[e]] + gc[ed];
    float ga = am > 0.f ? (neg ? -gy : gy) : 0.f;
    if (a.shared) {
      sga[e] = ga * m;
      sgb[e] = -ga;
    } else {
      atomicAdd(&a.g_alpha[w], ga * m);
      atomicAdd(&a.g_beta[w], -ga);
    }
    float gm = ga * al;
    if (e == i1) g2 += gm;
    else g1 += gm;
  }
#pragma unroll
  for (int e = 0; e < D; e++) {
    float gabs = (e == i1 ? g1 : 0.f) + (e == i2 && i2 != i1 ? g2 : 0.f);
    float gx = gp[off[e]] + (x[e] < 0.f ? -gabs : gabs);
    gp[off[e]] = gx;
    gc[(size_t)(s0 + e) * z + r] = -gx;
  }
}

template <bool FWD>
__device__ __forceinline__ void learned_row(int d, const LearnedArgs& a, float* p, float* c, float* X, int t, int s0,
                                            int r, int z, float* sga, float* sgb) {
#define CB_LROW(DD)                                                       \
  case DD:                                                                \
    if (FWD) learned_row_fwd<DD>(a, p, c, X, t, s0, r, z);                \
    else learned_row_bwd<DD>(a, p, c, X, t, s0, r, z, sga, sgb);          \
    break;
  switch (d) {
    CB_LROW(3)
    CB_LROW(4)
    CB_LROW(5)
    CB_LROW(6)
    CB_LROW(7)
    CB_LROW(8)
    CB_LROW(9)
    CB_LROW(10)
    default:
      if (FWD) learned_row_fwd<19>(a, p, c, X, t, s0, r, z);
      else learned_row_bwd<19>(a, p, c, X, t, s0, r, z, sga, sgb);
  }
#undef CB_LROW
}

// Shared weights: the row gradients of a layer summed over its Z threads (warp shuffles,
// one shared-memory add per warp), then one global add per entry.
__device__ __forceinline__ void reduce_shared_grads(const LearnedArgs& a, int t, int s0, int d, const float* sga,
                                                    const float* sgb, float* red, int tid, bool active) {
  const int lane = tid & 31;
  for (int e = 0; e < 19; e++) {
    if (e >= d) break;
    float va = active ? sga[e] : 0.f, vb = active ? sgb[e] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      va += __shfl_xor_sync(0xffffffffu, va, o);
      vb += __shfl_xor_sync(0xffffffffu, vb, o);
    }
    if (lane == 0) {
      atomicAdd(&red[2 * e], va);
      atomicAdd(&red[2 * e + 1], vb);
    }
  }
  __syncthreads();
  if (tid < d) {
    const size_t w = (size_t)t * a.code.n_entries + s0 + tid;
    atomicAdd(&a.g_alpha[w], red[2 * tid]);
    atomicAdd(&a.g_beta[w], red[2 * tid + 1]);
    red[2 * tid] = 0.f;
    red[2 * tid + 1] = 0.f;
  }
}

__global__ void __launch_bounds__(384) learned_forward_kernel(const __grid_constant__ LearnedArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const cbd::DevCode& c = a.code;
  const int z = c.z, nt = blockDim.x, tid = threadIdx.x;
  const int ncol = c.n_full / z, ws = (z + 31) / 32 + 1;
  float* post = reinterpret_cast<float*>(smem);
  uint32_t* hd = reinterpret_cast<uint32_t*>(post + c.n_full);
  uint32_t* s_ent = hd + ncol * ws;
  uint16_t* s_lstart = reinterpret_cast<uint16_t*>(s_ent + c.n_entries);
  __shared__ float s_loss;
  __shared__ unsigned int s_err;
  const long long f = blockIdx.x;
  if (f >= a.n_frames) return;
  for (int i = tid; i < c.n_entries; i += nt) s_ent[i] = c.entry[i];
  for (int i = tid; i <= c.rows_n; i += nt) s_lstart[i] = c.layer_start[i];
  if (tid == 0) {
    s_loss = 0.f;
    s_err = 0;
  }
  const size_t edges = (size_t)c.n_entries * z;
  float* c2v = a.c2v + (size_t)f * edges;
  float* X = a.X ? a.X + (size_t)f * a.T * edges : nullptr;
  const float* llr = a.llr + (size_t)f * c.e;
  for (int v = tid; v < c.n_full; v += nt) post[v] = 0.f;
  __syncthreads();
  if (c.map_is_offset) {
    for (int t = tid; t < c.e; t += nt) post[2 * z + t] = __fadd_rn(0.f, llr[t]);
  } else if (!c.has_repeats) {
    for (int t = tid; t < c.e; t += nt) post[c.map[t]] = __fadd_rn(0.f, llr[t]);
  } else {
    for (int v = tid; v < c.n_full; v += nt) {
      int b0 = c.inv_start[v], b1 = c.inv_start[v + 1];
      if (b0 == b1) continue;
      float s = 0.f;
      for (int i = b0; i < b1; i++) s = __fadd_rn(s, llr[c.inv_t[i]]);
      post[v] = s;
    }
  }
  __syncthreads();
  for (int v = c.k_info + tid; v < c.k; v += nt) post[v] = cbd::kKnownBitLlr;
  __syncthreads();
  int it = 0;
  const bool stop = a.early_stop != 0;
  const bool multi = a.multi_loss && a.P && a.cw_bits && a.loss;
  float lsum = 0.f;  // this thread's share of the loss
  if (!stop || some_check_fails(post, hd, s_ent, s_lstart, c.rows_n, ncol, z, tid, nt)) {
    it = a.T;
    for (int t = 0; t < a.T; t++) {
      for (int L = 0; L < c.rows_n; L++) {
        if (tid < z) {
          const int s0 = s_lstart[L];
          learned_row<true>(s_lstart[L + 1] - s0, a, post, c2v, X, t, s0, tid, z, nullptr, nullptr);
        }
        __syncthreads();
      }
      if (multi) {
        const int wpc = (c.n_full + 31) >> 5;
        float* Pt = a.P + ((size_t)f * a.T + t) * c.n_full;
        for (int v = tid; v < a.loss_bits; v += nt) {
          Pt[v] = post[v];
          int bit = (a.cw_bits[(size_t)f * wpc + (v >> 5)] >> (v & 31)) & 1;
          lsum += softplus_f(bit ? post[v] : -post[v]) * iter_loss_weight(a.multi_loss, t, a.T);
        }
      }
      if (stop && !some_check_fails(post, hd, s_ent, s_lstart, c.rows_n, ncol, z, tid, nt)) {
        it = t + 1;
        break;
      }
    }
  }
  // outputs
  if (a.post_out)
    for (int v = tid; v < c.n_full; v += nt) a.post_out[(size_t)f * c.n_full + v] = post[v];
  if (a.cw_bits && a.loss) {
    if (!multi) {
      const int wpc = (c.n_full + 31) >> 5;
      for (int v = tid; v < a.loss_bits; v += nt) {
        int bit = (a.cw_bits[(size_t)f * wpc + (v >> 5)] >> (v & 31)) & 1;
        lsum += softplus_f(bit ? post[v] : -post[v]);
      }
    }
    atomicAdd(&s_loss, lsum);
  }
  const int wpf = (c.k_info + 31) >> 5, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  unsigned int be = 0;
  // the sent words, one per thread, loaded before the ballots so that their latency
  // overlaps them; the decisions are staged in hd (free after the syndrome tests)
  const uint32_t* ref = a.ref_bits ? a.ref_bits + (size_t)f * wpf : nullptr;
  const uint32_t ref_w = (ref && tid < wpf) ? ref[tid] : 0u;
  if (ref) {
    for (int b0 = warp * 32; b0 < c.k_info; b0 += nw * 32) {
      int v = b0 + lane;
      uint32_t word = __ballot_sync(0xffffffffu, v < c.k_info && post[v] < 0.f);
      if (lane == 0) hd[b0 >> 5] = word;
    }
    __syncthreads();
    if (tid < wpf) be = __popc(hd[tid] ^ ref_w);
    for (int w = tid + nt; w < wpf; w += nt) be += __popc(hd[w] ^ ref[w]);
  }
  if (be) atomicAdd(&s_err, be);
  __syncthreads();
  if (tid == 0) {
    if (a.loss && a.cw_bits) atomicAdd(a.loss, s_loss / (float)a.loss_bits);
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

__global__ void __launch_bounds__(384) learned_backward_kernel(const __grid_constant__ LearnedArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const cbd::DevCode& c = a.code;
  const int z = c.z, nt = blockDim.x, tid = threadIdx.x;
  float* gp = reinterpret_cast<float*>(smem);
  float* red = gp + c.n_full;  // 2 x 19 floats
  const long long f = blockIdx.x;
  if (f >= a.n_frames) return;
  const size_t edges = (size_t)c.n_entries * z;
  float* gc = a.c2v + (size_t)f * edges;  // the message gradients reuse the message buffer
  const float* X = a.X + (size_t)f * a.T * edges;
  const int wpc = (c.n_full + 31) >> 5;
  const bool multi = a.multi_loss && a.P;
  const float scale = 1.f / ((float)a.loss_bits * (float)a.n_frames);
  for (int v = tid; v < c.n_full; v += nt) gp[v] = 0.f;
  for (size_t i = tid; i < edges; i += nt) gc[i] = 0.f;
  if (tid < 38) red[tid] = 0.f;
  __syncthreads();
  float sga[19], sgb[19];
  for (int t = a.T - 1; t >= 0; t--) {
    // the loss of iteration t's output (every iteration, or the last one)
    if (multi || t == a.T - 1) {
      const float* p = multi ? a.P + ((size_t)f * a.T + t) * c.n_full : a.post_out + (size_t)f * c.n_full;
      const float sc = multi ? scale * iter_loss_weight(a.multi_loss, t, a.T) : scale;
      for (int v = tid; v < a.loss_bits; v += nt) {
        int bit = (a.cw_bits[(size_t)f * wpc + (v >> 5)] >> (v & 31)) & 1;
        float sgn = bit ? -1.f : 1.f;
        gp[v] += -sgn * sigmoid_f(-sgn * p[v]) * sc;
      }
      __syncthreads();
    }
    for (int L = c.rows_n - 1; L >= 0; L--) {
      const int s0 = c.layer_start[L], d = c.layer_start[L + 1] - s0;
      if (tid < z) learned_row<false>(d, a, gp, gc, const_cast<float*>(X), t, s0, tid, z, sga, sgb);
      if (a.shared) reduce_shared_grads(a, t, s0, d, sga, sgb, red, tid, tid < z);
      __syncthreads();
    }
  }
}

// Adam (Kingma & Ba, 2015) on the scales and offsets
__global__ void adam_kernel(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace

size_t learned_smem_bytes(const cbd::DevCode& c) {
  const int ws = (c.z + 31) / 32 + 1;
  size_t b = (size_t)c.n_full * 4 + (size_t)(c.n_full / c.z) * ws * 4 + (size_t)c.n_entries * 4 +
             (size_t)(c.rows_n + 1) * 2 + 16;
  return (b + 15) & ~(size_t)15;
}

cudaError_t launch_learned(const LearnedArgs& a, bool forward, cudaStream_t s) {
  const int threads = ((a.code.z + 31) / 32) * 32;
  void* k = forward ? (void*)learned_forward_kernel : (void*)learned_backward_kernel;
  size_t smem = forward ? learned_smem_bytes(a.code) : (size_t)a.code.n_full * 4 + 2 * 19 * 4 + 16;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3((unsigned)a.n_frames), dim3(threads), args, smem, s);
}

cudaError_t launch_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, int step,
                        cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  adam_kernel<<<blocks, 256, 0, s>>>(w, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError();
}

}  // namespace cbk
