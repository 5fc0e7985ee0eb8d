// Belief propagation on a generic sparse LDPC code: the propagate loop of LdpcCode
// (crates/com-fec/src/ldpc.rs:509-557) with the three check rules of check_message
// (:449-493) and both schedules, for any parity-check matrix (PEG, alist, IRA, DVB-S2,
// or the lifted rows of a 5G NR code).
//
// One CTA decodes one codeword at a time (a persistent grid with an atomic work
// counter).  The posteriors sit in shared memory, and the check-to-variable messages,
// one per edge as in the reference, too when they fit; what does not fit (the messages
// of large codes, and the posteriors of the largest, e.g. DVB-S2 normal frames) sits in
// the CTA's slot of a global buffer.
//
//   * Layered: the rows run level by level (the level schedule of sparse_host.h), one
//     thread per row of the level, a barrier between levels.  This is the reference's
//     sequential row order exactly.
//   * Flooding: every row computes its new messages from the previous posteriors; then
//     every variable sums the channel LLR and its new messages in increasing row order,
//     as the reference's loop over the rows does.
//
// Every step is an explicitly rounded IEEE operation in the reference's order.  The
// min-sum rules are therefore bit-exact in f64 (and equal to the same algorithm in f32).
// The sum-product rule calls CUDA's tanh where the reference calls the platform libm,
// and in f64 computes 2 atanh with atanh2.cuh (in f32 CUDA's atanhf): results agree to
// rounding, not bit for bit.
#include <cuda_runtime.h>

#include "atanh2.cuh"
#include "decode_common.cuh"
#include "kernels.h"

namespace cbk {
namespace {

// TANH_BOUND of ldpc.rs:93; it rounds to 1 in f32, where the bound is the largest
// float below 1 (1 - 2^-24)
template <typename T>
__device__ __forceinline__ T tanh_bound();
template <>
__device__ __forceinline__ double tanh_bound<double>() { return 0.999999999999; }
template <>
__device__ __forceinline__ float tanh_bound<float>() { return __uint_as_float(0x3f7fffffu); }

__device__ __forceinline__ double tanh_t(double x) { return tanh(x); }
__device__ __forceinline__ float tanh_t(float x) { return tanhf(x); }

// f64::clamp(lo, hi)
template <typename T>
__device__ __forceinline__ T clamp_t(T x, T lo, T hi) {
  return x < lo ? lo : (x > hi ? hi : x);
}

// the check-node output 2 atanh(clamp(p, -TANH_BOUND, TANH_BOUND)) (ldpc.rs:451-466)
__device__ __forceinline__ double twice_atanh_t(double p) { return at2::twice_atanh(p, tanh_bound<double>()); }
__device__ __forceinline__ float twice_atanh_t(float p) {
  return mul_rn(2.0f, atanhf(clamp_t(p, -tanh_bound<float>(), tanh_bound<float>())));
}

// One check node.  The incoming message of edge i is post - c2v.  Layered: the outputs
// go to msg (replacing the old messages after they are read) and to post; flooding: to
// out only.  aux holds the prefix products of the sum-product rule.
// Edge k of a row: its message slot and its variable, in the row-major layout (slot
// e0 + k) or the transposed one (slot k m + pos, consecutive for consecutive threads).
struct EdgeSlots {
  const int32_t* vars;
  int base, stride;
  __device__ __forceinline__ int slot(int k) const { return base + k * stride; }
  __device__ __forceinline__ int var(int k) const { return vars[slot(k)]; }
};

template <typename T, int RULE, bool LAYERED>
__device__ __forceinline__ void check_row(const SparseDev& c, int row, int pos, T* post, T* msg, T* out, T* aux,
                                          T alpha) {
  const int d = c.row_start[row + 1] - c.row_start[row];
  const EdgeSlots es = c.tvars ? EdgeSlots{c.tvars, pos, c.m} : EdgeSlots{c.vars, c.row_start[row], 1};
  if (RULE == cbd::RULE_SUM_PRODUCT && sizeof(T) == 4) {
    // the product of the other tanh(L/2) by prefix and suffix products.  In f32 tanh is
    // cheap: the second pass computes it again from the unchanged post and msg, which
    // costs less than storing it (the messages of large codes live in global memory)
    T prefix = (T)1;
    for (int k = 0; k < d; k++) {
      const int e = es.slot(k), v = es.var(k);
      const T t = tanh_t(mul_rn(sub_rn(post[v], msg[e]), (T)0.5));
      aux[e] = prefix;
      prefix = mul_rn(prefix, t);
    }
    T suffix = (T)1;
    for (int k = d - 1; k >= 0; k--) {
      const int e = es.slot(k), v = es.var(k);
      const T l = sub_rn(post[v], msg[e]);
      const T t = tanh_t(mul_rn(l, (T)0.5));
      const T p = mul_rn(aux[e], suffix);
      suffix = mul_rn(suffix, t);
      const T o = twice_atanh_t(p);
      if (LAYERED) {
        msg[e] = o;
        post[v] = add_rn(l, o);
      } else {
        out[e] = o;
      }
    }
  } else if (RULE == cbd::RULE_SUM_PRODUCT) {
    // f64: the first pass keeps each edge's tanh(l/2) (34 FP64 instructions) in the edge's
    // message slot, whose old message it no longer needs, so that the second pass does
    // not compute it again; layered, l goes to the variable's posterior (no other row of
    // the level touches that variable)
    T prefix = (T)1;
    for (int k = 0; k < d; k++) {
      const int e = es.slot(k), v = es.var(k);
      const T l = sub_rn(post[v], msg[e]);
      const T t = tanh_t(mul_rn(l, (T)0.5));
      aux[e] = prefix;
      prefix = mul_rn(prefix, t);
      msg[e] = t;
      if (LAYERED) post[v] = l;
    }
    T suffix = (T)1;
    for (int k = d - 1; k >= 0; k--) {
      const int e = es.slot(k), v = es.var(k);
      const T t = msg[e];
      const T p = mul_rn(aux[e], suffix);
      suffix = mul_rn(suffix, t);
      const T o = twice_atanh_t(p);
      if (LAYERED) {
        msg[e] = o;
        post[v] = add_rn(post[v], o);
      } else {
        out[e] = o;
      }
    }
  } else if (sizeof(T) == 8) {
    // f64 min-sum with the reference's comparisons on the integer pipes: `l < 0` is the
    // sign bit of a nonzero, non-NaN l (-0.0 and NaN compare false, as in f64), the
    // magnitudes order as their bit patterns (NaN above infinity, so never `<`), and
    // s * mag with s = +-1 is mag with its sign bit flipped.  The scaled magnitudes are
    // the same for every edge, so they are computed once.  The results are the same
    // bits as the branch below.
    const long long kInf = 0x7ff0000000000000ll;
    int neg = 0, i1 = 0;
    long long b1 = kInf, b2 = kInf;
    for (int i = 0; i < d; i++) {
      const long long bl = __double_as_longlong((double)sub_rn(post[es.var(i)], msg[es.slot(i)]));
      const long long a = abs_bits(bl);
      neg ^= (int)(bl < 0 && a != 0 && a <= kInf);
      if (a < b1) {
        b2 = b1;
        b1 = a;
        i1 = i;
      } else if (a < b2) {
        b2 = a;
      }
    }
    const T m1 = (T)__longlong_as_double(b1), m2 = (T)__longlong_as_double(b2);
    const T n1 = RULE == cbd::RULE_NMS ? mul_rn(alpha, m1) : fmax(sub_rn(m1, alpha), (T)0);
    const T n2 = RULE == cbd::RULE_NMS ? mul_rn(alpha, m2) : fmax(sub_rn(m2, alpha), (T)0);
    for (int i = 0; i < d; i++) {
      const int e = es.slot(i), v = es.var(i);
      const T l = sub_rn(post[v], msg[e]);
      const long long bl = __double_as_longlong((double)l), a = abs_bits(bl);
      const int sneg = neg ^ (int)(bl < 0 && a != 0 && a <= kInf);
      const long long mb = __double_as_longlong((double)(i == i1 ? n2 : n1));
      const T o = (T)__longlong_as_double(mb ^ ((long long)sneg << 63));
      if (LAYERED) {
        msg[e] = o;
        post[v] = add_rn(l, o);
      } else {
        out[e] = o;
      }
    }
  } else {
    int neg = 0, i1 = 0;
    T m1 = infinity<T>(), m2 = infinity<T>();
    for (int i = 0; i < d; i++) {
      const T l = sub_rn(post[es.var(i)], msg[es.slot(i)]);
      neg ^= (int)(l < (T)0);
      const T a = fabs(l);
      if (a < m1) {
        m2 = m1;
        m1 = a;
        i1 = i;
      } else if (a < m2) {
        m2 = a;
      }
    }
    const T sign = neg ? (T)-1 : (T)1;
    for (int i = 0; i < d; i++) {
      const int e = es.slot(i), v = es.var(i);
      const T l = sub_rn(post[v], msg[e]);
      const T s = mul_rn(sign, l < (T)0 ? (T)-1 : (T)1);
      T mag = i == i1 ? m2 : m1;
      mag = RULE == cbd::RULE_NMS ? mul_rn(alpha, mag) : fmax(sub_rn(mag, alpha), (T)0);
      const T o = mul_rn(s, mag);
      if (LAYERED) {
        msg[e] = o;
        post[v] = add_rn(l, o);
      } else {
        out[e] = o;
      }
    }
  }
}

// The layered sum-product row of check_row with its tanh values and prefix products in
// registers (rows of at most MAXD edges): the same operations in the same order, without
// the prefix buffer.
template <typename T, int MAXD>
__device__ __forceinline__ void check_row_spa_regs(const SparseDev& c, int row, int pos, T* post, T* msg) {
  const int d = c.row_start[row + 1] - c.row_start[row];
  const EdgeSlots es = c.tvars ? EdgeSlots{c.tvars, pos, c.m} : EdgeSlots{c.vars, c.row_start[row], 1};
  T l[MAXD], t[MAXD], pre[MAXD];
  T prefix = (T)1;
#pragma unroll
  for (int k = 0; k < MAXD; k++) {
    if (k < d) {
      l[k] = sub_rn(post[es.var(k)], msg[es.slot(k)]);
      t[k] = tanh_t(mul_rn(l[k], (T)0.5));
      pre[k] = prefix;
      prefix = mul_rn(prefix, t[k]);
    }
  }
  T suffix = (T)1;
#pragma unroll
  for (int k = MAXD - 1; k >= 0; k--) {
    if (k < d) {
      const T p = mul_rn(pre[k], suffix);
      suffix = mul_rn(suffix, t[k]);
      const T o = twice_atanh_t(p);
      msg[es.slot(k)] = o;
      post[es.var(k)] = add_rn(l[k], o);
    }
  }
}

// One check node by a warp (layered schedule, levels of few rows): lane i takes edges
// i, i + 32, ... of the row.  Min-sum: a warp reduction of (minimum, first index of the
// minimum, second minimum) and of the sign parity gives the sequential loop's values
// exactly (ties keep the first index, as the strict `<` does).  Sum-product: the
// products of the other tanh(l/2) by warp scans, in chunks of 32 edges; the order of the
// multiplications differs from the sequential one (a rounding difference, within the
// tolerance the sum-product rule already has against the platform libm).
template <typename T, int RULE>
__device__ __forceinline__ void check_row_warp(const SparseDev& c, int row, T* post, T* msg, T alpha, int lane) {
  const int e0 = c.row_start[row], e1 = c.row_start[row + 1];
  if (RULE == cbd::RULE_SUM_PRODUCT) {
    // first pass over the chunks (at most 4: rows of at most 128 edges): the incoming
    // message, its tanh(l/2) and its exclusive prefix product, kept in registers; second
    // pass from the last chunk: the suffix products and the outputs
    T carry = (T)1;
    T pre_r[4], t_r[4], l_r[4];
    int nchunk = (e1 - e0 + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      pre_r[k] = (T)1;
      t_r[k] = (T)1;
      l_r[k] = (T)0;
    }
    for (int k = 0; k < nchunk && k < 4; k++) {
      const int e = e0 + k * 32 + lane;
      T l = (T)0, t = (T)1;
      if (e < e1) {
        l = sub_rn(post[c.vars[e]], msg[e]);
        t = tanh_t(mul_rn(l, (T)0.5));
      }
      // inclusive scan of products within the chunk
      T inc = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc = mul_rn(u, inc);
      }
      T exc = __shfl_up_sync(0xffffffffu, inc, 1);
      if (lane == 0) exc = (T)1;
      pre_r[k] = mul_rn(carry, exc);
      t_r[k] = t;
      l_r[k] = l;
      carry = mul_rn(carry, __shfl_sync(0xffffffffu, inc, 31));
    }
    T scarry = (T)1;
    for (int k = min(nchunk, 4) - 1; k >= 0; k--) {
      const int e = e0 + k * 32 + lane;
      T inc = t_r[k];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_down_sync(0xffffffffu, inc, o);
        if (lane + o < 32) inc = mul_rn(u, inc);
      }
      T exc = __shfl_down_sync(0xffffffffu, inc, 1);
      if (lane == 31) exc = (T)1;
      const T suf = mul_rn(scarry, exc);
      scarry = mul_rn(scarry, __shfl_sync(0xffffffffu, inc, 0));
      if (e < e1) {
        const T p = mul_rn(pre_r[k], suf);
        const T o = twice_atanh_t(p);
        msg[e] = o;
        post[c.vars[e]] = add_rn(l_r[k], o);
      }
    }
  } else if (sizeof(T) == 8) {
    // f64: the integer forms of check_row's f64 min-sum (the same bits); the reduction
    // keeps the first index among equal minima, as the strict `<` of the sequential loop
    const long long kInf = 0x7ff0000000000000ll;
    int neg = 0, i1 = 0x7fffffff;
    long long b1 = kInf, b2 = kInf;
    for (int e = e0 + lane; e < e1; e += 32) {
      const long long bl = __double_as_longlong((double)sub_rn(post[c.vars[e]], msg[e]));
      const long long a = abs_bits(bl);
      neg ^= (int)(bl < 0 && a != 0 && a <= kInf);
      if (a < b1) {
        b2 = b1;
        b1 = a;
        i1 = e - e0;
      } else if (a < b2) {
        b2 = a;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long bb1 = __shfl_xor_sync(0xffffffffu, b1, o);
      const long long bb2 = __shfl_xor_sync(0xffffffffu, b2, o);
      const int bi1 = __shfl_xor_sync(0xffffffffu, i1, o);
      neg ^= __shfl_xor_sync(0xffffffffu, neg, o);
      const bool mine = b1 < bb1 || (b1 == bb1 && i1 < bi1);
      const long long w2 = mine ? b2 : bb2, l1 = mine ? bb1 : b1;
      b1 = mine ? b1 : bb1;
      i1 = mine ? i1 : bi1;
      b2 = w2 < l1 ? w2 : l1;
    }
    const T m1 = (T)__longlong_as_double(b1), m2 = (T)__longlong_as_double(b2);
    const T n1 = RULE == cbd::RULE_NMS ? mul_rn(alpha, m1) : fmax(sub_rn(m1, alpha), (T)0);
    const T n2 = RULE == cbd::RULE_NMS ? mul_rn(alpha, m2) : fmax(sub_rn(m2, alpha), (T)0);
    for (int e = e0 + lane; e < e1; e += 32) {
      const int v = c.vars[e];
      const T l = sub_rn(post[v], msg[e]);
      const long long bl = __double_as_longlong((double)l), a = abs_bits(bl);
      const int sneg = neg ^ (int)(bl < 0 && a != 0 && a <= kInf);
      const long long mb = __double_as_longlong((double)((e - e0) == i1 ? n2 : n1));
      const T o = (T)__longlong_as_double(mb ^ ((long long)sneg << 63));
      msg[e] = o;
      post[v] = add_rn(l, o);
    }
  } else {
    int neg = 0, i1 = 0x7fffffff;
    T m1 = infinity<T>(), m2 = infinity<T>();
    for (int e = e0 + lane; e < e1; e += 32) {
      const T l = sub_rn(post[c.vars[e]], msg[e]);
      neg ^= (int)(l < (T)0);
      const T a = fabs(l);
      if (a < m1) {
        m2 = m1;
        m1 = a;
        i1 = e - e0;
      } else if (a < m2) {
        m2 = a;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T bm1 = __shfl_xor_sync(0xffffffffu, m1, o);
      const T bm2 = __shfl_xor_sync(0xffffffffu, m2, o);
      const int bi1 = __shfl_xor_sync(0xffffffffu, i1, o);
      neg ^= __shfl_xor_sync(0xffffffffu, neg, o);
      const bool mine = m1 < bm1 || (m1 == bm1 && i1 < bi1);
      const T w2 = mine ? m2 : bm2, l1 = mine ? bm1 : m1;
      m1 = mine ? m1 : bm1;
      i1 = mine ? i1 : bi1;
      m2 = fmin(w2, l1);
    }
    const T sign = neg ? (T)-1 : (T)1;
    for (int e = e0 + lane; e < e1; e += 32) {
      const int v = c.vars[e];
      const T l = sub_rn(post[v], msg[e]);
      const T s = mul_rn(sign, l < (T)0 ? (T)-1 : (T)1);
      T mag = (e - e0) == i1 ? m2 : m1;
      mag = RULE == cbd::RULE_NMS ? mul_rn(alpha, mag) : fmax(sub_rn(mag, alpha), (T)0);
      const T o = mul_rn(s, mag);
      msg[e] = o;
      post[v] = add_rn(l, o);
    }
  }
}

// hard_decisions_are_a_codeword (ldpc.rs:555-557), CTA-wide
template <typename T>
__device__ __forceinline__ bool some_row_fails(const SparseDev& c, const T* post) {
  int bad = 0;
  for (int r = threadIdx.x; r < c.m && !bad; r += blockDim.x) {
    int par = 0;
    for (int e = c.row_start[r]; e < c.row_start[r + 1]; e++) par ^= (int)(post[c.vars[e]] < (T)0);
    bad = par;
  }
  return __syncthreads_or(bad) != 0;
}

// REGS: the layered sum-product rows keep their tanh values and prefix products in
// registers (check_row_spa_regs; every row of at most kRegRowDegree edges)
template <typename T, int RULE, bool LAYERED, bool REGS>
__global__ void __launch_bounds__(512, sizeof(T) == 4 ? 2 : 1) sparse_kernel(const __grid_constant__ SparseArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SparseDev& c = a.code;
  const int tid = threadIdx.x, nt = blockDim.x;
  // the messages, then (when the schedule needs one) the second buffer: the flooding
  // schedule's new messages or the sum-product rule's prefix products
  const size_t bufs = (size_t)(a.has_aux ? 2 : 1) * c.slots;
  T* post;
  T* msg;
  if (a.msgs_in_smem) {
    post = reinterpret_cast<T*>(smem);
    msg = post + c.n;
  } else {
    const size_t per = bufs + (a.post_in_smem ? 0 : (size_t)c.n);
    msg = a.slots + (size_t)blockIdx.x * per;
    post = a.post_in_smem ? reinterpret_cast<T*>(smem) : msg + bufs;
  }
  T* aux = a.has_aux ? msg + c.slots : nullptr;
  const T alpha = (T)a.alpha;
  __shared__ long long s_cw;
  for (;;) {
    if (tid == 0) s_cw = (long long)atomicAdd(a.work_counter, 1ull);
    __syncthreads();
    const long long cw = s_cw;
    if (cw >= a.n_frames) break;
    const T* llr = a.llr + (size_t)cw * c.n;
    for (int v = tid; v < c.n; v += nt) post[v] = llr[v];
    for (int e = tid; e < c.slots; e += nt) {
      msg[e] = (T)0;
      if (aux) aux[e] = (T)0;
    }
    __syncthreads();
    int it = 0;
    if (some_row_fails(c, post)) {
      it = a.max_iterations;
      T* cur = msg;   // flooding: the messages of the previous iteration
      T* next = aux;  // flooding: the new ones
      for (int iter = 1; iter <= a.max_iterations; iter++) {
        if (LAYERED && a.warp_rows) {
          const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
          for (int L = 0; L < c.levels; L++) {
            const int r0 = c.level_start[L], r1 = c.level_start[L + 1];
            for (int i = r0 + warp; i < r1; i += nw) check_row_warp<T, RULE>(c, c.level_rows[i], post, msg, alpha, lane);
            __syncthreads();
          }
        } else if (LAYERED) {
          for (int L = 0; L < c.levels; L++) {
            const int r0 = c.level_start[L], r1 = c.level_start[L + 1];
            for (int i = r0 + tid; i < r1; i += nt) {
              if constexpr (REGS) check_row_spa_regs<T, kRegRowDegree>(c, c.level_rows[i], i, post, msg);
              else check_row<T, RULE, true>(c, c.level_rows[i], i, post, msg, nullptr, aux, alpha);
            }
            __syncthreads();
          }
        } else {
          // the sum-product rule keeps its prefix products in `next`, where its outputs go
          for (int r = tid; r < c.m; r += nt) check_row<T, RULE, false>(c, r, r, post, cur, next, next, alpha);
          __syncthreads();
          for (int v = tid; v < c.n; v += nt) {
            T s = llr[v];
            for (int k = c.col_start[v]; k < c.col_start[v + 1]; k++) s = add_rn(s, next[c.col_edges[k]]);
            post[v] = s;
          }
          T* t = cur;
          cur = next;
          next = t;
          __syncthreads();
        }
        if (!some_row_fails(c, post)) {
          it = iter;
          break;
        }
      }
    }
    if (a.post_out)
      for (int v = tid; v < c.n; v += nt) a.post_out[(size_t)cw * c.n + v] = post[v];
    if (tid == 0 && a.iters_out) a.iters_out[cw] = it;
    __syncthreads();
  }
}

// Layered decoding of small codes, a.group codewords per CTA, their posteriors and
// messages in shared memory one codeword after the other.  The rows of a level of all the
// group's codewords are spread over the threads, one row each, so that the warps run full
// even when a level has few rows (every warp instruction costs the same issue and pipe
// time whatever its active lanes).  Each codeword stops on its own syndrome: its rows
// are skipped from then on.  Results equal sparse_kernel's.
template <typename T>
__device__ __forceinline__ void group_syndrome(const SparseDev& c, const T* base, size_t per, int G,
                                               const int* check, volatile int* fail) {
  for (int i = threadIdx.x; i < G * c.m; i += blockDim.x) {
    const int g = i / c.m, r = i - g * c.m;
    if (!check[g] || fail[g]) continue;
    const T* post = base + g * per;
    int par = 0;
    for (int e = c.row_start[r]; e < c.row_start[r + 1]; e++) par ^= (int)(post[c.vars[e]] < (T)0);
    if (par) fail[g] = 1;
  }
}

// two CTAs of up to 512 threads fit an SM in f32 (at most 64 registers); one in f64, whose
// rows need more (without the bound the compiler held the f64 min-sum rows to 40 and spilled)
template <typename T, int RULE, bool REGS>
__global__ void __launch_bounds__(512, sizeof(T) == 4 ? 2 : 1) sparse_group_kernel(const __grid_constant__ SparseArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SparseDev& c = a.code;
  const int tid = threadIdx.x, nt = blockDim.x, G = a.group;
  const size_t bufs = (size_t)(a.has_aux ? 2 : 1) * c.slots;
  const size_t per = (size_t)c.n + bufs;  // elements of one codeword: posteriors, then messages
  T* base = reinterpret_cast<T*>(smem);
  __shared__ long long s_cw[kMaxGroup];
  __shared__ int s_run[kMaxGroup];   // 1 while the codeword decodes
  __shared__ int s_fail[kMaxGroup];  // its syndrome fails
  __shared__ int s_it[kMaxGroup];
  const T alpha = (T)a.alpha;
  for (;;) {
    if (tid == 0) {
      const unsigned long long b = atomicAdd(a.work_counter, (unsigned long long)G);
      for (int g = 0; g < G; g++) s_cw[g] = (long long)(b + g);
    }
    __syncthreads();
    if (s_cw[0] >= a.n_frames) break;
    for (int g = 0; g < G; g++) {
      T* post = base + g * per;
      T* msg = post + c.n;
      if (s_cw[g] < a.n_frames) {
        const T* llr = a.llr + (size_t)s_cw[g] * c.n;
        for (int v = tid; v < c.n; v += nt) post[v] = llr[v];
      }
      for (size_t e = tid; e < bufs; e += nt) msg[e] = (T)0;
    }
    if (tid < G) {
      s_run[tid] = s_cw[tid] < a.n_frames ? 1 : 0;
      s_fail[tid] = 0;
    }
    __syncthreads();
    group_syndrome(c, base, per, G, s_run, s_fail);
    __syncthreads();
    int any = 0;
    for (int g = 0; g < G; g++) any |= s_run[g] && s_fail[g];
    __syncthreads();
    if (tid < G) {
      s_run[tid] = s_run[tid] && s_fail[tid];
      s_it[tid] = s_run[tid] ? a.max_iterations : 0;
    }
    __syncthreads();
    for (int iter = 1; iter <= a.max_iterations && any; iter++) {
      for (int L = 0; L < c.levels; L++) {
        const int r0 = c.level_start[L], rl = c.level_start[L + 1] - r0;
        for (int i = tid; i < G * rl; i += nt) {
          const int g = i / rl, j = i - g * rl;
          if (!s_run[g]) continue;
          T* post = base + g * per;
          T* msg = post + c.n;
          if constexpr (REGS) check_row_spa_regs<T, kRegRowDegree>(c, c.level_rows[r0 + j], r0 + j, post, msg);
          else check_row<T, RULE, true>(c, c.level_rows[r0 + j], r0 + j, post, msg, nullptr,
                                        a.has_aux ? msg + c.slots : nullptr, alpha);
        }
        __syncthreads();
      }
      if (tid < G) s_fail[tid] = 0;
      __syncthreads();
      group_syndrome(c, base, per, G, s_run, s_fail);
      __syncthreads();
      any = 0;
      for (int g = 0; g < G; g++) any |= s_run[g] && s_fail[g];
      __syncthreads();
      if (tid < G && s_run[tid] && !s_fail[tid]) {
        s_run[tid] = 0;
        s_it[tid] = iter;
      }
      __syncthreads();
    }
    for (int g = 0; g < G; g++) {
      const long long cw = s_cw[g];
      if (cw >= a.n_frames) continue;
      const T* post = base + g * per;
      if (a.post_out)
        for (int v = tid; v < c.n; v += nt) a.post_out[(size_t)cw * c.n + v] = post[v];
      if (tid == 0 && a.iters_out) a.iters_out[cw] = s_it[g];
    }
    __syncthreads();
  }
}

template <typename T>
void* sparse_kernel_for(int rule, bool layered, bool regs) {
  if (layered) {
    if (rule == cbd::RULE_SUM_PRODUCT)
      return regs ? (void*)sparse_kernel<T, cbd::RULE_SUM_PRODUCT, true, true>
                  : (void*)sparse_kernel<T, cbd::RULE_SUM_PRODUCT, true, false>;
    if (rule == cbd::RULE_NMS) return (void*)sparse_kernel<T, cbd::RULE_NMS, true, false>;
    return (void*)sparse_kernel<T, cbd::RULE_OMS, true, false>;
  }
  if (rule == cbd::RULE_SUM_PRODUCT) return (void*)sparse_kernel<T, cbd::RULE_SUM_PRODUCT, false, false>;
  if (rule == cbd::RULE_NMS) return (void*)sparse_kernel<T, cbd::RULE_NMS, false, false>;
  return (void*)sparse_kernel<T, cbd::RULE_OMS, false, false>;
}

}  // namespace

void* sparse_kernel_ptr(int precision, int rule, bool layered, bool regs) {
  return precision == 0 ? sparse_kernel_for<double>(rule, layered, regs) : sparse_kernel_for<float>(rule, layered, regs);
}

template <typename T>
void* sparse_group_kernel_for(int rule, bool regs) {
  if (rule == cbd::RULE_SUM_PRODUCT)
    return regs ? (void*)sparse_group_kernel<T, cbd::RULE_SUM_PRODUCT, true>
                : (void*)sparse_group_kernel<T, cbd::RULE_SUM_PRODUCT, false>;
  if (rule == cbd::RULE_NMS) return (void*)sparse_group_kernel<T, cbd::RULE_NMS, false>;
  return (void*)sparse_group_kernel<T, cbd::RULE_OMS, false>;
}

void* sparse_group_kernel_ptr(int precision, int rule, bool regs) {
  return precision == 0 ? sparse_group_kernel_for<double>(rule, regs) : sparse_group_kernel_for<float>(rule, regs);
}

cudaError_t launch_sparse(void* kernel, const void* args, int grid, int threads, size_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* argv[] = {const_cast<void*>(args)};
  return cudaLaunchKernel(kernel, dim3(grid), dim3(threads), argv, smem, s);
}

}  // namespace cbk
