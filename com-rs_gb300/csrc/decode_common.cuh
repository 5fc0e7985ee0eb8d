// Device helpers shared by the decoders (decode.cu, nms_learned.cu): explicitly rounded
// arithmetic, and the block-wide syndrome test on packed hard decisions.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "dev_math.cuh"
#include "device_common.cuh"

namespace cbk {
namespace {

// One lifted row of a layer: thread r, degree D known at compile time.
// old state (a1, a2, mt) -> new state (n1, n2, nm); post updated in place.
// RULE (cbd::RULE_NMS or RULE_OMS) is a template parameter: with the rule read at run time
// the compiler computed both rules' magnitudes in every row and kept one (C2 in f64:
// 42.4 against 36.9 ms per 2048 codewords, 3.9 against 3.3 FP64 instructions per edge
// update).
template <typename T, int D, int RULE>
__device__ __forceinline__ void row_update(T* __restrict__ post, const uint32_t* __restrict__ ent, int r, int z,
                                           T a1, T a2, uint32_t mt, T alpha, T& n1, T& n2, uint32_t& nm) {
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
    if constexpr (sizeof(T) == 8) {
      // the old message as bits: the magnitude (never negative) with the old sign ORed
      // in, so that one subtraction is the FP64 work (p - (-m) is p + m, bit for bit)
      const long long mb = __double_as_longlong(e == old_i1 ? a2 : a1);
      x[e] = sub_rn(post[off[e]], __longlong_as_double(mb | ((long long)((mt >> (8 + e)) & 1u) << 63)));
    } else {
      T mag = (e == old_i1) ? a2 : a1;
      T old = ((mt >> (8 + e)) & 1u) ? -mag : mag;
      x[e] = sub_rn(post[off[e]], old);
    }
  }
  // check_message, min-sum branch (ldpc.rs:468-491): sign product with `l < 0`, strict
  // `<` for the minimum and its index, min(m2, a) for the second (equal for non-NaN,
  // and a NaN is skipped by both)
  uint32_t par;
  T m1, m2;
  int i1 = 0;
  if constexpr (sizeof(T) == 8) {
    // f64 on the integer pipes: the posteriors and messages are never -0.0 or NaN, so
    // `l < 0` is the sign bit, and the order of non-negative doubles is that of their
    // bit patterns; only the subtractions and additions stay on the FP64 pipe
    par = (uint32_t)((unsigned long long)__double_as_longlong(x[0]) >> 63);
    long long b1 = abs_bits(__double_as_longlong(x[0])), b2 = 0x7ff0000000000000ll;
#pragma unroll
    for (int e = 1; e < D; e++) {
      const long long bx = __double_as_longlong(x[e]);
      par ^= (uint32_t)((unsigned long long)bx >> 63);
      const long long av = abs_bits(bx);
      const bool lt = av < b1;
      b2 = lt ? b1 : (av < b2 ? av : b2);
      b1 = lt ? av : b1;
      i1 = lt ? e : i1;
    }
    m1 = __longlong_as_double(b1);
    m2 = __longlong_as_double(b2);
  } else {
    par = (uint32_t)(x[0] < (T)0);
    m1 = fmin(fabs(x[0]), infinity<T>());
    m2 = infinity<T>();
#pragma unroll
    for (int e = 1; e < D; e++) {
      par ^= (uint32_t)(x[e] < (T)0);
      T av = fabs(x[e]);
      bool lt = av < m1;
      m2 = lt ? m1 : fmin(m2, av);
      m1 = lt ? av : m1;
      i1 = lt ? e : i1;
    }
  }
  if constexpr (RULE == cbd::RULE_NMS) {
    n1 = mul_rn(alpha, m1);
    n2 = mul_rn(alpha, m2);
  } else {
    n1 = fmax(sub_rn(m1, alpha), (T)0);
    n2 = fmax(sub_rn(m2, alpha), (T)0);
  }
  nm = (uint32_t)i1;
#pragma unroll
  for (int e = 0; e < D; e++) {
    uint32_t ng;
    T o;
    if constexpr (sizeof(T) == 8) {
      const long long bx = __double_as_longlong(x[e]);
      ng = par ^ (uint32_t)((unsigned long long)bx >> 63);
      const long long mb = e == i1 ? __double_as_longlong(n2) : __double_as_longlong(n1);
      o = __longlong_as_double(mb ^ ((long long)ng << 63));
    } else {
      ng = par ^ (uint32_t)(x[e] < (T)0);
      T mag = (e == i1) ? n2 : n1;
      o = ng ? -mag : mag;
    }
    post[off[e]] = add_rn(x[e], o);
    nm |= ng << (8 + e);
  }
}

// Byte offset in post of edge e's variable for lifted row r, from the per-entry table
// {4 (col Z + shift), Z - shift} of DevCode::eaddr: 4 (col Z + (r + shift) mod Z) = 4 r + x,
// less 4 Z when r >= Z - shift.
struct EdgeAddrTable {
  const uint2* tab;
  int r, r4, z4;
  __device__ __forceinline__ int operator()(int e) const {
    const uint2 t = tab[e];
    const int o = r4 + (int)t.x;
    return r >= (int)t.y ? o - z4 : o;
  }
};

// f32 row update with fewer integer-pipe operations (same results as row_update for
// finite LLRs):
//   * the edge addresses come from a functor (packed entries, or the per-entry table);
//   * the minimum and second minimum are taken two edges at a time with min/max only
//     (min.xorsign.abs and the three-input min), and the minimum's sign bit collects
//     the sign product; the edges that receive the second minimum are those whose
//     magnitude equals the minimum (if several do, the two minima are equal, so every
//     edge gets the same magnitude, as in the reference);
//   * the sign test `x < 0` is the sign bit of x: the posteriors never hold -0.0 (they
//     start as 0.0 + LLR or 30.0, and a difference or sum is -0.0 only when an operand
//     already is), so no message input x = post - c2v is -0.0 either;
//   * outgoing signs are applied and collected with bit operations.
// State word: bits 0-4 an edge holding the second minimum, bits 8.. the outgoing sign of
// edge e at bit 8 + (D - 1 - e).
template <int D, int RULE, typename Addr>
__device__ __forceinline__ void row_update_lean(float* __restrict__ post, const Addr& addr, float a1, float a2,
                                                uint32_t mt, float alpha, float& n1, float& n2, uint32_t& nm) {
  int off[D];
  float x[D];
  const int old_i1 = (int)(mt & 31u);
  const uint32_t t0 = mt << (24 - D);  // the old sign of edge 0 at bit 31
#pragma unroll
  for (int e = 0; e < D; e++) {
    off[e] = addr(e);
    const float mag = (e == old_i1) ? a2 : a1;
    const float p = ld_post(post, off[e]);
    // p - (-mag) is p + mag, bit for bit
    x[e] = ((t0 << e) & 0x80000000u) ? __fadd_rn(p, mag) : __fsub_rn(p, mag);
  }
  // m1 carries the sign product (xor of the signs of all x) in its sign bit
  float m1 = infinity<float>(), m2 = infinity<float>();
#pragma unroll
  for (int e = 0; e + 1 < D; e += 2) {
    const float s = min_xorsign_abs(x[e], x[e + 1]);
    const float l = fmaxf(fabsf(x[e]), fabsf(x[e + 1]));
    m2 = min3f(m2, fmaxf(fabsf(m1), fabsf(s)), l);
    m1 = min_xorsign_abs(m1, s);
  }
  if (D & 1) {
    m2 = fminf(m2, fmaxf(fabsf(m1), fabsf(x[D - 1])));
    m1 = min_xorsign_abs(m1, x[D - 1]);
  }
  const uint32_t ps = __float_as_uint(m1) & 0x80000000u;
  m1 = fabsf(m1);
  if constexpr (RULE == cbd::RULE_NMS) {
    n1 = __fmul_rn(alpha, m1);
    n2 = __fmul_rn(alpha, m2);
  } else {
    n1 = fmaxf(__fsub_rn(m1, alpha), 0.0f);
    n2 = fmaxf(__fsub_rn(m2, alpha), 0.0f);
  }
  const uint32_t n1p = __float_as_uint(n1) | ps, n2p = __float_as_uint(n2) | ps;
  // n2 where |x| equals the minimum, else n1, by an integer multiply-add with the
  // comparison's mask (0 or all ones) on the FMA pipe; a second one sums the indices of
  // those edges: one edge's index when the minimum is unique; when several tie, m1 = m2
  // and any index gives the same old messages (the sum, at most 171, stays below bit 8)
  const uint32_t dneg = n1p - n2p;
  uint32_t sm = 0, i1 = 0;
#pragma unroll
  for (int e = 0; e < D; e++) {
    uint32_t eqm, magp;
    asm("set.eq.u32.f32 %0, %1, %2;" : "=r"(eqm) : "f"(fabsf(x[e])), "f"(m1));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(magp) : "r"(eqm), "r"(dneg), "r"(n1p));
    if (e) asm("mad.lo.u32 %0, %1, %2, %0;" : "+r"(i1) : "r"(eqm), "r"((uint32_t)-e));
    const uint32_t ob = magp ^ (__float_as_uint(x[e]) & 0x80000000u);
    st_post(post, off[e], __fadd_rn(x[e], __uint_as_float(ob)));
    sm = (sm << 1) | (ob >> 31);
  }
  nm = (sm << 8) | i1;
}

// The learned min-sum's weights of one row: alpha and beta of the previous and the
// current iteration, entry s0 + e, lifted row r; `stride` 1 and `roff` 0 when shared by
// the Z rows, else Z and r (global memory, launch parameters or shared memory).
struct LearnedRowW {
  const float *a_prev, *b_prev, *a_cur, *b_cur;
  int s0, stride, roff;
  __device__ __forceinline__ float mag(const float* al, const float* be, int e, float m) const {
    const int i = (s0 + e) * stride + roff;
    const float am = __fmaf_rn(al[i], m, -be[i]);
    return am > 0.f ? am : 0.f;
  }
};

// One lifted row of the learned min-sum (the forward of nms_learned.cu, same results):
// the state keeps the raw minimum and second minimum (the weights differ per edge), and
// each edge's message magnitude is max(alpha m - beta, 0) with its own weights, the
// previous iteration's for the old message.  `first`: no old messages yet.
template <int D, typename Addr>
__device__ __forceinline__ void row_update_learned(float* __restrict__ post, const Addr& addr, const LearnedRowW& w,
                                                   int t, bool first, float a1, float a2, uint32_t mt, float& n1,
                                                   float& n2, uint32_t& nm) {
  int off[D];
  float x[D];
  const int old_i1 = (int)(mt & 31u);
  const uint32_t t0 = mt << (24 - D);
#pragma unroll
  for (int e = 0; e < D; e++) {
    off[e] = addr(e);
    const float p = ld_post(post, off[e]);
    if (first) {
      x[e] = __fsub_rn(p, 0.f);
    } else {
      const float mag = w.mag(w.a_prev, w.b_prev, e, (e == old_i1) ? a2 : a1);
      x[e] = ((t0 << e) & 0x80000000u) ? __fadd_rn(p, mag) : __fsub_rn(p, mag);
    }
  }
  float m1 = infinity<float>(), m2 = infinity<float>();
#pragma unroll
  for (int e = 0; e + 1 < D; e += 2) {
    const float s = min_xorsign_abs(x[e], x[e + 1]);
    const float l = fmaxf(fabsf(x[e]), fabsf(x[e + 1]));
    m2 = min3f(m2, fmaxf(fabsf(m1), fabsf(s)), l);
    m1 = min_xorsign_abs(m1, s);
  }
  if (D & 1) {
    m2 = fminf(m2, fmaxf(fabsf(m1), fabsf(x[D - 1])));
    m1 = min_xorsign_abs(m1, x[D - 1]);
  }
  const uint32_t ps = __float_as_uint(m1) & 0x80000000u;
  m1 = fabsf(m1);
  uint32_t sm = 0;
  int i1 = 0;
#pragma unroll
  for (int e = 0; e < D; e++) {
    const bool eq = fabsf(x[e]) == m1;
    i1 = eq ? e : i1;
    const float mag = w.mag(w.a_cur, w.b_cur, e, eq ? m2 : m1);
    const uint32_t ob = __float_as_uint(mag) | ((ps ^ __float_as_uint(x[e])) & 0x80000000u);
    st_post(post, off[e], __fadd_rn(x[e], __uint_as_float(ob)));
    sm = (sm << 1) | (ob >> 31);
  }
  n1 = m1;
  n2 = m2;
  nm = (sm << 8) | (uint32_t)i1;
}

template <typename Addr>
__device__ __forceinline__ void row_dispatch_learned(int d, float* post, const Addr& addr, const LearnedRowW& w, int t,
                                                     bool first, float a1, float a2, uint32_t mt, float& n1,
                                                     float& n2, uint32_t& nm) {
  switch (d) {
    case 3: row_update_learned<3>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 4: row_update_learned<4>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 5: row_update_learned<5>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 6: row_update_learned<6>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 7: row_update_learned<7>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 8: row_update_learned<8>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 9: row_update_learned<9>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    case 10: row_update_learned<10>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
    default: row_update_learned<19>(post, addr, w, t, first, a1, a2, mt, n1, n2, nm); break;
  }
}

template <int RULE, typename Addr>
__device__ __forceinline__ void row_dispatch_lean(int d, float* post, const Addr& addr, float a1, float a2,
                                                  uint32_t mt, float alpha, float& n1, float& n2, uint32_t& nm) {
  switch (d) {
    case 3: row_update_lean<3, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 4: row_update_lean<4, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 5: row_update_lean<5, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 6: row_update_lean<6, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 7: row_update_lean<7, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 8: row_update_lean<8, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 9: row_update_lean<9, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    case 10: row_update_lean<10, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
    default: row_update_lean<19, RULE>(post, addr, a1, a2, mt, alpha, n1, n2, nm); break;
  }
}

// the row update of the f64 decoder (f32 rows take row_dispatch_lean)
template <typename T, int RULE>
__device__ __forceinline__ void row_dispatch(int d, T* post, const uint32_t* ent, int r, int z, T a1, T a2,
                                             uint32_t mt, T alpha, T& n1, T& n2, uint32_t& nm) {
  switch (d) {
    case 3: row_update<T, 3, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 4: row_update<T, 4, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 5: row_update<T, 5, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 6: row_update<T, 6, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 7: row_update<T, 7, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 8: row_update<T, 8, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 9: row_update<T, 9, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    case 10: row_update<T, 10, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
    default: row_update<T, 19, RULE>(post, ent, r, z, a1, a2, mt, alpha, n1, n2, nm); break;
  }
}

// check-node state of one lifted row: f32 as an 8-byte {n1, n2} record plus a plane of
// meta words (12 bytes a row, so more of the slots stay in L2); f64 as a 16-byte
// {n1, n2} record plus a plane of meta words
template <typename T>
struct StateSlot;
// f32 state in two planes: {n1, n2} (8 bytes) and the meta word (4 bytes)
template <>
struct StateSlot<float> {
  uint2* mag;
  uint32_t* meta;
  uint64_t pol;
  __device__ __forceinline__ StateSlot(unsigned char* base, int rows)
      : mag(reinterpret_cast<uint2*>(base)), meta(reinterpret_cast<uint32_t*>(base + (size_t)rows * 8)),
        pol(l2_evict_last_policy()) {}
  __device__ __forceinline__ void load(int row, float& a1, float& a2, uint32_t& mt) const {
    uint32_t x, y, w;
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(x), "=r"(y) : "l"(mag + row), "l"(pol));
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(w) : "l"(meta + row), "l"(pol));
    a1 = __uint_as_float(x);
    a2 = __uint_as_float(y);
    mt = w;
  }
  __device__ __forceinline__ void store(int row, float n1, float n2, uint32_t nm) const {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(mag + row), "r"(__float_as_uint(n1)),
                 "r"(__float_as_uint(n2)), "l"(pol)
                 : "memory");
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(meta + row), "r"(nm), "l"(pol) : "memory");
  }
  static __host__ __device__ size_t bytes(int rows) { return (size_t)rows * 12; }
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

}  // namespace
}  // namespace cbk
