// Layered normalised/offset min-sum decoding of 5G NR LDPC codewords in f32, with the base
// graph's structure fixed at compile time.
//
// Restates LdpcCode::propagate and check_message (crates/com-fec/src/ldpc.rs:449-557) on
// the lifted NR graphs of crates/com-fec/src/nr/ldpc.rs:124-134, with the LLR placement of
// NrLdpc::full_llr (nr/ldpc.rs:191-197): the algorithm, the state layout and the results
// of the generic layered decoder (decode.cu), bit for bit.
//
// What is fixed at compile time: the rows of the base graph, their degrees and columns,
// and the level schedule (rows of one level share no column and run between the same two
// barriers).  Each row's update is specialised to its degree and to its entries'
// positions in the launch parameters, and the whole iteration is one straight-line body.
// The lifting is a policy: `RuntimeLifting` reads Z and the shifts from the launch
// parameters (the library's nvcc build, any code of the base graph); a `FixedLifting`
// with Z and all shifts as constants is generated per code and compiled at run time by
// NVRTC (decode_nr.cu), which turns every edge address into an immediate offset.
//
// This file is also NVRTC source: it includes only dev_math.cuh and the generated
// schedule, and uses no host headers.
#pragma once
#include "dev_math.cuh"

namespace cbn {
using namespace cbk;

#include "nr_bg_schedule.inc"

template <int BG>
struct Graph;
template <>
struct Graph<1> : BaseGraph1 {};
template <>
struct Graph<2> : BaseGraph2 {};

constexpr int kMaxEntries = 316;
constexpr int kMaxRows = 46;

// the per-frame record (cbd::FrameResult, cb_frame_result)
struct FrameRecord {
  uint32_t bit_errors;
  uint8_t frame_error;
  uint8_t iterations;
  uint16_t reserved;
};

// Launch parameters (plain data, the same layout under nvcc and NVRTC).
struct NrArgs {
  int32_t z, n_full, k, k_info, e, rows, n_entries;
  int32_t map_kind;          // 0: output bit t is full-word bit 2Z + t; 1: `map`; 2: `inv_*` (repeats)
  const int32_t* map;        // [E] full-word position of output bit t
  const int32_t* inv_start;  // [n_full + 1]
  const int32_t* inv_t;      // [E] output bits of full-word bit v, in increasing order
  int32_t max_iterations;
  int32_t rule;              // 1: normalised min-sum, 2: offset min-sum
  float alpha;               // the scale or the offset
  int32_t reserved;
  const float* llr;          // [n_frames][E]
  int64_t n_frames;
  uint32_t* bits_out;        // [n_frames][ceil(K'/32)] (optional)
  float* app_out;            // [n_frames][K'] (optional)
  int32_t* iters_out;        // [n_frames] (optional)
  const uint32_t* ref_bits;  // [n_frames][ceil(K'/32)] sent bits (optional)
  FrameRecord* results;      // [n_frames] (optional)
  unsigned char* state;      // per resident CTA: nr_state_bytes(rows Z)
  unsigned long long* work_counter;  // zeroed before the launch
  uint32_t entry[kMaxEntries];       // (column << 16) | shift, row-major
  uint2 eaddr[kMaxEntries];          // {4 shift, 4 column Z}
  uint16_t layer_start[kMaxRows + 1];
};

// the check-node state of a CTA: an 8-byte plane {n1, n2} and a 4-byte plane of meta words
// (bits 0-7 the edge whose message has the second minimum's magnitude, read as bits 0-4;
// bits 8.. the outgoing signs)
__host__ __device__ inline size_t nr_state_bytes(int lifted_rows) {
  return (((size_t)lifted_rows * 12) + 255) & ~(size_t)255;
}

__host__ __device__ inline size_t nr_smem_bytes(int n_full, int z, int rows, int n_entries) {
  const int ws = (z + 31) / 32 + 1;
  size_t b = (size_t)n_full * 4;
  b += (size_t)(n_full / z) * ws * 4;  // packed hard decisions
  b += (size_t)n_entries * 4;           // entries
  b += (size_t)(rows + 1) * 2 + 16;     // layer starts
  return (b + 15) & ~(size_t)15;
}

// The learned min-sum (shared weights per base-graph entry and iteration): the plain
// decoder's arguments, an optional full-posterior output, and the weights in the launch
// parameters (read through the constant cache: every thread of a CTA reads the same one).
constexpr int kNrMaxLearnedWeights = 3200;  // per kind: (iterations + 1) x entries
struct NrLearnedArgs {
  NrArgs a;
  float* post_out;  // [n_frames][n_full] a posteriori LLRs of the whole word (optional)
  float alpha[kNrMaxLearnedWeights];  // [1 + iteration][entry] scales (row 0: 0)
  float beta[kNrMaxLearnedWeights];   // [1 + iteration][entry] offsets (row 0: +inf)
};

// Weights of one iteration for the rows: none (the plain decoder's rule), or the
// learned scales and offsets of this iteration (cur) and of the previous one (prev, for
// the old messages), indexed by entry, as (scale, offset) pairs in shared memory.
struct NrNoWeights {
  static constexpr bool learned = false;
};
struct NrRowWeights {
  static constexpr bool learned = true;
  const float2 *prev, *cur;
  __device__ __forceinline__ float ap(int i) const { return prev[i].x; }
  __device__ __forceinline__ float bp(int i) const { return prev[i].y; }
  __device__ __forceinline__ float ac(int i) const { return cur[i].x; }
  __device__ __forceinline__ float bc(int i) const { return cur[i].y; }
};
struct NrNoWeightSet {
  static constexpr bool learned = false;
  __device__ __forceinline__ NrNoWeights at(int) const { return {}; }
};
// The weight rows [T + 1][entries] of the launch parameters: row t + 1 holds iteration
// t's, row 0 the scale 0 and the offset +inf, whose magnitude max(0 m - inf, 0) is 0 for
// every old message of the first iteration (which has none): no branch on the first
// iteration in the rows.  Each iteration's row is staged in shared memory, in the buffer
// the iteration before last used (two buffers of `ne` pairs): the rows then read them
// with one 8-byte shared load per edge and message (10.2 against 11.6 ms for 8192 C2
// codewords and 10 iterations reading the launch parameters through a pointer, 10.3 from
// a constant array).
struct NrParamWeightSet {
  static constexpr bool learned = true;
  float2* buf;  // shared memory: 2 x ne pairs
  const float* alpha;
  const float* beta;
  int ne;  // entries
  __device__ __forceinline__ NrRowWeights at(int t) const {
    float2* cur = buf + ((t + 1) & 1) * ne;
    for (int i = threadIdx.x; i < ne; i += blockDim.x)
      cur[i] = make_float2(alpha[(t + 1) * ne + i], beta[(t + 1) * ne + i]);
    if (t == 0) {
      float2* first = buf + (t & 1) * ne;
      for (int i = threadIdx.x; i < ne; i += blockDim.x) first[i] = make_float2(alpha[i], beta[i]);
    }
    __syncthreads();
    return {buf + (t & 1) * ne, cur};
  }
};

// shared memory of the learned kernel: the plain decoder's and the two weight buffers
__host__ __device__ inline size_t nr_learned_smem_bytes(int n_full, int z, int rows, int n_entries) {
  return nr_smem_bytes(n_full, z, rows, n_entries) + (size_t)n_entries * 2 * sizeof(float2);
}

// Z and the shifts from the launch parameters
struct RuntimeLifting {
  static constexpr bool fixed = false;
  static constexpr int z = 0;
  static constexpr int shift[1] = {0};
  static constexpr int rule = 0;  // the min-sum rule from the launch parameters
};

// How many rows ahead of its update a row's check-node state is loaded (0: at the row's
// start), per lifting policy; the results are the same.  Fixed lifting: two (C2, 8192
// codewords on GB300: 15.32 ms, one row ahead 15.53, none 16.1, before the multiply-add
// output choice).  Runtime lifting: the registers of the loads in flight make that
// kernel spill (23.5 ms with two rows ahead, 17.4 with none).
template <class K>
struct NrTuning {
  static constexpr int ahead = K::fixed ? 2 : 0;
};

// Byte offset in the posteriors of entry T's variable for lifted row r (r4 = 4 r):
// 4 (column Z + (r + shift) mod Z).  Since r + shift < 2Z, the residue is the unsigned
// minimum of u = 4 (r + shift) and u - 4Z (one `viaddmin`); with a fixed lifting the
// column's offset is an immediate of the shared-memory access.  (A comparison of r with
// Z - shift selecting between two immediates issues more instructions: 17.6 against
// 16.7 ms per 8192 C2 codewords.)
template <int BG, class K, int T>
__device__ __forceinline__ int edge_offset(const NrArgs& a, int r, int r4, int z4) {
  if constexpr (K::fixed) {
    constexpr int sh = K::shift[T], c = Graph<BG>::col[T];
    const uint32_t u = (uint32_t)r4 + (uint32_t)(4 * sh);
    return 4 * c * K::z + (int)__viaddmin_u32(u, (uint32_t)(-4 * K::z), u);
  } else {
    // r + shift < 2Z: (r + shift) mod Z is the unsigned minimum of u and u - Z
    const uint2 t = a.eaddr[T];
    const uint32_t u = (uint32_t)r4 + t.x;
    return (int)(t.y + __viaddmin_u32(u, (uint32_t)-z4, u));
  }
}

// the edge offsets of a row, entries S0 + I .. S0 + D - 1 (a compile-time loop)
template <int BG, class K, int S0, int I, int D>
__device__ __forceinline__ void row_offsets(int (&off)[D], const NrArgs& a, int r, int r4, int z4) {
  if constexpr (I < D) {
    off[I] = edge_offset<BG, K, S0 + I>(a, r, r4, z4);
    row_offsets<BG, K, S0, I + 1, D>(off, a, r, r4, z4);
  }
}

__device__ __forceinline__ float ld_f(const unsigned char* post, int off) {
  return *reinterpret_cast<const float*>(post + off);
}
__device__ __forceinline__ void st_f(unsigned char* post, int off, float v) {
  *reinterpret_cast<float*>(post + off) = v;
}

// One lifted row of base row L (degree D, entries S0 ..): old state (a1, a2, mt) -> new
// state (n1, n2, nm), posteriors updated in place.  The operations of row_update_lean
// (decode_common.cuh), with the addresses from edge_offset.
template <int BG, class K, int S0, int D, int RULE>
__device__ __forceinline__ void nr_row(unsigned char* post, const NrArgs& a, int r, int r4, int z4, float a1,
                                       float a2, uint32_t mt, float alpha, float& n1, float& n2, uint32_t& nm) {
  int off[D];
  float x[D];
  const int old_i1 = (int)(mt & 31u);
  const uint32_t t0 = mt << (24 - D);  // the old sign of edge 0 at bit 31
  row_offsets<BG, K, S0, 0, D>(off, a, r, r4, z4);
#pragma unroll
  for (int i = 0; i < D; i++) {
    const float mag = (i == old_i1) ? a2 : a1;
    // p - (s ? -mag : mag) as p + (the negated old message)
    const uint32_t neg = (__float_as_uint(mag) ^ 0x80000000u) ^ ((t0 << i) & 0x80000000u);
    x[i] = __fadd_rn(ld_f(post, off[i]), __uint_as_float(neg));
  }
  float m1 = __int_as_float(0x7f800000), m2 = __int_as_float(0x7f800000);
#pragma unroll
  for (int i = 0; i + 1 < D; i += 2) {
    const float s = min_xorsign_abs(x[i], x[i + 1]);
    const float l = fmaxf(fabsf(x[i]), fabsf(x[i + 1]));
    m2 = min3f(m2, fmaxf(fabsf(m1), fabsf(s)), l);
    m1 = min_xorsign_abs(m1, s);
  }
  if (D & 1) {
    m2 = fminf(m2, fmaxf(fabsf(m1), fabsf(x[D - 1])));
    m1 = min_xorsign_abs(m1, x[D - 1]);
  }
  const uint32_t ps = __float_as_uint(m1) & 0x80000000u;
  m1 = fabsf(m1);
  if constexpr (RULE == 1) {  // normalised min-sum
    n1 = __fmul_rn(alpha, m1);
    n2 = __fmul_rn(alpha, m2);
  } else {  // offset min-sum
    n1 = fmaxf(__fsub_rn(m1, alpha), 0.0f);
    n2 = fmaxf(__fsub_rn(m2, alpha), 0.0f);
  }
  const uint32_t n1p = __float_as_uint(n1) | ps, n2p = __float_as_uint(n2) | ps;
  // Each edge's magnitude is n2 where |x| equals the minimum, else n1.  The choice is an
  // integer multiply-add by the comparison's mask (0 or all ones), which runs on the FMA
  // pipe beside the ALU-bound rest (14.5 against 15.2 ms per 8192 C2 codewords with two
  // selects).  The same multiply-add sums the indices of those edges: when one edge holds
  // the minimum the sum is its index; when several tie, m1 = m2, the two magnitudes of
  // the state are equal and any index gives the same old messages.  The sum (at most
  // 0 + 1 + ... + 18) stays below the sign bits at bit 8.
  // (The runtime-lifting build: 17.4 against 18.6 ms.)
  const uint32_t dneg = n1p - n2p;
  uint32_t sm = 0, i1 = 0;
#pragma unroll
  for (int i = 0; i < D; i++) {
    uint32_t eqm, magp;
    asm("set.eq.u32.f32 %0, %1, %2;" : "=r"(eqm) : "f"(fabsf(x[i])), "f"(m1));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(magp) : "r"(eqm), "r"(dneg), "r"(n1p));
    if (i) asm("mad.lo.u32 %0, %1, %2, %0;" : "+r"(i1) : "r"(eqm), "r"((uint32_t)-i));
    const uint32_t ob = magp ^ (__float_as_uint(x[i]) & 0x80000000u);
    st_f(post, off[i], __fadd_rn(x[i], __uint_as_float(ob)));
    sm = (sm << 1) | (ob >> 31);
  }
  nm = (sm << 8) | i1;
}

// The learned message magnitude max(alpha m - beta, 0), alpha m - beta rounded once (a
// fused multiply-add) as the training forward (nms_learned.cu) and LearnedRowW
// (decode_common.cuh) compute it.  fmaxf agrees with their `am > 0 ? am : 0` except
// perhaps on the sign of a zero from am = -0; a message of magnitude zero adds or
// subtracts zero whatever its sign, so the posteriors are the same bits (the sign bit kept
// for it only ever multiplies that zero again).
__device__ __forceinline__ float learned_mag(float al, float be, float m) {
  return fmaxf(__fmaf_rn(al, m, -be), 0.f);
}

// One lifted row of the learned min-sum (row_update_learned of decode_common.cuh, with
// the addresses from edge_offset and the weights of entry S0 + i): the state keeps the
// raw minimum and second minimum, each edge's message magnitude is max(alpha m - beta, 0)
// with its own weights, the previous iteration's for the old message (in the first
// iteration the state is zero and the weight row gives 0: x = p - 0, as the training
// forward's first iteration).
// The row's update from its edge offsets; s0 is its first entry (the weights' index).
template <int D, class RW>
__device__ __forceinline__ void nr_row_learned_at(unsigned char* post, const int (&off)[D], int s0, const RW& w,
                                                  float a1, float a2, uint32_t mt, float& n1, float& n2,
                                                  uint32_t& nm) {
  float x[D];
  const int old_i1 = (int)(mt & 31u);
  const uint32_t t0 = mt << (24 - D);
#pragma unroll
  for (int i = 0; i < D; i++) {
    const float mag = learned_mag(w.ap(s0 + i), w.bp(s0 + i), (i == old_i1) ? a2 : a1);
    const uint32_t neg = (__float_as_uint(mag) ^ 0x80000000u) ^ ((t0 << i) & 0x80000000u);
    x[i] = __fadd_rn(ld_f(post, off[i]), __uint_as_float(neg));
  }
  float m1 = __int_as_float(0x7f800000), m2 = __int_as_float(0x7f800000);
#pragma unroll
  for (int i = 0; i + 1 < D; i += 2) {
    const float s = min_xorsign_abs(x[i], x[i + 1]);
    const float l = fmaxf(fabsf(x[i]), fabsf(x[i + 1]));
    m2 = min3f(m2, fmaxf(fabsf(m1), fabsf(s)), l);
    m1 = min_xorsign_abs(m1, s);
  }
  if (D & 1) {
    m2 = fminf(m2, fmaxf(fabsf(m1), fabsf(x[D - 1])));
    m1 = min_xorsign_abs(m1, x[D - 1]);
  }
  const uint32_t ps = __float_as_uint(m1) & 0x80000000u;
  m1 = fabsf(m1);
  // the raw magnitude m2 where |x| equals the minimum, else m1, and the index sum, by the
  // multiply-adds of nr_row
  const uint32_t dneg = __float_as_uint(m1) - __float_as_uint(m2);
  uint32_t sm = 0, i1 = 0;
#pragma unroll
  for (int i = 0; i < D; i++) {
    uint32_t eqm, mb;
    asm("set.eq.u32.f32 %0, %1, %2;" : "=r"(eqm) : "f"(fabsf(x[i])), "f"(m1));
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(mb) : "r"(eqm), "r"(dneg), "r"(__float_as_uint(m1)));
    if (i) asm("mad.lo.u32 %0, %1, %2, %0;" : "+r"(i1) : "r"(eqm), "r"((uint32_t)-i));
    const float mag = learned_mag(w.ac(s0 + i), w.bc(s0 + i), __uint_as_float(mb));
    const uint32_t ob = __float_as_uint(mag) | ((ps ^ __float_as_uint(x[i])) & 0x80000000u);
    st_f(post, off[i], __fadd_rn(x[i], __uint_as_float(ob)));
    sm = (sm << 1) | (ob >> 31);
  }
  n1 = m1;
  n2 = m2;
  nm = (sm << 8) | i1;
}

template <int BG, class K, int S0, int D, class RW>
__device__ __forceinline__ void nr_row_learned(unsigned char* post, const NrArgs& a, int r, int r4, int z4,
                                               const RW& w, float a1, float a2, uint32_t mt, float& n1, float& n2,
                                               uint32_t& nm) {
  int off[D];
  row_offsets<BG, K, S0, 0, D>(off, a, r, r4, z4);
  nr_row_learned_at<D>(post, off, S0, w, a1, a2, mt, n1, n2, nm);
}

struct NrState {
  unsigned char* mag;
  unsigned char* meta;
  uint64_t pol;
  __device__ __forceinline__ void load(int row, float& a1, float& a2, uint32_t& mt) const {
    uint32_t x, y, w;
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(x), "=r"(y)
                 : "l"(mag + (size_t)row * 8), "l"(pol));
    asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(w) : "l"(meta + (size_t)row * 4), "l"(pol));
    a1 = __uint_as_float(x);
    a2 = __uint_as_float(y);
    mt = w;
  }
  __device__ __forceinline__ void store(int row, float n1, float n2, uint32_t nm) const {
    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(mag + (size_t)row * 8),
                 "r"(__float_as_uint(n1)), "r"(__float_as_uint(n2)), "l"(pol)
                 : "memory");
    asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;" ::"l"(meta + (size_t)row * 4), "r"(nm), "l"(pol)
                 : "memory");
  }
};

// The learned rows 0-3 of base graph 1 (degree 19 each, the schedule's first four levels)
// as one rolled loop over a single copy of their code, their edge offsets from the launch
// parameters' table: the kernel's code shrinks by a fifth, for a few more instructions
// on a quarter of the edges.
__device__ __forceinline__ void nr_dense_rows_bg1(unsigned char* post, const NrArgs& a, const NrState& st,
                                                  const NrRowWeights& w, int tid, int r4, int z4, int z, bool active,
                                                  bool first) {
#pragma unroll 1
  for (int q = 0; q < 4; q++) {
    if (active) {
      float a1 = 0.0f, a2 = 0.0f, n1, n2;
      uint32_t mt = 0, nm;
      if (!first) st.load(q * z + tid, a1, a2, mt);
      int off[19];
#pragma unroll
      for (int i = 0; i < 19; i++) {
        const uint2 t = a.eaddr[19 * q + i];
        const uint32_t u = (uint32_t)r4 + t.x;
        off[i] = (int)(t.y + __viaddmin_u32(u, (uint32_t)-z4, u));
      }
      nr_row_learned_at<19>(post, off, 19 * q, w, a1, a2, mt, n1, n2, nm);
      st.store(q * z + tid, n1, n2, nm);
    }
    __syncthreads();
  }
}

// One layered iteration: the rows in schedule order, a barrier after each level.  With
// NrTuning::ahead = 2 the state of row Q arrives as a*, that of row Q + 1 as b*, and row
// Q + 2's is loaded here (c*), so that the L2 latency of the loads is not the first wait
// of every row; with ahead = 0 each row loads its own state.
template <int BG, class K, int Q, int RULE, class W>
__device__ __forceinline__ void nr_iteration(unsigned char* post, const NrArgs& a, const NrState& st, int r, int r4,
                                             int z4, int z, bool active, bool first, float alpha, const W& w,
                                             float a1, float a2, uint32_t mt, float b1, float b2, uint32_t bt) {
  if constexpr (Q < Graph<BG>::rows) {
    constexpr int L = Graph<BG>::order[Q];
    constexpr int S0 = Graph<BG>::start[L];
    constexpr int D = Graph<BG>::start[L + 1] - S0;
    constexpr int ahead = NrTuning<K>::ahead;
    const int zz = K::fixed ? K::z : z;
    float c1 = 0.0f, c2 = 0.0f;
    uint32_t ct = 0;
    if constexpr (ahead == 2 && Q + 2 < Graph<BG>::rows) {
      if (active && !first) st.load(Graph<BG>::order[Q + 2] * zz + r, c1, c2, ct);
    }
    if (active) {
      // the row index passes through an empty asm so that the compiler recomputes each
      // row's addresses where they are used instead of hoisting all of them out of the
      // iteration loop (they would not fit in registers)
      int rr = r, rr4 = r4;
      asm volatile("" : "+r"(rr), "+r"(rr4));
      if constexpr (ahead == 0) {
        if (!first) st.load(L * zz + rr, a1, a2, mt);
      }
      float n1, n2;
      uint32_t nm;
      if constexpr (W::learned)
        nr_row_learned<BG, K, S0, D>(post, a, rr, rr4, z4, w, a1, a2, mt, n1, n2, nm);
      else
        nr_row<BG, K, S0, D, RULE>(post, a, rr, rr4, z4, a1, a2, mt, alpha, n1, n2, nm);
      st.store(L * zz + rr, n1, n2, nm);
    }
    if constexpr (Graph<BG>::level_end[Q] != 0) __syncthreads();
    nr_iteration<BG, K, Q + 1, RULE>(post, a, st, r, r4, z4, z, active, first, alpha, w, b1, b2, bt, c1, c2, ct);
  }
}

// the parity (sign bits of the hard decisions) of lifted row r of base row L: entries
// T .. TE - 1 at compile time
template <int BG, class K, int T, int TE>
__device__ __forceinline__ uint32_t row_parity(const unsigned char* post, const NrArgs& a, int r, int r4, int z4) {
  if constexpr (T < TE) {
    return (uint32_t)(ld_f(post, edge_offset<BG, K, T>(a, r, r4, z4)) < 0.0f) ^
           row_parity<BG, K, T + 1, TE>(post, a, r, r4, z4);
  } else {
    return 0u;
  }
}

// some_check_fails (dev_math.cuh) with stage 1, the rows of the first two base rows, at
// compile time: the same answer, exactly "H c != 0" (C2 on GB300, runtime lifting: 18.2
// against 18.6 ms per 8192 codewords)
template <int BG, class K>
__device__ __forceinline__ bool some_nr_check_fails(const float* post, uint32_t* hd, const uint32_t* ent,
                                                    const uint16_t* lstart, const NrArgs& a, int ncol, int z, int tid,
                                                    int nt, int r4, int z4) {
  int bad = 0;
  if (tid < z) {
    int rr = tid, rr4 = r4;
    asm volatile("" : "+r"(rr), "+r"(rr4));
    const unsigned char* p = reinterpret_cast<const unsigned char*>(post);
    bad = (int)row_parity<BG, K, Graph<BG>::start[0], Graph<BG>::start[1]>(p, a, rr, rr4, z4);
    if (!bad) bad = (int)row_parity<BG, K, Graph<BG>::start[1], Graph<BG>::start[2]>(p, a, rr, rr4, z4);
  }
  if (__syncthreads_or(bad)) return true;
  return some_packed_check_fails(post, hd, ent, lstart, a.rows, ncol, z, tid, nt);
}

// The decoder arguments, the learned weights (none for the plain rule) and the whole
// word's a posteriori output of a launch's parameters.
__device__ __forceinline__ const NrArgs& nr_args_of(const NrArgs& p) { return p; }
__device__ __forceinline__ const NrArgs& nr_args_of(const NrLearnedArgs& p) { return p.a; }
__device__ __forceinline__ NrNoWeightSet nr_weights_of(const NrArgs&) { return {}; }
__device__ __forceinline__ NrParamWeightSet nr_weights_of(const NrLearnedArgs& p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const NrArgs& a = p.a;
  float2* buf = reinterpret_cast<float2*>(smem + nr_smem_bytes(a.n_full, a.z, a.rows, a.n_entries));
  return {buf, p.alpha, p.beta, a.n_entries};
}
__device__ __forceinline__ float* nr_post_out_of(const NrArgs&) { return nullptr; }
__device__ __forceinline__ float* nr_post_out_of(const NrLearnedArgs& p) { return p.post_out; }

// Persistent decoder: each CTA takes codewords from the work counter, one thread per
// lifted row, posteriors in shared memory, check-node state in its own L2-resident slot.
// P = NrArgs: the plain rule; P = NrLearnedArgs: the learned min-sum with shared weights
// (its a.max_iterations is the network's T).  The body stays in the kernel: as a device
// function taking the parameters by reference the plain decoder ran 9 % slower.
template <int BG, class K, class P = NrArgs>
__global__ void __launch_bounds__(384, 2) layered_nr_kernel(const __grid_constant__ P p) {
  const NrArgs& a = nr_args_of(p);
  const auto wset = nr_weights_of(p);
  float* const post_out = nr_post_out_of(p);
  extern __shared__ __align__(16) unsigned char smem[];
  const int z = K::fixed ? K::z : a.z;
  const int nt = blockDim.x, tid = threadIdx.x;
  const int n_full = a.n_full, ncol = n_full / z;
  const int ws = (z + 31) / 32 + 1;
  float* post = reinterpret_cast<float*>(smem);
  uint32_t* hd = reinterpret_cast<uint32_t*>(post + n_full);
  uint32_t* s_ent = hd + ncol * ws;
  uint16_t* s_lstart = reinterpret_cast<uint16_t*>(s_ent + a.n_entries);
  __shared__ long long s_cw;
  __shared__ unsigned int s_err;
  const int lifted = a.rows * z;
  unsigned char* slot = a.state + (size_t)blockIdx.x * nr_state_bytes(lifted);
  const NrState st{slot, slot + (size_t)lifted * 8, l2_evict_last_policy()};
  const bool nms = a.rule == 1;
  const float alpha = a.alpha;
  const int max_it = a.max_iterations;
  const int wpf = (a.k_info + 31) >> 5;
  const bool active = tid < z;
  const int r4 = 4 * tid, z4 = 4 * z;
  for (int i = tid; i < a.n_entries; i += nt) s_ent[i] = a.entry[i];
  for (int i = tid; i <= a.rows; i += nt) s_lstart[i] = a.layer_start[i];

  for (;;) {
    if (tid == 0) {
      s_cw = (long long)atomicAdd(a.work_counter, 1ull);
      s_err = 0;
    }
    __syncthreads();
    const long long cw = s_cw;
    if (cw >= a.n_frames) break;

    // ---- channel LLRs of the full word (NrLdpc::full_llr): 0.0 + LLR, punctured and
    // unsent bits 0.0, fillers KNOWN_BIT_LLR
    const float* llr = a.llr + (size_t)cw * a.e;
    for (int v = tid; v < n_full; v += nt) post[v] = 0.0f;
    __syncthreads();
    if (a.map_kind == 0) {
      if ((a.e & 3) == 0 && (reinterpret_cast<uintptr_t>(a.llr) & 15) == 0) {
        const float4* l4 = reinterpret_cast<const float4*>(llr);
        for (int q = tid; q < (a.e >> 2); q += nt) {
          const float4 v = __ldcs(l4 + q);
          float* d = post + 2 * z + 4 * q;
          d[0] = __fadd_rn(0.0f, v.x);
          d[1] = __fadd_rn(0.0f, v.y);
          d[2] = __fadd_rn(0.0f, v.z);
          d[3] = __fadd_rn(0.0f, v.w);
        }
      } else {
        for (int t = tid; t < a.e; t += nt) post[2 * z + t] = __fadd_rn(0.0f, __ldcs(llr + t));
      }
    } else if (a.map_kind == 1) {
      for (int t = tid; t < a.e; t += nt) post[a.map[t]] = __fadd_rn(0.0f, __ldcs(llr + t));
    } else {
      for (int v = tid; v < n_full; v += nt) {
        const int b0 = a.inv_start[v], b1 = a.inv_start[v + 1];
        if (b0 == b1) continue;
        float s = 0.0f;
        for (int i = b0; i < b1; i++) s = __fadd_rn(s, llr[a.inv_t[i]]);
        post[v] = s;
      }
    }
    __syncthreads();
    for (int v = a.k_info + tid; v < a.k; v += nt) post[v] = 30.0f;  // KNOWN_BIT_LLR, signal.rs:37
    __syncthreads();

    // ---- propagate (ldpc.rs:509-551): syndrome test before the first iteration and after each
    int it = 0;
    // (the test before the first iteration, once per codeword, runs the table-driven
    // stage 1: with the compile-time one here too the kernel spills registers)
    if (some_check_fails(post, hd, s_ent, s_lstart, a.rows, ncol, z, tid, nt)) {
      it = max_it;
      for (int iter = 1; iter <= max_it; iter++) {
        float a1 = 0.0f, a2 = 0.0f, b1 = 0.0f, b2 = 0.0f;
        uint32_t mt = 0, bt = 0;
        unsigned char* pb = reinterpret_cast<unsigned char*>(post);
        // (rows 0-3 first in the schedule, in order, 19 entries each; the loop's barrier after
        // each of them is the schedule's, as each is a level of its own)
        constexpr bool DENSE = decltype(wset)::learned && K::fixed && BG == 1 && Graph<BG>::order[0] == 0 &&
                               Graph<BG>::order[1] == 1 && Graph<BG>::order[2] == 2 && Graph<BG>::order[3] == 3 &&
                               Graph<BG>::start[4] == 76;
        if constexpr (DENSE) {
          // the learned min-sum on base graph 1: rows 0-3 in a rolled loop, then the rest
          const auto w = wset.at(iter - 1);
          nr_dense_rows_bg1(pb, a, st, w, tid, r4, z4, z, active, iter == 1);
          if (active && iter != 1) {
            st.load(Graph<BG>::order[4] * z + tid, a1, a2, mt);
            st.load(Graph<BG>::order[5] * z + tid, b1, b2, bt);
          }
          nr_iteration<BG, K, 4, K::rule>(pb, a, st, tid, r4, z4, z, active, iter == 1, alpha, w, a1, a2, mt, b1, b2,
                                          bt);
        } else {
        if constexpr (NrTuning<K>::ahead == 2) {
          if (active && iter != 1) {
            st.load(Graph<BG>::order[0] * z + tid, a1, a2, mt);
            st.load(Graph<BG>::order[1] * z + tid, b1, b2, bt);
          }
        }
        // the min-sum rule at compile time: the code's own when the lifting is fixed, else
        // one branch around the whole iteration (read in the rows, the compiler computed
        // both rules' magnitudes in every row: 14.7 against 14.2 ms per 8192 C2 codewords)
        if constexpr (K::rule != 0) {
          nr_iteration<BG, K, 0, K::rule>(pb, a, st, tid, r4, z4, z, active, iter == 1, alpha, wset.at(iter - 1), a1,
                                          a2, mt, b1, b2, bt);
        } else if (nms) {
          nr_iteration<BG, K, 0, 1>(pb, a, st, tid, r4, z4, z, active, iter == 1, alpha, wset.at(iter - 1), a1, a2, mt,
                                    b1, b2, bt);
        } else {
          nr_iteration<BG, K, 0, 2>(pb, a, st, tid, r4, z4, z, active, iter == 1, alpha, wset.at(iter - 1), a1, a2, mt,
                                    b1, b2, bt);
        }
        }
        if (!some_nr_check_fails<BG, K>(post, hd, s_ent, s_lstart, a, ncol, z, tid, nt, r4, z4)) {
          it = iter;
          break;
        }
      }
    }

    // ---- outputs: hard decisions (signal.rs:47-49), counts (errors.rs:39-42); the decision
    // words are staged in hd and written 16 bytes at a time when the row of words allows it
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    // the sent words, one per thread, loaded before the decisions are formed so that
    // their latency overlaps the ballots (a load per warp and word after each ballot
    // made the epilogue wait on memory K'/32/warps times per codeword)
    const uint32_t* ref = a.ref_bits ? a.ref_bits + (size_t)cw * wpf : nullptr;
    const uint32_t ref_w = (ref && tid < wpf) ? ref[tid] : 0u;
    for (int b0 = warp * 32; b0 < a.k_info; b0 += nw * 32) {
      const int v = b0 + lane;
      const bool bit = v < a.k_info && post[v] < 0.0f;
      const uint32_t word = __ballot_sync(0xffffffffu, bit);
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
      for (int v = tid; v < a.k_info; v += nt) a.app_out[(size_t)cw * a.k_info + v] = post[v];
    if (post_out)
      for (int v = tid; v < n_full; v += nt) post_out[(size_t)cw * n_full + v] = post[v];
    if (be) atomicAdd(&s_err, be);
    __syncthreads();
    if (tid == 0) {
      if (a.iters_out) a.iters_out[cw] = it;
      if (a.results) {
        FrameRecord rec;
        rec.bit_errors = s_err;
        rec.frame_error = s_err > 0;
        rec.iterations = (uint8_t)it;
        rec.reserved = 0;
        a.results[cw] = rec;
      }
    }
    __syncthreads();
  }
}

}  // namespace cbn
