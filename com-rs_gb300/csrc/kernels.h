// Host-side launchers of the CUDA kernels (decode.cu, gen.cu), called by the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device_common.cuh"

namespace cbk {

// Decoder launch: n_frames codewords of E channel LLRs each (element type T).
template <typename T>
struct DecodeArgs {
  cbd::DevCode code;
  cbd::DecCfg cfg;
  const T* llr;             // [n_frames][E]
  int64_t n_frames;
  uint32_t* bits_out;       // [n_frames][ceil(K'/32)] packed hard decisions, LSB first (optional)
  T* app_out;               // [n_frames][K'] a posteriori LLRs (optional)
  T* post_out;              // [n_frames][n_full] all posteriors (optional)
  int32_t* iters_out;       // [n_frames] (optional)
  const uint32_t* ref_bits; // [n_frames][ceil(K'/32)] sent info bits (optional)
  cbd::FrameResult* results;  // [n_frames] counts against ref_bits (optional)
  T* state;                 // check-node state, state_bytes_per_slot() per resident CTA
  int32_t* work_counter;    // zeroed before the launch
  int32_t* status;          // error word (0 = ok)
  // learned min-sum (f32): the check message of iteration t, edge e is
  // s max(alpha[t,e] m - beta[t,e], 0); weights [t][entry] (shared) or [t][entry][r]
  const float* l_alpha = nullptr;
  const float* l_beta = nullptr;
  int32_t l_shared = 0;
  int32_t l_smem = 0;  // 1: each iteration's (shared) weights staged in shared memory
};

// The learned decoder with its weights in the launch parameters (weights shared across
// Z, at most kMaxParamWeights per kind): warp-uniform reads through the constant cache.
constexpr int kMaxParamWeights = 3200;
struct LearnedParamArgs {
  DecodeArgs<float> d;
  float alpha[kMaxParamWeights];
  float beta[kMaxParamWeights];
};
cudaError_t launch_decode_learned_param(const LearnedParamArgs& a, int grid, cudaStream_t stream);

// the number of resident CTAs the persistent decoder launches and the state each needs
int decode_grid_size(const cbd::DevCode& code, int precision, int device);
size_t decode_state_bytes_per_slot(const cbd::DevCode& code, int precision);
template <typename T>
cudaError_t launch_decode(const DecodeArgs<T>& a, int grid, cudaStream_t stream);

// Frame generation: info bits, NR encode, rate matching, Gray QAM map, measured-power
// AWGN, max-log demap.  One CTA per frame.
template <typename T>
struct GenArgs {
  cbd::DevCode code;
  int32_t m, mbits;            // modulation order and bits per symbol
  const double* points;        // [2 m] normalised points (re, im interleaved), f64
  double log_m;                // ln M (the uniform log-prior of the demapper)
  double b_ebn0;               // (log2 M * R) * db2lin(Eb/N0), computed on the host
  uint64_t seed, name_hash, cond, first_frame;
  int64_t n_frames;
  const uint64_t* jumps;       // [bits + noise threads + 1][4]: jump polynomials of the chunk starts
  int32_t bits_per_chunk, syms_per_chunk, n_pad;
  T* llr_out;                  // [n_frames][E]
  uint32_t* info_out;          // [n_frames][ceil(K'/32)]
  // optional: per-frame Eb/N0 (dB; replaces b_ebn0 by b_bits * 10^(Eb/N0 / 10)) and the
  // full codeword, packed [n_frames][ceil(n_full/32)] (the targets of training)
  const float* ebn0_frames = nullptr;
  double b_bits = 0.0;
  uint32_t* cw_out = nullptr;
  int32_t exact = 0;           // demapper: 1 Jacobian::Exact (log-sum-exp), 0 max-log
};
constexpr int kGenThreads = 128;
// The NR frame generator (gen_one) draws the information bits with its first warp and the
// noise with the other three, whose threads jump to their noise chunks while the first
// warp draws the bits: 128 jumps a frame instead of 256 (a jump costs about 256 steps of
// the generator, four times a bit chunk's own draws).
constexpr int kGenBitsThreads = 32;
constexpr int kGenNoiseThreads = kGenThreads - kGenBitsThreads;

// The generation parameters of one frame (everything but the code).
template <typename T>
struct GenFrame {
  int32_t m, mbits, n_pad, bits_per_chunk, syms_per_chunk;
  const double* points;
  double log_m, b_ebn0;
  const uint64_t* jumps;
  uint64_t seed, name_hash, cond, frame_index;
  T* llr_out;          // this frame's E LLRs
  uint32_t* info_out;  // its packed info bits
  uint32_t* cw_out;    // its packed codeword (optional)
  int32_t exact;       // demapper: 1 exact (log-sum-exp), 0 max-log
};

// ---- mixed batches (mix.cu, gen.cu): codewords of different codes in one launch
// per (code, modulation) pair: the generator's tables
struct GenConfig {
  int32_t m, mbits, n_pad, bits_per_chunk, syms_per_chunk;
  const double* points;
  double log_m;
  const uint64_t* jumps;
};
// one codeword of a mixed batch
struct MixItem {
  int32_t code;         // index into the batch's codes
  int32_t config;       // index into the batch's generator configs
  uint64_t cond, frame; // its stream position: stream(seed, name, cond, frame)
  double b_ebn0;        // (log2 M * R) * db2lin(Eb/N0), computed on the host
  int64_t llr_offset;   // its LLRs in the batch buffer (elements)
  int64_t info_offset;  // its packed info bits (words)
  int32_t index;        // its position in the caller's order (the result slot)
  int32_t reserved;
};
struct GenMixArgs {
  const cbd::DevCode* codes;
  const GenConfig* configs;
  const MixItem* items;
  int64_t n_items;
  uint64_t seed, name_hash;
  const uint64_t* epoch;   // optional: frames advance by epoch * epoch_stride per replay
  uint64_t epoch_stride;
  float* llr;
  uint32_t* info;
};
cudaError_t launch_gen_mix(const GenMixArgs& a, size_t smem, cudaStream_t stream);

// a lifting-size class of a mixed batch and its slot layout in a 384-thread CTA
struct MixClass {
  int32_t z, slot_threads, slots, rows_per_thread;
  int64_t first, count;  // its items in the sorted batch
  int32_t smem_per_slot, state_per_slot, max_ncol, reserved;
};
struct MixDecodeArgs {
  const cbd::DevCode* codes;
  const MixItem* items;     // sorted by class
  const MixClass* classes;
  int32_t n_classes, rule, max_it;
  float alpha;
  const float* llr;
  const uint32_t* info;
  cbd::FrameResult* results;  // by MixItem::index
  unsigned long long* counters;  // one queue per class
  unsigned char* state;
  size_t state_per_cta;
};
size_t mix_slot_smem_bytes(int z);
int mix_decode_grid(size_t smem, int device);
cudaError_t launch_mix_decode(const MixDecodeArgs& a, int grid, size_t smem, cudaStream_t stream);
size_t gen_smem_bytes(const cbd::DevCode& c, int m, int mbits, int n_pad);

// Learned min-sum (nms_learned.cu): forward (training or evaluation) and backward.
struct LearnedArgs {
  cbd::DevCode code;
  int32_t T;           // unrolled iterations
  int32_t shared;      // 1: weights per base-graph edge, 0: per lifted edge
  int32_t early_stop;  // 1: syndrome stop after each iteration (evaluation)
  const float* alpha;  // scales, then
  const float* beta;   // offsets
  const float* llr;    // [n_frames][E]
  int64_t n_frames;
  const uint32_t* cw_bits;  // [n_frames][ceil(n_full/32)] targets (training)
  float* X;                 // [n_frames][T][edges] saved inputs (training)
  float* c2v;               // [n_frames][edges] messages, then their gradients
  float* post_out;          // [n_frames][n_full]
  float* loss;              // sum over frames of the mean bit loss (training)
  float* P;                 // [n_frames][T][n_full] posteriors after each iteration (multi-loss)
  int32_t multi_loss;       // 0: last output; 1: every iteration's, 1/T each; 2: ramp 2(t+1)/(T(T+1))
  int32_t loss_bits;        // the loss covers codeword bits [0, loss_bits): n_full, or K' (the information bits)
  float* g_alpha;           // gradients of the mean loss (backward)
  float* g_beta;
  const uint32_t* ref_bits;   // evaluation: sent info bits
  cbd::FrameResult* results;  // evaluation records
  int32_t* iters_out;
};
size_t learned_smem_bytes(const cbd::DevCode& code);
cudaError_t launch_learned(const LearnedArgs& a, bool forward, cudaStream_t stream);
cudaError_t launch_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, int step,
                        cudaStream_t stream);
template <typename T>
cudaError_t launch_gen(const GenArgs<T>& a, cudaStream_t stream);

// ---- generic sparse codes (sparse.cu)
struct SparseDev {
  int32_t n, m, edges, levels;
  const int32_t* row_start;    // m + 1
  const int32_t* vars;         // edges
  const int32_t* col_start;    // n + 1
  const int32_t* col_edges;    // edges, per variable in row order
  const int32_t* level_start;  // levels + 1
  const int32_t* level_rows;   // m
  // transposed layout of the messages (global-memory messages, a thread per row): edge k
  // of the row at schedule position p is slot k m + p, and tvars[k m + p] its variable;
  // col_edges then holds slots.  Null: the row-major layout of the edges.
  const int32_t* tvars;        // max row degree x m
  int32_t slots;               // message slots of one buffer: edges, or max row degree x m
};
template <typename T>
struct SparseArgs {
  SparseDev code;
  double alpha;  // NMS scale or OMS offset
  int32_t max_iterations;
  int32_t post_in_smem;  // 1: the posteriors live in shared memory, else in `slots` too
  int32_t msgs_in_smem;  // 1: the edge messages live in shared memory, else in `slots`
  int32_t warp_rows;     // layered: one warp per row (levels of few rows), else one thread
  int32_t has_aux;       // 1: a second buffer of `slots` (flooding's new messages, or the
                         // sum-product rule's prefix products when they are not in registers)
  int32_t group;         // codewords per CTA (sparse_group_kernel; 1 for sparse_kernel)
  const T* llr;          // [n_frames][n]
  int64_t n_frames;
  T* post_out;           // [n_frames][n] (nullable)
  int32_t* iters_out;    // [n_frames] (nullable)
  T* slots;              // [grid][(1 + has_aux) slots (+ n when !post_in_smem)] when !msgs_in_smem
  unsigned long long* work_counter;
};
// the kernel of a precision (0: f64, 1: f32), rule and schedule; regs: the layered
// sum-product rows in registers, for codes whose rows have at most kRegRowDegree edges
constexpr int kRegRowDegree = 8;
void* sparse_kernel_ptr(int precision, int rule, bool layered, bool regs);
// the layered kernel with several codewords per CTA (small codes: messages and
// posteriors of the group in shared memory, one thread per row)
constexpr int kMaxGroup = 8;
void* sparse_group_kernel_ptr(int precision, int rule, bool regs);
cudaError_t launch_sparse(void* kernel, const void* args, int grid, int threads, size_t smem, cudaStream_t stream);

// ---- systematic encoders of generic codes (sparse_encode.cu)
struct SumsEncodeArgs {
  const uint8_t* info;      // [n_frames][k]
  uint8_t* coded;           // [n_frames][n]
  int64_t n_frames;
  int32_t k, n, rank, words;
  const int32_t* info_pos;  // k
  const int32_t* pivots;    // rank
  const uint32_t* pmat;     // words x rank, word-major
};
struct AccumulateEncodeArgs {
  const uint8_t* info;       // [n_frames][k]
  uint8_t* coded;            // [n_frames][n]
  int64_t n_frames;
  int32_t k, n, m;
  const int32_t* row_start;  // m + 1
  const int32_t* vars;       // edges
};
size_t sums_encode_smem(int words);
size_t accumulate_encode_smem(int k, int m);
cudaError_t launch_sums_encode(const SumsEncodeArgs& a, cudaStream_t stream);
cudaError_t launch_accumulate_encode(const AccumulateEncodeArgs& a, cudaStream_t stream);

// ---- the link of a specification over a generic code (link.cu)
struct LinkRecord {
  uint32_t raw_bit_errors;    // metric ber: uncoded errors of the trial's symbols
  uint32_t coded_bit_errors;  // metric coded_ber: errors of the decoded payload
  uint32_t block_errors;      // metric bler: blocks with an error
  uint32_t iterations;        // decoder iterations summed over the blocks
};
struct LinkGenArgs {
  int32_t k, n, blocks, rank;
  const int32_t* info_pos;   // k
  const int32_t* pivots;     // rank
  const uint32_t* pmat;      // ceil(k/32) x rank, word-major
  const int32_t* perm;       // n x blocks interleaver (null: none)
  int32_t m, mbits, n_pad, bits_per_chunk, syms_per_chunk;
  const double* points;      // [2 m]
  double log_m, b_ebn0;
  int32_t exact;
  const uint64_t* jumps;     // [2 threads + 1][4]
  // the grid slicer of the metric ber
  int32_t side;
  double step, re0, im0;
  const int32_t* lookup;     // [m]: the label of cell (row, col) at row * side + col
  uint64_t seed, name_hash, cond, first_trial;
  int64_t n_trials;
  double* llr_out;           // [n_trials][n x blocks], deinterleaved (f64 decoder)
  float* llr_out_f32;        // the same rounded to f32 (f32 decoder); one of the two is null
  uint32_t* payload_out;     // [n_trials][blocks][ceil(k/32)]
  uint32_t* raw_errors_out;  // [n_trials]
};
struct LinkCountArgs {
  int32_t k, n, blocks;
  const int32_t* info_pos;
  const double* post;        // [n_trials x blocks][n] (f64 decoder)
  const float* post_f32;     // the same from an f32 decoder; one of the two is null
  const int32_t* iters;      // [n_trials x blocks]
  const uint32_t* payload;   // [n_trials][blocks][ceil(k/32)]
  const uint32_t* raw_errors;
  int64_t n_trials;
  LinkRecord* out;
};
size_t link_gen_smem_bytes(int m, int mbits, int k, int n, int blocks, int n_pad);
cudaError_t launch_link_gen(const LinkGenArgs& a, cudaStream_t stream);
cudaError_t launch_link_count(const LinkCountArgs& a, cudaStream_t stream);

// ---- the NR code through the generic decoder (nr_generic.cu)
template <typename T>
struct NrEpilogueArgs {
  const T* post;          // [n_frames][n_full]
  const int32_t* iters_in;  // [n_frames]
  int64_t n_frames;
  int32_t n_full, k_info;
  uint32_t* bits_out;       // [n_frames][ceil(K'/32)] (nullable)
  T* app_out;               // [n_frames][K'] (nullable)
  int32_t* iters_out;       // (nullable)
  const uint32_t* ref_bits;   // sent info bits (nullable)
  cbd::FrameResult* results;  // (nullable)
};
template <typename T>
cudaError_t launch_full_llr(const cbd::DevCode& code, const T* llr, int64_t n_frames, T* full, cudaStream_t stream);
template <typename T>
cudaError_t launch_nr_epilogue(const NrEpilogueArgs<T>& a, cudaStream_t stream);

}  // namespace cbk
