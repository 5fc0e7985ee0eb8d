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
};

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
  const uint64_t* jumps;       // [2 * threads][4]: jump polynomials of the chunk starts
  int32_t bits_per_chunk, syms_per_chunk, n_pad;
  T* llr_out;                  // [n_frames][E]
  uint32_t* info_out;          // [n_frames][ceil(K'/32)]
  // optional: per-frame Eb/N0 (dB; replaces b_ebn0 by b_bits * 10^(Eb/N0 / 10)) and the
  // full codeword, packed [n_frames][ceil(n_full/32)] (the targets of training)
  const float* ebn0_frames = nullptr;
  double b_bits = 0.0;
  uint32_t* cw_out = nullptr;
};
constexpr int kGenThreads = 128;

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
  int32_t multi_loss;       // 1: loss of every iteration's output, weight 1/T each
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

}  // namespace cbk
