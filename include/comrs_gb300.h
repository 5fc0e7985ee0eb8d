/* comrs_gb300.h -- C ABI of the GB300 BICM-LDPC Monte Carlo trial.
 *
 * The drop-in boundary of com-rs's BICM-LDPC hot path (5G NR LDPC encode, Gray QAM,
 * AWGN, max-log demap, layered min-sum decode, error counts) on one GPU.  Every call
 * returns a status; host buffers are caller-owned; device buffers belong to the code
 * object.  Calls on one code object are serialised by an internal mutex.
 *
 * Reference interfaces replaced (paths inside the com-rs project):
 *   cb_code_create        NrLdpc::with_options + LdpcDecoder settings
 *                         (crates/com-fec/src/nr/ldpc.rs:101-162,
 *                          crates/com-fec/src/ldpc.rs:165-172, :113-123)
 *   cb_encode             BlockCode::encode_block of NrLdpc (nr/ldpc.rs:209-214)
 *   cb_decode             BlockCode::decode_block / SoftDecode::app_into of NrLdpc
 *                         (nr/ldpc.rs:216-240), batched
 *   cb_run_frames         the body of Scenario::trial for a BICM-LDPC link, frame f
 *                         drawing from stream(seed, name, condition, f)
 *                         (crates/com-sim/src/runner.rs:435-447,
 *                          crates/com-sim/src/scenario.rs:201-219)
 *   status codes          com_core::Error::{Config, Shape, Numerical, Condition, Io}
 *                         (crates/com-core/src/error.rs:25-40)
 */
#ifndef COMRS_GB300_H
#define COMRS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CB_OK = 0,
  CB_ERR_CONFIG = -1,    /* invalid settings (Error::Config) */
  CB_ERR_SHAPE = -2,     /* wrong buffer sizes (Error::Shape) */
  CB_ERR_NUMERICAL = -3, /* Error::Numerical */
  CB_ERR_CONDITION = -4, /* Error::Condition */
  CB_ERR_IO = -5,        /* Error::Io */
  CB_ERR_CUDA = -6       /* a CUDA call failed */
} cb_status;
/* No kernel of this library waits on another kernel, another CTA or the host: work is
 * handed out by atomic counters and every launch ends on its own, so no call has a
 * device wait that could time out. */

typedef enum { CB_RULE_SUM_PRODUCT = 0, CB_RULE_NMS = 1, CB_RULE_OMS = 2 } cb_rule;
typedef enum { CB_F64 = 0, CB_F32 = 1 } cb_precision;

/* Code and decoder settings.  Keyword surface of the reference's Python NrLdpc
 * (bindings/com-py/src/fec/nr.rs:52-83). */
typedef struct {
  int32_t k_info;         /* K': information bits per code block */
  int32_t e;              /* E: transmitted bits (rate matching output) */
  int32_t base_graph;     /* 0: the TS 38.212 rule (nr/ldpc.rs:78-81); 1 or 2 forced */
  int32_t lifting_size;   /* 0: smallest Z with kb Z >= K' (nr/ldpc.rs:117-123); else forced */
  int32_t rv;             /* redundancy version 0..3 */
  int32_t qm;             /* bit interleaver rows (1: none) */
  int32_t rule;           /* cb_rule */
  double alpha;           /* NMS scale or OMS offset */
  int32_t layered;        /* 1: layered schedule (only layered is built on the GPU) */
  int32_t max_iterations; /* >= 0 */
  int32_t precision;      /* cb_precision: arithmetic of LLRs and messages */
  int32_t device;         /* CUDA device ordinal */
} cb_code_desc;

/* Per-frame record of cb_run_frames, in frame order (8 bytes). */
typedef struct {
  uint32_t bit_errors; /* errors among the K' information bits */
  uint8_t frame_error; /* bit_errors > 0 */
  uint8_t iterations;  /* decoder iterations (0: the channel word was a codeword) */
  uint16_t reserved;
} cb_frame_result;

typedef struct cb_code cb_code;

/* Library version string. */
const char* cb_version(void);

/* Build a code on a device.  *out is NULL on error; cb_last_error(NULL) names it. */
cb_status cb_code_create(const cb_code_desc* desc, cb_code** out);
void cb_code_destroy(cb_code* code);

/* The message of the last error of `code` (or of the calling thread when NULL). */
const char* cb_last_error(const cb_code* code);

/* The demapper of the frame generator (cb_run_frames, cb_generate_frames and the
 * learned decoder's training frames): 0 max-log (the default), 1 exact, the log-sum-exp
 * of each half of the labels (Jacobian::MaxLog / Jacobian::Exact of
 * crates/com-mapping/src/demapper.rs:82-146).  The exact demapper calls CUDA's exp and
 * log where the reference calls the platform libm. */
cb_status cb_code_set_demapper(cb_code* code, int32_t exact);

/* Compile, without a GPU, the decoders of an f32 layered min-sum code for its base graph
 * and lifting size (Z and every shift as constants: the plain rule's and the learned
 * min-sum's evaluation) and store them in the on-disk cache that the code's first device
 * call reads (for build steps that warm the cache).
 * CB_ERR_CONFIG for other codes, CB_ERR_IO when no compiler is found or it fails. */
cb_status cb_code_prepare(cb_code* code);

/* info[0..16): base graph, Z, K', E, K (systematic columns), n_full, lifted rows,
 * edges, iLS, max row degree, rv, qm, core-inverse terms, 1 if the rate matching is
 * the plain offset 2Z + t, base-graph entries, and the decoder that runs: -1 before the
 * code's first device call, 0 the generic layered decoder (f64, sum-product, flooding),
 * 1 the f32 layered min-sum built for the base graph, 2 the same compiled at run time for
 * this code's lifting size (Z and every shift as constants; needs the CUDA toolkit's nvcc
 * or libnvrtc, see COMRS_NO_JIT, COMRS_NVCC and COMRS_JIT_CACHE in the integration notes). */
cb_status cb_code_info(const cb_code* code, int64_t info[16]);

/* The construction tables: `entries` = n_entries records (base row, base column,
 * shift mod Z) in layer order; `bit_map` = the E rate-matching positions.  Either
 * pointer may be NULL.  Sizes from cb_code_info. */
cb_status cb_code_tables(const cb_code* code, int32_t* entries, int32_t* bit_map);

/* Encode n_frames blocks: info = n_frames x K' bytes (0/1), out = n_frames x E bytes. */
cb_status cb_encode(cb_code* code, const uint8_t* info, int64_t n_frames, uint8_t* out);

/* Decode n_frames blocks of E channel LLRs (double for CB_F64, float for CB_F32),
 * host buffers.  bits: n_frames x ceil(K'/8) bytes, packed LSB first (optional);
 * app: n_frames x K' a posteriori LLRs of the information bits (optional);
 * iterations: n_frames int32 (optional).  Page-locked LLRs (cudaHostAlloc,
 * cudaHostRegister) are read by the decoder in place; others are copied to the device in
 * chunks that overlap the decoding.  The results are the same. */
cb_status cb_decode(cb_code* code, const void* llr, int64_t n_frames, uint8_t* bits, void* app,
                    int32_t* iterations);

/* cb_decode on device buffers and a caller stream (cudaStream_t, NULL = default):
 * bits: n_frames x ceil(K'/32) uint32 words, packed LSB first.  The device calls of one
 * code object share its work counter and per-CTA state: enqueue them on one stream, or
 * let each finish before the next starts on another. */
cb_status cb_decode_device(cb_code* code, const void* llr_dev, int64_t n_frames, uint32_t* bits_dev,
                           void* app_dev, int32_t* iterations_dev, void* stream);

/* Monte Carlo frames [first_frame, first_frame + n_frames) of one condition: frame f
 * draws its K' bits, padding bits and noise from stream(seed, name, condition, f), with
 * name_hash = FNV-1a 64 of the scenario name (crates/com-core/src/rng.rs:58-65).
 * modulation_order: 4, 16, 64 or 256 (Gray square QAM, unit energy).  Results in
 * frame order into `out` (host, n_frames records). */
cb_status cb_run_frames(cb_code* code, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                        uint64_t condition, uint64_t first_frame, int64_t n_frames, double ebn0_db,
                        cb_frame_result* out);

/* The E channel LLRs and the K' information bits of frames [first_frame, +n_frames)
 * as cb_run_frames draws them (llr: n_frames x E, double or float by precision;
 * info: n_frames x K' bytes).  For checks and for LLR dumps. */
cb_status cb_generate_frames(cb_code* code, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                             uint64_t condition, uint64_t first_frame, int64_t n_frames, double ebn0_db,
                             void* llr, uint8_t* info);

/* cb_run_frames on a caller stream (cudaStream_t, NULL = default) with the per-frame
 * records in device memory (results_dev: n_frames records).  The LLR scratch belongs to
 * the code object.  Asynchronous: the caller synchronises its stream. */
cb_status cb_run_frames_device(cb_code* code, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                               uint64_t condition, uint64_t first_frame, int64_t n_frames, double ebn0_db,
                               cb_frame_result* results_dev, void* stream);

/* cb_generate_frames on a caller stream into device buffers: llr_dev n_frames x E
 * (double or float), info_dev n_frames x ceil(K'/32) uint32 words, LSB first. */
cb_status cb_generate_frames_device(cb_code* code, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                                    uint64_t condition, uint64_t first_frame, int64_t n_frames, double ebn0_db,
                                    void* llr_dev, uint32_t* info_dev, void* stream);

/* ---- Learned (neural) min-sum.  No counterpart in the reference: the layered min-sum
 * of cb_decode with, at iteration t and edge e, the check message
 * s * max(alpha[t,e] * m - beta[t,e], 0), trained on the GPU by its own forward and
 * backward kernels.  The plain normalised min-sum (alpha = the code's alpha, beta = 0)
 * is its starting point and its fallback.  Runs on an f32 code object, which must
 * outlive it.  Weights are indexed [t][entry][r] (per lifted edge: entry = base-graph
 * entry in table order, r = lifted row in its layer) or [t][entry] (shared = 1). */
typedef struct cb_nms cb_nms;
cb_status cb_nms_create(cb_code* code, int32_t iterations, int32_t shared, cb_nms** out);
void cb_nms_destroy(cb_nms* nms);
/* info[0..4): weights per kind, iterations, shared, training steps taken */
cb_status cb_nms_info(const cb_nms* nms, int64_t info[4]);
cb_status cb_nms_get_weights(cb_nms* nms, float* alpha, float* beta);
/* sets the weights and restarts the optimiser */
cb_status cb_nms_set_weights(cb_nms* nms, const float* alpha, const float* beta);
/* the n_full posteriors after exactly `iterations` iterations of n frames of E LLRs */
cb_status cb_nms_forward(cb_nms* nms, const float* llr, int64_t n_frames, float* post);
/* the bits the training loss covers: 0 all n_full codeword bits (the default), 1 the K'
 * information bits (the bits whose errors the frame error rate counts) */
cb_status cb_nms_set_loss_bits(cb_nms* nms, int32_t info_only);
/* the mean loss (binary cross-entropy of the soft output against the n_full codeword
 * bytes `cw`, over the bits of cb_nms_set_loss_bits; multi_loss 0: of the last output,
 * 1: the mean over the outputs of all T iterations, 2: their weighted mean with weights
 * 2 (t + 1) / (T (T + 1)), t = 0..T-1) of n frames and its gradients (nullable outputs) */
cb_status cb_nms_gradients(cb_nms* nms, const float* llr, const uint8_t* cw, int64_t n_frames, int32_t multi_loss,
                           float* g_alpha, float* g_beta, double* loss);
/* one Adam step (learning rate lr) on `batch` frames drawn by the frame generator at
 * Eb/N0 uniform in [ebn0_lo, ebn0_hi] dB (condition 2^64 - 1 of the stream, frames
 * step * batch + i); the batch's mean loss before the step into *loss */
cb_status cb_nms_train_step(cb_nms* nms, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                            int64_t batch, double ebn0_lo, double ebn0_hi, double lr, int32_t multi_loss,
                            double* loss);
/* decode n frames of E LLRs (host) with the learned decoder and the syndrome stop after
 * each iteration: the n_full posteriors (nullable) and the iterations used (nullable).
 * Runs the layered decoder with the network's weights (the same results as the
 * training forward, which runs all iterations) */
cb_status cb_nms_decode(cb_nms* nms, const float* llr, int64_t n_frames, float* post, int32_t* iterations);
/* the same on device buffers, enqueued on `stream` (cudaStream_t, NULL = default); it
 * runs on the code object's scratch, so the ordering rule of cb_decode_device holds */
cb_status cb_nms_decode_device(cb_nms* nms, const float* llr_dev, int64_t n_frames, float* post_dev,
                               int32_t* iterations_dev, void* stream);
/* cb_run_frames with the learned decoder (syndrome stop after each iteration) */
cb_status cb_nms_run_frames(cb_nms* nms, int32_t modulation_order, uint64_t seed, uint64_t name_hash,
                            uint64_t condition, uint64_t first_frame, int64_t n_frames, double ebn0_db,
                            cb_frame_result* out);

/* ---- Mixed batches: codewords of different base graphs, lifting sizes, rates,
 * modulations and Eb/N0 generated and decoded together.  The batch's codewords are
 * sorted by lifting size into classes; one persistent kernel decodes every class,
 * each CTA split into slots that take codewords from the class's queue one after
 * another (per-codeword early exit, work stealing).  Generator and decoder are
 * captured once as a CUDA graph and replayed by cb_mix_run.  Every record equals
 * cb_run_frames of the item's own code on the same stream position. */
typedef struct {
  int32_t base_graph;       /* 1 or 2 */
  int32_t lifting_size;     /* Z */
  int32_t k_info, e;        /* K' and E; the rate matching must be the plain 2Z + t */
  int32_t modulation_order; /* 4, 16, 64, 256 */
  int32_t reserved;
  double ebn0_db;
  uint64_t condition, frame; /* stream(seed, name, condition, frame + epoch * n_items) */
} cb_mix_item;
typedef struct cb_mix cb_mix;
cb_status cb_mix_create(const cb_mix_item* items, int64_t n_items, uint64_t seed, uint64_t name_hash, double alpha,
                        int32_t max_iterations, int32_t device, cb_mix** out);
void cb_mix_destroy(cb_mix* mix);
const char* cb_mix_last_error(const cb_mix* mix);
/* per class (up to `capacity`), 8 values: Z, codewords, rows per thread, slots per
 * CTA, threads per slot, shared bytes per slot, resident CTAs, first sorted item */
cb_status cb_mix_classes(const cb_mix* mix, int32_t capacity, int64_t* info, int32_t* n_classes);
/* the autotuner's knob: lifted rows per thread (1 or 2) of one class */
cb_status cb_mix_set_rows_per_thread(cb_mix* mix, int32_t class_index, int32_t rows_per_thread);
/* generate and decode the batch at `epoch` (replays the graph); records in the items'
 * order into `out` (host, n_items records; NULL to skip the copy) */
cb_status cb_mix_run(cb_mix* mix, uint64_t epoch, cb_frame_result* out);
/* the best of `reps` event-timed decode phases of one class (-1: all classes) */
cb_status cb_mix_time_decode(cb_mix* mix, int32_t class_index, int32_t reps, double* ms);
/* The frames the batch's generator writes at `epoch` (one replay): the f32 channel LLRs
 * the decoder reads and the K' information bits, in the items' order (item i's E_i LLRs,
 * then item i + 1's; llr: sum of E_i floats, info: sum of K'_i bytes 0/1; either may be
 * NULL).  For checks of the decoder against a reference decoder on the same LLRs. */
cb_status cb_mix_frames(cb_mix* mix, uint64_t epoch, float* llr, uint8_t* info);

/* ---- Generic sparse LDPC codes: LdpcCode::decode_llr (crates/com-fec/src/ldpc.rs:497-505)
 * for any parity-check matrix given by its rows (LdpcCode::from_rows / from_alist,
 * ldpc.rs:222-239, :350-370; PEG, IRA and DVB-S2 codes, or the lifted rows of an NR
 * code), with the decoder settings of LdpcDecoder (ldpc.rs:165-172): the sum-product,
 * normalised or offset min-sum rule (check_message, ldpc.rs:449-493), the layered or
 * flooding schedule (propagate, ldpc.rs:509-553).  Row r lists its variables at
 * vars[row_start[r] .. row_start[r + 1]) (0-based; each at most once per row); its
 * messages follow that order, as the reference's edges do.  The min-sum rules are
 * bit-exact in f64; the sum-product rule calls CUDA's tanh/atanh where the reference
 * calls the platform libm.  Device resources are made on the first decode. */
typedef struct cb_ldpc cb_ldpc;
cb_status cb_ldpc_create(int32_t n, int32_t m, const int32_t* row_start, const int32_t* vars, int32_t rule,
                         double alpha, int32_t layered, int32_t max_iterations, int32_t precision, int32_t device,
                         cb_ldpc** out);
void cb_ldpc_destroy(cb_ldpc* code);
/* the last error of `code` (or of the calling thread's last cb_ldpc call when NULL) */
const char* cb_ldpc_last_error(const cb_ldpc* code);
/* info[0..8): n, m, edges, largest row degree, largest column degree, levels of the
 * layered schedule, rows of its largest level, 1 if layered */
cb_status cb_ldpc_info(const cb_ldpc* code, int64_t info[8]);
/* the layered schedule: level_start[levels + 1] and level_rows[m] (nullable) */
cb_status cb_ldpc_levels(const cb_ldpc* code, int32_t* level_start, int32_t* level_rows);
/* decode n_frames words of n channel LLRs (host, f64 or f32 as the precision): the n
 * posteriors of every frame into `post` and the iterations used into `iterations`
 * (both host, nullable) */
cb_status cb_ldpc_decode(cb_ldpc* code, const void* llr, int64_t n_frames, void* post, int32_t* iterations);
/* the same on device buffers, enqueued on `stream` (cudaStream_t, NULL = default).  The
 * decodes of one code object share its work counter and message slots: enqueue them on
 * one stream, or let each finish before the next starts on another. */
cb_status cb_ldpc_decode_device(cb_ldpc* code, const void* llr_dev, int64_t n_frames, void* post_dev,
                                int32_t* iterations_dev, void* stream);
/* LdpcCode::set_decoder (bindings/com-py/src/fec/ldpc_code.rs:74-86): new decoder
 * settings, checked as cb_ldpc_create checks them; the device tables are rebuilt on the
 * next decode when the rule or the schedule changes, so no decode of this code may be
 * in flight on another stream */
cb_status cb_ldpc_set_decoder(cb_ldpc* code, int32_t rule, double alpha, int32_t layered, int32_t max_iterations);
/* LdpcCode::girth (ldpc.rs:412-446): the length of the shortest cycle of the Tanner
 * graph (0 without cycle); host only */
cb_status cb_ldpc_girth(const cb_ldpc* code, int32_t* girth);
/* The systematic encoder (host only; the encode calls below then run on the GPU):
 * CB_ENC_SUMS is that of LdpcCode::from_rows (ldpc.rs:216-231): H reduced with the
 * pivots searched from the last column (crates/com-math/src/gf2.rs:121-150), the
 * columns without a pivot the information positions, every pivot bit a sum of
 * information bits; CB_ENC_ACCUMULATE that of LdpcCode::accumulate (ldpc.rs:233-256):
 * the first n - m bits the information, parity bit n - m + r the running sum of checks
 * 0..r, for dual-diagonal (IRA) checks only (CB_ERR_CONFIG with the reference's message
 * otherwise).  Writes k and, when info_positions is not NULL, the k information
 * positions (at most n entries). */
#define CB_ENC_SUMS 0
#define CB_ENC_ACCUMULATE 1
cb_status cb_ldpc_set_encoder(cb_ldpc* code, int32_t kind, int32_t* k, int32_t* info_positions);
/* LdpcCode::encode_block (ldpc.rs:753-791) of n_frames blocks: k information bits per
 * frame (u8, bit 0 used) into n coded bits per frame (u8); host buffers.  Needs an
 * encoder (cb_ldpc_set_encoder). */
cb_status cb_ldpc_encode(cb_ldpc* code, const uint8_t* info, int64_t n_frames, uint8_t* coded);
/* the same on device buffers, enqueued on `stream` (cudaStream_t, NULL = default) */
cb_status cb_ldpc_encode_device(cb_ldpc* code, const uint8_t* info_dev, int64_t n_frames, uint8_t* coded_dev,
                                void* stream);
/* LdpcCode::peg (ldpc.rs:289-313, :586-634): the rows of a code of n variables and
 * n - k checks by progressive edge growth, every variable of degree var_degree, the
 * ties broken by Rng::new(seed) (crates/com-core/src/rng.rs); host only.  Writes
 * row_start[n - k + 1] and vars[n var_degree], each row's variables in the order they
 * were linked (the reference's rows, hence its alist files). */
cb_status cb_ldpc_peg(int32_t n, int32_t k, int32_t var_degree, uint64_t seed, int32_t* row_start, int32_t* vars);

/* ---- The link of a com-spec specification over a generic code: the blocks
 * fec_encode -> map -> awgn_ebn0 -> demap -> fec_decode of a Link (crates/com-spec/src/
 * link.rs:109-124) as specs/bicm_ldpc.yaml chains them, one trial per call unit:
 *   fec_encode (blocks/coding/fec.rs:60-78): k x blocks payload bits drawn with Rng::bit,
 *     every block encoded (the from_rows encoder), the codewords one after the other,
 *     then, when `interleave` is set, Interleaver::random(n x blocks, interleaver_seed);
 *   map (blocks/coding/map.rs:31-47): padding bits to a multiple of log2 M, Gray QAM;
 *   awgn_ebn0 (blocks/channel.rs:141-156): the measured mean power, b = log2 M k / n;
 *   demap (map.rs:55-77): exact (exact_demap = 1, the block's default) or max-log LLRs;
 *   fec_decode (fec.rs:88-102): deinterleave, decode every block with the code's decoder.
 * Trial t of condition c draws from stream(seed, name, c, t).  Per trial the counts of
 * the metrics (crates/com-spec/src/metrics.rs:254-351): ber (uncoded decisions of the
 * power-scaled samples by the grid slicer), coded_ber, bler.  The code object must have
 * the CB_ENC_SUMS encoder and outlive the link; both are used under their locks.  The
 * LLRs are computed in f64; a CB_F32 code decodes them rounded once to f32 (the
 * reference decodes in f64: a CB_F64 code is the parity configuration). */
typedef struct {
  uint32_t raw_bit_errors;   /* ber: errors of the n_sym log2 M sent bits */
  uint32_t coded_bit_errors; /* coded_ber: errors of the k x blocks payload bits */
  uint32_t block_errors;     /* bler: blocks with an error */
  uint32_t iterations;       /* decoder iterations summed over the blocks */
} cb_link_record;
typedef struct cb_link cb_link;
cb_status cb_link_create(cb_ldpc* code, int32_t blocks, int32_t modulation_order, int32_t interleave,
                         uint64_t interleaver_seed, int32_t exact_demap, cb_link** out);
void cb_link_destroy(cb_link* link);
const char* cb_link_last_error(const cb_link* link);
/* info[0..8): k, n, blocks, M, sent bits per trial (n x blocks + padding), payload bits
 * per trial, padding bits, 1 if interleaved */
cb_status cb_link_info(const cb_link* link, int64_t info[8]);
/* the interleaver's permutation perm[n x blocks]: stream bit t is coded bit perm[t]
 * (Interleaver::perm, crates/com-fec/src/interleaving.rs:52-55); host only */
cb_status cb_link_interleaver(const cb_link* link, int32_t* perm);
/* trials [first_trial, first_trial + n_trials) of one condition; records in trial order
 * into `out` (host) */
cb_status cb_link_run_trials(cb_link* link, uint64_t seed, uint64_t name_hash, uint64_t condition,
                             uint64_t first_trial, int64_t n_trials, double ebn0_db, cb_link_record* out);
/* cb_link_run_trials enqueued on `stream` (cudaStream_t, NULL = default) with the records in
 * device memory; the link's scratch holds at most 1 GB of trials per call (CB_ERR_SHAPE
 * beyond).  Asynchronous: the caller synchronises its stream.  It decodes with the code
 * object's scratch, so the rule of cb_ldpc_decode_device applies to the two together. */
cb_status cb_link_run_trials_device(cb_link* link, uint64_t seed, uint64_t name_hash, uint64_t condition,
                                    uint64_t first_trial, int64_t n_trials, double ebn0_db, cb_link_record* out_dev,
                                    void* stream);
/* the same trials' decoder inputs: llr [n_trials][n x blocks] (deinterleaved), payload
 * [n_trials][k x blocks] bytes and the uncoded bit errors [n_trials] (each nullable) */
cb_status cb_link_generate(cb_link* link, uint64_t seed, uint64_t name_hash, uint64_t condition,
                           uint64_t first_trial, int64_t n_trials, double ebn0_db, double* llr, uint8_t* payload,
                           uint32_t* raw_errors);

/* cb_decode_device for callers that cannot allocate device memory (a host framework
 * that owns all device memory through its own pool, or a real-time loop that forbids
 * cudaMalloc after start-up).  No counterpart in the reference: it is an addition of
 * this library.  Calls no cudaMalloc, cudaFree or allocating library routine: its
 * scratch (work counter and per-CTA check-node state) is a static 32 MiB device array
 * that every GPU loading the library holds until exit.  The first call on a device
 * looks up that array's device address; make that first call before any stream
 * capture.  All calls share the array, so calls that overlap on the GPU (two streams,
 * two threads) race: serialise them.  Codes whose per-CTA state exceeds the array
 * (CB_ERR_SHAPE) or whose rate matching is not the plain offset 2Z + t (rv 0, Qm 1, no
 * filler bits sent; CB_ERR_CONFIG) are rejected.  Fewer CTAs run when the state of
 * all resident CTAs does not fit, so large codes decode more slowly than with
 * cb_decode_device.  Outputs as cb_decode_device. */
cb_status cb_decode_device_noalloc(cb_code* code, const void* llr_dev, int64_t n_frames, uint32_t* bits_dev,
                                   int32_t* iterations_dev, void* stream);

/* The state of the xoshiro256** generator after `steps` draws from `state` (jump-ahead
 * by a polynomial; Rng::state / Rng::from_state, crates/com-core/src/rng.rs:83-96). */
cb_status cb_xoshiro_jump(const uint64_t state[4], uint64_t steps, uint64_t out[4]);

#ifdef __cplusplus
}
#endif

#endif /* COMRS_GB300_H */
