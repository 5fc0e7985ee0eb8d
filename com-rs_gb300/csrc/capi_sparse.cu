// The C ABI of generic sparse LDPC codes (cb_ldpc_* of include/comrs_gb300.h):
// LdpcCode::decode_llr (crates/com-fec/src/ldpc.rs:497-505) on the GPU for any
// parity-check matrix, with the decoder settings of LdpcDecoder (ldpc.rs:165-172);
// LdpcCode::encode_block (ldpc.rs:753-791) on the GPU with the encoder of from_rows or
// accumulate; and the host-side constructions (progressive edge growth, girth).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/comrs_gb300.h"
#include "kernels.h"
#include "sparse_host.h"

namespace {

thread_local std::string g_ldpc_thread_error;

// shared memory the edge messages may take before they move to global slots: keeps
// two CTAs resident per SM; and the posteriors, before they move there too
constexpr size_t kSmemMsgBudget = 100 * 1024;
constexpr size_t kSmemPostBudget = 200 * 1024;
// shared memory of a CTA of several small codewords: two CTAs per SM
constexpr size_t kGroupSmem = 100 * 1024;

}  // namespace

struct cb_ldpc {
  std::mutex mu;
  int device = 0, precision = 0, rule = 0, layered = 1, max_iterations = 0;
  double alpha = 0;
  cbh::SparseCode host;
  bool dev_ready = false;
  cbk::SparseDev dev{};
  int32_t* d_tables = nullptr;
  unsigned long long* d_counter = nullptr;
  void* d_slots = nullptr;
  int grid = 0, threads = 0;
  size_t smem = 0;
  bool msgs_in_smem = false;
  bool post_in_smem = true;
  bool warp_rows = false;
  bool regs = false;     // layered sum-product rows in registers
  bool has_aux = true;   // a second message buffer
  int group = 1;         // codewords per CTA
  void* kernel = nullptr;
  cudaStream_t stream = nullptr;
  void* d_llr = nullptr;
  size_t llr_cap = 0;
  void* d_post = nullptr;
  size_t post_cap = 0;
  int32_t* d_iters = nullptr;
  size_t iters_cap = 0;
  // the systematic encoder: host tables, their device copy, staging buffers
  cbh::SparseEncoder enc;
  bool enc_ready = false;
  int32_t* d_enc = nullptr;
  void* d_info = nullptr;
  size_t info_cap = 0;
  void* d_coded = nullptr;
  size_t coded_cap = 0;
  mutable std::string err;  // the last error, set by const calls too
};

namespace {

cb_status lfail(const cb_ldpc* c, cb_status s, const std::string& msg) {
  if (c) c->err = msg;
  g_ldpc_thread_error = msg;
  return s;
}

#define LDPC_CUDA(c, call)                                                                      \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return lfail((c), CB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

cudaError_t grow_buf(void** ptr, size_t& cap, size_t bytes) {
  if (bytes <= cap) return cudaSuccess;
  const size_t want = std::max(bytes, cap * 3 / 2);
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(ptr, want);
  if (e == cudaSuccess) cap = want;
  return e;
}

size_t elem(const cb_ldpc* c) { return c->precision == CB_F64 ? 8 : 4; }

// device tables, launch shape and message storage, on first use
cb_status ensure_stream(cb_ldpc* c) {
  LDPC_CUDA(c, cudaSetDevice(c->device));
  if (!c->stream) LDPC_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  return CB_OK;
}

// the decoder's device tables and message slots (the stream and the staging buffers stay)
void release_decoder(cb_ldpc* c) {
  if (!c->dev_ready) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->d_tables);
  cudaFree(c->d_counter);
  cudaFree(c->d_slots);
  c->d_tables = nullptr;
  c->d_counter = nullptr;
  c->d_slots = nullptr;
  c->dev = cbk::SparseDev{};
  c->dev_ready = false;
}

cb_status ensure_device(cb_ldpc* c) {
  if (c->dev_ready) return CB_OK;
  const cbh::SparseCode& h = c->host;
  if (cb_status st = ensure_stream(c)) return st;
  // the launch shape decides the message layout: a thread per row with messages in
  // global memory takes the transposed one
  c->warp_rows = c->layered && h.max_level_rows <= 8 && h.max_row_degree <= 128;
  // rows of few edges keep the sum-product's tanh values and prefix products in registers;
  // a second message buffer is then needed by the flooding schedule, or by the
  // sum-product rule on longer rows (one thread a row)
  c->regs = c->layered && c->rule == CB_RULE_SUM_PRODUCT && !c->warp_rows && h.max_row_degree <= cbk::kRegRowDegree;
  c->has_aux = !c->layered || (c->rule == CB_RULE_SUM_PRODUCT && !c->warp_rows && !c->regs);
  const size_t post_bytes = (size_t)h.n * elem(c);
  const size_t msg_bytes_rm = (size_t)(c->has_aux ? 2 : 1) * h.edges * elem(c);
  c->msgs_in_smem = post_bytes + msg_bytes_rm <= kSmemMsgBudget;
  c->post_in_smem = post_bytes <= kSmemPostBudget;
  const bool transposed = !c->msgs_in_smem && !c->warp_rows;
  std::vector<int32_t> tvars, col_slots;
  if (transposed) {
    // position of every row in the schedule: its place in the level order (layered) or
    // its index (flooding)
    std::vector<int32_t> pos(h.m);
    for (int i = 0; i < h.m; i++) pos[c->layered ? h.level_rows[i] : i] = i;
    const size_t nslot = (size_t)h.max_row_degree * h.m;
    tvars.assign(nslot, 0);
    std::vector<int32_t> slot_of_edge(h.edges);
    for (int r = 0; r < h.m; r++)
      for (int e = h.row_start[r]; e < h.row_start[r + 1]; e++) {
        const size_t sl = (size_t)(e - h.row_start[r]) * h.m + pos[r];
        tvars[sl] = h.vars[e];
        slot_of_edge[e] = (int32_t)sl;
      }
    col_slots.resize(h.edges);
    for (int k = 0; k < h.edges; k++) col_slots[k] = slot_of_edge[h.col_edges[k]];
  }
  const size_t words = h.row_start.size() + h.vars.size() + h.col_start.size() + h.col_edges.size() +
                       h.level_start.size() + h.level_rows.size() + tvars.size();
  LDPC_CUDA(c, cudaMalloc(&c->d_tables, words * 4));
  int32_t* p = c->d_tables;
  auto put = [&](const std::vector<int32_t>& v, const int32_t*& dst) -> cudaError_t {
    dst = p;
    cudaError_t e = cudaMemcpy(p, v.data(), v.size() * 4, cudaMemcpyHostToDevice);
    p += v.size();
    return e;
  };
  cbk::SparseDev& d = c->dev;
  d.n = h.n;
  d.m = h.m;
  d.edges = h.edges;
  d.levels = h.levels;
  LDPC_CUDA(c, put(h.row_start, d.row_start));
  LDPC_CUDA(c, put(h.vars, d.vars));
  LDPC_CUDA(c, put(h.col_start, d.col_start));
  LDPC_CUDA(c, put(transposed ? col_slots : h.col_edges, d.col_edges));
  LDPC_CUDA(c, put(h.level_start, d.level_start));
  LDPC_CUDA(c, put(h.level_rows, d.level_rows));
  d.tvars = nullptr;
  if (transposed) LDPC_CUDA(c, put(tvars, d.tvars));
  d.slots = transposed ? (int32_t)((size_t)h.max_row_degree * h.m) : h.edges;
  LDPC_CUDA(c, cudaMalloc(&c->d_counter, sizeof(unsigned long long)));
  // threads: a level's rows (layered), one warp per row when the levels hold few rows
  // (at most 8) of at most 128 edges, else a thread per row; a share of the rows and
  // variables (flooding)
  if (c->warp_rows) {
    c->threads = 32 * h.max_level_rows;
  } else {
    const int want = c->layered ? h.max_level_rows : std::max(h.m, h.n) / 4;
    c->threads = std::min(512, std::max(64, (want + 31) / 32 * 32));
  }
  const size_t msg_bytes = (size_t)(c->has_aux ? 2 : 1) * d.slots * elem(c);
  c->smem = c->msgs_in_smem ? ((post_bytes + msg_bytes + 15) & ~(size_t)15)
                            : (c->post_in_smem ? ((post_bytes + 15) & ~(size_t)15) : 0);
  const size_t slot_bytes = msg_bytes + (c->post_in_smem ? 0 : post_bytes);
  c->kernel = cbk::sparse_kernel_ptr(c->precision == CB_F64 ? 0 : 1, c->rule, c->layered != 0, c->regs);
  // small layered codes with one thread per row: several codewords per CTA (up to
  // kGroupSmem of shared memory), so that the rows of a level fill the warps
  c->group = 1;
  if (c->layered && !c->warp_rows && c->msgs_in_smem) {
    const size_t per = (h.n + (size_t)(c->has_aux ? 2 : 1) * h.edges) * elem(c);
    c->group = (int)std::min<size_t>(cbk::kMaxGroup, kGroupSmem / per);
    if (c->group >= 2) {
      c->kernel = cbk::sparse_group_kernel_ptr(c->precision == CB_F64 ? 0 : 1, c->rule, c->regs);
      c->smem = (c->group * per + 15) & ~(size_t)15;
      c->threads = std::min(512, (c->group * h.max_level_rows + 31) / 32 * 32);
    } else {
      c->group = 1;
    }
  }
  LDPC_CUDA(c, cudaFuncSetAttribute(c->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
  int per_sm = 0, sms = 0;
  LDPC_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c->kernel, c->threads, c->smem));
  LDPC_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  c->grid = std::max(1, per_sm * sms);
  if (!c->msgs_in_smem) {
    // the global slots of all resident CTAs, at most 2 GB
    const int cap = (int)std::max<size_t>(1, ((size_t)2 << 30) / slot_bytes);
    c->grid = std::min(c->grid, cap);
    LDPC_CUDA(c, cudaMalloc(&c->d_slots, (size_t)c->grid * slot_bytes));
  }
  c->dev_ready = true;
  return CB_OK;
}

template <typename T>
cb_status decode_impl(cb_ldpc* c, const T* llr, int64_t n, T* post, int32_t* iters, cudaStream_t s) {
  if (n == 0) return CB_OK;
  cbk::SparseArgs<T> a;
  a.code = c->dev;
  a.alpha = c->alpha;
  a.max_iterations = c->max_iterations;
  a.msgs_in_smem = c->msgs_in_smem ? 1 : 0;
  a.post_in_smem = c->post_in_smem ? 1 : 0;
  a.warp_rows = c->warp_rows ? 1 : 0;
  a.has_aux = c->has_aux ? 1 : 0;
  a.group = c->group;
  a.llr = llr;
  a.n_frames = n;
  a.post_out = post;
  a.iters_out = iters;
  a.slots = reinterpret_cast<T*>(c->d_slots);
  a.work_counter = c->d_counter;
  LDPC_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), s));
  const int grid = (int)std::min<int64_t>(c->grid, (n + c->group - 1) / c->group);
  LDPC_CUDA(c, cbk::launch_sparse(c->kernel, &a, grid, c->threads, c->smem, s));
  return CB_OK;
}

// shared memory the encoders may take per CTA
constexpr size_t kEncodeSmemLimit = 200 * 1024;

// the encoder's tables on the device: sums: info positions, pivots, packed rows;
// accumulate: the rows of H
cb_status ensure_encoder(cb_ldpc* c) {
  if (c->enc.kind == cbh::kEncoderNone)
    return lfail(c, CB_ERR_CONFIG, "the code has no encoder: call cb_ldpc_set_encoder first");
  if (c->enc_ready) return CB_OK;
  if (cb_status st = ensure_stream(c)) return st;
  const cbh::SparseEncoder& e = c->enc;
  const cbh::SparseCode& h = c->host;
  std::vector<int32_t> tab;
  if (e.kind == cbh::kEncoderSums) {
    if (cbk::sums_encode_smem(e.words) > kEncodeSmemLimit)
      return lfail(c, CB_ERR_CONFIG, "k = " + std::to_string(e.k) + " is too large for the encoder");
    tab.insert(tab.end(), e.info.begin(), e.info.end());
    tab.insert(tab.end(), e.pivots.begin(), e.pivots.end());
    for (uint32_t w : e.pmat) tab.push_back((int32_t)w);
  } else {
    if (cbk::accumulate_encode_smem(e.k, h.m) > kEncodeSmemLimit)
      return lfail(c, CB_ERR_CONFIG, "n = " + std::to_string(h.n) + " is too large for the encoder");
    tab.insert(tab.end(), h.row_start.begin(), h.row_start.end());
    tab.insert(tab.end(), h.vars.begin(), h.vars.end());
  }
  LDPC_CUDA(c, cudaMalloc(&c->d_enc, std::max<size_t>(1, tab.size()) * 4));
  LDPC_CUDA(c, cudaMemcpy(c->d_enc, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
  c->enc_ready = true;
  return CB_OK;
}

cb_status encode_impl(cb_ldpc* c, const uint8_t* info, int64_t n, uint8_t* coded, cudaStream_t s) {
  if (n == 0) return CB_OK;
  const cbh::SparseEncoder& e = c->enc;
  const cbh::SparseCode& h = c->host;
  if (e.kind == cbh::kEncoderSums) {
    cbk::SumsEncodeArgs a;
    a.info = info;
    a.coded = coded;
    a.n_frames = n;
    a.k = e.k;
    a.n = h.n;
    a.rank = (int32_t)e.pivots.size();
    a.words = e.words;
    a.info_pos = c->d_enc;
    a.pivots = c->d_enc + e.k;
    a.pmat = reinterpret_cast<const uint32_t*>(c->d_enc + e.k + e.pivots.size());
    LDPC_CUDA(c, cbk::launch_sums_encode(a, s));
  } else {
    cbk::AccumulateEncodeArgs a;
    a.info = info;
    a.coded = coded;
    a.n_frames = n;
    a.k = e.k;
    a.n = h.n;
    a.m = h.m;
    a.row_start = c->d_enc;
    a.vars = c->d_enc + h.m + 1;
    LDPC_CUDA(c, cbk::launch_accumulate_encode(a, s));
  }
  return CB_OK;
}

cb_status check_decoder_settings(int32_t rule, double alpha, int32_t max_iterations) {
  if (rule != CB_RULE_SUM_PRODUCT && rule != CB_RULE_NMS && rule != CB_RULE_OMS)
    return lfail(nullptr, CB_ERR_CONFIG, "rule must be sum-product, normalised or offset min-sum");
  if (max_iterations < 0) return lfail(nullptr, CB_ERR_CONFIG, "max_iterations must be >= 0");
  if (!std::isfinite(alpha)) return lfail(nullptr, CB_ERR_CONFIG, "alpha must be finite");
  return CB_OK;
}

}  // namespace

// ------------------------------------------------------------------ the spec link
struct cb_link {
  std::mutex mu;
  cb_ldpc* code = nullptr;
  int blocks = 1, m = 0, mbits = 0, n_pad = 0, bpc = 0, spc = 0, exact = 0;
  bool interleave = false;
  uint64_t il_seed = 0;
  double log_m = 0;
  std::vector<double> pts;
  std::vector<uint64_t> jumps;
  std::vector<int32_t> perm, lookup;
  int side = 0;
  double step = 0, re0 = 0, im0 = 0;
  bool dev_ready = false;
  int32_t* d_tab = nullptr;   // perm (n x blocks, when interleaved) then lookup (m)
  double* d_points = nullptr;
  uint64_t* d_jumps = nullptr;
  void* d_llr = nullptr;
  size_t llr_cap = 0;
  void* d_post = nullptr;
  size_t post_cap = 0;
  void* d_iters = nullptr;
  size_t iters_cap = 0;
  void* d_payload = nullptr;
  size_t payload_cap = 0;
  void* d_raw = nullptr;
  size_t raw_cap = 0;
  void* d_rec = nullptr;
  size_t rec_cap = 0;
  mutable std::string err;  // the last error, set by const calls too
};

namespace {

thread_local std::string g_link_thread_error;

cb_status kfail(const cb_link* l, cb_status s, const std::string& msg) {
  if (l) l->err = msg;
  g_link_thread_error = msg;
  return s;
}

#define LINK_CUDA(l, call)                                                                      \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return kfail((l), CB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// the axis levels of nearest.rs Slicer::detect: sorted, equal within 1e-9 of the span
// merged
std::vector<double> axis_levels(std::vector<double> l) {
  std::sort(l.begin(), l.end());
  const double span = std::max(std::fabs(l.back() - l[0]), 1e-300);
  std::vector<double> out;
  for (double v : l)
    if (out.empty() || std::fabs(out.back() - v) > 1e-9 * span) out.push_back(v);
  return out;
}

size_t link_trial_bytes(const cb_link* l) {
  const size_t nb = (size_t)l->code->host.n * l->blocks;
  return nb * 16 + (size_t)l->blocks * 4 + (size_t)l->blocks * ((l->code->enc.k + 31) / 32) * 4 + 4 +
         sizeof(cbk::LinkRecord);
}

cb_status link_ensure_device(cb_link* l) {
  if (l->dev_ready) return CB_OK;
  cb_ldpc* c = l->code;
  if (cb_status st = ensure_encoder(c)) return kfail(l, st, c->err);
  if (cb_status st = ensure_device(c)) return kfail(l, st, c->err);
  std::vector<int32_t> tab = l->perm;
  tab.insert(tab.end(), l->lookup.begin(), l->lookup.end());
  LINK_CUDA(l, cudaMalloc(&l->d_tab, tab.size() * 4));
  LINK_CUDA(l, cudaMemcpy(l->d_tab, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice));
  LINK_CUDA(l, cudaMalloc(&l->d_points, l->pts.size() * 8));
  LINK_CUDA(l, cudaMemcpy(l->d_points, l->pts.data(), l->pts.size() * 8, cudaMemcpyHostToDevice));
  LINK_CUDA(l, cudaMalloc(&l->d_jumps, l->jumps.size() * 8));
  LINK_CUDA(l, cudaMemcpy(l->d_jumps, l->jumps.data(), l->jumps.size() * 8, cudaMemcpyHostToDevice));
  const size_t smem = cbk::link_gen_smem_bytes(l->m, l->mbits, c->enc.k, c->host.n, l->blocks, l->n_pad);
  if (smem > kEncodeSmemLimit) return kfail(l, CB_ERR_CONFIG, "the trial does not fit the generator's shared memory");
  l->dev_ready = true;
  return CB_OK;
}

// trials [first, first + n) into the link's device buffers: generation, decoding and,
// when `count` is set, the records
cb_status link_run_device(cb_link* l, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first, int64_t n,
                          double ebn0_db, bool count, cudaStream_t s, cbk::LinkRecord* out_dev = nullptr) {
  cb_ldpc* c = l->code;
  // the code's decoder or encoder may have been changed since the link was made
  if (c->enc.kind != cbh::kEncoderSums)
    return kfail(l, CB_ERR_CONFIG, "the link needs the from_rows encoder: cb_ldpc_set_encoder(CB_ENC_SUMS)");
  if (cb_status st = ensure_encoder(c)) return kfail(l, st, c->err);
  if (cb_status st = ensure_device(c)) return kfail(l, st, c->err);
  const cbh::SparseEncoder& e = c->enc;
  const int nb = c->host.n * l->blocks, wk = (e.k + 31) / 32;
  LINK_CUDA(l, grow_buf(&l->d_llr, l->llr_cap, (size_t)n * nb * 8));
  LINK_CUDA(l, grow_buf(&l->d_post, l->post_cap, (size_t)n * nb * 8));
  LINK_CUDA(l, grow_buf(&l->d_iters, l->iters_cap, (size_t)n * l->blocks * 4));
  LINK_CUDA(l, grow_buf(&l->d_payload, l->payload_cap, (size_t)n * l->blocks * wk * 4));
  LINK_CUDA(l, grow_buf(&l->d_raw, l->raw_cap, (size_t)n * 4));
  LINK_CUDA(l, grow_buf(&l->d_rec, l->rec_cap, (size_t)n * sizeof(cbk::LinkRecord)));
  cbk::LinkGenArgs a;
  a.k = e.k;
  a.n = c->host.n;
  a.blocks = l->blocks;
  a.rank = (int32_t)e.pivots.size();
  a.info_pos = c->d_enc;
  a.pivots = c->d_enc + e.k;
  a.pmat = reinterpret_cast<const uint32_t*>(c->d_enc + e.k + e.pivots.size());
  a.perm = l->interleave ? l->d_tab : nullptr;
  a.m = l->m;
  a.mbits = l->mbits;
  a.n_pad = l->n_pad;
  a.bits_per_chunk = l->bpc;
  a.syms_per_chunk = l->spc;
  a.points = l->d_points;
  a.log_m = l->log_m;
  // b = log2 M k / n (com-spec blocks/channel.rs:145-149, block.rs:59-61), times db2lin
  const double rate = (double)e.k / (double)c->host.n;
  a.b_ebn0 = ((double)l->mbits * rate) * std::pow(10.0, ebn0_db / 10.0);
  a.exact = l->exact;
  a.jumps = l->d_jumps;
  a.side = l->side;
  a.step = l->step;
  a.re0 = l->re0;
  a.im0 = l->im0;
  a.lookup = l->d_tab + l->perm.size();
  a.seed = seed;
  a.name_hash = name_hash;
  a.cond = cond;
  a.first_trial = first;
  a.n_trials = n;
  const bool f64 = c->precision == CB_F64;
  a.llr_out = f64 ? (double*)l->d_llr : nullptr;
  a.llr_out_f32 = f64 ? nullptr : (float*)l->d_llr;
  a.payload_out = (uint32_t*)l->d_payload;
  a.raw_errors_out = (uint32_t*)l->d_raw;
  LINK_CUDA(l, cbk::launch_link_gen(a, s));
  if (cb_status st = f64 ? decode_impl<double>(c, (const double*)l->d_llr, n * l->blocks, (double*)l->d_post,
                                               (int32_t*)l->d_iters, s)
                          : decode_impl<float>(c, (const float*)l->d_llr, n * l->blocks, (float*)l->d_post,
                                               (int32_t*)l->d_iters, s))
    return kfail(l, st, c->err);
  if (count) {
    cbk::LinkCountArgs ca;
    ca.k = e.k;
    ca.n = c->host.n;
    ca.blocks = l->blocks;
    ca.info_pos = c->d_enc;
    ca.post = f64 ? (const double*)l->d_post : nullptr;
    ca.post_f32 = f64 ? nullptr : (const float*)l->d_post;
    ca.iters = (const int32_t*)l->d_iters;
    ca.payload = (const uint32_t*)l->d_payload;
    ca.raw_errors = (const uint32_t*)l->d_raw;
    ca.n_trials = n;
    ca.out = out_dev ? out_dev : (cbk::LinkRecord*)l->d_rec;
    LINK_CUDA(l, cbk::launch_link_count(ca, s));
  }
  return CB_OK;
}

// trials per chunk: at most 1 GB of buffers
int64_t link_chunk(const cb_link* l, int64_t n) {
  return std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)(((size_t)1 << 30) / link_trial_bytes(l))));
}

}  // namespace

extern "C" {

cb_status cb_ldpc_create(int32_t n, int32_t m, const int32_t* row_start, const int32_t* vars, int32_t rule,
                         double alpha, int32_t layered, int32_t max_iterations, int32_t precision, int32_t device,
                         cb_ldpc** out) {
  if (!out) return lfail(nullptr, CB_ERR_CONFIG, "null output pointer");
  *out = nullptr;
  if (cb_status st = check_decoder_settings(rule, alpha, max_iterations)) return st;
  if (precision != CB_F64 && precision != CB_F32) return lfail(nullptr, CB_ERR_CONFIG, "precision must be f64 or f32");
  cb_ldpc* c = new cb_ldpc;
  std::string err;
  if (!cbh::build_sparse_code(n, m, row_start, vars, c->host, err)) {
    delete c;
    return lfail(nullptr, CB_ERR_CONFIG, err);
  }
  c->device = device;
  c->precision = precision;
  c->rule = rule;
  c->alpha = alpha;
  c->layered = layered ? 1 : 0;
  c->max_iterations = max_iterations;
  *out = c;
  return CB_OK;
}

void cb_ldpc_destroy(cb_ldpc* c) {
  if (!c) return;
  if (c->dev_ready || c->stream || c->enc_ready) {
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_tables);
    cudaFree(c->d_counter);
    cudaFree(c->d_slots);
    cudaFree(c->d_llr);
    cudaFree(c->d_post);
    cudaFree(c->d_iters);
    cudaFree(c->d_enc);
    cudaFree(c->d_info);
    cudaFree(c->d_coded);
    if (c->stream) cudaStreamDestroy(c->stream);
  }
  delete c;
}

const char* cb_ldpc_last_error(const cb_ldpc* c) { return c ? c->err.c_str() : g_ldpc_thread_error.c_str(); }

cb_status cb_ldpc_info(const cb_ldpc* c, int64_t* info) {
  if (!c || !info) return lfail(c, CB_ERR_CONFIG, "null argument");
  const cbh::SparseCode& h = c->host;
  const int64_t v[8] = {h.n, h.m, h.edges, h.max_row_degree, h.max_col_degree, h.levels, h.max_level_rows,
                        c->layered};
  std::copy(v, v + 8, info);
  return CB_OK;
}

cb_status cb_ldpc_levels(const cb_ldpc* c, int32_t* level_start, int32_t* level_rows) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null argument");
  if (level_start) std::copy(c->host.level_start.begin(), c->host.level_start.end(), level_start);
  if (level_rows) std::copy(c->host.level_rows.begin(), c->host.level_rows.end(), level_rows);
  return CB_OK;
}

cb_status cb_ldpc_decode_device(cb_ldpc* c, const void* llr, int64_t n_frames, void* post, int32_t* iterations,
                                void* stream) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (n_frames < 0) return lfail(c, CB_ERR_SHAPE, "n_frames must be >= 0");
  if (n_frames > 0 && !llr) return lfail(c, CB_ERR_SHAPE, "null LLRs");
  std::lock_guard<std::mutex> lock(c->mu);
  if (cb_status st = ensure_device(c)) return st;
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the default stream
  if (c->precision == CB_F64)
    return decode_impl<double>(c, (const double*)llr, n_frames, (double*)post, iterations, s);
  return decode_impl<float>(c, (const float*)llr, n_frames, (float*)post, iterations, s);
}

cb_status cb_ldpc_decode(cb_ldpc* c, const void* llr, int64_t n_frames, void* post, int32_t* iterations) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (n_frames < 0) return lfail(c, CB_ERR_SHAPE, "n_frames must be >= 0");
  if (n_frames == 0) return CB_OK;
  if (!llr) return lfail(c, CB_ERR_SHAPE, "null LLRs");
  std::lock_guard<std::mutex> lock(c->mu);
  if (cb_status st = ensure_device(c)) return st;
  const size_t per = (size_t)c->host.n * elem(c);
  // chunks of at most 1 GB of LLRs
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n_frames, (int64_t)(((size_t)1 << 30) / per)));
  LDPC_CUDA(c, grow_buf(&c->d_llr, c->llr_cap, chunk * per));
  if (post) LDPC_CUDA(c, grow_buf(&c->d_post, c->post_cap, chunk * per));
  if (iterations) LDPC_CUDA(c, grow_buf((void**)&c->d_iters, c->iters_cap, chunk * 4));
  for (int64_t f0 = 0; f0 < n_frames; f0 += chunk) {
    const int64_t k = std::min(chunk, n_frames - f0);
    LDPC_CUDA(c, cudaMemcpyAsync(c->d_llr, (const char*)llr + f0 * per, k * per, cudaMemcpyHostToDevice, c->stream));
    cb_status st = c->precision == CB_F64
                       ? decode_impl<double>(c, (const double*)c->d_llr, k, post ? (double*)c->d_post : nullptr,
                                             iterations ? c->d_iters : nullptr, c->stream)
                       : decode_impl<float>(c, (const float*)c->d_llr, k, post ? (float*)c->d_post : nullptr,
                                            iterations ? c->d_iters : nullptr, c->stream);
    if (st) return st;
    if (post)
      LDPC_CUDA(c, cudaMemcpyAsync((char*)post + f0 * per, c->d_post, k * per, cudaMemcpyDeviceToHost, c->stream));
    if (iterations)
      LDPC_CUDA(c, cudaMemcpyAsync(iterations + f0, c->d_iters, k * 4, cudaMemcpyDeviceToHost, c->stream));
    LDPC_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return CB_OK;
}

cb_status cb_ldpc_set_decoder(cb_ldpc* c, int32_t rule, double alpha, int32_t layered, int32_t max_iterations) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (cb_status st = check_decoder_settings(rule, alpha, max_iterations)) {
    c->err = g_ldpc_thread_error;
    return st;
  }
  std::lock_guard<std::mutex> lock(c->mu);
  // the kernel and the message layout follow the rule and the schedule
  if (rule != c->rule || (layered ? 1 : 0) != c->layered) release_decoder(c);
  c->rule = rule;
  c->alpha = alpha;
  c->layered = layered ? 1 : 0;
  c->max_iterations = max_iterations;
  return CB_OK;
}

cb_status cb_ldpc_girth(const cb_ldpc* c, int32_t* girth) {
  if (!c || !girth) return lfail(c, CB_ERR_CONFIG, "null argument");
  *girth = cbh::girth(c->host);
  return CB_OK;
}

cb_status cb_ldpc_set_encoder(cb_ldpc* c, int32_t kind, int32_t* k, int32_t* info_positions) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (kind != CB_ENC_SUMS && kind != CB_ENC_ACCUMULATE)
    return lfail(c, CB_ERR_CONFIG, "the encoder must be CB_ENC_SUMS or CB_ENC_ACCUMULATE");
  std::lock_guard<std::mutex> lock(c->mu);
  if (c->enc.kind != kind) {
    cbh::SparseEncoder enc;
    std::string err;
    const bool ok = kind == CB_ENC_SUMS ? cbh::reduce_sums(c->host, enc, err) : cbh::check_accumulate(c->host, enc, err);
    if (!ok) return lfail(c, CB_ERR_CONFIG, err);
    if (c->enc_ready) {
      cudaSetDevice(c->device);
      if (c->stream) cudaStreamSynchronize(c->stream);
      cudaFree(c->d_enc);
      c->d_enc = nullptr;
      c->enc_ready = false;
    }
    c->enc = std::move(enc);
  }
  if (k) *k = c->enc.k;
  if (info_positions) std::copy(c->enc.info.begin(), c->enc.info.end(), info_positions);
  return CB_OK;
}

cb_status cb_ldpc_encode_device(cb_ldpc* c, const uint8_t* info, int64_t n_frames, uint8_t* coded, void* stream) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (n_frames < 0) return lfail(c, CB_ERR_SHAPE, "n_frames must be >= 0");
  if (n_frames > 0 && (!info || !coded)) return lfail(c, CB_ERR_SHAPE, "null information or coded bits");
  std::lock_guard<std::mutex> lock(c->mu);
  if (cb_status st = ensure_encoder(c)) return st;
  return encode_impl(c, info, n_frames, coded, (cudaStream_t)stream);  // NULL: the default stream
}

cb_status cb_ldpc_encode(cb_ldpc* c, const uint8_t* info, int64_t n_frames, uint8_t* coded) {
  if (!c) return lfail(nullptr, CB_ERR_CONFIG, "null code");
  if (n_frames < 0) return lfail(c, CB_ERR_SHAPE, "n_frames must be >= 0");
  if (n_frames == 0) return CB_OK;
  if (!info || !coded) return lfail(c, CB_ERR_SHAPE, "null information or coded bits");
  std::lock_guard<std::mutex> lock(c->mu);
  if (cb_status st = ensure_encoder(c)) return st;
  const size_t k = (size_t)c->enc.k, n = (size_t)c->host.n;
  // chunks of at most 1 GB of coded bits
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n_frames, (int64_t)(((size_t)1 << 30) / n)));
  LDPC_CUDA(c, grow_buf(&c->d_info, c->info_cap, chunk * k));
  LDPC_CUDA(c, grow_buf(&c->d_coded, c->coded_cap, chunk * n));
  for (int64_t f0 = 0; f0 < n_frames; f0 += chunk) {
    const int64_t cnt = std::min(chunk, n_frames - f0);
    LDPC_CUDA(c, cudaMemcpyAsync(c->d_info, info + f0 * k, cnt * k, cudaMemcpyHostToDevice, c->stream));
    if (cb_status st = encode_impl(c, (const uint8_t*)c->d_info, cnt, (uint8_t*)c->d_coded, c->stream)) return st;
    LDPC_CUDA(c, cudaMemcpyAsync(coded + f0 * n, c->d_coded, cnt * n, cudaMemcpyDeviceToHost, c->stream));
    LDPC_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return CB_OK;
}

cb_status cb_ldpc_peg(int32_t n, int32_t k, int32_t var_degree, uint64_t seed, int32_t* row_start, int32_t* vars) {
  if (!row_start || !vars) return lfail(nullptr, CB_ERR_CONFIG, "null output pointer");
  std::vector<std::vector<int32_t>> rows;
  std::string err;
  if (!cbh::peg_rows(n, k, var_degree, seed, rows, err)) return lfail(nullptr, CB_ERR_CONFIG, err);
  int32_t e = 0;
  row_start[0] = 0;
  for (size_t r = 0; r < rows.size(); r++) {
    for (int32_t v : rows[r]) vars[e++] = v;
    row_start[r + 1] = e;
  }
  return CB_OK;
}


cb_status cb_link_create(cb_ldpc* code, int32_t blocks, int32_t modulation_order, int32_t interleave,
                         uint64_t interleaver_seed, int32_t exact_demap, cb_link** out) {
  if (!out) return kfail(nullptr, CB_ERR_CONFIG, "null output pointer");
  *out = nullptr;
  if (!code) return kfail(nullptr, CB_ERR_CONFIG, "null code");
  if (code->enc.kind != cbh::kEncoderSums)
    return kfail(nullptr, CB_ERR_CONFIG, "the link needs the from_rows encoder: cb_ldpc_set_encoder(CB_ENC_SUMS)");
  if (blocks < 1) return kfail(nullptr, CB_ERR_CONFIG, "blocks must be >= 1");
  const int64_t nb = (int64_t)code->host.n * blocks;
  if (nb > ((int64_t)1 << 24)) return kfail(nullptr, CB_ERR_CONFIG, "n x blocks must be at most 2^24");
  cb_link* l = new cb_link;
  l->code = code;
  l->blocks = blocks;
  l->m = modulation_order;
  if (!cbh::qam_points(modulation_order, l->pts, l->log_m)) {
    delete l;
    return kfail(nullptr, CB_ERR_CONFIG, "modulation order must be 4, 16, 64 or 256");
  }
  const cbh::GenTables t = cbh::gen_tables(code->enc.k * blocks, (int)nb, modulation_order, cbk::kGenThreads,
                                            cbk::kGenThreads);
  l->mbits = t.mbits;
  l->n_pad = t.n_pad;
  l->bpc = t.bits_per_chunk;
  l->spc = t.syms_per_chunk;
  l->jumps = t.jumps;
  l->exact = exact_demap ? 1 : 0;
  l->interleave = interleave != 0;
  l->il_seed = interleaver_seed;
  if (l->interleave) {
    // Interleaver::random (interleaving.rs:63-67): Rng::new(seed).shuffle (rng.rs:218-222)
    l->perm.resize(nb);
    for (int64_t i = 0; i < nb; i++) l->perm[i] = (int32_t)i;
    cbd::Xoshiro r = cbd::xoshiro_seed(interleaver_seed);
    for (int64_t i = nb - 1; i >= 1; i--) std::swap(l->perm[i], l->perm[cbd::xoshiro_below(r, (uint64_t)i + 1)]);
  }
  // the grid slicer of the square QAM (nearest.rs Slicer::detect)
  std::vector<double> re(l->m), im(l->m);
  for (int i = 0; i < l->m; i++) {
    re[i] = l->pts[2 * i];
    im[i] = l->pts[2 * i + 1];
  }
  const std::vector<double> lre = axis_levels(re), lim = axis_levels(im);
  l->side = (int)lre.size();
  l->step = (lre.back() - lre[0]) / (double)(l->side - 1);
  l->re0 = lre[0];
  l->im0 = lim[0];
  l->lookup.assign(l->m, 0);
  for (int i = 0; i < l->m; i++) {
    const int col = (int)std::round((re[i] - lre[0]) / l->step), row = (int)std::round((im[i] - lim[0]) / l->step);
    l->lookup[row * l->side + col] = i;
  }
  *out = l;
  return CB_OK;
}

void cb_link_destroy(cb_link* l) {
  if (!l) return;
  if (l->dev_ready || l->d_llr) {
    cudaSetDevice(l->code->device);
    if (l->code->stream) cudaStreamSynchronize(l->code->stream);
    cudaFree(l->d_tab);
    cudaFree(l->d_points);
    cudaFree(l->d_jumps);
    cudaFree(l->d_llr);
    cudaFree(l->d_post);
    cudaFree(l->d_iters);
    cudaFree(l->d_payload);
    cudaFree(l->d_raw);
    cudaFree(l->d_rec);
  }
  delete l;
}

const char* cb_link_last_error(const cb_link* l) { return l ? l->err.c_str() : g_link_thread_error.c_str(); }

cb_status cb_link_info(const cb_link* l, int64_t info[8]) {
  if (!l || !info) return kfail(l, CB_ERR_CONFIG, "null argument");
  const int64_t nb = (int64_t)l->code->host.n * l->blocks;
  const int64_t v[8] = {l->code->enc.k, l->code->host.n, l->blocks, l->m, nb + l->n_pad,
                        (int64_t)l->code->enc.k * l->blocks, l->n_pad, l->interleave ? 1 : 0};
  std::copy(v, v + 8, info);
  return CB_OK;
}

cb_status cb_link_interleaver(const cb_link* l, int32_t* perm) {
  if (!l || !perm) return kfail(l, CB_ERR_CONFIG, "null argument");
  if (!l->interleave) return kfail(l, CB_ERR_CONFIG, "the link has no interleaver");
  std::copy(l->perm.begin(), l->perm.end(), perm);
  return CB_OK;
}

cb_status cb_link_run_trials(cb_link* l, uint64_t seed, uint64_t name_hash, uint64_t condition, uint64_t first_trial,
                             int64_t n_trials, double ebn0_db, cb_link_record* out) {
  if (!l) return kfail(nullptr, CB_ERR_CONFIG, "null link");
  if (n_trials < 0) return kfail(l, CB_ERR_SHAPE, "n_trials must be >= 0");
  if (n_trials == 0) return CB_OK;
  if (!out) return kfail(l, CB_ERR_SHAPE, "null records");
  std::lock_guard<std::mutex> lock(l->mu);
  std::lock_guard<std::mutex> lock_code(l->code->mu);
  if (cb_status st = link_ensure_device(l)) return st;
  const int64_t chunk = link_chunk(l, n_trials);
  for (int64_t f0 = 0; f0 < n_trials; f0 += chunk) {
    const int64_t cnt = std::min(chunk, n_trials - f0);
    if (cb_status st = link_run_device(l, seed, name_hash, condition, first_trial + f0, cnt, ebn0_db, true,
                                       l->code->stream))
      return st;
    LINK_CUDA(l, cudaMemcpyAsync(out + f0, l->d_rec, cnt * sizeof(cb_link_record), cudaMemcpyDeviceToHost,
                                 l->code->stream));
    LINK_CUDA(l, cudaStreamSynchronize(l->code->stream));
  }
  return CB_OK;
}

cb_status cb_link_run_trials_device(cb_link* l, uint64_t seed, uint64_t name_hash, uint64_t condition,
                                    uint64_t first_trial, int64_t n_trials, double ebn0_db, cb_link_record* out_dev,
                                    void* stream) {
  if (!l) return kfail(nullptr, CB_ERR_CONFIG, "null link");
  if (n_trials < 0) return kfail(l, CB_ERR_SHAPE, "n_trials must be >= 0");
  if (n_trials == 0) return CB_OK;
  if (!out_dev) return kfail(l, CB_ERR_SHAPE, "null records");
  std::lock_guard<std::mutex> lock(l->mu);
  std::lock_guard<std::mutex> lock_code(l->code->mu);
  if (cb_status st = link_ensure_device(l)) return st;
  const int64_t cap = link_chunk(l, INT64_MAX);
  if (n_trials > cap) return kfail(l, CB_ERR_SHAPE, "at most " + std::to_string(cap) + " trials per device call");
  return link_run_device(l, seed, name_hash, condition, first_trial, n_trials, ebn0_db, true,
                         (cudaStream_t)stream,  // NULL: the default stream
                         reinterpret_cast<cbk::LinkRecord*>(out_dev));
}

cb_status cb_link_generate(cb_link* l, uint64_t seed, uint64_t name_hash, uint64_t condition, uint64_t first_trial,
                           int64_t n_trials, double ebn0_db, double* llr, uint8_t* payload, uint32_t* raw_errors) {
  if (!l) return kfail(nullptr, CB_ERR_CONFIG, "null link");
  if (n_trials < 0) return kfail(l, CB_ERR_SHAPE, "n_trials must be >= 0");
  if (n_trials == 0) return CB_OK;
  std::lock_guard<std::mutex> lock(l->mu);
  std::lock_guard<std::mutex> lock_code(l->code->mu);
  if (cb_status st = link_ensure_device(l)) return st;
  const int k = l->code->enc.k, nb = l->code->host.n * l->blocks, wk = (k + 31) / 32;
  const int64_t chunk = link_chunk(l, n_trials);
  std::vector<uint32_t> words;
  for (int64_t f0 = 0; f0 < n_trials; f0 += chunk) {
    const int64_t cnt = std::min(chunk, n_trials - f0);
    if (cb_status st = link_run_device(l, seed, name_hash, condition, first_trial + f0, cnt, ebn0_db, false,
                                       l->code->stream))
      return st;
    cudaStream_t s = l->code->stream;
    std::vector<float> l32;
    if (llr && l->code->precision == CB_F64)
      LINK_CUDA(l, cudaMemcpyAsync(llr + f0 * nb, l->d_llr, cnt * nb * 8, cudaMemcpyDeviceToHost, s));
    if (llr && l->code->precision != CB_F64) {
      l32.resize((size_t)cnt * nb);
      LINK_CUDA(l, cudaMemcpyAsync(l32.data(), l->d_llr, l32.size() * 4, cudaMemcpyDeviceToHost, s));
    }
    if (raw_errors) LINK_CUDA(l, cudaMemcpyAsync(raw_errors + f0, l->d_raw, cnt * 4, cudaMemcpyDeviceToHost, s));
    if (payload) {
      words.resize((size_t)cnt * l->blocks * wk);
      LINK_CUDA(l, cudaMemcpyAsync(words.data(), l->d_payload, words.size() * 4, cudaMemcpyDeviceToHost, s));
    }
    LINK_CUDA(l, cudaStreamSynchronize(s));
    for (size_t i = 0; i < l32.size(); i++) llr[f0 * nb + i] = (double)l32[i];
    if (payload)
      for (int64_t t = 0; t < cnt; t++)
        for (int b = 0; b < l->blocks; b++)
          for (int i = 0; i < k; i++)
            payload[((f0 + t) * l->blocks + b) * k + i] =
                (uint8_t)((words[((size_t)t * l->blocks + b) * wk + i / 32] >> (i % 32)) & 1u);
  }
  return CB_OK;
}

}  // extern "C"
