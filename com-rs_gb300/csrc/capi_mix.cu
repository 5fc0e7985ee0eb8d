// The C ABI of mixed batches (include/comrs_gb300.h, cb_mix_*): thousands of
// codewords of different codes, generated and decoded by one graph of two kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/comrs_gb300.h"
#include "code_host.h"
#include "dev_code.h"
#include "kernels.h"

namespace {
thread_local std::string g_mix_error;
constexpr size_t kSlotSmemBudget = 113 * 1024;  // two 384-thread CTAs per SM
constexpr int kCtaThreads = 384;
}  // namespace

struct cb_mix {
  std::mutex mu;
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t seed = 0, name_hash = 0;
  float alpha = 0.75f;
  int max_it = 25;
  int64_t n = 0;
  std::vector<cbh::NrCode> codes;
  std::vector<cbd::DevCode> dev_codes;
  std::vector<cbk::GenConfig> configs;
  std::vector<cbk::MixItem> items;    // sorted by class
  std::vector<cbk::MixClass> classes;
  size_t gen_smem = 0, dec_smem = 0, state_per_cta = 0;
  int grid = 0;
  int64_t llr_elems = 0, info_words = 0;
  // device
  cbd::DevCode* d_codes = nullptr;
  cbk::GenConfig* d_configs = nullptr;
  std::vector<void*> d_tables;
  cbk::MixItem* d_items = nullptr;
  cbk::MixClass* d_classes = nullptr;
  float* d_llr = nullptr;
  uint32_t* d_info = nullptr;
  cbd::FrameResult* d_results = nullptr;
  unsigned long long* d_counters = nullptr;
  unsigned long long* d_counters_init = nullptr;
  unsigned char* d_state = nullptr;
  uint64_t* d_epoch = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::string err;
};

namespace {

cb_status mfail(cb_mix* m, cb_status s, const std::string& msg) {
  if (m) m->err = msg;
  g_mix_error = msg;
  return s;
}

#define MIX_CUDA(m, call)                                                                          \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return mfail((m), CB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// the slot layout of a class for `rho` rows per thread (0 slots: not a valid layout)
void layout(cbk::MixClass& k, int rho) {
  int rows = (k.z + rho - 1) / rho;
  k.slot_threads = std::max(32, ((rows + 31) / 32) * 32);
  k.rows_per_thread = rho;
  k.smem_per_slot = (int32_t)cbk::mix_slot_smem_bytes(k.z);
  int by_threads = kCtaThreads / k.slot_threads;
  int by_smem = (int)(kSlotSmemBudget / (size_t)k.smem_per_slot);
  k.slots = std::min({by_threads, by_smem, 15});
  k.state_per_slot = (int32_t)((size_t)cbh::kMaxLayers * k.z * 12);
  k.max_ncol = 68;
}

// sizes that depend on the class layouts: shared memory, state, grid
cb_status relayout(cb_mix* m) {
  m->dec_smem = 0;
  m->state_per_cta = 0;
  for (auto& k : m->classes) {
    if (k.slots < 1) return mfail(m, CB_ERR_CONFIG, "no slot layout fits a class");
    m->dec_smem = std::max(m->dec_smem, (size_t)k.slots * k.smem_per_slot);
    m->state_per_cta = std::max(m->state_per_cta, (size_t)k.slots * k.state_per_slot);
  }
  m->dec_smem = (m->dec_smem + 15) & ~(size_t)15;
  m->state_per_cta = (m->state_per_cta + 255) & ~(size_t)255;
  m->grid = cbk::mix_decode_grid(m->dec_smem, m->device);
  if (m->grid <= 0) return mfail(m, CB_ERR_CUDA, "the mixed-batch decoder does not fit an SM");
  if (m->d_state) cudaFree(m->d_state);
  m->d_state = nullptr;
  MIX_CUDA(m, cudaMalloc(&m->d_state, m->state_per_cta * m->grid));
  MIX_CUDA(m, cudaMemcpy(m->d_classes, m->classes.data(), sizeof(cbk::MixClass) * m->classes.size(),
                         cudaMemcpyHostToDevice));
  if (m->exec) cudaGraphExecDestroy(m->exec);
  m->exec = nullptr;
  return CB_OK;
}

cbk::GenMixArgs gen_args(cb_mix* m) {
  cbk::GenMixArgs g{};
  g.codes = m->d_codes;
  g.configs = m->d_configs;
  g.items = m->d_items;
  g.n_items = m->n;
  g.seed = m->seed;
  g.name_hash = m->name_hash;
  g.epoch = m->d_epoch;
  g.epoch_stride = (uint64_t)m->n;
  g.llr = m->d_llr;
  g.info = m->d_info;
  return g;
}

cbk::MixDecodeArgs dec_args(cb_mix* m) {
  cbk::MixDecodeArgs a{};
  a.codes = m->d_codes;
  a.items = m->d_items;
  a.classes = m->d_classes;
  a.n_classes = (int32_t)m->classes.size();
  a.rule = cbd::RULE_NMS;
  a.max_it = m->max_it;
  a.alpha = m->alpha;
  a.llr = m->d_llr;
  a.info = m->d_info;
  a.results = m->d_results;
  a.counters = m->d_counters;
  a.state = m->d_state;
  a.state_per_cta = m->state_per_cta;
  return a;
}

// the decode phase of class `only` (-1: all), its queues reset from `init`
cb_status launch_decode_phase(cb_mix* m, const std::vector<unsigned long long>& init, cudaStream_t s) {
  MIX_CUDA(m, cudaMemcpyAsync(m->d_counters_init, init.data(), 8 * init.size(), cudaMemcpyHostToDevice, s));
  MIX_CUDA(m, cudaMemcpyAsync(m->d_counters, m->d_counters_init, 8 * init.size(), cudaMemcpyDeviceToDevice, s));
  MIX_CUDA(m, cbk::launch_mix_decode(dec_args(m), m->grid, m->dec_smem, s));
  return CB_OK;
}

// the generator then the decoder, captured once and replayed
cb_status ensure_graph(cb_mix* m) {
  if (m->exec) return CB_OK;
  std::vector<unsigned long long> zero(m->classes.size(), 0ull);
  MIX_CUDA(m, cudaMemcpy(m->d_counters_init, zero.data(), 8 * zero.size(), cudaMemcpyHostToDevice));
  cudaGraph_t graph = nullptr;
  MIX_CUDA(m, cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaMemcpyAsync(m->d_counters, m->d_counters_init, 8 * zero.size(), cudaMemcpyDeviceToDevice,
                                  m->stream);
  if (e == cudaSuccess) e = cbk::launch_gen_mix(gen_args(m), m->gen_smem, m->stream);
  if (e == cudaSuccess) e = cbk::launch_mix_decode(dec_args(m), m->grid, m->dec_smem, m->stream);
  cudaError_t e2 = cudaStreamEndCapture(m->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return mfail(m, CB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  e = cudaGraphInstantiate(&m->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return mfail(m, CB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  return CB_OK;
}

}  // namespace

extern "C" {

cb_status cb_mix_create(const cb_mix_item* items, int64_t n, uint64_t seed, uint64_t name_hash, double alpha,
                        int32_t max_iterations, int32_t device, cb_mix** out) {
  if (!items || !out || n <= 0 || n > (1 << 30)) return mfail(nullptr, CB_ERR_CONFIG, "bad items");
  if (max_iterations < 0 || max_iterations > 255) return mfail(nullptr, CB_ERR_CONFIG, "max_iterations in 0..255");
  *out = nullptr;
  cb_mix* m = new cb_mix();
  m->device = device;
  m->seed = seed;
  m->name_hash = name_hash;
  m->alpha = (float)alpha;
  m->max_it = max_iterations;
  m->n = n;
  // distinct codes and (code, modulation) generator configs
  std::map<std::tuple<int, int, int, int>, int> code_id;
  std::map<std::pair<int, int>, int> config_id;
  std::vector<cbh::GenTables> tables;
  std::vector<std::vector<double>> points;
  std::vector<double> log_m;
  std::vector<int> mods;
  std::vector<cbk::MixItem> its((size_t)n);
  for (int64_t i = 0; i < n; i++) {
    const cb_mix_item& d = items[i];
    auto key = std::make_tuple(d.base_graph, d.lifting_size, d.k_info, d.e);
    auto f = code_id.find(key);
    int cid;
    if (f == code_id.end()) {
      cbh::CodeSpec spec;
      spec.k_info = d.k_info;
      spec.e = d.e;
      spec.bg = d.base_graph;
      spec.z = d.lifting_size;
      cbh::NrCode h;
      std::string err;
      if (!cbh::build_nr_code(spec, h, err)) {
        delete m;
        return mfail(nullptr, CB_ERR_CONFIG, "item " + std::to_string(i) + ": " + err);
      }
      if (!h.map_is_offset || !cbk::degrees_supported(h)) {
        delete m;
        return mfail(nullptr, CB_ERR_CONFIG,
                     "item " + std::to_string(i) + ": mixed batches need the plain rate matching 2Z + t");
      }
      cid = (int)m->codes.size();
      code_id[key] = cid;
      m->codes.push_back(h);
    } else {
      cid = f->second;
    }
    auto ck = std::make_pair(cid, (int)d.modulation_order);
    auto g = config_id.find(ck);
    int gid;
    if (g == config_id.end()) {
      std::vector<double> pts;
      double lm;
      if (!cbh::qam_points(d.modulation_order, pts, lm)) {
        delete m;
        return mfail(nullptr, CB_ERR_CONFIG, "item " + std::to_string(i) + ": modulation order 4, 16, 64 or 256");
      }
      gid = (int)tables.size();
      config_id[ck] = gid;
      tables.push_back(cbh::gen_tables(m->codes[cid].k_info, m->codes[cid].e, d.modulation_order, cbk::kGenBitsThreads,
                                       cbk::kGenNoiseThreads));
      points.push_back(pts);
      log_m.push_back(lm);
      mods.push_back(d.modulation_order);
    } else {
      gid = g->second;
    }
    if (!std::isfinite(d.ebn0_db)) {
      delete m;
      return mfail(nullptr, CB_ERR_CONFIG, "item " + std::to_string(i) + ": Eb/N0 must be finite");
    }
    cbk::MixItem& it = its[(size_t)i];
    it.code = cid;
    it.config = gid;
    it.cond = d.condition;
    it.frame = d.frame;
    // b = log2 M * R (com-spec blocks/channel.rs:145-149), times db2lin (units.rs:38-40)
    const cbh::NrCode& h = m->codes[cid];
    double b = (double)__builtin_ctz(d.modulation_order) * ((double)h.k_info / (double)h.e);
    it.b_ebn0 = b * std::pow(10.0, d.ebn0_db / 10.0);
    it.index = (int32_t)i;
  }
  // classes by lifting size, largest first
  std::stable_sort(its.begin(), its.end(), [&](const cbk::MixItem& a, const cbk::MixItem& b) {
    return m->codes[a.code].z > m->codes[b.code].z;
  });
  int64_t llr = 0, info = 0;
  for (int64_t i = 0; i < n; i++) {
    cbk::MixItem& it = its[(size_t)i];
    const cbh::NrCode& h = m->codes[it.code];
    it.llr_offset = llr;
    it.info_offset = info;
    llr += ((int64_t)h.e + 3) & ~3ll;
    info += (h.k_info + 31) / 32;
    if (m->classes.empty() || m->classes.back().z != h.z) {
      cbk::MixClass k{};
      k.z = h.z;
      k.first = i;
      layout(k, 1);
      m->classes.push_back(k);
    }
    m->classes.back().count++;
  }
  m->items = its;
  m->llr_elems = llr;
  m->info_words = info;
  // device state
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  m->dev_codes.resize(m->codes.size());
  for (size_t i = 0; i < m->codes.size(); i++) cbk::fill_dev_code(m->codes[i], m->dev_codes[i]);
  m->gen_smem = 0;
  for (auto& kv : config_id) {
    const cbh::NrCode& h = m->codes[kv.first.first];
    const cbh::GenTables& t = tables[kv.second];
    m->gen_smem = std::max(m->gen_smem, cbk::gen_smem_bytes(m->dev_codes[kv.first.first], mods[kv.second], t.mbits,
                                                            t.n_pad));
    (void)h;
  }
  m->configs.resize(tables.size());
  for (size_t g = 0; g < tables.size() && e == cudaSuccess; g++) {
    void* pd = nullptr;
    void* jd = nullptr;
    e = cudaMalloc(&pd, sizeof(double) * points[g].size());
    if (e == cudaSuccess) e = cudaMemcpy(pd, points[g].data(), sizeof(double) * points[g].size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&jd, 8 * tables[g].jumps.size());
    if (e == cudaSuccess) e = cudaMemcpy(jd, tables[g].jumps.data(), 8 * tables[g].jumps.size(), cudaMemcpyHostToDevice);
    m->d_tables.push_back(pd);
    m->d_tables.push_back(jd);
    cbk::GenConfig& c = m->configs[g];
    c.m = mods[g];
    c.mbits = tables[g].mbits;
    c.n_pad = tables[g].n_pad;
    c.bits_per_chunk = tables[g].bits_per_chunk;
    c.syms_per_chunk = tables[g].syms_per_chunk;
    c.points = (const double*)pd;
    c.log_m = log_m[g];
    c.jumps = (const uint64_t*)jd;
  }
  if (e == cudaSuccess) e = cudaMalloc(&m->d_codes, sizeof(cbd::DevCode) * m->dev_codes.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(m->d_codes, m->dev_codes.data(), sizeof(cbd::DevCode) * m->dev_codes.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_configs, sizeof(cbk::GenConfig) * m->configs.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(m->d_configs, m->configs.data(), sizeof(cbk::GenConfig) * m->configs.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_items, sizeof(cbk::MixItem) * n);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_items, m->items.data(), sizeof(cbk::MixItem) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_classes, sizeof(cbk::MixClass) * m->classes.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_llr, 4 * (size_t)m->llr_elems);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_info, 4 * (size_t)m->info_words);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_results, sizeof(cbd::FrameResult) * n);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_counters, 8 * m->classes.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_counters_init, 8 * m->classes.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_epoch, 64);
  if (e == cudaSuccess) e = cudaMemset(m->d_epoch, 0, 64);
  if (e != cudaSuccess) {
    std::string msg = std::string("CUDA: ") + cudaGetErrorString(e);
    cb_mix_destroy(m);
    return mfail(nullptr, CB_ERR_CUDA, msg);
  }
  if (cb_status st = relayout(m)) {
    std::string msg = m->err;
    cb_mix_destroy(m);
    return mfail(nullptr, st, msg);
  }
  *out = m;
  return CB_OK;
}

void cb_mix_destroy(cb_mix* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->exec) cudaGraphExecDestroy(m->exec);
  for (void* p : m->d_tables)
    if (p) cudaFree(p);
  void* bufs[] = {m->d_codes, m->d_configs, m->d_items, m->d_classes, m->d_llr, m->d_info, m->d_results,
                  m->d_counters, m->d_counters_init, m->d_state, m->d_epoch};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

const char* cb_mix_last_error(const cb_mix* m) { return m ? m->err.c_str() : g_mix_error.c_str(); }

cb_status cb_mix_classes(const cb_mix* m, int32_t capacity, int64_t* info, int32_t* n_classes) {
  if (!m || !n_classes) return mfail(nullptr, CB_ERR_CONFIG, "NULL argument");
  *n_classes = (int32_t)m->classes.size();
  for (int32_t i = 0; i < capacity && i < (int32_t)m->classes.size() && info; i++) {
    const cbk::MixClass& k = m->classes[i];
    int64_t* o = info + 8 * i;
    o[0] = k.z;
    o[1] = k.count;
    o[2] = k.rows_per_thread;
    o[3] = k.slots;
    o[4] = k.slot_threads;
    o[5] = k.smem_per_slot;
    o[6] = m->grid;
    o[7] = k.first;
  }
  return CB_OK;
}

cb_status cb_mix_set_rows_per_thread(cb_mix* m, int32_t cls, int32_t rho) {
  if (!m || cls < 0 || cls >= (int32_t)m->classes.size() || (rho != 1 && rho != 2))
    return mfail(m, CB_ERR_CONFIG, "class index or rows per thread (1 or 2)");
  std::lock_guard<std::mutex> lock(m->mu);
  MIX_CUDA(m, cudaSetDevice(m->device));
  cbk::MixClass k = m->classes[cls];
  layout(k, rho);
  if (k.slots < 1) return mfail(m, CB_ERR_CONFIG, "no slot layout for these rows per thread");
  m->classes[cls] = k;
  return relayout(m);
}

cb_status cb_mix_run(cb_mix* m, uint64_t epoch, cb_frame_result* out) {
  if (!m) return mfail(nullptr, CB_ERR_CONFIG, "NULL argument");
  std::lock_guard<std::mutex> lock(m->mu);
  MIX_CUDA(m, cudaSetDevice(m->device));
  if (cb_status st = ensure_graph(m)) return st;
  MIX_CUDA(m, cudaMemcpyAsync(m->d_epoch, &epoch, 8, cudaMemcpyHostToDevice, m->stream));
  MIX_CUDA(m, cudaGraphLaunch(m->exec, m->stream));
  if (out)
    MIX_CUDA(m, cudaMemcpyAsync(out, m->d_results, sizeof(cb_frame_result) * m->n, cudaMemcpyDeviceToHost, m->stream));
  MIX_CUDA(m, cudaStreamSynchronize(m->stream));
  return CB_OK;
}

cb_status cb_mix_frames(cb_mix* m, uint64_t epoch, float* llr, uint8_t* info) {
  if (!m) return mfail(nullptr, CB_ERR_CONFIG, "NULL argument");
  std::lock_guard<std::mutex> lock(m->mu);
  MIX_CUDA(m, cudaSetDevice(m->device));
  if (cb_status st = ensure_graph(m)) return st;
  MIX_CUDA(m, cudaMemcpyAsync(m->d_epoch, &epoch, 8, cudaMemcpyHostToDevice, m->stream));
  MIX_CUDA(m, cudaGraphLaunch(m->exec, m->stream));
  std::vector<float> h_llr((size_t)m->llr_elems);
  std::vector<uint32_t> h_info((size_t)m->info_words);
  MIX_CUDA(m, cudaMemcpyAsync(h_llr.data(), m->d_llr, 4 * h_llr.size(), cudaMemcpyDeviceToHost, m->stream));
  MIX_CUDA(m, cudaMemcpyAsync(h_info.data(), m->d_info, 4 * h_info.size(), cudaMemcpyDeviceToHost, m->stream));
  MIX_CUDA(m, cudaStreamSynchronize(m->stream));
  // the caller's layout: the items in their own order, each item's E LLRs and K' bits
  std::vector<int64_t> lo((size_t)m->n + 1, 0), io((size_t)m->n + 1, 0);
  std::vector<const cbk::MixItem*> by_index((size_t)m->n);
  for (const cbk::MixItem& it : m->items) by_index[(size_t)it.index] = &it;
  for (int64_t i = 0; i < m->n; i++) {
    const cbh::NrCode& h = m->codes[by_index[(size_t)i]->code];
    lo[(size_t)i + 1] = lo[(size_t)i] + h.e;
    io[(size_t)i + 1] = io[(size_t)i] + h.k_info;
  }
  for (int64_t i = 0; i < m->n; i++) {
    const cbk::MixItem& it = *by_index[(size_t)i];
    const cbh::NrCode& h = m->codes[it.code];
    if (llr) std::memcpy(llr + lo[(size_t)i], h_llr.data() + it.llr_offset, sizeof(float) * h.e);
    if (info)
      for (int b = 0; b < h.k_info; b++)
        info[io[(size_t)i] + b] = (uint8_t)((h_info[(size_t)it.info_offset + (b >> 5)] >> (b & 31)) & 1u);
  }
  return CB_OK;
}

cb_status cb_mix_time_decode(cb_mix* m, int32_t cls, int32_t reps, double* ms) {
  if (!m || !ms || reps < 1 || cls < -1 || cls >= (int32_t)m->classes.size())
    return mfail(m, CB_ERR_CONFIG, "bad arguments");
  std::lock_guard<std::mutex> lock(m->mu);
  MIX_CUDA(m, cudaSetDevice(m->device));
  if (cb_status st = ensure_graph(m)) return st;
  uint64_t epoch = 0;
  MIX_CUDA(m, cudaMemcpyAsync(m->d_epoch, &epoch, 8, cudaMemcpyHostToDevice, m->stream));
  MIX_CUDA(m, cudaGraphLaunch(m->exec, m->stream));  // generates the batch's LLRs
  std::vector<unsigned long long> init(m->classes.size());
  for (size_t k = 0; k < m->classes.size(); k++)
    init[k] = (cls < 0 || (int32_t)k == cls) ? 0ull : (unsigned long long)m->classes[k].count;
  cudaEvent_t e0, e1;
  MIX_CUDA(m, cudaEventCreate(&e0));
  MIX_CUDA(m, cudaEventCreate(&e1));
  float best = 1e30f;
  for (int r = 0; r <= reps; r++) {
    MIX_CUDA(m, cudaEventRecord(e0, m->stream));
    if (cb_status st = launch_decode_phase(m, init, m->stream)) return st;
    MIX_CUDA(m, cudaEventRecord(e1, m->stream));
    MIX_CUDA(m, cudaEventSynchronize(e1));
    float t = 0;
    MIX_CUDA(m, cudaEventElapsedTime(&t, e0, e1));
    if (r > 0) best = std::min(best, t);  // the first is a warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = best;
  return CB_OK;
}

}  // extern "C"
