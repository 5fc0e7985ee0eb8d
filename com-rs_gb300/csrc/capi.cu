// The C ABI of include/comrs_gb300.h: code objects, device buffers, chunked launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/comrs_gb300.h"
#include "code_host.h"
#include "dev_code.h"
#include "kernels.h"
#include "nr_decode.h"

#define CB_VERSION_STRING "comrs_gb300 0.1.0 (sm_103a)"

namespace {

thread_local std::string g_thread_error;

struct GenCache {
  int m = 0, mbits = 0, n_pad = 0, bpc = 0, spc = 0;
  double log_m = 0;
  std::vector<double> points;  // 2m
  double* d_points = nullptr;
  uint64_t* d_jumps = nullptr;
};

}  // namespace

struct cb_code {
  std::mutex mu;
  int device = 0;
  int precision = 0;
  cbh::NrCode host;
  cbd::DevCode dev;
  cbd::DecCfg cfg;
  int32_t* d_map = nullptr;
  int32_t* d_inv_start = nullptr;
  int32_t* d_inv_t = nullptr;
  void* d_state = nullptr;
  int decode_grid = 0;
  unsigned long long* d_counter = nullptr;
  int32_t* d_status = nullptr;
  cudaStream_t stream = nullptr;
  // host decodes: a copy stream and, per LLR buffer, "copied" and "read by the decoder"
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_copied[2] = {nullptr, nullptr};
  cudaEvent_t ev_read[2] = {nullptr, nullptr};
  // scratch, grown on demand
  void* d_llr = nullptr;
  size_t llr_cap = 0;
  uint32_t* d_bits = nullptr;
  size_t bits_cap = 0;
  uint32_t* d_info = nullptr;
  size_t info_cap = 0;
  void* d_app = nullptr;
  size_t app_cap = 0;
  int32_t* d_iters = nullptr;
  size_t iters_cap = 0;
  cbd::FrameResult* d_results = nullptr;
  size_t results_cap = 0;
  uint8_t* d_u8 = nullptr;
  size_t u8_cap = 0;
  std::vector<uint32_t> h_words;
  std::map<int, GenCache> gen;
  bool dev_ready = false;
  std::string err;
  int exact_demap = 0;  // the frame generator's demapper: 1 exact, 0 max-log
  // the sum-product rule and the flooding schedule: the generic decoder on the lifted rows
  cb_ldpc* generic = nullptr;
  void* d_full = nullptr;
  size_t full_cap = 0;
  void* d_post = nullptr;
  size_t post_cap = 0;
  int32_t* d_giters = nullptr;
  size_t giters_cap = 0;
  // f32 layered min-sum: the graph-specialised decoder (layered_nr.cuh), its launch
  // parameters (the code part filled once) and why it is not the code's own build, if not
  bool use_nr = false;
  cbk::NrKernel nr;
  cbn::NrArgs nr_args;
  std::string nr_note;
  int noalloc_grid = 0;  // resident CTAs of cb_decode_device_noalloc's kernel (0: not yet known)
};

namespace {

cb_status fail(cb_code* c, cb_status s, const std::string& msg) {
  if (c) c->err = msg;
  g_thread_error = msg;
  return s;
}

cb_status cuda_fail(cb_code* c, cudaError_t e, const char* what) {
  return fail(c, CB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CB_CUDA(c, call)                                   \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
  } while (0)

template <typename P>
cudaError_t grow(P*& ptr, size_t& cap, size_t bytes) {
  if (bytes <= cap) return cudaSuccess;
  const size_t want = std::max(bytes, cap * 3 / 2);
  if (ptr) cudaFree((void*)ptr);
  ptr = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc((void**)&ptr, want);
  if (e == cudaSuccess) cap = want;
  return e;
}

size_t elem_size(const cb_code* c) { return c->precision == CB_F64 ? sizeof(double) : sizeof(float); }

// frames per launch chunk of the host-buffer calls: the LLR scratch stays within 2 GB
int64_t chunk_frames(const cb_code* c) {
  size_t per = (size_t)c->host.e * elem_size(c) + 64;
  int64_t n = (int64_t)((size_t)2048 << 20) / (int64_t)per;
  return std::max<int64_t>(1, std::min<int64_t>(n, 65536));
}

// the NR word through the generic decoder: full word, decode, epilogue
template <typename T>
cb_status generic_decode_impl(cb_code* c, const T* llr, int64_t n, uint32_t* bits, T* app, int32_t* iters,
                              const uint32_t* ref, cbd::FrameResult* results, cudaStream_t s) {
  const size_t full_bytes = (size_t)n * c->host.n_full * sizeof(T);
  CB_CUDA(c, grow(c->d_full, c->full_cap, full_bytes));
  CB_CUDA(c, grow(c->d_post, c->post_cap, full_bytes));
  CB_CUDA(c, grow(c->d_giters, c->giters_cap, (size_t)n * 4));
  CB_CUDA(c, cbk::launch_full_llr<T>(c->dev, llr, n, reinterpret_cast<T*>(c->d_full), s));
  if (cb_status st = cb_ldpc_decode_device(c->generic, c->d_full, n, c->d_post, c->d_giters, s))
    return fail(c, st, std::string("generic decoder: ") + cb_ldpc_last_error(c->generic));
  cbk::NrEpilogueArgs<T> e;
  e.post = reinterpret_cast<const T*>(c->d_post);
  e.iters_in = c->d_giters;
  e.n_frames = n;
  e.n_full = c->host.n_full;
  e.k_info = c->host.k_info;
  e.bits_out = bits;
  e.app_out = app;
  e.iters_out = iters;
  e.ref_bits = ref;
  e.results = results;
  CB_CUDA(c, cbk::launch_nr_epilogue<T>(e, s));
  return CB_OK;
}

template <typename T>
cb_status decode_device_impl(cb_code* c, const T* llr, int64_t n, uint32_t* bits, T* app, int32_t* iters,
                             const uint32_t* ref, cbd::FrameResult* results, cudaStream_t s) {
  if (c->generic) return generic_decode_impl<T>(c, llr, n, bits, app, iters, ref, results, s);
  if constexpr (sizeof(T) == 4) {
    if (c->use_nr) {
      cbn::NrArgs& a = c->nr_args;
      a.llr = llr;
      a.n_frames = n;
      a.bits_out = bits;
      a.app_out = app;
      a.iters_out = iters;
      a.ref_bits = ref;
      a.results = reinterpret_cast<cbn::FrameRecord*>(results);
      a.state = reinterpret_cast<unsigned char*>(c->d_state);
      a.work_counter = c->d_counter;
      CB_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), s));
      CB_CUDA(c, cbk::nr_launch(c->nr, a, (int)std::min<int64_t>(c->decode_grid, n), s));
      return CB_OK;
    }
  }
  cbk::DecodeArgs<T> a;
  a.code = c->dev;
  a.cfg = c->cfg;
  a.llr = llr;
  a.n_frames = n;
  a.bits_out = bits;
  a.app_out = app;
  a.post_out = nullptr;
  a.iters_out = iters;
  a.ref_bits = ref;
  a.results = results;
  a.state = reinterpret_cast<T*>(c->d_state);
  a.work_counter = reinterpret_cast<int32_t*>(c->d_counter);
  a.status = c->d_status;
  CB_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), s));
  int grid = (int)std::min<int64_t>(c->decode_grid, n);
  CB_CUDA(c, cbk::launch_decode<T>(a, grid, s));
  return CB_OK;
}

cb_status gen_config(cb_code* c, int m, GenCache** out) {
  auto it = c->gen.find(m);
  if (it != c->gen.end()) { *out = &it->second; return CB_OK; }
  GenCache g;
  if (!cbh::qam_points(m, g.points, g.log_m)) return fail(c, CB_ERR_CONFIG, "modulation order must be 4, 16, 64 or 256");
  g.m = m;
  const cbh::GenTables t = cbh::gen_tables(c->host.k_info, c->host.e, m, cbk::kGenBitsThreads, cbk::kGenNoiseThreads);
  g.mbits = t.mbits;
  g.n_pad = t.n_pad;
  g.bpc = t.bits_per_chunk;
  g.spc = t.syms_per_chunk;
  const std::vector<uint64_t>& polys = t.jumps;
  CB_CUDA(c, cudaMalloc(&g.d_points, sizeof(double) * 2 * m));
  CB_CUDA(c, cudaMemcpy(g.d_points, g.points.data(), sizeof(double) * 2 * m, cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMalloc(&g.d_jumps, polys.size() * 8));
  CB_CUDA(c, cudaMemcpy(g.d_jumps, polys.data(), polys.size() * 8, cudaMemcpyHostToDevice));
  auto res = c->gen.emplace(m, g);
  *out = &res.first->second;
  return CB_OK;
}

template <typename T>
cb_status gen_device(cb_code* c, GenCache* g, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first,
                     int64_t n, double ebn0_db, T* llr, uint32_t* info, cudaStream_t s,
                     const float* ebn0_frames = nullptr, uint32_t* cw_out = nullptr) {
  cbk::GenArgs<T> a;
  a.code = c->dev;
  a.m = g->m;
  a.mbits = g->mbits;
  a.points = g->d_points;
  a.log_m = g->log_m;
  // b = log2 M * R (com-spec blocks/channel.rs:145-149), times db2lin (units.rs:38-40)
  double rate = (double)c->host.k_info / (double)c->host.e;
  double b = (double)g->mbits * rate;
  a.b_ebn0 = b * std::pow(10.0, ebn0_db / 10.0);
  a.seed = seed;
  a.name_hash = name_hash;
  a.cond = cond;
  a.first_frame = first;
  a.n_frames = n;
  a.jumps = g->d_jumps;
  a.bits_per_chunk = g->bpc;
  a.syms_per_chunk = g->spc;
  a.n_pad = g->n_pad;
  a.llr_out = llr;
  a.info_out = info;
  a.ebn0_frames = ebn0_frames;
  a.b_bits = b;
  a.cw_out = cw_out;
  a.exact = c->exact_demap;
  CB_CUDA(c, cbk::launch_gen<T>(a, s));
  return CB_OK;
}

template <typename T>
cb_status run_frames_impl(cb_code* c, int m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first,
                          int64_t n, double ebn0_db, cb_frame_result* out, void* llr_host, uint8_t* info_host) {
  GenCache* g;
  cb_status st = gen_config(c, m, &g);
  if (st) return st;
  const int wpf = (c->host.k_info + 31) / 32;
  const int64_t chunk = chunk_frames(c);
  for (int64_t done = 0; done < n; done += chunk) {
    int64_t cnt = std::min(chunk, n - done);
    CB_CUDA(c, grow(c->d_llr, c->llr_cap, (size_t)cnt * c->host.e * sizeof(T)));
    CB_CUDA(c, grow(c->d_info, c->info_cap, (size_t)cnt * wpf * 4));
    CB_CUDA(c, grow(c->d_results, c->results_cap, (size_t)cnt * sizeof(cbd::FrameResult)));
    T* llr = reinterpret_cast<T*>(c->d_llr);
    st = gen_device<T>(c, g, seed, name_hash, cond, first + (uint64_t)done, cnt, ebn0_db, llr, c->d_info, c->stream);
    if (st) return st;
    if (out) {
      st = decode_device_impl<T>(c, llr, cnt, nullptr, nullptr, nullptr, c->d_info, c->d_results, c->stream);
      if (st) return st;
      CB_CUDA(c, cudaMemcpyAsync(out + done, c->d_results, (size_t)cnt * sizeof(cb_frame_result),
                                 cudaMemcpyDeviceToHost, c->stream));
    }
    if (llr_host)
      CB_CUDA(c, cudaMemcpyAsync(reinterpret_cast<T*>(llr_host) + (size_t)done * c->host.e, llr,
                                 (size_t)cnt * c->host.e * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    if (info_host) {
      c->h_words.resize((size_t)cnt * wpf);
      CB_CUDA(c, cudaMemcpyAsync(c->h_words.data(), c->d_info, (size_t)cnt * wpf * 4, cudaMemcpyDeviceToHost,
                                 c->stream));
      CB_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int64_t f = 0; f < cnt; f++)
        for (int i = 0; i < c->host.k_info; i++)
          info_host[(size_t)(done + f) * c->host.k_info + i] =
              (uint8_t)((c->h_words[(size_t)f * wpf + i / 32] >> (i % 32)) & 1u);
    }
  }
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  return CB_OK;
}

// frames on a caller stream: results (and optionally the LLRs / info words) in device
// memory; the LLRs go to the caller's buffer or to the code's scratch
template <typename T>
cb_status trial_device_impl(cb_code* c, int m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first,
                            int64_t n, double ebn0_db, cbd::FrameResult* results, T* llr_dev, uint32_t* info_dev,
                            cudaStream_t s) {
  GenCache* g;
  cb_status st = gen_config(c, m, &g);
  if (st) return st;
  const int wpf = (c->host.k_info + 31) / 32;
  if (!llr_dev) {
    CB_CUDA(c, grow(c->d_llr, c->llr_cap, (size_t)n * c->host.e * sizeof(T)));
    llr_dev = reinterpret_cast<T*>(c->d_llr);
  }
  if (!info_dev) {
    CB_CUDA(c, grow(c->d_info, c->info_cap, (size_t)n * wpf * 4));
    info_dev = c->d_info;
  }
  st = gen_device<T>(c, g, seed, name_hash, cond, first, n, ebn0_db, llr_dev, info_dev, s);
  if (st || !results) return st;
  return decode_device_impl<T>(c, llr_dev, n, nullptr, nullptr, nullptr, info_dev, results, s);
}

// the decisions (packed to bytes), a posteriori LLRs and iteration counts of frames
// [done, done + cnt) from the device buffers to the caller's host buffers, on the code's
// stream
template <typename T>
cb_status copy_back(cb_code* c, int64_t done, int64_t cnt, int wpf, int bpf, uint8_t* bits, T* app, int32_t* iters) {
  if (bits) {
    if (bpf == wpf * 4) {
      CB_CUDA(c, cudaMemcpyAsync(bits + (size_t)done * bpf, c->d_bits, (size_t)cnt * bpf, cudaMemcpyDeviceToHost,
                                 c->stream));
    } else {
      c->h_words.resize((size_t)cnt * wpf);
      CB_CUDA(c, cudaMemcpyAsync(c->h_words.data(), c->d_bits, (size_t)cnt * wpf * 4, cudaMemcpyDeviceToHost,
                                 c->stream));
      CB_CUDA(c, cudaStreamSynchronize(c->stream));
      for (int64_t f = 0; f < cnt; f++) std::memcpy(bits + (size_t)(done + f) * bpf, &c->h_words[(size_t)f * wpf], bpf);
    }
  }
  if (app)
    CB_CUDA(c, cudaMemcpyAsync(app + (size_t)done * c->host.k_info, c->d_app, (size_t)cnt * c->host.k_info * sizeof(T),
                               cudaMemcpyDeviceToHost, c->stream));
  if (iters) CB_CUDA(c, cudaMemcpyAsync(iters + done, c->d_iters, (size_t)cnt * 4, cudaMemcpyDeviceToHost, c->stream));
  return CB_OK;
}

// The address at which `device` reads a host buffer in place (page-locked memory, mapped
// under unified addressing, and allocated for that device or portable to every device),
// or nullptr
template <typename T>
const T* mapped_host(const T* p, int device) {
  cudaPointerAttributes pa;
  unsigned int flags = 0;
  if (cudaPointerGetAttributes(&pa, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (pa.type != cudaMemoryTypeHost || !pa.devicePointer) return nullptr;
  if (pa.device != device) {
    if (cudaHostGetFlags(&flags, const_cast<T*>(p)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (!(flags & cudaHostAllocPortable)) return nullptr;
  }
  return static_cast<const T*>(pa.devicePointer);
}

template <typename T>
cb_status decode_host_impl(cb_code* c, const T* llr, int64_t n, uint8_t* bits, T* app, int32_t* iters) {
  const int wpf = (c->host.k_info + 31) / 32;
  const int bpf = (c->host.k_info + 7) / 8;
  // Page-locked host LLRs: the decoder reads them where they are (over NVLink-C2C on a
  // Grace host), one launch per chunk of frames with no staging copy; only the decisions,
  // a posteriori LLRs and counts come back by copies.
  if (const T* dev_llr = mapped_host(llr, c->device)) {
    const int64_t chunk = std::min<int64_t>(n, chunk_frames(c));
    CB_CUDA(c, grow(c->d_bits, c->bits_cap, (size_t)chunk * wpf * 4));
    if (app) CB_CUDA(c, grow(c->d_app, c->app_cap, (size_t)chunk * c->host.k_info * sizeof(T)));
    if (iters) CB_CUDA(c, grow(c->d_iters, c->iters_cap, (size_t)chunk * 4));
    for (int64_t done = 0; done < n; done += chunk) {
      const int64_t cnt = std::min(chunk, n - done);
      cb_status st = decode_device_impl<T>(c, dev_llr + (size_t)done * c->host.e, cnt, c->d_bits,
                                           app ? reinterpret_cast<T*>(c->d_app) : nullptr,
                                           iters ? c->d_iters : nullptr, nullptr, nullptr, c->stream);
      if (st) return st;
      if (cb_status rs = copy_back(c, done, cnt, wpf, bpf, bits, app, iters)) return rs;
    }
    CB_CUDA(c, cudaStreamSynchronize(c->stream));
    return CB_OK;
  }
  // Host LLRs in chunks: chunk i + 1 is copied on the copy stream while chunk i decodes on
  // the code's stream, through two device buffers (an event per buffer marks its copy
  // done, another the decode that read it); decisions and counts go back on the decode
  // stream.  Each chunk holds at least one persistent grid's worth of codewords.
  const size_t per = (size_t)c->host.e * sizeof(T);
  const int64_t grid = std::max(1, c->decode_grid);
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(chunk_frames(c) / 2,
                                                               std::max<int64_t>(grid, (n + 3) / 4)));
  const int64_t buf_frames = std::min(chunk, n);
  CB_CUDA(c, grow(c->d_llr, c->llr_cap, 2 * (size_t)buf_frames * per));
  CB_CUDA(c, grow(c->d_bits, c->bits_cap, (size_t)buf_frames * wpf * 4));
  if (app) CB_CUDA(c, grow(c->d_app, c->app_cap, (size_t)buf_frames * c->host.k_info * sizeof(T)));
  if (iters) CB_CUDA(c, grow(c->d_iters, c->iters_cap, (size_t)buf_frames * 4));
  for (int64_t done = 0, i = 0; done < n; done += chunk, i++) {
    const int64_t cnt = std::min(chunk, n - done);
    const int half = (int)(i & 1);
    T* d_llr = reinterpret_cast<T*>(reinterpret_cast<char*>(c->d_llr) + (size_t)half * buf_frames * per);
    // the copy waits until the decode two chunks back has read this buffer
    if (i >= 2) CB_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->ev_read[half], 0));
    CB_CUDA(c, cudaMemcpyAsync(d_llr, llr + (size_t)done * c->host.e, (size_t)cnt * per, cudaMemcpyHostToDevice,
                               c->copy_stream));
    CB_CUDA(c, cudaEventRecord(c->ev_copied[half], c->copy_stream));
    CB_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_copied[half], 0));
    cb_status st = decode_device_impl<T>(c, d_llr, cnt, c->d_bits, app ? reinterpret_cast<T*>(c->d_app) : nullptr,
                                         iters ? c->d_iters : nullptr, nullptr, nullptr, c->stream);
    if (st) return st;
    CB_CUDA(c, cudaEventRecord(c->ev_read[half], c->stream));
    if (cb_status rs = copy_back(c, done, cnt, wpf, bpf, bits, app, iters)) return rs;
  }
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  return CB_OK;
}


// Device resources are created on first use, so that a code object (its tables and the
// host encoder) also exists on a machine without a GPU.
cb_status ensure_device(cb_code* c) {
  if (c->dev_ready) return CB_OK;
  const cbh::NrCode& h = c->host;
  cbd::DevCode& v = c->dev;
  CB_CUDA(c, cudaSetDevice(c->device));
  CB_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CB_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  for (int i = 0; i < 2; i++) {
    CB_CUDA(c, cudaEventCreateWithFlags(&c->ev_copied[i], cudaEventDisableTiming));
    CB_CUDA(c, cudaEventCreateWithFlags(&c->ev_read[i], cudaEventDisableTiming));
  }
  CB_CUDA(c, cudaMalloc(&c->d_map, sizeof(int32_t) * h.e));
  CB_CUDA(c, cudaMemcpy(c->d_map, h.map.data(), sizeof(int32_t) * h.e, cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMalloc(&c->d_inv_start, sizeof(int32_t) * (h.n_full + 1)));
  CB_CUDA(c, cudaMemcpy(c->d_inv_start, h.inv_start.data(), sizeof(int32_t) * (h.n_full + 1), cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMalloc(&c->d_inv_t, sizeof(int32_t) * h.e));
  CB_CUDA(c, cudaMemcpy(c->d_inv_t, h.inv_t.data(), sizeof(int32_t) * h.e, cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMalloc(&c->d_counter, 64));
  CB_CUDA(c, cudaMalloc(&c->d_status, 64));
  CB_CUDA(c, cudaMemset(c->d_status, 0, 64));
  v.map = c->d_map;
  v.inv_start = c->d_inv_start;
  v.inv_t = c->d_inv_t;
  // f32 layered min-sum: the graph-specialised decoder, built for this code's lifting when
  // the run-time compiler is at hand, else the base graph's build
  if (c->precision == CB_F32 && !c->generic && c->cfg.layered &&
      (c->cfg.rule == cbd::RULE_NMS || c->cfg.rule == cbd::RULE_OMS)) {
    c->nr = cbk::nr_kernel(h, c->device, true, &c->nr_note, false, c->cfg.rule);
    int g = c->nr.fn ? cbk::nr_grid_size(c->nr, h, c->device) : 0;
    if (g <= 0 && c->nr.specialized) {
      cudaGetLastError();
      c->nr_note = "the specialised decoder's occupancy query failed";
      c->nr = cbk::nr_kernel(h, c->device, false, nullptr);
      g = cbk::nr_grid_size(c->nr, h, c->device);
    }
    if (g > 0) {
      c->use_nr = true;
      c->decode_grid = g;
      cbk::fill_nr_args(h, c->nr_args);
      c->nr_args.map = c->d_map;
      c->nr_args.inv_start = c->d_inv_start;
      c->nr_args.inv_t = c->d_inv_t;
      c->nr_args.max_iterations = c->cfg.max_iterations;
      c->nr_args.rule = c->cfg.rule;
      c->nr_args.alpha = (float)c->cfg.alpha;
    }
    cudaGetLastError();
  }
  if (!c->use_nr) c->decode_grid = cbk::decode_grid_size(v, c->precision, c->device);
  if (c->decode_grid <= 0) return fail(c, CB_ERR_CUDA, "the decoder does not fit an SM (occupancy 0)");
  CB_CUDA(c, cudaMalloc(&c->d_state, cbk::decode_state_bytes_per_slot(v, c->precision) * c->decode_grid));
  c->dev_ready = true;
  return CB_OK;
}

}  // namespace

extern "C" {

const char* cb_version(void) { return CB_VERSION_STRING; }

const char* cb_last_error(const cb_code* c) { return c ? c->err.c_str() : g_thread_error.c_str(); }

cb_status cb_code_create(const cb_code_desc* d, cb_code** out) {
  if (!out) return fail(nullptr, CB_ERR_CONFIG, "out is NULL");
  *out = nullptr;
  if (!d) return fail(nullptr, CB_ERR_CONFIG, "desc is NULL");
  if (d->precision != CB_F64 && d->precision != CB_F32) return fail(nullptr, CB_ERR_CONFIG, "precision is 0 or 1");
  if (d->rule != CB_RULE_SUM_PRODUCT && d->rule != CB_RULE_NMS && d->rule != CB_RULE_OMS)
    return fail(nullptr, CB_ERR_CONFIG, "rule must be sum_product, normalized_min_sum or offset_min_sum");
  if (d->max_iterations < 0 || d->max_iterations > 255) return fail(nullptr, CB_ERR_CONFIG, "max_iterations in 0..255");
  if (!(std::isfinite(d->alpha))) return fail(nullptr, CB_ERR_CONFIG, "alpha must be finite");
  cbh::CodeSpec spec;
  spec.k_info = d->k_info;
  spec.e = d->e;
  spec.bg = d->base_graph;
  spec.z = d->lifting_size;
  spec.rv = d->rv;
  spec.qm = d->qm;
  cb_code* c = new cb_code();
  std::string err;
  if (!cbh::build_nr_code(spec, c->host, err)) {
    delete c;
    return fail(nullptr, CB_ERR_CONFIG, err);
  }
  // the decoder is compiled for the row degrees of the NR base graphs
  if (!cbk::degrees_supported(c->host)) {
    delete c;
    return fail(nullptr, CB_ERR_CONFIG, "a base-graph row degree outside 3..10 and 19");
  }
  c->device = d->device;
  c->precision = d->precision;
  c->cfg.rule = d->rule;
  c->cfg.alpha = d->alpha;
  c->cfg.layered = d->layered;
  c->cfg.max_iterations = d->max_iterations;
  cbk::fill_dev_code(c->host, c->dev);
  if (d->rule == CB_RULE_SUM_PRODUCT || !d->layered) {
    // lifted row (L, r) holds, for the entries (j, s) of base row L in table order, the
    // variable j Z + (r + s) mod Z (nr/ldpc.rs:124-134)
    const cbh::NrCode& h = c->host;
    std::vector<int32_t> start(1, 0), vars;
    vars.reserve((size_t)h.edges);
    for (int L = 0; L < h.rows_n; L++)
      for (int r = 0; r < h.z; r++) {
        for (int t = h.layer_start[L]; t < h.layer_start[L + 1]; t++)
          vars.push_back(h.entry_col[t] * h.z + (r + h.entry_shift[t]) % h.z);
        start.push_back((int32_t)vars.size());
      }
    if (cb_status st = cb_ldpc_create(h.n_full, h.rows_n * h.z, start.data(), vars.data(), d->rule, d->alpha,
                                      d->layered, d->max_iterations, d->precision, d->device, &c->generic)) {
      std::string msg = cb_ldpc_last_error(nullptr);
      delete c;
      return fail(nullptr, st, msg);
    }
  }
  *out = c;
  return CB_OK;
}

void cb_code_destroy(cb_code* c) {
  if (!c) return;
  if (c->dev_ready || c->stream) cudaSetDevice(c->device);
  for (auto& kv : c->gen) {
    cudaFree(kv.second.d_points);
    cudaFree(kv.second.d_jumps);
  }
  cb_ldpc_destroy(c->generic);
  void* bufs[] = {c->d_map, c->d_inv_start, c->d_inv_t, c->d_state, c->d_counter, c->d_status, c->d_llr, c->d_bits,
                  c->d_info, c->d_app, c->d_iters, c->d_results, c->d_u8, c->d_full, c->d_post, c->d_giters};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (int i = 0; i < 2; i++) {
    if (c->ev_copied[i]) cudaEventDestroy(c->ev_copied[i]);
    if (c->ev_read[i]) cudaEventDestroy(c->ev_read[i]);
  }
  delete c;
}

cb_status cb_code_set_demapper(cb_code* c, int32_t exact) {
  if (!c) return fail(nullptr, CB_ERR_CONFIG, "NULL code");
  if (exact != 0 && exact != 1) return fail(c, CB_ERR_CONFIG, "demapper: 0 (max-log) or 1 (exact)");
  std::lock_guard<std::mutex> lock(c->mu);
  c->exact_demap = exact;
  return CB_OK;
}

cb_status cb_code_prepare(cb_code* c) {
  if (!c) return fail(nullptr, CB_ERR_CONFIG, "NULL code");
  if (c->precision != CB_F32 || c->generic || !c->cfg.layered ||
      (c->cfg.rule != cbd::RULE_NMS && c->cfg.rule != cbd::RULE_OMS))
    return fail(c, CB_ERR_CONFIG, "only f32 layered min-sum codes run a decoder compiled for their lifting");
  std::lock_guard<std::mutex> lock(c->mu);
  std::string note;
  if (!cbk::nr_prepare(c->host, &note, false, c->cfg.rule))
    return fail(c, CB_ERR_IO, "no decoder compiled for this lifting: " + note);
  if (!cbk::nr_prepare(c->host, &note, true))
    return fail(c, CB_ERR_IO, "no learned decoder compiled for this lifting: " + note);
  return CB_OK;
}

cb_status cb_code_info(const cb_code* c, int64_t info[16]) {
  if (!c || !info) return fail(nullptr, CB_ERR_CONFIG, "NULL argument");
  const cbh::NrCode& h = c->host;
  const int64_t kind = !c->dev_ready ? -1 : !c->use_nr ? 0 : c->nr.specialized ? 2 : 1;
  int64_t v[16] = {h.bg, h.z, h.k_info, h.e, h.k, h.n_full, (int64_t)h.rows_n * h.z, h.edges, h.ils, h.max_degree,
                   h.rv, h.qm, (int64_t)h.core_terms.size(), h.map_is_offset ? 1 : 0, (int64_t)h.entry_col.size(),
                   kind};
  std::memcpy(info, v, sizeof v);
  return CB_OK;
}

cb_status cb_code_tables(const cb_code* c, int32_t* entries, int32_t* bit_map) {
  if (!c) return fail(nullptr, CB_ERR_CONFIG, "NULL code");
  const cbh::NrCode& h = c->host;
  if (entries) {
    int t = 0;
    for (int L = 0; L < h.rows_n; L++)
      for (int i = h.layer_start[L]; i < h.layer_start[L + 1]; i++, t++) {
        entries[3 * t] = L;
        entries[3 * t + 1] = h.entry_col[i];
        entries[3 * t + 2] = h.entry_shift[i];
      }
  }
  if (bit_map) std::memcpy(bit_map, h.map.data(), sizeof(int32_t) * h.e);
  return CB_OK;
}

cb_status cb_encode(cb_code* c, const uint8_t* info, int64_t n, uint8_t* out) {
  if (!c || !info || !out || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  std::lock_guard<std::mutex> lock(c->mu);
  // host encoder over the same construction tables (the GPU encoder lives inside the
  // frame generator, where the bits are drawn)
  const cbh::NrCode& h = c->host;
  std::vector<uint8_t> cw(h.n_full), syn(4 * h.z);
  for (int64_t f = 0; f < n; f++) {
    std::fill(cw.begin(), cw.end(), 0);
    for (int i = 0; i < h.k_info; i++) cw[i] = info[(size_t)f * h.k_info + i] & 1;
    for (int L = 0; L < 4; L++)
      for (int r = 0; r < h.z; r++) {
        uint8_t a = 0;
        for (int t = h.layer_start[L]; t < h.layer_start[L + 1]; t++)
          if (h.entry_col[t] < h.cols_k) a ^= cw[h.entry_col[t] * h.z + (r + h.entry_shift[t]) % h.z];
        syn[L * h.z + r] = a;
      }
    for (int blk = 0; blk < 4; blk++)
      for (int r = 0; r < h.z; r++) {
        uint8_t a = 0;
        for (auto& ct : h.core_terms)
          if (ct.block == blk) a ^= syn[ct.src * h.z + (r + ct.shift) % h.z];
        cw[h.k + blk * h.z + r] = a;
      }
    for (int L = 4; L < h.rows_n; L++)
      for (int r = 0; r < h.z; r++) {
        int own = h.k + L * h.z + r;
        uint8_t a = 0;
        for (int t = h.layer_start[L]; t < h.layer_start[L + 1]; t++) {
          int col = h.entry_col[t] * h.z + (r + h.entry_shift[t]) % h.z;
          if (col != own) a ^= cw[col];
        }
        cw[own] = a;
      }
    for (int t = 0; t < h.e; t++) out[(size_t)f * h.e + t] = cw[h.map[t]];
  }
  return CB_OK;
}

cb_status cb_decode(cb_code* c, const void* llr, int64_t n, uint8_t* bits, void* app, int32_t* iters) {
  if (!c || !llr || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  if (c->precision == CB_F64)
    return decode_host_impl<double>(c, (const double*)llr, n, bits, (double*)app, iters);
  return decode_host_impl<float>(c, (const float*)llr, n, bits, (float*)app, iters);
}

cb_status cb_decode_device(cb_code* c, const void* llr, int64_t n, uint32_t* bits, void* app, int32_t* iters,
                           void* stream) {
  if (!c || !llr || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == CB_F64)
    return decode_device_impl<double>(c, (const double*)llr, n, bits, (double*)app, iters, nullptr, nullptr, s);
  return decode_device_impl<float>(c, (const float*)llr, n, bits, (float*)app, iters, nullptr, nullptr, s);
}

cb_status cb_run_frames(cb_code* c, int32_t m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first,
                        int64_t n, double ebn0_db, cb_frame_result* out) {
  if (!c || !out || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  if (!std::isfinite(ebn0_db)) return fail(c, CB_ERR_CONFIG, "Eb/N0 must be finite");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  if (c->precision == CB_F64)
    return run_frames_impl<double>(c, m, seed, name_hash, cond, first, n, ebn0_db, out, nullptr, nullptr);
  return run_frames_impl<float>(c, m, seed, name_hash, cond, first, n, ebn0_db, out, nullptr, nullptr);
}

cb_status cb_generate_frames(cb_code* c, int32_t m, uint64_t seed, uint64_t name_hash, uint64_t cond,
                             uint64_t first, int64_t n, double ebn0_db, void* llr, uint8_t* info) {
  if (!c || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  if (!std::isfinite(ebn0_db)) return fail(c, CB_ERR_CONFIG, "Eb/N0 must be finite");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  if (c->precision == CB_F64)
    return run_frames_impl<double>(c, m, seed, name_hash, cond, first, n, ebn0_db, nullptr, llr, info);
  return run_frames_impl<float>(c, m, seed, name_hash, cond, first, n, ebn0_db, nullptr, llr, info);
}

cb_status cb_run_frames_device(cb_code* c, int32_t m, uint64_t seed, uint64_t name_hash, uint64_t cond,
                               uint64_t first, int64_t n, double ebn0_db, cb_frame_result* results_dev, void* stream) {
  if (!c || !results_dev || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  if (!std::isfinite(ebn0_db)) return fail(c, CB_ERR_CONFIG, "Eb/N0 must be finite");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  cbd::FrameResult* r = reinterpret_cast<cbd::FrameResult*>(results_dev);
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == CB_F64)
    return trial_device_impl<double>(c, m, seed, name_hash, cond, first, n, ebn0_db, r, nullptr, nullptr, s);
  return trial_device_impl<float>(c, m, seed, name_hash, cond, first, n, ebn0_db, r, nullptr, nullptr, s);
}

cb_status cb_generate_frames_device(cb_code* c, int32_t m, uint64_t seed, uint64_t name_hash, uint64_t cond,
                                    uint64_t first, int64_t n, double ebn0_db, void* llr_dev, uint32_t* info_dev,
                                    void* stream) {
  if (!c || !llr_dev || !info_dev || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  if (!std::isfinite(ebn0_db)) return fail(c, CB_ERR_CONFIG, "Eb/N0 must be finite");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  if (n == 0) return CB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == CB_F64)
    return trial_device_impl<double>(c, m, seed, name_hash, cond, first, n, ebn0_db, nullptr, (double*)llr_dev,
                                     info_dev, s);
  return trial_device_impl<float>(c, m, seed, name_hash, cond, first, n, ebn0_db, nullptr, (float*)llr_dev,
                                  info_dev, s);
}

cb_status cb_xoshiro_jump(const uint64_t state[4], uint64_t steps, uint64_t out[4]) {
  if (!state || !out) return fail(nullptr, CB_ERR_CONFIG, "NULL argument");
  uint64_t s[4] = {state[0], state[1], state[2], state[3]};
  cbh::xoshiro_apply_jump(s, cbh::xoshiro_jump_poly(steps));
  std::memcpy(out, s, sizeof s);
  return CB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- learned min-sum
struct cb_nms {
  cb_code* code = nullptr;
  int T = 0, shared = 0, step = 0;
  // evaluation on the graph-specialised decoder (layered_nr_kernel with NrLearnedArgs):
  // its kernel and grid (0: not usable, -1: not yet looked at)
  cbk::NrKernel nr;
  int nr_grid = -1;
  int info_only_loss = 0;  // 1: the loss covers the K' information bits only
  int64_t nw = 0;        // weights per kind (scales, offsets)
  float* d_w = nullptr;  // [2 nw]: scales then offsets
  // a host copy of d_w for the launch parameters of evaluation, valid until the weights
  // change (cb_nms_set_weights, a training step)
  std::vector<float> h_w;
  bool h_w_valid = false;
  float* d_g = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  float* d_X = nullptr;
  size_t X_cap = 0;
  float* d_P = nullptr;
  size_t P_cap = 0;
  float* d_c2v = nullptr;
  size_t c2v_cap = 0;
  float* d_post = nullptr;
  size_t post_cap = 0;
  float* d_llr = nullptr;
  size_t llr_cap = 0;
  uint32_t* d_cw = nullptr;
  size_t cw_cap = 0;
  uint32_t* d_info = nullptr;
  size_t info_cap = 0;
  float* d_ebn0 = nullptr;
  size_t ebn0_cap = 0;
  float* d_loss = nullptr;
  cbd::FrameResult* d_res = nullptr;
  size_t res_cap = 0;
  std::vector<uint32_t> h_words;
};

namespace {

cb_status nms_buffers(cb_nms* h, int64_t n, bool train) {
  cb_code* c = h->code;
  const size_t edges = (size_t)c->dev.n_entries * c->dev.z;
  CB_CUDA(c, grow(h->d_c2v, h->c2v_cap, (size_t)n * edges * 4));
  CB_CUDA(c, grow(h->d_llr, h->llr_cap, (size_t)n * c->host.e * 4));
  CB_CUDA(c, grow(h->d_post, h->post_cap, (size_t)n * c->host.n_full * 4));
  CB_CUDA(c, grow(h->d_info, h->info_cap, (size_t)n * ((c->host.k_info + 31) / 32) * 4));
  CB_CUDA(c, grow(h->d_res, h->res_cap, (size_t)n * sizeof(cbd::FrameResult)));
  if (train) {
    CB_CUDA(c, grow(h->d_X, h->X_cap, (size_t)n * h->T * edges * 4));
    CB_CUDA(c, grow(h->d_P, h->P_cap, (size_t)n * h->T * c->host.n_full * 4));
    CB_CUDA(c, grow(h->d_cw, h->cw_cap, (size_t)n * ((c->host.n_full + 31) / 32) * 4));
    CB_CUDA(c, grow(h->d_ebn0, h->ebn0_cap, (size_t)n * 4));
  }
  return CB_OK;
}

// Whether the network's weights go in the launch parameters: shared, small enough, and a
// large lifting.  With Z >= 128 few CTAs share an SM and the weights stay in the constant
// cache (BG1 Z = 384: 3.9 against 3.2 Gbit/s from global memory), and shared memory has
// no room left beside the posteriors; with small Z a dozen CTAs at different iterations
// thrash that cache, and each iteration's weights are staged in shared memory instead.
// Then `w` receives a host copy of the weights (scales then offsets).
// The graph-specialised learned kernel serves evaluation when the code's plain decoder is
// the graph-specialised one, the weights are shared and fit the launch parameters, and
// the lifting is large: the same results as the table-driven learned decoder, at 1.40x
// the plain decoder's time per iteration on BG1 Z = 384 (C5 at its FER 1e-3 point: 8.5 ms
// for 8192 frames, 13.8 ms with the table-driven kernel).  With Z = 52 (C4) a dozen CTAs
// share an SM, and with its weights read from the launch parameters it ran 2.5-3.4x the
// plain decoder's time per iteration, slower than the table-driven kernel with its weights
// in shared memory, which such codes keep.
int nms_nr_grid(cb_nms* h) {
  cb_code* c = h->code;
  if (h->nr_grid >= 0) return h->nr_grid;
  h->nr_grid = 0;
  // the weight rows of T iterations and the first iteration's zero row
  if (!c->use_nr || !h->shared || c->dev.z < 128 || h->nw + c->dev.n_entries > cbn::kNrMaxLearnedWeights) return 0;
  h->nr = cbk::nr_kernel(c->host, c->device, c->nr.specialized, nullptr, true);
  int g = h->nr.fn ? cbk::nr_learned_grid_size(h->nr, c->host, c->device) : 0;
  if (g <= 0 && h->nr.specialized) {
    cudaGetLastError();
    h->nr = cbk::nr_kernel(c->host, c->device, false, nullptr, true);
    g = h->nr.fn ? cbk::nr_learned_grid_size(h->nr, c->host, c->device) : 0;
  }
  cudaGetLastError();
  // the code's state slots were allocated for the plain decoder's grid
  h->nr_grid = std::max(0, std::min(g, c->decode_grid));
  return h->nr_grid;
}

cb_status nms_param_weights(cb_nms* h, std::vector<float>& w, bool& in_params) {
  cb_code* c = h->code;
  in_params = nms_nr_grid(h) > 0 || (h->shared && h->nw <= cbk::kMaxParamWeights && c->dev.z >= 128);
  if (!in_params) return CB_OK;
  if (!h->h_w_valid) {
    h->h_w.resize((size_t)2 * h->nw);
    CB_CUDA(c, cudaMemcpyAsync(h->h_w.data(), h->d_w, h->h_w.size() * 4, cudaMemcpyDeviceToHost, c->stream));
    CB_CUDA(c, cudaStreamSynchronize(c->stream));
    h->h_w_valid = true;
  }
  w = h->h_w;
  return CB_OK;
}

// evaluation of the learned min-sum: the layered decoder with the network's weights and
// the syndrome stop (the same results as the training forward with an early stop)
cb_status nms_eval(cb_nms* h, const float* llr, int64_t n, const uint32_t* ref, cbd::FrameResult* results,
                   float* post, int32_t* iters, cudaStream_t s, const std::vector<float>* param_w) {
  cb_code* c = h->code;
  cbk::DecodeArgs<float> a;
  a.code = c->dev;
  a.cfg = c->cfg;
  a.cfg.max_iterations = h->T;
  a.llr = llr;
  a.n_frames = n;
  a.bits_out = nullptr;
  a.app_out = nullptr;
  a.post_out = post;
  a.iters_out = iters;
  a.ref_bits = ref;
  a.results = results;
  a.state = reinterpret_cast<float*>(c->d_state);
  a.work_counter = reinterpret_cast<int32_t*>(c->d_counter);
  a.status = c->d_status;
  a.l_alpha = h->d_w;
  a.l_beta = h->d_w + h->nw;
  a.l_shared = h->shared;
  // shared weights not in the launch parameters: each iteration's staged in shared memory
  a.l_smem = h->shared && !param_w;
  CB_CUDA(c, cudaMemsetAsync(c->d_counter, 0, sizeof(unsigned long long), s));
  if (param_w && h->nr_grid > 0) {
    // ~30 KB of launch parameters: built once per call site, copied by the launch
    static thread_local cbn::NrLearnedArgs la;
    la.a = c->nr_args;
    la.a.max_iterations = h->T;
    la.a.llr = llr;
    la.a.n_frames = n;
    la.a.bits_out = nullptr;
    la.a.app_out = nullptr;
    la.a.iters_out = iters;
    la.a.ref_bits = ref;
    la.a.results = reinterpret_cast<cbn::FrameRecord*>(results);
    la.a.state = reinterpret_cast<unsigned char*>(c->d_state);
    la.a.work_counter = c->d_counter;
    la.post_out = post;
    // row 0: scale 0, offset +inf (no old messages in the first iteration); then the
    // network's rows
    const int ne = c->dev.n_entries;
    std::fill(la.alpha, la.alpha + ne, 0.0f);
    std::fill(la.beta, la.beta + ne, std::numeric_limits<float>::infinity());
    std::memcpy(la.alpha + ne, param_w->data(), (size_t)h->nw * 4);
    std::memcpy(la.beta + ne, param_w->data() + h->nw, (size_t)h->nw * 4);
    CB_CUDA(c, cbk::nr_learned_launch(h->nr, la, (int)std::min<int64_t>(h->nr_grid, n), s));
    return CB_OK;
  }
  const int grid = (int)std::min<int64_t>(c->decode_grid, n);
  if (param_w) {
    // ~30 KB of launch parameters: built once per call site, copied by the launch
    static thread_local cbk::LearnedParamArgs pa;
    pa.d = a;
    std::memcpy(pa.alpha, param_w->data(), (size_t)h->nw * 4);
    std::memcpy(pa.beta, param_w->data() + h->nw, (size_t)h->nw * 4);
    CB_CUDA(c, cbk::launch_decode_learned_param(pa, grid, s));
  } else {
    CB_CUDA(c, cbk::launch_decode<float>(a, grid, s));
  }
  return CB_OK;
}

cbk::LearnedArgs nms_args(cb_nms* h, int64_t n) {
  cbk::LearnedArgs a{};
  a.code = h->code->dev;
  a.T = h->T;
  a.shared = h->shared;
  a.early_stop = 0;
  a.alpha = h->d_w;
  a.beta = h->d_w + h->nw;
  a.llr = h->d_llr;
  a.n_frames = n;
  a.c2v = h->d_c2v;
  a.post_out = h->d_post;
  a.g_alpha = h->d_g;
  a.g_beta = h->d_g + h->nw;
  a.loss_bits = h->info_only_loss ? h->code->host.k_info : h->code->host.n_full;
  return a;
}

// forward (+ backward) of n frames already in d_llr / d_cw; loss into d_loss
cb_status nms_fwd_bwd(cb_nms* h, int64_t n, bool backward, int multi, cudaStream_t s) {
  cb_code* c = h->code;
  cbk::LearnedArgs a = nms_args(h, n);
  a.cw_bits = h->d_cw;
  a.X = backward ? h->d_X : nullptr;
  a.loss = h->d_loss;
  a.P = h->d_P;
  a.multi_loss = multi;
  CB_CUDA(c, cudaMemsetAsync(h->d_loss, 0, sizeof(float), s));
  CB_CUDA(c, cbk::launch_learned(a, true, s));
  if (backward) {
    CB_CUDA(c, cudaMemsetAsync(h->d_g, 0, sizeof(float) * 2 * h->nw, s));
    CB_CUDA(c, cbk::launch_learned(a, false, s));
  }
  return CB_OK;
}

}  // namespace

extern "C" {

cb_status cb_nms_create(cb_code* c, int32_t iterations, int32_t shared, cb_nms** out) {
  if (!c || !out) return fail(c, CB_ERR_CONFIG, "NULL argument");
  *out = nullptr;
  if (c->precision != CB_F32) return fail(c, CB_ERR_CONFIG, "the learned min-sum runs on an f32 code object");
  if (iterations < 1 || iterations > 255) return fail(c, CB_ERR_CONFIG, "iterations in 1..255");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = ensure_device(c)) return st;
  cb_nms* h = new cb_nms();
  h->code = c;
  h->T = iterations;
  h->shared = shared ? 1 : 0;
  h->nw = (int64_t)iterations * c->dev.n_entries * (shared ? 1 : c->dev.z);
  std::vector<float> w(2 * h->nw, 0.f);
  for (int64_t i = 0; i < h->nw; i++) w[i] = (float)c->cfg.alpha;  // the plain min-sum
  cudaError_t e = cudaMalloc(&h->d_w, sizeof(float) * 2 * h->nw);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_g, sizeof(float) * 2 * h->nw);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_m, sizeof(float) * 2 * h->nw);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_v, sizeof(float) * 2 * h->nw);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_loss, 64);
  if (e == cudaSuccess) e = cudaMemcpy(h->d_w, w.data(), sizeof(float) * 2 * h->nw, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(h->d_m, 0, sizeof(float) * 2 * h->nw);
  if (e == cudaSuccess) e = cudaMemset(h->d_v, 0, sizeof(float) * 2 * h->nw);
  if (e != cudaSuccess) {
    cb_nms_destroy(h);
    return cuda_fail(c, e, "cb_nms_create");
  }
  *out = h;
  return CB_OK;
}

void cb_nms_destroy(cb_nms* h) {
  if (!h) return;
  cudaSetDevice(h->code->device);
  void* bufs[] = {h->d_w, h->d_g, h->d_m, h->d_v, h->d_X, h->d_P, h->d_c2v, h->d_post, h->d_llr, h->d_cw, h->d_info,
                  h->d_ebn0, h->d_loss, h->d_res};
  for (void* p : bufs)
    if (p) cudaFree(p);
  delete h;
}

cb_status cb_nms_info(const cb_nms* h, int64_t info[4]) {
  if (!h || !info) return fail(nullptr, CB_ERR_CONFIG, "NULL argument");
  info[0] = h->nw;
  info[1] = h->T;
  info[2] = h->shared;
  info[3] = h->step;
  return CB_OK;
}

cb_status cb_nms_get_weights(cb_nms* h, float* alpha, float* beta) {
  if (!h) return fail(nullptr, CB_ERR_CONFIG, "NULL argument");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (alpha) CB_CUDA(c, cudaMemcpy(alpha, h->d_w, sizeof(float) * h->nw, cudaMemcpyDeviceToHost));
  if (beta) CB_CUDA(c, cudaMemcpy(beta, h->d_w + h->nw, sizeof(float) * h->nw, cudaMemcpyDeviceToHost));
  return CB_OK;
}

cb_status cb_nms_set_weights(cb_nms* h, const float* alpha, const float* beta) {
  if (!h || !alpha || !beta) return fail(nullptr, CB_ERR_CONFIG, "NULL argument");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  h->h_w_valid = false;
  CB_CUDA(c, cudaMemcpy(h->d_w, alpha, sizeof(float) * h->nw, cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMemcpy(h->d_w + h->nw, beta, sizeof(float) * h->nw, cudaMemcpyHostToDevice));
  CB_CUDA(c, cudaMemset(h->d_m, 0, sizeof(float) * 2 * h->nw));
  CB_CUDA(c, cudaMemset(h->d_v, 0, sizeof(float) * 2 * h->nw));
  h->step = 0;
  return CB_OK;
}

cb_status cb_nms_forward(cb_nms* h, const float* llr, int64_t n, float* post) {
  if (!h || !llr || !post || n < 0) return fail(nullptr, CB_ERR_CONFIG, "NULL argument or negative count");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (n == 0) return CB_OK;
  if (cb_status st = nms_buffers(h, n, false)) return st;
  CB_CUDA(c, cudaMemcpyAsync(h->d_llr, llr, (size_t)n * c->host.e * 4, cudaMemcpyHostToDevice, c->stream));
  cbk::LearnedArgs a = nms_args(h, n);
  CB_CUDA(c, cbk::launch_learned(a, true, c->stream));
  CB_CUDA(c, cudaMemcpyAsync(post, h->d_post, (size_t)n * c->host.n_full * 4, cudaMemcpyDeviceToHost, c->stream));
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  return CB_OK;
}

cb_status cb_nms_set_loss_bits(cb_nms* h, int32_t info_only) {
  if (!h) return fail(nullptr, CB_ERR_CONFIG, "null learned decoder");
  h->info_only_loss = info_only ? 1 : 0;
  return CB_OK;
}

cb_status cb_nms_gradients(cb_nms* h, const float* llr, const uint8_t* cw, int64_t n, int32_t multi_loss,
                           float* g_alpha, float* g_beta, double* loss) {
  if (!h || !llr || !cw || n <= 0) return fail(nullptr, CB_ERR_CONFIG, "NULL argument or no frames");
  if (multi_loss < 0 || multi_loss > 2) return fail(nullptr, CB_ERR_CONFIG, "multi_loss is 0, 1 or 2");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (cb_status st = nms_buffers(h, n, true)) return st;
  const int wpc = (c->host.n_full + 31) / 32;
  h->h_words.assign((size_t)n * wpc, 0u);
  for (int64_t f = 0; f < n; f++)
    for (int v = 0; v < c->host.n_full; v++)
      if (cw[(size_t)f * c->host.n_full + v] & 1) h->h_words[(size_t)f * wpc + v / 32] |= 1u << (v % 32);
  CB_CUDA(c, cudaMemcpyAsync(h->d_llr, llr, (size_t)n * c->host.e * 4, cudaMemcpyHostToDevice, c->stream));
  CB_CUDA(c, cudaMemcpyAsync(h->d_cw, h->h_words.data(), h->h_words.size() * 4, cudaMemcpyHostToDevice, c->stream));
  if (cb_status st = nms_fwd_bwd(h, n, true, multi_loss, c->stream)) return st;
  float l = 0.f;
  CB_CUDA(c, cudaMemcpyAsync(&l, h->d_loss, 4, cudaMemcpyDeviceToHost, c->stream));
  if (g_alpha) CB_CUDA(c, cudaMemcpyAsync(g_alpha, h->d_g, sizeof(float) * h->nw, cudaMemcpyDeviceToHost, c->stream));
  if (g_beta)
    CB_CUDA(c, cudaMemcpyAsync(g_beta, h->d_g + h->nw, sizeof(float) * h->nw, cudaMemcpyDeviceToHost, c->stream));
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = (double)l / (double)n;
  return CB_OK;
}

cb_status cb_nms_train_step(cb_nms* h, int32_t m, uint64_t seed, uint64_t name_hash, int64_t batch, double lo,
                            double hi, double lr, int32_t multi_loss, double* loss) {
  if (!h || batch <= 0 || !(hi >= lo) || !(lr > 0) || multi_loss < 0 || multi_loss > 2)
    return fail(nullptr, CB_ERR_CONFIG, "bad training arguments");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  GenCache* g;
  if (cb_status st = gen_config(c, m, &g)) return st;
  if (cb_status st = nms_buffers(h, batch, true)) return st;
  // per-frame Eb/N0, uniform in [lo, hi], from a SplitMix64 sequence of (seed, step)
  std::vector<float> eb((size_t)batch);
  uint64_t st = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(h->step + 1));
  for (int64_t i = 0; i < batch; i++)
    eb[i] = (float)(lo + (hi - lo) * (double)(cbd::splitmix64(st) >> 11) * (1.0 / 9007199254740992.0));
  CB_CUDA(c, cudaMemcpyAsync(h->d_ebn0, eb.data(), (size_t)batch * 4, cudaMemcpyHostToDevice, c->stream));
  // training frames: condition 2^64 - 1 of the scenario, frame step * batch + i
  if (cb_status s2 = gen_device<float>(c, g, seed, name_hash, ~0ull, (uint64_t)h->step * batch, batch, lo, h->d_llr,
                                       h->d_info, c->stream, h->d_ebn0, h->d_cw))
    return s2;
  if (cb_status s3 = nms_fwd_bwd(h, batch, true, multi_loss, c->stream)) return s3;
  h->step++;
  h->h_w_valid = false;
  CB_CUDA(c, cbk::launch_adam(h->d_w, h->d_g, h->d_m, h->d_v, 2 * h->nw, (float)lr, h->step, c->stream));
  float l = 0.f;
  CB_CUDA(c, cudaMemcpyAsync(&l, h->d_loss, 4, cudaMemcpyDeviceToHost, c->stream));
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = (double)l / (double)batch;
  return CB_OK;
}

cb_status cb_nms_decode(cb_nms* h, const float* llr, int64_t n, float* post, int32_t* iterations) {
  if (!h || (!llr && n > 0) || n < 0) return fail(nullptr, CB_ERR_CONFIG, "NULL argument or negative count");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (n == 0) return CB_OK;
  std::vector<float> pw;
  bool in_params = false;
  if (cb_status st = nms_param_weights(h, pw, in_params)) return st;
  const int64_t chunk = 16384;
  for (int64_t done = 0; done < n; done += chunk) {
    const int64_t cnt = std::min(chunk, n - done);
    if (cb_status st = nms_buffers(h, cnt, false)) return st;
    CB_CUDA(c, grow(c->d_iters, c->iters_cap, (size_t)cnt * 4));
    CB_CUDA(c, cudaMemcpyAsync(h->d_llr, llr + (size_t)done * c->host.e, (size_t)cnt * c->host.e * 4,
                               cudaMemcpyHostToDevice, c->stream));
    if (cb_status st = nms_eval(h, h->d_llr, cnt, nullptr, nullptr, post ? h->d_post : nullptr, c->d_iters, c->stream,
                                in_params ? &pw : nullptr))
      return st;
    if (post)
      CB_CUDA(c, cudaMemcpyAsync(post + (size_t)done * c->host.n_full, h->d_post, (size_t)cnt * c->host.n_full * 4,
                                 cudaMemcpyDeviceToHost, c->stream));
    if (iterations)
      CB_CUDA(c, cudaMemcpyAsync(iterations + done, c->d_iters, (size_t)cnt * 4, cudaMemcpyDeviceToHost, c->stream));
  }
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  return CB_OK;
}

cb_status cb_nms_decode_device(cb_nms* h, const float* llr, int64_t n, float* post, int32_t* iterations,
                               void* stream) {
  if (!h || (!llr && n > 0) || n < 0) return fail(nullptr, CB_ERR_CONFIG, "NULL argument or negative count");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (n == 0) return CB_OK;
  std::vector<float> pw;
  bool in_params = false;
  if (cb_status st = nms_param_weights(h, pw, in_params)) return st;
  // the persistent decoder takes any number of frames; its per-CTA state is the code's
  return nms_eval(h, llr, n, nullptr, nullptr, post, iterations, (cudaStream_t)stream, in_params ? &pw : nullptr);
}

cb_status cb_nms_run_frames(cb_nms* h, int32_t m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first,
                            int64_t n, double ebn0_db, cb_frame_result* out) {
  if (!h || !out || n < 0) return fail(nullptr, CB_ERR_CONFIG, "NULL argument or negative count");
  cb_code* c = h->code;
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (n == 0) return CB_OK;
  GenCache* g;
  if (cb_status st = gen_config(c, m, &g)) return st;
  std::vector<float> pw;
  bool in_params = false;
  if (cb_status st = nms_param_weights(h, pw, in_params)) return st;
  const int64_t chunk = 16384;
  for (int64_t done = 0; done < n; done += chunk) {
    int64_t cnt = std::min(chunk, n - done);
    if (cb_status st = nms_buffers(h, cnt, false)) return st;
    if (cb_status st = gen_device<float>(c, g, seed, name_hash, cond, first + done, cnt, ebn0_db, h->d_llr, h->d_info,
                                         c->stream))
      return st;
    if (cb_status st = nms_eval(h, h->d_llr, cnt, h->d_info, h->d_res, nullptr, nullptr, c->stream,
                                in_params ? &pw : nullptr))
      return st;
    CB_CUDA(c, cudaMemcpyAsync(out + done, h->d_res, (size_t)cnt * sizeof(cb_frame_result), cudaMemcpyDeviceToHost,
                               c->stream));
  }
  CB_CUDA(c, cudaStreamSynchronize(c->stream));
  return CB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- decode without allocation
// Some callers cannot call cudaMalloc: a host framework that owns every byte of device
// memory through its own pool, or a real-time loop that forbids allocation once it has
// started (a cudaMalloc may block and synchronise the device).  For them
// cb_decode_device_noalloc keeps the decoder's scratch (its work counter and the
// check-node state of each resident CTA) in this file-scope array, which every GPU that
// loads the library holds until the process exits.
constexpr size_t kNoallocScratchBytes = (size_t)32 << 20;  // 32 MiB
constexpr size_t kNoallocCounterBytes = 256;
constexpr int kNoallocMaxDevices = 64;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoallocMaxDevices] = {};

// The device address of the scratch array on `device` (the current device).  In host
// code the array's name is only a host-side stand-in, so the address comes from
// cudaGetSymbolAddress, once per device.
cb_status noalloc_scratch(cb_code* c, int device, void** out) {
  if (device < 0 || device >= kNoallocMaxDevices) return fail(c, CB_ERR_CONFIG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[device] = p;
  }
  *out = g_noalloc_ptr[device];
  return CB_OK;
}

template <typename T>
cb_status decode_noalloc_impl(cb_code* c, void* scratch, const T* llr, int64_t n, uint32_t* bits, int32_t* iters,
                              cudaStream_t s) {
  // f32 layered min-sum runs the base graph's graph-specialised decoder (built into this
  // library: a run-time compiled module would allocate device memory when it loads)
  const bool nr = sizeof(T) == 4 && (c->cfg.rule == cbd::RULE_NMS || c->cfg.rule == cbd::RULE_OMS);
  const cbk::NrKernel k = nr ? cbk::nr_kernel(c->host, c->device, false, nullptr) : cbk::NrKernel{};
  const bool use_nr = nr && k.fn;
  const size_t slot = use_nr ? cbn::nr_state_bytes(c->host.rows_n * c->host.z)
                             : cbk::decode_state_bytes_per_slot(c->dev, c->precision);
  const int64_t fit = (int64_t)((kNoallocScratchBytes - kNoallocCounterBytes) / slot);
  if (fit < 1)
    return fail(c, CB_ERR_SHAPE,
                "the check-node state of one CTA (" + std::to_string(slot) + " bytes) exceeds the " +
                    std::to_string(kNoallocScratchBytes >> 20) + " MiB scratch of cb_decode_device_noalloc");
  if (c->noalloc_grid <= 0)  // the occupancy query once per code object
    c->noalloc_grid = use_nr ? cbk::nr_grid_size(k, c->host, c->device)
                             : cbk::decode_grid_size(c->dev, c->precision, c->device);
  const int occupancy = c->noalloc_grid;
  if (occupancy <= 0) return fail(c, CB_ERR_CUDA, "the decoder does not fit an SM (occupancy 0)");
  // the work counter must start at zero; the state slots need no clearing (the first
  // iteration of every codeword reads no state)
  CB_CUDA(c, cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), s));
  const int grid = (int)std::min<int64_t>(std::min<int64_t>(occupancy, fit), n);
  if (use_nr) {
    cbn::NrArgs a;
    cbk::fill_nr_args(c->host, a);
    a.max_iterations = c->cfg.max_iterations;
    a.rule = c->cfg.rule;
    a.alpha = (float)c->cfg.alpha;
    a.llr = reinterpret_cast<const float*>(llr);
    a.n_frames = n;
    a.bits_out = bits;
    a.iters_out = iters;
    a.work_counter = reinterpret_cast<unsigned long long*>(scratch);
    a.state = reinterpret_cast<unsigned char*>(scratch) + kNoallocCounterBytes;
    CB_CUDA(c, cbk::nr_launch(k, a, grid, s));
    return CB_OK;
  }
  cbk::DecodeArgs<T> a;
  a.code = c->dev;
  a.cfg = c->cfg;
  a.llr = llr;
  a.n_frames = n;
  a.bits_out = bits;
  a.app_out = nullptr;
  a.post_out = nullptr;
  a.iters_out = iters;
  a.ref_bits = nullptr;
  a.results = nullptr;
  a.work_counter = reinterpret_cast<int32_t*>(scratch);
  a.state = reinterpret_cast<T*>(reinterpret_cast<unsigned char*>(scratch) + kNoallocCounterBytes);
  a.status = nullptr;
  CB_CUDA(c, cbk::launch_decode<T>(a, grid, s));
  return CB_OK;
}
}  // namespace

extern "C" cb_status cb_decode_device_noalloc(cb_code* c, const void* llr, int64_t n, uint32_t* bits,
                                              int32_t* iters, void* stream) {
  if (!c || !llr || n < 0) return fail(c, CB_ERR_CONFIG, "NULL argument or negative count");
  if (!c->host.map_is_offset)
    return fail(c, CB_ERR_CONFIG,
                "cb_decode_device_noalloc needs the plain rate matching (rv 0, Qm 1, no filler bits sent)");
  if (c->generic)
    return fail(c, CB_ERR_CONFIG, "cb_decode_device_noalloc runs the layered min-sum only");
  std::lock_guard<std::mutex> lock(c->mu);
  CB_CUDA(c, cudaSetDevice(c->device));
  if (n == 0) return CB_OK;
  void* scratch = nullptr;
  if (cb_status st = noalloc_scratch(c, c->device, &scratch)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  if (c->precision == CB_F64)
    return decode_noalloc_impl<double>(c, scratch, (const double*)llr, n, bits, iters, s);
  return decode_noalloc_impl<float>(c, scratch, (const float*)llr, n, bits, iters, s);
}
