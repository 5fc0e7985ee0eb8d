// Mixed batches: codewords of different base graphs, lifting sizes, rates and
// modulations decoded by one persistent kernel, each with its own early exit.
//
// The batch's codewords are sorted by lifting size into classes.  The kernel walks the
// classes in order; for class k every CTA splits its 384 threads into `slots` groups of
// `slot_threads` threads (a multiple of 32, synchronised by their own named barrier).
// Each slot pulls one codeword after another from the class's atomic queue (work
// stealing), decodes it with the layered min-sum of decode.cu (the same row updates,
// the same syndrome test, so every result equals the single-code path bit for bit) and
// takes the next codeword as soon as its own syndrome test passes.  A thread of a slot
// owns `rows_per_thread` lifted rows of each layer: the autotuner picks that number per
// class (more rows per thread = more slots in flight for small Z).
#include <cuda_runtime.h>

#include "decode_common.cuh"
#include "kernels.h"

namespace cbk {
namespace {

__device__ __forceinline__ void slot_sync(int bar, int n) { asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(n) : "memory"); }

// OR of `bad` over the slot's threads (flag starts at 0 and is left at 0)
__device__ __forceinline__ bool slot_any(int bad, int* flag, int bar, int n, int lt) {
  if (bad) atomicOr(flag, 1);
  slot_sync(bar, n);
  const int f = *(volatile int*)flag;
  slot_sync(bar, n);
  if (lt == 0) *flag = 0;
  return f != 0;
}

// Whether some check fails, for one slot: stage 1 on the rows of the first two
// layers, stage 2 on packed hard decisions (the test of decode.cu's some_check_fails).
__device__ bool slot_check_fails(const float* post, uint32_t* hd, const uint32_t* ent, const uint16_t* lstart,
                                 int rows_n, int ncol, int z, int lt, int nt, int bar, int* flag) {
  int bad = 0;
  for (int r = lt; r < z && !bad; r += nt)
    for (int L = 0; L < 2 && !bad; L++) {
      uint32_t par = 0;
      for (int t = lstart[L]; t < lstart[L + 1]; t++) {
        const uint32_t en = ent[t];
        int cc = r + (int)(en & 0xffffu);
        cc -= (cc >= z) ? z : 0;
        par ^= (uint32_t)(post[(int)(en >> 16) * z + cc] < 0.f);
      }
      bad = (int)par;
    }
  if (slot_any(bad, flag, bar, nt, lt)) return true;
  build_hard_decisions(post, hd, ncol, z, lt, nt);
  slot_sync(bar, nt);
  const int wz = (z + 31) >> 5, ws = wz + 1;
  for (int task = lt; task < rows_n * wz && !bad; task += nt) {
    const int L = task / wz, g = task - L * wz;
    const int r0 = g * 32, nrows = min(32, z - r0);
    uint32_t par = 0;
    for (int t = lstart[L]; t < lstart[L + 1]; t++) {
      const uint32_t en = ent[t];
      const uint32_t* col = hd + (en >> 16) * ws;
      int o = r0 + (int)(en & 0xffffu);
      o -= (o >= z) ? z : 0;
      uint32_t win = window32(col, o);
      if (o + nrows > z) win |= window32(col, 0) << (z - o);
      par ^= win;
    }
    const uint32_t mask = nrows == 32 ? 0xffffffffu : ((1u << nrows) - 1u);
    bad = (par & mask) != 0u;
  }
  return slot_any(bad, flag, bar, nt, lt);
}

// Decode one codeword of the batch in a slot; RHO rows per thread.
template <int RHO>
__device__ void decode_item(const MixDecodeArgs& a, const MixItem& it, unsigned char* sm, int ncol_max,
                            const StateSlot<float>& st, int lt, int nt, int bar, int* flag, unsigned int* err) {
  const cbd::DevCode& c = a.codes[it.code];
  const int z = c.z;
  const int ws = (z + 31) / 32 + 1;
  float* post = reinterpret_cast<float*>(sm);
  uint32_t* hd = reinterpret_cast<uint32_t*>(post + 68 * z);
  uint32_t* s_ent = hd + ncol_max * ws;
  uint2* s_addr = reinterpret_cast<uint2*>(s_ent + cbh::kMaxEntries);
  uint16_t* s_lstart = reinterpret_cast<uint16_t*>(s_addr + cbh::kMaxEntries);
  uint8_t* s_order = reinterpret_cast<uint8_t*>(s_lstart + cbh::kMaxLayers + 1);
  uint8_t* s_end = s_order + cbh::kMaxLayers;
  const int ncol = c.n_full / z;
  for (int i = lt; i < c.n_entries; i += nt) {
    s_ent[i] = c.entry[i];
    s_addr[i] = c.eaddr[i];
  }
  for (int i = lt; i <= c.rows_n; i += nt) s_lstart[i] = c.layer_start[i];
  for (int i = lt; i < c.rows_n; i += nt) {
    s_order[i] = c.layer_order[i];
    s_end[i] = c.level_end[i];
  }
  const float* llr = a.llr + it.llr_offset;
  for (int v = lt; v < c.n_full; v += nt) post[v] = 0.f;
  slot_sync(bar, nt);
  // the batch's codes all use the plain rate matching 2Z + t
  for (int t = lt; t < c.e; t += nt) post[2 * z + t] = __fadd_rn(0.f, __ldcs(llr + t));
  slot_sync(bar, nt);
  for (int v = c.k_info + lt; v < c.k; v += nt) post[v] = cbd::kKnownBitLlr;
  slot_sync(bar, nt);
  int iters = 0;
  const int rows_n = c.rows_n;
  if (slot_check_fails(post, hd, s_ent, s_lstart, rows_n, ncol, z, lt, nt, bar, flag)) {
    iters = a.max_it;
    for (int iter = 1; iter <= a.max_it; iter++) {
      // the base rows by levels, as decode.cu runs them; each row's state is loaded where
      // it is used (loaded one row ahead: 17.56 against 17.40 ms per decode phase)
      for (int k = 0; k < rows_n; k++) {
        const int L = s_order[k];
        const int s0 = s_lstart[L], d = s_lstart[L + 1] - s0;
#pragma unroll
        for (int q = 0; q < RHO; q++) {
          const int r = lt + q * nt;
          if (r < z) {
            float a1 = 0.f, a2 = 0.f, n1, n2;
            uint32_t mt = 0u, nm;
            if (iter > 1) st.load(L * z + r, a1, a2, mt);
            if (a.rule == cbd::RULE_NMS)
              row_dispatch_lean<cbd::RULE_NMS>(d, post, EdgeAddrTable{s_addr + s0, r, 4 * r, 4 * z}, a1, a2, mt,
                                               a.alpha, n1, n2, nm);
            else
              row_dispatch_lean<cbd::RULE_OMS>(d, post, EdgeAddrTable{s_addr + s0, r, 4 * r, 4 * z}, a1, a2, mt,
                                               a.alpha, n1, n2, nm);
            st.store(L * z + r, n1, n2, nm);
          }
        }
        if (s_end[k]) slot_sync(bar, nt);
      }
      if (!slot_check_fails(post, hd, s_ent, s_lstart, rows_n, ncol, z, lt, nt, bar, flag)) {
        iters = iter;
        break;
      }
    }
  }
  // counts against the sent info bits: the sent words, one per thread, loaded before the
  // ballots so that their latency overlaps them, against the decisions staged in hd (free
  // after the syndrome test)
  const int wpf = (c.k_info + 31) >> 5, lane = lt & 31, warp = lt >> 5, nw = nt >> 5;
  const uint32_t* ref = a.info + it.info_offset;
  const uint32_t ref_w = lt < wpf ? ref[lt] : 0u;
  for (int b0 = warp * 32; b0 < c.k_info; b0 += nw * 32) {
    int v = b0 + lane;
    uint32_t word = __ballot_sync(0xffffffffu, v < c.k_info && post[v] < 0.f);
    if (lane == 0) hd[b0 >> 5] = word;
  }
  slot_sync(bar, nt);
  unsigned int be = lt < wpf ? __popc(hd[lt] ^ ref_w) : 0u;
  for (int w = lt + nt; w < wpf; w += nt) be += __popc(hd[w] ^ ref[w]);
  if (be) atomicAdd(err, be);
  slot_sync(bar, nt);
  if (lt == 0) {
    cbd::FrameResult r;
    r.bit_errors = *err;
    r.frame_error = *err > 0;
    r.iterations = (uint8_t)iters;
    r.reserved = 0;
    a.results[it.index] = r;
    *err = 0;
  }
}

__global__ void __launch_bounds__(384, 2) mix_decode_kernel(const __grid_constant__ MixDecodeArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ long long s_item[16];
  __shared__ int s_flag[16];
  __shared__ unsigned int s_err[16];
  const int tid = threadIdx.x;
  if (tid < 16) {
    s_flag[tid] = 0;
    s_err[tid] = 0;
  }
  __syncthreads();
  for (int k = 0; k < a.n_classes; k++) {
    const MixClass cls = a.classes[k];
    const int slot = tid / cls.slot_threads;
    if (slot < cls.slots) {
      const int lt = tid - slot * cls.slot_threads, nt = cls.slot_threads, bar = slot + 1;
      unsigned char* sm = smem + (size_t)slot * cls.smem_per_slot;
      const StateSlot<float> st(a.state + (size_t)blockIdx.x * a.state_per_cta + (size_t)slot * cls.state_per_slot,
                                cbh::kMaxLayers * cls.z);
      for (;;) {
        if (lt == 0) s_item[slot] = (long long)atomicAdd(&a.counters[k], 1ull);
        slot_sync(bar, nt);
        const long long i = s_item[slot];
        slot_sync(bar, nt);
        if (i >= cls.count) break;
        const MixItem it = a.items[cls.first + i];
        if (cls.rows_per_thread == 1) decode_item<1>(a, it, sm, cls.max_ncol, st, lt, nt, bar, &s_flag[slot], &s_err[slot]);
        else decode_item<2>(a, it, sm, cls.max_ncol, st, lt, nt, bar, &s_flag[slot], &s_err[slot]);
      }
    }
    __syncthreads();
  }
}

}  // namespace

size_t mix_slot_smem_bytes(int z) {
  const int ws = (z + 31) / 32 + 1;
  size_t b = (size_t)68 * z * 4 + (size_t)68 * ws * 4 + (size_t)cbh::kMaxEntries * (4 + 8) +
             (size_t)(cbh::kMaxLayers + 1) * 2 + (size_t)cbh::kMaxLayers * 2;
  return (b + 15) & ~(size_t)15;
}

int mix_decode_grid(size_t smem, int device) {
  void* k = (void*)mix_decode_kernel;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  int per_sm = 0, sms = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 384, smem);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return per_sm * sms;
}

cudaError_t launch_mix_decode(const MixDecodeArgs& a, int grid, size_t smem, cudaStream_t s) {
  void* k = (void*)mix_decode_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3(grid), dim3(384), args, smem, s);
}

}  // namespace cbk
