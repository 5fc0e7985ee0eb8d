// The link of a com-spec specification over a generic LDPC code, one trial per CTA:
//   fec_encode  k x blocks bits, one next_u64 each (crates/com-spec/src/blocks/coding/
//               fec.rs:60-78), the blocks' codewords one after the other (the from_rows
//               encoder of crates/com-fec/src/ldpc.rs:753-791), then the random
//               interleaver: stream bit t is coded bit perm[t] (interleaving.rs:63-67);
//   map         the padding bits to a multiple of log2 M, Gray QAM labels MSB first
//               (blocks/coding/map.rs:31-47);
//   awgn_ebn0   sigma^2 = P / (log2 M k / n 10^(Eb/N0 / 10)), P the mean power summed in
//               symbol order (blocks/channel.rs:141-156, blocks/frame.rs:250-259);
//   demap       exact or max-log LLRs (blocks/coding/map.rs:55-77);
//   fec_decode  the first n x blocks LLRs deinterleaved: decoder input perm[t] takes LLR t
//               (fec.rs:88-102); the blocks then go through the generic decoder.  With
//               an f32 decoder the f64 LLRs are rounded once to f32.
// The uncoded bit errors of the metric ber are counted here: the samples scaled by
// sqrt(energy(x) / energy(y)) and decided by the grid slicer of the square QAM
// (crates/com-spec/src/metrics.rs:254-284, :374-383, crates/com-math/src/nearest.rs),
// against the sent bits.  link_count_kernel then counts the coded_ber and bler errors
// (metrics.rs:334-351) from the decoder's posteriors.
//
// The draws of a trial are split over the CTA's threads as in the NR frame generator:
// each thread jumps to its chunk of the stream with a precomputed polynomial.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "qam_f64.cuh"

namespace cbk {
namespace {

constexpr int NT = kGenThreads;

// the grid slicer's cell of one coordinate: round((x - x0) / step), clamped
__device__ __forceinline__ int grid_cell(double x, double x0, double step, int side) {
  const double c = round(__ddiv_rn(__dsub_rn(x, x0), step));
  return (int)fmin(fmax(c, 0.0), (double)(side - 1));
}

// byte offset of the generator's tail buffers (8-byte aligned, after the labels and
// padding bits)
__host__ __device__ inline size_t link_gen_tail_offset(int m, int n_sym, int mbits) {
  return ((size_t)2 * m * 8 + (size_t)2 * n_sym * 8 + (size_t)n_sym + (size_t)mbits + 7) & ~(size_t)7;
}

__global__ void __launch_bounds__(NT) link_gen_kernel(const __grid_constant__ LinkGenArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t trial = blockIdx.x;
  if (trial >= a.n_trials) return;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int kb = a.k * a.blocks, nb = a.n * a.blocks;
  const int n_sym = (nb + a.n_pad) / a.mbits;
  const int wk = (a.k + 31) >> 5;  // packed words of one block's information bits
  // shared layout: points (2m doubles) | received samples (2 n_sym doubles) | labels
  // (n_sym) | padding bits | (8-byte aligned) packed information words (blocks x wk) |
  // payload bytes (kb) | coded bytes (nb); the received samples' energies (n_sym doubles)
  // take the place of the last three once the labels are formed
  double* pts = reinterpret_cast<double*>(smem);
  double* ys = pts + 2 * a.m;
  uint8_t* lab = reinterpret_cast<uint8_t*>(ys + 2 * n_sym);
  uint8_t* pad = lab + n_sym;
  uint32_t* uw = reinterpret_cast<uint32_t*>(smem + link_gen_tail_offset(a.m, n_sym, a.mbits));
  uint8_t* pay = reinterpret_cast<uint8_t*>(uw + a.blocks * wk);
  uint8_t* cw = pay + kb;
  double* yen = reinterpret_cast<double*>(uw);
  __shared__ double s_sigma2, s_ex, s_gain;
  __shared__ double s_en[256];  // the labels' energies
  __shared__ unsigned int s_err;
  const uint64_t t_idx = a.first_trial + (uint64_t)trial;

  for (int i = tid; i < 2 * a.m; i += NT) pts[i] = a.points[i];
  if (tid == 0) s_err = 0;
  // ---- the payload: chunk [tid * bpc, (tid + 1) * bpc) of the k x blocks bits
  {
    const int b0 = tid * a.bits_per_chunk, b1 = min(b0 + a.bits_per_chunk, kb);
    if (b0 < b1) {
      cbd::Xoshiro r = cbd::stream(a.seed, a.name_hash, a.cond, t_idx);
      cbd::xoshiro_jump(r, a.jumps + 4 * tid);
      for (int i = b0; i < b1; i++) pay[i] = (uint8_t)(cbd::xoshiro_next(r) >> 63);
    }
    if (tid == 0 && a.n_pad) {
      cbd::Xoshiro p = cbd::stream(a.seed, a.name_hash, a.cond, t_idx);
      cbd::xoshiro_jump(p, a.jumps + 4 * (2 * NT));
      for (int i = 0; i < a.n_pad; i++) pad[i] = (uint8_t)(cbd::xoshiro_next(p) >> 63);
    }
  }
  __syncthreads();
  // ---- the payload packed per block, for the encoder and for the coded error counts
  for (int task = warp; task < a.blocks * wk; task += NT / 32) {
    const int blk = task / wk, w = task - blk * wk, i = w * 32 + lane;
    const uint32_t word = __ballot_sync(0xffffffffu, i < a.k && pay[blk * a.k + i]);
    if (lane == 0) {
      uw[task] = word;
      a.payload_out[trial * (int64_t)(a.blocks * wk) + task] = word;
    }
  }
  __syncthreads();
  // ---- encode every block: information bits at their positions, parity bit t the
  // parity of (row t of the reduced H) AND (the packed information word)
  for (int task = tid; task < kb; task += NT) {
    const int blk = task / a.k, i = task - blk * a.k;
    cw[blk * a.n + a.info_pos[i]] = pay[task];
  }
  for (int task = tid; task < a.blocks * a.rank; task += NT) {
    const int blk = task / a.rank, t = task - blk * a.rank;
    uint32_t acc = 0;
    for (int w = 0; w < wk; w++) acc ^= __ldg(a.pmat + (size_t)w * a.rank + t) & uw[blk * wk + w];
    cw[blk * a.n + a.pivots[t]] = (uint8_t)(__popc(acc) & 1);
  }
  __syncthreads();
  // ---- labels: stream bit t is coded bit perm[t], then the padding bits
  for (int s = tid; s < n_sym; s += NT) {
    int idx = 0;
    for (int b = 0; b < a.mbits; b++) {
      const int t = s * a.mbits + b;
      const int bit = t < nb ? cw[a.perm ? a.perm[t] : t] : pad[t - nb];
      idx = (idx << 1) | bit;
    }
    lab[s] = (uint8_t)idx;
  }
  __syncthreads();
  // ---- measured power, summed in symbol order
  label_energies(pts, a.m, s_en, tid, NT);
  __syncthreads();
  if (tid == 0) {
    const double e = energy_sum(lab, n_sym, s_en);
    s_ex = e;
    s_sigma2 = __ddiv_rn(__ddiv_rn(__dadd_rn(0.0, e), (double)n_sym), a.b_ebn0);
  }
  __syncthreads();
  const double sigma2 = s_sigma2;
  // ---- noise and LLRs, symbol chunk [tid * spc, (tid + 1) * spc); the LLR of stream bit
  // t goes to decoder input perm[t]
  double* llr = a.llr_out ? a.llr_out + trial * (int64_t)nb : nullptr;
  float* llr32 = a.llr_out_f32 ? a.llr_out_f32 + trial * (int64_t)nb : nullptr;
  {
    const int s0 = tid * a.syms_per_chunk, s1 = min(s0 + a.syms_per_chunk, n_sym);
    if (s0 < s1) {
      cbd::Xoshiro r = cbd::stream(a.seed, a.name_hash, a.cond, t_idx);
      cbd::xoshiro_jump(r, a.jumps + 4 * (NT + tid));
      const double sd = __dsqrt_rn(sigma2);
      const double inv_s2 = __drcp_rn(sigma2);  // RN(1 / sigma2), for neg_div_by
      for (int s = s0; s < s1; s++) {
        double nre, nim;
        complex_gaussian_f64(r, nre, nim);
        const int li = lab[s];
        const double yre = __dadd_rn(pts[2 * li], __dmul_rn(nre, sd));
        const double yim = __dadd_rn(pts[2 * li + 1], __dmul_rn(nim, sd));
        ys[2 * s] = yre;
        ys[2 * s + 1] = yim;
        yen[s] = __dadd_rn(__dmul_rn(yre, yre), __dmul_rn(yim, yim));
        const int t0 = s * a.mbits;
        demap_f64(pts, a.m, a.mbits, a.log_m, a.exact != 0, yre, yim, sigma2, inv_s2, nb - t0, [&](int o, double v) {
          const int t = t0 + o;
          const int pos = a.perm ? a.perm[t] : t;
          if (llr32) llr32[pos] = (float)v;
          else llr[pos] = v;
        });
      }
    }
  }
  __syncthreads();
  // ---- metric ber: the gain sqrt(energy(x) / energy(y)), both summed in symbol order;
  // each |y|^2 was formed by the thread that drew y, so the sequential chain on one lane is
  // one FP64 addition per symbol
  if (tid == 0) {
    double e = 0.0;
#pragma unroll 8
    for (int s = 0; s < n_sym; s++) e = __dadd_rn(e, yen[s]);
    const double ey = __dadd_rn(0.0, e), ex = __dadd_rn(0.0, s_ex);
    s_gain = ey > 0.0 ? __dsqrt_rn(__ddiv_rn(ex, ey)) : 1.0;
  }
  __syncthreads();
  {
    const double g = s_gain;
    unsigned int errs = 0;
    for (int s = tid; s < n_sym; s += NT) {
      const double zr = __dmul_rn(ys[2 * s], g), zi = __dmul_rn(ys[2 * s + 1], g);
      const int col = grid_cell(zr, a.re0, a.step, a.side), row = grid_cell(zi, a.im0, a.step, a.side);
      errs += __popc((unsigned)(a.lookup[row * a.side + col] ^ lab[s]));
    }
    atomicAdd(&s_err, errs);
  }
  __syncthreads();
  if (tid == 0) a.raw_errors_out[trial] = s_err;
}

// one trial per CTA: the decided information bits of every block against the payload
__global__ void __launch_bounds__(NT) link_count_kernel(const __grid_constant__ LinkCountArgs a) {
  const int64_t trial = blockIdx.x;
  if (trial >= a.n_trials) return;
  const int wk = (a.k + 31) >> 5;
  __shared__ unsigned int s_coded, s_blocks;
  __shared__ unsigned int s_blk;
  if (threadIdx.x == 0) s_coded = s_blocks = 0;
  __syncthreads();
  for (int blk = 0; blk < a.blocks; blk++) {
    if (threadIdx.x == 0) s_blk = 0;
    __syncthreads();
    const int64_t base = (trial * a.blocks + blk) * (int64_t)a.n;
    const uint32_t* u = a.payload + trial * (int64_t)(a.blocks * wk) + blk * wk;
    unsigned int e = 0;
    for (int i = threadIdx.x; i < a.k; i += NT) {
      const int v = a.info_pos[i];
      const unsigned dec = (a.post_f32 ? a.post_f32[base + v] < 0.0f : a.post[base + v] < 0.0) ? 1u : 0u;
      e += dec ^ ((u[i >> 5] >> (i & 31)) & 1u);
    }
    if (e) atomicAdd(&s_blk, e);
    __syncthreads();
    if (threadIdx.x == 0) {
      s_coded += s_blk;
      s_blocks += s_blk > 0;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    unsigned int its = 0;
    for (int blk = 0; blk < a.blocks; blk++) its += (unsigned int)a.iters[trial * a.blocks + blk];
    LinkRecord r;
    r.raw_bit_errors = a.raw_errors[trial];
    r.coded_bit_errors = s_coded;
    r.block_errors = s_blocks;
    r.iterations = its;
    a.out[trial] = r;
  }
}

}  // namespace

size_t link_gen_smem_bytes(int m, int mbits, int k, int n, int blocks, int n_pad) {
  const int nb = n * blocks, n_sym = (nb + n_pad) / mbits, wk = (k + 31) / 32;
  const size_t tail = (size_t)blocks * wk * 4 + (size_t)k * blocks + nb;
  return link_gen_tail_offset(m, n_sym, mbits) + std::max(tail, (size_t)n_sym * 8) + 16;
}

cudaError_t launch_link_gen(const LinkGenArgs& a, cudaStream_t stream) {
  if (a.n_trials <= 0) return cudaSuccess;
  const size_t smem = link_gen_smem_bytes(a.m, a.mbits, a.k, a.n, a.blocks, a.n_pad);
  void* k = (void*)link_gen_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3((unsigned)a.n_trials), dim3(NT), args, smem, stream);
}

cudaError_t launch_link_count(const LinkCountArgs& a, cudaStream_t stream) {
  if (a.n_trials <= 0) return cudaSuccess;
  void* k = (void*)link_count_kernel;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3((unsigned)a.n_trials), dim3(NT), args, 0, stream);
}

}  // namespace cbk
