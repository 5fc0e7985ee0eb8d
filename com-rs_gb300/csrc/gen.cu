// One BICM-LDPC frame per CTA: info bits, NR encoding, rate matching, Gray QAM
// mapping, measured-power AWGN and max-log LLRs, regenerated on the device from the
// frame's stream(seed, name, condition, frame) exactly as the reference draws them.
//
// Draw order of a frame (the spec chain of com-spec): K' bits, one next_u64 each
// (source::bits, crates/com-mapping/src/source.rs:30-32, Rng::bit rng.rs:146-148); the
// padding bits of map (blocks/coding/map.rs:36-38); then two uniforms per symbol for
// its complex Gaussian (rng.rs:161-167).  The draws are split over the CTA's threads in
// contiguous chunks (the bits over the first warp, the noise over the other three); each
// thread reaches its chunk's start with a xoshiro256**
// jump-ahead polynomial (the state after n steps is P_n(T) s, P_n = x^n mod the
// characteristic polynomial of the transition T), so every value equals the
// sequential draw.
//
// Encoding: LdpcCode::encode_block with Encoder::Core (crates/com-fec/src/ldpc.rs:
// 774-786): the syndromes of the four core base rows, the core parity from the
// block-circulant inverse of the core (computed on the host), then every extension
// parity bit from its own row.  Rate matching is BitSelection::select
// (crates/com-fec/src/puncture.rs:144-148) over the positions of nr/ldpc.rs:135-160.
//
// Channel and demapper:
//   sigma^2 = P_meas / (log2 M * R * 10^(Eb/N0 / 10))  (crates/com-channel/src/awgn.rs:
//   139-141, com-spec blocks/channel.rs:141-156, P_meas = the mean power of the frame's
//   symbols summed in symbol order, blocks/frame.rs:256-259);
//   y = x + sqrt(sigma^2) * CN(0, 1)  (awgn.rs:94-99);
//   L_b = max_{i: b=0} metric_i - max_{i: b=1} metric_i, metric_i = -|y - x_i|^2 /
//   sigma^2 - ln M  (crates/com-mapping/src/demapper.rs:82-146, :270-297), or with the
//   exact demapper the log-sum-exp of each half of the labels.
// f64 frames compute all of it in f64 with the correctly-rounded log/sin/cos of
// crmath_fast.cuh (crmath.cuh's values): bit-identical to the reference's draws up to
// the platform libm's last bit.  f32 frames draw the same bits and the same uniforms, take the Gaussian in f32
// and the max-log LLRs per I/Q dimension (the Gray square QAM labels split into an
// imaginary-part and a real-part Gray code, so the max-log LLRs separate exactly).
#include <cuda_runtime.h>

#include "crmath.cuh"
#include "decode_common.cuh"
#include "kernels.h"
#include "qam_f64.cuh"

namespace cbk {
namespace {

constexpr int NT = kGenThreads;

__device__ __forceinline__ int gray(int i) { return i ^ (i >> 1); }

// f32 noise and max-log (or exact) demapping of the symbols [s0, s1) of a frame, H bits
// per dimension.  The square QAM's label is gray(row) * side + gray(col): the first H
// bits come from the imaginary part, the last H from the real part, so each bit's LLR is
// a one-dimensional max-log (exact: log-sum-exp) over the side levels of its dimension;
// the level metrics of both dimensions are computed once per symbol.
template <int H, typename T>
__device__ __forceinline__ void noise_demap_f32(const cbd::DevCode& c, const GenFrame<T>& a, cbd::Xoshiro& r,
                                                const uint8_t* lab, const double* pts, int s0, int s1, float sd,
                                                float inv_s2, T* out) {
  constexpr int SIDE = 1 << H, MB = 2 * H;
  // the PAM levels of each dimension, ascending: real level q is point gray(q),
  // imaginary level q is point gray(side - 1 - q) * side
  float lev_re[SIDE], lev_im[SIDE];
#pragma unroll
  for (int q = 0; q < SIDE; q++) {
    lev_re[q] = (float)pts[2 * gray(q)];
    lev_im[q] = (float)pts[2 * (gray(SIDE - 1 - q) * SIDE) + 1];
  }
  for (int s = s0; s < s1; s++) {
    uint64_t x1 = cbd::xoshiro_next(r) >> 11, x2 = cbd::xoshiro_next(r) >> 11;
    // 1 - u1 = (2^53 - x1) 2^-53 exactly, then rounded once to f32
    float one_minus_u1 = __ull2float_rn((1ull << 53) - x1) * 1.1102230246251565e-16f;
    float u2 = __ull2float_rn(x2 >> 29) * 5.9604644775390625e-08f;  // top 24 bits of u2
    float rad = sqrtf(-2.0f * logf(one_minus_u1)) * 0.70710678f;
    float sn, cs;
    sincospif(2.0f * u2, &sn, &cs);
    int li = lab[s];
    float yre = (float)pts[2 * li] + rad * cs * sd;
    float yim = (float)pts[2 * li + 1] + rad * sn * sd;
    float met_re[SIDE], met_im[SIDE];
#pragma unroll
    for (int q = 0; q < SIDE; q++) {
      float dr = yre - lev_re[q], di = yim - lev_im[q];
      met_re[q] = -(dr * dr) * inv_s2;
      met_im[q] = -(di * di) * inv_s2;
    }
#pragma unroll
    for (int o = 0; o < MB; o++) {
      const int t = s * MB + o;
      if (t >= c.e) break;
      const bool upper = o < H;
      const int bitpos = upper ? (H - 1 - o) : (MB - 1 - o);
      float m0 = -INFINITY, m1 = -INFINITY;
#pragma unroll
      for (int q = 0; q < SIDE; q++) {
        const int lbl = upper ? gray(SIDE - 1 - q) : gray(q);
        const float met = upper ? met_im[q] : met_re[q];
        if ((lbl >> bitpos) & 1) m1 = fmaxf(m1, met);
        else m0 = fmaxf(m0, met);
      }
      if (a.exact) {
        // exact log-sum-exp per dimension: the other dimension's sum is common to both
        // halves of the labels and cancels
        float e0 = 0.f, e1 = 0.f;
#pragma unroll
        for (int q = 0; q < SIDE; q++) {
          const int lbl = upper ? gray(SIDE - 1 - q) : gray(q);
          const float met = upper ? met_im[q] : met_re[q];
          if ((lbl >> bitpos) & 1) e1 += expf(met - m1);
          else e0 += expf(met - m0);
        }
        out[t] = (T)(m0 + logf(e0) - m1 - logf(e1));
      } else {
        out[t] = (T)(m0 - m1);
      }
    }
  }
}

// One frame by one CTA of NT threads: code `c`, frame parameters `a`.
template <typename T>
__device__ __forceinline__ void gen_one(const cbd::DevCode& c, const GenFrame<T>& a, unsigned char* smem) {
  const int z = c.z, tid = threadIdx.x;
  const int n_sym = (c.e + a.n_pad) / a.mbits;
  const int wz = (z + 31) >> 5, ws = wz + 1, ncol = c.n_full / z;
  // shared layout: points (2M doubles) | packed codeword columns (ncol x ws words: Z bits
  // each, then a zero word) | packed core syndromes (4 x ws) | codeword bytes (n_full) |
  // labels
  double* pts = reinterpret_cast<double*>(smem);
  uint32_t* cwp = reinterpret_cast<uint32_t*>(pts + 2 * a.m);
  uint32_t* synp = cwp + ncol * ws;
  uint8_t* cw = reinterpret_cast<uint8_t*>(synp + 4 * ws);
  uint8_t* lab = cw + c.n_full;
  uint8_t* pad = lab + n_sym;  // padding bits (< mbits)
  __shared__ double s_sigma2;
  // f32 frames: the label histogram; f64 frames: the labels' energies
  __shared__ double s_tab[256];
  unsigned int* s_hist = reinterpret_cast<unsigned int*>(s_tab);
  const uint64_t fidx = a.frame_index;

  for (int i = tid; i < 2 * a.m; i += NT) pts[i] = a.points[i];
  // ---- info bits by the first warp, thread t the chunk [t bpc, (t + 1) bpc); the thread
  // whose chunk ends at K' draws the padding bits next, as they follow the info bits.
  // Meanwhile each thread of the other warps jumps to the start of its noise chunk
  // (symbols [(t - BT) spc, ...)), which it draws after the encoding.
  constexpr int BT = kGenBitsThreads;
  cbd::Xoshiro rn = cbd::stream(a.seed, a.name_hash, a.cond, fidx);
  if (tid < BT) {
    const int b0 = tid * a.bits_per_chunk, b1 = min(b0 + a.bits_per_chunk, c.k_info);
    if (b0 < b1) {
      cbd::xoshiro_jump(rn, a.jumps + 4 * tid);
      for (int i = b0; i < b1; i++) cw[i] = (uint8_t)(cbd::xoshiro_next(rn) >> 63);
      if (b1 == c.k_info)
        for (int i = 0; i < a.n_pad; i++) pad[i] = (uint8_t)(cbd::xoshiro_next(rn) >> 63);
    }
  } else if ((tid - BT) * a.syms_per_chunk < n_sym) {
    cbd::xoshiro_jump(rn, a.jumps + 4 * tid);
  }
  for (int i = c.k_info + tid; i < c.n_full; i += NT) cw[i] = 0;
  __syncthreads();
  // packed info bits for the error counts
  {
    const int lane = tid & 31, warp = tid >> 5;
    for (int b0 = warp * 32; b0 < c.k_info; b0 += (NT / 32) * 32) {
      int v = b0 + lane;
      uint32_t word = __ballot_sync(0xffffffffu, v < c.k_info && cw[v]);
      if (lane == 0) a.info_out[b0 >> 5] = word;
    }
  }
  // ---- encoder on packed columns, 32 lifted rows per word: the rows r0 .. r0 + 31 of an
  // entry (j, s) read the Z-bit column j from bit (r0 + s) mod Z on (window32, wrapping
  // at Z); the XOR over a row's entries is then the parity of 32 rows at once
  const int lane = tid & 31, warp = tid >> 5;
  for (int task = warp; task < c.cols_k * wz; task += NT / 32) {  // pack the systematic columns
    const int j = task / wz, w = task - j * wz, b = w * 32 + lane;
    const uint32_t word = __ballot_sync(0xffffffffu, b < z && cw[j * z + b]);
    if (lane == 0) {
      cwp[j * ws + w] = word;
      if (w == wz - 1) cwp[j * ws + wz] = 0u;
    }
  }
  __syncthreads();
  // the 32-row window of a packed Z-bit column from row r0 with shift s (rows past Z read 0)
  auto window = [&](const uint32_t* col, int r0, int shift) -> uint32_t {
    int o = r0 + shift;
    o -= (o >= z) ? z : 0;
    uint32_t win = window32(col, o);
    const int nrows = min(32, z - r0);
    if (o + nrows > z) win |= window32(col, 0) << (z - o);
    return nrows == 32 ? win : (win & ((1u << nrows) - 1u));
  };
  // core syndromes over the systematic columns
  for (int task = tid; task < 4 * wz; task += NT) {
    const int L = task / wz, g = task - L * wz;
    uint32_t acc = 0;
    for (int t = c.layer_start[L]; t < c.layer_start[L + 1]; t++) {
      const uint32_t en = c.entry[t];
      const int j = (int)(en >> 16);
      if (j < c.cols_k) acc ^= window(cwp + j * ws, g * 32, (int)(en & 0xffffu));
    }
    synp[L * ws + g] = acc;
    if (g == wz - 1) synp[L * ws + wz] = 0u;
  }
  __syncthreads();
  // core parity: block-circulant inverse of the core
  for (int task = tid; task < 4 * wz; task += NT) {
    const int blk = task / wz, g = task - blk * wz;
    uint32_t acc = 0;
    for (int t = 0; t < c.n_core_terms; t++) {
      const uint32_t ct = c.core_term[t];
      if ((int)(ct >> 20) != blk) continue;
      acc ^= window(synp + (int)((ct >> 16) & 15u) * ws, g * 32, (int)(ct & 0xffffu));
    }
    uint32_t* col = cwp + (c.cols_k + blk) * ws;
    col[g] = acc;
    if (g == wz - 1) col[wz] = 0u;
  }
  __syncthreads();
  // extension parity: row L >= 4 closes on its own column cols_k + L (shift 0) and reads
  // only systematic and core parity columns
  for (int task = 4 * wz + tid; task < c.rows_n * wz; task += NT) {
    const int L = task / wz, g = task - L * wz;
    uint32_t acc = 0;
    for (int t = c.layer_start[L]; t < c.layer_start[L + 1]; t++) {
      const uint32_t en = c.entry[t];
      const int j = (int)(en >> 16);
      if (j != c.cols_k + L) acc ^= window(cwp + j * ws, g * 32, (int)(en & 0xffffu));
    }
    uint32_t* col = cwp + (c.cols_k + L) * ws;
    col[g] = acc;
    if (g == wz - 1) col[wz] = 0u;
  }
  __syncthreads();
  // the parity bits back to bytes, for the labels
  for (int v = c.k + tid; v < c.n_full; v += NT) {
    const int j = v / z, b = v - j * z;
    cw[v] = (uint8_t)((cwp[j * ws + (b >> 5)] >> (b & 31)) & 1u);
  }
  __syncthreads();
  if (a.cw_out) {  // the full codeword, packed
    const int lane = tid & 31, warp = tid >> 5;
    for (int b0 = warp * 32; b0 < c.n_full; b0 += (NT / 32) * 32) {
      int v = b0 + lane;
      uint32_t word = __ballot_sync(0xffffffffu, v < c.n_full && cw[v]);
      if (lane == 0) a.cw_out[b0 >> 5] = word;
    }
  }
  // ---- labels, MSB first (bits_to_index, com-math bits.rs:68-70)
  for (int s = tid; s < n_sym; s += NT) {
    int idx = 0;
    for (int b = 0; b < a.mbits; b++) {
      int t = s * a.mbits + b;
      int bit = t < c.e ? cw[c.map_is_offset ? 2 * z + t : c.map[t]] : pad[t - c.e];
      idx = (idx << 1) | bit;
    }
    lab[s] = (uint8_t)idx;
  }
  __syncthreads();
  // ---- measured power (com-math lib.rs:146-148)
  if (sizeof(T) == 8) {
    // f64 frames: summed in symbol order, as the reference
    label_energies(pts, a.m, s_tab, tid, NT);
    __syncthreads();
    if (tid == 0) {
      const double e = energy_sum(lab, n_sym, s_tab);
      double p = __ddiv_rn(__dadd_rn(0.0, e), (double)n_sym);
      s_sigma2 = __ddiv_rn(p, a.b_ebn0);
    }
  } else {
    // f32 frames: the label histogram, then the sum over the M labels
    for (int i = tid; i < a.m; i += NT) s_hist[i] = 0;
    __syncthreads();
    for (int s = tid; s < n_sym; s += NT) atomicAdd(&s_hist[lab[s]], 1u);
    __syncthreads();
    if (tid == 0) {
      float e = 0.0f;
      for (int i = 0; i < a.m; i++) {
        float re = (float)pts[2 * i], im = (float)pts[2 * i + 1];
        e += (float)s_hist[i] * (re * re + im * im);
      }
      s_sigma2 = (double)(e / (float)n_sym / (float)a.b_ebn0);
    }
  }
  __syncthreads();
  const double sigma2 = s_sigma2;
  // ---- noise and demapping by the threads past the first warp, symbol chunk
  // [(tid - BT) spc, (tid - BT + 1) spc), from the state they jumped to
  if (tid < BT) return;
  int s0 = (tid - BT) * a.syms_per_chunk, s1 = min(s0 + a.syms_per_chunk, n_sym);
  if (s0 >= s1) return;
  cbd::Xoshiro& r = rn;
  T* out = a.llr_out;
  if (sizeof(T) == 8) {
    const double sd = __dsqrt_rn(sigma2);
    const double inv_s2 = __drcp_rn(sigma2);  // RN(1 / sigma2), for neg_div_by
    for (int s = s0; s < s1; s++) {
      double nre, nim;
      complex_gaussian_f64(r, nre, nim);
      const int li = lab[s];
      const double yre = __dadd_rn(pts[2 * li], __dmul_rn(nre, sd));
      const double yim = __dadd_rn(pts[2 * li + 1], __dmul_rn(nim, sd));
      const int t0 = s * a.mbits;
      demap_f64(pts, a.m, a.mbits, a.log_m, a.exact != 0, yre, yim, sigma2, inv_s2, c.e - t0,
                [&](int o, double v) { out[t0 + o] = (T)v; });
    }
  } else {
    const float sd = (float)__dsqrt_rn(sigma2);
    const float inv_s2 = (float)(1.0 / sigma2);
    switch (a.mbits) {
      case 2: noise_demap_f32<1>(c, a, r, lab, pts, s0, s1, sd, inv_s2, out); break;
      case 4: noise_demap_f32<2>(c, a, r, lab, pts, s0, s1, sd, inv_s2, out); break;
      case 6: noise_demap_f32<3>(c, a, r, lab, pts, s0, s1, sd, inv_s2, out); break;
      default: noise_demap_f32<4>(c, a, r, lab, pts, s0, s1, sd, inv_s2, out); break;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(NT) gen_kernel(const __grid_constant__ GenArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const long long frame = (long long)blockIdx.x;
  if (frame >= a.n_frames) return;
  const cbd::DevCode& c = a.code;
  GenFrame<T> g;
  g.m = a.m;
  g.mbits = a.mbits;
  g.n_pad = a.n_pad;
  g.bits_per_chunk = a.bits_per_chunk;
  g.syms_per_chunk = a.syms_per_chunk;
  g.points = a.points;
  g.log_m = a.log_m;
  if (!a.ebn0_frames) g.b_ebn0 = a.b_ebn0;
  else if (sizeof(T) == 8) g.b_ebn0 = a.b_bits * pow(10.0, (double)a.ebn0_frames[frame] / 10.0);
  else g.b_ebn0 = (double)((float)a.b_bits * exp10f(a.ebn0_frames[frame] / 10.0f));
  g.jumps = a.jumps;
  g.seed = a.seed;
  g.name_hash = a.name_hash;
  g.cond = a.cond;
  g.frame_index = a.first_frame + (uint64_t)frame;
  g.llr_out = a.llr_out + (size_t)frame * c.e;
  g.info_out = a.info_out + (size_t)frame * ((c.k_info + 31) >> 5);
  g.cw_out = a.cw_out ? a.cw_out + (size_t)frame * ((c.n_full + 31) >> 5) : nullptr;
  g.exact = a.exact;
  gen_one<T>(c, g, smem);
}

// The frames of a mixed batch: CTA i generates item i of the batch (its own code,
// modulation, Eb/N0 and stream position) into the batch's LLR and info buffers.
__global__ void __launch_bounds__(NT) gen_mix_kernel(const __grid_constant__ GenMixArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const long long i = (long long)blockIdx.x;
  if (i >= a.n_items) return;
  const MixItem it = a.items[i];
  const GenConfig gc = a.configs[it.config];
  const cbd::DevCode& c = a.codes[it.code];
  GenFrame<float> g;
  g.m = gc.m;
  g.mbits = gc.mbits;
  g.n_pad = gc.n_pad;
  g.bits_per_chunk = gc.bits_per_chunk;
  g.syms_per_chunk = gc.syms_per_chunk;
  g.points = gc.points;
  g.log_m = gc.log_m;
  g.b_ebn0 = it.b_ebn0;
  g.jumps = gc.jumps;
  g.seed = a.seed;
  g.name_hash = a.name_hash;
  g.cond = it.cond;
  g.frame_index = it.frame + (a.epoch ? *a.epoch * a.epoch_stride : 0ull);
  g.llr_out = a.llr + it.llr_offset;
  g.info_out = a.info + it.info_offset;
  g.cw_out = nullptr;
  g.exact = 0;
  gen_one<float>(c, g, smem);
}
}  // namespace

size_t gen_smem_bytes(const cbd::DevCode& c, int m, int mbits, int n_pad) {
  int n_sym = (c.e + n_pad) / mbits;
  const int ws = (c.z + 31) / 32 + 1, ncol = c.n_full / c.z;
  return (size_t)2 * m * sizeof(double) + (size_t)(ncol + 4) * ws * 4 + c.n_full + n_sym + 16;
}

template <typename T>
cudaError_t launch_gen(const GenArgs<T>& a, cudaStream_t stream) {
  size_t smem = gen_smem_bytes(a.code, a.m, a.mbits, a.n_pad);
  void* k = (void*)gen_kernel<T>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3((unsigned)a.n_frames), dim3(NT), args, smem, stream);
}

template cudaError_t launch_gen<double>(const GenArgs<double>&, cudaStream_t);
template cudaError_t launch_gen<float>(const GenArgs<float>&, cudaStream_t);

cudaError_t launch_gen_mix(const GenMixArgs& a, size_t smem, cudaStream_t stream) {
  void* k = (void*)gen_mix_kernel;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  void* args[] = {(void*)&a};
  return cudaLaunchKernel(k, dim3((unsigned)a.n_items), dim3(NT), args, smem, stream);
}

}  // namespace cbk
