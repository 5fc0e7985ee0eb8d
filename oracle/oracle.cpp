// ORACLE — test infrastructure, not product code.
//
// A frozen CPU restatement of the com-rs BICM-LDPC Monte Carlo trial, used only by the
// tests, by `__graft_entry__.smoke()` as the checker, and by `bench.py` as the timed CPU
// baseline (`cpu_baseline` and `--impl reference`).  Nothing in the product links it.
//
// Every function names the reference file:line it restates (paths inside the com-rs
// project).  Compile with -O2 -ffp-contract=off: the reference never fuses a multiply
// into an add (Cargo.toml:109), and neither does this file.
//
// Pinning (checked by tests/test_oracle.py):
//   * RNG known answers of crates/com-core/src/rng.rs:300-305;
//   * the 28 NR-LDPC encodings of the reference's Sionna fixture
//     (tests/oracle/sionna_vectors.npz, copied to tests/golden/ by make_golden.py),
//     and decode(4 - 8c) == u for K' <= 1024 (tests/test_sionna_vectors.py:104-115);
//   * the structure assertions of crates/com-fec/src/nr/ldpc.rs:249-282;
//   * the AFF3CT layered-NMS FER curve (validation/aff3ct/*.json), statistically.
//
// Noise transcendental functions: the reference calls the platform libm (Rust std on
// Linux = glibc) for ln/sin/cos (crates/com-core/src/rng.rs:161-167).  This file offers
// two modes: NOISE_LIBM (glibc, the reference on this host) and NOISE_CR (the
// correctly-rounded value, computed in binary128 and rounded once).  The GPU kernels
// are bit-exact to NOISE_CR; the tests measure how often NOISE_LIBM differs.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#if defined(__x86_64__)
#include <quadmath.h>
typedef __float128 qreal_t;
static inline qreal_t q_log(qreal_t x) { return logq(x); }
static inline qreal_t q_sin(qreal_t x) { return sinq(x); }
static inline qreal_t q_cos(qreal_t x) { return cosq(x); }
#else
// aarch64 Linux: long double is IEEE binary128
typedef long double qreal_t;
static inline qreal_t q_log(qreal_t x) { return logl(x); }
static inline qreal_t q_sin(qreal_t x) { return sinl(x); }
static inline qreal_t q_cos(qreal_t x) { return cosl(x); }
#endif

#include "../com-rs_gb300/csrc/nr_base_graphs.inc"

namespace oracle {

// ------------------------------------------------------------------ rng.rs
// crates/com-core/src/rng.rs:49-55
static inline uint64_t splitmix64(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// rng.rs:58-65
static uint64_t fnv1a64(const uint8_t* b, size_t n) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (size_t i = 0; i < n; i++) { h ^= b[i]; h *= 0x00000100000001B3ull; }
  return h;
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

enum NoiseMode { NOISE_LIBM = 0, NOISE_CR = 1 };

struct Rng {
  uint64_t s[4];
  // rng.rs:75-79
  explicit Rng(uint64_t seed) {
    uint64_t st = seed;
    for (int i = 0; i < 4; i++) s[i] = splitmix64(st);
  }
  // rng.rs:100-111
  uint64_t next_u64() {
    uint64_t result = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return result;
  }
  // rng.rs:115-117
  double uniform() { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
  // rng.rs:146-148
  uint8_t bit() { return (uint8_t)(next_u64() >> 63); }
  // rng.rs:125-128
  uint64_t below(uint64_t n) {
    uint64_t v = (uint64_t)(uniform() * (double)n);
    return std::min(v, n - 1);
  }
  // rng.rs:218-222
  void shuffle(std::vector<int32_t>& v) {
    for (size_t i = v.size(); i-- > 1;) std::swap(v[i], v[below(i + 1)]);
  }
  // rng.rs:152-157
  double gaussian() {
    double u1 = uniform(), u2 = uniform();
    double r = std::sqrt(-2.0 * std::log(1.0 - u1));
    return r * std::cos(2.0 * M_PI * u2);
  }
  // rng.rs:161-167 (FRAC_1_SQRT_2 = 0.7071067811865476)
  void complex_gaussian(double& re, double& im, NoiseMode mode) {
    double u1 = uniform(), u2 = uniform();
    double a = 1.0 - u1;
    double th = 2.0 * M_PI * u2;
    double l, sn, cs;
    if (mode == NOISE_LIBM) {
      l = std::log(a);
      sn = std::sin(th);
      cs = std::cos(th);
    } else {
      l = (double)q_log((qreal_t)a);
      sn = (double)q_sin((qreal_t)th);
      cs = (double)q_cos((qreal_t)th);
    }
    double r = std::sqrt(-2.0 * l) * 0.70710678118654752440;
    re = r * cs;
    im = r * sn;
  }
};

// rng.rs:270-278
static Rng stream(uint64_t base_seed, uint64_t name_hash, uint64_t condition, uint64_t trial) {
  uint64_t st = base_seed ^ name_hash;
  uint64_t a = splitmix64(st);
  st = a ^ condition;
  uint64_t b = splitmix64(st);
  st = b ^ trial;
  uint64_t c = splitmix64(st);
  return Rng(c);
}

// units.rs:38-40
static double db2lin(double x) { return std::pow(10.0, x / 10.0); }

// ------------------------------------------------------------------ LDPC (ldpc.rs)
enum Rule { RULE_SUM_PRODUCT = 0, RULE_NMS = 1, RULE_OMS = 2 };
static const double KNOWN_BIT_LLR = 30.0;           // signal.rs:37
static const double TANH_BOUND = 0.999999999999;    // ldpc.rs:93

struct Code {
  // generic LdpcCode part (ldpc.rs:183-196)
  int n = 0;                          // n_full
  std::vector<std::vector<int>> rows; // variables of every check
  std::vector<int> start;             // edge offsets
  int k = 0;                          // systematic bits (K)
  int core = 0;                       // core checks (Encoder::Core), 0 for Sums
  std::vector<std::vector<int>> solve;
  // generic (alist) codes: Encoder::Sums
  std::vector<int> info;
  std::vector<std::pair<int, std::vector<int>>> sums;
  bool accumulate = false;  // Encoder::Accumulate (IRA codes)
  // decoder settings (ldpc.rs:165-172)
  Rule rule = RULE_SUM_PRODUCT;
  double alpha = 0.8;
  bool layered = true;
  int max_iterations = 50;
  bool exact_demap = false;  // the trial's demapper: Jacobian::Exact, else MaxLog
  // NrLdpc part (nr/ldpc.rs:65-75)
  bool nr = false;
  int bg = 0, z = 0, ils = 0, k_info = 0, e = 0;
  std::vector<int> map;  // BitSelection positions after the interleaver
  std::string error;
};

// gf2 inverse of the core block: row j lists the checks whose syndromes sum to parity
// bit k + j (ldpc.rs:568-584).  The inverse of an invertible matrix is unique, so a
// plain Gauss-Jordan on [B | I] gives the same rows as the reference's pivot order
// (the reference's own test ldpc.rs:931-954 checks exactly this equality).
static bool core_inverse(const Code& c, std::vector<std::vector<int>>& solve) {
  int core = c.core, k = c.k;
  int words = (core + 63) / 64;
  std::vector<std::vector<uint64_t>> a(core, std::vector<uint64_t>(2 * words, 0));
  for (int r = 0; r < core; r++) {
    for (int v : c.rows[r])
      if (v >= k) a[r][(v - k) / 64] ^= 1ull << ((v - k) % 64);
    a[r][words + r / 64] |= 1ull << (r % 64);
  }
  for (int col = 0; col < core; col++) {
    int w = col / 64;
    uint64_t b = 1ull << (col % 64);
    int piv = -1;
    for (int r = col; r < core; r++)
      if (a[r][w] & b) { piv = r; break; }
    if (piv < 0) return false;
    std::swap(a[col], a[piv]);
    for (int r = 0; r < core; r++)
      if (r != col && (a[r][w] & b))
        for (int x = 0; x < 2 * words; x++) a[r][x] ^= a[col][x];
  }
  solve.assign(core, {});
  for (int r = 0; r < core; r++)
    for (int cc = 0; cc < core; cc++)
      if (a[r][words + cc / 64] & (1ull << (cc % 64))) solve[r].push_back(cc);
  return true;
}

static void assemble_start(Code& c) {
  c.start.assign(c.rows.size() + 1, 0);
  for (size_t i = 0; i < c.rows.size(); i++) c.start[i + 1] = c.start[i] + (int)c.rows[i].size();
}

// nr/ldpc.rs:78-81
static int nr_base_graph(int k_info, int e) {
  double r = (double)k_info / (double)e;
  return (k_info <= 292 || (k_info <= 3824 && r <= 0.67) || r <= 0.25) ? 2 : 1;
}

// NrLdpc::with_options (nr/ldpc.rs:101-162), plus an explicit lifting size (z_force):
// the base-graph-2 codes with K' = 10 Z of the benchmark configurations are not reached
// by the Z rule of :110-123, so z_force composes the same steps with a given Z.
static bool nr_build(Code& c, int k_info, int e, int bg_force, int z_force, int rv, int qm) {
  if (!(k_info >= 1 && e >= 1)) { c.error = "need K' >= 1 and E >= 1"; return false; }
  if (!(rv >= 0 && rv <= 3 && qm >= 1 && e % qm == 0)) { c.error = "rv <= 3 and Qm | E"; return false; }
  int bg = bg_force ? bg_force : nr_base_graph(k_info, e);
  if (bg != 1 && bg != 2) { c.error = "the base graph is 1 or 2"; return false; }
  int k_cb = bg == 1 ? 8448 : 3840;
  if (k_info > k_cb) { c.error = "K' exceeds one code block"; return false; }
  int kb = bg == 1 ? 22 : (k_info > 640 ? 10 : k_info > 560 ? 9 : k_info > 192 ? 8 : 6);
  int z = -1, ils = -1;
  for (int i = 0; i < 8; i++)
    for (int t = 0; t < NR_LIFTING_SET_SIZES[i]; t++) {
      int zz = NR_LIFTING_SETS[i][t];
      bool ok = z_force ? (zz == z_force) : (kb * zz >= k_info);
      if (ok && (z < 0 || zz < z)) { z = zz; ils = i; }
    }
  if (z < 0) { c.error = "no lifting size"; return false; }
  int cols_k = bg == 1 ? 22 : 10, rows_n = bg == 1 ? 46 : 42;
  if (z_force && cols_k * z < k_info) { c.error = "K' exceeds the lifted systematic part"; return false; }
  const unsigned short(*table)[10] = bg == 1 ? NR_BG1 : NR_BG2;
  int entries = bg == 1 ? NR_BG1_ENTRIES : NR_BG2_ENTRIES;
  int k = cols_k * z, n_full = (cols_k + rows_n) * z;
  c.rows.assign((size_t)rows_n * z, {});
  for (int t = 0; t < entries; t++) {
    int i = table[t][0], j = table[t][1];
    int shift = table[t][2 + ils] % z;
    for (int r = 0; r < z; r++) c.rows[(size_t)i * z + r].push_back(j * z + (r + shift) % z);
  }
  // LdpcCode::from_core_rows (ldpc.rs:270-287)
  c.n = n_full;
  c.k = k;
  c.core = 4 * z;
  assemble_start(c);
  if (!core_inverse(c, c.solve)) { c.error = "the core block is singular"; return false; }
  c.info.resize(k);
  for (int i = 0; i < k; i++) c.info[i] = i;
  // circular buffer and k0 (nr/ldpc.rs:135-147)
  int ncb = n_full - 2 * z;
  int num = rv == 0 ? 0 : bg == 1 ? (rv == 1 ? 17 : rv == 2 ? 33 : 56) : (rv == 1 ? 13 : rv == 2 ? 25 : 43);
  int den = bg == 1 ? 66 : 50;
  long k0 = (long)num * ncb / ((long)den * z) * z;
  std::vector<int> sel;
  sel.reserve(e);
  long j = 0;
  while ((int)sel.size() < e) {
    int col = (int)(2 * z + (k0 + j) % ncb);
    if (!(col >= k_info && col < k)) sel.push_back(col);
    j++;
  }
  // Interleaver::block(qm, e/qm).interleave(sel) (nr/ldpc.rs:158-160, interleaving.rs:58-61)
  c.map.resize(e);
  int cols = e / qm;
  for (int t = 0; t < e; t++) c.map[t] = sel[(size_t)(t % qm) * cols + t / qm];
  c.nr = true;
  c.bg = bg;
  c.z = z;
  c.ils = ils;
  c.k_info = k_info;
  c.e = e;
  return true;
}

// LdpcCode::encode_block with Encoder::Core (ldpc.rs:753-791, :774-786)
static void encode_core(const Code& c, const uint8_t* u, uint8_t* cw) {
  int k = c.k;
  std::fill(cw, cw + c.n, 0);
  for (int i = 0; i < k; i++) cw[i] = u[i] & 1;
  std::vector<uint8_t> syn(c.core);
  for (int r = 0; r < c.core; r++) {
    uint8_t a = 0;
    for (int v : c.rows[r])
      if (v < k) a ^= cw[v];
    syn[r] = a;
  }
  for (int jj = 0; jj < c.core; jj++) {
    uint8_t a = 0;
    for (int r : c.solve[jj]) a ^= syn[r];
    cw[k + jj] = a;
  }
  for (size_t r = c.core; r < c.rows.size(); r++) {
    uint8_t a = 0;
    for (int v : c.rows[r])
      if (v != k + (int)r) a ^= cw[v];
    cw[k + r] = a;
  }
}

static bool is_codeword(const Code& c, const uint8_t* cw) {
  for (auto& row : c.rows) {
    uint8_t a = 0;
    for (int v : row) a ^= cw[v];
    if (a) return false;
  }
  return true;
}

// check_message (ldpc.rs:449-493), in the arithmetic type T
template <typename T>
static void check_message(const Code& c, const T* incoming, T* out, int d, std::vector<T>& scratch) {
  if (c.rule == RULE_SUM_PRODUCT) {
    scratch.resize(d);
    for (int i = 0; i < d; i++) scratch[i] = std::tanh(incoming[i] / (T)2.0);
    T prefix = 1.0;
    for (int i = 0; i < d; i++) { out[i] = prefix; prefix *= scratch[i]; }
    T suffix = 1.0;
    for (int i = d - 1; i >= 0; i--) {
      T p = out[i] * suffix;
      suffix *= scratch[i];
      // TANH_BOUND rounds to 1 in f32: there the bound is the largest float below 1
      const T bound = sizeof(T) == 4 ? (T)std::nextafter(1.0f, 0.0f) : (T)TANH_BOUND;
      T cl = std::min(std::max(p, -bound), bound);
      out[i] = (T)2.0 * std::atanh(cl);
    }
    return;
  }
  T sign = 1.0;
  for (int i = 0; i < d; i++) sign *= incoming[i] < (T)0.0 ? (T)-1.0 : (T)1.0;
  T m1 = std::numeric_limits<T>::infinity(), m2 = m1;
  int i1 = 0;
  for (int i = 0; i < d; i++) {
    T a = std::fabs(incoming[i]);
    if (a < m1) { m2 = m1; m1 = a; i1 = i; }
    else if (a < m2) m2 = a;
  }
  T alpha = (T)c.alpha;
  for (int i = 0; i < d; i++) {
    T mag = i == i1 ? m2 : m1;
    T s = sign * (incoming[i] < (T)0.0 ? (T)-1.0 : (T)1.0);
    T m;
    if (c.rule == RULE_NMS) m = alpha * mag;
    else { m = mag - alpha; m = m > (T)0.0 ? m : (T)0.0; }  // (mag - b).max(0.0)
    out[i] = s * m;
  }
}

// hard_decisions_are_a_codeword (ldpc.rs:555-557)
template <typename T>
static bool hd_codeword(const Code& c, const T* post) {
  for (auto& row : c.rows) {
    uint8_t a = 0;
    for (int v : row) a ^= (uint8_t)(post[v] < (T)0.0);
    if (a) return false;
  }
  return true;
}

// propagate (ldpc.rs:509-551): post holds the channel LLRs on entry
template <typename T>
static int propagate(const Code& c, const T* channel, T* post) {
  if (hd_codeword(c, post)) return 0;
  int edges = c.start.back();
  std::vector<T> c2v(edges, (T)0.0), new_c2v(c.layered ? 0 : edges, (T)0.0);
  std::vector<T> incoming, scratch;
  for (int it = 1; it <= c.max_iterations; it++) {
    if (c.layered) {
      for (size_t r = 0; r < c.rows.size(); r++) {
        const auto& row = c.rows[r];
        T* msgs = &c2v[c.start[r]];
        int d = (int)row.size();
        incoming.resize(d);
        for (int i = 0; i < d; i++) incoming[i] = post[row[i]] - msgs[i];
        check_message<T>(c, incoming.data(), msgs, d, scratch);
        for (int i = 0; i < d; i++) post[row[i]] = incoming[i] + msgs[i];
      }
    } else {
      for (size_t r = 0; r < c.rows.size(); r++) {
        const auto& row = c.rows[r];
        int d = (int)row.size();
        incoming.resize(d);
        for (int i = 0; i < d; i++) incoming[i] = post[row[i]] - c2v[c.start[r] + i];
        check_message<T>(c, incoming.data(), &new_c2v[c.start[r]], d, scratch);
      }
      for (int v = 0; v < c.n; v++) post[v] = channel[v];
      for (size_t r = 0; r < c.rows.size(); r++) {
        const auto& row = c.rows[r];
        for (size_t i = 0; i < row.size(); i++) post[row[i]] += new_c2v[c.start[r] + i];
      }
      std::swap(c2v, new_c2v);
    }
    if (hd_codeword(c, post)) return it;
  }
  return c.max_iterations;
}

// NrLdpc::full_llr (nr/ldpc.rs:191-197) with BitSelection::accumulate_into (puncture.rs:157-176)
template <typename T>
static void full_llr(const Code& c, const T* llr, T* full) {
  for (int v = 0; v < c.n; v++) full[v] = (T)0.0;
  for (int t = 0; t < c.e; t++) full[c.map[t]] += llr[t];
  for (int v = c.k_info; v < c.k; v++) full[v] = (T)KNOWN_BIT_LLR;
}

// NrLdpc::decode_block / app_into (nr/ldpc.rs:216-240): returns the iterations
template <typename T>
static int nr_decode(const Code& c, const T* llr, uint8_t* bits, T* app, T* post_out) {
  std::vector<T> full(c.n), post;
  full_llr<T>(c, llr, full.data());
  post = full;
  int it = propagate<T>(c, full.data(), post.data());
  if (bits)
    for (int i = 0; i < c.k_info; i++) bits[i] = (uint8_t)(post[i] < (T)0.0);
  if (app)
    for (int i = 0; i < c.k_info; i++) app[i] = post[i];
  if (post_out)
    for (int v = 0; v < c.n; v++) post_out[v] = post[v];
  return it;
}

// ------------------------------------------------------------------ mapping
// Constellation::new(Qam, m) (constellation.rs:168-202), normalized (:396),
// pam_levels (:449-451), gray (com-math bits.rs:37-39)
struct Qam {
  int m = 0, bits = 0;
  std::vector<double> re, im;
  double log_m = 0;  // ln(M), demapper.rs:279
};
static bool qam_new(int m, Qam& q) {
  int side = (int)std::lround(std::sqrt((double)m));
  if (m < 4 || (m & (m - 1)) || side * side != m) return false;
  std::vector<double> lv(side);
  for (int i = 0; i < side; i++) lv[i] = 2.0 * (double)i - ((double)side - 1.0);
  std::vector<double> nre, nim;
  for (int r = 0; r < side; r++) {
    double imv = lv[side - 1 - r];
    for (int t = 0; t < side; t++) {
      int tt = (r % 2 == 1) ? side - 1 - t : t;
      nre.push_back(lv[tt]);
      nim.push_back(imv);
    }
  }
  q.m = m;
  q.bits = __builtin_ctz(m);
  q.re.assign(m, 0);
  q.im.assign(m, 0);
  for (int i = 0; i < m; i++) {
    int g = i ^ (i >> 1);
    q.re[g] = nre[i];
    q.im[g] = nim[i];
  }
  // energy = power(points) = (sum |x|^2) / M (com-math lib.rs:138-148), scale 1/sqrt(Es)
  double e = 0.0;
  for (int i = 0; i < m; i++) e += q.re[i] * q.re[i] + q.im[i] * q.im[i];
  double es = e / (double)m;
  double s = 1.0 / std::sqrt(es);
  for (int i = 0; i < m; i++) { q.re[i] *= s; q.im[i] *= s; }
  q.log_m = std::log((double)m);
  return true;
}

// llr_kernel + llr_from_metrics + LabelHalves, max-log (demapper.rs:82-146, :270-297)
// Jacobian::Exact (demapper.rs:82-133): per half of the labels, the largest metric and
// the sum of exp(metric - max) in label order; L = m0 + ln s0 - m1 - ln s1
static void demap_exact(const Qam& q, double yre, double yim, double sigma2, double* out) {
  double metric[256];
  double uniform = -q.log_m;
  for (int i = 0; i < q.m; i++) {
    double dr = yre - q.re[i], di = yim - q.im[i];
    double ns = dr * dr + di * di;
    metric[i] = -ns / sigma2 + uniform;
  }
  for (int o = 0; o < q.bits; o++) {
    int shift = q.bits - 1 - o;
    double m0 = -std::numeric_limits<double>::infinity(), m1 = m0;
    for (int i = 0; i < q.m; i++) {
      if (((i >> shift) & 1) == 0) m0 = std::fmax(m0, metric[i]);
      else m1 = std::fmax(m1, metric[i]);
    }
    if (!std::isfinite(m0) || !std::isfinite(m1)) {
      out[o] = m0 - m1;
      continue;
    }
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < q.m; i++) {
      if (((i >> shift) & 1) == 0) s0 += std::exp(metric[i] - m0);
      else s1 += std::exp(metric[i] - m1);
    }
    out[o] = m0 + std::log(s0) - m1 - std::log(s1);
  }
}

static void demap_maxlog(const Qam& q, double yre, double yim, double sigma2, double* out) {
  double metric[256];
  double uniform = -q.log_m;
  for (int i = 0; i < q.m; i++) {
    double dr = yre - q.re[i], di = yim - q.im[i];
    double ns = dr * dr + di * di;  // num-complex norm_sqr
    metric[i] = -ns / sigma2 + uniform;
  }
  for (int o = 0; o < q.bits; o++) {
    int shift = q.bits - 1 - o;
    double m0 = -std::numeric_limits<double>::infinity(), m1 = m0;
    for (int i = 0; i < q.m; i++) {
      if (((i >> shift) & 1) == 0) m0 = std::fmax(m0, metric[i]);
      else m1 = std::fmax(m1, metric[i]);
    }
    out[o] = m0 - m1;
  }
}

// ------------------------------------------------------------------ the trial
struct FrameResult {
  uint32_t bit_errors;
  uint8_t frame_error;
  uint8_t iterations;
  uint16_t pad;
};

// One BICM-LDPC frame, in the order of the spec chain fec_encode -> map -> awgn_ebn0
// -> demap(max_log) -> fec_decode (com-spec blocks/coding/fec.rs:60-102,
// blocks/coding/map.rs:31-77, blocks/channel.rs:141-156, blocks/frame.rs:250-259) and
// the frame counts of validation/src/lib.rs:163-169.  `precision` 0 = f64 LLRs and
// decoder, 1 = the f64 LLRs rounded to f32 and decoded in f32.
static FrameResult run_trial(const Code& c, const Qam& q, Rng& rng, double ebn0_db, int precision,
                             NoiseMode mode, uint8_t* info_out, double* llr_out) {
  int kk = c.k_info, e = c.e, mb = q.bits;
  std::vector<uint8_t> u(c.k, 0), cw(c.n);
  for (int i = 0; i < kk; i++) u[i] = rng.bit();  // source::bits (source.rs:30-32)
  encode_core(c, u.data(), cw.data());
  std::vector<uint8_t> bits(e);
  for (int t = 0; t < e; t++) bits[t] = cw[c.map[t]];  // BitSelection::select
  while ((int)bits.size() % mb != 0) bits.push_back(rng.bit());  // map.rs:36-38
  int ns = (int)bits.size() / mb;
  std::vector<double> xr(ns), xi(ns);
  double energy = 0.0;
  for (int s = 0; s < ns; s++) {
    int idx = 0;
    for (int b = 0; b < mb; b++) idx = (idx << 1) | (bits[(size_t)s * mb + b] & 1);
    xr[s] = q.re[idx];
    xi[s] = q.im[idx];
  }
  for (int s = 0; s < ns; s++) energy += xr[s] * xr[s] + xi[s] * xi[s];
  double p = (0.0 + energy) / (double)ns;                       // frame.rs:256-259
  double rate = (double)kk / (double)e;                         // block.rs:59-61
  double b = (double)mb * rate;                                 // channel.rs:145-149
  double sigma2 = p * 1.0 / (b * db2lin(ebn0_db));              // awgn.rs:139-141
  double sd = std::sqrt(sigma2);                                // awgn.rs:94-99
  for (int s = 0; s < ns; s++) {
    double nr, ni;
    rng.complex_gaussian(nr, ni, mode);
    xr[s] += nr * sd;
    xi[s] += ni * sd;
  }
  std::vector<double> llr((size_t)ns * mb);
  for (int s = 0; s < ns; s++) {
    if (c.exact_demap) demap_exact(q, xr[s], xi[s], sigma2, &llr[(size_t)s * mb]);
    else demap_maxlog(q, xr[s], xi[s], sigma2, &llr[(size_t)s * mb]);
  }
  // fec_decode reads the first E LLRs of the stream (the padding bits are dropped)
  std::vector<uint8_t> dec(kk);
  int it;
  if (precision == 0) {
    it = nr_decode<double>(c, llr.data(), dec.data(), nullptr, nullptr);
  } else {
    std::vector<float> lf(e);
    for (int t = 0; t < e; t++) lf[t] = (float)llr[t];
    it = nr_decode<float>(c, lf.data(), dec.data(), nullptr, nullptr);
  }
  uint32_t be = 0;
  for (int i = 0; i < kk; i++) be += (dec[i] & 1) != (u[i] & 1);  // errors.rs:39-42
  if (info_out) std::memcpy(info_out, u.data(), kk);
  if (llr_out) std::memcpy(llr_out, llr.data(), sizeof(double) * e);
  FrameResult r;
  r.bit_errors = be;
  r.frame_error = be > 0;
  r.iterations = (uint8_t)it;
  r.pad = 0;
  return r;
}

// Runs frames [first, first + n) of one condition over `threads` workers; frame f draws
// from stream(seed, name, cond, f) (runner.rs:435-447), results in frame order.
static void run_frames(const Code& c, const Qam& q, uint64_t seed, uint64_t name_hash, uint64_t cond,
                       uint64_t first, uint64_t n, double ebn0_db, int precision, NoiseMode mode,
                       int threads, FrameResult* out) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<uint64_t> next(0);
  auto work = [&]() {
    for (;;) {
      uint64_t i = next.fetch_add(1);
      if (i >= n) break;
      Rng rng = stream(seed, name_hash, cond, first + i);
      out[i] = run_trial(c, q, rng, ebn0_db, precision, mode, nullptr, nullptr);
    }
  };
  if (threads == 1) { work(); return; }
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(work);
  for (auto& t : pool) t.join();
}

// ------------------------------------------------------------------ alist (ldpc.rs:350-742)
static bool parse_alist(const char* text, Code& c) {
  std::vector<long> nums;
  const char* p = text;
  while (*p) {
    if (*p == '#') { while (*p && *p != '\n') p++; continue; }
    if (*p >= '0' && *p <= '9') { nums.push_back(strtol(p, (char**)&p, 10)); continue; }
    p++;
  }
  size_t pos = 0;
  auto next = [&](long& v) { if (pos >= nums.size()) return false; v = nums[pos++]; return true; };
  long n, m, mc, mr;
  if (!next(n) || !next(m) || !next(mc) || !next(mr) || n <= 0 || m <= 0) { c.error = "alist header"; return false; }
  std::vector<long> cd(n), rd(m);
  for (long i = 0; i < n; i++) if (!next(cd[i])) { c.error = "alist col degrees"; return false; }
  for (long i = 0; i < m; i++) if (!next(rd[i])) { c.error = "alist row degrees"; return false; }
  long edges = 0, redges = 0;
  for (long d : cd) edges += d;
  for (long d : rd) redges += d;
  size_t rest = nums.size() - pos;
  bool padded = rest == (size_t)(n * mc + m * mr);
  if (!padded && rest != (size_t)(2 * edges)) { c.error = "alist list sizes"; return false; }
  for (long i = 0; i < n; i++) pos += padded ? mc : cd[i];
  c.rows.assign(m, {});
  for (long r = 0; r < m; r++) {
    long w = padded ? mr : rd[r];
    for (long t = 0; t < w; t++) {
      long v = nums[pos++];
      if (t < rd[r]) c.rows[r].push_back((int)v - 1);
    }
  }
  (void)redges;
  c.n = (int)n;
  return true;
}

// LdpcCode::from_rows (ldpc.rs:216-231): reduced H, pivots from gf2::Matrix::reduce.
// The parity bits of an (n, k) code are fixed by the information bits whatever the
// elimination order only for a given set of information positions; the reference
// reduces from the last column (com-math gf2.rs), which this restates: pivots are
// searched from the last column down, so the parity positions are the highest
// independent columns.
static bool from_rows(Code& c) {
  int n = c.n, m = (int)c.rows.size();
  int words = (n + 63) / 64;
  std::vector<std::vector<uint64_t>> a(m, std::vector<uint64_t>(words, 0));
  for (int r = 0; r < m; r++)
    for (int v : c.rows[r]) a[r][v / 64] ^= 1ull << (v % 64);
  std::vector<int> pivots;
  int row = 0;
  for (int col = n - 1; col >= 0 && row < m; col--) {
    int w = col / 64;
    uint64_t b = 1ull << (col % 64);
    int piv = -1;
    for (int r = row; r < m; r++) if (a[r][w] & b) { piv = r; break; }
    if (piv < 0) continue;
    std::swap(a[row], a[piv]);
    for (int r = 0; r < m; r++)
      if (r != row && (a[r][w] & b))
        for (int x = 0; x < words; x++) a[r][x] ^= a[row][x];
    pivots.push_back(col);
    row++;
  }
  std::vector<char> is_piv(n, 0);
  for (int pc : pivots) is_piv[pc] = 1;
  c.info.clear();
  for (int v = 0; v < n; v++) if (!is_piv[v]) c.info.push_back(v);
  c.sums.clear();
  for (size_t t = 0; t < pivots.size(); t++) {
    std::vector<int> deps;
    for (int v : c.info) if (a[t][v / 64] & (1ull << (v % 64))) deps.push_back(v);
    c.sums.push_back({pivots[t], deps});
  }
  c.k = (int)c.info.size();
  c.core = 0;
  assemble_start(c);
  return true;
}

// LdpcCode::accumulate (ldpc.rs:241-256): the dual-diagonal structure is checked by the
// library under test; the oracle only takes k = n - m and the information bits first
static bool from_rows_accumulate(Code& c) {
  int m = (int)c.rows.size();
  if (!(m > 0 && m < c.n)) { c.error = "bad accumulate code size"; return false; }
  c.k = c.n - m;
  c.info.clear();
  for (int i = 0; i < c.k; i++) c.info.push_back(i);
  c.accumulate = true;
  c.core = 0;
  assemble_start(c);
  return true;
}

// Encoder::Accumulate (ldpc.rs:765-772): parity bit k + r is the running sum of the
// information bits of checks 0..r
static void encode_accumulate(const Code& c, const uint8_t* u, uint8_t* cw) {
  std::fill(cw, cw + c.n, 0);
  for (int i = 0; i < c.k; i++) cw[i] = u[i] & 1;
  uint8_t prev = 0;
  for (size_t r = 0; r < c.rows.size(); r++) {
    uint8_t a = 0;
    for (int v : c.rows[r]) if (v < c.k) a ^= cw[v];
    prev ^= a;
    cw[c.k + r] = prev;
  }
}

static void encode_sums(const Code& c, const uint8_t* u, uint8_t* cw) {
  std::fill(cw, cw + c.n, 0);
  for (size_t i = 0; i < c.info.size(); i++) cw[c.info[i]] = u[i] & 1;
  for (auto& pr : c.sums) {
    uint8_t a = 0;
    for (int v : pr.second) a ^= cw[v];
    cw[pr.first] = a;
  }
}

// ------------------------------------------------------------------ spec link
// The link fec_encode -> map -> awgn_ebn0 -> demap -> fec_decode of a com-spec
// specification over a generic LdpcCode (the PEG code of specs/bicm_ldpc.yaml), with
// its metrics:
//   Encode::apply (crates/com-spec/src/blocks/coding/fec.rs:60-78): k x blocks bits,
//   the blocks' codewords one after the other, then Interleaver::random(len, seed)
//   (crates/com-fec/src/interleaving.rs:63-67, out[i] = in[perm[i]]);
//   Map and Demap (blocks/coding/map.rs:31-77); AwgnEbn0 (blocks/channel.rs:141-156,
//   b = log2 M k / n, block.rs:59-61);
//   Decode::apply (fec.rs:88-102): deinterleave (x[perm[i]] = y[i]), decode every block,
//   hard decisions at the information positions (ldpc.rs:793-796);
//   ber: the samples scaled by sqrt(energy(x) / energy(y)), the grid slicer's decisions
//   against the sent bits (crates/com-spec/src/metrics.rs:254-284, :374-383,
//   crates/com-math/src/nearest.rs); coded_ber and bler (metrics.rs:334-351).

static std::vector<int32_t> random_perm(int n, uint64_t seed) {
  std::vector<int32_t> perm(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  Rng r(seed);
  r.shuffle(perm);
  return perm;
}

// nearest.rs Slicer::detect for a square QAM: the levels of each axis (sorted, equal
// within 1e-9 of the span merged), the step of the real levels, a lookup by cell
struct GridSlicer {
  int side = 0;
  double step = 0, re0 = 0, im0 = 0;
  std::vector<int> lookup;
};

static std::vector<double> axis_levels(std::vector<double> l) {
  std::sort(l.begin(), l.end());
  double span = std::max(std::fabs(l.back() - l[0]), 1e-300);
  std::vector<double> out;
  for (double v : l)
    if (out.empty() || std::fabs(out.back() - v) > 1e-9 * span) out.push_back(v);
  return out;
}

static GridSlicer grid_slicer(const Qam& q) {
  GridSlicer g;
  std::vector<double> re = axis_levels(q.re), im = axis_levels(q.im);
  g.side = (int)re.size();
  g.step = (re.back() - re[0]) / (double)(g.side - 1);
  g.re0 = re[0];
  g.im0 = im[0];
  g.lookup.assign(q.m, 0);
  for (int i = 0; i < q.m; i++) {
    int c = (int)std::round((q.re[i] - re[0]) / g.step), r = (int)std::round((q.im[i] - im[0]) / g.step);
    g.lookup[r * g.side + c] = i;
  }
  return g;
}

static int grid_cell(const GridSlicer& g, double x, double x0) {
  double c = std::round((x - x0) / g.step);
  return (int)std::min(std::max(c, 0.0), (double)(g.side - 1));
}

struct LinkCounts {
  int64_t raw_errors, raw_bits, coded_errors, coded_bits, block_errors, blocks, iterations;
};

static LinkCounts link_trial(const Code& c, const Qam& q, const GridSlicer& g, int blocks,
                             const std::vector<int32_t>* perm, Rng& rng, double ebn0_db, NoiseMode mode,
                             double* llr_out, uint8_t* payload_out) {
  const int k = c.k, n = c.n, mb = q.bits, nb = n * blocks;
  std::vector<uint8_t> u((size_t)k * blocks), coded(nb);
  for (auto& b : u) b = rng.bit();  // fec.rs:63
  for (int b = 0; b < blocks; b++) {
    if (c.accumulate) encode_accumulate(c, &u[(size_t)b * k], &coded[(size_t)b * n]);
    else encode_sums(c, &u[(size_t)b * k], &coded[(size_t)b * n]);
  }
  std::vector<uint8_t> bits(nb);
  for (int i = 0; i < nb; i++) bits[i] = perm ? coded[(*perm)[i]] : coded[i];
  while ((int)bits.size() % mb != 0) bits.push_back(rng.bit());  // map.rs:36-38
  const int ns = (int)bits.size() / mb;
  std::vector<double> xr(ns), xi(ns), yr(ns), yi(ns);
  for (int s = 0; s < ns; s++) {
    int idx = 0;
    for (int b = 0; b < mb; b++) idx = (idx << 1) | (bits[(size_t)s * mb + b] & 1);
    xr[s] = q.re[idx];
    xi[s] = q.im[idx];
  }
  double ex = 0.0;
  for (int s = 0; s < ns; s++) ex += xr[s] * xr[s] + xi[s] * xi[s];
  double p = (0.0 + ex) / (double)ns;
  double rate = (double)k / (double)n;
  double sigma2 = p * 1.0 / ((double)mb * rate * db2lin(ebn0_db));
  double sd = std::sqrt(sigma2);
  for (int s = 0; s < ns; s++) {
    double nr, ni;
    rng.complex_gaussian(nr, ni, mode);
    yr[s] = xr[s] + nr * sd;
    yi[s] = xi[s] + ni * sd;
  }
  std::vector<double> llr((size_t)ns * mb);
  for (int s = 0; s < ns; s++) {
    if (c.exact_demap) demap_exact(q, yr[s], yi[s], sigma2, &llr[(size_t)s * mb]);
    else demap_maxlog(q, yr[s], yi[s], sigma2, &llr[(size_t)s * mb]);
  }
  LinkCounts r{};
  // ber: energy(x) and energy(y) over the window (every symbol), g = sqrt(px / pz)
  double ey = 0.0;
  for (int s = 0; s < ns; s++) ey += yr[s] * yr[s] + yi[s] * yi[s];
  double ex0 = 0.0 + ex, ey0 = 0.0 + ey;
  double gain = ey0 > 0.0 ? std::sqrt(ex0 / ey0) : 1.0;
  for (int s = 0; s < ns; s++) {
    double zr = yr[s] * gain, zi = yi[s] * gain;
    int lab = g.lookup[grid_cell(g, zi, g.im0) * g.side + grid_cell(g, zr, g.re0)];
    for (int b = 0; b < mb; b++) r.raw_errors += ((lab >> (mb - 1 - b)) & 1) != bits[(size_t)s * mb + b];
  }
  r.raw_bits = (int64_t)ns * mb;
  // fec_decode: the first n x blocks LLRs, deinterleaved, block by block
  std::vector<double> dl(nb), post(n);
  for (int i = 0; i < nb; i++) {
    if (perm) dl[(*perm)[i]] = llr[i];
    else dl[i] = llr[i];
  }
  for (int b = 0; b < blocks; b++) {
    std::copy(&dl[(size_t)b * n], &dl[(size_t)b * n] + n, post.begin());
    r.iterations += propagate<double>(c, &dl[(size_t)b * n], post.data());
    int e = 0;
    for (int i = 0; i < k; i++) e += (uint8_t)(post[c.info[i]] < 0.0) != u[(size_t)b * k + i];
    r.coded_errors += e;
    r.block_errors += e > 0;
  }
  r.coded_bits = (int64_t)k * blocks;
  r.blocks = blocks;
  if (llr_out) std::memcpy(llr_out, dl.data(), sizeof(double) * nb);
  if (payload_out) std::memcpy(payload_out, u.data(), u.size());
  return r;
}

// ------------------------------------------------------------------ learned min-sum
// Test oracle of this project's neural min-sum (no counterpart in the reference): the
// layered min-sum of propagate() with, at iteration t and edge e, the check message
//   y_e = s_e * max(alpha[t, e] * m_e - beta[t, e], 0)
// (s_e the sign product and m_e the minimum magnitude over the row's other edges, as
// check_message, ldpc.rs:468-491), run for exactly T iterations, and its loss
//   L = sum over the frame's bits [0, loss_bits) (n_full, or K') of
//       softplus(-(1 - 2 c_v) post_v) / loss_bits
// with the gradient of L with respect to every alpha and beta by reverse-mode
// differentiation of the T unrolled iterations (the minimum is differentiated
// through its argmin; sign and max(., 0) through their derivatives almost everywhere).
// Weights are indexed [t][entry][r] (per lifted edge) or [t][entry] (shared across Z),
// entry = the base-graph entry of the edge in table order, r its lifted row in the layer.
struct Learned {
  const Code* c;
  int T;
  bool shared;
  std::vector<int> lstart;  // base row -> first entry
  int multi = 0;  // 0: the last output's loss; 1: every iteration's, 1/T each; 2: ramp 2(t+1)/(T(T+1))
  int loss_bits = 0;  // the loss covers codeword bits [0, loss_bits): n_full, or K'
};

static void learned_layers(const Code& c, std::vector<int>& lstart) {
  const unsigned short(*table)[10] = c.bg == 1 ? NR_BG1 : NR_BG2;
  int entries = c.bg == 1 ? NR_BG1_ENTRIES : NR_BG2_ENTRIES;
  int rows_n = c.bg == 1 ? 46 : 42;
  lstart.assign(rows_n + 1, 0);
  for (int t = 0; t < entries; t++) lstart[table[t][0] + 1]++;
  for (int i = 0; i < rows_n; i++) lstart[i + 1] += lstart[i];
}

static inline size_t widx(const Learned& L, int t, int entry, int r) {
  int ne = L.lstart.back();
  return L.shared ? (size_t)t * ne + entry : ((size_t)t * ne + entry) * L.c->z + r;
}

static double softplus(double x) { return x > 0 ? x + std::log1p(std::exp(-x)) : std::log1p(std::exp(x)); }
static double sigmoid(double x) { return x >= 0 ? 1.0 / (1.0 + std::exp(-x)) : std::exp(x) / (1.0 + std::exp(x)); }
// the f32 forms of the GPU's training kernels (nms_learned.cu), with libm's expf
static float softplus(float x) { return x > 0.f ? x + std::log1p(std::exp(-x)) : std::log1p(std::exp(x)); }
static float sigmoid(float x) { return 1.f / (1.f + std::exp(-x)); }

// Forward (and backward when ga != nullptr) of one frame in arithmetic R; returns the
// loss.  R = double is the reference arithmetic.  R = float repeats the GPU's f32
// operations one by one (the same messages, argmins and active sets, so the adjoint takes
// the same subgradient) and scales the loss gradient as the GPU does, by
// 1 / (loss_bits n_frames) in f32 (`frames`); the gradients still accumulate in f64.
template <typename R>
static double learned_frame(const Learned& L, const R* full_llr, const uint8_t* cw, const double* alpha,
                            const double* beta, R* post_out, double* ga, double* gb, int64_t frames = 1) {
  const Code& c = *L.c;
  const int z = c.z, rows_n = (int)L.lstart.size() - 1, T = L.T;
  const int edges = c.start.back();
  std::vector<R> post(full_llr, full_llr + c.n), c2v(edges, (R)0);
  std::vector<R> X((size_t)T * edges), P;
  if (L.multi) P.assign((size_t)T * c.n, (R)0);
  for (int t = 0; t < T; t++) {
    for (int Ly = 0; Ly < rows_n; Ly++)
      for (int r = 0; r < z; r++) {
        int row = Ly * z + r, d = (int)c.rows[row].size(), e0 = c.start[row];
        R* x = &X[(size_t)t * edges + e0];
        for (int i = 0; i < d; i++) x[i] = post[c.rows[row][i]] - c2v[e0 + i];
        bool par = false;
        R m1 = (R)INFINITY, m2 = (R)INFINITY;
        int i1 = 0;
        for (int i = 0; i < d; i++) {
          par ^= x[i] < 0;
          R a = std::fabs(x[i]);
          if (a < m1) { m2 = m1; m1 = a; i1 = i; } else if (a < m2) m2 = a;
        }
        for (int i = 0; i < d; i++) {
          R m = i == i1 ? m2 : m1;
          bool neg = par ^ (x[i] < 0);
          size_t w = widx(L, t, L.lstart[Ly] + i, r);
          R a = std::fma((R)alpha[w], m, -(R)beta[w]);
          R mag = a > 0 ? a : (R)0;
          R y = neg ? -mag : mag;
          c2v[e0 + i] = y;
          post[c.rows[row][i]] = x[i] + y;
        }
      }
    if (L.multi) std::copy(post.begin(), post.end(), P.begin() + (size_t)t * c.n);
  }
  auto bit_loss = [&](const R* p) {
    double l = 0.0;
    for (int v = 0; v < L.loss_bits; v++) l += (double)softplus(cw[v] ? p[v] : -p[v]);
    return l / (double)L.loss_bits;
  };
  double loss = 0.0;
  auto weight = [&](int t) { return L.multi == 2 ? 2.0 * (t + 1) / ((double)T * (T + 1)) : 1.0 / (double)T; };
  if (L.multi)
    for (int t = 0; t < T; t++) loss += bit_loss(&P[(size_t)t * c.n]) * weight(t);
  else
    loss = bit_loss(post.data());
  if (post_out) std::copy(post.begin(), post.end(), post_out);
  if (!ga) return loss;
  // reverse sweep
  std::vector<R> gp(c.n, (R)0), gc(edges, (R)0);
  auto add_loss_grad = [&](const R* p, int t) {
    if (sizeof(R) == 8) {
      const double w = L.multi ? weight(t) : 1.0;
      for (int v = 0; v < L.loss_bits; v++) {
        double sgn = 1.0 - 2.0 * cw[v];
        gp[v] += (R)(-sgn * sigmoid((double)(-sgn * p[v])) * w / (double)L.loss_bits);
      }
    } else {
      const float scale = 1.f / ((float)L.loss_bits * (float)frames);
      const float wt = L.multi == 2 ? 2.f * (float)(t + 1) / ((float)T * (float)(T + 1)) : 1.f / (float)T;
      const float sc = L.multi ? scale * wt : scale;
      for (int v = 0; v < L.loss_bits; v++) {
        float sgn = cw[v] ? -1.f : 1.f;
        gp[v] += -sgn * sigmoid((float)(-sgn * (float)p[v])) * sc;
      }
    }
  };
  std::vector<R> gabs(32);
  for (int t = T - 1; t >= 0; t--) {
    if (L.multi || t == T - 1) add_loss_grad(L.multi ? &P[(size_t)t * c.n] : post.data(), t);
    for (int Ly = rows_n - 1; Ly >= 0; Ly--)
      for (int r = 0; r < z; r++) {
        int row = Ly * z + r, d = (int)c.rows[row].size(), e0 = c.start[row];
        const R* x = &X[(size_t)t * edges + e0];
        bool par = false;
        R m1 = (R)INFINITY, m2 = (R)INFINITY;
        int i1 = 0, i2 = 0;
        for (int i = 0; i < d; i++) {
          par ^= x[i] < 0;
          R a = std::fabs(x[i]);
          if (a < m1) { m2 = m1; i2 = i1; m1 = a; i1 = i; } else if (a < m2) { m2 = a; i2 = i; }
        }
        if (d == 1) i2 = i1;
        std::fill(gabs.begin(), gabs.begin() + d, (R)0);
        for (int i = 0; i < d; i++) {
          int v = c.rows[row][i];
          R m = i == i1 ? m2 : m1;
          bool neg = par ^ (x[i] < 0);
          size_t w = widx(L, t, L.lstart[Ly] + i, r);
          R a = std::fma((R)alpha[w], m, -(R)beta[w]);
          R g_y = gp[v] + gc[e0 + i];
          R g_a = a > 0 ? (neg ? -g_y : g_y) : (R)0;
          ga[w] += (double)(g_a * m);
          gb[w] -= (double)g_a;
          R g_m = g_a * (R)alpha[w];
          gabs[i == i1 ? i2 : i1] += g_m;
        }
        for (int i = 0; i < d; i++) {
          int v = c.rows[row][i];
          R g_x = gp[v] + (x[i] < 0 ? -gabs[i] : gabs[i]);
          gp[v] = g_x;
          gc[e0 + i] = -g_x;
        }
      }
  }
  return loss;
}

}  // namespace oracle

// ================================================================== C ABI (ctypes)
using namespace oracle;

extern "C" {

uint64_t or_rng_first(uint64_t seed) { Rng r(seed); return r.next_u64(); }
uint64_t or_fnv1a64(const uint8_t* b, size_t n) { return fnv1a64(b, n); }

// n raw next_u64 draws of stream(seed, name_hash, cond, trial)
void or_stream_draws(uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t trial, uint64_t n, uint64_t* out) {
  Rng r = stream(seed, name_hash, cond, trial);
  for (uint64_t i = 0; i < n; i++) out[i] = r.next_u64();
}

// n complex gaussians from Rng::new(seed); mode 0 = glibc, 1 = correctly rounded
void or_complex_gaussians(uint64_t seed, uint64_t n, int mode, double* re, double* im) {
  Rng r(seed);
  for (uint64_t i = 0; i < n; i++) r.complex_gaussian(re[i], im[i], (NoiseMode)mode);
}

void* or_code_new(int k_info, int e, int bg, int z, int rv, int qm, char* err, int errlen) {
  Code* c = new Code();
  if (!nr_build(*c, k_info, e, bg, z, rv, qm)) {
    if (err && errlen > 0) snprintf(err, errlen, "%s", c->error.c_str());
    delete c;
    return nullptr;
  }
  return c;
}

void* or_code_from_alist(const char* text, char* err, int errlen) {
  Code* c = new Code();
  if (!parse_alist(text, *c) || !from_rows(*c)) {
    if (err && errlen > 0) snprintf(err, errlen, "%s", c->error.c_str());
    delete c;
    return nullptr;
  }
  return c;
}

// a generic code from its rows (row_start[m + 1], vars): Encoder::Sums of from_rows, or
// Encoder::Accumulate when `accumulate` is set
void* or_code_from_rows(int n, int m, const int32_t* row_start, const int32_t* vars, int accumulate, char* err,
                        int errlen) {
  Code* c = new Code();
  c->n = n;
  c->rows.assign(m, {});
  for (int r = 0; r < m; r++)
    for (int e = row_start[r]; e < row_start[r + 1]; e++) c->rows[r].push_back(vars[e]);
  if (!(accumulate ? from_rows_accumulate(*c) : from_rows(*c))) {
    if (err && errlen > 0) snprintf(err, errlen, "%s", c->error.c_str());
    delete c;
    return nullptr;
  }
  return c;
}

// the information positions of a generic code (k entries)
void or_code_info_positions(void* h, int32_t* out) {
  Code* c = (Code*)h;
  for (size_t i = 0; i < c->info.size(); i++) out[i] = c->info[i];
}

void or_code_free(void* h) { delete (Code*)h; }

// out[0..8] = bg, z, k_info, e, K, n_full, rows, edges, ils
void or_code_info(void* h, int64_t* out) {
  Code* c = (Code*)h;
  out[0] = c->bg; out[1] = c->z; out[2] = c->k_info; out[3] = c->e; out[4] = c->k;
  out[5] = c->n; out[6] = (int64_t)c->rows.size(); out[7] = c->start.back(); out[8] = c->ils;
}

void or_code_bit_map(void* h, int64_t* out) {
  Code* c = (Code*)h;
  for (int t = 0; t < c->e; t++) out[t] = c->map[t];
}

// the lifted rows as (row, variable) pairs in edge order
void or_code_edges(void* h, int32_t* rows_out, int32_t* vars_out) {
  Code* c = (Code*)h;
  int t = 0;
  for (size_t r = 0; r < c->rows.size(); r++)
    for (int v : c->rows[r]) { rows_out[t] = (int32_t)r; vars_out[t] = v; t++; }
}

void or_code_set_decoder(void* h, int rule, double alpha, int layered, int max_iterations) {
  Code* c = (Code*)h;
  c->rule = (Rule)rule;
  c->alpha = alpha;
  c->layered = layered != 0;
  c->max_iterations = max_iterations;
}

// NrLdpc::encode_block: k_info bits -> e bits
void or_encode(void* h, const uint8_t* info, uint8_t* out) {
  Code* c = (Code*)h;
  std::vector<uint8_t> u(c->k, 0), cw(c->n);
  for (int i = 0; i < c->k_info; i++) u[i] = info[i] & 1;
  encode_core(*c, u.data(), cw.data());
  for (int t = 0; t < c->e; t++) out[t] = cw[c->map[t]];
}

// LdpcCode::encode_block on the full word: K bits -> n_full bits (Core or Sums)
void or_encode_full(void* h, const uint8_t* u, uint8_t* out) {
  Code* c = (Code*)h;
  if (c->core) encode_core(*c, u, out);
  else if (c->accumulate) encode_accumulate(*c, u, out);
  else encode_sums(*c, u, out);
}

int or_is_codeword(void* h, const uint8_t* cw) { return is_codeword(*(Code*)h, cw); }

// NrLdpc decode of e LLRs: bits (k_info), app (k_info) and post (n_full) optional
int or_decode_f64(void* h, const double* llr, uint8_t* bits, double* app, double* post) {
  return nr_decode<double>(*(Code*)h, llr, bits, app, post);
}
int or_decode_f32(void* h, const float* llr, uint8_t* bits, float* app, float* post) {
  return nr_decode<float>(*(Code*)h, llr, bits, app, post);
}

// LdpcCode::decode_llr on n_full LLRs
int or_decode_llr_f64(void* h, const double* full, double* post) {
  Code* c = (Code*)h;
  for (int v = 0; v < c->n; v++) post[v] = full[v];
  return propagate<double>(*c, full, post);
}
int or_decode_llr_f32(void* h, const float* full, float* post) {
  Code* c = (Code*)h;
  for (int v = 0; v < c->n; v++) post[v] = full[v];
  return propagate<float>(*c, full, post);
}

int or_qam_points(int m, double* re, double* im, double* log_m) {
  Qam q;
  if (!qam_new(m, q)) return -1;
  for (int i = 0; i < m; i++) { re[i] = q.re[i]; im[i] = q.im[i]; }
  *log_m = q.log_m;
  return 0;
}

void or_code_set_demapper(void* h, int exact) { ((Code*)h)->exact_demap = exact != 0; }
void or_demap_exact(int m, const double* yre, const double* yim, int64_t n, double sigma2, double* out) {
  Qam q;
  if (!qam_new(m, q)) return;
  for (int64_t s = 0; s < n; s++) demap_exact(q, yre[s], yim[s], sigma2, out + s * q.bits);
}
void or_demap_maxlog(int m, const double* yre, const double* yim, int64_t n, double sigma2, double* out) {
  Qam q;
  qam_new(m, q);
  for (int64_t s = 0; s < n; s++) demap_maxlog(q, yre[s], yim[s], sigma2, out + s * q.bits);
}

// one frame: info bits (k_info) and the e channel LLRs optionally returned
int or_trial(void* h, int m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t frame, double ebn0_db,
             int precision, int noise_mode, uint8_t* info_out, double* llr_out, uint32_t* result) {
  Code* c = (Code*)h;
  Qam q;
  if (!qam_new(m, q)) return -1;
  Rng rng = stream(seed, name_hash, cond, frame);
  FrameResult r = run_trial(*c, q, rng, ebn0_db, precision, (NoiseMode)noise_mode, info_out, llr_out);
  result[0] = r.bit_errors;
  result[1] = r.frame_error;
  result[2] = r.iterations;
  return 0;
}

// frames [first, first+n) on `threads` workers (0 = all cores); out = 8 bytes per frame
int or_run_frames(void* h, int m, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first, uint64_t n,
                  double ebn0_db, int precision, int noise_mode, int threads, void* out) {
  Code* c = (Code*)h;
  Qam q;
  if (!qam_new(m, q)) return -1;
  run_frames(*c, q, seed, name_hash, cond, first, n, ebn0_db, precision, (NoiseMode)noise_mode, threads,
             (FrameResult*)out);
  return 0;
}

// AFF3CT-style BPSK link on a generic code (validation/tests/aff3ct.rs:151-158 with
// validation/src/lib.rs:67-71): errors over all coded bits; returns (bit errors, it)
int or_bpsk_frame(void* h, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t trial, double noise_var,
                  uint32_t* result) {
  Code* c = (Code*)h;
  Rng rng = stream(seed, name_hash, cond, trial);
  std::vector<uint8_t> u(c->k), cw(c->n);
  for (int i = 0; i < c->k; i++) u[i] = rng.bit();
  if (c->core) encode_core(*c, u.data(), cw.data());
  else encode_sums(*c, u.data(), cw.data());
  double s = std::sqrt(noise_var);
  std::vector<double> llr(c->n), post(c->n);
  for (int v = 0; v < c->n; v++) {
    double x = 1.0 - 2.0 * (double)cw[v];
    double y = x + s * rng.gaussian();
    llr[v] = 2.0 * y / noise_var;
  }
  post = llr;
  int it = propagate<double>(*c, llr.data(), post.data());
  uint32_t be = 0;
  for (int v = 0; v < c->n; v++) be += (uint8_t)(post[v] < 0.0) != cw[v];
  result[0] = be;
  result[1] = (uint32_t)it;
  return 0;
}

// the codewords and channel LLRs of frames [first, first + n) of or_bpsk_frame's link
// (frame f draws from stream(seed, name_hash, cond, f)), `threads` threads
void or_bpsk_llr_batch(void* h, uint64_t seed, uint64_t name_hash, uint64_t cond, uint64_t first, int64_t n,
                       double noise_var, int threads, uint8_t* cw_out, double* llr_out) {
  const Code* c = (const Code*)h;
  auto work = [&](int64_t f0, int64_t f1) {
    std::vector<uint8_t> u(c->k);
    for (int64_t f = f0; f < f1; f++) {
      Rng rng = stream(seed, name_hash, cond, first + (uint64_t)f);
      uint8_t* cw = cw_out + f * c->n;
      double* llr = llr_out + f * c->n;
      for (int i = 0; i < c->k; i++) u[i] = rng.bit();
      if (c->core) encode_core(*c, u.data(), cw);
      else encode_sums(*c, u.data(), cw);
      const double s = std::sqrt(noise_var);
      for (int v = 0; v < c->n; v++) {
        double x = 1.0 - 2.0 * (double)cw[v];
        double y = x + s * rng.gaussian();
        llr[v] = 2.0 * y / noise_var;
      }
    }
  };
  threads = std::max(1, threads);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(work, n * t / threads, n * (t + 1) / threads);
  for (auto& th : pool) th.join();
}

// learned min-sum: forward (post_out n_full, optional) and gradients (ga/gb, optional,
// accumulated) of `n` frames of e received LLRs and n_full codeword bits; returns the
// mean loss over the frames
double or_learned(void* h, int T, int shared, int multi, const double* alpha, const double* beta, const double* llr,
                  const uint8_t* cw, int64_t n, double* post_out, double* ga, double* gb, int info_only) {
  Code* c = (Code*)h;
  Learned L{c, T, shared != 0, {}, multi, info_only ? c->k_info : c->n};
  learned_layers(*c, L.lstart);
  std::vector<double> full(c->n);
  double tot = 0.0;
  for (int64_t f = 0; f < n; f++) {
    full_llr<double>(*c, llr + f * c->e, full.data());
    tot += learned_frame<double>(L, full.data(), cw + f * c->n, alpha, beta, post_out ? post_out + f * c->n : nullptr,
                                 ga, gb);
  }
  return tot / (double)n;
}

// The same in the GPU's f32 arithmetic: f32 LLRs and posteriors, gradients of the mean
// loss over the n frames (already divided by n, in f32 as the GPU scales them).
double or_learned_f32(void* h, int T, int shared, int multi, const double* alpha, const double* beta,
                      const float* llr, const uint8_t* cw, int64_t n, float* post_out, double* ga, double* gb,
                      int info_only) {
  Code* c = (Code*)h;
  Learned L{c, T, shared != 0, {}, multi, info_only ? c->k_info : c->n};
  learned_layers(*c, L.lstart);
  std::vector<float> full(c->n);
  double tot = 0.0;
  for (int64_t f = 0; f < n; f++) {
    full_llr<float>(*c, llr + f * c->e, full.data());
    tot += learned_frame<float>(L, full.data(), cw + f * c->n, alpha, beta, post_out ? post_out + f * c->n : nullptr,
                                ga, gb, n);
  }
  return tot / (double)n;
}

int64_t or_learned_num_weights(void* h, int T, int shared) {
  Code* c = (Code*)h;
  std::vector<int> ls;
  learned_layers(*c, ls);
  return (int64_t)T * ls.back() * (shared ? 1 : c->z);
}

// Trials [first, first + n) of the spec link over a generic code (from_rows or
// accumulate) with `blocks` codewords per trial, the random interleaver of seed
// `il_seed` (il_seed < 0: none), M-QAM, the demapper of or_code_set_demapper and the
// code's decoder; 7 counts per trial into out (raw errors, raw bits, coded errors,
// coded bits, block errors, blocks, iterations); optionally the deinterleaved LLRs
// [n][blocks x n] and the payload bits [n][blocks x k].
int or_link_trials(void* h, int blocks, int64_t il_seed, int m, uint64_t seed, uint64_t name_hash, uint64_t cond,
                   uint64_t first, uint64_t n, double ebn0_db, int noise, int threads, int64_t* out, double* llr_out,
                   uint8_t* payload_out) {
  Code* c = (Code*)h;
  Qam q;
  if (!qam_new(m, q)) return -1;
  GridSlicer g = grid_slicer(q);
  std::vector<int32_t> perm;
  if (il_seed >= 0) perm = random_perm(c->n * blocks, (uint64_t)il_seed);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<uint64_t> next(0);
  auto work = [&]() {
    for (;;) {
      uint64_t i = next.fetch_add(1);
      if (i >= n) break;
      Rng rng = stream(seed, name_hash, cond, first + i);
      LinkCounts r = link_trial(*c, q, g, blocks, il_seed >= 0 ? &perm : nullptr, rng, ebn0_db, (NoiseMode)noise,
                                llr_out ? llr_out + i * (size_t)c->n * blocks : nullptr,
                                payload_out ? payload_out + i * (size_t)c->k * blocks : nullptr);
      int64_t* o = out + 7 * i;
      o[0] = r.raw_errors; o[1] = r.raw_bits; o[2] = r.coded_errors; o[3] = r.coded_bits;
      o[4] = r.block_errors; o[5] = r.blocks; o[6] = r.iterations;
    }
  };
  if (threads == 1) {
    work();
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++) pool.emplace_back(work);
    for (auto& t : pool) t.join();
  }
  return 0;
}

// Interleaver::random(n, seed)
void or_random_perm(int n, uint64_t seed, int32_t* out) {
  std::vector<int32_t> p = random_perm(n, seed);
  std::memcpy(out, p.data(), sizeof(int32_t) * n);
}

}  // extern "C"
