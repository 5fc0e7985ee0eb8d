// Host-side NR code construction for the GPU kernels (see code_host.h).
#include "code_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "nr_base_graphs.inc"

namespace cbh {

// TS 38.212 Sec. 7.2.2 as in nr/ldpc.rs:78-81
static int base_graph_rule(int k_info, int e) {
  double r = (double)k_info / (double)e;
  return (k_info <= 292 || (k_info <= 3824 && r <= 0.67) || r <= 0.25) ? 2 : 1;
}

// Gauss-Jordan inverse of a square GF(2) matrix held as rows of 64-bit words.
static bool gf2_inverse(std::vector<std::vector<uint64_t>>& a, int n, std::vector<std::vector<uint64_t>>& inv) {
  int words = (n + 63) / 64;
  inv.assign(n, std::vector<uint64_t>(words, 0));
  for (int r = 0; r < n; r++) inv[r][r / 64] |= 1ull << (r % 64);
  for (int col = 0; col < n; col++) {
    int w = col / 64;
    uint64_t b = 1ull << (col % 64);
    int piv = -1;
    for (int r = col; r < n; r++)
      if (a[r][w] & b) { piv = r; break; }
    if (piv < 0) return false;
    std::swap(a[col], a[piv]);
    std::swap(inv[col], inv[piv]);
    for (int r = 0; r < n; r++) {
      if (r != col && (a[r][w] & b)) {
        for (int x = 0; x < words; x++) { a[r][x] ^= a[col][x]; inv[r][x] ^= inv[col][x]; }
      }
    }
  }
  return true;
}

bool build_nr_code(const CodeSpec& s, NrCode& c, std::string& err) {
  if (!(s.k_info >= 1 && s.e >= 1)) { err = "need K' >= 1 and E >= 1"; return false; }
  if (!(s.rv >= 0 && s.rv <= 3 && s.qm >= 1 && s.e % s.qm == 0)) { err = "need rv <= 3 and Qm | E"; return false; }
  int bg = s.bg ? s.bg : base_graph_rule(s.k_info, s.e);
  if (bg != 1 && bg != 2) { err = "the base graph is 1 or 2"; return false; }
  int k_cb = bg == 1 ? 8448 : 3840;
  if (s.k_info > k_cb) { err = "K' exceeds one code block; segment the block first"; return false; }
  int kb = bg == 1 ? 22 : (s.k_info > 640 ? 10 : s.k_info > 560 ? 9 : s.k_info > 192 ? 8 : 6);
  int z = -1, ils = -1;
  for (int i = 0; i < 8; i++)
    for (int t = 0; t < NR_LIFTING_SET_SIZES[i]; t++) {
      int zz = NR_LIFTING_SETS[i][t];
      bool ok = s.z ? zz == s.z : kb * zz >= s.k_info;
      if (ok && (z < 0 || zz < z)) { z = zz; ils = i; }
    }
  if (z < 0) { err = s.z ? "not a lifting size of TS 38.212 Table 5.3.2-1" : "no lifting size"; return false; }
  c.bg = bg;
  c.z = z;
  c.ils = ils;
  c.cols_k = bg == 1 ? 22 : 10;
  c.rows_n = bg == 1 ? 46 : 42;
  c.k = c.cols_k * z;
  if (s.k_info > c.k) { err = "K' exceeds the systematic part of the lifted code"; return false; }
  c.n_full = (c.cols_k + c.rows_n) * z;
  c.k_info = s.k_info;
  c.e = s.e;
  c.rv = s.rv;
  c.qm = s.qm;
  const unsigned short(*table)[10] = bg == 1 ? NR_BG1 : NR_BG2;
  int entries = bg == 1 ? NR_BG1_ENTRIES : NR_BG2_ENTRIES;
  c.layer_start.assign(c.rows_n + 1, 0);
  c.entry_col.clear();
  c.entry_shift.clear();
  for (int t = 0; t < entries; t++) {
    c.entry_col.push_back(table[t][1]);
    c.entry_shift.push_back((uint16_t)(table[t][2 + ils] % z));
    c.layer_start[table[t][0] + 1]++;
  }
  c.max_degree = 0;
  for (int i = 0; i < c.rows_n; i++) {
    c.max_degree = std::max(c.max_degree, c.layer_start[i + 1]);
    c.layer_start[i + 1] += c.layer_start[i];
  }
  c.edges = entries * z;

  // core block B: core checks (base rows 0..3) on core parity columns (cols_k..cols_k+3)
  int core = 4 * z, words = (core + 63) / 64;
  std::vector<std::vector<uint64_t>> b(core, std::vector<uint64_t>(words, 0)), inv;
  for (int i = 0; i < 4; i++)
    for (int t = c.layer_start[i]; t < c.layer_start[i + 1]; t++) {
      int j = c.entry_col[t];
      if (j < c.cols_k) continue;
      int blk = j - c.cols_k, sh = c.entry_shift[t];
      for (int r = 0; r < z; r++) {
        int col = blk * z + (r + sh) % z;
        b[i * z + r][col / 64] ^= 1ull << (col % 64);
      }
    }
  if (!gf2_inverse(b, core, inv)) { err = "the core block is singular"; return false; }
  // every block of the inverse is a circulant: read its shifts from its first row and
  // check the other rows
  c.core_terms.clear();
  auto bit = [&](int r, int col) { return (inv[r][col / 64] >> (col % 64)) & 1; };
  for (int blk = 0; blk < 4; blk++)
    for (int src = 0; src < 4; src++) {
      std::vector<int> shifts;
      for (int cc = 0; cc < z; cc++)
        if (bit(blk * z, src * z + cc)) shifts.push_back(cc);
      for (int r = 1; r < z; r++)
        for (int cc = 0; cc < z; cc++) {
          bool want = std::find(shifts.begin(), shifts.end(), ((cc - r) % z + z) % z) != shifts.end();
          if ((bool)bit(blk * z + r, src * z + cc) != want) { err = "core inverse is not block-circulant"; return false; }
        }
      for (int sh : shifts) c.core_terms.push_back({(uint16_t)blk, (uint16_t)src, (uint16_t)sh});
    }
  if ((int)c.core_terms.size() > kMaxCoreTerms) { err = "core inverse too dense"; return false; }

  // rate matching (nr/ldpc.rs:135-160)
  c.ncb = c.n_full - 2 * z;
  int num = s.rv == 0 ? 0 : bg == 1 ? (s.rv == 1 ? 17 : s.rv == 2 ? 33 : 56) : (s.rv == 1 ? 13 : s.rv == 2 ? 25 : 43);
  int den = bg == 1 ? 66 : 50;
  c.k0 = (int)((long)num * c.ncb / ((long)den * z) * z);
  std::vector<int32_t> sel;
  sel.reserve(s.e);
  long j = 0;
  while ((int)sel.size() < s.e) {
    int col = (int)(2 * z + (c.k0 + j) % c.ncb);
    if (!(col >= s.k_info && col < c.k)) sel.push_back(col);
    j++;
    if (j > (long)c.ncb * ((long)s.e / std::max(1, c.ncb - (c.k - s.k_info)) + 2)) { err = "rate matching"; return false; }
  }
  c.map.assign(s.e, 0);
  int cols = s.e / s.qm;
  c.map_is_offset = true;
  for (int t = 0; t < s.e; t++) {
    c.map[t] = sel[(size_t)(t % s.qm) * cols + t / s.qm];
    if (c.map[t] != 2 * z + t) c.map_is_offset = false;
  }
  c.inv_start.assign(c.n_full + 1, 0);
  for (int t = 0; t < s.e; t++) c.inv_start[c.map[t] + 1]++;
  c.has_repeats = false;
  for (int v = 0; v < c.n_full; v++) {
    if (c.inv_start[v + 1] > 1) c.has_repeats = true;
    c.inv_start[v + 1] += c.inv_start[v];
  }
  c.inv_t.assign(s.e, 0);
  std::vector<int32_t> fill(c.inv_start.begin(), c.inv_start.end() - 1);
  for (int t = 0; t < s.e; t++) c.inv_t[fill[c.map[t]]++] = t;
  return true;
}

// ------------------------------------------------------------------ xoshiro jump-ahead
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline void xoshiro_step(uint64_t s[4]) {
  uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl(s[3], 45);
}

// 512-bit polynomial helpers over GF(2) (bit i = coefficient of x^i)
struct P512 {
  uint64_t w[8];
};

// The characteristic polynomial of the state transition, by Berlekamp-Massey on the
// sequence of one state bit (the transition of xoshiro256 has a primitive
// characteristic polynomial of degree 256, so the minimal polynomial of any nonzero
// bit sequence it generates is that polynomial).  Returned as its low 256 coefficients
// (the x^256 coefficient is 1).
static void char_poly(uint64_t out[4]) {
  const int N = 512;
  std::vector<int> seq(N);
  uint64_t s[4] = {0x0123456789abcdefull, 0xfedcba9876543210ull, 0x0f1e2d3c4b5a6978ull, 0x8796a5b4c3d2e1f0ull};
  for (int i = 0; i < N; i++) {
    seq[i] = (int)(s[0] & 1);
    xoshiro_step(s);
  }
  std::vector<int> C(N + 1, 0), B(N + 1, 0), T;
  C[0] = B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < N; n++) {
    int d = seq[n];
    for (int i = 1; i <= L; i++) d ^= C[i] & seq[n - i];
    if (d == 0) { m++; continue; }
    T = C;
    for (int i = 0; i + m <= N; i++) C[i + m] ^= B[i];
    if (2 * L <= n) { L = n + 1 - L; B = T; m = 1; }
    else m++;
  }
  // connection polynomial C(x) = 1 + c1 x + ... + cL x^L; P(x) = x^L C(1/x)
  std::memset(out, 0, 4 * sizeof(uint64_t));
  for (int i = 0; i < L; i++)  // coefficient of x^i in P is C[L - i]
    if (C[L - i]) out[i / 64] |= 1ull << (i % 64);
}

// r ^= (a << sh) for a 256-bit a into a 512-bit r
static inline void xor_shifted(P512& r, const uint64_t a[4], int sh) {
  int ws = sh / 64, bs = sh % 64;
  for (int q = 0; q < 4; q++) {
    r.w[q + ws] ^= a[q] << bs;
    if (bs && q + ws + 1 < 8) r.w[q + ws + 1] ^= a[q] >> (64 - bs);
  }
}

static void polymulmod(const uint64_t a[4], const uint64_t b[4], const uint64_t p[4], uint64_t out[4]) {
  P512 r;
  std::memset(&r, 0, sizeof r);
  for (int i = 0; i < 256; i++)
    if ((a[i / 64] >> (i % 64)) & 1) xor_shifted(r, b, i);
  // reduce degrees 511..256 with x^256 = p(x)
  for (int d = 511; d >= 256; d--)
    if ((r.w[d / 64] >> (d % 64)) & 1) {
      r.w[d / 64] ^= 1ull << (d % 64);
      xor_shifted(r, p, d - 256);
    }
  std::memcpy(out, r.w, 4 * sizeof(uint64_t));
}

static const uint64_t* the_char_poly() {
  static uint64_t p[4];
  static bool have = [] { char_poly(p); return true; }();
  (void)have;
  return p;
}

JumpPoly xoshiro_jump_mul(const JumpPoly& a, const JumpPoly& b) {
  JumpPoly r;
  polymulmod(a.w, b.w, the_char_poly(), r.w);
  return r;
}

JumpPoly xoshiro_jump_poly(uint64_t n) {
  const uint64_t* p = the_char_poly();
  uint64_t result[4] = {1, 0, 0, 0};  // x^0
  uint64_t base[4] = {2, 0, 0, 0};    // x^1
  while (n) {
    if (n & 1) polymulmod(result, base, p, result);
    polymulmod(base, base, p, base);
    n >>= 1;
  }
  JumpPoly j;
  std::memcpy(j.w, result, sizeof j.w);
  return j;
}

void xoshiro_apply_jump(uint64_t s[4], const JumpPoly& p) {
  uint64_t acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < 256; i++) {
    if ((p.w[i / 64] >> (i % 64)) & 1)
      for (int q = 0; q < 4; q++) acc[q] ^= s[q];
    xoshiro_step(s);
  }
  std::memcpy(s, acc, sizeof acc);
}

bool qam_points(int m, std::vector<double>& pts, double& log_m) {
  int side = (int)std::lround(std::sqrt((double)m));
  if (m < 4 || (m & (m - 1)) || side * side != m || m > 256) return false;
  std::vector<double> lv(side), nre, nim;
  for (int i = 0; i < side; i++) lv[i] = 2.0 * (double)i - ((double)side - 1.0);
  for (int r = 0; r < side; r++)
    for (int t = 0; t < side; t++) {
      int tt = (r % 2 == 1) ? side - 1 - t : t;
      nre.push_back(lv[tt]);
      nim.push_back(lv[side - 1 - r]);
    }
  pts.assign(2 * m, 0.0);
  for (int i = 0; i < m; i++) {
    int g = i ^ (i >> 1);
    pts[2 * g] = nre[i];
    pts[2 * g + 1] = nim[i];
  }
  double e = 0.0;
  for (int i = 0; i < m; i++) e += pts[2 * i] * pts[2 * i] + pts[2 * i + 1] * pts[2 * i + 1];
  double s = 1.0 / std::sqrt(e / (double)m);
  for (double& v : pts) v *= s;
  log_m = std::log((double)m);
  return true;
}

GenTables gen_tables(int k_info, int e, int m, int bits_threads, int noise_threads) {
  GenTables g;
  g.mbits = __builtin_ctz(m);
  g.n_pad = (g.mbits - e % g.mbits) % g.mbits;
  int n_sym = (e + g.n_pad) / g.mbits;
  g.bits_per_chunk = (k_info + bits_threads - 1) / bits_threads;
  g.syms_per_chunk = (n_sym + noise_threads - 1) / noise_threads;
  g.jumps.assign((size_t)(bits_threads + noise_threads + 1) * 4, 0);
  JumpPoly step_b = xoshiro_jump_poly((uint64_t)g.bits_per_chunk), cur = xoshiro_jump_poly(0);
  for (int t = 0; t < bits_threads; t++) {
    std::memcpy(&g.jumps[(size_t)t * 4], cur.w, 32);
    cur = xoshiro_jump_mul(cur, step_b);
  }
  JumpPoly step_s = xoshiro_jump_poly(2ull * g.syms_per_chunk);
  cur = xoshiro_jump_poly((uint64_t)k_info + g.n_pad);
  for (int t = 0; t < noise_threads; t++) {
    std::memcpy(&g.jumps[(size_t)(bits_threads + t) * 4], cur.w, 32);
    cur = xoshiro_jump_mul(cur, step_s);
  }
  JumpPoly padp = xoshiro_jump_poly((uint64_t)k_info);
  std::memcpy(&g.jumps[(size_t)(bits_threads + noise_threads) * 4], padp.w, 32);
  return g;
}

}  // namespace cbh
