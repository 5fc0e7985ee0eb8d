#include "sparse_host.h"

#include <algorithm>
#include <cstdint>

#include "xoshiro.h"

namespace cbh {

bool build_sparse_code(int n, int m, const int32_t* row_start, const int32_t* vars, SparseCode& out,
                       std::string& err) {
  if (n <= 0 || m <= 0) {
    err = "a matrix of " + std::to_string(m) + " x " + std::to_string(n);
    return false;
  }
  if (!row_start || !vars) {
    err = "null row offsets or variables";
    return false;
  }
  if (row_start[0] != 0) {
    err = "the row offsets must start at 0";
    return false;
  }
  for (int r = 0; r < m; r++)
    if (row_start[r + 1] < row_start[r]) {
      err = "the row offsets decrease at row " + std::to_string(r);
      return false;
    }
  const int edges = row_start[m];
  SparseCode c;
  c.n = n;
  c.m = m;
  c.edges = edges;
  c.row_start.assign(row_start, row_start + m + 1);
  c.vars.assign(vars, vars + edges);
  std::vector<int> mark(n, -1), deg(n, 0);
  for (int r = 0; r < m; r++) {
    const int d = row_start[r + 1] - row_start[r];
    c.max_row_degree = std::max(c.max_row_degree, d);
    for (int e = row_start[r]; e < row_start[r + 1]; e++) {
      const int v = vars[e];
      if (v < 0 || v >= n) {
        err = "check " + std::to_string(r) + " refers to the missing variable " + std::to_string(v);
        return false;
      }
      if (mark[v] == r) {
        err = "check " + std::to_string(r) + " lists variable " + std::to_string(v) + " twice";
        return false;
      }
      mark[v] = r;
      deg[v]++;
    }
  }
  // the edges of every variable, rows in increasing order
  c.col_start.assign(n + 1, 0);
  for (int v = 0; v < n; v++) {
    c.col_start[v + 1] = c.col_start[v] + deg[v];
    c.max_col_degree = std::max(c.max_col_degree, deg[v]);
  }
  c.col_edges.assign(edges, 0);
  std::vector<int> fill(c.col_start.begin(), c.col_start.end() - 1);
  for (int r = 0; r < m; r++)
    for (int e = row_start[r]; e < row_start[r + 1]; e++) c.col_edges[fill[vars[e]]++] = e;
  // levels
  std::vector<int> last(n, -1), level(m, 0);
  for (int r = 0; r < m; r++) {
    int lv = 0;
    for (int e = row_start[r]; e < row_start[r + 1]; e++) lv = std::max(lv, last[vars[e]] + 1);
    level[r] = lv;
    for (int e = row_start[r]; e < row_start[r + 1]; e++) last[vars[e]] = lv;
    c.levels = std::max(c.levels, lv + 1);
  }
  c.level_start.assign(c.levels + 1, 0);
  for (int r = 0; r < m; r++) c.level_start[level[r] + 1]++;
  for (int l = 0; l < c.levels; l++) {
    c.max_level_rows = std::max(c.max_level_rows, c.level_start[l + 1]);
    c.level_start[l + 1] += c.level_start[l];
  }
  c.level_rows.assign(m, 0);
  std::vector<int> lf(c.level_start.begin(), c.level_start.end() - 1);
  for (int r = 0; r < m; r++) c.level_rows[lf[level[r]]++] = r;
  out = std::move(c);
  return true;
}

bool reduce_sums(const SparseCode& code, SparseEncoder& out, std::string& err) {
  const int n = code.n, m = code.m;
  const size_t words = (size_t)(n + 63) / 64;
  // H as rows of 64-bit words; a repeated variable was rejected when the code was built
  std::vector<uint64_t> h((size_t)m * words, 0);
  for (int r = 0; r < m; r++)
    for (int e = code.row_start[r]; e < code.row_start[r + 1]; e++) {
      const int v = code.vars[e];
      h[r * words + v / 64] |= 1ull << (v % 64);
    }
  auto bit = [&](int r, int col) { return (h[r * words + col / 64] >> (col % 64)) & 1; };
  std::vector<int32_t> pivots;
  int lead = 0;
  for (int col = n - 1; col >= 0 && lead < m; col--) {
    int p = lead;
    while (p < m && !bit(p, col)) p++;
    if (p == m) continue;
    if (p != lead) std::swap_ranges(h.begin() + p * words, h.begin() + (p + 1) * words, h.begin() + lead * words);
    const uint64_t* src = &h[lead * words];
    for (int r = 0; r < m; r++)
      if (r != lead && bit(r, col)) {
        uint64_t* dst = &h[r * words];
        for (size_t w = 0; w < words; w++) dst[w] ^= src[w];
      }
    pivots.push_back(col);
    lead++;
  }
  std::vector<char> is_pivot(n, 0);
  for (int c : pivots) is_pivot[c] = 1;
  SparseEncoder enc;
  enc.kind = kEncoderSums;
  for (int v = 0; v < n; v++)
    if (!is_pivot[v]) enc.info.push_back(v);
  if (enc.info.empty()) {
    err = "the code has no information bits";
    return false;
  }
  enc.k = (int)enc.info.size();
  enc.pivots = pivots;
  enc.words = (enc.k + 31) / 32;
  const size_t rank = pivots.size();
  enc.pmat.assign((size_t)enc.words * rank, 0);
  for (size_t t = 0; t < rank; t++)
    for (int i = 0; i < enc.k; i++)
      if (bit((int)t, enc.info[i])) enc.pmat[(size_t)(i / 32) * rank + t] |= 1u << (i % 32);
  out = std::move(enc);
  return true;
}

bool check_accumulate(const SparseCode& code, SparseEncoder& out, std::string& err) {
  const int n = code.n, m = code.m;
  if (!(m > 0 && m < n)) {
    err = std::to_string(m) + " checks for " + std::to_string(n) + " bits";
    return false;
  }
  const int k = n - m;
  auto list = [](const std::vector<int32_t>& v) {
    std::string s = "[";
    for (size_t i = 0; i < v.size(); i++) s += (i ? ", " : "") + std::to_string(v[i]);
    return s + "]";
  };
  for (int r = 0; r < m; r++) {
    std::vector<int32_t> parity;
    for (int e = code.row_start[r]; e < code.row_start[r + 1]; e++)
      if (code.vars[e] >= k) parity.push_back(code.vars[e]);
    std::vector<int32_t> expected;
    if (r > 0) expected.push_back(k + r - 1);
    expected.push_back(k + r);
    std::vector<int32_t> sorted = parity;
    std::sort(sorted.begin(), sorted.end());
    if (sorted != expected) {
      err = "check " + std::to_string(r) + " is not dual-diagonal: parity bits " + list(parity) + ", expected " +
            list(expected);
      return false;
    }
  }
  SparseEncoder enc;
  enc.kind = kEncoderAccumulate;
  enc.k = k;
  enc.info.resize(k);
  for (int i = 0; i < k; i++) enc.info[i] = i;
  out = std::move(enc);
  return true;
}

namespace {

// the check of lowest degree among the candidates, the ties broken by one draw
int lowest_degree(const std::vector<int32_t>& cands, const std::vector<std::vector<int32_t>>& check_vars,
                  cbd::Xoshiro& rng) {
  size_t d = SIZE_MAX;
  for (int c : cands) d = std::min(d, check_vars[c].size());
  std::vector<int32_t> best;
  for (int c : cands)
    if (check_vars[c].size() == d) best.push_back(c);
  return best[cbd::xoshiro_below(rng, best.size())];
}

bool linked(const std::vector<int32_t>& checks, int c) {
  return std::find(checks.begin(), checks.end(), c) != checks.end();
}

// the candidates of a new edge of variable v: the checks the breadth-first expansion
// from v never reaches; when it reaches them all, those of its last level not linked to
// v yet (any check not linked to v when there are none)
std::vector<int32_t> farthest_checks(int v, const std::vector<std::vector<int32_t>>& check_vars,
                                     const std::vector<std::vector<int32_t>>& var_checks) {
  const int m = (int)check_vars.size();
  std::vector<char> reached(m, 0);
  std::vector<int32_t> frontier = var_checks[v];
  for (int c : frontier) reached[c] = 1;
  int n_reached = (int)frontier.size();  // the checks of a variable are distinct
  std::vector<int32_t> last_level = var_checks[v];
  for (;;) {
    std::vector<int32_t> level;
    for (int c : frontier)
      for (int u : check_vars[c])
        for (int c2 : var_checks[u])
          if (!reached[c2]) {
            reached[c2] = 1;
            n_reached++;
            level.push_back(c2);
          }
    if (level.empty() || n_reached == m) {
      std::vector<int32_t> out;
      for (int c = 0; c < m; c++)
        if (!reached[c]) out.push_back(c);
      if (!out.empty()) return out;
      for (int c : level.empty() ? last_level : level)
        if (!linked(var_checks[v], c)) out.push_back(c);
      if (out.empty())
        for (int c = 0; c < m; c++)
          if (!linked(var_checks[v], c)) out.push_back(c);
      return out;
    }
    last_level = level;
    frontier.swap(level);
  }
}

}  // namespace

bool peg_rows(int n, int k, int var_degree, uint64_t seed, std::vector<std::vector<int32_t>>& rows,
              std::string& err) {
  if (!(k < n && k > 0)) {
    err = "PEG needs 0 < k < n, got k = " + std::to_string(k) + ", n = " + std::to_string(n);
    return false;
  }
  const int m = n - k;
  if (!(var_degree >= 1 && var_degree <= m)) {
    err = "variable degree " + std::to_string(var_degree) + " for " + std::to_string(m) + " checks";
    return false;
  }
  cbd::Xoshiro rng = cbd::xoshiro_seed(seed);
  std::vector<std::vector<int32_t>> check_vars(m), var_checks(n);
  std::vector<int32_t> all(m);
  for (int c = 0; c < m; c++) all[c] = c;
  for (int v = 0; v < n; v++)
    for (int e = 0; e < var_degree; e++) {
      const int c = e == 0 ? lowest_degree(all, check_vars, rng)
                           : lowest_degree(farthest_checks(v, check_vars, var_checks), check_vars, rng);
      check_vars[c].push_back(v);
      var_checks[v].push_back(c);
    }
  rows = std::move(check_vars);
  return true;
}

int girth(const SparseCode& code) {
  const int n = code.n, m = code.m;
  std::vector<int32_t> edge_row(code.edges);
  for (int r = 0; r < m; r++)
    for (int e = code.row_start[r]; e < code.row_start[r + 1]; e++) edge_row[e] = r;
  // nodes: variables 0 .. n - 1, then checks n .. n + m - 1
  const int nodes = n + m;
  std::vector<int32_t> dist(nodes), parent(nodes), queue(nodes);
  long best = -1;
  for (int s = 0; s < n; s++) {
    std::fill(dist.begin(), dist.end(), -1);
    std::fill(parent.begin(), parent.end(), -1);
    dist[s] = 0;
    int head = 0, tail = 0;
    queue[tail++] = s;
    while (head < tail) {
      const int x = queue[head++];
      auto visit = [&](int y) {
        if (dist[y] < 0) {
          dist[y] = dist[x] + 1;
          parent[y] = x;
          queue[tail++] = y;
        } else if (parent[x] != y) {
          const long len = (long)dist[x] + dist[y] + 1;
          if (best < 0 || len < best) best = len;
        }
      };
      if (x < n) {
        for (int i = code.col_start[x]; i < code.col_start[x + 1]; i++) visit(n + edge_row[code.col_edges[i]]);
      } else {
        for (int e = code.row_start[x - n]; e < code.row_start[x - n + 1]; e++) visit(code.vars[e]);
      }
    }
  }
  return best < 0 ? 0 : (int)best;
}

}  // namespace cbh
