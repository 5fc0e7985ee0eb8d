#include "sparse_host.h"

#include <algorithm>

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

}  // namespace cbh
