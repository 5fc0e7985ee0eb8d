// Host-side tables of a generic sparse LDPC code for the GPU decoder: the rows of the
// parity-check matrix, the edges of every variable in row order, and the level schedule
// that runs the layered decoder's rows in parallel without changing its results.
//
// Follows LdpcCode::from_rows / assemble (crates/com-fec/src/ldpc.rs:197-239): the
// messages of check c sit at edges start[c] .. start[c + 1], row after row, in the order
// of the row's variables.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cbh {

struct SparseCode {
  int n = 0, m = 0, edges = 0;
  int max_row_degree = 0, max_col_degree = 0;
  std::vector<int32_t> row_start;  // m + 1
  std::vector<int32_t> vars;       // edges: the variables of every row
  std::vector<int32_t> col_start;  // n + 1
  std::vector<int32_t> col_edges;  // edges: the edges of every variable, in increasing row order
  // Layered schedule.  The level of a row is one more than the highest level of an
  // earlier row sharing a variable with it (0 if none).  Rows of one level share no
  // variable, and the rows of every variable have increasing levels in row order, so
  // running the levels one after the other, the rows of a level at once, performs the
  // reference's sequential row order exactly.
  int levels = 0, max_level_rows = 0;
  std::vector<int32_t> level_start;  // levels + 1
  std::vector<int32_t> level_rows;   // m: the rows of every level, in increasing order
};

// Checks the rows (0 < n, 0 < m, offsets increasing from 0, variables in [0, n), no
// variable twice in a row) and builds the tables.
bool build_sparse_code(int n, int m, const int32_t* row_start, const int32_t* vars, SparseCode& out,
                       std::string& err);

}  // namespace cbh
