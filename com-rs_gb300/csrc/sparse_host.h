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

// The systematic encoder of a code: the information positions and how the parity bits
// follow from the information bits.
enum EncoderKind { kEncoderNone = -1, kEncoderSums = 0, kEncoderAccumulate = 1 };

struct SparseEncoder {
  int kind = kEncoderNone;
  int k = 0;
  std::vector<int32_t> info;    // k increasing positions: information bit i sits at info[i]
  std::vector<int32_t> pivots;  // sums: the parity position of every leading row of the reduced H
  int words = 0;                // sums: 32-bit words of a packed information word
  // sums, words x pivots, word-major: bit b of word (w, t) is set when parity bit t sums
  // information bit 32 w + b
  std::vector<uint32_t> pmat;
};

// LdpcCode::from_rows (crates/com-fec/src/ldpc.rs:216-231): the reduced row echelon
// form of H with the pivots searched from the last column to the first
// (crates/com-math/src/gf2.rs:121-150); the information bits are the columns without a
// pivot, and the parity bit of every leading row is the sum of the information bits
// that row keeps.  False for a code without information bits.
bool reduce_sums(const SparseCode& code, SparseEncoder& out, std::string& err);

// LdpcCode::accumulate (ldpc.rs:233-256): an irregular repeat-accumulate code, check r
// holding information bits (below k = n - m) and the parity bits k + r and, for r > 0,
// k + r - 1 only.  False, with the reference's message, for another structure.
bool check_accumulate(const SparseCode& code, SparseEncoder& out, std::string& err);

// LdpcCode::peg (ldpc.rs:289-313, :586-634): progressive edge growth of a code of n
// variables and n - k checks, every variable of degree var_degree, the ties broken by
// Rng::new(seed).below.  rows[c] lists the variables of check c in the order they were
// linked.  False, with the reference's message, for invalid sizes.
bool peg_rows(int n, int k, int var_degree, uint64_t seed, std::vector<std::vector<int32_t>>& rows,
              std::string& err);

// LdpcCode::girth (ldpc.rs:412-446): the length of the shortest cycle of the Tanner
// graph by a breadth-first search from every variable; 0 without cycle.
int girth(const SparseCode& code);

}  // namespace cbh
