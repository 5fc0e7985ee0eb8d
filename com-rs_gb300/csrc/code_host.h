// Host-side construction of a 5G NR LDPC code for the GPU kernels.
//
// Builds, once per code, everything the kernels read: the base-graph entries of every
// layer with their shifts reduced mod Z, the circulant terms of the inverse of the core
// block (the encoder), the rate-matching positions and the xoshiro256** jump
// polynomials that let many threads draw one frame's stream in parallel.
//
// Follows NrLdpc::with_options (crates/com-fec/src/nr/ldpc.rs:101-162) and
// LdpcCode::from_core_rows (crates/com-fec/src/ldpc.rs:270-287); the explicit lifting
// size composes the same steps for a given Z (the K' = 10 Z base-graph-2 codes).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace cbh {

constexpr int kMaxLayers = 46;
constexpr int kMaxEntries = 316;
constexpr int kMaxCoreTerms = 64;

struct CodeSpec {
  int k_info = 0, e = 0;
  int bg = 0;  // 0: TS 38.212 Sec. 7.2.2 rule
  int z = 0;   // 0: the smallest lifting size with kb Z >= K'
  int rv = 0, qm = 1;
};

// One circulant term of the core inverse: parity block `block`, bit r, sums the core
// syndrome block `src` at bit (r + shift) mod Z.
struct CoreTerm {
  uint16_t block, src, shift;
};

struct NrCode {
  int bg = 0, z = 0, ils = 0;
  int cols_k = 0, rows_n = 0;  // systematic base columns (22/10), base rows (46/42)
  int k = 0, n_full = 0, k_info = 0, e = 0, rv = 0, qm = 1;
  int ncb = 0, k0 = 0;
  int max_degree = 0, edges = 0;
  // layers in base-row order: entries layer_start[i] .. layer_start[i+1]
  std::vector<int> layer_start;
  std::vector<uint16_t> entry_col;    // base column j
  std::vector<uint16_t> entry_shift;  // V mod Z
  std::vector<CoreTerm> core_terms;   // sorted by block
  // rate matching: output bit t carries full-word bit map[t]
  std::vector<int32_t> map;
  bool map_is_offset = false;         // map[t] == 2Z + t for every t
  // inverse of the map for the LLR scatter: for full bit v, the t's in increasing order
  std::vector<int32_t> inv_start, inv_t;
  bool has_repeats = false;
};

bool build_nr_code(const CodeSpec& spec, NrCode& out, std::string& err);

// xoshiro256** jump-ahead: the polynomial x^n mod P(x), P the characteristic
// polynomial of the generator's linear state transition (256 coefficients).
struct JumpPoly {
  uint64_t w[4];
};
JumpPoly xoshiro_jump_poly(uint64_t n);
// the polynomial of the jump a + b from those of a and b
JumpPoly xoshiro_jump_mul(const JumpPoly& a, const JumpPoly& b);
// applies a jump polynomial to a state (host copy of the device routine, for tests)
void xoshiro_apply_jump(uint64_t s[4], const JumpPoly& p);

// Gray square QAM of order m, unit average energy: 2m doubles (re, im) by label, and
// ln m (crates/com-mapping/src/constellation.rs:168-202, :396; demapper.rs:279)
bool qam_points(int m, std::vector<double>& pts, double& log_m);

// The frame generator's chunking of one frame's draws over `threads` threads and the
// jump polynomials of the chunk starts: [threads] info-bit chunks, [threads] symbol
// chunks, then the padding bits (4 words each).
struct GenTables {
  int mbits = 0, n_pad = 0, bits_per_chunk = 0, syms_per_chunk = 0;
  std::vector<uint64_t> jumps;
};
// Chunks of a frame's draws: the K' information bits over `bits_threads` threads, the
// noise symbols over `noise_threads`; jumps holds the jump polynomials of the bit chunks'
// starts, then of the noise chunks' starts, then of the padding bits' start (after the
// information bits).
GenTables gen_tables(int k_info, int e, int m, int bits_threads, int noise_threads);

}  // namespace cbh
