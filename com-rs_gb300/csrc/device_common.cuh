// Shared device-side pieces: the per-frame xoshiro256** streams, the code descriptor
// handed to every kernel, and the per-frame result record.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "code_host.h"
#include "xoshiro.h"

namespace cbd {

// ---------------------------------------------------------------- xoshiro256**
// Xoshiro, splitmix64, xoshiro_seed, stream and xoshiro_next are in xoshiro.h.

// state after n steps, n given by its jump polynomial x^n mod P(x)
__device__ __forceinline__ void xoshiro_jump(Xoshiro& r, const uint64_t* poly) {
  uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll 1
  for (int w = 0; w < 4; w++) {
    uint64_t bits = poly[w];
#pragma unroll 4
    for (int b = 0; b < 64; b++) {
      uint64_t mask = 0ull - ((bits >> b) & 1ull);
      a0 ^= r.s0 & mask;
      a1 ^= r.s1 & mask;
      a2 ^= r.s2 & mask;
      a3 ^= r.s3 & mask;
      xoshiro_advance(r);
    }
  }
  r.s0 = a0;
  r.s1 = a1;
  r.s2 = a2;
  r.s3 = a3;
}

// ---------------------------------------------------------------- code descriptor
struct DevCode {
  int32_t bg, z, cols_k, rows_n, n_full, k, k_info, e, qm;
  int32_t max_degree, n_entries, n_core_terms;
  int32_t map_is_offset, has_repeats;
  const int32_t* map;        // E positions (device), unused when map_is_offset
  const int32_t* inv_start;  // n_full + 1 (device), when !map_is_offset
  const int32_t* inv_t;      // E (device)
  uint16_t layer_start[cbh::kMaxLayers + 1];
  uint32_t entry[cbh::kMaxEntries];      // (base column << 16) | shift
  uint32_t core_term[cbh::kMaxCoreTerms];  // (block << 20) | (src << 16) | shift
  uint2 eaddr[cbh::kMaxEntries];           // {4 (column Z + shift), Z - shift}
  // the layered schedule by levels: the layers in the order the decoder runs them, and a
  // flag per position set when a barrier follows it (layers between two barriers share
  // no column, so their lifted rows run at once with the sequential order's results)
  uint8_t layer_order[cbh::kMaxLayers];
  uint8_t level_end[cbh::kMaxLayers];
};

// decoder settings (crates/com-fec/src/ldpc.rs:165-172)
enum RuleId { RULE_SUM_PRODUCT = 0, RULE_NMS = 1, RULE_OMS = 2 };
struct DecCfg {
  int32_t rule;
  int32_t max_iterations;
  int32_t layered;
  double alpha;  // scale of the NMS or offset of the OMS
};

// per-frame result record: bit errors, frame error, iterations
struct FrameResult {
  uint32_t bit_errors;
  uint8_t frame_error;
  uint8_t iterations;
  uint16_t reserved;
};

constexpr float kKnownBitLlr = 30.0f;  // KNOWN_BIT_LLR, crates/com-core/src/signal.rs:37

}  // namespace cbd
