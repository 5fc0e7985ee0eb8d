// The device descriptor of a host-built NR code (host code shared by the ABI files).
#pragma once
#include <cstring>

#include "code_host.h"
#include "device_common.cuh"

namespace cbk {

// every field but the device pointers of the rate-matching tables
inline void fill_dev_code(const cbh::NrCode& h, cbd::DevCode& v) {
  std::memset(&v, 0, sizeof v);
  v.bg = h.bg;
  v.z = h.z;
  v.cols_k = h.cols_k;
  v.rows_n = h.rows_n;
  v.n_full = h.n_full;
  v.k = h.k;
  v.k_info = h.k_info;
  v.e = h.e;
  v.qm = h.qm;
  v.max_degree = h.max_degree;
  v.n_entries = (int)h.entry_col.size();
  v.n_core_terms = (int)h.core_terms.size();
  v.map_is_offset = h.map_is_offset;
  v.has_repeats = h.has_repeats;
  for (int i = 0; i <= h.rows_n; i++) v.layer_start[i] = (uint16_t)h.layer_start[i];
  for (int t = 0; t < v.n_entries; t++) {
    v.entry[t] = ((uint32_t)h.entry_col[t] << 16) | h.entry_shift[t];
    v.eaddr[t].x = 4u * ((uint32_t)h.entry_col[t] * (uint32_t)h.z + h.entry_shift[t]);
    v.eaddr[t].y = (uint32_t)h.z - h.entry_shift[t];
  }
  for (int t = 0; t < v.n_core_terms; t++)
    v.core_term[t] = ((uint32_t)h.core_terms[t].block << 20) | ((uint32_t)h.core_terms[t].src << 16) |
                     h.core_terms[t].shift;
}

// the row degrees the decoders are compiled for (3..10 and 19)
inline bool degrees_supported(const cbh::NrCode& h) {
  for (int L = 0; L < h.rows_n; L++) {
    int deg = h.layer_start[L + 1] - h.layer_start[L];
    if (!((deg >= 3 && deg <= 10) || deg == 19)) return false;
  }
  return true;
}

}  // namespace cbk
