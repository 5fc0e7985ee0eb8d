// The device descriptor of a host-built NR code (host code shared by the ABI files).
#pragma once
#include <algorithm>
#include <cstring>
#include <vector>

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
  // levels of the base rows: one more than the highest level of an earlier row sharing
  // a column; rows of one level share no column, and every column meets its rows in
  // increasing order of levels
  {
    std::vector<int> last(h.cols_k + h.rows_n + 64, -1), level(h.rows_n, 0);
    int levels = 0;
    for (int L = 0; L < h.rows_n; L++) {
      int lv = 0;
      for (int t = h.layer_start[L]; t < h.layer_start[L + 1]; t++) lv = std::max(lv, last[h.entry_col[t]] + 1);
      level[L] = lv;
      for (int t = h.layer_start[L]; t < h.layer_start[L + 1]; t++) last[h.entry_col[t]] = lv;
      levels = std::max(levels, lv + 1);
    }
    int pos = 0;
    for (int lv = 0; lv < levels; lv++) {
      for (int L = 0; L < h.rows_n; L++)
        if (level[L] == lv) v.layer_order[pos++] = (uint8_t)L;
      v.level_end[pos - 1] = 1;
    }
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
