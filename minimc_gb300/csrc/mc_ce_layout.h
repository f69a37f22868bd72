// Layout of the continuous-energy tables shared by the host builder
// (mc_ce_tables.cpp, plain C++) and the device code (mc_ce.cuh).
#pragma once

#include <cstdint>

namespace mc {

constexpr int kCEMaxReactions = 4;

// One (particle type, nuclide) of Continuous (src/Continuous.hpp): the total
// evaluation and the reactions in input order (src/Continuous.cpp:74-86).
struct CENuclideDesc {
  int32_t present;                       // data exists for this particle type
  int32_t total;                         // table index of the total evaluation
  int32_t n_rx;                          // reactions (<= kCEMaxReactions)
  int32_t rx_kind[kCEMaxReactions];      // 0 capture, 1 scatter, 2 fission
  int32_t rx_table[kCEMaxReactions];     // table index of each reaction's evaluation
  int32_t rx_nubar[kCEMaxReactions];     // fission: nubar table, else -1
  int32_t rx_tsl[kCEMaxReactions];       // scatter: thermal scattering library, else -1
  int32_t pad;
  double awr;
  double total_T;                        // evaluation temperatures (K)
  double rx_T[kCEMaxReactions];
};

}  // namespace mc
