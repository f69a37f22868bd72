// Continuous-energy tables built on the host from the problem model.
//
// The reference evaluates every cross section by its own std::map
// (ContinuousMap::at, src/ContinuousMap.hpp:21-39): upper_bound over the
// table's energies, snap at both ends, linear interpolation.  The device
// replaces the per-table tree walks with one search of a unionized grid:
//
//   * union: every energy of every table, sorted and unique.  For an energy
//     E, j = upper_bound(union, E); for a table with energies x (all of them
//     in the union), upper_bound(x, E) = lower_bound(x, union[j]), which is
//     tabulated once per distinct energy axis in `umap`.  The search itself
//     starts from a bucket of the order-preserving integer key of E, so the
//     index equals the reference's bit for bit.
//   * exact tables: every table's own (x, y), interpolated on the device
//     with the reference's formula and rounding.
//   * FP32 union tables: each nuclide's reaction cross sections, its total
//     and each material's running sums evaluated at every union energy.  The
//     union holds every breakpoint of every table, so linear interpolation
//     between union points reproduces the same piecewise-linear functions,
//     rounded to FP32.  They are valid when no cross section depends on
//     temperature: every material cell has a constant temperature at which
//     every total and scatter evaluation is valid
//     (ContinuousEvaluation::IsValid, src/ContinuousEvaluation.cpp:17-20)
//     and no thermal scattering library applies.
#pragma once

#include "mc_ce_layout.h"
#include "mc_model.hpp"

#include <cstdint>
#include <vector>

namespace mc {

struct CETables {
  // unionized grid and its search buckets
  std::vector<double> union_e;
  std::vector<uint64_t> union_key;   // bit patterns of union_e (positive doubles)
  std::vector<uint32_t> bucket;      // [n_buckets + 1] first candidate index per bucket
  uint64_t key0 = 0;                 // key of union_e[0]
  int32_t shift = 0;                 // bucket = (key - key0) >> shift
  int32_t n_buckets = 0;
  // every table (total, reactions, nubar) of every (type, nuclide)
  std::vector<uint32_t> tab_off;     // [n_tables + 1]
  std::vector<int32_t> tab_grid;     // distinct energy axis of each table
  std::vector<double> tab_x, tab_y;
  std::vector<uint32_t> umap;        // [n_grids][n_union + 1]
  int32_t n_grids = 0;
  std::vector<CENuclideDesc> nuc;    // [2 types][n_nuclides]
  double max_nubar = 0;
  // FP32 union tables
  bool fast_ok = false;
  std::string fast_reason;           // why not, when not
  int32_t kmax = 1;                  // nuclides per material, padded row length
  std::vector<float> union_inv;      // [n_union] 1 / (e[j] - e[j-1]); [0] = 0
  std::vector<float> mat_flight;     // [2][M][n_union][2]: N * micro total, N * sum afrac nubar sigma_f
  std::vector<float> mat_ncdf;       // [2][M][n_union][kmax] running afrac * total
  std::vector<float> nuc_rx;         // [2][N][n_union][4] running reaction sums (input order, -1 past the last), total
  std::vector<float> nuc_nubar;      // [2][N][n_union]
};

// Builds the tables; throws std::runtime_error for inputs the device path
// does not cover (more than kCEMaxReactions reactions per nuclide).
CETables build_ce_tables(const Model& m);

// ContinuousMap::at on a table's (x, y) (the reference's arithmetic)
double table_at(const Table1D& t, double E);

}  // namespace mc
