// minimc's result file (.out): the batch size line followed by
// EstimatorSet::to_string (src/minimc.cpp:20-21, src/Estimator.cpp:48-56,
// 207-213, src/Scorable.cpp:51-70, src/Bins.cpp:84-170,
// src/Sensitivity.cpp:25-28).
#pragma once

#include "mc_model.hpp"

#include <string>

namespace mc {

// Text of the result file for per-bin score sums and sums of squares (in
// estimator order, as the engine returns them) normalised by total_weight
// (the batch size).
std::string format_output(const Model& m, const double* sum, const double* sum_sq, double total_weight,
                          unsigned long long batchsize);

}  // namespace mc
