// Result-file text in minimc's format (see mc_output.hpp for the reference
// functions).  Numbers use the C library's "%e" conversion, which is what
// iostream's std::scientific at the default precision produces.
#include "mc_output.hpp"

#include <cmath>
#include <cstdio>

namespace mc {

namespace {

void sci(std::string& out, double v) {
  char buf[64];
  std::snprintf(buf, sizeof buf, "%e, ", v);
  out += buf;
}

// Bins::to_string of one dimension
std::string bins_text(const Bins1D& b) {
  std::string s;
  switch (b.kind) {
  case kLinspace:
    // LinspaceBins: lower + i * width for i < n_bins - 1
    for (uint64_t i = 0; i + 1 < b.n_bins; i++) sci(s, b.lower + static_cast<double>(i) * b.width);
    return s;
  case kLogspace:
    for (uint64_t i = 0; i + 1 < b.n_bins; i++)
      sci(s, std::pow(b.base, b.log_lower + static_cast<double>(i) * b.log_width));
    return s;
  case kBoundaries:
    for (double v : b.boundaries) sci(s, v);
    return s;
  default:
    return "none";
  }
}

// Scorable::GetScoreAsString
std::string score_text(const double* sum, const double* sum_sq, size_t n, double total_weight) {
  std::string t = "mean\n----\n";
  for (size_t i = 0; i < n; i++) sci(t, sum[i] / total_weight);
  t += "\n\n";
  t += "std dev\n-------\n";
  for (size_t i = 0; i < n; i++) sci(t, std::sqrt(sum_sq[i] - sum[i] * sum[i] / total_weight) / total_weight);
  t += "\n\n";
  return t;
}

}  // namespace

std::string format_output(const Model& m, const double* sum, const double* sum_sq, double total_weight,
                          unsigned long long batchsize) {
  std::string out = std::to_string(batchsize) + "\n";
  size_t off = 0;
  for (const Estimator& e : m.estimators) {
    std::string t = e.name + "\n" + std::string(e.name.size(), '=') + "\n\n";
    // ParticleBins::to_string
    t += "cosine\n------\n" + bins_text(e.cosine) + "\n\n";
    t += "energy\n------\n" + bins_text(e.energy) + "\n\n";
    const size_t n = e.size();
    t += score_text(sum + off, sum_sq + off, n, total_weight);
    off += n;
    // Sensitivity::to_string (src/Sensitivity.cpp:25-28): name
    // "<estimator>::<perturbation>" (src/Scorable.cpp:22-29)
    for (int32_t k : e.sensitivities) {
      const std::string name = e.name + "::" + m.perturbations[static_cast<size_t>(k)].name;
      t += name + "\n" + std::string(name.size(), '=') + "\n\n" + score_text(sum + off, sum_sq + off, n, total_weight) +
           "\n";
      off += n;
    }
    out += "\n" + t + "\n";
  }
  return out;
}

}  // namespace mc
