// minimc_gb300_driver.hpp -- the GB300 engine as minimc Driver subclasses.
//
// Reference-side glue, compiled inside the reference's tree (it includes
// the reference's Driver.hpp, src/Driver.hpp:17-50): minimc's per-particle
// TransportMethod::Transport (src/TransportMethod.hpp:42-43) cannot be
// batched, so the engine drops in where Driver::Solve (src/Driver.hpp:30)
// runs every history.  GpuFixedSource and GpuKEigenvalue are built from the
// same XML root as FixedSource / KEigenvalue (the Driver base builds the
// World, estimators and Particle::transport_method on the CPU as before),
// load the problem into an engine context, and run it through the C ABI
// (minimc_gb300.h).  CreateGpuDriver mirrors Driver::Create
// (src/Driver.cpp:18-35).
//
// The reference's EstimatorSet keeps its scores private, so Solve returns
// the initial estimator set and the run's per-bin sums stay with the
// driver: Sums() / SumsSquared() in mc_estimator_info order, and
// ResultText() gives the reference's own result-file text for them
// (batch size line, then EstimatorSet::to_string; src/minimc.cpp:20-21).
// Link with -lminimc_gb300.
#ifndef MINIMC_GB300_DRIVER_HPP
#define MINIMC_GB300_DRIVER_HPP

#include "Driver.hpp"
#include "XMLDocument.hpp"
#include "minimc_gb300.h"
#include "pugixml.hpp"

#include <filesystem>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace minimc_gb300 {

// an engine context holding one problem; errors become exceptions with the
// engine's message (the reference's exception text where it has one)
class EngineProblem {
public:
  EngineProblem(const std::string& xml_text, const std::string& base_dir, int device) {
    if (mc_create(&ctx_, device) != MC_OK) throw std::runtime_error("minimc_gb300: no usable CUDA device");
    Check(mc_load_xml(ctx_, xml_text.c_str(), base_dir.c_str()));
    Check(mc_problem_info_get(ctx_, &info_));
  }
  ~EngineProblem() { mc_destroy(ctx_); }
  EngineProblem(const EngineProblem&) = delete;
  EngineProblem& operator=(const EngineProblem&) = delete;

  void Check(int rc) const {
    if (rc == MC_OK) return;
    char msg[2048] = {0};
    mc_last_error(ctx_, msg, sizeof msg);
    throw std::runtime_error(msg);
  }
  mc_ctx* ctx() const { return ctx_; }
  const mc_problem_info& info() const { return info_; }

  // the result file text for sums normalised by total_weight
  std::string Text(const std::vector<double>& sum, const std::vector<double>& sq, double total_weight) const {
    size_t need = 0;
    Check(mc_output_text(ctx_, sum.data(), sq.data(), info_.histories, total_weight, nullptr, 0, &need));
    std::string s(need + 1, '\0');
    Check(mc_output_text(ctx_, sum.data(), sq.data(), info_.histories, total_weight, s.data(), s.size(), &need));
    s.resize(need);
    return s;
  }

private:
  mc_ctx* ctx_{nullptr};
  mc_problem_info info_{};
};

inline std::string ReadText(const std::filesystem::path& p) {
  std::ifstream f(p);
  if (!f) throw std::runtime_error("cannot read " + p.string());
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

// FixedSource::Solve (src/FixedSource.cpp:22-77) on the GPU
class GpuFixedSource : public Driver {
public:
  GpuFixedSource(const pugi::xml_node& root, const std::string& xml_text, const std::string& base_dir,
                 int device = 0)
      : Driver{root}, engine_{xml_text, base_dir, device} {}
  EstimatorSet Solve() override {
    const size_t nb = engine_.info().total_bins;
    sum_.assign(nb, 0.0);
    sq_.assign(nb, 0.0);
    mc_tally_out out{};
    out.sum = sum_.data();
    out.sum_sq = sq_.data();
    mc_run_opts opts{};  // histories and seed from the problem
    engine_.Check(mc_run_fixed_source(engine_.ctx(), &opts, &out));
    return init_estimator_set;
  }
  const std::vector<double>& Sums() const { return sum_; }
  const std::vector<double>& SumsSquared() const { return sq_; }
  std::string ResultText() const { return engine_.Text(sum_, sq_, static_cast<double>(batchsize)); }

private:
  EngineProblem engine_;
  std::vector<double> sum_, sq_;
};

// KEigenvalue::Solve (src/KEigenvalue.cpp:36-84, a stub in the reference)
// on the GPU: k per cycle, its mean and standard error over the active
// cycles, tallies over the active cycles
class GpuKEigenvalue : public Driver {
public:
  GpuKEigenvalue(const pugi::xml_node& root, const std::string& xml_text, const std::string& base_dir,
                 int device = 0)
      : Driver{root}, engine_{xml_text, base_dir, device} {}
  EstimatorSet Solve() override {
    const mc_problem_info& info = engine_.info();
    k_cycle_.assign(info.inactive + info.active, 0.0);
    sum_.assign(info.total_bins, 0.0);
    sq_.assign(info.total_bins, 0.0);
    mc_keig_out out{};
    out.k_cycle = k_cycle_.data();
    out.sum = sum_.data();
    out.sum_sq = sq_.data();
    mc_run_opts opts{};
    engine_.Check(mc_run_keigenvalue(engine_.ctx(), &opts, &out));
    k_mean_ = out.k_mean;
    k_std_ = out.k_std;
    return init_estimator_set;
  }
  const std::vector<double>& KPerCycle() const { return k_cycle_; }
  double KMean() const { return k_mean_; }
  double KStd() const { return k_std_; }
  const std::vector<double>& Sums() const { return sum_; }
  std::string ResultText() const {
    return engine_.Text(sum_, sq_, static_cast<double>(batchsize) * engine_.info().active);
  }

private:
  EngineProblem engine_;
  std::vector<double> k_cycle_, sum_, sq_;
  double k_mean_{0}, k_std_{0};
};

// Driver::Create (src/Driver.cpp:18-35) with the engine: the problem type
// selects the driver; data files resolve against the input's directory
inline std::unique_ptr<Driver> CreateGpuDriver(const std::filesystem::path& xml_filepath, int device = 0) {
  const std::string text = ReadText(xml_filepath);
  const std::string dir = xml_filepath.has_parent_path() ? xml_filepath.parent_path().string() : std::string();
  auto doc = std::make_unique<XMLDocument>(xml_filepath);
  const std::string problem_type = doc->root.child("problemtype").first_child().name();
  if (problem_type == "fixedsource") return std::make_unique<GpuFixedSource>(doc->root, text, dir, device);
  if (problem_type == "keigenvalue") return std::make_unique<GpuKEigenvalue>(doc->root, text, dir, device);
  throw std::runtime_error("unknown problem type: " + problem_type);
}

}  // namespace minimc_gb300

#endif  // MINIMC_GB300_DRIVER_HPP
