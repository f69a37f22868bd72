// C entry points around the reference's own driver, for comparing the
// oracle (and through it the GPU engine) with the reference's code.
// TEST INFRASTRUCTURE ONLY.
#include "CSGSurface.hpp"
#include "Cell.hpp"
#include "Driver.hpp"
#include "FixedSource.hpp"
#include "Estimator.hpp"
#include "Material.hpp"
#include "Nuclide.hpp"
#include "Particle.hpp"
#include "Source.hpp"
#include "World.hpp"
#include "XMLDocument.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>
#include <stdexcept>
#include <exception>
#include <iostream>
#include <sstream>
#include <streambuf>
#include <string>

namespace {
void copy_message(const std::exception& e, char* err, size_t errn) {
  if (err && errn) {
    std::strncpy(err, e.what(), errn - 1);
    err[errn - 1] = 0;
  }
}
// Discards everything written to it.  It keeps no buffer or other state,
// so the reference's worker threads may report progress through it at the
// same time (a string stream in its place is a data race).
class NullBuf : public std::streambuf {
 protected:
  int overflow(int c) override { return traits_type::not_eof(c); }
  std::streamsize xsputn(const char*, std::streamsize n) override { return n; }
};

// FixedSource with its World visible, constructed exactly as
// Driver::Create does (document first, then the driver)
struct ProbedFixedSource : FixedSource {
  using FixedSource::FixedSource;
  const World& the_world() const { return world; }
};

// the iteration orders of the World, one line per cell:
// "cell: surface,surface,... | nuclide,nuclide,..." (std::map keyed by
// shared_ptr: allocation order in this process)
std::string world_orders(const World& world) {
  std::string s;
  for (const Cell& c : world.cells) {
    s += c.name + ":";
    for (const auto& [surf, sense] : c.surface_senses) s += " " + surf->name;
    s += " |";
    if (c.material)
      for (const auto& [nuc, afrac] : c.material->afracs) s += " " + nuc->name;
    s += "\n";
  }
  return s;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): the counter-based
// generator the k-eigenvalue loop resamples the next source with
void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c[0];
    const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c[2];
    const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    c[0] = hi1 ^ c[1] ^ k0;
    c[1] = lo1;
    c[2] = hi0 ^ c[3] ^ k1;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// The reference's KEigenvalue::Solve is a stub (src/KEigenvalue.cpp:36-62).
// This driver completes it with the reference's own objects only: the
// Driver constructor builds the World, the estimators and
// Particle::transport_method (src/Driver.cpp:37-52); cycle 0 starts from
// Source::Sample(1..N) of <initialsource> as the KEigenvalue constructor
// does (src/KEigenvalue.cpp:31-33); each source particle runs
// Particle::Transport (src/Particle.cpp:42-44) and hands its fission
// secondaries over with Particle::MoveSecondariesTo (src/Particle.cpp:
// 102-104); the cycle's bank is the histories' secondaries in source order,
// k = M / N, and the next N sources are drawn uniformly from the bank with
// a Philox stream keyed by (seed, cycle) -- the loop the engine and the
// CPU restatement run, so all three can be compared cycle by cycle.
// Source j of cycle c > 0 is seeded with seed + c N + j.  Scores of active
// cycles are committed per history (ScorableProxy::CommitHistory), each
// worker thread with its own EstimatorSet, merged at the end.
// One guard the reference's transport lacks: a source site in a void cell
// (a fission site banked by a particle that grazed a surface, failed to
// cross under the fixed nudge and collided beyond it) would make
// SurfaceTracking::Transport dereference the void's null material
// (src/TransportMethod.cpp:58-59), so such a particle is counted as lost
// and banks nothing -- what the CPU restatement and the engine do.
struct KeigHarness : Driver {
  explicit KeigHarness(const pugi::xml_node& root)
      : Driver{root}, source{root.child("problemtype").child("keigenvalue").child("initialsource")} {}
  EstimatorSet Solve() override { return init_estimator_set; }

  struct Site {
    Point pos;
    Direction dir;
    Energy energy;
  };

  // Philox key of a cycle's resampling: splitmix64 of seed, cycle and a salt
  uint64_t key_of(uint32_t cycle) const {
    return splitmix64(static_cast<uint64_t>(seed) * 0x9E3779B97F4A7C15ull +
                      static_cast<uint64_t>(cycle) * 0xD1B54A32D192ED03ull + 0x52455341ull);
  }
  const World& the_world() const { return world; }

  int run(uint32_t inactive, uint32_t active, int nthreads, double* k_cycle, uint64_t* bank_size,
          std::unique_ptr<EstimatorSet>& result, double* seconds, uint64_t* lost_out) {
    std::atomic<uint64_t> lost{0};
    const uint64_t N = batchsize;
    nthreads = std::max(1, nthreads);
    std::vector<Site> src;
    std::vector<std::vector<Site>> per_hist(N);
    std::vector<EstimatorSet> est(nthreads, init_estimator_set);
    const auto t0 = std::chrono::steady_clock::now();
    for (uint32_t c = 0; c < inactive + active; c++) {
      const bool act = c >= inactive;
      std::atomic<uint64_t> next{0};
      auto worker = [&](int t) {
        for (uint64_t j; (j = next++) < N;) {
          std::vector<Site>& v = per_hist[j];
          v.clear();
          if (!world.FindCellContaining(c == 0 ? source.Sample(static_cast<RNG::result_type>(j + 1)).GetPosition()
                                               : src[j].pos)
                   .material) {
            lost++;
            continue;
          }
          Particle p = c == 0 ? source.Sample(static_cast<RNG::result_type>(j + 1))
                              : Particle{src[j].pos, src[j].dir, src[j].energy, Particle::Type::neutron,
                                         static_cast<RNG::result_type>(seed + static_cast<uint64_t>(c) * N + j)};
          auto proxy = est[t].GetProxy();
          p.Transport(proxy, world);
          Bank b;
          p.MoveSecondariesTo(b);
          while (!b.empty()) {  // the bank's back is the last secondary banked
            const Particle& q = b.back();
            v.push_back({q.GetPosition(), q.GetDirection(), q.GetEnergy()});
            b.pop_back();
          }
          std::reverse(v.begin(), v.end());
          if (act) proxy.CommitHistory();
        }
      };
      std::vector<std::thread> pool;
      for (int t = 1; t < nthreads; t++) pool.emplace_back(worker, t);
      worker(0);
      for (auto& th : pool) th.join();
      std::vector<Site> bank;
      for (uint64_t j = 0; j < N; j++) bank.insert(bank.end(), per_hist[j].begin(), per_hist[j].end());
      const uint64_t M = bank.size();
      if (k_cycle) k_cycle[c] = static_cast<double>(M) / static_cast<double>(N);
      if (bank_size) bank_size[c] = M;
      if (M == 0) return -2;
      const uint64_t key = key_of(c);
      src.clear();
      src.reserve(N);
      for (uint64_t j = 0; j < N; j++) {
        uint32_t ctr[4] = {static_cast<uint32_t>(j), static_cast<uint32_t>(j >> 32), 0x72657361u, 0};
        philox4x32_10(ctr, static_cast<uint32_t>(key), static_cast<uint32_t>(key >> 32));
        const double u = ((ctr[0] >> 5) * 67108864.0 + (ctr[1] >> 6)) * (1.0 / 9007199254740992.0);
        uint64_t idx = static_cast<uint64_t>(u * static_cast<double>(M));
        if (idx >= M) idx = M - 1;
        src.push_back(bank[idx]);
      }
    }
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (lost_out) *lost_out = lost;
    result = std::make_unique<EstimatorSet>(init_estimator_set);
    for (const auto& e : est) *result += e;
    return 0;
  }

  Source source;
};

}  // namespace

extern "C" {

// Fixed source: FixedSource(root).Solve() as Driver::Create and minimc's
// main run it; the named estimator's bin means (Scorable::GetScore(i,
// batchsize), src/Scorable.cpp:32-35) in mean[nbins] and the World's
// iteration orders of this run in orders
int ref_solve(const char* xml_path, const char* estimator, uint64_t nbins, double* mean, char* orders,
              size_t ordersn, char* text, size_t textn, char* err, size_t errn) {
  // the reference reports progress on stdout; keep the caller's output clean
  std::streambuf* saved = std::cout.rdbuf();
  NullBuf sink;
  std::cout.rdbuf(&sink);
  int rc = 0;
  try {
    std::unique_ptr<ProbedFixedSource> driver;
    {
      auto doc = std::make_unique<XMLDocument>(xml_path);
      const std::string problem_type = doc->root.child("problemtype").first_child().name();
      if (problem_type != "fixedsource") throw std::runtime_error("fixed-source problems only");
      driver = std::make_unique<ProbedFixedSource>(doc->root);
    }
    if (orders && ordersn) {
      const std::string s = world_orders(driver->the_world());
      std::strncpy(orders, s.c_str(), ordersn - 1);
      orders[ordersn - 1] = 0;
    }
    const EstimatorSet result = driver->Solve();
    if (text && textn) {
      // the result file as minimc's main writes it (src/minimc.cpp:20-21)
      std::ostringstream os;
      os << driver->batchsize << std::endl;
      os << result.to_string();
      const std::string t = os.str();
      std::strncpy(text, t.c_str(), textn - 1);
      text[textn - 1] = 0;
    }
    if (estimator && estimator[0]) {
      const Estimator& e = result.FindEstimatorByName(estimator);
      for (uint64_t i = 0; i < nbins; i++) mean[i] = e.GetScore(i, static_cast<Real>(driver->batchsize));
    }
  }
  catch (const std::exception& e) {
    copy_message(e, err, errn);
    rc = -1;
  }
  std::cout.rdbuf(saved);
  return rc;
}

// k-eigenvalue over the reference's own transport (KeigHarness above):
// k per cycle and bank sizes in k_cycle / bank_size [inactive + active]; the
// named estimator's bin means over the active histories
// (Scorable::GetScore(i, N * active)) in mean[nbins]; the transport's
// wall-clock in *seconds; source particles found in a void in *lost; the
// World's iteration orders in orders
int ref_keig(const char* xml_path, uint32_t inactive, uint32_t active, int threads, double* k_cycle,
             uint64_t* bank_size, const char* estimator, uint64_t nbins, double* mean, double* seconds,
             uint64_t* lost, char* orders, size_t ordersn, char* err, size_t errn) {
  std::streambuf* saved = std::cout.rdbuf();
  NullBuf sink;
  std::cout.rdbuf(&sink);
  int rc = 0;
  try {
    std::unique_ptr<KeigHarness> driver;
    {
      auto doc = std::make_unique<XMLDocument>(xml_path);
      const std::string problem_type = doc->root.child("problemtype").first_child().name();
      if (problem_type != "keigenvalue") throw std::runtime_error("k-eigenvalue problems only");
      driver = std::make_unique<KeigHarness>(doc->root);
    }
    if (orders && ordersn) {
      const std::string s = world_orders(driver->the_world());
      std::strncpy(orders, s.c_str(), ordersn - 1);
      orders[ordersn - 1] = 0;
    }
    std::unique_ptr<EstimatorSet> result;
    rc = driver->run(inactive, active, threads, k_cycle, bank_size, result, seconds, lost);
    if (rc == 0 && estimator && estimator[0]) {
      const Estimator& e = result->FindEstimatorByName(estimator);
      const Real w = static_cast<Real>(driver->batchsize) * static_cast<Real>(active);
      for (uint64_t i = 0; i < nbins; i++) mean[i] = e.GetScore(i, w);
    }
  }
  catch (const std::exception& e) {
    copy_message(e, err, errn);
    rc = -1;
  }
  std::cout.rdbuf(saved);
  return rc;
}

}  // extern "C"
