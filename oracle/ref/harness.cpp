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
#include "World.hpp"
#include "XMLDocument.hpp"

#include <cstdint>
#include <cstring>
#include <memory>
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

}  // extern "C"
