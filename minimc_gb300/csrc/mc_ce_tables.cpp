// Continuous-energy table builder (layout and rationale in mc_ce_tables.hpp).
#include "mc_ce_tables.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <stdexcept>

namespace mc {

namespace {

uint64_t key_of(double e) {
  uint64_t k;
  std::memcpy(&k, &e, sizeof k);
  return k;
}

}  // namespace

double table_at(const Table1D& t, double E) {
  const size_t hi = static_cast<size_t>(std::upper_bound(t.x.begin(), t.x.end(), E) - t.x.begin());
  if (hi == t.x.size()) return t.y.back();
  if (hi == 0) return t.y.front();
  const double k_hi = t.x[hi], v_hi = t.y[hi], k_lo = t.x[hi - 1], v_lo = t.y[hi - 1];
  return v_lo + (v_hi - v_lo) / (k_hi - k_lo) * (E - k_lo);
}

CETables build_ce_tables(const Model& m) {
  CETables c;
  const size_t N = m.nuclides.size(), M = m.materials.size(), T = 2;
  c.nuc.assign(T * N, CENuclideDesc{});

  // ---- every table, with its distinct energy axis
  std::vector<const Table1D*> tabs;
  std::map<std::vector<double>, int32_t> grid_id;
  std::vector<const std::vector<double>*> grids;
  auto add_table = [&](const Table1D& t) -> int32_t {
    if (t.x.empty()) throw std::runtime_error("continuous-energy table without entries");
    auto it = grid_id.find(t.x);
    int32_t g;
    if (it == grid_id.end()) {
      g = static_cast<int32_t>(grids.size());
      grid_id.emplace(t.x, g);
      grids.push_back(&t.x);
    }
    else {
      g = it->second;
    }
    c.tab_grid.push_back(g);
    tabs.push_back(&t);
    return static_cast<int32_t>(tabs.size() - 1);
  };
  for (size_t t = 0; t < T; t++) {
    for (size_t n = 0; n < N; n++) {
      const Nuclide& nuc = m.nuclides[n];
      CENuclideDesc& d = c.nuc[t * N + n];
      for (int k = 0; k < kCEMaxReactions; k++) {
        d.rx_kind[k] = -1;
        d.rx_table[k] = -1;
        d.rx_nubar[k] = -1;
        d.rx_tsl[k] = -1;
      }
      if (!nuc.present[t]) continue;
      const CEData& ce = nuc.ce[t];
      if (ce.reactions.size() > static_cast<size_t>(kCEMaxReactions))
        throw std::runtime_error("nuclide " + nuc.name + ": more than " + std::to_string(kCEMaxReactions) +
                                 " continuous-energy reactions");
      d.present = 1;
      d.awr = ce.awr;
      d.total = add_table(ce.total.xs);
      d.total_T = ce.total.temperature;
      d.n_rx = static_cast<int32_t>(ce.reactions.size());
      for (size_t k = 0; k < ce.reactions.size(); k++) {
        const CEReaction& r = ce.reactions[k];
        d.rx_kind[k] = r.kind;
        d.rx_table[k] = add_table(r.eval.xs);
        d.rx_T[k] = r.eval.temperature;
        d.rx_tsl[k] = r.tsl;
        if (r.kind == kFission && r.has_nubar) {
          d.rx_nubar[k] = add_table(r.nubar);
          for (double v : r.nubar.y) c.max_nubar = std::max(c.max_nubar, v);
        }
      }
    }
  }
  c.tab_off.push_back(0);
  for (const Table1D* t : tabs) {
    c.tab_x.insert(c.tab_x.end(), t->x.begin(), t->x.end());
    c.tab_y.insert(c.tab_y.end(), t->y.begin(), t->y.end());
    c.tab_off.push_back(static_cast<uint32_t>(c.tab_x.size()));
  }
  c.n_grids = static_cast<int32_t>(grids.size());

  // ---- union grid (energies are positive, so their bit patterns sort like
  // the values)
  for (const auto* g : grids) c.union_e.insert(c.union_e.end(), g->begin(), g->end());
  std::sort(c.union_e.begin(), c.union_e.end());
  c.union_e.erase(std::unique(c.union_e.begin(), c.union_e.end()), c.union_e.end());
  if (c.union_e.empty()) throw std::runtime_error("continuous-energy problem without cross-section tables");
  if (!(c.union_e.front() > 0)) throw std::runtime_error("continuous-energy tables need positive energies");
  const size_t nu = c.union_e.size();
  for (double e : c.union_e) c.union_key.push_back(key_of(e));

  // buckets: about two per union point
  c.key0 = c.union_key.front();
  const uint64_t range = c.union_key.back() - c.key0;
  uint64_t target = 1;
  while (target < 2 * nu && target < (1ull << 22)) target <<= 1;
  int shift = 0;
  while ((range >> shift) >= target) shift++;
  c.shift = shift;
  c.n_buckets = static_cast<int32_t>((range >> shift) + 1);
  c.bucket.resize(static_cast<size_t>(c.n_buckets) + 1);
  for (size_t b = 0; b <= static_cast<size_t>(c.n_buckets); b++) {
    const uint64_t kb = c.key0 + (static_cast<uint64_t>(b) << shift);
    c.bucket[b] = static_cast<uint32_t>(std::upper_bound(c.union_key.begin(), c.union_key.end(), kb) -
                                        c.union_key.begin());
  }

  // union index -> position in each distinct axis
  c.umap.resize(static_cast<size_t>(c.n_grids) * (nu + 1));
  for (int32_t g = 0; g < c.n_grids; g++) {
    const std::vector<double>& x = *grids[g];
    uint32_t* row = c.umap.data() + static_cast<size_t>(g) * (nu + 1);
    size_t i = 0;
    for (size_t j = 0; j < nu; j++) {
      while (i < x.size() && x[i] < c.union_e[j]) i++;
      row[j] = static_cast<uint32_t>(i);
    }
    row[nu] = static_cast<uint32_t>(x.size());
  }

  // ---- FP32 union tables, when valid
  c.fast_ok = true;
  for (const Cell& cl : m.cells) {
    if (cl.material < 0) continue;
    const ScalarField& f = m.fields.at(static_cast<size_t>(cl.temperature));
    if (f.linear) {
      c.fast_ok = false;
      c.fast_reason = "cell " + cl.name + ": temperature varies in space";
      break;
    }
    const Material& mt = m.materials[static_cast<size_t>(cl.material)];
    for (int32_t n : mt.nuclides) {
      for (size_t t = 0; t < T; t++) {
        const Nuclide& nuc = m.nuclides[static_cast<size_t>(n)];
        if (!nuc.present[t]) continue;
        const CEData& ce = nuc.ce[t];
        if (!ce.total.IsValid(f.c)) {
          c.fast_ok = false;
          c.fast_reason = "nuclide " + nuc.name + ": total not evaluated at the temperature of cell " + cl.name;
        }
        if (ce.reactions.size() > 3) {
          c.fast_ok = false;
          c.fast_reason = "nuclide " + nuc.name + ": more than 3 reactions";
        }
        for (const CEReaction& r : ce.reactions) {
          if (r.kind == kScatter && (r.tsl >= 0 || !r.eval.IsValid(f.c))) {
            c.fast_ok = false;
            c.fast_reason = "nuclide " + nuc.name + ": scattering depends on temperature in cell " + cl.name;
          }
        }
      }
    }
    if (!c.fast_ok) break;
  }
  size_t kmax = 1;
  for (const Material& mt : m.materials) kmax = std::max(kmax, mt.nuclides.size());
  c.kmax = static_cast<int32_t>(kmax);
  if (!c.fast_ok) return c;

  c.union_inv.assign(nu, 0.0f);
  for (size_t j = 1; j < nu; j++) c.union_inv[j] = static_cast<float>(1.0 / (c.union_e[j] - c.union_e[j - 1]));
  std::vector<double> tot(T * N * nu, 0), nsf(T * N * nu, 0);
  c.nuc_rx.assign(T * N * nu * 4, -1.0f);
  c.nuc_nubar.assign(T * N * nu, 0.0f);
  for (size_t t = 0; t < T; t++) {
    for (size_t n = 0; n < N; n++) {
      const Nuclide& nuc = m.nuclides[n];
      if (!nuc.present[t]) continue;
      const CEData& ce = nuc.ce[t];
      for (size_t j = 0; j < nu; j++) {
        const double E = c.union_e[j];
        const size_t i = (t * N + n) * nu + j;
        tot[i] = table_at(ce.total.xs, E);
        double acc = 0;
        for (size_t k = 0; k < ce.reactions.size(); k++) {
          const CEReaction& r = ce.reactions[k];
          const double xs = table_at(r.eval.xs, E);
          acc = acc + xs;
          c.nuc_rx[i * 4 + k] = static_cast<float>(acc);
          if (r.kind == kFission && r.has_nubar) {
            const double nb = table_at(r.nubar, E);
            c.nuc_nubar[i] = static_cast<float>(nb);
            nsf[i] = nb * xs;
          }
        }
        c.nuc_rx[i * 4 + 3] = static_cast<float>(tot[i]);
      }
    }
  }
  c.mat_flight.assign(T * M * nu * 2, 0.0f);
  c.mat_ncdf.assign(T * M * nu * kmax, 0.0f);
  for (size_t t = 0; t < T; t++) {
    for (size_t mi = 0; mi < M; mi++) {
      const Material& mt = m.materials[mi];
      for (size_t j = 0; j < nu; j++) {
        const size_t row = (t * M + mi) * nu + j;
        double acc = 0, nu_acc = 0;
        for (size_t k = 0; k < mt.nuclides.size(); k++) {
          const size_t i = (t * N + static_cast<size_t>(mt.nuclides[k])) * nu + j;
          acc = acc + mt.afrac[k] * tot[i];
          nu_acc = nu_acc + mt.afrac[k] * nsf[i];
          c.mat_ncdf[row * kmax + k] = static_cast<float>(acc);
        }
        for (size_t k = mt.nuclides.size(); k < kmax; k++) c.mat_ncdf[row * kmax + k] = static_cast<float>(acc);
        c.mat_flight[row * 2 + 0] = static_cast<float>(mt.number_density * acc);
        c.mat_flight[row * 2 + 1] = static_cast<float>(mt.number_density * nu_acc);
      }
    }
  }
  return c;
}

}  // namespace mc
