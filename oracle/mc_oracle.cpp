// CPU oracle: a restatement of minimc's particle-history path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU engine
// (tests, __graft_entry__.smoke) and the timed CPU baseline of bench.py.  The
// product never links or calls it.
//
// It follows the reference line by line on the problem model loaded by the
// project's XML loader (minimc_gb300/csrc/mc_model.cpp):
//   FixedSource::StartWorker      src/FixedSource.cpp:40-77
//   SurfaceTracking::Transport    src/TransportMethod.cpp:52-77
//   CellDeltaTracking::Transport  src/TransportMethod.cpp:88-122
//   Particle::Stream/Scatter/SampleNuclide/BankSecondaries
//                                 src/Particle.cpp:46-124
//   Direction(rng), Direction(d, mu, phi)   src/Point.cpp:90-121
//   CSGSurface::Distance/Contains, SolveQuadratic  src/CSGSurface.cpp:71-174
//   Cell::Contains/NearestSurface src/Cell.cpp:27-51
//   World::FindCellContaining     src/World.cpp:26-37
//   Material::GetMicroscopicTotal src/Material.cpp:52-61
//   Multigroup::Interact/Scatter/Fission   src/Multigroup.cpp:49-73,245-286
//   Source::Sample                src/Source.cpp:143-154
//   ScorableProxy::Score/CommitHistory     src/Scorable.cpp:81-106
// Random numbers come from std::minstd_rand and the standard library's
// distributions, exactly as in the reference (src/BasicTypes.hpp:27).
//
// The k-eigenvalue harness completes the reference's stub
// (src/KEigenvalue.cpp:36-62): cycle 0 starts from Source::Sample(1..N),
// each cycle transports N particles, collects their fission secondaries
// (Particle::MoveSecondariesTo) in source order, sets k = M/N and draws the
// next N sources uniformly from the bank with a Philox4x32-10 stream.
//
// Compiled with -ffp-contract=off so every product and sum rounds separately,
// as in the reference built for x86-64.
#include "mc_model.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <list>
#include <map>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

using mc::Model;
using RNG = std::minstd_rand;

constexpr double kPi = M_PI;
constexpr double kNudge = 10 * std::numeric_limits<double>::epsilon();
constexpr double kOnAxis = 0.9;
constexpr double kInf = std::numeric_limits<double>::infinity();

enum Event { kBirth = 0, kScatter, kCapture, kFission, kSurfaceCross, kLeak, kVirtual, kReflect, kLost };

struct Vec {
  double x = 0, y = 0, z = 0;
};
double Dot(const Vec& a, const Vec& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
Vec Cross(const Vec& a, const Vec& b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
Vec Normalized(Vec p) {
  const double n = std::sqrt(Dot(p, p));
  p.x /= n;
  p.y /= n;
  p.z /= n;
  return p;
}

// Direction(RNG&)
Vec IsotropicDirection(RNG& rng) {
  Vec d;
  d.x = std::uniform_real_distribution{-1., +1.}(rng);
  const double sin_theta = std::sqrt(1 - d.x * d.x);
  const double phi = std::uniform_real_distribution{0., 2 * kPi}(rng);
  d.y = sin_theta * std::cos(phi);
  d.z = sin_theta * std::sin(phi);
  return d;
}

// Direction(d, mu, phi)
Vec Rotate(const Vec& d, double mu, double phi) {
  const bool is_off_xaxis = d.x <= kOnAxis && d.x > -kOnAxis;
  const Vec xaxis = is_off_xaxis ? Vec{1, 0, 0} : Vec{0, 1, 0};
  const Vec u = Normalized(Cross(d, xaxis));
  const Vec v = Normalized(Cross(d, u));
  const double a = std::sqrt(1 - mu * mu) * std::cos(phi);
  const double b = std::sqrt(1 - mu * mu) * std::sin(phi);
  const Vec uc{a * u.x, a * u.y, a * u.z}, vc{b * v.x, b * v.y, b * v.z}, dc{mu * d.x, mu * d.y, mu * d.z};
  return Normalized(Vec{uc.x + vc.x + dc.x, uc.y + vc.y + dc.y, uc.z + vc.z + dc.z});
}

double SolveQuadratic(double a, double b, double c) {
  const double discriminant{b * b - 4 * a * c};
  if (discriminant <= 0) return kInf;
  const double lesser{b > 0 ? (-b - std::sqrt(discriminant)) / (2 * a) : (2 * c) / (-b + std::sqrt(discriminant))};
  const double greater{b > 0 ? (2 * c) / (-b - std::sqrt(discriminant)) : (-b + std::sqrt(discriminant)) / (2 * a)};
  if (lesser > 0) return lesser;
  if (greater > 0) return greater;
  return kInf;
}

struct Oracle {
  Model m;
  int quirks = 0;  // 0: robust geometry (default), 1: the reference's exact semantics
  std::string err;

  // ---- geometry --------------------------------------------------------
  double Distance(int s, const Vec& o, const Vec& d) const {
    const mc::Surface& S = m.surfaces[s];
    auto plane = [](double c, double p, double u) {
      const double v = c - p;
      const double t = v / u;
      return t > 0 ? t : kInf;
    };
    switch (S.kind) {
    case mc::kPlaneX: return plane(S.p[0], Dot(o, {1, 0, 0}), Dot(d, {1, 0, 0}));
    case mc::kPlaneY: return plane(S.p[0], Dot(o, {0, 1, 0}), Dot(d, {0, 1, 0}));
    case mc::kPlaneZ: return plane(S.p[0], Dot(o, {0, 0, 1}), Dot(d, {0, 0, 1}));
    case mc::kSphere: {
      const Vec oc{o.x - S.p[0], o.y - S.p[1], o.z - S.p[2]};
      return SolveQuadratic(1, 2 * Dot(oc, d), Dot(oc, oc) - S.p[3] * S.p[3]);
    }
    default: {
      const Vec w = S.kind == mc::kCylinderX ? Vec{1, 0, 0} : S.kind == mc::kCylinderY ? Vec{0, 1, 0} : Vec{0, 0, 1};
      const double pp = Dot(o, o), pw = Dot(o, w), dw = Dot(d, w), pd = Dot(o, d);
      return SolveQuadratic(1 - dw * dw, 2 * (pd - pw * dw), pp - pw * pw - S.p[0] * S.p[0]);
    }
    }
  }

  bool Contains(int s, const Vec& p) const {
    const mc::Surface& S = m.surfaces[s];
    switch (S.kind) {
    case mc::kPlaneX: return Dot(p, {1, 0, 0}) < S.p[0];
    case mc::kPlaneY: return Dot(p, {0, 1, 0}) < S.p[0];
    case mc::kPlaneZ: return Dot(p, {0, 0, 1}) < S.p[0];
    case mc::kSphere: {
      const Vec pc{p.x - S.p[0], p.y - S.p[1], p.z - S.p[2]};
      return Dot(pc, pc) < S.p[3] * S.p[3];
    }
    default: {
      const Vec w = S.kind == mc::kCylinderX ? Vec{1, 0, 0} : S.kind == mc::kCylinderY ? Vec{0, 1, 0} : Vec{0, 0, 1};
      const double pp = Dot(p, p), pw = Dot(p, w);
      const double r = S.p[0];
      return quirks ? std::sqrt(pp - pw * pw) < r * r : pp - pw * pw < r * r;
    }
    }
  }

  bool CellContains(int c, const Vec& p) const {
    const mc::Cell& cl = m.cells[c];
    for (size_t k = 0; k < cl.surfaces.size(); k++)
      if (Contains(cl.surfaces[k], p) != (cl.within[k] != 0)) return false;
    return true;
  }

  int FindCellContaining(const Vec& p) const {
    for (size_t c = 0; c < m.cells.size(); c++)
      if (CellContains(static_cast<int>(c), p)) return static_cast<int>(c);
    return -1;
  }

  // min_element over the cell's surfaces with `Distance(l) < Distance(r)`;
  // `skip` (robust geometry only) reads as infinitely far
  int NearestSurface(int c, const Vec& p, const Vec& d, double& dist, int skip = -1) const {
    const mc::Cell& cl = m.cells[c];
    if (cl.surfaces.empty()) return -1;
    auto D = [&](size_t k) { return cl.surfaces[k] == skip ? kInf : Distance(cl.surfaces[k], p, d); };
    size_t best = 0;
    for (size_t k = 1; k < cl.surfaces.size(); k++)
      if (D(k) < D(best)) best = k;
    dist = D(best);
    return cl.surfaces[best];
  }

  // robust geometry: the side of a crossed surface follows the direction
  bool MovingPositive(int s, const Vec& p, const Vec& d) const {
    const mc::Surface& S = m.surfaces[s];
    switch (S.kind) {
    case mc::kPlaneX: return d.x > 0;
    case mc::kPlaneY: return d.y > 0;
    case mc::kPlaneZ: return d.z > 0;
    case mc::kSphere: return (p.x - S.p[0]) * d.x + (p.y - S.p[1]) * d.y + (p.z - S.p[2]) * d.z > 0;
    case mc::kCylinderX: return p.y * d.y + p.z * d.z > 0;
    case mc::kCylinderY: return p.x * d.x + p.z * d.z > 0;
    default: return p.x * d.x + p.y * d.y > 0;
    }
  }

  int FindCellCrossing(const Vec& p, int crossed, bool to_positive) const {
    for (size_t c = 0; c < m.cells.size(); c++) {
      const mc::Cell& cl = m.cells[c];
      bool in = true;
      for (size_t k = 0; k < cl.surfaces.size() && in; k++) {
        const bool inside = cl.surfaces[k] == crossed ? !to_positive : Contains(cl.surfaces[k], p);
        in = inside == (cl.within[k] != 0);
      }
      if (in) return static_cast<int>(c);
    }
    return -1;
  }

  // ---- physics (multigroup) ---------------------------------------------
  struct P {
    Vec pos, dir;
    uint64_t g = 1;  // group, 1-based
    double E = 0;
    int type = 0;
    int cell = -1;
    int event = kBirth;
    int surf = -1;
    int skip = -1;
    RNG rng;
    std::list<P> secondaries;
  };

  double NuclideTotal(int n, const P& p) const { return m.nuclides[n].mg[p.type].total.at(p.g - 1); }

  double MaterialTotal(int mat, const P& p) const {
    const mc::Material& M = m.materials[mat];
    double acc = 0;
    for (size_t k = 0; k < M.nuclides.size(); k++) acc = acc + M.afrac[k] * NuclideTotal(M.nuclides[k], p);
    return acc;
  }

  int SampleNuclide(P& p) const {
    const mc::Material& M = m.materials[m.cells[p.cell].material];
    const double threshold = MaterialTotal(m.cells[p.cell].material, p) * std::uniform_real_distribution{}(p.rng);
    double accumulated = 0;
    for (size_t k = 0; k < M.nuclides.size(); k++) {
      accumulated += M.afrac[k] * NuclideTotal(M.nuclides[k], p);
      if (accumulated > threshold) return M.nuclides[k];
    }
    return M.nuclides.back();
  }

  void BankSecondaries(P& p, const Vec& dir, uint64_t g) const {
    P s;
    s.pos = p.pos;
    s.dir = dir;
    s.g = g;
    s.type = 0;
    s.rng.seed(p.rng());
    s.cell = p.cell;
    p.secondaries.push_back(std::move(s));
  }

  void MGInteract(int n, P& p) const {
    const mc::MGData& d = m.nuclides[n].mg[p.type];
    const uint64_t G = m.groups;
    const double threshold{std::uniform_real_distribution{}(p.rng) * d.total.at(p.g - 1)};
    double accumulated{0};
    const int kinds[3] = {mc::kCapture, mc::kScatter, mc::kFission};
    for (int kind : kinds) {
      const bool present = kind == mc::kCapture ? d.has_capture : kind == mc::kScatter ? d.has_scatter : d.has_fission;
      if (!present) continue;
      const std::vector<double>& xs = kind == mc::kCapture ? d.capture : kind == mc::kScatter ? d.scatter : d.fission;
      accumulated += xs.at(p.g - 1);
      if (accumulated > threshold) {
        if (kind == mc::kCapture) {
          p.event = kCapture;
        }
        else if (kind == mc::kScatter) {
          p.event = kScatter;
          const double t = std::uniform_real_distribution{}(p.rng);
          double acc{0};
          for (uint64_t g = 1; g <= G; g++) {
            acc += d.scatter_prob[(p.g - 1) * G + (g - 1)];
            if (acc > t) {
              p.g = g;
              p.dir = IsotropicDirection(p.rng);
              return;
            }
          }
        }
        else {
          p.event = kFission;
          const uint64_t gin = p.g;
          const size_t yield(d.nubar.at(gin - 1) + std::uniform_real_distribution{}(p.rng));
          for (size_t i = 0; i < yield; i++) {
            const double t = std::uniform_real_distribution{}(p.rng);
            double acc{0};
            for (uint64_t g = 1; g <= G; g++) {
              acc += d.chi[(gin - 1) * G + (g - 1)];
              if (acc > t) {
                const Vec dir = IsotropicDirection(p.rng);
                BankSecondaries(p, dir, g);
                break;
              }
            }
          }
        }
        return;
      }
    }
  }

  // ---- scoring ------------------------------------------------------------
  double EnergyValue(const P& p) const { return m.energy_mode == mc::kMultigroup ? static_cast<double>(p.g) : p.E; }

  size_t BinIndex(size_t e, const P& p) const {
    const mc::Estimator& est = m.estimators[e];
    const size_t ci = est.has_cosine ? est.cosine.index(Dot(Vec{est.cosine_dir[0], est.cosine_dir[1], est.cosine_dir[2]}, p.dir)) : 0;
    return est.energy.size() * ci + est.energy.index(EnergyValue(p));
  }

  std::vector<size_t> offsets;

  void Score(const P& p, std::map<size_t, double>& pending) const {
    if (p.event != kSurfaceCross && p.event != kLeak) return;
    for (size_t e = 0; e < m.estimators.size(); e++) {
      const auto& est = m.estimators[e];
      if (est.kind != mc::kCurrent || est.surface != p.surf) continue;
      pending[offsets[e] + BinIndex(e, p)] += 1;
    }
  }

  void ScoreTrack(const P& p, double d, std::map<size_t, double>& pending) const {
    for (size_t e = 0; e < m.estimators.size(); e++) {
      const auto& est = m.estimators[e];
      if (est.kind != mc::kTrackLength || est.cell != p.cell) continue;
      pending[offsets[e] + BinIndex(e, p)] += d;
    }
  }

  void Stream(P& p, double d) const {
    p.pos.x += p.dir.x * d;
    p.pos.y += p.dir.y * d;
    p.pos.z += p.dir.z * d;
  }

  // ---- transport ------------------------------------------------------------
  struct Stats {
    uint64_t events = 0, lost = 0, capped = 0;
    double ktl = 0;
  };

  // SurfaceTracking / CellDeltaTracking::Transport for one particle
  void Transport(P& p, std::map<size_t, double>& pending, Stats& st, bool score, uint32_t max_events,
                 uint32_t* nev_out) const {
    p.cell = FindCellContaining(p.pos);
    uint32_t nev = 0;
    if (p.cell < 0 || m.cells[p.cell].material < 0) {
      p.event = kLost;
      st.lost++;
      if (nev_out) *nev_out += 0;
      return;
    }
    const bool delta = m.tracking == mc::kCellDeltaTracking;
    while (p.event != kCapture && p.event != kLeak && p.event != kFission && p.event != kLost) {
      const int mat = m.cells[p.cell].material;
      const double micro = MaterialTotal(mat, p);
      const double distance_to_collision =
          std::exponential_distribution{m.materials[mat].number_density * micro}(p.rng);
      double dsurf;
      const int s = NearestSurface(p.cell, p.pos, p.dir, dsurf, p.skip);
      const bool collide = delta ? !(dsurf < distance_to_collision) : distance_to_collision < dsurf;
      if (collide) {
        if (score) ScoreTrack(p, distance_to_collision, pending);
        st.ktl += distance_to_collision * m.materials[mat].number_density * NuSigmaF(mat, p);
        Stream(p, distance_to_collision);
        p.skip = -1;
        if (delta) (void)std::bernoulli_distribution{micro / micro}(p.rng);
        const int n = SampleNuclide(p);
        MGInteract(n, p);
      }
      else if (m.surfaces[s].reflective) {
        if (score) ScoreTrack(p, dsurf, pending);
        st.ktl += dsurf * m.materials[mat].number_density * NuSigmaF(mat, p);
        Stream(p, dsurf);
        const int kind = m.surfaces[s].kind;
        if (kind == mc::kPlaneX) p.dir.x = -p.dir.x;
        else if (kind == mc::kPlaneY) p.dir.y = -p.dir.y;
        else p.dir.z = -p.dir.z;
        p.event = kReflect;
        p.surf = s;
        p.skip = s;
      }
      else {
        const double d = dsurf + kNudge;
        if (score) ScoreTrack(p, d, pending);
        st.ktl += d * m.materials[mat].number_density * NuSigmaF(mat, p);
        Stream(p, d);
        if (quirks) {
          p.cell = FindCellContaining(p.pos);
        }
        else {
          p.cell = FindCellCrossing(p.pos, s, MovingPositive(s, p.pos, p.dir));
          p.skip = s;
        }
        p.surf = s;
        if (p.cell < 0) {
          p.event = kLost;
          st.lost++;
        }
        else {
          p.event = m.cells[p.cell].material >= 0 ? kSurfaceCross : kLeak;
        }
      }
      if (score) Score(p, pending);
      nev++;
      st.events++;
      if (nev >= max_events && p.event != kCapture && p.event != kLeak && p.event != kFission && p.event != kLost) {
        st.capped++;
        p.event = kLost;
      }
    }
    if (nev_out) *nev_out += nev;
  }

  double NuSigmaF(int mat, const P& p) const {
    const mc::Material& M = m.materials[mat];
    double acc = 0;
    for (size_t k = 0; k < M.nuclides.size(); k++) {
      const mc::MGData& d = m.nuclides[M.nuclides[k]].mg[p.type];
      if (d.has_fission) acc = acc + M.afrac[k] * (d.nubar[p.g - 1] * d.fission[p.g - 1]);
    }
    return acc;
  }

  // Source::Sample(seed)
  P SampleSource(uint64_t seed) const {
    RNG rng{static_cast<RNG::result_type>(seed)};
    P p;
    p.pos = {m.source.position[0], m.source.position[1], m.source.position[2]};
    if (m.source.direction == mc::kDirConstant) {
      p.dir = {m.source.dir[0], m.source.dir[1], m.source.dir[2]};
    }
    else if (m.source.direction == mc::kDirIsotropic) {
      p.dir = IsotropicDirection(rng);
    }
    else {
      const double mu = std::sqrt(std::uniform_real_distribution{}(rng));
      const double phi = std::uniform_real_distribution{0., 2 * kPi}(rng);
      p.dir = Rotate(Vec{m.source.dir[0], m.source.dir[1], m.source.dir[2]}, mu, phi);
    }
    p.g = m.source.group;
    p.E = m.source.energy;
    p.type = m.source.type;
    p.rng.seed(rng());
    return p;
  }
};

// splitmix64 + run key, as the GPU engine derives its Philox keys
uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t run_key(uint64_t seed, uint64_t cycle, uint64_t salt) {
  return splitmix64(seed * 0x9E3779B97F4A7C15ull + cycle * 0xD1B54A32D192ED03ull + salt);
}

// Philox4x32-10 (Salmon et al., SC'11)
void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = 0xD2511F53ull * c[0], p1 = 0xCD9E8D57ull * c[2];
    const uint32_t n0 = static_cast<uint32_t>(p1 >> 32) ^ c[1] ^ k0;
    const uint32_t n2 = static_cast<uint32_t>(p0 >> 32) ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = static_cast<uint32_t>(p1);
    c[2] = n2;
    c[3] = static_cast<uint32_t>(p0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

template <class F>
void parallel_for(uint64_t n, int threads, F&& body) {
  std::atomic<uint64_t> next{0};
  auto worker = [&](int tid) {
    for (;;) {
      const uint64_t i = next.fetch_add(1);
      if (i >= n) break;
      body(tid, i);
    }
  };
  if (threads <= 1) {
    worker(0);
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(worker, t);
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

struct orc_stats {
  uint64_t events, lost, capped, secondaries;
  double seconds;
  double k_tracklength;
};

void* orc_create(const char* xml, const char* base_dir, char* err, size_t errn) {
  auto* o = new Oracle();
  try {
    o->m = mc::load_model(xml, base_dir ? base_dir : "");
  }
  catch (const std::exception& e) {
    if (err && errn) {
      std::strncpy(err, e.what(), errn - 1);
      err[errn - 1] = 0;
    }
    delete o;
    return nullptr;
  }
  size_t off = 0;
  for (const auto& e : o->m.estimators) {
    o->offsets.push_back(off);
    off += e.size();
  }
  return o;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

void orc_set_quirks(void* h, int q) { static_cast<Oracle*>(h)->quirks = q; }

uint64_t orc_total_bins(void* h) { return static_cast<Oracle*>(h)->m.total_bins(); }

void orc_find_cell(void* h, const double* xyz, uint64_t n, int32_t* out) {
  auto* o = static_cast<Oracle*>(h);
  for (uint64_t i = 0; i < n; i++) out[i] = o->FindCellContaining({xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
}

void orc_nearest_surface(void* h, const int32_t* cell, const double* xyz, const double* uvw, uint64_t n, int32_t* surf,
                         double* dist) {
  auto* o = static_cast<Oracle*>(h);
  for (uint64_t i = 0; i < n; i++) {
    double d = kInf;
    surf[i] = cell[i] < 0 ? -1
                          : o->NearestSurface(cell[i], {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]},
                                              {uvw[3 * i], uvw[3 * i + 1], uvw[3 * i + 2]}, d);
    dist[i] = d;
  }
}

void orc_surface_distance(void* h, int32_t s, const double* xyz, const double* uvw, uint64_t n, double* out) {
  auto* o = static_cast<Oracle*>(h);
  for (uint64_t i = 0; i < n; i++)
    out[i] = o->Distance(s, {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}, {uvw[3 * i], uvw[3 * i + 1], uvw[3 * i + 2]});
}

void orc_surface_contains(void* h, int32_t s, const double* xyz, uint64_t n, int8_t* out) {
  auto* o = static_cast<Oracle*>(h);
  for (uint64_t i = 0; i < n; i++) out[i] = o->Contains(s, {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}) ? 1 : 0;
}

void orc_philox(uint32_t* c, uint32_t k0, uint32_t k1) { philox(c, k0, k1); }

// Direction(d, mu, phi) and Direction(x, y, z) (src/Point.cpp:98-129)
void orc_rotate(const double* d, double mu, double phi, double* out) {
  const Vec r = Rotate(Vec{d[0], d[1], d[2]}, mu, phi);
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
}
void orc_normalize(const double* d, double* out) {
  const Vec r = Normalized(Vec{d[0], d[1], d[2]});
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
}

// Material::GetMicroscopicTotal of a neutron of group g in cell c
double orc_material_total(void* h, int32_t cell, uint64_t g) {
  auto* o = static_cast<Oracle*>(h);
  const int mat = o->m.cells.at(cell).material;
  if (mat < 0) return 0;
  Oracle::P p;
  p.g = g;
  p.type = 0;
  return o->MaterialTotal(mat, p);
}

// minstd + generate_canonical values for a seed (RNG parity checks)
void orc_minstd_canonical(uint64_t seed, uint64_t n, double* out) {
  RNG rng{static_cast<RNG::result_type>(seed)};
  for (uint64_t i = 0; i < n; i++) out[i] = std::uniform_real_distribution{}(rng);
}

// FixedSource::Solve over histories [0, n) with seeds seed + i
int orc_run_fixed_source(void* h, uint64_t n, uint64_t seed, int threads, uint32_t max_events, double* sum, double* sq,
                         uint32_t* hist_events, int8_t* hist_fate, orc_stats* stats) {
  auto* o = static_cast<Oracle*>(h);
  if (o->m.energy_mode != mc::kMultigroup) return -1;
  const size_t nb = std::max<size_t>(1, o->m.total_bins());
  threads = std::max(1, threads);
  std::vector<std::vector<double>> ts(threads, std::vector<double>(nb, 0)), tq(threads, std::vector<double>(nb, 0));
  std::vector<Oracle::Stats> st(threads);
  std::vector<uint64_t> sec(threads, 0);
  const auto t0 = std::chrono::steady_clock::now();
  parallel_for(n, threads, [&](int tid, uint64_t i) {
    std::map<size_t, double> pending;
    std::list<Oracle::P> bank;
    bank.push_back(o->SampleSource(seed + i));
    uint32_t nev = 0;
    int8_t fate = -1;
    while (!bank.empty()) {
      o->Transport(bank.back(), pending, st[tid], true, max_events, &nev);
      if (fate < 0) fate = static_cast<int8_t>(bank.back().event);
      sec[tid] += bank.back().secondaries.size();
      bank.splice(bank.begin(), bank.back().secondaries);
      bank.pop_back();
    }
    for (const auto& [b, s] : pending) {
      ts[tid][b] += s;
      tq[tid][b] += s * s;
    }
    if (hist_events) hist_events[i] = nev;
    if (hist_fate) hist_fate[i] = fate;
  });
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t b = 0; b < o->m.total_bins(); b++) {
    double a = 0, q = 0;
    for (int t = 0; t < threads; t++) {
      a += ts[t][b];
      q += tq[t][b];
    }
    if (sum) sum[b] = a;
    if (sq) sq[b] = q;
  }
  if (stats) {
    *stats = orc_stats{};
    for (int t = 0; t < threads; t++) {
      stats->events += st[t].events;
      stats->lost += st[t].lost;
      stats->capped += st[t].capped;
      stats->secondaries += sec[t];
    }
    stats->seconds = secs;
  }
  return 0;
}

// k-eigenvalue harness; k_cycle/bank: [inactive + active]
int orc_run_keigenvalue(void* h, uint64_t N, uint64_t seed, uint32_t inactive, uint32_t active, int threads,
                        uint32_t max_cycles_timed, double* k_cycle, uint64_t* bank_size, double* sum, double* sq,
                        orc_stats* stats) {
  auto* o = static_cast<Oracle*>(h);
  if (o->m.energy_mode != mc::kMultigroup) return -1;
  threads = std::max(1, threads);
  const size_t nb = std::max<size_t>(1, o->m.total_bins());
  std::vector<std::vector<double>> ts(threads, std::vector<double>(nb, 0)), tq(threads, std::vector<double>(nb, 0));
  std::vector<Oracle::Stats> st(threads);
  struct SiteRec {
    Vec pos, dir;
    uint64_t g;
  };
  std::vector<SiteRec> source(N);
  std::vector<std::vector<SiteRec>> per_hist(N);
  const uint32_t cycles = inactive + active;
  const auto t0 = std::chrono::steady_clock::now();
  double ktl_active = 0;
  for (uint32_t c = 0; c < cycles && (max_cycles_timed == 0 || c < max_cycles_timed); c++) {
    const bool act = c >= inactive;
    std::vector<double> ktl(threads, 0);
    parallel_for(N, threads, [&](int tid, uint64_t j) {
      Oracle::P p;
      if (c == 0) {
        p = o->SampleSource(j + 1);  // src/KEigenvalue.cpp:31-33
      }
      else {
        p.pos = source[j].pos;
        p.dir = source[j].dir;
        p.g = source[j].g;
        p.type = 0;
        p.rng.seed(static_cast<RNG::result_type>(seed + static_cast<uint64_t>(c) * N + j));
      }
      std::map<size_t, double> pending;
      Oracle::Stats& s = st[tid];
      const double k0 = s.ktl;
      o->Transport(p, pending, s, act, 1000000u, nullptr);
      ktl[tid] += s.ktl - k0;
      per_hist[j].clear();
      for (const auto& q : p.secondaries) per_hist[j].push_back({q.pos, q.dir, q.g});
      if (act) {
        for (const auto& [b, v] : pending) {
          ts[tid][b] += v;
          tq[tid][b] += v * v;
        }
      }
    });
    std::vector<SiteRec> bank;
    for (uint64_t j = 0; j < N; j++) bank.insert(bank.end(), per_hist[j].begin(), per_hist[j].end());
    const uint64_t M = bank.size();
    if (k_cycle) k_cycle[c] = static_cast<double>(M) / static_cast<double>(N);
    if (bank_size) bank_size[c] = M;
    double kt = 0;
    for (double v : ktl) kt += v;
    if (act) ktl_active += kt / static_cast<double>(N);
    if (M == 0) return -2;
    const uint64_t key = run_key(seed, c, 0x52455341ull);
    for (uint64_t j = 0; j < N; j++) {
      uint32_t ctr[4] = {static_cast<uint32_t>(j), static_cast<uint32_t>(j >> 32), 0x72657361u, 0};
      philox(ctr, static_cast<uint32_t>(key), static_cast<uint32_t>(key >> 32));
      const double u = ((ctr[0] >> 5) * 67108864.0 + (ctr[1] >> 6)) * (1.0 / 9007199254740992.0);
      uint64_t idx = static_cast<uint64_t>(u * static_cast<double>(M));
      if (idx >= M) idx = M - 1;
      source[j] = bank[idx];
    }
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t b = 0; b < o->m.total_bins(); b++) {
    double a = 0, q = 0;
    for (int t = 0; t < threads; t++) {
      a += ts[t][b];
      q += tq[t][b];
    }
    if (sum) sum[b] = a;
    if (sq) sq[b] = q;
  }
  if (stats) {
    *stats = orc_stats{};
    for (int t = 0; t < threads; t++) {
      stats->events += st[t].events;
      stats->lost += st[t].lost;
      stats->capped += st[t].capped;
    }
    stats->seconds = secs;
    stats->k_tracklength = active ? ktl_active / active : 0;
  }
  return 0;
}

}  // extern "C"
