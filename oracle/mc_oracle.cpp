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
//   TotalCrossSectionPerturbation::Stream  src/Perturbation.cpp:68-78
//   CurrentTotalCrossSectionSensitivity::GetScore  src/Sensitivity.cpp:55-58
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
constexpr double kBoltzmann = 8.617333262145e-11;     // MeV / K
constexpr double kNeutronMass = 1.045354912280858e-18;  // MeV (s / cm)^2

enum Event { kBirth = 0, kScatter, kCapture, kFission, kSurfaceCross, kLeak, kVirtual, kReflect, kLost };

struct Vec {
  double x = 0, y = 0, z = 0;
};
double Dot(const Vec& a, const Vec& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
Vec Cross(const Vec& a, const Vec& b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
Vec Scale(const Vec& a, double s) { return {a.x * s, a.y * s, a.z * s}; }
Vec Add(const Vec& a, const Vec& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
Vec Sub(const Vec& a, const Vec& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
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
    bool resample_failed = false;  // thermal scattering resample limit hit
    double eff[4] = {0, 0, 0, 0};  // indirect effect of each perturbation (Particle::indirect_effects)
    RNG rng;
    std::list<P> secondaries;
  };

  double NuclideTotal(int n, const P& p) const {
    if (m.energy_mode == mc::kMultigroup) return m.nuclides[n].mg[p.type].total.at(p.g - 1);
    return CETotal(m.nuclides[n].ce[p.type], p);
  }

  // Nuclide::GetMajorant; Multigroup::GetMajorant is GetTotal (src/Multigroup.cpp:40-43)
  double NuclideMajorant(int n, const P& p) const {
    if (m.energy_mode == mc::kMultigroup) return m.nuclides[n].mg[p.type].total.at(p.g - 1);
    return CEMajorant(m.nuclides[n].ce[p.type], p);
  }

  // Material::GetMicroscopicMajorant (src/Material.cpp:41-50)
  double MaterialMajorant(int mat, const P& p) const {
    const mc::Material& M = m.materials[mat];
    double acc = 0;
    for (size_t k = 0; k < M.nuclides.size(); k++) acc = acc + M.afrac[k] * NuclideMajorant(M.nuclides[k], p);
    return acc;
  }

  // ---- physics (continuous energy) --------------------------------------
  // ContinuousMap::at (src/ContinuousMap.hpp:21-39): bracket by
  // upper_bound, snap at both ends, linear interpolation
  static double MapAt(const mc::Table1D& t, double k) {
    const size_t hi = static_cast<size_t>(std::upper_bound(t.x.begin(), t.x.end(), k) - t.x.begin());
    if (hi == t.x.size()) return t.y.back();
    if (hi == 0) return t.y.front();
    const double k_hi = t.x[hi], v_hi = t.y[hi], k_lo = t.x[hi - 1], v_lo = t.y[hi - 1];
    return v_lo + (v_hi - v_lo) / (k_hi - k_lo) * (k - k_lo);
  }

  // the cell's ScalarField at the particle, and its upper bound
  double CellT(const P& p) const { return m.fields[m.cells[p.cell].temperature].at(p.pos.x, p.pos.y, p.pos.z); }
  double CellTmax(const P& p) const { return m.fields[m.cells[p.cell].temperature].upper; }

  // ContinuousScatter::IsFreeGasScatteringValid (src/ContinuousReaction.cpp:205-223)
  bool FreeGasValid(double awr, const P& p, double T) const {
    if (p.type != mc::kNeutron) return false;
    if (awr <= 1.0) return true;
    return p.E < 500 * kBoltzmann * T / awr;
  }

  // ContinuousScatter::GetFreeGasScatterAdjustment (src/ContinuousReaction.cpp:225-237)
  static double FreeGasAdjustment(double awr, double E, double T) {
    if (T == 0) return 1;
    const double x = std::sqrt(E / (kBoltzmann * T));
    const double arg = awr * x * x;
    return (1 + 1 / (2 * arg)) * std::erf(std::sqrt(arg)) + std::exp(-arg) / std::sqrt(kPi * arg);
  }

  // ContinuousScatter::GetCrossSection / GetMajorant at temperature T
  // (src/ContinuousReaction.cpp:85-120)
  double ScatterXS(const mc::CEData& d, const mc::CEReaction& r, const P& p, double T) const {
    const double xs = MapAt(r.eval.xs, p.E);
    if (r.eval.IsValid(T)) return xs;
    if (FreeGasValid(d.awr, p, T))
      return xs / FreeGasAdjustment(d.awr, p.E, r.eval.temperature) * FreeGasAdjustment(d.awr, p.E, T);
    return xs;
  }

  // ThermalScattering::IsValid (src/ThermalScattering.cpp:100-103)
  bool TSLValid(const mc::CEReaction& r, const P& p) const {
    return r.tsl >= 0 && p.type == mc::kNeutron && p.E < m.tsl[r.tsl].cutoff_energy();
  }

  // ContinuousReaction::GetCrossSection (src/ContinuousReaction.cpp:51-54,
  // :102-120): a valid thermal scattering library replaces the scatter
  // cross section
  double ReactionXS(const mc::CEData& d, const mc::CEReaction& r, const P& p, double T) const {
    if (r.kind != mc::kScatter) return MapAt(r.eval.xs, p.E);
    if (TSLValid(r, p)) return TSLTotal(m.tsl[r.tsl], p.E, CellT(p));
    return ScatterXS(d, r, p, T);
  }

  // ContinuousReaction::GetMajorant (src/ContinuousReaction.cpp:45-49, :81-100)
  double ReactionMajorant(const mc::CEData& d, const mc::CEReaction& r, const P& p, double T_max) const {
    if (r.kind != mc::kScatter) return MapAt(r.eval.xs, p.E);
    if (TSLValid(r, p)) return MapAt(m.tsl[r.tsl].majorant, p.E);
    return ScatterXS(d, r, p, T_max);
  }

  // Continuous::ReactionsModifyTotal (src/Continuous.cpp:88-93)
  bool ModifiesTotal(const mc::CEData& d, const P& p) const {
    for (const auto& r : d.reactions)
      if (r.kind == mc::kScatter && TSLValid(r, p)) return true;
    return false;
  }

  // Continuous::GetTotal (src/Continuous.cpp:45-58)
  double CETotal(const mc::CEData& d, const P& p) const {
    const double T = CellT(p);
    if (!ModifiesTotal(d, p) && d.total.IsValid(T)) return MapAt(d.total.xs, p.E);
    double acc = 0;
    for (const auto& r : d.reactions) acc = acc + ReactionXS(d, r, p, T);
    return acc;
  }

  // Continuous::GetMajorant (src/Continuous.cpp:28-43): the cell's maximum
  // temperature
  double CEMajorant(const mc::CEData& d, const P& p) const {
    const double T = CellTmax(p);
    if (!ModifiesTotal(d, p) && d.total.IsValid(T)) return MapAt(d.total.xs, p.E);
    double acc = 0;
    for (const auto& r : d.reactions) acc = acc + ReactionMajorant(d, r, p, T);
    return acc;
  }

  // ---- thermal scattering (src/ThermalScattering.cpp) --------------------
  static size_t UpperIndex(const std::vector<double>& v, double x) {
    return static_cast<size_t>(std::upper_bound(v.begin(), v.end(), x) - v.begin());
  }

  // temperature bracket shared by GetTotal and the partitions' Evaluate:
  // T_max and above use the top interval, below T_min both ends are the
  // first point
  static void TBracket(const std::vector<double>& Ts, double T, size_t& lo, size_t& hi, bool& below, bool& above) {
    const size_t cand = UpperIndex(Ts, T);
    above = cand == Ts.size();
    hi = above ? cand - 1 : cand;
    below = hi == 0;
    lo = below ? hi : hi - 1;
  }

  // BetaPartition / AlphaPartition::Evaluate (src/ThermalScattering.cpp:183-256)
  static double PODEvaluate(const mc::PODPartitionSet& P, size_t part, size_t cdf_index, size_t g_index, double T) {
    const std::vector<double>& Ts = P.T[part];
    size_t lo, hi;
    bool below, above;
    TBracket(Ts, T, lo, hi, below, above);
    const size_t r = P.S[part].size(), nT = Ts.size();
    const std::vector<double>& S = P.S[part];
    const std::vector<double>& C = P.cdf_modes[part];
    const std::vector<double>& G = P.g_t_modes[part];
    double v_hi = 0, v_lo = 0;
    for (size_t o = 0; o < r; o++) {
      v_hi += S[o] * C[cdf_index * r + o] * G[(g_index * nT + hi) * r + o];
      v_lo += S[o] * C[cdf_index * r + o] * G[(g_index * nT + lo) * r + o];
    }
    const double T_hi = Ts[hi], T_lo = Ts[lo];
    return v_lo + (v_hi - v_lo) / (T_hi - T_lo) * (T - T_lo);
  }

  // ThermalScattering::EvaluateInelastic (src/ThermalScattering.cpp:260-269)
  static double EvaluateInelastic(const mc::TSLData& t, size_t E_index, size_t T_index) {
    const size_t r = t.xs_rank;
    double result = 0;
    for (size_t o = 0; o < r; o++) result += t.xs_S[o] * t.xs_E_modes[E_index * r + o] * t.xs_T_modes[T_index * r + o];
    return result;
  }

  // ThermalScattering::GetTotal (src/ThermalScattering.cpp:111-157)
  static double TSLTotal(const mc::TSLData& t, double E, double T) {
    const std::vector<double>& Es = t.xs_E;
    const size_t E_hi_i = UpperIndex(Es, E);
    if (E_hi_i == Es.size()) return std::numeric_limits<double>::quiet_NaN();  // asserted by the reference
    const bool below_E_min = E_hi_i == 0;
    const size_t E_lo_i = below_E_min ? E_hi_i : E_hi_i - 1;
    size_t T_lo_i, T_hi_i;
    bool below_T_min, above_T_max;
    TBracket(t.xs_T, T, T_lo_i, T_hi_i, below_T_min, above_T_max);
    const double xs_E_lo_T_lo = EvaluateInelastic(t, E_lo_i, T_lo_i);
    const double xs_E_lo_T_hi = EvaluateInelastic(t, E_lo_i, T_hi_i);
    const double xs_E_hi_T_lo = EvaluateInelastic(t, E_hi_i, T_lo_i);
    const double xs_E_hi_T_hi = EvaluateInelastic(t, E_hi_i, T_hi_i);
    const double E_lo = Es[E_lo_i], E_hi = Es[E_hi_i];
    const double r_E = below_E_min ? 1 : (E - E_lo) / (E_hi - E_lo);
    const double xs_T_lo = xs_E_lo_T_lo + r_E * (xs_E_hi_T_lo - xs_E_lo_T_lo);
    const double xs_T_hi = xs_E_lo_T_hi + r_E * (xs_E_hi_T_hi - xs_E_lo_T_hi);
    const double T_lo = t.xs_T[T_lo_i], T_hi = t.xs_T[T_hi_i];
    const double r_T = below_T_min ? 1 : above_T_max ? 0 : (T - T_lo) / (T_hi - T_lo);
    return xs_T_lo + r_T * (xs_T_hi - xs_T_lo);
  }

  // partition holding global grid index i, and i within it
  static size_t Partition(const mc::PODPartitionSet& P, size_t i, size_t& local) {
    const size_t ps = static_cast<size_t>(std::upper_bound(P.ends.begin(), P.ends.end(), i) - P.ends.begin());
    local = ps == 0 ? i : i - P.ends[ps - 1];
    return ps;
  }

  // ThermalScattering::SampleBeta (src/ThermalScattering.cpp:271-338);
  // false when the resample limit is exceeded (the reference throws)
  static bool SampleBeta(const mc::TSLData& t, RNG& rng, double E, double T, double& beta) {
    const std::vector<double>& Es = t.beta.concat;
    const size_t E_hi_i = UpperIndex(Es, E);
    if (E_hi_i == Es.size()) return false;  // the reference asserts E < cutoff
    const double r = E_hi_i != 0 ? (E - Es[E_hi_i - 1]) / (Es[E_hi_i] - Es[E_hi_i - 1]) : 1;
    const size_t E_s_i = r <= std::uniform_real_distribution{}(rng) ? E_hi_i - 1 : E_hi_i;
    const double E_s = Es[E_s_i];
    size_t E_s_i_local;
    const size_t ps = Partition(t.beta, E_s_i, E_s_i_local);
    const std::vector<double>& Fs = t.beta.F[ps];
    for (size_t resamples = 0; resamples < 10; resamples++) {
      const double F = std::uniform_real_distribution{}(rng);
      const size_t F_hi_i = UpperIndex(Fs, F);
      const double F_lo = F_hi_i != 0 ? Fs[F_hi_i - 1] : 0;
      const double F_hi = F_hi_i != Fs.size() ? Fs[F_hi_i] : 1;
      const double b_lo = F_hi_i != 0 ? PODEvaluate(t.beta, ps, F_hi_i - 1, E_s_i_local, T) : -E_s / (kBoltzmann * T);
      const double b_hi = F_hi_i != Fs.size() ? PODEvaluate(t.beta, ps, F_hi_i, E_s_i_local, T) : t.beta_cutoff;
      const double b_prime = b_lo + (F - F_lo) / (F_hi - F_lo) * (b_hi - b_lo);
      const double b_min = -E / (kBoltzmann * T);
      if (b_min <= b_prime) {
        beta = b_prime;
        return true;
      }
    }
    return false;
  }

  // std::upper_bound over CDF indices [0, n) with the predicate a < Evaluate(i):
  // the standard library's bisection, so a non-monotone reconstruction
  // probes the same points
  static size_t UpperBoundAlpha(const mc::TSLData& t, size_t ps, size_t b_local, double T, size_t n, double a) {
    size_t first = 0, len = n;
    while (len > 0) {
      const size_t half = len >> 1, middle = first + half;
      if (a < PODEvaluate(t.alpha, ps, middle, b_local, T)) {
        len = half;
      }
      else {
        first = middle + 1;
        len = len - half - 1;
      }
    }
    return first;
  }

  // ThermalScattering::SampleAlpha (src/ThermalScattering.cpp:340-463),
  // including its interpolation factor as written (:363-365)
  static bool SampleAlpha(const mc::TSLData& t, RNG& rng, double b, double E, double T, double& alpha) {
    const double abs_b = std::abs(b);
    const int sgn_b = (0 < b) - (b < 0);
    const std::vector<double>& betas = t.alpha.concat;
    const size_t b_hi_i = UpperIndex(betas, abs_b);
    if (b_hi_i == betas.size()) return false;  // betas.at() throws in the reference
    const bool snap_to_lower = ((sgn_b == 1 && t.beta_cutoff <= betas[b_hi_i]) ||
                                (sgn_b == -1 && -betas[b_hi_i] < -E / (kBoltzmann * T)));
    const bool snap_to_min = b_hi_i == 0;
    const double r = snap_to_lower ? 0
                     : snap_to_min ? 1
                                   : (abs_b - betas[b_hi_i - 1] / (betas[b_hi_i] - betas[b_hi_i - 1]));
    const bool lower = r <= std::uniform_real_distribution{}(rng);
    if (lower && b_hi_i == 0) return false;  // betas.at(-1) throws in the reference
    const size_t b_s_i = lower ? b_hi_i - 1 : b_hi_i;
    const double b_s = sgn_b * betas[b_s_i];
    const double sqrt_E = std::sqrt(E);
    const double b_s_sqrt_E_bkT = std::sqrt(E + b_s * kBoltzmann * T);
    const double akT = t.awr * kBoltzmann * T;
    const double b_s_a_min = std::pow(sqrt_E - b_s_sqrt_E_bkT, 2) / akT;
    const double b_s_a_max = std::pow(sqrt_E + b_s_sqrt_E_bkT, 2) / akT;
    size_t b_s_i_local;
    const size_t ps = Partition(t.alpha, b_s_i, b_s_i_local);
    const std::vector<double>& Fs = t.alpha.F[ps];
    auto find_cdf = [&](double a) {
      const size_t F_a_hi_i = UpperBoundAlpha(t, ps, b_s_i_local, T, Fs.size(), a);
      const double F_a_lo = F_a_hi_i != 0 ? Fs[F_a_hi_i - 1] : 0;
      const double F_a_hi = F_a_hi_i != Fs.size() ? Fs[F_a_hi_i] : 1;
      const double a_lo = F_a_hi_i != 0 ? PODEvaluate(t.alpha, ps, F_a_hi_i - 1, b_s_i_local, T) : 0;
      const double a_hi = F_a_hi_i != Fs.size() ? PODEvaluate(t.alpha, ps, F_a_hi_i, b_s_i_local, T) : t.alpha_cutoff;
      return F_a_lo + (a - a_lo) * (F_a_hi - F_a_lo) / (a_hi - a_lo);
    };
    const double F_min = find_cdf(b_s_a_min);
    const double F_max = find_cdf(b_s_a_max);
    for (size_t resamples = 0; resamples < 10; resamples++) {
      const double F = F_min + std::uniform_real_distribution{}(rng) * (F_max - F_min);
      const size_t F_hi_i = UpperIndex(Fs, F);
      const double F_lo = F_hi_i != 0 ? Fs[F_hi_i - 1] : 0;
      const double F_hi = F_hi_i != Fs.size() ? Fs[F_hi_i] : 1;
      const double a_lo = F_hi_i != 0 ? PODEvaluate(t.alpha, ps, F_hi_i - 1, b_s_i_local, T) : 0;
      const double a_hi = F_hi_i != Fs.size() ? PODEvaluate(t.alpha, ps, F_hi_i, b_s_i_local, T) : t.alpha_cutoff;
      const double a_prime = a_lo + (F - F_lo) / (F_hi - F_lo) * (a_hi - a_lo);
      if (b_s_a_min < a_prime && a_prime < b_s_a_max) {
        const double b_sqrt_E_bkT = std::sqrt(E + b * kBoltzmann * T);
        const double b_a_min = std::pow(sqrt_E - b_sqrt_E_bkT, 2) / akT;
        const double b_a_max = std::pow(sqrt_E + b_sqrt_E_bkT, 2) / akT;
        alpha = b_a_min + (a_prime - b_s_a_min) * (b_a_max - b_a_min) / (b_s_a_max - b_s_a_min);
        return true;
      }
    }
    return false;
  }

  // ThermalScattering::Scatter (src/ThermalScattering.cpp:159-171)
  bool TSLScatter(const mc::TSLData& t, P& p, double T) const {
    const double E = p.E;
    double beta, alpha;
    if (!SampleBeta(t, p.rng, E, T, beta)) return false;
    if (!SampleAlpha(t, p.rng, beta, E, T, alpha)) return false;
    const double E_p = E + beta * kBoltzmann * T;
    const double mu = (E + E_p - alpha * t.awr * kBoltzmann * T) / (2 * std::sqrt(E * E_p));
    const double phi = 2 * kPi * std::uniform_real_distribution{}(p.rng);
    p.dir = Rotate(p.dir, mu, phi);
    p.E = E_p;
    return true;
  }

  // Continuous::Interact (src/Continuous.cpp:60-72)
  void CEInteract(int n, P& p) const {
    const mc::CEData& d = m.nuclides[n].ce[p.type];
    const double T = CellT(p);
    for (;;) {
      const double threshold = std::uniform_real_distribution{}(p.rng) * CETotal(d, p);
      double accumulated{0};
      for (const auto& r : d.reactions) {
        accumulated += ReactionXS(d, r, p, T);
        if (accumulated > threshold) {
          if (r.kind == mc::kCapture) {
            p.event = kCapture;
          }
          else if (r.kind == mc::kScatter) {
            if (TSLValid(r, p)) {
              p.event = kScatter;
              // the reference throws past the resample limits
              if (!TSLScatter(m.tsl[r.tsl], p, T)) {
                p.event = kLost;
                p.resample_failed = true;
              }
            }
            else {
              FreeGasScatter(d, p, T);
            }
          }
          else {
            CEFission(r, p);
          }
          return;
        }
      }
      // no reaction found: resample (tail recursion in the reference)
    }
  }

  // ContinuousScatter::Interact without a thermal scattering library
  // (src/ContinuousReaction.cpp:119-189): free-gas target velocity by
  // rejection, elastic scattering in the centre-of-mass frame
  void FreeGasScatter(const mc::CEData& d, P& p, double T) const {
    p.event = kScatter;
    const double awr = d.awr;
    constexpr double m_n = kNeutronMass;
    const double E = p.E;
    const double s_n = std::sqrt(2. * E / m_n);
    const Vec v_n = Scale(p.dir, s_n);
    const double beta = std::sqrt((awr * m_n) / (2. * kBoltzmann * T));
    const double y = beta * s_n;
    double x, mu;
    do {
      const double xi_1 = std::uniform_real_distribution{}(p.rng);
      const double xi_2 = std::uniform_real_distribution{}(p.rng);
      if (std::uniform_real_distribution{}(p.rng) < 2 / (std::sqrt(kPi) * y + 2)) {
        x = std::sqrt(-std::log(xi_1 * xi_2));
      }
      else {
        const double xi_3 = std::uniform_real_distribution{}(p.rng);
        const double z = std::cos(kPi * xi_3 / 2);
        x = std::sqrt(-std::log(xi_1) - std::log(xi_2) * z * z);
      }
      mu = 2 * std::uniform_real_distribution{}(p.rng) - 1;
    } while (std::uniform_real_distribution{}(p.rng) >= std::sqrt(x * x + y * y - 2 * x * y * mu) / (x + y));
    const double s_T = x / beta;
    const double phi = 2 * kPi * std::uniform_real_distribution{}(p.rng);
    const Vec v_T = Scale(Rotate(p.dir, mu, phi), s_T);
    const Vec num = Add(v_n, Scale(v_T, awr));
    const double den = 1 + awr;
    const Vec v_cm{num.x / den, num.y / den, num.z / den};
    const Vec V_n = Sub(v_n, v_cm);
    const double mu_cm = 2 * std::uniform_real_distribution{}(p.rng) - 1;
    const double phi_cm = 2 * kPi * std::uniform_real_distribution{}(p.rng);
    const Vec V_dir = Rotate(Normalized(V_n), mu_cm, phi_cm);
    const Vec V_prime = Scale(V_dir, std::sqrt(Dot(V_n, V_n)));
    const Vec v_prime = Add(V_prime, v_cm);
    const double E_prime = 0.5 * m_n * Dot(v_prime, v_prime);
    // Particle::Scatter (src/Particle.cpp:55-65)
    const double mu_lab = Dot(p.dir, Normalized(v_prime));
    const double phi_lab = 2 * kPi * std::uniform_real_distribution{}(p.rng);
    p.dir = Rotate(p.dir, mu_lab, phi_lab);
    p.E = E_prime;
  }

  // ContinuousFission::Interact (src/ContinuousReaction.cpp:252-265): the
  // secondaries keep the incident energy
  void CEFission(const mc::CEReaction& r, P& p) const {
    p.event = kFission;
    const size_t yield(MapAt(r.nubar, p.E) + std::uniform_real_distribution{}(p.rng));
    for (size_t i = 0; i < yield; i++) {
      const Vec dir = IsotropicDirection(p.rng);
      BankSecondaries(p, dir, p.g, p.E);
    }
  }

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

  void BankSecondaries(P& p, const Vec& dir, uint64_t g, double E = 0) const {
    P s;
    s.pos = p.pos;
    s.dir = dir;
    s.g = g;
    s.E = E;
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

  // EstimatorProxy::Score (src/Estimator.cpp:104-110): the estimator, then
  // each sensitivity, whose score is the indirect effect times the
  // estimator's (src/Sensitivity.cpp:55-58); ScorableProxy::Score skips
  // zero scores (src/Scorable.cpp:80-99)
  void Score(const P& p, std::map<size_t, double>& pending) const {
    if (p.event != kSurfaceCross && p.event != kLeak) return;
    for (size_t e = 0; e < m.estimators.size(); e++) {
      const auto& est = m.estimators[e];
      if (est.kind != mc::kCurrent || est.surface != p.surf) continue;
      const double score = 1;
      const size_t b = BinIndex(e, p);
      pending[offsets[e] + b] += score;
      for (size_t k = 0; k < est.sensitivities.size(); k++) {
        const double s = p.eff[est.sensitivities[k]] * score;
        if (s != 0) pending[offsets[e] + est.size() * (k + 1) + b] += s;
      }
    }
  }

  // TotalCrossSectionPerturbation::Stream (src/Perturbation.cpp:68-78),
  // accumulated by Particle::Stream before the move (src/Particle.cpp:46-50)
  void Indirect(P& p, int mat, double cpd, double d) const {
    for (size_t k = 0; k < m.perturbations.size(); k++) {
      const auto& nucs = m.materials[mat].nuclides;
      if (std::find(nucs.begin(), nucs.end(), m.perturbations[k].nuclide) == nucs.end()) continue;
      p.eff[k] += 1 / cpd - d;
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
    uint64_t events = 0, lost = 0, capped = 0, resample = 0;
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
    // Particle::SetPerturbations before each particle's transport
    // (src/FixedSource.cpp:63-65)
    for (double& e : p.eff) e = 0;
    while (p.event != kCapture && p.event != kLeak && p.event != kFission && p.event != kLost) {
      const int mat = m.cells[p.cell].material;
      // GetCollisionProbabilityDensity: total (surface tracking) or
      // majorant (delta tracking), src/TransportMethod.cpp:79-82,124-127
      const double cpd = delta ? MaterialMajorant(mat, p) : MaterialTotal(mat, p);
      const double distance_to_collision =
          std::exponential_distribution{m.materials[mat].number_density * cpd}(p.rng);
      double dsurf;
      const int s = NearestSurface(p.cell, p.pos, p.dir, dsurf, p.skip);
      const bool collide = delta ? !(dsurf < distance_to_collision) : distance_to_collision < dsurf;
      if (collide) {
        if (score) ScoreTrack(p, distance_to_collision, pending);
        st.ktl += distance_to_collision * m.materials[mat].number_density * NuSigmaF(mat, p);
        if (delta && !std::bernoulli_distribution{MaterialTotal(mat, p) / cpd}(p.rng)) {
          // virtual collision (src/TransportMethod.cpp:111-115)
          Indirect(p, mat, cpd, distance_to_collision);
          Stream(p, distance_to_collision);
          p.event = kVirtual;
        }
        else {
          Indirect(p, mat, cpd, distance_to_collision);
          Stream(p, distance_to_collision);
          p.skip = -1;
          const int n = SampleNuclide(p);
          if (m.energy_mode == mc::kMultigroup) MGInteract(n, p);
          else CEInteract(n, p);
          if (p.event == kLost) (p.resample_failed ? st.resample : st.lost)++;
        }
      }
      else if (m.surfaces[s].reflective) {
        if (score) ScoreTrack(p, dsurf, pending);
        st.ktl += dsurf * m.materials[mat].number_density * NuSigmaF(mat, p);
        Indirect(p, mat, cpd, dsurf);
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
        Indirect(p, mat, cpd, d);
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

  // sum of afrac * nubar * sigma_f (the k track-length estimator, an extension)
  double NuSigmaF(int mat, const P& p) const {
    const mc::Material& M = m.materials[mat];
    double acc = 0;
    for (size_t k = 0; k < M.nuclides.size(); k++) {
      if (m.energy_mode == mc::kMultigroup) {
        const mc::MGData& d = m.nuclides[M.nuclides[k]].mg[p.type];
        if (d.has_fission) acc = acc + M.afrac[k] * (d.nubar[p.g - 1] * d.fission[p.g - 1]);
      }
      else {
        for (const auto& r : m.nuclides[M.nuclides[k]].ce[p.type].reactions)
          if (r.kind == mc::kFission && r.has_nubar) acc = acc + M.afrac[k] * (MapAt(r.nubar, p.E) * MapAt(r.eval.xs, p.E));
      }
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
  uint64_t resample;
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
    off += e.span();
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
  p.cell = cell;
  return o->MaterialTotal(mat, p);
}

// Material::GetMicroscopicTotal and GetMicroscopicMajorant of neutrons of
// continuous energies E[i] at points xyz[i] of cell c
int orc_material_xs_ce(void* h, int32_t cell, const double* E, const double* xyz, uint64_t n, double* total,
                       double* majorant) {
  auto* o = static_cast<Oracle*>(h);
  if (o->m.energy_mode != mc::kContinuous) return -1;
  const int mat = o->m.cells.at(cell).material;
  if (mat < 0) return -1;
  for (uint64_t i = 0; i < n; i++) {
    Oracle::P p;
    p.type = 0;
    p.cell = cell;
    p.E = E[i];
    p.pos = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    total[i] = o->MaterialTotal(mat, p);
    majorant[i] = o->MaterialMajorant(mat, p);
  }
  return 0;
}

// std::map::upper_bound positions in the energy tables of nuclide `nuc`:
// out[i * 6 + t] for t = total, then each reaction in input order, then
// nubar (-1 where absent)
int orc_energy_index(void* h, int32_t nuc, const double* E, uint64_t n, int64_t* out) {
  auto* o = static_cast<Oracle*>(h);
  if (o->m.energy_mode != mc::kContinuous) return -1;
  const mc::CEData& d = o->m.nuclides.at(nuc).ce[0];
  std::vector<std::map<double, double>> maps;
  std::vector<const mc::Table1D*> tabs{&d.total.xs};
  for (const auto& r : d.reactions) tabs.push_back(&r.eval.xs);
  for (const auto& r : d.reactions)
    if (r.has_nubar) tabs.push_back(&r.nubar);
  for (const auto* t : tabs) {
    std::map<double, double> mp;
    for (size_t i = 0; i < t->x.size(); i++) mp[t->x[i]] = t->y[i];
    maps.push_back(std::move(mp));
  }
  // the position of map::upper_bound is that of std::upper_bound over the
  // map's (sorted, unique) keys; walking the map iterator would be linear
  std::vector<std::vector<double>> keys;
  for (const auto& mp : maps) {
    std::vector<double> k;
    k.reserve(mp.size());
    for (const auto& kv : mp) k.push_back(kv.first);
    keys.push_back(std::move(k));
  }
  for (uint64_t i = 0; i < n; i++) {
    for (size_t t = 0; t < 6; t++) {
      if (t >= keys.size()) {
        out[i * 6 + t] = -1;
        continue;
      }
      const auto it = std::upper_bound(keys[t].begin(), keys[t].end(), E[i]);
      out[i * 6 + t] = static_cast<int64_t>(it - keys[t].begin());
    }
  }
  return 0;
}

// ContinuousScatter::Interact's free-gas kinematics for n neutrons of
// energy E moving along +x, particle i seeded with seed + i: outgoing
// energies and lab cosines
void orc_free_gas(double awr, double T, double E, uint64_t n, uint64_t seed, double* E_out, double* mu_out) {
  Oracle o;
  mc::CEData d;
  d.awr = awr;
  for (uint64_t i = 0; i < n; i++) {
    Oracle::P p;
    p.E = E;
    p.dir = {1, 0, 0};
    p.rng.seed(static_cast<RNG::result_type>(seed + i));
    o.FreeGasScatter(d, p, T);
    E_out[i] = p.E;
    mu_out[i] = p.dir.x;
  }
}

// ThermalScattering::SampleBeta then SampleAlpha for (E[i], T[i]), sample i
// drawing from minstd seeded with seed + i; NaN and a count on failure
int orc_sample_tsl(void* h, int32_t tsl, const double* E, const double* T, uint64_t n, uint64_t seed, double* beta,
                   double* alpha, uint64_t* failures) {
  auto* o = static_cast<Oracle*>(h);
  if (tsl < 0 || static_cast<size_t>(tsl) >= o->m.tsl.size()) return -1;
  const mc::TSLData& t = o->m.tsl[static_cast<size_t>(tsl)];
  uint64_t fails = 0;
  for (uint64_t i = 0; i < n; i++) {
    RNG rng{static_cast<RNG::result_type>(seed + i)};
    double b = std::numeric_limits<double>::quiet_NaN(), a = b;
    if (!Oracle::SampleBeta(t, rng, E[i], T[i], b) || !Oracle::SampleAlpha(t, rng, b, E[i], T[i], a)) {
      fails++;
      if (!(b == b) || a != a) a = std::numeric_limits<double>::quiet_NaN();
    }
    beta[i] = b;
    alpha[i] = a;
  }
  if (failures) *failures = fails;
  return 0;
}

// ThermalScattering::GetTotal at (E[i], T[i])
int orc_tsl_total(void* h, int32_t tsl, const double* E, const double* T, uint64_t n, double* out) {
  auto* o = static_cast<Oracle*>(h);
  if (tsl < 0 || static_cast<size_t>(tsl) >= o->m.tsl.size()) return -1;
  for (uint64_t i = 0; i < n; i++) out[i] = Oracle::TSLTotal(o->m.tsl[static_cast<size_t>(tsl)], E[i], T[i]);
  return 0;
}

// Reorders the nuclides of material `mat` (names separated by spaces) and
// renormalizes its atom fractions summed in that order.  The reference
// iterates a material's nuclides in std::map order of their shared_ptr
// addresses (src/Material.hpp:20), i.e. in the order its process happened to
// allocate them; comparisons with the reference's own code set that order.
int orc_set_material_order(void* h, int32_t mat, const char* names) {
  auto* o = static_cast<Oracle*>(h);
  if (mat < 0 || static_cast<size_t>(mat) >= o->m.materials.size()) return -1;
  mc::Material& M = o->m.materials[static_cast<size_t>(mat)];
  std::vector<int32_t> order;
  std::string s(names), tok;
  size_t pos = 0;
  while (pos <= s.size()) {
    const size_t e = s.find(' ', pos);
    tok = s.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
    if (!tok.empty()) {
      int32_t idx = -1;
      for (size_t k = 0; k < M.nuclides.size(); k++)
        if (o->m.nuclides[static_cast<size_t>(M.nuclides[k])].name == tok) idx = static_cast<int32_t>(k);
      if (idx < 0) return -2;
      order.push_back(idx);
    }
    if (e == std::string::npos) break;
    pos = e + 1;
  }
  if (order.size() != M.nuclides.size()) return -3;
  std::vector<int32_t> nuc;
  std::vector<double> raw;
  for (int32_t k : order) {
    nuc.push_back(M.nuclides[static_cast<size_t>(k)]);
    raw.push_back(M.afrac_raw[static_cast<size_t>(k)]);
  }
  double sum = 0;
  for (double v : raw) sum += v;
  M.nuclides = nuc;
  M.afrac_raw = raw;
  M.afrac.clear();
  for (double v : raw) M.afrac.push_back(v / sum);
  return 0;
}

int32_t orc_cell_material(void* h, int32_t cell) {
  auto* o = static_cast<Oracle*>(h);
  if (cell < 0 || static_cast<size_t>(cell) >= o->m.cells.size()) return -1;
  return o->m.cells[static_cast<size_t>(cell)].material;
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
      stats->resample += st[t].resample;
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
  threads = std::max(1, threads);
  const size_t nb = std::max<size_t>(1, o->m.total_bins());
  std::vector<std::vector<double>> ts(threads, std::vector<double>(nb, 0)), tq(threads, std::vector<double>(nb, 0));
  std::vector<Oracle::Stats> st(threads);
  struct SiteRec {
    Vec pos, dir;
    uint64_t g;
    double E;
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
        p.E = source[j].E;
        p.type = 0;
        p.rng.seed(static_cast<RNG::result_type>(seed + static_cast<uint64_t>(c) * N + j));
      }
      std::map<size_t, double> pending;
      Oracle::Stats& s = st[tid];
      const double k0 = s.ktl;
      o->Transport(p, pending, s, act, 1000000u, nullptr);
      ktl[tid] += s.ktl - k0;
      per_hist[j].clear();
      for (const auto& q : p.secondaries) per_hist[j].push_back({q.pos, q.dir, q.g, q.E});
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
      stats->resample += st[t].resample;
    }
    stats->seconds = secs;
    stats->k_tracklength = active ? ktl_active / active : 0;
  }
  return 0;
}

}  // extern "C"
