// Per-particle helpers shared by the history-schedule transport kernels
// (multigroup: mc_transport.cu, continuous energy: mc_transport_ce.cu).
#pragma once

#include "mc_kernels.cuh"

#include <type_traits>

namespace mcd {
namespace hist {

constexpr int kStack = 32;    // fixed-source secondaries per history in flight
constexpr int kPending = 24;  // distinct tally bins per history

template <class Rng>
struct Particle {
  double x, y, z, u, v, w;
  int g;          // multigroup group, 0-based
  double E;       // continuous energy, MeV
  int j;          // continuous energy: union-grid upper_bound index of E
  int cell;
  int surf;       // last surface crossed (current estimator)
  int skip;       // robust crossing: surface just left, ignored until the next collision
  int event;
  int type;
  uint32_t nev;
  double eff[kMaxPert];  // indirect effect of each perturbation (Particle::indirect_effects)
  Rng rng;
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// start a particle from the problem's Source (src/Source.cpp:143-154)
template <class Rng>
__device__ __forceinline__ void sample_source(const DevWorld& w, const RunParams& rp, unsigned long long i,
                                              Particle<Rng>& p) {
  p.x = w.src_pos[0];
  p.y = w.src_pos[1];
  p.z = w.src_pos[2];
  p.type = w.src_type;
  if constexpr (std::is_same_v<Rng, MinstdRng>) {
    // Source::Sample(seed): a fresh RNG{seed} samples position, direction,
    // energy and type in that order, then the particle is seeded with rng()
    MinstdRng s;
    s.seed(rp.ref_source_seeds ? rp.seed + i : i + 1);
    if (w.src_dir_kind == 0) {
      p.u = w.src_dir[0];
      p.v = w.src_dir[1];
      p.w = w.src_dir[2];
    }
    else if (w.src_dir_kind == 1) {
      isotropic(s, p.u, p.v, p.w);
    }
    else {
      // IsotropicFlux::Sample (src/Source.cpp:113-120)
      const double mu = __dsqrt_rn(s.u01());
      const double phi = dadd(dmul(s.u01(), 2 * kPi), 0.0);
      p.u = w.src_dir[0];
      p.v = w.src_dir[1];
      p.w = w.src_dir[2];
      rotate(p.u, p.v, p.w, mu, phi);
    }
    p.rng.seed(s.next());
  }
  else {
    p.rng.init(rp.run_key, i, 0);
    if (w.src_dir_kind == 0) {
      p.u = w.src_dir[0];
      p.v = w.src_dir[1];
      p.w = w.src_dir[2];
    }
    else if (w.src_dir_kind == 1) {
      if (rp.fast) isotropic_fast(p.rng, p.u, p.v, p.w);
      else isotropic(p.rng, p.u, p.v, p.w);
    }
    else {
      const double mu = sqrt(p.rng.u01());
      const double phi = 2 * kPi * p.rng.u01();
      p.u = w.src_dir[0];
      p.v = w.src_dir[1];
      p.w = w.src_dir[2];
      rotate(p.u, p.v, p.w, mu, phi);
    }
  }
  if (w.energy_mode == 0) p.g = static_cast<int>(w.src_energy) - 1;
  else p.E = w.src_energy;
}

template <class Rng>
__device__ __forceinline__ void start_from_site(const RunParams& rp, unsigned long long i, const Site& s,
                                                Particle<Rng>& p, int energy_mode) {
  p.x = s.x;
  p.y = s.y;
  p.z = s.z;
  p.u = s.u;
  p.v = s.v;
  p.w = s.w;
  if (energy_mode == 0) p.g = static_cast<int>(s.energy) - 1;
  else p.E = s.energy;
  p.type = 0;
  if constexpr (std::is_same_v<Rng, MinstdRng>) {
    // k-eigenvalue sources: particle i of a cycle is seeded with base + i;
    // mc_transport_bank passes the site's own key
    p.rng.seed(rp.minstd_base ? rp.minstd_base + i : s.key);
  }
  else {
    if (rp.minstd_base) p.rng.init(rp.run_key, i, 0);
    else p.rng.init(rp.run_key, s.key, 1);
  }
}

template <class Rng>
__device__ __forceinline__ double uniform(Rng& rng, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return static_cast<double>(rng.u01f());
  }
  return rng.u01();
}

// exponential_distribution{sigma}: -log(1 - U) / sigma
template <class Rng>
__device__ __forceinline__ double sample_flight(Rng& rng, double sigma, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return flight_fast(rng.u01f(), sigma);
  }
  return ddiv(-log(dsub(1.0, rng.u01())), sigma);
}

template <class Rng>
__device__ __forceinline__ void sample_isotropic(Rng& rng, double& u, double& v, double& w, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) {
      isotropic_fast(rng, u, v, w);
      return;
    }
  }
  isotropic(rng, u, v, w);
}

// the same with the direction's FP32 copy (no conversions in the fast form)
template <class Rng>
__device__ __forceinline__ void sample_isotropic(Rng& rng, double& u, double& v, double& w, float& fu, float& fv,
                                                 float& fw, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) {
      isotropic_fast(rng, u, v, w, fu, fv, fw);
      return;
    }
  }
  isotropic(rng, u, v, w);
  fu = __double2float_rn(u);
  fv = __double2float_rn(v);
  fw = __double2float_rn(w);
}

// first index k in [0, n) with cdf[k] > threshold, or -1
__device__ __forceinline__ int cdf_search(const double* cdf, int n, int, double threshold) {
  return cdf_first_above(cdf, n, threshold);
}

// score helpers -----------------------------------------------------------

template <class Rng>
__device__ __forceinline__ double energy_value(const DevWorld& w, const Particle<Rng>& p) {
  // ParticleBins::VisitEnergy: group number or energy
  return w.energy_mode == 0 ? static_cast<double>(p.g + 1) : p.E;
}

// Per-history scores go to the history's row of a dense array (few bins,
// committed by a separate kernel) or to a per-thread list (many bins).
// FP64 reduction into global memory marked evict-first in L2: the dense
// score array streams through L2 (it is read back once, by the commit), so
// it should not push out the bank and the fission records the next kernels
// read.  The slot belongs to this thread's history and only a later kernel
// reads it, so the reduction needs no ordering against this thread's other
// memory operations (no memory clobber).  The multigroup kernel uses it
// (2.7 % off the two-zone cycle); in the continuous-energy kernel the same
// code measured 1 % slower, so that kernel keeps the plain atomic.
__device__ __forceinline__ void red_add_evict_first(double* p, double v) {
  asm volatile(
      "{\n\t.reg .b64 pol;\n\t"
      "createpolicy.fractional.L2::evict_first.b64 pol, 1.0;\n\t"
      "red.global.add.L2::cache_hint.f64 [%0], %1, pol;\n\t}" ::"l"(p),
      "d"(v));
}

template <bool EVICT_FIRST>
struct ScorerT {
  Pending<kPending>* list;
  double* dense;                // this history's column of the bin-major array
  unsigned long long stride;    // histories per bin row
  __device__ __forceinline__ void add(uint32_t b, double s) {
    if (dense) {
      if constexpr (EVICT_FIRST) red_add_evict_first(dense + b * stride, s);
      else atomicAdd(dense + b * stride, s);
    }
    else {
      list->add(b, s);
    }
  }
};
using Scorer = ScorerT<false>;

// ParticleBins::GetIndex of the particle: group form (multigroup) or
// energy form (continuous energy)
template <bool CE, class Rng>
__device__ __forceinline__ uint64_t bin_of(const DevWorld& w, int e, const Particle<Rng>& p) {
  if constexpr (CE) return particle_bin(w, e, p.u, p.v, p.w, p.E);
  else return particle_bin_mg(w, e, p.u, p.v, p.w, p.g);
}

// EstimatorSetProxy::Score (src/Estimator.cpp:247-251) for the current
// estimator (src/Estimator.cpp:142-151): 1 on a crossing of its surface.
// With PERT, each of its sensitivities scores the particle's indirect effect
// times that 1 into the same bin of its own block
// (CurrentTotalCrossSectionSensitivity::GetScore, src/Sensitivity.cpp:55-58);
// zero scores are skipped as ScorableProxy::Score does.
template <bool CE = false, bool PERT = false, class Rng, class S>
__device__ __forceinline__ void score_event(const DevWorld& w, const Particle<Rng>& p, S& sc) {
  if (p.event != kSurfaceCross && p.event != kLeak) return;
  for (int e = 0; e < w.n_est; e++) {
    if (__ldg(w.est_kind + e) != 0 || __ldg(w.est_target + e) != p.surf) continue;
    const uint64_t b = __ldg(w.est_offset + e) + bin_of<CE>(w, e, p);
    sc.add(static_cast<uint32_t>(b), 1.0);
    if constexpr (PERT) {
      const int ns = __ldg(w.est_nsens + e);
      const uint64_t size = __ldg(w.est_size + e);
      for (int k = 0; k < ns; k++) {
        const int q = __ldg(w.est_sens + e * kMaxSens + k);
        double s = 0;
#pragma unroll
        for (int j = 0; j < kMaxPert; j++)
          if (j == q) s = p.eff[j];
        if (s != 0) sc.add(static_cast<uint32_t>(b + size * static_cast<uint64_t>(k + 1)), s);
      }
    }
  }
}

// Perturbation::Stream of each perturbation before the particle moves d
// (src/Particle.cpp:46-50, src/Perturbation.cpp:68-78): where the cell's
// material holds the perturbed nuclide, the indirect effect grows by
// 1 / cpd - d, cpd being the microscopic collision probability density the
// flight was sampled with (total, or majorant under delta tracking)
template <bool PERT, class Rng>
__device__ __forceinline__ void indirect_stream(const DevWorld& w, Particle<Rng>& p, int m, double cpd, double d) {
  if constexpr (PERT) {
    const int mask = __ldg(w.mat_pert + m);
    if (mask) {
      const double r = dsub(ddiv(1.0, cpd), d);
#pragma unroll
      for (int k = 0; k < kMaxPert; k++)
        if ((mask >> k) & 1) p.eff[k] = dadd(p.eff[k], r);
    }
  }
}

// Particle::SetPerturbations (src/Particle.cpp:71-73): every particle of a
// history, secondaries included, starts with no indirect effect
template <bool PERT, class Rng>
__device__ __forceinline__ void reset_indirect(Particle<Rng>& p) {
  if constexpr (PERT) {
#pragma unroll
    for (int k = 0; k < kMaxPert; k++) p.eff[k] = 0;
  }
}

// track-length estimator (extension): flight length inside the cell
template <bool CE = false, class Rng, class S>
__device__ __forceinline__ void score_track(const DevWorld& w, const Particle<Rng>& p, double d, S& sc) {
  for (int e = 0; e < w.n_est; e++) {
    if (__ldg(w.est_kind + e) != 1 || __ldg(w.est_target + e) != p.cell) continue;
    const uint64_t b = __ldg(w.est_offset + e) + bin_of<CE>(w, e, p);
    sc.add(static_cast<uint32_t>(b), d);
  }
}

__device__ __forceinline__ void stream(double& x, double& y, double& z, double u, double v, double w, double d) {
  // Particle::Stream (src/Particle.cpp:46-53): position += direction * d
  x = dadd(x, dmul(u, d));
  y = dadd(y, dmul(v, d));
  z = dadd(z, dmul(w, d));
}

// block-shared tally cache for problems with few bins
constexpr int kSharedBins = 512;

struct TallySink {
  double* ssum;  // shared or nullptr
  double* ssq;
  double* gsum;
  double* gsq;
  __device__ __forceinline__ void commit(const Pending<kPending>& pend) {
    for (int i = 0; i < pend.n; i++) {
      const double s = pend.score[i];
      const uint32_t b = pend.bin[i];
      if (ssum) {
        atomicAdd(ssum + b, s);
        atomicAdd(ssq + b, s * s);
      }
      else {
        atomicAdd(gsum + b, s);
        atomicAdd(gsq + b, s * s);
      }
    }
  }
};

}  // namespace hist
}  // namespace mcd
