// Continuous-energy history kernel: SurfaceTracking / CellDeltaTracking
// ::Transport (src/TransportMethod.cpp:52-127) with Continuous physics
// (src/Continuous.cpp:26-72, src/ContinuousReaction.cpp:45-265).
//
// The schedule is the multigroup history kernel's (mc_transport.cu): a
// persistent grid, one particle per thread, warp-collective refill from a
// global history queue.  Per particle the union-grid index of the current
// energy is kept in a register and recomputed only when the energy changes.
//
// Cross sections come from one of two forms (mc_ce.cuh): the exact FP64
// tables (reference rounding; always with the minstd stream) or, for Philox
// streams in fast mode when no cross section depends on temperature, the
// FP32 union tables, with free-gas kinematics in FP32.
#pragma once

#include "mc_ce.cuh"
#include "mc_history.cuh"

#include <type_traits>

namespace mcd {

using namespace hist;

// Each translation unit that includes this header instantiates its own
// subset of the kernel's variants (internal linkage), so that the variants
// compile in parallel.
namespace {

constexpr int kInteractTries = 64;  // Continuous::Interact resampling bound

// k-eigenvalue fission records keep the incident energy (the sites inherit
// it, src/ContinuousReaction.cpp:258-264) in the slot the multigroup path
// uses for its chi row
__device__ __forceinline__ void set_record_energy(FissionRec& f, double E) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(E));
  f.chi_index = static_cast<uint32_t>(b);
  f.pad = static_cast<uint32_t>(b >> 32);
}
__device__ __forceinline__ double record_energy(const FissionRec& f) {
  return __longlong_as_double(static_cast<long long>(static_cast<unsigned long long>(f.chi_index) |
                                                     (static_cast<unsigned long long>(f.pad) << 32)));
}

template <class Rng>
constexpr bool is_philox() {
  return std::is_same_v<Rng, PhiloxRng>;
}

// Particle::SampleNuclide (src/Particle.cpp:110-124): index within the
// material's nuclide list
template <class Rng>
__device__ __forceinline__ int ce_sample_nuclide(const DevWorld& w, Particle<Rng>& p, int m, bool fx,
                                                 const UnionPos& up, bool fast, TslMemo* memo) {
  const int nb = __ldg(w.mat_begin + m), K = __ldg(w.mat_begin + m + 1) - nb;
  if (fx) {
    const size_t row = static_cast<size_t>(p.type * w.n_materials + m) * w.ce.nu;
    const float* ra = w.ce.mat_ncdf + (row + up.jl) * w.ce.kmax;
    const float* rb = w.ce.mat_ncdf + (row + up.jh) * w.ce.kmax;
    const float thr = __fmul_rn(lerpf(__ldg(ra + K - 1), __ldg(rb + K - 1), up.f), p.rng.u01f());
    for (int k = 0; k < K - 1; k++)
      if (lerpf(__ldg(ra + k), __ldg(rb + k), up.f) > thr) return k;
    return K - 1;
  }
  const double T = cell_temperature(w, p.cell, p.x, p.y, p.z);
  const double thr = dmul(ce_material_micro(w, m, p.type, p.j, p.E, T, T, false, memo), uniform(p.rng, fast));
  double acc = 0;
  for (int k = 0; k < K; k++) {
    const int nuc = __ldg(w.mat_nuc + nb + k);
    acc = dadd(acc, dmul(__ldg(w.mat_afrac + nb + k),
                         ce_nuclide_total(w, ce_desc(w, p.type, nuc), p.type, p.j, p.E, T, T, false, memo)));
    if (acc > thr) return k;
  }
  return K - 1;  // unreachable in the reference (assert)
}

// Continuous::Interact's reaction choice (src/Continuous.cpp:60-72):
// reaction slot, or -1 if the resampling bound was hit
template <class Rng>
__device__ __forceinline__ int ce_pick_reaction(const DevWorld& w, Particle<Rng>& p, int nuc,
                                                const mc::CENuclideDesc& d, bool fx, const UnionPos& up, bool fast,
                                                TslMemo* memo) {
  if (fx) {
    const size_t row = static_cast<size_t>(p.type * w.n_nuclides + nuc) * w.ce.nu;
    const float4 a = __ldg(w.ce.nuc_rx + row + up.jl), b = __ldg(w.ce.nuc_rx + row + up.jh);
    const float c0 = lerpf(a.x, b.x, up.f), c1 = lerpf(a.y, b.y, up.f), c2 = lerpf(a.z, b.z, up.f);
    const float tot = lerpf(a.w, b.w, up.f);
    for (int it = 0; it < kInteractTries; it++) {
      const float thr = __fmul_rn(p.rng.u01f(), tot);
      if (c0 > thr) return 0;
      if (c1 > thr) return 1;
      if (c2 > thr) return 2;
    }
    return -1;
  }
  const double T = cell_temperature(w, p.cell, p.x, p.y, p.z);
  const double total = ce_nuclide_total(w, d, p.type, p.j, p.E, T, T, false, memo);
  for (int it = 0; it < kInteractTries; it++) {
    const double thr = dmul(uniform(p.rng, fast), total);
    double acc = 0;
    for (int k = 0; k < d.n_rx; k++) {
      acc = dadd(acc, ce_reaction_xs(w, d, k, p.type, p.j, p.E, T, T, false, memo));
      if (acc > thr) return k;
    }
  }
  return -1;
}

template <class Rng>
__device__ __forceinline__ double ce_nubar(const DevWorld& w, const Particle<Rng>& p, int nuc,
                                           const mc::CENuclideDesc& d, int k, bool fx, const UnionPos& up) {
  if (fx) {
    const float* nb = w.ce.nuc_nubar + static_cast<size_t>(p.type * w.n_nuclides + nuc) * w.ce.nu;
    return static_cast<double>(lerpf(__ldg(nb + up.jl), __ldg(nb + up.jh), up.f));
  }
  return ce_table_at(w.ce, d.rx_nubar[k], p.j, p.E);
}

// ---------------------------------------------------------------------------
// FX: FP32 union tables (launched only for Philox streams in fast mode when
// the tables are valid); otherwise the exact tables, with FP32 free-gas
// kinematics when the stream is Philox in fast mode
// TQ: thermal-scatter queue (ParkRec in mc_kernels.cuh): thermal scatters
// inside the surrogate's box park the particle for a batched sampler
// launch; a launch with rp.n_resume set continues parked particles instead
// of starting histories
template <class Rng, bool KEIG, int MINB, bool FX, bool PERT = false, bool TQ = false>
__global__ void __launch_bounds__(256, MINB) k_history_ce(const DevWorld w, const RunParams rp) {
  static_assert(!(PERT && (FX || KEIG)), "indirect effects need the exact tables of a fixed-source run");
  static_assert(!TQ || (is_philox<Rng>() && !KEIG && !FX && !PERT), "the thermal queue serves Philox fixed source");
  extern __shared__ double smem[];
  const bool use_smem = rp.total_bins <= kSharedBins && rp.score && !rp.nb;
  TallySink sink{use_smem ? smem : nullptr, use_smem ? smem + kSharedBins : nullptr, rp.tally_sum, rp.tally_sq};
  if (use_smem) {
    for (int i = threadIdx.x; i < 2 * kSharedBins; i += blockDim.x) smem[i] = 0;
    __syncthreads();
  }
  const unsigned lane = lane_id();
  const bool fast = rp.fast != 0;
  constexpr bool fx = FX;
  const bool ffg = FX || (is_philox<Rng>() && fast);
  Particle<Rng> p;
  Pending<kPending> pend;
  pend.clear();
  Scorer sc{&pend, nullptr, rp.n};
  Site stack[KEIG ? 1 : kStack];
  int sp = 0;
  bool alive = false, done = false;
  unsigned long long hist = 0;
  unsigned long long my_events = 0, my_lost = 0, my_capped = 0, my_overflow = 0, my_sec = 0, my_resample = 0;
  double my_ktl = 0;
  uint32_t hist_nev = 0;
  int8_t fate = 0;
  bool dropped = false;  // a secondary did not fit the stack (see the multigroup kernel)
  bool parked = false;  // this event parked the particle on the thermal queue
  TslMemo memo;         // the last thermal-scattering total evaluated
  memo.fast32 = ffg;
  unsigned long long* const head = (TQ && rp.head) ? rp.head : &rp.ctr->next;
  const bool resume = TQ && rp.n_resume != nullptr;
  const unsigned long long n_queue =
      resume ? (*rp.n_resume < rp.park_cap ? *rp.n_resume : rp.park_cap) : rp.n;

  auto finish_history = [&]() {
    if (rp.score && !rp.nb) {
      sink.commit(pend);
      if (pend.overflow) my_overflow++;
    }
    pend.clear();
    if (rp.hist_events) rp.hist_events[hist] = hist_nev;
    if (rp.hist_fate) rp.hist_fate[hist] = fate;
  };
  auto mark_lost = [&]() {
    rp.ctr->lost_xyz[0] = p.x;
    rp.ctr->lost_xyz[1] = p.y;
    rp.ctr->lost_xyz[2] = p.z;
  };

  for (;;) {
    // ---- refill: lanes without a live particle take the next history
    const bool want = !alive && !done;
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (mask) {
      const int leader = __ffs(mask) - 1;
      unsigned long long base = 0;
      if (lane == static_cast<unsigned>(leader)) base = atomicAdd(head, static_cast<unsigned long long>(__popc(mask)));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (want) {
        const unsigned long long qi = base + __popc(mask & ((1u << lane) - 1u));
        hist = qi;
        if (qi >= n_queue) {
          done = true;
        }
        else if (resume) {
          if constexpr (TQ) {
            // a parked particle: restore it and apply its sampled scatter
            const ParkRec& R = rp.park_in[qi];
            p.x = R.x;
            p.y = R.y;
            p.z = R.z;
            p.u = R.u;
            p.v = R.v;
            p.w = R.w;
            p.E = R.E;
            p.cell = R.cell;
            p.surf = R.surf;
            p.skip = R.skip;
            p.type = R.type;
            p.nev = R.nev;
            p.rng.restore(rp.run_key, R.rng_id, R.rng_tag, R.rng_pos);
            hist = R.hist;
            hist_nev = R.hist_nev;
            fate = static_cast<int8_t>(R.fate);
            dropped = (R.flags & 1) != 0;
            sp = 0;
            pend.clear();
            for (int k = 0; k < (R.pend_n & 0xff); k++) pend.add(R.pend_bin[k], R.pend_score[k]);
            pend.overflow = ((R.pend_n >> 8) & 1) != 0;
            sc.dense = rp.nb ? rp.pend + hist : nullptr;
            const DevTSL& tl = w.tsl[R.tsl];
            bool ok = false;
            if (rp.tq_mode >= 2) {
              // a POD-exact sample (guided or plain queue): continue the
              // particle's stream after the sampler's draws and apply the
              // kinematics exactly as the inline sampler does
              const GuideOut go = rp.tq_res[qi];
              p.rng.restore(rp.run_key, R.rng_id, R.rng_tag, go.rng_pos);
              if (go.ok) {
                if (rp.tq_fast) tsl_apply<true>(tl, p.rng, R.T, go.beta, go.alpha, p.E, p.u, p.v, p.w);
                else tsl_apply<false>(tl, p.rng, R.T, go.beta, go.alpha, p.E, p.u, p.v, p.w);
                ok = true;
              }
            }
            else {
              const float2 ba = rp.tq_out[qi];
              if (isfinite(ba.x) && isfinite(ba.y)) {
                // ThermalScattering::Scatter's kinematics (src/ThermalScattering.cpp:159-171);
                // the outgoing energy in FP64, the cosine and the rotation in
                // FP32 in fast mode (the surrogate's (beta, alpha) are FP32)
                const double kT = kBoltzmann * R.T;
                const double Ep = p.E + static_cast<double>(ba.x) * kT;
                if (Ep > 0) {
                  if (ffg) {
                    const float num = __double2float_rn(p.E + Ep - static_cast<double>(ba.y) * tl.awr * kT);
                    const float mu =
                        fminf(1.0f, fmaxf(-1.0f, __fdiv_rn(num, 2.0f * __fsqrt_rn(__double2float_rn(p.E * Ep)))));
                    float dx = static_cast<float>(p.u), dy = static_cast<float>(p.v), dz = static_cast<float>(p.w);
                    rotate_f(dx, dy, dz, mu, p.rng.u01f());
                    p.u = dx;
                    p.v = dy;
                    p.w = dz;
                  }
                  else {
                    const double mu = fmin(1.0, fmax(-1.0, (p.E + Ep - static_cast<double>(ba.y) * tl.awr * kT) /
                                                               (2.0 * sqrt(p.E * Ep))));
                    rotate(p.u, p.v, p.w, mu, 2 * kPi * p.rng.u01());
                  }
                  p.E = Ep;
                  ok = true;
                }
              }
              if (!ok) {  // not representable: the POD sampler, inline
                ok = tl.fast_ok && ffg ? tsl_scatter<true>(tl, p.rng, R.T, p.E, p.u, p.v, p.w)
                                       : tsl_scatter<false>(tl, p.rng, R.T, p.E, p.u, p.v, p.w);
              }
            }
            p.event = ok ? kScatter : kLostEvent;
            if (!ok) my_resample++;
            p.j = ce_search(w.ce, p.E);
            // the scatter event's bookkeeping (a scatter scores no current)
            p.nev++;
            hist_nev++;
            my_events++;
            alive = true;
            if (ok && p.nev >= rp.max_events) {
              my_capped++;
              p.event = kLostEvent;
            }
            if (p.event == kLostEvent) {
              if (fate == kBirth) fate = kLostEvent;
              alive = false;
              finish_history();
            }
          }
        }
        else {
          if (rp.from_bank) start_from_site(rp, hist, source_site(rp, hist), p, 1);
          else sample_source(w, rp, hist, p);
          p.cell = find_cell(w, p.x, p.y, p.z);
          p.j = ce_search(w.ce, p.E);
          p.event = kBirth;
          p.surf = -1;
          p.skip = -1;
          p.nev = 0;
          reset_indirect<PERT>(p);
          hist_nev = 0;
          fate = kBirth;
          dropped = false;
          alive = true;
          sc.dense = rp.nb ? rp.pend + hist : nullptr;
          if constexpr (KEIG) rp.fis[hist].n = 0;
          if (p.cell < 0 || __ldg(w.cell_mat + p.cell) < 0) {
            alive = false;
            my_lost++;
            p.event = kLostEvent;
            fate = kLostEvent;
            mark_lost();
            rp.ctr->pad[0] = static_cast<unsigned long long>(p.cell + 1);
            rp.ctr->pad[1] = hist;
            finish_history();
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;

    if (alive) {
      // ---- one event
      const int t = p.type;
      const int m = __ldg(w.cell_mat + p.cell);
      const bool delta = w.tracking == 1;
      const double density = __ldg(w.mat_density + m);
      UnionPos up{0, 0, 0.0f};
      double sigma, nsf = 0, cpd = 0, T_pos = 0;
      if (fx) {
        up = ce_union_pos(w.ce, p.j, p.E);
        const size_t row = static_cast<size_t>(t * w.n_materials + m) * w.ce.nu;
        const float2 a = __ldg(w.ce.mat_flight + row + up.jl), b = __ldg(w.ce.mat_flight + row + up.jh);
        sigma = static_cast<double>(lerpf(a.x, b.x, up.f));
        if (KEIG) nsf = static_cast<double>(lerpf(a.y, b.y, up.f));
      }
      else {
        // GetCollisionProbabilityDensity: total, or the majorant at the
        // cell's maximum temperature (src/TransportMethod.cpp:79-82,124-127)
        T_pos = cell_temperature(w, p.cell, p.x, p.y, p.z);
        cpd = delta ? ce_material_micro(w, m, t, p.j, p.E, cell_temperature_max(w, p.cell), T_pos, true, &memo)
                    : ce_material_micro(w, m, t, p.j, p.E, T_pos, T_pos, false, &memo);
        sigma = dmul(density, cpd);
        if (KEIG) nsf = dmul(density, ce_material_nusigf(w, m, t, p.j, p.E));
      }
      const double dcol = sample_flight(p.rng, sigma, fast);
      double dsurf;
      const int s = nearest_surface(w, p.cell, p.x, p.y, p.z, p.u, p.v, p.w, dsurf, p.skip,
                                    std::is_same_v<Rng, PhiloxRng> && fast);
      const bool collide = delta ? !(dsurf < dcol) : (dcol < dsurf);
      const bool refl = !collide && __ldg(w.surf_refl + s) != 0;
      bool real = true;
      if (collide && delta) {
        // bernoulli(total / majorant) before the particle moves
        // (src/TransportMethod.cpp:106-110); the FP32 tables hold no
        // temperature dependence, so there the ratio is one
        const double u = uniform(p.rng, fast);
        if (!fx) real = u < ddiv(ce_material_micro(w, m, t, p.j, p.E, T_pos, T_pos, false, &memo), cpd);
      }
      // the move -- to the collision, onto a reflecting plane, or across a
      // surface plus the nudge -- once for the whole warp (FP64 issue does
      // not shrink with the active lanes)
      const double dcross = dadd(dsurf, kNudge);
      const double dmove = collide ? dcol : (refl ? dsurf : dcross);
      if (rp.score) score_track<true>(w, p, dmove, sc);
      if (KEIG) my_ktl += dmove * nsf;
      indirect_stream<PERT>(w, p, m, cpd, dmove);
      stream(p.x, p.y, p.z, p.u, p.v, p.w, dmove);
      if (collide) {
        if (!real) {
          p.event = kVirtualCollision;
        }
        else {
          p.skip = -1;
          const int k = ce_sample_nuclide(w, p, m, fx, up, fast, &memo);
          const int nuc = __ldg(w.mat_nuc + __ldg(w.mat_begin + m) + k);
          const mc::CENuclideDesc& d = ce_desc(w, t, nuc);
          const int r = ce_pick_reaction(w, p, nuc, d, fx, up, fast, &memo);
          const int kind = r < 0 ? -1 : d.rx_kind[r];
          if (kind == 0) {
            p.event = kCapture;
          }
          else if (kind == 1) {
            p.event = kScatter;
            const double T = cell_temperature(w, p.cell, p.x, p.y, p.z);
            if (!fx && ce_tsl_valid(w, d, r, t, p.E)) {
              // ThermalScattering::Scatter; past its resample limits the
              // reference throws, here the history ends and is counted
              const DevTSL& tl = w.tsl[d.rx_tsl[r]];
              if constexpr (TQ) {
                // the POD-exact forms (modes 2, 3) sample what the inline
                // sampler below would (the FP32 form when ffg and the
                // library allow it, else FP64) and need no trained box
                const bool exact_q = rp.tq_mode >= 2;
                if (rp.tq && d.rx_tsl[r] == rp.tq_tsl && sp == 0 && pend.n <= kParkPending &&
                    (exact_q ? ((ffg && tl.fast_ok) == (rp.tq_fast != 0))
                             : (p.E >= rp.tq_box[0] && p.E <= rp.tq_box[1] && T >= rp.tq_box[2] &&
                                T <= rp.tq_box[3]))) {
                  // park for the batched surrogate sampler
                  const unsigned am = __activemask();
                  const int ld = __ffs(am) - 1;
                  unsigned long long pb = 0;
                  if (lane == static_cast<unsigned>(ld))
                    pb = atomicAdd(rp.park_count, static_cast<unsigned long long>(__popc(am)));
                  pb = __shfl_sync(am, pb, ld);
                  const unsigned long long slot = pb + __popc(am & ((1u << lane) - 1u));
                  if (slot < rp.park_cap) {
                    if (exact_q) {
                      GuideRow g;
                      g.E = p.E;
                      g.T = T;
                      g.rng_id = static_cast<unsigned long long>(p.rng.h0) |
                                 (static_cast<unsigned long long>(p.rng.h1) << 32);
                      g.rng_pos = p.rng.save();
                      g.rng_tag = p.rng.tag;
                      rp.tq_rows[slot] = g;
                    }
                    else {
                      const float u1 = p.rng.u01f(), u2 = p.rng.u01f();
                      rp.tq_in[slot] = make_float4(static_cast<float>(p.E), static_cast<float>(T), u1, u2);
                    }
                    ParkRec& R = rp.park_out[slot];
                    R.x = p.x;
                    R.y = p.y;
                    R.z = p.z;
                    R.u = p.u;
                    R.v = p.v;
                    R.w = p.w;
                    R.E = p.E;
                    R.T = T;
                    R.hist = hist;
                    R.rng_id = static_cast<unsigned long long>(p.rng.h0) |
                               (static_cast<unsigned long long>(p.rng.h1) << 32);
                    R.cell = p.cell;
                    R.surf = p.surf;
                    R.skip = p.skip;
                    R.type = p.type;
                    R.nev = p.nev;
                    R.hist_nev = hist_nev;
                    R.rng_pos = p.rng.save();
                    R.rng_tag = p.rng.tag;
                    R.fate = fate;
                    R.flags = dropped ? 1 : 0;
                    R.pend_n = pend.n | (pend.overflow ? 0x100 : 0);
                    R.tsl = d.rx_tsl[r];
                    for (int k = 0; k < pend.n && k < kParkPending; k++) {
                      R.pend_bin[k] = pend.bin[k];
                      R.pend_score[k] = pend.score[k];
                    }
                    parked = true;
                  }
                }
              }
              if (!parked) {
                const bool ok = ffg && tl.fast_ok ? tsl_scatter<true>(tl, p.rng, T, p.E, p.u, p.v, p.w)
                                                  : tsl_scatter<false>(tl, p.rng, T, p.E, p.u, p.v, p.w);
                if (!ok) {
                  my_resample++;
                  p.event = kLostEvent;
                }
              }
            }
            else {
              bool ok;
              if (ffg) ok = free_gas_fast(p.rng, static_cast<float>(d.awr), static_cast<float>(T), p.E, p.u, p.v, p.w);
              else ok = free_gas_exact(p.rng, d.awr, T, p.E, p.u, p.v, p.w);
              if (!ok) my_resample++;
            }
            p.j = ce_search(w.ce, p.E);
          }
          else if (kind == 2) {
            p.event = kFission;
            const double nubar = ce_nubar(w, p, nuc, d, r, fx, up);
            const unsigned yield = static_cast<unsigned>(dadd(nubar, uniform(p.rng, fast)));
            if constexpr (KEIG) {
              FissionRec f;
              f.x = p.x;
              f.y = p.y;
              f.z = p.z;
              f.g = -1;
              f.n = yield;
              f.rng = p.rng.save();
              if constexpr (is_philox<Rng>()) {
                f.tag = p.rng.tag;
                f.id = static_cast<unsigned long long>(p.rng.h0) | (static_cast<unsigned long long>(p.rng.h1) << 32);
              }
              else {
                f.tag = 0;
                f.id = 0;
              }
              set_record_energy(f, p.E);
              rp.fis[hist] = f;
            }
            else {
              // ContinuousFission::Interact: isotropic secondaries at the
              // incident energy, each seeded with rng()
              for (unsigned i = 0; i < yield; i++) {
                Site st;
                sample_isotropic(p.rng, st.u, st.v, st.w, fast);
                st.x = p.x;
                st.y = p.y;
                st.z = p.z;
                st.energy = p.E;
                st.key = p.rng.child_key();
                if (sp < kStack) {
                  stack[sp++] = st;
                }
                else {
                  my_overflow++;
                  dropped = true;
                }
                my_sec++;
              }
            }
          }
          else {
            // the reference resamples forever (src/Continuous.cpp:70-71)
            my_resample++;
            p.event = kLostEvent;
            my_lost++;
            mark_lost();
          }
        }
      }
      else {
        if (refl) {
          const int kind = __ldg(w.surf_kind + s);
          if (kind == kPlaneX) p.u = -p.u;
          else if (kind == kPlaneY) p.v = -p.v;
          else p.w = -p.w;
          p.event = kReflect;
          p.surf = s;
          p.skip = s;
        }
        else {
          if (w.quirks) {
            p.cell = find_cell(w, p.x, p.y, p.z);
          }
          else {
            p.cell = find_cell_crossing(w, p.x, p.y, p.z, s, moving_positive(w, s, p.x, p.y, p.z, p.u, p.v, p.w));
            p.skip = s;
          }
          p.surf = s;
          if (p.cell < 0) {
            p.event = kLostEvent;
            my_lost++;
            mark_lost();
          }
          else {
            p.event = __ldg(w.cell_mat + p.cell) >= 0 ? kSurfaceCross : kLeak;
          }
        }
      }
      if constexpr (TQ) {
        if (parked) {  // the history continues in a resume launch
          parked = false;
          alive = false;
          pend.clear();
          continue;
        }
      }
      if (rp.score) score_event<true, PERT>(w, p, sc);
      p.nev++;
      hist_nev++;
      my_events++;
      const bool dead = p.event == kCapture || p.event == kLeak || p.event == kFission || p.event == kLostEvent;
      if (!dead && p.nev >= rp.max_events) {
        my_capped++;
        p.event = kLostEvent;
      }
      if (dead || p.event == kLostEvent) {
        if (fate == kBirth) fate = static_cast<int8_t>(p.event);
        alive = false;
        if (!KEIG && sp > 0 && !dropped) {
          // next particle of the same history (src/FixedSource.cpp:63-72)
          const Site st = stack[--sp];
          p.x = st.x;
          p.y = st.y;
          p.z = st.z;
          p.u = st.u;
          p.v = st.v;
          p.w = st.w;
          p.E = st.energy;
          p.j = ce_search(w.ce, p.E);
          p.type = 0;
          if constexpr (is_philox<Rng>()) p.rng.init(rp.run_key, st.key, 1);
          else p.rng.seed(st.key);
          p.cell = find_cell(w, p.x, p.y, p.z);
          p.event = kBirth;
          p.surf = -1;
          p.skip = -1;
          p.nev = 0;
          reset_indirect<PERT>(p);
          alive = p.cell >= 0 && __ldg(w.cell_mat + p.cell) >= 0;
          if (!alive) my_lost++;
        }
        if (!alive) {
          sp = 0;  // nothing of this history may carry over to the next
          finish_history();
        }
      }
    }
  }

  for (int off = 16; off > 0; off >>= 1) {
    my_events += __shfl_down_sync(0xffffffffu, my_events, off);
    my_lost += __shfl_down_sync(0xffffffffu, my_lost, off);
    my_capped += __shfl_down_sync(0xffffffffu, my_capped, off);
    my_overflow += __shfl_down_sync(0xffffffffu, my_overflow, off);
    my_sec += __shfl_down_sync(0xffffffffu, my_sec, off);
    my_resample += __shfl_down_sync(0xffffffffu, my_resample, off);
    my_ktl += __shfl_down_sync(0xffffffffu, my_ktl, off);
  }
  if (lane == 0) {
    atomicAdd(&rp.ctr->events, my_events);
    if (my_lost) atomicAdd(&rp.ctr->lost, my_lost);
    if (my_capped) atomicAdd(&rp.ctr->capped, my_capped);
    if (my_overflow) atomicAdd(&rp.ctr->overflow, my_overflow);
    if (my_sec) atomicAdd(&rp.ctr->secondaries, my_sec);
    if (my_resample) atomicAdd(&rp.ctr->resample, my_resample);
    if (KEIG) atomicAdd(&rp.ctr->k_tracklength, my_ktl);
  }
  if (use_smem) {
    __syncthreads();
    for (int i = threadIdx.x; i < static_cast<int>(rp.total_bins); i += blockDim.x) {
      if (smem[i] != 0) atomicAdd(rp.tally_sum + i, smem[i]);
      if (smem[kSharedBins + i] != 0) atomicAdd(rp.tally_sq + i, smem[kSharedBins + i]);
    }
  }
}

template <class K>
int occupancy_of(K kernel, int block, size_t smem) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem);
  return n;
}

constexpr size_t kCeSmem = 2 * kSharedBins * sizeof(double);
// register budget of the exact-table fixed-source kernels with Philox
// streams (thermal problems): two resident blocks per SM (128 registers,
// a few hundred bytes of spills) hide more latency than one (~185)
constexpr int kExactFixedMinb = 2;

}  // namespace

// launchers of the variant groups, one translation unit each
// (mc_transport_ce_*.cu)
namespace cevar {
// FP32-table kernels in the multigroup kernel's occupancy variants: MINB 1
// and 3 (mc_transport_ce_fx1.cu), 4, 5 and 6 (mc_transport_ce_fx2.cu)
bool has_fx1(int minb);
int occupancy_fx1(int minb, int block, bool keig);
void launch_fx1(int minb, const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream);
int occupancy_fx2(int minb, int block, bool keig);
void launch_fx2(int minb, const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream);
// exact tables, both stream families (mc_transport_ce_exact.cu)
int occupancy_exact(int rng_mode, int block, bool keig);
void launch_exact(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block, cudaStream_t stream);
// indirect effects of perturbations; the thermal-scatter queue
// (mc_transport_ce_ext.cu)
void launch_pert(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block, cudaStream_t stream);
void launch_tq(const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream);
}  // namespace cevar

}  // namespace mcd
