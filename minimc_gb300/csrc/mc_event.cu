// Event schedule: the particle-history loop split into event kernels over
// compacted queues (SoA particle state in HBM).
//
//   init     : one thread per history; source sampling or bank load, cell
//              search; live particles enter the active queue
//   advance  : per active particle: Sigma_t lookup, distance to collision
//              (exponential_distribution), Cell::NearestSurface, classify;
//              crossings are relocated and scored here and re-queued,
//              collisions go to the collision queue
//              (SurfaceTracking::Transport, src/TransportMethod.cpp:56-75)
//   collide  : per collision: Particle::SampleNuclide, Multigroup::Interact
//              (src/Multigroup.cpp:49-73); survivors re-queued; fixed-source
//              fission secondaries get new slots and join the queue;
//              k-eigenvalue fissions are recorded for the site kernel
//   sites    : k-eigenvalue fission sites generated from the recorded
//              stream position (Multigroup::Fission, src/Multigroup.cpp:267-286)
//   commit   : per-history pending scores -> sums and sums of squares
//              (ScorableProxy::CommitHistory, src/Scorable.cpp:101-106)
//
// Queue slots are appended with one atomic per warp (ballot + popc).  Every
// particle's random stream is saved as one word between kernels and resumed
// exactly, so the event and history schedules draw identical numbers and give
// identical results for the same seed.
#include "mc_event.cuh"

#include <type_traits>

namespace mcd {

namespace {

constexpr int kMaxSec = 8;  // fixed-source secondaries per fission kept in registers

__device__ __forceinline__ unsigned lane() { return threadIdx.x & 31u; }

// warp-aggregated append of `want` lanes to a queue; returns the slot
__device__ __forceinline__ unsigned queue_slot(unsigned* counter, bool want) {
  const unsigned active = __activemask();
  const unsigned mask = __ballot_sync(active, want);
  if (!mask) return 0;
  const int leader = __ffs(mask) - 1;
  unsigned base = 0;
  if (lane() == static_cast<unsigned>(leader)) base = atomicAdd(counter, static_cast<unsigned>(__popc(mask)));
  base = __shfl_sync(active, base, leader);
  return base + __popc(mask & ((1u << lane()) - 1u));
}

template <class Rng>
__device__ __forceinline__ void load_rng(const EvParams& ep, unsigned i, Rng& rng) {
  rng.restore(ep.rp.run_key, ep.st.id[i], ep.st.tag[i] & 1u, ep.st.rng[i]);
}

template <class Rng>
__device__ __forceinline__ double uni(Rng& rng, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return static_cast<double>(rng.u01f());
  }
  return rng.u01();
}

template <class Rng>
__device__ __forceinline__ void iso(Rng& rng, double& u, double& v, double& w, bool fast) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) {
      isotropic_fast(rng, u, v, w);
      return;
    }
  }
  isotropic(rng, u, v, w);
}

__device__ __forceinline__ int first_above(const double* cdf, int n, double threshold) {
  return cdf_first_above(cdf, n, threshold);
}

// particle death bookkeeping shared by all kernels
__device__ __forceinline__ void particle_died(const EvParams& ep, unsigned i, int event) {
  const unsigned h = ep.st.hist[i];
  if (ep.rp.hist_events) atomicAdd(ep.rp.hist_events + h, ep.st.nev[i]);
  if (ep.rp.hist_fate && !(ep.st.tag[i] & 1u)) ep.rp.hist_fate[h] = static_cast<int8_t>(event);
}

__device__ __forceinline__ void pend_add(const EvParams& ep, unsigned h, uint64_t bin, double s) {
  atomicAdd(ep.rp.pend + bin * ep.rp.n + h, s);  // bin-major
}

}  // namespace

// ---------------------------------------------------------------------------
template <class Rng>
__global__ void __launch_bounds__(256) k_ev_init(const DevWorld w, const EvParams ep) {
  const unsigned long long n = ep.rp.n;
  const bool fast = ep.rp.fast != 0;
  unsigned long long lost = 0;
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    double x, y, z, u, v, ww;
    int g = 0;
    Rng rng;
    unsigned long long id = i;
    uint8_t tag = 0;
    if (ep.rp.from_bank) {
      const Site s = source_site(ep.rp, i);
      x = s.x; y = s.y; z = s.z; u = s.u; v = s.v; ww = s.w;
      g = static_cast<int>(s.energy) - 1;
      if constexpr (std::is_same_v<Rng, MinstdRng>) {
        rng.seed(ep.rp.minstd_base ? ep.rp.minstd_base + i : s.key);
      }
      else {
        if (!ep.rp.minstd_base) {
          id = s.key;
          tag = 1;
        }
        rng.init(ep.rp.run_key, id, tag);
      }
    }
    else {
      x = w.src_pos[0]; y = w.src_pos[1]; z = w.src_pos[2];
      tag = w.src_type == 1 ? 2 : 0;
      if constexpr (std::is_same_v<Rng, MinstdRng>) {
        MinstdRng s;
        s.seed(ep.rp.ref_source_seeds ? ep.rp.seed + i : i + 1);
        if (w.src_dir_kind == 0) { u = w.src_dir[0]; v = w.src_dir[1]; ww = w.src_dir[2]; }
        else if (w.src_dir_kind == 1) isotropic(s, u, v, ww);
        else {
          const double mu = __dsqrt_rn(s.u01());
          const double phi = dadd(dmul(s.u01(), 2 * kPi), 0.0);
          u = w.src_dir[0]; v = w.src_dir[1]; ww = w.src_dir[2];
          rotate(u, v, ww, mu, phi);
        }
        rng.seed(s.next());
      }
      else {
        rng.init(ep.rp.run_key, i, 0);
        if (w.src_dir_kind == 0) { u = w.src_dir[0]; v = w.src_dir[1]; ww = w.src_dir[2]; }
        else if (w.src_dir_kind == 1) iso(rng, u, v, ww, fast);
        else {
          const double mu = sqrt(rng.u01());
          const double phi = 2 * kPi * rng.u01();
          u = w.src_dir[0]; v = w.src_dir[1]; ww = w.src_dir[2];
          rotate(u, v, ww, mu, phi);
        }
      }
      g = static_cast<int>(w.src_energy) - 1;
    }
    const int cell = find_cell(w, x, y, z);
    const unsigned slot = static_cast<unsigned>(i);
    ep.st.x[slot] = x; ep.st.y[slot] = y; ep.st.z[slot] = z;
    ep.st.u[slot] = u; ep.st.v[slot] = v; ep.st.w[slot] = ww;
    ep.st.g[slot] = g;
    ep.st.cell[slot] = cell;
    ep.st.skip[slot] = -1;
    ep.st.nev[slot] = 0;
    ep.st.hist[slot] = slot;
    ep.st.id[slot] = id;
    ep.st.tag[slot] = tag;
    ep.st.rng[slot] = rng.save();
    if (ep.rp.keig) ep.rp.fis[slot].n = 0;
    const bool ok = cell >= 0 && __ldg(w.cell_mat + cell) >= 0;
    if (!ok) {
      lost++;
      ep.rp.ctr->lost_xyz[0] = x;
      ep.rp.ctr->lost_xyz[1] = y;
      ep.rp.ctr->lost_xyz[2] = z;
      if (ep.rp.hist_fate) ep.rp.hist_fate[slot] = kLostEvent;
      if (ep.rp.hist_events) ep.rp.hist_events[slot] = 0;
    }
    else if (ep.rp.hist_events) {
      ep.rp.hist_events[slot] = 0;
    }
    const unsigned q = queue_slot(ep.cnt + 1, ok);
    if (ok) ep.q_out[q] = static_cast<int32_t>(slot);
  }
  if (lost) atomicAdd(&ep.rp.ctr->lost, lost);
}

// ---------------------------------------------------------------------------
template <class Rng>
__global__ void __launch_bounds__(256) k_ev_advance_mg(const DevWorld w, const EvParams ep) {
  const unsigned n_in = ep.cnt[0];
  const bool fast = ep.rp.fast != 0;
  unsigned long long my_events = 0, my_lost = 0, my_capped = 0;
  double my_ktl = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x;; k += gridDim.x * blockDim.x) {
    if (__all_sync(0xffffffffu, k >= n_in)) break;
    const int32_t qi = k < n_in ? ep.q_in[k] : -1;  // -1: slot lost to an overflow
    const bool have = qi >= 0;
    bool to_coll = false, to_next = false;
    unsigned i = 0;
    if (have) {
      i = static_cast<unsigned>(qi);
      Rng rng;
      load_rng(ep, i, rng);
      double x = ep.st.x[i], y = ep.st.y[i], z = ep.st.z[i];
      const double u = ep.st.u[i], v = ep.st.v[i], ww = ep.st.w[i];
      const int g = ep.st.g[i];
      int cell = ep.st.cell[i];
      int skip = ep.st.skip[i];
      const unsigned h = ep.st.hist[i];
      const int t = (ep.st.tag[i] >> 1) & 1;
      const int m = __ldg(w.cell_mat + cell);
      const size_t mg = (static_cast<size_t>(t) * w.n_materials + m) * w.G + g;
      const double sigma = __ldg(w.mat_mg_sigma + mg);  // number_density * micro, tabulated
      const double dcol = mg_flight(w, rng, fast, mg, sigma);
      double dsurf;
      const int s = nearest_surface(w, cell, x, y, z, u, v, ww, dsurf, skip, std::is_same_v<Rng, PhiloxRng> && fast);
      const bool collide = w.tracking == 1 ? !(dsurf < dcol) : (dcol < dsurf);
      const bool score = ep.rp.score != 0;
      auto track = [&](double d) {
        if (ep.rp.keig) my_ktl += d * __ldg(w.mat_mg_nusigf + mg);
        if (!score) return;
        for (int e = 0; e < w.n_est; e++) {
          if (__ldg(w.est_kind + e) != 1 || __ldg(w.est_target + e) != cell) continue;
          pend_add(ep, h, __ldg(w.est_offset + e) + particle_bin_mg(w, e, u, v, ww, g), d);
        }
      };
      int event;
      if (collide) {
        track(dcol);
        move(fast, x, y, z, u, v, ww, dcol);
        skip = -1;
        to_coll = true;
        event = kScatter;  // placeholder; the collide kernel decides
      }
      else if (__ldg(w.surf_refl + s)) {
        track(dsurf);
        move(fast, x, y, z, u, v, ww, dsurf);
        const int kind = __ldg(w.surf_kind + s);
        double nu = u, nv = v, nw = ww;
        if (kind == kPlaneX) nu = -u;
        else if (kind == kPlaneY) nv = -v;
        else nw = -ww;
        ep.st.u[i] = nu;
        ep.st.v[i] = nv;
        ep.st.w[i] = nw;
        skip = s;
        event = kReflect;
        to_next = true;
      }
      else {
        const double d = dadd(dsurf, kNudge);
        track(d);
        move(fast, x, y, z, u, v, ww, d);
        if (w.quirks) {
          cell = find_cell(w, x, y, z);
        }
        else {
          cell = find_cell_crossing(w, x, y, z, s, moving_positive(w, s, x, y, z, u, v, ww));
          skip = s;
        }
        if (cell < 0) {
          event = kLostEvent;
          my_lost++;
          ep.rp.ctr->lost_xyz[0] = x;
          ep.rp.ctr->lost_xyz[1] = y;
          ep.rp.ctr->lost_xyz[2] = z;
        }
        else {
          event = __ldg(w.cell_mat + cell) >= 0 ? kSurfaceCross : kLeak;
        }
        if (score && (event == kSurfaceCross || event == kLeak)) {
          for (int e = 0; e < w.n_est; e++) {
            if (__ldg(w.est_kind + e) != 0 || __ldg(w.est_target + e) != s) continue;
            pend_add(ep, h, __ldg(w.est_offset + e) + particle_bin_mg(w, e, u, v, ww, g), 1.0);
          }
        }
        to_next = event == kSurfaceCross;
      }
      const uint32_t nev = ep.st.nev[i] + 1;
      my_events++;
      ep.st.x[i] = x;
      ep.st.y[i] = y;
      ep.st.z[i] = z;
      ep.st.cell[i] = cell;
      ep.st.skip[i] = skip;
      ep.st.nev[i] = nev;
      ep.st.rng[i] = rng.save();
      if (!to_coll && !to_next) {
        particle_died(ep, i, event);
      }
      else if (to_next && nev >= ep.rp.max_events) {
        to_next = false;
        my_capped++;
        particle_died(ep, i, kLostEvent);
      }
    }
    const unsigned qc = queue_slot(ep.cnt + 2, to_coll);
    if (to_coll) ep.q_coll[qc] = static_cast<int32_t>(i);
    const unsigned qn = queue_slot(ep.cnt + 1, to_next);
    if (to_next) ep.q_out[qn] = static_cast<int32_t>(i);
  }
  for (int off = 16; off > 0; off >>= 1) {
    my_events += __shfl_down_sync(0xffffffffu, my_events, off);
    my_lost += __shfl_down_sync(0xffffffffu, my_lost, off);
    my_capped += __shfl_down_sync(0xffffffffu, my_capped, off);
    my_ktl += __shfl_down_sync(0xffffffffu, my_ktl, off);
  }
  if (lane() == 0) {
    if (my_events) atomicAdd(&ep.rp.ctr->events, my_events);
    if (my_lost) atomicAdd(&ep.rp.ctr->lost, my_lost);
    if (my_capped) atomicAdd(&ep.rp.ctr->capped, my_capped);
    if (my_ktl != 0) atomicAdd(&ep.rp.ctr->k_tracklength, my_ktl);
  }
}

// ---------------------------------------------------------------------------
template <class Rng>
__global__ void __launch_bounds__(256) k_ev_collide_mg(const DevWorld w, const EvParams ep) {
  const unsigned n_in = ep.cnt[2];
  const bool fast = ep.rp.fast != 0;
  const int G = w.G;
  unsigned long long my_overflow = 0, my_sec = 0, my_capped = 0;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x;; k += gridDim.x * blockDim.x) {
    const bool have = k < n_in;
    if (__all_sync(0xffffffffu, !have)) break;
    bool to_next = false;
    int n_sec = 0;
    unsigned i = 0;
    Site sec[kMaxSec];
    if (have) {
      i = static_cast<unsigned>((ep.cnt[4] ? ep.q_sorted : ep.q_coll)[k]);
      Rng rng;
      load_rng(ep, i, rng);
      const int t = (ep.st.tag[i] >> 1) & 1;
      const int cell = ep.st.cell[i];
      const int m = __ldg(w.cell_mat + cell);
      int g = ep.st.g[i];
      const size_t mg = (static_cast<size_t>(t) * w.n_materials + m) * G + g;
      const double micro = __ldg(w.mat_mg_total + mg);
      // CellDeltaTracking's real/virtual test; multigroup majorant == total
      if (w.tracking == 1) (void)uni(rng, fast);
      const int nb = __ldg(w.mat_begin + m), ne = __ldg(w.mat_begin + m + 1);
      const int nuc = __ldg(w.mat_nuc + nb + mg_pick_nuclide(w, rng, fast, mg, ne - nb, micro));
      const size_t ng = (static_cast<size_t>(t) * w.n_nuclides + nuc) * G + g;
      const int rx = mg_pick_reaction(w, rng, fast, ng);
      int event = kScatter;
      if (rx < 0) {
        // no reaction selected (threshold at the top of the CDF): the
        // reference's Interact falls through without touching the particle
        // (src/Multigroup.cpp:70-72, assert compiled out), so it flies on
        to_next = true;
      }
      else if (rx == 0) {
        event = kCapture;
      }
      else if (rx == 1) {
        const int go = mg_pick_outgoing(w, rng, fast, ng);
        if (go >= 0) {
          g = go;
          double u, v, ww;
          iso(rng, u, v, ww, fast);
          ep.st.u[i] = u;
          ep.st.v[i] = v;
          ep.st.w[i] = ww;
          ep.st.g[i] = g;
        }
        to_next = true;
      }
      else if (rx == 2) {
        event = kFission;
        const unsigned yield = mg_yield(w, rng, fast, ng);
        if (ep.rp.keig) {
          FissionRec& f = ep.rp.fis[ep.st.hist[i]];
          f.x = ep.st.x[i];
          f.y = ep.st.y[i];
          f.z = ep.st.z[i];
          f.g = g;
          f.n = yield;
          f.rng = rng.save();
          f.tag = ep.st.tag[i];
          f.id = ep.st.id[i];
          f.chi_index = static_cast<uint32_t>(ng);
        }
        else {
          // secondaries, sampled now in the reference's draw order
          const double* chi = w.mg_chi_cdf + ng * G;
          for (unsigned y = 0; y < yield; y++) {
            const double thr = uni(rng, fast);
            const int go = first_above(chi, G, thr);
            if (go < 0) continue;
            Site s;
            iso(rng, s.u, s.v, s.w, fast);
            s.energy = go;
            s.key = rng.child_key();
            if (n_sec < kMaxSec) sec[n_sec++] = s;
            else my_overflow++;
          }
        }
      }
      ep.st.rng[i] = rng.save();
      if (!to_next) particle_died(ep, i, event);
    }
    const unsigned qn = queue_slot(ep.cnt + 1, to_next);
    if (to_next) ep.q_out[qn] = static_cast<int32_t>(i);
    // fixed-source secondaries: new slots, same history, into the next queue
    const unsigned total_sec = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(n_sec));
    if (total_sec) {
      unsigned base = 0;
      unsigned excl = n_sec;
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned yv = __shfl_up_sync(0xffffffffu, excl, off);
        if (lane() >= static_cast<unsigned>(off)) excl += yv;
      }
      excl -= n_sec;
      if (lane() == 0) base = atomicAdd(ep.cnt + 3, total_sec);
      base = __shfl_sync(0xffffffffu, base, 0);
      unsigned qbase = 0;
      if (lane() == 0) qbase = atomicAdd(ep.cnt + 1, total_sec);
      qbase = __shfl_sync(0xffffffffu, qbase, 0);
      for (int s = 0; s < n_sec; s++) {
        const unsigned slot = base + excl + s;
        if (slot >= ep.capacity) {
          my_overflow++;
          ep.q_out[qbase + excl + s] = -1;
          continue;
        }
        ep.st.x[slot] = ep.st.x[i];
        ep.st.y[slot] = ep.st.y[i];
        ep.st.z[slot] = ep.st.z[i];
        ep.st.u[slot] = sec[s].u;
        ep.st.v[slot] = sec[s].v;
        ep.st.w[slot] = sec[s].w;
        ep.st.g[slot] = static_cast<int>(sec[s].energy);
        ep.st.cell[slot] = ep.st.cell[i];
        ep.st.skip[slot] = -1;
        ep.st.nev[slot] = 0;
        ep.st.hist[slot] = ep.st.hist[i];
        ep.st.tag[slot] = 1;
        if constexpr (std::is_same_v<Rng, MinstdRng>) {
          ep.st.id[slot] = 0;
          ep.st.rng[slot] = MinstdRng::seed_state(sec[s].key);
        }
        else {
          ep.st.id[slot] = sec[s].key;
          ep.st.rng[slot] = 4u;  // counter 0, buffer empty
        }
        ep.q_out[qbase + excl + s] = static_cast<int32_t>(slot);
        my_sec++;
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    my_overflow += __shfl_down_sync(0xffffffffu, my_overflow, off);
    my_sec += __shfl_down_sync(0xffffffffu, my_sec, off);
    my_capped += __shfl_down_sync(0xffffffffu, my_capped, off);
  }
  if (lane() == 0) {
    if (my_overflow) atomicAdd(&ep.rp.ctr->overflow, my_overflow);
    if (my_sec) atomicAdd(&ep.rp.ctr->secondaries, my_sec);
  }
}

// ---------------------------------------------------------------------------
// k-eigenvalue fission sites from the recorded stream positions
// (Multigroup::Fission, src/Multigroup.cpp:267-286: per site a chi group,
// an isotropic direction, then rng() seeds the secondary)
// histories first, first + stride, ... of the problem
template <class Rng>
__device__ __forceinline__ void fission_sites_mg(const DevWorld& w, const RunParams& rp, unsigned long long first,
                                                 unsigned long long stride) {
  const unsigned long long n = rp.n;
  const bool fast = rp.fast != 0;
  const int G = w.G;
  unsigned long long my_overflow = 0;
  for (unsigned long long h = first; h < n; h += stride) {
    const FissionRec f = rp.fis[h];
    uint32_t written = 0;
    if (f.n) {
      Rng rng;
      rng.restore(rp.run_key, f.id, f.tag & 1u, f.rng);
      // chi column of the fissioning (type, nuclide, incident group)
      const double* chi = w.mg_chi_cdf + static_cast<size_t>(f.chi_index) * G;
      Site* slots = rp.bank + h * rp.max_yield;
      for (uint32_t y = 0; y < f.n; y++) {
        const double thr = uni(rng, fast);
        const int go = first_above(chi, G, thr);
        if (go < 0) continue;
        Site s;
        iso(rng, s.u, s.v, s.w, fast);
        s.x = f.x;
        s.y = f.y;
        s.z = f.z;
        s.energy = static_cast<double>(go + 1);
        s.key = rng.child_key();
        if (written < rp.max_yield) slots[written++] = s;
        else my_overflow++;
      }
    }
    rp.bank_count[h] = written;
  }
  if (my_overflow) atomicAdd(&rp.ctr->overflow, my_overflow);
}

template <class Rng>
__global__ void __launch_bounds__(256) k_fission_sites_mg(const DevWorld w, const RunParams rp) {
  fission_sites_mg<Rng>(w, rp, static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x,
                        static_cast<unsigned long long>(gridDim.x) * blockDim.x);
}

// Sites straight into the compacted bank.  Where every record yields exactly
// min(n, max_yield) sites (multigroup: no chi draw can fall past the end of
// its cdf, which the caller checks against the largest uniform the stream
// draws; continuous energy: always), the counts are known before sampling
// and a scan of them (launch_direct_bank_scan, mc_transport.cu) gives every
// history its place in the bank.

// The multigroup direct-bank CTA: the draws are those of fission_sites_mg,
// site for site.  A site draws a fixed number of 32-bit words -- the chi
// threshold (1 in the FP32 form, 2 in FP64), the isotropic direction (2, 4)
// and the secondary's key (2) -- so site y of a record starts y times that
// many words into the record's stream, and each site is sampled by a thread
// of its own.
template <bool FAST>
__global__ void __launch_bounds__(kSitesOutHist) k_fission_sites_out_mg(const DevWorld w, const RunParams rp,
                                                                        const unsigned long long* offsets,
                                                                        const unsigned long long* total,
                                                                        unsigned long long cap, uint4* out) {
  constexpr uint32_t kWordsPerSite = FAST ? 1u + 2u + 2u : 2u + 4u + 2u;
  sites_out_cta_by_site(rp.n, offsets, total, cap, out, [&](unsigned long long h, uint32_t y, Site* dst) {
    const FissionRec f = rp.fis[h];
    PhiloxRng rng;
    rng.restore(rp.run_key, f.id, f.tag & 1u, philox_skip(f.rng, y * kWordsPerSite));
    const int G = w.G;
    const double* chi = w.mg_chi_cdf + static_cast<size_t>(f.chi_index) * G;
    // go >= 0: the cdf ends above every threshold this stream draws
    const int go = first_above(chi, G, uni(rng, FAST));
    Site s;
    iso(rng, s.u, s.v, s.w, FAST);
    s.x = f.x;
    s.y = f.y;
    s.z = f.z;
    s.energy = static_cast<double>(go + 1);
    s.key = rng.child_key();
    *dst = s;
  });
}

// Batched problems on the direct bank path: CTAs run over the concatenated
// histories (a CTA may span problems); history h belongs to the problem p
// with off[p] <= h < off[p + 1], whose world and run key it samples with.
template <bool FAST>
__global__ void __launch_bounds__(kSitesOutHist) k_fission_sites_out_mg_batch(
    const DevWorld* worlds, const RunParams* rps, const unsigned long long* off, int P, unsigned long long N,
    const FissionRec* fis, const uint32_t* count, const unsigned long long* offsets, const unsigned long long* total,
    unsigned long long cap, uint4* out) {
  extern __shared__ uint4 stage[];  // [kSitesOutHist * max_yield] sites
  sites_out_cta(N, count, offsets, total, cap, out, stage, [&](unsigned long long h, uint32_t c, Site* dst) {
    int lo = 0, hi = P;  // off[lo] <= h < off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (off[mid] <= h) lo = mid;
      else hi = mid;
    }
    const FissionRec f = fis[h];
    PhiloxRng rng;
    rng.restore(rps[lo].run_key, f.id, f.tag & 1u, f.rng);
    const int G = worlds[lo].G;
    const double* chi = worlds[lo].mg_chi_cdf + static_cast<size_t>(f.chi_index) * G;
    for (uint32_t y = 0; y < c; y++) {
      const int go = first_above(chi, G, uni(rng, FAST));
      Site s;
      iso(rng, s.u, s.v, s.w, FAST);
      s.x = f.x;
      s.y = f.y;
      s.z = f.z;
      s.energy = static_cast<double>(go + 1);
      s.key = rng.child_key();
      dst[y] = s;
    }
  });
}

// batched problems: CTA b serves problem block_problem[b], as the rank-th of
// its block_first[p + 1] - block_first[p] CTAs
__global__ void __launch_bounds__(256) k_fission_sites_mg_batch(const DevWorld* worlds, const RunParams* rps,
                                                                const uint32_t* block_problem,
                                                                const uint32_t* block_first) {
  __shared__ DevWorld w;
  __shared__ RunParams rp;
  const uint32_t p = block_problem[blockIdx.x];
  if (threadIdx.x == 0) {
    w = worlds[p];
    rp = rps[p];
  }
  __syncthreads();
  const unsigned long long rank = blockIdx.x - block_first[p], nb = block_first[p + 1] - block_first[p];
  fission_sites_mg<PhiloxRng>(w, rp, rank * blockDim.x + threadIdx.x, nb * blockDim.x);
}

// ---------------------------------------------------------------------------
// per-history dense scores -> sum, sum of squares
// (ScorableProxy::CommitHistory, src/Scorable.cpp:101-106).  The array is
// bin-major ([bin][history]); blockIdx.y is the bin, threads stride over
// histories with coalesced reads, skip zeros with an integer test, keep the
// two sums in registers, reduce per warp and per block, and write one atomic
// per block.  Entries read are set back to zero, so the array is clean for
// the next run without a memset.
__global__ void __launch_bounds__(256) k_commit_dense(const RunParams rp) {
  __shared__ double ws[8], wq[8];
  // per warp, the nonzero scores of one step packed together: the FP64
  // sums then issue per 32 nonzero scores instead of per 32 histories
  // (most histories leave a bin at zero, and an FP64 instruction costs the
  // whole warp however few of its lanes need it)
  __shared__ double packed[8][128];
  const unsigned b = blockIdx.y;
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double* row = rp.pend + static_cast<size_t>(b) * rp.n;
  double s = 0, q = 0;
  const unsigned long long S = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  unsigned long long h = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  // four independent loads in flight per thread (the array is read once);
  // the bound is the warp's last lane's, so every lane of a warp takes the
  // same trips (the shuffles below need the whole warp); what is left goes
  // to the per-lane loop after it
  for (unsigned long long hw = h - lane; hw + 31 + 3 * S < rp.n; h += 4 * S, hw += 4 * S) {
    double v[4];
#pragma unroll
    for (int j = 0; j < 4; j++) v[j] = __ldcs(row + h + j * S);
    unsigned c = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (__double_as_longlong(v[j]) != 0) {
        c++;
        row[h + j * S] = 0;
      }
    }
    // exclusive prefix of the counts over the warp
    unsigned x = c;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= static_cast<unsigned>(off)) x += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, x, 31);
    unsigned o = x - c;
#pragma unroll
    for (int j = 0; j < 4; j++)
      if (__double_as_longlong(v[j]) != 0) packed[wid][o++] = v[j];
    __syncwarp();
    for (unsigned k = lane; k < total; k += 32) {
      const double t = packed[wid][k];
      s += t;
      q += t * t;
    }
    __syncwarp();
  }
  for (; h < rp.n; h += S) {
    const double v = row[h];
    if (__double_as_longlong(v) != 0) {
      s += v;
      q += v * v;
      row[h] = 0;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, off);
    q += __shfl_down_sync(0xffffffffu, q, off);
  }
  if (lane == 0) {
    ws[wid] = s;
    wq[wid] = q;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ts = 0, tq = 0;
    for (int i = 0; i < static_cast<int>(blockDim.x >> 5); i++) {
      ts += ws[i];
      tq += wq[i];
    }
    if (ts != 0) atomicAdd(rp.tally_sum + b, ts);
    if (tq != 0) atomicAdd(rp.tally_sq + b, tq);
  }
}

cudaError_t launch_fission_sites_mg(const DevWorld& w, const RunParams& rp, int rng_mode, int grid,
                                    cudaStream_t stream) {
  if (rng_mode == 1) k_fission_sites_mg<MinstdRng><<<grid, 256, 0, stream>>>(w, rp);
  else k_fission_sites_mg<PhiloxRng><<<grid, 256, 0, stream>>>(w, rp);
  return cudaGetLastError();
}

size_t sites_out_smem(uint32_t max_yield) { return static_cast<size_t>(kSitesOutHist) * max_yield * sizeof(Site); }

bool sites_out_fits(uint32_t max_yield) { return sites_out_smem(max_yield) <= kSitesOutMaxSmem; }

cudaError_t launch_fission_sites_out_mg(const DevWorld& w, const RunParams& rp, const unsigned long long* offsets,
                                        const unsigned long long* total, unsigned long long cap, Site* out,
                                        cudaStream_t stream) {
  const unsigned grid = static_cast<unsigned>((rp.n + kSitesOutHist - 1) / kSitesOutHist);
  auto* o = reinterpret_cast<uint4*>(out);
  if (rp.fast) k_fission_sites_out_mg<true><<<grid, kSitesOutHist, 0, stream>>>(w, rp, offsets, total, cap, o);
  else k_fission_sites_out_mg<false><<<grid, kSitesOutHist, 0, stream>>>(w, rp, offsets, total, cap, o);
  return cudaGetLastError();
}

cudaError_t launch_fission_sites_out_mg_batch(const DevWorld* worlds, const RunParams* rps,
                                              const unsigned long long* off, int P, unsigned long long N,
                                              uint32_t max_yield, bool fast, const FissionRec* fis,
                                              const uint32_t* count, const unsigned long long* offsets,
                                              const unsigned long long* total, Site* out, cudaStream_t stream) {
  const size_t smem = sites_out_smem(max_yield);
  if (smem > kSitesOutMaxSmem) return cudaErrorInvalidValue;
  const unsigned grid = static_cast<unsigned>((N + kSitesOutHist - 1) / kSitesOutHist);
  const unsigned long long cap = N * max_yield;
  auto* o = reinterpret_cast<uint4*>(out);
  if (fast)
    k_fission_sites_out_mg_batch<true><<<grid, kSitesOutHist, smem, stream>>>(worlds, rps, off, P, N, fis, count,
                                                                               offsets, total, cap, o);
  else
    k_fission_sites_out_mg_batch<false><<<grid, kSitesOutHist, smem, stream>>>(worlds, rps, off, P, N, fis, count,
                                                                                offsets, total, cap, o);
  return cudaGetLastError();
}

cudaError_t sites_out_batch_prepare(uint32_t max_yield) {
  const int smem = static_cast<int>(sites_out_smem(max_yield));
  cudaError_t e = cudaFuncSetAttribute(k_fission_sites_out_mg_batch<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_fission_sites_out_mg_batch<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

cudaError_t launch_fission_sites_mg_batch(const DevWorld* worlds, const RunParams* rps, const uint32_t* block_problem,
                                          const uint32_t* block_first, int grid, cudaStream_t stream) {
  k_fission_sites_mg_batch<<<grid, 256, 0, stream>>>(worlds, rps, block_problem, block_first);
  return cudaGetLastError();
}

cudaError_t launch_commit_dense(const RunParams& rp, int grid, cudaStream_t stream) {
  if (rp.nb <= 0) return cudaSuccess;
  // about `grid` blocks in total, spread over the bins
  const unsigned per_bin = static_cast<unsigned>(std::max(1, grid / rp.nb));
  const unsigned needed = static_cast<unsigned>((rp.n + 255) / 256);
  const dim3 g(std::min(per_bin, std::max(1u, needed)), static_cast<unsigned>(rp.nb));
  k_commit_dense<<<g, 256, 0, stream>>>(rp);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// launches

// next-queue count becomes the input count of the following iteration
__global__ void k_ev_swap(unsigned* cnt) {
  cnt[0] = cnt[1];
  cnt[1] = 0;
  cnt[2] = 0;
}

__global__ void k_ev_reset(unsigned* cnt, unsigned slots) {
  cnt[0] = 0;
  cnt[1] = 0;
  cnt[2] = 0;
  cnt[3] = slots;
  cnt[4] = 0;
}

// the collision queue's sort key of particle slot i
__device__ __forceinline__ int ev_sort_key(const DevWorld& w, const EvParams& ep, unsigned i) {
  const int t = (ep.st.tag[i] >> 1) & 1;
  const int m = __ldg(w.cell_mat + ep.st.cell[i]);
  return (t * w.n_materials + m) * w.G + ep.st.g[i];
}

// counting sort of the collision queue (when it is long enough): key counts
__global__ void __launch_bounds__(256) k_ev_sort_count(const DevWorld w, const EvParams ep) {
  __shared__ unsigned h[kEvSortKeys];
  const unsigned n = ep.cnt[2];
  if (n < ep.sort_min) return;  // the same for every block
  for (int k = threadIdx.x; k < kEvSortKeys; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x)
    atomicAdd(h + ev_sort_key(w, ep, static_cast<unsigned>(ep.q_coll[j])), 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < ep.sort_keys; k += blockDim.x)
    if (h[k]) atomicAdd(ep.sort_hist + k, h[k]);
}

// one block: exclusive scan of the counts into write positions, counts
// cleared for the next step, and the flag that tells the collide kernel
// which queue to read
__global__ void __launch_bounds__(kEvSortKeys) k_ev_sort_offsets(EvParams ep) {
  __shared__ unsigned s[kEvSortKeys];
  const unsigned n = ep.cnt[2];
  const bool sort = n >= ep.sort_min;
  const int k = threadIdx.x;
  const unsigned v = (sort && k < ep.sort_keys) ? ep.sort_hist[k] : 0;
  s[k] = v;
  __syncthreads();
  for (int off = 1; off < kEvSortKeys; off <<= 1) {
    const unsigned y = k >= off ? s[k - off] : 0;
    __syncthreads();
    s[k] += y;
    __syncthreads();
  }
  if (k < ep.sort_keys) {
    ep.sort_hist[kEvSortKeys + k] = s[k] - v;
    ep.sort_hist[k] = 0;
  }
  if (k == 0) ep.cnt[4] = sort ? 1u : 0u;
}

__global__ void __launch_bounds__(256) k_ev_sort_scatter(const DevWorld w, const EvParams ep) {
  if (!ep.cnt[4]) return;
  const unsigned n = ep.cnt[2];
  for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int32_t i = ep.q_coll[j];
    const unsigned pos = atomicAdd(ep.sort_hist + kEvSortKeys + ev_sort_key(w, ep, static_cast<unsigned>(i)), 1u);
    ep.q_sorted[pos] = i;
  }
}

template <class Rng>
static cudaError_t launch_all(const DevWorld& w, EvParams ep, const EvLaunch& L, cudaStream_t stream,
                              EvStepHook hook, void* hook_ctx) {
  const int block = 256;
  cudaError_t e;
  // slots [0, n) hold the histories' primaries; secondaries are appended
  k_ev_reset<<<1, 1, 0, stream>>>(ep.cnt, static_cast<unsigned>(ep.rp.n));
  // init appends the live primaries to the queue through cnt[1]
  int32_t* qa = ep.q_in;
  int32_t* qb = ep.q_out;
  ep.q_out = qa;
  k_ev_init<Rng><<<L.grid, block, 0, stream>>>(w, ep);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (hook) hook(hook_ctx, 2);
  // qa holds the live set.  Each iteration: swap counts on the device,
  // advance + collide from qa into qb, swap the queue pointers on the host.
  // The host reads the queue size only every check_every iterations.
  unsigned* pinned = nullptr;
  unsigned host_count = 1;
  for (unsigned iter = 0; iter < L.max_iterations; iter++) {
    k_ev_swap<<<1, 1, 0, stream>>>(ep.cnt);
    ep.q_in = qa;
    ep.q_out = qb;
    k_ev_advance_mg<Rng><<<L.grid, block, 0, stream>>>(w, ep);
    if (ep.sort_keys > 0) {
      k_ev_sort_count<<<L.grid, 256, 0, stream>>>(w, ep);
      k_ev_sort_offsets<<<1, kEvSortKeys, 0, stream>>>(ep);
      k_ev_sort_scatter<<<L.grid, 256, 0, stream>>>(w, ep);
      if (hook) hook(hook_ctx, 3);
    }
    k_ev_collide_mg<Rng><<<L.grid, block, 0, stream>>>(w, ep);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (hook) hook(hook_ctx, 3);
    std::swap(qa, qb);
    if ((iter + 1) % L.check_every == 0) {
      e = cudaMemcpyAsync(&host_count, ep.cnt + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
      if (e != cudaSuccess) return e;
      if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return e;
      if (host_count == 0) break;
    }
  }
  (void)pinned;
  if (host_count != 0) return cudaErrorLaunchTimeout;  // the iteration cap was reached
  // fission sites and the score commit are launched by the caller, after it
  // has checked the particle store did not overflow
  return cudaSuccess;
}

cudaError_t launch_event_mg(const DevWorld& w, const EvParams& ep, const EvLaunch& L, int rng_mode,
                            cudaStream_t stream, EvStepHook hook, void* hook_ctx) {
  if (rng_mode == 1) return launch_all<MinstdRng>(w, ep, L, stream, hook, hook_ctx);
  return launch_all<PhiloxRng>(w, ep, L, stream, hook, hook_ctx);
}

}  // namespace mcd
