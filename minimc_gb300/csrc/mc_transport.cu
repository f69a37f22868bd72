// Transport kernels: the particle-history loop of
//   FixedSource::StartWorker (src/FixedSource.cpp:40-77)
//   -> Particle::Transport -> SurfaceTracking / CellDeltaTracking::Transport
//      (src/TransportMethod.cpp:52-127)
// recast for the GPU.
//
// History schedule ("fused"): a persistent grid, one particle per thread.
// Every loop trip each live lane performs exactly one event; lanes whose
// history ended take the next history index from a global queue with one
// atomic per warp, so warps stay full until the queue drains.  Particle
// state lives in registers; HBM traffic is the source bank, the fission bank
// and the tallies.
#include "mc_history.cuh"

#include <type_traits>

namespace mcd {

using namespace hist;

namespace {

// fission: Multigroup::Fission (src/Multigroup.cpp:267-286).  The number of
// secondaries is floor(nubar + U); each draws its group from chi (incident
// group column) and an isotropic direction, then is seeded with rng()
// (Particle::BankSecondaries, src/Particle.cpp:96-100).
template <class Rng, class Emit>
__device__ __forceinline__ void mg_fission(const DevWorld& w, Particle<Rng>& p, int t, int nuc, bool fast,
                                           Emit&& emit) {
  const int G = w.G;
  const size_t base = (static_cast<size_t>(t) * w.n_nuclides + nuc) * G;
  const unsigned yield = mg_yield(w, p.rng, fast, base + p.g);
  const double* chi = w.mg_chi_cdf + (base + p.g) * G;
  for (unsigned i = 0; i < yield; i++) {
    const double thr = uniform(p.rng, fast);
    const int go = cdf_search(chi, G, 1, thr);
    if (go < 0) continue;
    Site s;
    sample_isotropic(p.rng, s.u, s.v, s.w, fast);
    s.x = p.x;
    s.y = p.y;
    s.z = p.z;
    s.energy = static_cast<double>(go + 1);
    s.key = p.rng.child_key();
    emit(s);
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// multigroup history loop of one CTA: the body of the single-problem kernel
// (world and run parameters in the kernel's parameter space) and of the
// batched kernel (copied into shared memory per CTA)
template <class Rng, bool KEIG, bool PERT = false>
__device__ __forceinline__ void history_mg(const DevWorld& w, const RunParams& rp, double* smem) {
  const bool use_smem = rp.total_bins <= kSharedBins && rp.score && !rp.nb;
  TallySink sink{use_smem ? smem : nullptr, use_smem ? smem + kSharedBins : nullptr, rp.tally_sum, rp.tally_sq};
  if (use_smem) {
    for (int i = threadIdx.x; i < 2 * kSharedBins; i += blockDim.x) smem[i] = 0;
    __syncthreads();
  }
  const unsigned lane = lane_id();
  const bool fast = rp.fast != 0;
  Particle<Rng> p;
  float fu = 0, fv = 0, fw = 0;  // the direction in FP32, for the box cells' preselection
  Pending<kPending> pend;
  pend.clear();
  ScorerT<true> sc{&pend, nullptr, rp.n};
  Site stack[KEIG ? 1 : kStack];
  int sp = 0;
  bool alive = false, done = false;
  unsigned long long hist = 0;
  unsigned long long my_events = 0, my_lost = 0, my_capped = 0, my_overflow = 0, my_sec = 0;
  double my_ktl = 0;
  uint32_t hist_nev = 0;
  int8_t fate = 0;
  // a secondary did not fit the stack: the history's result is invalid
  // (reported as an overflow), so its remaining particles are dropped,
  // which also bounds supercritical fixed-source chains
  bool dropped = false;

  // history complete: ScorableProxy::CommitHistory (src/Scorable.cpp:101-106)
  auto finish_history = [&]() {
    if (rp.score && !rp.nb) {
      sink.commit(pend);
      if (pend.overflow) my_overflow++;
    }
    pend.clear();
    if (rp.hist_events) rp.hist_events[hist] = hist_nev;
    if (rp.hist_fate) rp.hist_fate[hist] = fate;
  };

  for (;;) {
    // ---- refill: lanes without a live particle take the next history
    const bool want = !alive && !done;
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (mask) {
      const int leader = __ffs(mask) - 1;
      unsigned long long base = 0;
      if (lane == static_cast<unsigned>(leader)) base = atomicAdd(&rp.ctr->next, static_cast<unsigned long long>(__popc(mask)));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (want) {
        hist = base + __popc(mask & ((1u << lane) - 1u));
        if (hist >= rp.n) {
          done = true;
        }
        else {
          if (rp.from_bank) start_from_site(rp, hist, source_site(rp, hist), p, 0);
          else sample_source(w, rp, hist, p);
          fu = __double2float_rn(p.u);
          fv = __double2float_rn(p.v);
          fw = __double2float_rn(p.w);
          p.cell = find_cell(w, p.x, p.y, p.z);
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
            // the reference throws (src/World.cpp:34-36) or dereferences a
            // void material; the GPU counts the particle as lost
            alive = false;
            my_lost++;
            p.event = kLostEvent;
            fate = kLostEvent;
            rp.ctr->lost_xyz[0] = p.x;
            rp.ctr->lost_xyz[1] = p.y;
            rp.ctr->lost_xyz[2] = p.z;
            rp.ctr->pad[0] = static_cast<unsigned long long>(p.cell + 1);
            rp.ctr->pad[1] = hist;
            finish_history();
          }
        }
      }
    }
    if (__all_sync(0xffffffffu, done)) break;

    if (alive) {
      // ---- one event (SurfaceTracking::Transport body, src/TransportMethod.cpp:56-75)
      const int t = p.type;
      const int m = __ldg(w.cell_mat + p.cell);
      const size_t mg = (static_cast<size_t>(t) * w.n_materials + m) * w.G + p.g;
      const double micro = __ldg(w.mat_mg_total + mg);
      const double sigma = __ldg(w.mat_mg_sigma + mg);  // number_density * micro, tabulated
      const double dcol = mg_flight(w, p.rng, fast, mg, sigma);
      double dsurf;
      const int s = nearest_surface(w, p.cell, p.x, p.y, p.z, p.u, p.v, p.w, fu, fv, fw, dsurf, p.skip,
                                    std::is_same_v<Rng, PhiloxRng> && fast);
      const bool delta = w.tracking == 1;
      const bool collide = delta ? !(dsurf < dcol) : (dcol < dsurf);
      const bool refl = !collide && __ldg(w.surf_refl + s) != 0;
      // The move is the same arithmetic in every branch -- to the collision,
      // onto a reflecting plane, or across a surface plus the nudge -- so it
      // runs once for the whole warp (FP64 issue does not shrink with the
      // active lanes), before the branch-specific work.
      const double dcross = dadd(dsurf, kNudge);
      const double dmove = collide ? dcol : (refl ? dsurf : dcross);
      if (rp.score) score_track(w, p, dmove, sc);
      if (KEIG) my_ktl += dmove * __ldg(w.mat_mg_nusigf + mg);
      indirect_stream<PERT>(w, p, m, micro, dmove);
      move(fast, p.x, p.y, p.z, p.u, p.v, p.w, dmove);
      if (collide) {
        p.skip = -1;
        // multigroup majorant == total, so CellDeltaTracking's rejection
        // (src/TransportMethod.cpp:106-108) always accepts; it still draws
        if (delta) (void)uniform(p.rng, fast);
        // Particle::SampleNuclide (src/Particle.cpp:110-124)
        const int nb = __ldg(w.mat_begin + m), ne = __ldg(w.mat_begin + m + 1);
        const int nuc = __ldg(w.mat_nuc + nb + mg_pick_nuclide(w, p.rng, fast, mg, ne - nb, micro));
        // Multigroup::Interact (src/Multigroup.cpp:49-73)
        const size_t ng = (static_cast<size_t>(t) * w.n_nuclides + nuc) * w.G + p.g;
        const int rx = mg_pick_reaction(w, p.rng, fast, ng);
        if (rx == 0) {
          p.event = kCapture;
        }
        else if (rx == 1) {
          // Multigroup::Scatter (src/Multigroup.cpp:249-265)
          p.event = kScatter;
          const int go = mg_pick_outgoing(w, p.rng, fast, ng);
          if (go >= 0) {
            p.g = go;
            sample_isotropic(p.rng, p.u, p.v, p.w, fu, fv, fw, fast);
          }
        }
        else if (rx == 2) {
          p.event = kFission;
          if constexpr (KEIG) {
            // record the fission; its sites are drawn by the sites kernel
            // from the stream position after the yield draw
            const unsigned yield = mg_yield(w, p.rng, fast, ng);
            FissionRec f;
            f.x = p.x;
            f.y = p.y;
            f.z = p.z;
            f.g = p.g;
            f.n = yield;
            f.rng = p.rng.save();
            if constexpr (std::is_same_v<Rng, PhiloxRng>) {
              f.tag = p.rng.tag;
              f.id = static_cast<unsigned long long>(p.rng.h0) | (static_cast<unsigned long long>(p.rng.h1) << 32);
            }
            else {
              f.tag = 0;
              f.id = 0;
            }
            f.chi_index = static_cast<uint32_t>(ng);
            f.pad = 0;
            rp.fis[hist] = f;
          }
          else {
            mg_fission(w, p, t, nuc, fast, [&](const Site& st) {
              if (sp < kStack) stack[sp++] = st;
              else {
                my_overflow++;
                dropped = true;
              }
              my_sec++;
            });
          }
        }
      }
      else {
        if (refl) {
          // reflective boundary (extension): stop on the plane, mirror the
          // normal component, stay in the cell
          const int kind = __ldg(w.surf_kind + s);
          if (kind == kPlaneX) {
            p.u = -p.u;
            fu = -fu;
          }
          else if (kind == kPlaneY) {
            p.v = -p.v;
            fv = -fv;
          }
          else {
            p.w = -p.w;
            fw = -fw;
          }
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
            rp.ctr->lost_xyz[0] = p.x;
            rp.ctr->lost_xyz[1] = p.y;
            rp.ctr->lost_xyz[2] = p.z;
          }
          else {
            p.event = __ldg(w.cell_mat + p.cell) >= 0 ? kSurfaceCross : kLeak;
          }
        }
      }
      if (rp.score) score_event<false, PERT>(w, p, sc);
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
          // next particle of the same history (FixedSource bank loop,
          // src/FixedSource.cpp:63-72)
          const Site st = stack[--sp];
          p.x = st.x;
          p.y = st.y;
          p.z = st.z;
          p.u = st.u;
          p.v = st.v;
          p.w = st.w;
          fu = __double2float_rn(p.u);
          fv = __double2float_rn(p.v);
          fw = __double2float_rn(p.w);
          p.g = static_cast<int>(st.energy) - 1;
          p.type = 0;  // BankSecondaries creates neutrons
          if constexpr (std::is_same_v<Rng, PhiloxRng>) p.rng.init(rp.run_key, st.key, 1);
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

  // ---- counters: warp reduce, one atomic per warp
  for (int off = 16; off > 0; off >>= 1) {
    my_events += __shfl_down_sync(0xffffffffu, my_events, off);
    my_lost += __shfl_down_sync(0xffffffffu, my_lost, off);
    my_capped += __shfl_down_sync(0xffffffffu, my_capped, off);
    my_overflow += __shfl_down_sync(0xffffffffu, my_overflow, off);
    my_sec += __shfl_down_sync(0xffffffffu, my_sec, off);
    my_ktl += __shfl_down_sync(0xffffffffu, my_ktl, off);
  }
  if (lane == 0) {
    atomicAdd(&rp.ctr->events, my_events);
    if (my_lost) atomicAdd(&rp.ctr->lost, my_lost);
    if (my_capped) atomicAdd(&rp.ctr->capped, my_capped);
    if (my_overflow) atomicAdd(&rp.ctr->overflow, my_overflow);
    if (my_sec) atomicAdd(&rp.ctr->secondaries, my_sec);
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

// multigroup history kernel
// MINB: minimum resident 256-thread blocks per SM the register allocation
// must allow (1 = compiler's choice); the autotuner picks among variants
template <class Rng, bool KEIG, int MINB>
__global__ void __launch_bounds__(256, MINB) k_history_mg(const DevWorld w, const RunParams rp) {
  extern __shared__ double smem[];
  history_mg<Rng, KEIG>(w, rp, smem);
}

// fixed-source kernel carrying the indirect effects of perturbations and
// scoring sensitivity estimators
template <class Rng>
__global__ void __launch_bounds__(256, 1) k_history_mg_pert(const DevWorld w, const RunParams rp) {
  extern __shared__ double smem[];
  history_mg<Rng, false, true>(w, rp, smem);
}

// batched k-eigenvalue transport, a persistent grid over all problems:
// each problem's histories form its own global queue; a CTA starts on the
// problem its block table assigns (CTAs in proportion to the histories),
// drains that queue, then visits the other problems in turn and helps
// drain any queue that still holds histories, so small problems' CTAs do
// not idle while large ones run.  The world and run parameters of the
// problem a CTA serves sit in shared memory.  A history's result depends
// only on its problem, index and stream, not on the CTA that runs it.
template <int MINB>
__global__ void __launch_bounds__(256, MINB) k_history_mg_batch(const DevWorld* worlds, const RunParams* rps,
                                                                const uint32_t* block_problem, int P) {
  extern __shared__ double smem[];
  __shared__ DevWorld w;
  __shared__ RunParams rp;
  __shared__ int q_serve;
  const uint32_t p0 = block_problem[blockIdx.x];
  int q = 0;  // problems visited: p0, p0 + 1, ... (mod P)
  for (;;) {
    if (threadIdx.x == 0) {
      // the next problem whose queue still holds histories (a stale read
      // costs one empty visit); the CTA's own problem is always served
      while (q > 0 && q < P) {
        const uint32_t p = (p0 + static_cast<uint32_t>(q)) % static_cast<uint32_t>(P);
        if (*reinterpret_cast<volatile unsigned long long*>(&rps[p].ctr->next) < rps[p].n) break;
        q++;
      }
      q_serve = q;
      if (q < P) {
        const uint32_t p = (p0 + static_cast<uint32_t>(q)) % static_cast<uint32_t>(P);
        w = worlds[p];
        rp = rps[p];
      }
    }
    __syncthreads();
    if (q_serve >= P) break;
    history_mg<PhiloxRng, true>(w, rp, smem);
    q = q_serve + 1;
    __syncthreads();  // every warp is done with this problem's parameters
  }
}

// ---------------------------------------------------------------------------
// launches

namespace {
template <class K>
int occupancy(K kernel, int block, size_t smem) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, smem);
  return n;
}
}  // namespace

namespace {
template <int MINB>
int occupancy_mg(int rng_mode, int block, bool keig) {
  const size_t smem = 2 * kSharedBins * sizeof(double);
  if (rng_mode == 1) return keig ? occupancy(k_history_mg<MinstdRng, true, MINB>, block, smem)
                                 : occupancy(k_history_mg<MinstdRng, false, MINB>, block, smem);
  return keig ? occupancy(k_history_mg<PhiloxRng, true, MINB>, block, smem)
              : occupancy(k_history_mg<PhiloxRng, false, MINB>, block, smem);
}

template <int MINB>
void launch_mg(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block, cudaStream_t stream) {
  const size_t smem = 2 * kSharedBins * sizeof(double);
  if (rng_mode == 1) {
    if (rp.keig) k_history_mg<MinstdRng, true, MINB><<<grid, block, smem, stream>>>(w, rp);
    else k_history_mg<MinstdRng, false, MINB><<<grid, block, smem, stream>>>(w, rp);
  }
  else {
    if (rp.keig) k_history_mg<PhiloxRng, true, MINB><<<grid, block, smem, stream>>>(w, rp);
    else k_history_mg<PhiloxRng, false, MINB><<<grid, block, smem, stream>>>(w, rp);
  }
}
}  // namespace

namespace {
template <int MINB>
void launch_mg_batch(const DevWorld* worlds, const RunParams* rps, const uint32_t* block_problem, int grid, int P,
                     cudaStream_t stream) {
  k_history_mg_batch<MINB><<<grid, 256, 2 * kSharedBins * sizeof(double), stream>>>(worlds, rps, block_problem, P);
}
template <int MINB>
int occupancy_mg_batch() {
  return occupancy(k_history_mg_batch<MINB>, 256, 2 * kSharedBins * sizeof(double));
}
}  // namespace

cudaError_t launch_history_mg_batch(const DevWorld* worlds, const RunParams* rps, const uint32_t* block_problem,
                                    int grid, int P, cudaStream_t stream, int variant) {
  if (P < 1) return cudaErrorInvalidValue;
  switch (variant) {
  case 1: launch_mg_batch<3>(worlds, rps, block_problem, grid, P, stream); break;
  case 2: launch_mg_batch<4>(worlds, rps, block_problem, grid, P, stream); break;
  case 3: launch_mg_batch<5>(worlds, rps, block_problem, grid, P, stream); break;
  case 4: launch_mg_batch<6>(worlds, rps, block_problem, grid, P, stream); break;
  default: launch_mg_batch<1>(worlds, rps, block_problem, grid, P, stream); break;
  }
  return cudaGetLastError();
}

int history_batch_blocks_per_sm(int variant) {
  switch (variant) {
  case 1: return occupancy_mg_batch<3>();
  case 2: return occupancy_mg_batch<4>();
  case 3: return occupancy_mg_batch<5>();
  case 4: return occupancy_mg_batch<6>();
  default: return occupancy_mg_batch<1>();
  }
}

// variants: minimum 256-thread blocks per SM of 1 (compiler's choice), 3, 4,
// 5 and 6 -- register budgets of 255, 85, 64, 51 and 42 per thread
int history_variants() { return 5; }

int history_blocks_per_sm(int energy_mode, int rng_mode, int block, bool keig, bool fast, int variant) {
  (void)fast;
  if (energy_mode != 0) return 1;
  switch (variant) {
  case 1: return occupancy_mg<3>(rng_mode, block, keig);
  case 2: return occupancy_mg<4>(rng_mode, block, keig);
  case 3: return occupancy_mg<5>(rng_mode, block, keig);
  case 4: return occupancy_mg<6>(rng_mode, block, keig);
  default: return occupancy_mg<1>(rng_mode, block, keig);
  }
}

cudaError_t launch_history_mg(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block,
                              cudaStream_t stream, int variant) {
  if (w.n_pert > 0 && !rp.keig) {
    const size_t smem = 2 * kSharedBins * sizeof(double);
    if (rng_mode == 1) k_history_mg_pert<MinstdRng><<<grid, block, smem, stream>>>(w, rp);
    else k_history_mg_pert<PhiloxRng><<<grid, block, smem, stream>>>(w, rp);
    return cudaGetLastError();
  }
  switch (variant) {
  case 1: launch_mg<3>(w, rp, rng_mode, grid, block, stream); break;
  case 2: launch_mg<4>(w, rp, rng_mode, grid, block, stream); break;
  case 3: launch_mg<5>(w, rp, rng_mode, grid, block, stream); break;
  case 4: launch_mg<6>(w, rp, rng_mode, grid, block, stream); break;
  default: launch_mg<1>(w, rp, rng_mode, grid, block, stream); break;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fission bank: exclusive scan of per-history counts (three-phase block
// scan), compaction in history order, uniform resampling

namespace {
constexpr int kScanBlock = 1024;

// inclusive scan of v over a CTA of kScanBlock threads; *cta_total (every
// thread) = the CTA's sum
__device__ __forceinline__ unsigned long long cta_scan(unsigned long long v, unsigned long long* warp_sums,
                                                      unsigned long long* cta_total) {
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long x = v;
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= static_cast<unsigned>(off)) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned long long s = warp_sums[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= static_cast<unsigned>(off)) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  *cta_total = warp_sums[31];
  return (wid ? warp_sums[wid - 1] : 0) + x;
}

__global__ void k_scan_blocks(const uint32_t* count, unsigned long long n, unsigned long long* offsets,
                              unsigned long long* block_sums) {
  __shared__ unsigned long long warp_sums[32];
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * kScanBlock + threadIdx.x;
  const unsigned long long v = i < n ? count[i] : 0;
  unsigned long long tot;
  const unsigned long long x = cta_scan(v, warp_sums, &tot);
  if (i < n) offsets[i] = x - v;
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// The direct bank path's prefix sum, from the fission records themselves:
// history h yields min(n_h, max_yield) sites (sites past max_yield are
// dropped and counted, as the slot kernel does).  Pass 1 reads each
// record's n (one field of a 56-byte record, so the pass reads the whole
// record array), writes the capped counts to the compact count array and
// sums each CTA's counts; the one-CTA scan turns the sums into CTA
// prefixes and the bank size; pass 2 scans each CTA's counts again, from
// the compact array, and writes the finished offsets.
__global__ void __launch_bounds__(kScanBlock) k_count_block_sums(const RunParams rp, unsigned long long* block_sums) {
  __shared__ unsigned long long warp_sums[32];
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * kScanBlock + threadIdx.x;
  const uint32_t f = i < rp.n ? rp.fis[i].n : 0u;
  const uint32_t c = f < rp.max_yield ? f : rp.max_yield;
  if (i < rp.n) {
    rp.bank_count[i] = c;
    if (f > rp.max_yield) atomicAdd(&rp.ctr->overflow, static_cast<unsigned long long>(f - rp.max_yield));
  }
  unsigned long long v = c;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned long long s = warp_sums[threadIdx.x];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kScanBlock) k_count_offsets(const RunParams rp,
                                                              const unsigned long long* block_prefix,
                                                              unsigned long long* offsets) {
  __shared__ unsigned long long warp_sums[32];
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * kScanBlock + threadIdx.x;
  const uint32_t c = i < rp.n ? rp.bank_count[i] : 0u;
  unsigned long long tot;
  const unsigned long long x = cta_scan(c, warp_sums, &tot);
  if (i < rp.n) offsets[i] = block_prefix[blockIdx.x] + x - c;
}

__global__ void k_scan_sums(unsigned long long* block_sums, unsigned long long nb, unsigned long long* total) {
  // single block; nb is small (n / 1024)
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (unsigned long long base = 0; base < nb; base += blockDim.x) {
    const unsigned long long i = base + threadIdx.x;
    const unsigned long long v = i < nb ? block_sums[i] : 0;
    __shared__ unsigned long long buf[1024];
    buf[threadIdx.x] = v;
    __syncthreads();
    for (unsigned off = 1; off < blockDim.x; off <<= 1) {
      const unsigned long long y = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    if (i < nb) block_sums[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(unsigned long long* offsets, unsigned long long n, const unsigned long long* block_sums) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * kScanBlock + threadIdx.x;
  if (i < n) offsets[i] += block_sums[blockIdx.x];
}

__global__ void k_compact(const Site* slots, const uint32_t* count, const unsigned long long* offsets,
                          unsigned long long n, uint32_t max_yield, Site* out) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = count[i];
  const unsigned long long o = offsets[i];
  for (uint32_t k = 0; k < c; k++) out[o + k] = slots[i * max_yield + k];
}

// next source j = bank[floor(U_j * M)], U_j from Philox(key, counter j)
__global__ void k_resample(const Site* bank, const unsigned long long* total, unsigned long long n,
                           unsigned long long key, Site* next) {
  const unsigned long long j = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const unsigned long long m = *total;
  if (m == 0) return;
  next[j] = bank[resample_index(key, j, m)];
}
}  // namespace

cudaError_t launch_bank_scan(const uint32_t* count, unsigned long long n, unsigned long long* offsets,
                             unsigned long long* scratch_sums, unsigned long long* total, cudaStream_t stream) {
  const unsigned long long nb = (n + kScanBlock - 1) / kScanBlock;
  k_scan_blocks<<<static_cast<unsigned>(nb), kScanBlock, 0, stream>>>(count, n, offsets, scratch_sums);
  k_scan_sums<<<1, 1024, 0, stream>>>(scratch_sums, nb, total);
  k_scan_add<<<static_cast<unsigned>(nb), kScanBlock, 0, stream>>>(offsets, n, scratch_sums);
  return cudaGetLastError();
}

cudaError_t launch_direct_bank_scan(const RunParams& rp, unsigned long long* offsets, unsigned long long* scratch_sums,
                                    unsigned long long* total, cudaStream_t stream) {
  const unsigned long long nb = (rp.n + kScanBlock - 1) / kScanBlock;
  k_count_block_sums<<<static_cast<unsigned>(nb), kScanBlock, 0, stream>>>(rp, scratch_sums);
  k_scan_sums<<<1, 1024, 0, stream>>>(scratch_sums, nb, total);
  k_count_offsets<<<static_cast<unsigned>(nb), kScanBlock, 0, stream>>>(rp, scratch_sums, offsets);
  return cudaGetLastError();
}

cudaError_t launch_bank_compact(const Site* slots, const uint32_t* count, const unsigned long long* offsets,
                                unsigned long long n, uint32_t max_yield, Site* out, cudaStream_t stream) {
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  k_compact<<<blocks, 256, 0, stream>>>(slots, count, offsets, n, max_yield, out);
  return cudaGetLastError();
}

cudaError_t launch_resample(const Site* bank, const unsigned long long* total, unsigned long long n,
                            unsigned long long key, Site* next, cudaStream_t stream) {
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  k_resample<<<blocks, 256, 0, stream>>>(bank, total, n, key, next);
  return cudaGetLastError();
}

}  // namespace mcd
