// Continuous-energy history kernel: launch dispatch and the k-eigenvalue
// fission-site kernel.  The kernel template lives in mc_history_ce.cuh; its
// variants are instantiated in mc_transport_ce_{fx1,fx2,exact,ext}.cu.
#include "mc_history_ce.cuh"

namespace mcd {

// ---------------------------------------------------------------------------
// k-eigenvalue sites of the continuous-energy fissions: the stream resumes
// after the yield draw; each site draws an isotropic direction and is
// seeded with rng(), at the incident energy
namespace {
template <class Rng>
__global__ void __launch_bounds__(256) k_fission_sites_ce(const RunParams rp) {
  const bool fast = rp.fast != 0;
  unsigned long long my_overflow = 0;
  for (unsigned long long h = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; h < rp.n;
       h += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const FissionRec f = rp.fis[h];
    uint32_t written = 0;
    if (f.n) {
      Rng rng;
      rng.restore(rp.run_key, f.id, f.tag & 1u, f.rng);
      const double E = record_energy(f);
      Site* slots = rp.bank + h * rp.max_yield;
      for (uint32_t y = 0; y < f.n; y++) {
        Site s;
        sample_isotropic(rng, s.u, s.v, s.w, fast);
        s.x = f.x;
        s.y = f.y;
        s.z = f.z;
        s.energy = E;
        s.key = rng.child_key();
        if (written < rp.max_yield) slots[written++] = s;
        else my_overflow++;
      }
    }
    rp.bank_count[h] = written;
  }
  if (my_overflow) atomicAdd(&rp.ctr->overflow, my_overflow);
}

// direct bank path: the same draws as k_fission_sites_ce, each history's
// min(n, max_yield) sites staged at their bank positions
template <class Rng>
__global__ void __launch_bounds__(kSitesOutHist) k_fission_sites_out_ce(const RunParams rp,
                                                                        const unsigned long long* offsets,
                                                                        const unsigned long long* total,
                                                                        unsigned long long cap, uint4* out) {
  extern __shared__ uint4 stage[];  // minstd: [kSitesOutHist * max_yield] sites
  const bool fast = rp.fast != 0;
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    // a site draws a fixed number of 32-bit words -- the isotropic direction
    // (2 in the FP32 form, 4 in FP64) and the secondary's key (2) -- so each
    // site starts at a known stream position and has a thread of its own
    const uint32_t words = (fast ? 2u : 4u) + 2u;
    sites_out_cta_by_site(rp.n, offsets, total, cap, out, [&](unsigned long long h, uint32_t y, Site* dst) {
      const FissionRec f = rp.fis[h];
      PhiloxRng rng;
      rng.restore(rp.run_key, f.id, f.tag & 1u, philox_skip(f.rng, y * words));
      Site s;
      sample_isotropic(rng, s.u, s.v, s.w, fast);
      s.x = f.x;
      s.y = f.y;
      s.z = f.z;
      s.energy = record_energy(f);
      s.key = rng.child_key();
      *dst = s;
    });
  }
  else {
    sites_out_cta(rp.n, rp.bank_count, offsets, total, cap, out, stage,
                  [&](unsigned long long h, uint32_t c, Site* dst) {
                    const FissionRec f = rp.fis[h];
                    Rng rng;
                    rng.restore(rp.run_key, f.id, f.tag & 1u, f.rng);
                    const double E = record_energy(f);
                    for (uint32_t y = 0; y < c; y++) {
                      Site s;
                      sample_isotropic(rng, s.u, s.v, s.w, fast);
                      s.x = f.x;
                      s.y = f.y;
                      s.z = f.z;
                      s.energy = E;
                      s.key = rng.child_key();
                      dst[y] = s;
                    }
                  });
  }
}

constexpr int kMinb[5] = {1, 3, 4, 5, 6};  // occupancy variants (autotuner index)
}  // namespace

cudaError_t launch_fission_sites_out_ce(const RunParams& rp, int rng_mode, const unsigned long long* offsets,
                                        const unsigned long long* total, unsigned long long cap, Site* out,
                                        cudaStream_t stream) {
  const unsigned grid = static_cast<unsigned>((rp.n + kSitesOutHist - 1) / kSitesOutHist);
  auto* o = reinterpret_cast<uint4*>(out);
  if (rng_mode == 1) {
    // minstd: one thread per history, its sites staged whole
    const size_t smem = sites_out_smem(rp.max_yield);
    if (smem > kSitesOutMaxSmem) return cudaErrorInvalidValue;
    // the attribute is per device, so it is set at every launch (a host-side call)
    const cudaError_t e = cudaFuncSetAttribute(k_fission_sites_out_ce<MinstdRng>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    k_fission_sites_out_ce<MinstdRng><<<grid, kSitesOutHist, smem, stream>>>(rp, offsets, total, cap, o);
  }
  else {
    // Philox: one thread per site through a fixed window (no dynamic shared memory)
    k_fission_sites_out_ce<PhiloxRng><<<grid, kSitesOutHist, 0, stream>>>(rp, offsets, total, cap, o);
  }
  return cudaGetLastError();
}

bool ce_uses_fp32_tables(const DevWorld& w, int rng_mode, bool fast) {
  return rng_mode != 1 && fast && w.ce.fast_ok && w.n_pert == 0;
}

int history_blocks_per_sm_ce(const DevWorld& w, int rng_mode, int block, bool keig, bool fast, int variant) {
  if (!ce_uses_fp32_tables(w, rng_mode, fast)) return cevar::occupancy_exact(rng_mode, block, keig);
  const int minb = kMinb[variant >= 0 && variant < 5 ? variant : 0];
  return cevar::has_fx1(minb) ? cevar::occupancy_fx1(minb, block, keig) : cevar::occupancy_fx2(minb, block, keig);
}

cudaError_t launch_history_ce_tq(const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream) {
  cevar::launch_tq(w, rp, grid, block, stream);
  return cudaGetLastError();
}

cudaError_t launch_history_ce(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block,
                              cudaStream_t stream, int variant) {
  if (w.n_pert > 0 && !rp.keig) {
    // perturbations: the exact tables, with indirect effects
    cevar::launch_pert(w, rp, rng_mode, grid, block, stream);
    return cudaGetLastError();
  }
  if (!ce_uses_fp32_tables(w, rng_mode, rp.fast != 0)) {
    cevar::launch_exact(w, rp, rng_mode, grid, block, stream);
    return cudaGetLastError();
  }
  const int minb = kMinb[variant >= 0 && variant < 5 ? variant : 0];
  if (cevar::has_fx1(minb)) cevar::launch_fx1(minb, w, rp, grid, block, stream);
  else cevar::launch_fx2(minb, w, rp, grid, block, stream);
  return cudaGetLastError();
}

cudaError_t launch_fission_sites_ce(const RunParams& rp, int rng_mode, int grid, cudaStream_t stream) {
  if (rng_mode == 1) k_fission_sites_ce<MinstdRng><<<grid, 256, 0, stream>>>(rp);
  else k_fission_sites_ce<PhiloxRng><<<grid, 256, 0, stream>>>(rp);
  return cudaGetLastError();
}

}  // namespace mcd
