// Kernel launch interface shared by the transport kernels and the C ABI.
#pragma once

#include "mc_device.cuh"

#include <type_traits>

namespace mcd {

// mc_site layout (include/minimc_gb300.h)
struct Site {
  double x, y, z, u, v, w, energy;
  unsigned long long key;
};

// a k-eigenvalue fission: where, the incident group and the stream
// position right after the yield draw, from which the sites are generated
// by a separate kernel (keeps the per-site sampling out of the transport loop)
struct FissionRec {
  double x, y, z;
  int32_t g;
  uint32_t n;
  uint32_t rng;
  uint32_t tag;
  unsigned long long id;
  uint32_t chi_index;  // (type, nuclide, incident group) row of the chi table
  uint32_t pad;
};

// most tally bins kept densely per history; more bins use a per-thread list
constexpr int kDenseBins = 64;

// Thermal-scatter queue (surrogate sampler).  A fixed-source particle whose
// collision is a thermal scatter of the surrogate's library, inside its
// trained (E, T) box, is parked: its state goes to a ParkRec and its
// sampler inputs (E, T and two uniforms from its own stream) to a float4
// row; the history kernel moves on.  One batched tensor-core launch samples
// (beta, alpha) for all parked rows, and a resume launch of the history
// kernel applies each outcome and continues the particle.
constexpr int kParkPending = 4;  // pending tally bins a parked history may carry
constexpr int kTqRounds = 6;     // park/sample/resume rounds; the last resume samples inline

struct ParkRec {
  double x, y, z, u, v, w, E, T;
  unsigned long long hist;
  unsigned long long rng_id;   // Philox counter words h0 | h1 << 32
  int32_t cell, surf, skip, type;
  uint32_t nev, hist_nev;
  uint32_t rng_pos;            // PhiloxRng::save()
  uint32_t rng_tag;
  int32_t fate;                // history fate so far
  int32_t flags;               // bit 0: dropped secondaries
  int32_t pend_n;              // pending tally entries (<= kParkPending); bit 8: overflow
  int32_t tsl;
  uint32_t pend_bin[kParkPending];
  double pend_score[kParkPending];
};

struct RunParams {
  unsigned long long n;        // source particles (histories)
  unsigned long long seed;     // run seed
  unsigned long long run_key;  // Philox key of this run/cycle
  unsigned long long minstd_base;  // k-eigenvalue: minstd seed of source 0 of the cycle
  uint32_t cycle;
  uint32_t max_events;
  int32_t keig;        // 1: bank fission sites and end the history
  int32_t score;       // 1: accumulate estimator scores
  int32_t fast;        // 1: FP32 sampling arithmetic
  int32_t from_bank;   // 1: particles come from src[]; 0: sampled from Source
  int32_t ref_source_seeds;  // 1: source i uses Source::Sample(seed + i)
  uint32_t max_yield;
  const Site* src;
  Site* bank;          // k-eigenvalue: [n * max_yield] per-history slots
  uint32_t* bank_count;  // [n]
  double* tally_sum;
  double* tally_sq;
  unsigned long long total_bins;
  uint32_t* hist_events;
  int8_t* hist_fate;
  DevCounters* ctr;
  double* pend;        // dense per-history scores [n][nb] when nb <= kDenseBins
  int32_t nb;
  FissionRec* fis;     // k-eigenvalue fission records [n]
  // thermal-scatter queue (continuous-energy fixed source, Philox streams)
  int32_t tq;                          // 1: park thermal scatters of library tq_tsl inside tq_box
  int32_t tq_tsl;
  double tq_box[4];                    // E min, E max (MeV), T min, T max (K)
  unsigned long long* head;            // queue head of this launch (null: &ctr->next)
  const unsigned long long* n_resume;  // resume launch: parked records to continue (device count)
  const ParkRec* park_in;
  const float2* tq_out;                // (beta, alpha) per parked record; NaN: sample inline
  ParkRec* park_out;
  float4* tq_in;                       // (E, T, u1, u2) per parked record
  unsigned long long* park_count;      // records parked by this launch
  unsigned long long park_cap;
  int32_t direct_sites;  // k-eigenvalue: sites go straight into the bank (no slot kernel)
  // thermal-scatter queue forms: 1 the quantile surrogate (tq_in / tq_out),
  // 2 the guided sampler and 3 the plain POD queue (tq_rows / tq_res: POD-exact
  // samples drawn from the particle's own stream)
  int32_t tq_mode;
  GuideRow* tq_rows;
  const GuideOut* tq_res;
  // resampling fused into the source read (k-eigenvalue cycles after the
  // first): with resample_m set, source i is the bank entry the resampling
  // draw picks -- resample_bank[resample_index(resample_key, i, *resample_m)]
  // -- and src is not read
  const Site* resample_bank;
  const unsigned long long* resample_m;
  unsigned long long resample_key;
  int32_t tq_fast;  // thermal queue modes 2, 3: the queue samples the FP32 POD form (else the exact one)
};

// KEigenvalue's next source, uniform over the bank: source j is bank entry
// floor(U_j * M), U_j a 53-bit uniform from Philox(key; j, "resa").  The
// resampling kernels and the fused source read share this draw.
__device__ __forceinline__ unsigned long long resample_index(unsigned long long key, unsigned long long j,
                                                             unsigned long long m) {
  const uint4 c = philox_block(static_cast<uint32_t>(j), static_cast<uint32_t>(j >> 32), 0x72657361u, 0u,
                               static_cast<uint32_t>(key), static_cast<uint32_t>(key >> 32));
  const double u = ((c.x >> 5) * 67108864.0 + (c.y >> 6)) * (1.0 / 9007199254740992.0);
  const unsigned long long idx = static_cast<unsigned long long>(u * static_cast<double>(m));
  return idx < m ? idx : m - 1;
}

// source site i of a run from a bank (*resample_m >= 1: callers never
// resample an empty bank)
__device__ __forceinline__ Site source_site(const RunParams& rp, unsigned long long i) {
  if (rp.resample_m) return rp.resample_bank[resample_index(rp.resample_key, i, *rp.resample_m)];
  return rp.src[i];
}

// k-eigenvalue sites from fission records and the per-history commit of
// dense scores (mc_event.cu)
cudaError_t launch_fission_sites_mg(const DevWorld& w, const RunParams& rp, int rng_mode, int grid,
                                    cudaStream_t stream);
cudaError_t launch_commit_dense(const RunParams& rp, int grid, cudaStream_t stream);

// k-eigenvalue sites straight into a compacted bank, where every fission
// record's site count is known before sampling (multigroup: Philox streams
// and chi cdfs that all end above the largest uniform the stream draws;
// continuous energy: always): per-history counts min(n, max_yield) into
// bank_count with their scan (launch_direct_bank_scan), then the sites,
// staged per CTA of kSitesOutHist histories in shared memory and stored to
// `out` (device or
// page-locked host memory, 16-byte aligned) with coalesced 16-byte writes;
// sites at or past `cap` are not written
constexpr int kSitesOutHist = 128;
constexpr size_t kSitesOutMaxSmem = 192 * 1024;
size_t sites_out_smem(uint32_t max_yield);
bool sites_out_fits(uint32_t max_yield);
cudaError_t launch_fission_sites_out_mg(const DevWorld& w, const RunParams& rp, const unsigned long long* offsets,
                                        const unsigned long long* total, unsigned long long cap, Site* out,
                                        cudaStream_t stream);
// batched problems (Philox): histories concatenated, offsets off[0..P].
// sites_out_batch_prepare sets the kernel's shared-memory limit (a host
// call, made before a graph capture of the launch)
cudaError_t sites_out_batch_prepare(uint32_t max_yield);
cudaError_t launch_fission_sites_out_mg_batch(const DevWorld* worlds, const RunParams* rps,
                                              const unsigned long long* off, int P, unsigned long long N,
                                              uint32_t max_yield, bool fast, const FissionRec* fis,
                                              const uint32_t* count, const unsigned long long* offsets,
                                              const unsigned long long* total, Site* out, cudaStream_t stream);
cudaError_t launch_fission_sites_out_ce(const RunParams& rp, int rng_mode, const unsigned long long* offsets,
                                        const unsigned long long* total, unsigned long long cap, Site* out,
                                        cudaStream_t stream);

// One CTA of the direct bank path.  The CTA owns histories
// [blockIdx.x * kSitesOutHist, ...) of n; sample(h, c, dst) writes history
// h's c = count[h] sites to dst (shared memory, at the history's bank
// position relative to the CTA's first site); then the CTA stores its
// contiguous share of the bank with coalesced 16-byte writes, skipping sites
// at or past cap.
template <class Sample>
__device__ __forceinline__ void sites_out_cta(unsigned long long n, const uint32_t* count,
                                              const unsigned long long* offsets, const unsigned long long* total,
                                              unsigned long long cap, uint4* out, uint4* stage, Sample&& sample) {
  static_assert(sizeof(Site) % sizeof(uint4) == 0, "sites are stored as 16-byte words");
  const unsigned long long first = static_cast<unsigned long long>(blockIdx.x) * kSitesOutHist;
  const unsigned long long last = first + kSitesOutHist < n ? first + kSitesOutHist : n;
  const unsigned long long base = offsets[first];
  const unsigned long long end = last < n ? offsets[last] : *total;
  const unsigned long long h = first + threadIdx.x;
  if (h < n) {
    const uint32_t c = count[h];
    if (c) sample(h, c, reinterpret_cast<Site*>(stage) + (offsets[h] - base));
  }
  __syncthreads();
  const unsigned long long m = end - base;
  const unsigned long long keep = base >= cap ? 0 : (m < cap - base ? m : cap - base);
  constexpr unsigned kWords = sizeof(Site) / sizeof(uint4);
  for (unsigned long long i = threadIdx.x; i < keep * kWords; i += kSitesOutHist) out[base * kWords + i] = stage[i];
}

// The same CTA with one thread per site instead of one per history: the
// CTA's histories' bank offsets go to shared memory, each thread finds the
// history and the index y of its site there, and site(h, y, dst) writes
// that one site (a history's sites are then sampled by neighbouring
// threads side by side, not one after another by one thread).  The CTA's
// sites pass through a window of kSitesOutHist sites in shared memory, one
// window after another, so its footprint (9 KB) does not grow with the
// largest yield and the kernel keeps its occupancy; each window is stored
// with coalesced 16-byte writes.  blockDim.x must be kSitesOutHist.
template <class SiteFn>
__device__ __forceinline__ void sites_out_cta_by_site(unsigned long long n, const unsigned long long* offsets,
                                                      const unsigned long long* total, unsigned long long cap,
                                                      uint4* out, SiteFn&& site) {
  static_assert(sizeof(Site) % sizeof(uint4) == 0, "sites are stored as 16-byte words");
  constexpr unsigned kWords = sizeof(Site) / sizeof(uint4);
  __shared__ unsigned long long s_off[kSitesOutHist + 1];
  __shared__ uint4 win[kSitesOutHist * kWords];
  const unsigned long long first = static_cast<unsigned long long>(blockIdx.x) * kSitesOutHist;
  const unsigned long long last = first + kSitesOutHist < n ? first + kSitesOutHist : n;
  const int H = static_cast<int>(last - first);
  const unsigned long long base = offsets[first];
  const unsigned long long end = last < n ? offsets[last] : *total;
  for (int i = threadIdx.x; i < H; i += blockDim.x) s_off[i] = offsets[first + i] - base;
  if (threadIdx.x == 0) s_off[H] = end - base;
  __syncthreads();
  const unsigned long long m = end - base;
  for (unsigned long long w0 = 0; w0 < m; w0 += kSitesOutHist) {
    const unsigned long long j = w0 + threadIdx.x;
    if (j < m) {
      // the history whose sites hold j: the last k with s_off[k] <= j
      int lo = 0, hi = H;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (s_off[mid] <= j) lo = mid;
        else hi = mid;
      }
      site(first + lo, static_cast<uint32_t>(j - s_off[lo]), reinterpret_cast<Site*>(win) + threadIdx.x);
    }
    __syncthreads();
    const unsigned long long at = base + w0;
    const unsigned long long cnt = m - w0 < kSitesOutHist ? m - w0 : kSitesOutHist;
    const unsigned long long keep = at >= cap ? 0 : (cnt < cap - at ? cnt : cap - at);
    for (unsigned long long i = threadIdx.x; i < keep * kWords; i += kSitesOutHist) out[at * kWords + i] = win[i];
    __syncthreads();
  }
}

// A Philox stream position (PhiloxRng::save's packing) s words further on
__device__ __forceinline__ uint32_t philox_skip(uint32_t packed, uint32_t s) {
  const uint32_t p = 4u * (packed >> 3) + (packed & 7u) - 4u + s;  // word index of the next draw
  return ((p / 4u + 1u) << 3) | (p % 4u);
}

// launches (mc_transport.cu)
// history-schedule kernel variants differ only in their occupancy target
// (register budget); results are identical, the autotuner times them
int history_variants();
cudaError_t launch_history_mg(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block,
                              cudaStream_t stream, int variant);
int history_blocks_per_sm(int energy_mode, int rng_mode, int block, bool keig, bool fast, int variant);

// batched multigroup k-eigenvalue transport (mc_transport.cu): CTA b starts
// on problem block_problem[b], then helps drain the other P - 1 problems'
// queues
cudaError_t launch_history_mg_batch(const DevWorld* worlds, const RunParams* rps, const uint32_t* block_problem,
                                    int grid, int P, cudaStream_t stream, int variant);
int history_batch_blocks_per_sm(int variant);
cudaError_t launch_fission_sites_mg_batch(const DevWorld* worlds, const RunParams* rps, const uint32_t* block_problem,
                                          const uint32_t* block_first, int grid, cudaStream_t stream);

// one k-eigenvalue cycle's results kept on the device (mc_batch.cu): bank
// size M and k = M / n into out[3 * i .. 3 * i + 2] = (k, M, k_tracklength),
// the run counters added into acc (lost_xyz and pad kept from the first
// cycle that lost a particle); an empty bank sets acc->next and leaves
// *total = 1, so that the cycles queued behind it read bank entry 0 -- a
// site some earlier cycle wrote (mc_keig_cycles runs the first cycle on its
// own and checks its bank) -- until the caller reports the error
cudaError_t launch_keig_record(const DevCounters* ctr, unsigned long long* total, unsigned long long n,
                               double* out, DevCounters* acc, cudaStream_t stream);

// batched k-eigenvalue cycle bookkeeping (mc_batch.cu)
struct BatchCycle {
  int P;
  int max_cycles;
  unsigned long long N;                 // histories of all problems
  const unsigned long long* off;        // [P + 1] first history of each problem
  const unsigned long long* seeds;      // [P]
  RunParams* rps;                       // [P]
  DevCounters* ctr;                     // [P]
  unsigned long long* start;            // [P] first banked site of each problem
  unsigned long long* M;                // [P] banked sites
  double* k;                            // [P][max_cycles]
  unsigned long long* stats;            // [P][4] events, lost, capped, overflow (all cycles)
  uint32_t* cycle;                      // current cycle
  int* died;                            // a problem's bank was empty
};
// sets every problem's cycle fields (keys, source) for the current cycle
cudaError_t launch_batch_begin(const BatchCycle& b, const Site* src, cudaStream_t s);
// per-problem bank sizes and k from the global scan; counter totals
cudaError_t launch_batch_tally(const BatchCycle& b, const unsigned long long* offsets,
                               const unsigned long long* total, cudaStream_t s);
// next sources of every problem from its part of the compacted bank; cycle++
cudaError_t launch_batch_resample(const BatchCycle& b, const Site* bank, Site* next, cudaStream_t s);

// continuous energy (mc_transport_ce.cu)
bool ce_uses_fp32_tables(const DevWorld& w, int rng_mode, bool fast);
cudaError_t launch_history_ce(const DevWorld& w, const RunParams& rp, int rng_mode, int grid, int block,
                              cudaStream_t stream, int variant);
int history_blocks_per_sm_ce(const DevWorld& w, int rng_mode, int block, bool keig, bool fast, int variant);
// fixed source with the thermal-scatter queue (Philox streams, exact tables):
// a source launch (rp.n_resume null) or a resume launch
cudaError_t launch_history_ce_tq(const DevWorld& w, const RunParams& rp, int grid, int block, cudaStream_t stream);
cudaError_t launch_fission_sites_ce(const RunParams& rp, int rng_mode, int grid, cudaStream_t stream);

// thermal scattering sampler and totals (mc_tsl.cu); rng_mode 1 = minstd
// seeded seed + i, else Philox keyed by `key`, counter i
cudaError_t launch_sample_tsl(const DevTSL* tsl, bool fast, int rng_mode, const double* E, const double* T,
                              unsigned long long n, unsigned long long seed, unsigned long long key, double* beta,
                              double* alpha, unsigned long long* failures, cudaStream_t stream);
cudaError_t launch_tsl_total(const DevTSL* tsl, const double* E, const double* T, unsigned long long n, double* out,
                             cudaStream_t stream);
// multigroup transfer of thermal scatters (mc_tsl.cu): rows of (E, T)
// repeated over n samples, and the samples' outgoing groups counted per row
constexpr int kMaxTransferGroups = 64;
cudaError_t launch_expand_rows(const double* E_rows, const double* T_rows, unsigned rows, unsigned long long n,
                               double* E, double* T, cudaStream_t stream);
cudaError_t launch_group_bins(const double* beta, unsigned rows, unsigned long long n, const double* E_rows,
                              const double* T_rows, const double* bounds, int G, unsigned long long* counts,
                              cudaStream_t stream);

// thin SVD of the POD table pipeline by one-sided Jacobi rotations
// (mc_pod.cu): V = I, then sweeps until one makes no rotation, then the
// column norms of A V
cudaError_t launch_jacobi_init(double* V, int n, cudaStream_t stream);
cudaError_t launch_jacobi_sweep(double* A, double* V, int m, int n, double tol, unsigned* rotations,
                                cudaStream_t stream);
cudaError_t launch_column_norms(const double* A, int m, int n, double* S, cudaStream_t stream);

// bank compaction and resampling (mc_transport.cu)
cudaError_t launch_bank_scan(const uint32_t* count, unsigned long long n, unsigned long long* offsets,
                             unsigned long long* scratch_sums, unsigned long long* total, cudaStream_t stream);
// the direct bank path's counts (min(n, max_yield) per fission record, into
// rp.bank_count, overflow counted in rp.ctr), their exclusive prefix sum and
// the bank size, in three launches
cudaError_t launch_direct_bank_scan(const RunParams& rp, unsigned long long* offsets, unsigned long long* scratch_sums,
                                    unsigned long long* total, cudaStream_t stream);
cudaError_t launch_bank_compact(const Site* slots, const uint32_t* count, const unsigned long long* offsets,
                                unsigned long long n, uint32_t max_yield, Site* out, cudaStream_t stream);
cudaError_t launch_resample(const Site* bank, const unsigned long long* total, unsigned long long n,
                            unsigned long long key, Site* next, cudaStream_t stream);

// parity probes (mc_probe.cu)
cudaError_t launch_find_cell(const DevWorld& w, const double* xyz, unsigned long long n, int32_t* cell,
                             cudaStream_t stream);
cudaError_t launch_nearest_surface(const DevWorld& w, const int32_t* cell, const double* xyz, const double* uvw,
                                   unsigned long long n, int32_t* surf, double* dist, cudaStream_t stream);
cudaError_t launch_surface_distance(const DevWorld& w, int32_t s, const double* xyz, const double* uvw,
                                    unsigned long long n, double* dist, cudaStream_t stream);
cudaError_t launch_surface_contains(const DevWorld& w, int32_t s, const double* xyz, unsigned long long n,
                                    int8_t* out, cudaStream_t stream);
cudaError_t launch_material_xs_mg(const DevWorld& w, int32_t cell, const double* energy, unsigned long long n,
                                  double* total, double* majorant, cudaStream_t stream);
cudaError_t launch_material_xs_ce(const DevWorld& w, int32_t cell, const double* energy, const double* xyz,
                                  unsigned long long n, double* total, double* majorant, cudaStream_t stream);
cudaError_t launch_energy_index(const DevWorld& w, int32_t nuclide, const double* energy, unsigned long long n,
                                long long* out, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Multigroup collision choices, shared by the history and event schedules so
// that both draw the same numbers and take the same decisions.  The exact
// form follows the reference (FP64 thresholds against FP64 running sums);
// the fast form (Philox streams, fast_math) forms the threshold in FP32 and
// searches the FP32 copies of the same running sums.

// Particle::SampleNuclide (src/Particle.cpp:110-124); a material of one
// nuclide returns it whatever the threshold (micro * U < micro), so only
// the draw is made
template <class Rng>
__device__ __forceinline__ int mg_pick_nuclide(const DevWorld& w, Rng& rng, bool fast, size_t mg, int count,
                                               double micro) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) {
      const float u = rng.u01f();
      if (count == 1) return 0;
      const int k = cdf_first_above_f(w.mat_mg_nuc_cdf_f + mg * w.max_mat_nuc, count,
                                      __fmul_rn(__ldg(w.mat_mg_total_f + mg), u));
      return k < 0 ? count - 1 : k;
    }
  }
  const double u = rng.u01();
  if (count == 1) return 0;
  const int k = cdf_first_above(w.mat_mg_nuc_cdf + mg * w.max_mat_nuc, count, dmul(micro, u));
  return k < 0 ? count - 1 : k;  // unreachable in the reference (assert)
}

// Multigroup::Interact's reaction (src/Multigroup.cpp:49-73): 0 capture,
// 1 scatter, 2 fission, -1 none (threshold at the top of the CDF)
template <class Rng>
__device__ __forceinline__ int mg_pick_reaction(const DevWorld& w, Rng& rng, bool fast, size_t ng) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return cdf_first_above_f(w.mg_rx_cdf_f + ng * 3, 3, __fmul_rn(rng.u01f(), __ldg(w.mg_total_f + ng)));
  }
  return cdf_first_above(w.mg_rx_cdf + ng * 3, 3, dmul(rng.u01(), __ldg(w.mg_total + ng)));
}

// Multigroup::Scatter's outgoing group (src/Multigroup.cpp:249-265), or -1
template <class Rng>
__device__ __forceinline__ int mg_pick_outgoing(const DevWorld& w, Rng& rng, bool fast, size_t ng) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return cdf_first_above_f(w.mg_scat_cdf_f + ng * w.G, w.G, rng.u01f());
  }
  return cdf_first_above(w.mg_scat_cdf + ng * w.G, w.G, rng.u01());
}

// Multigroup::Fission's yield floor(nubar + U) (src/Multigroup.cpp:267-272)
template <class Rng>
__device__ __forceinline__ unsigned mg_yield(const DevWorld& w, Rng& rng, bool fast, size_t ng) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return static_cast<unsigned>(__fadd_rn(__ldg(w.mg_nubar_f + ng), rng.u01f()));
  }
  return static_cast<unsigned>(dadd(__ldg(w.mg_nubar + ng), rng.u01()));
}

// exponential flight in a multigroup material: -log(1 - U) / sigma, the
// fast form from the FP32 macroscopic total
template <class Rng>
__device__ __forceinline__ double mg_flight(const DevWorld& w, Rng& rng, bool fast, size_t mg, double sigma) {
  if constexpr (std::is_same_v<Rng, PhiloxRng>) {
    if (fast) return flight_fast_f(rng.u01f(), __ldg(w.mat_mg_sigma_f + mg));
  }
  return ddiv(-log(dsub(1.0, rng.u01())), sigma);
}

// Particle::Stream: position += direction * d; the fast form rounds each
// coordinate once (fused multiply-add)
__device__ __forceinline__ void move(bool fast, double& x, double& y, double& z, double u, double v, double w,
                                     double d) {
  if (fast) {
    x = fma(u, d, x);
    y = fma(v, d, y);
    z = fma(w, d, z);
  }
  else {
    x = dadd(x, dmul(u, d));
    y = dadd(y, dmul(v, d));
    z = dadd(z, dmul(w, d));
  }
}

// Philox helper shared with the host-side resampler description
__host__ __device__ inline unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace mcd
