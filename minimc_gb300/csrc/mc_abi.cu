// C ABI (include/minimc_gb300.h): context, world upload and the solvers.
#include "../../include/minimc_gb300.h"
#include "mc_ce_tables.hpp"
#include "mc_event.cuh"
#include "mc_kernels.cuh"
#include "mc_mlp.cuh"
#include "mc_tsl.cuh"
#include "mc_model.hpp"
#include "mc_output.hpp"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <exception>
#include <mutex>
#include <string>
#include <vector>

using mcd::DevCounters;
using mcd::DevWorld;
using mcd::RunParams;
using mcd::Site;

static_assert(sizeof(mc_site) == sizeof(Site), "mc_site layout");

struct DevBuffer {
  void* p = nullptr;
  size_t bytes = 0;
};

// device scratch buffers of a context, grown on demand
enum ScratchSlot {
  kSrc = 0,
  kSlots,
  kCount,
  kOffsets,
  kScanSums,
  kTotal,        // (unused: the bank size lives after the run counters)
  kBank,
  kHistEvents,
  kHistFate,
  kProbeIn,
  kProbeIn2,
  kProbeOut,
  kEvState,
  kEvQueues,
  kEvCnt,
  kEvPend,
  kEvFis,
  kTslFail,
  kParkA,
  kParkB,
  kTqIn,
  kTqOut,
  kTqCnt,
  kTqRows,
  kTqRes,
  kGroupRows,     // thermal group transfer: rows, bounds, counts
  kGroupSamples,  // thermal group transfer: one chunk's samples
  kCycleRec,      // mc_keig_cycles: per-cycle records and counters
  kEvPend2,       // second dense per-history score array (alternate runs)
  kPodA,          // mc_pod_svd: the matrix being orthogonalised
  kPodV,          // mc_pod_svd: V, the singular values and the rotation count
  kScratchSlots,  // number of slots
};

struct mc_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::string ce_fast_reason;  // why the FP32 union tables are off, if they are
  bool loaded = false;
  mc::Model model;
  std::vector<void*> world_allocs;
  DevWorld dw{};
  int32_t geometry_mode = MC_GEOMETRY_ROBUST;
  uint32_t max_yield = 1;
  // smallest last entry of a chi cdf that a fission can draw from (+inf
  // without fission): the direct bank path needs it above every threshold
  double chi_last_min = HUGE_VAL;
  // page-locked staging for the values a call reads back at its one
  // synchronisation: bank size, then the counters
  void* h_small = nullptr;
  uint64_t total_bins = 0;
  DevCounters* d_ctr = nullptr;
  unsigned long long* d_total = nullptr;  // bank size, right after the counters (one read-back)
  double* d_sum = nullptr;
  double* d_sq = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  std::vector<cudaEvent_t> ev_pool;  // per-cycle timing events of mc_keig_cycles
  // second stream: the dense-score commit overlaps the bank kernels there
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool side_pending = false;  // the main stream has not yet waited for ev_join
  double last_kernel_ms = 0;  // main transport kernel(s) of the last run_transport
  // Two dense per-history score arrays (scratch kEvPend, kEvPend2) used by
  // alternate scored runs, so that the commit of one run (side stream) can
  // overlap the next run's transport: a run waits only for the commit that
  // last read the array it is about to fill.  A commit zeroes what it reads.
  int pend_next = 0;
  bool pend_zero[2] = {false, false};  // known to be all zero (of pend_zero_bytes)
  size_t pend_zero_bytes[2] = {0, 0};
  cudaEvent_t ev_commit[2] = {nullptr, nullptr};
  bool commit_pending[2] = {false, false};
  uint64_t launches = 0;
  // scratch, grown on demand
  DevBuffer scratch[kScratchSlots];
  int last_schedule = MC_SCHEDULE_HISTORY;
  // autotuner: history-kernel variant (occupancy target) chosen by timing
  int variant = 0;
  bool tune_pending = false;
  double tune_ms[16] = {};
  // the tuner's other choices: schedule for MC_SCHEDULE_AUTO, block size
  // (0: the run's own), event-schedule collision-queue sort threshold (0:
  // never); and the caller's queue-sort request of the current run
  // (mc_run_opts.queue_sort_min)
  int tuned_schedule = MC_SCHEDULE_HISTORY;
  int tuned_block = 0;
  unsigned ev_sort_min = 0;
  unsigned sort_min_req = 0;
  int last_grid = 0, last_block = 0;
  // MLP surrogate of the thermal scattering sampler
  mcd::MlpNet mlp[2];            // beta, alpha networks
  mcd::MlpNet mlp_scratch;       // gradient checks
  mcd::MlpBatch mlp_batch;       // training batch buffers
  int mlp_batch_cap = 0;
  mcd::MlpBox mlp_box{};
  int32_t mlp_tsl = -1;          // library the networks were trained for
  // guide network of the guided (POD-exact) thermal sampler
  mcd::MlpNet guide;
  mcd::MlpBox guide_box{};
  int32_t guide_tsl = -1;
  std::vector<bool> tsl_fast_ok;  // per library: every partition's rank fits the FP32 POD form
  std::vector<void*> mlp_allocs;
  // k-eigenvalue state
  struct {
    bool active = false;
    uint64_t n = 0, seed = 1;
    uint32_t inactive = 0, act = 0, cycle = 0;
    int rng = 0, fast = 0, block = 256, schedule = 0, bank_path = 0;
    uint32_t max_events = 1000000;
    std::vector<double> k, ktl;
    std::vector<uint64_t> bank;
    double transport_ms = 0, kernel_ms = 0;
    uint64_t events = 0, lost = 0, capped = 0, overflow = 0;
    uint64_t launches0 = 0;
    // the next cycle's source is still the resampling of the last bank
    // (scratch kBank, size in d_total): the next transport draws it as it
    // reads its sources; anything else that needs the source, or that
    // would overwrite the bank first, writes it out (materialize_source)
    bool src_pending = false;
    unsigned long long src_key = 0;
  } keig;
};

namespace {

// compaction that never writes past the caller's capacity
__global__ void k_compact_capped(const Site* slots, const uint32_t* count, const unsigned long long* offsets,
                                 unsigned long long n, uint32_t max_yield, Site* out, unsigned long long cap) {
  const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t c = count[i];
  const unsigned long long o = offsets[i];
  for (uint32_t k = 0; k < c; k++)
    if (o + k < cap) out[o + k] = slots[i * max_yield + k];
}

// the compacted bank, min(*total, cap) sites, into page-locked host memory:
// coalesced 16-byte stores (the bank size stays on the device, so the copy
// needs no host round trip first)
static_assert(sizeof(Site) % sizeof(uint4) == 0, "sites are copied as 16-byte words");
__global__ void k_copy_bank_out(const uint4* bank, const unsigned long long* total, unsigned long long cap,
                                uint4* out) {
  const unsigned long long m = *total < cap ? *total : cap;
  const unsigned long long words = m * (sizeof(Site) / sizeof(uint4));
  for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < words;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
    out[i] = __ldcs(bank + i);
}



int fail(mc_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CUDA_TRY(ctx, expr)                                                               \
  do {                                                                                     \
    cudaError_t e_ = (expr);                                                               \
    if (e_ != cudaSuccess) return fail((ctx), MC_ERR_DEVICE, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int upload(mc_ctx* c, const std::vector<T>& v, const T** out) {
  const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(c, MC_ERR_OOM, "cudaMalloc failed for world tables");
  c->world_allocs.push_back(p);
  if (!v.empty()) CUDA_TRY(c, cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  *out = static_cast<const T*>(p);
  return MC_OK;
}

void* scratch(mc_ctx* c, int slot, size_t bytes) {
  DevBuffer& b = c->scratch[slot];
  if (b.bytes >= bytes && b.p) return b.p;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (cudaMalloc(&b.p, std::max<size_t>(bytes, 256)) != cudaSuccess) {
    b.p = nullptr;
    return nullptr;
  }
  b.bytes = std::max<size_t>(bytes, 256);
  return b.p;
}

void free_world(mc_ctx* c) {
  for (void* p : c->world_allocs) cudaFree(p);
  c->world_allocs.clear();
  c->loaded = false;
  c->mlp_tsl = -1;  // the surrogate belongs to the problem's library
}

// POD partitions of a thermal scattering library: concatenated tables with
// per-partition offsets, plus FP32 copies for the fast form (S * CDF modes,
// and the grid-temperature modes)
int build_pod(mc_ctx* c, const mc::PODPartitionSet& P, mcd::DevPOD& d) {
  const size_t np = P.F.size();
  d.n_parts = static_cast<int32_t>(np);
  d.n_grid = static_cast<int32_t>(P.concat.size());
  std::vector<uint32_t> ends, F_off, cdf_off, S_off, T_off, g_off;
  std::vector<int32_t> nF, rank, nT;
  std::vector<double> F, cdf, S, T, g;
  std::vector<float> cs, gf;
  for (size_t p = 0; p < np; p++) {
    const size_t r = P.S[p].size();
    if (r == 0 || r > 1024) return fail(c, MC_ERR_INPUT, "thermal scattering partition rank out of range");
    ends.push_back(static_cast<uint32_t>(P.ends[p]));
    nF.push_back(static_cast<int32_t>(P.F[p].size()));
    rank.push_back(static_cast<int32_t>(r));
    nT.push_back(static_cast<int32_t>(P.T[p].size()));
    F_off.push_back(static_cast<uint32_t>(F.size()));
    F.insert(F.end(), P.F[p].begin(), P.F[p].end());
    cdf_off.push_back(static_cast<uint32_t>(cdf.size()));
    for (size_t i = 0; i < P.F[p].size(); i++) {
      for (size_t o = 0; o < r; o++) {
        const double v = P.cdf_modes[p][i * r + o];
        cdf.push_back(v);
        cs.push_back(static_cast<float>(P.S[p][o] * v));
      }
    }
    S_off.push_back(static_cast<uint32_t>(S.size()));
    S.insert(S.end(), P.S[p].begin(), P.S[p].end());
    T_off.push_back(static_cast<uint32_t>(T.size()));
    T.insert(T.end(), P.T[p].begin(), P.T[p].end());
    g_off.push_back(static_cast<uint32_t>(g.size()));
    for (double v : P.g_t_modes[p]) {
      g.push_back(v);
      gf.push_back(static_cast<float>(v));
    }
  }
  int rc;
  if ((rc = upload(c, P.concat, &d.grid)) != MC_OK) return rc;
  if ((rc = upload(c, ends, &d.ends)) != MC_OK) return rc;
  if ((rc = upload(c, nF, &d.nF)) != MC_OK) return rc;
  if ((rc = upload(c, rank, &d.rank)) != MC_OK) return rc;
  if ((rc = upload(c, nT, &d.nT)) != MC_OK) return rc;
  if ((rc = upload(c, F_off, &d.F_off)) != MC_OK) return rc;
  if ((rc = upload(c, F, &d.F)) != MC_OK) return rc;
  if ((rc = upload(c, cdf_off, &d.cdf_off)) != MC_OK) return rc;
  if ((rc = upload(c, cdf, &d.cdf)) != MC_OK) return rc;
  if ((rc = upload(c, cs, &d.cs)) != MC_OK) return rc;
  if ((rc = upload(c, S_off, &d.S_off)) != MC_OK) return rc;
  if ((rc = upload(c, S, &d.S)) != MC_OK) return rc;
  if ((rc = upload(c, T_off, &d.T_off)) != MC_OK) return rc;
  if ((rc = upload(c, T, &d.T)) != MC_OK) return rc;
  if ((rc = upload(c, g_off, &d.g_off)) != MC_OK) return rc;
  if ((rc = upload(c, g, &d.g)) != MC_OK) return rc;
  if ((rc = upload(c, gf, &d.gf)) != MC_OK) return rc;
  // monotone flags of the FP32 form: at each tabulated temperature the
  // reconstruction x_F = sum_o cs[F][o] gf[g][T][o] must rise from F to F + 1
  // by more than four times the bound on the FP32 dot products' rounding
  // (r * 2^-24 * sum_o |cs gf| for each); a convex combination of two
  // such columns (the sampler's temperature interpolation) then rises too
  // (bit 0); the same for the exact form, from the FP64 tables with the
  // FP64 rounding bound (bit 1)
  std::vector<uint8_t> mono(P.concat.size(), 0);
  for (size_t p = 0; p < np; p++) {
    const size_t r = P.S[p].size(), nFp = P.F[p].size(), nTp = P.T[p].size();
    const size_t first = p == 0 ? 0 : P.ends[p - 1];
    const float* csp = cs.data() + cdf_off[p];
    const float* gfp = gf.data() + g_off[p];
    const double* cdp = cdf.data() + cdf_off[p];
    const double* Sp = S.data() + S_off[p];
    const double* gdp = g.data() + g_off[p];
    for (size_t gi = 0; first + gi < P.ends[p]; gi++) {
      bool ok32 = true, ok64 = true;
      for (size_t t = 0; t < nTp && (ok32 || ok64); t++) {
        const float* v = gfp + (gi * nTp + t) * r;
        const double* vd = gdp + (gi * nTp + t) * r;
        double prev = 0, prev_err = 0, prevd = 0, prevd_err = 0;
        for (size_t f = 0; f < nFp; f++) {
          double x = 0, a = 0, xd = 0, ad = 0;
          for (size_t o = 0; o < r; o++) {
            const double term = static_cast<double>(csp[f * r + o]) * v[o];
            x += term;
            a += std::fabs(term);
            const double td = Sp[o] * cdp[f * r + o] * vd[o];
            xd += td;
            ad += std::fabs(td);
          }
          const double err = static_cast<double>(r) * 0x1p-24 * a;
          const double errd = static_cast<double>(r) * 0x1p-52 * ad;
          if (f > 0 && !(x - prev > 4.0 * (err + prev_err))) ok32 = false;
          if (f > 0 && !(xd - prevd > 4.0 * (errd + prevd_err))) ok64 = false;
          prev = x;
          prev_err = err;
          prevd = xd;
          prevd_err = errd;
        }
      }
      mono[first + gi] = static_cast<uint8_t>((ok32 ? 1 : 0) | (ok64 ? 2 : 0));
    }
  }
  if ((rc = upload(c, mono, &d.mono)) != MC_OK) return rc;
  return MC_OK;
}

// thermal scattering libraries (src/ThermalScattering.hpp)
int build_tsl(mc_ctx* c) {
  const mc::Model& m = c->model;
  std::vector<mcd::DevTSL> libs;
  c->tsl_fast_ok.clear();
  for (const mc::TSLData& t : m.tsl) {
    mcd::DevTSL d{};
    d.beta_cutoff = t.beta_cutoff;
    d.alpha_cutoff = t.alpha_cutoff;
    d.awr = t.awr;
    d.cutoff_energy = t.cutoff_energy();
    d.xs_nE = static_cast<int32_t>(t.xs_E.size());
    d.xs_nT = static_cast<int32_t>(t.xs_T.size());
    d.xs_rank = static_cast<int32_t>(t.xs_rank);
    d.maj_n = static_cast<int32_t>(t.majorant.x.size());
    if (d.xs_nE == 0 || d.xs_nT == 0 || d.maj_n == 0 || t.beta.F.empty() || t.alpha.F.empty())
      return fail(c, MC_ERR_INPUT, "thermal scattering library with empty tables");
    int rc;
    if ((rc = upload(c, t.xs_E, &d.xs_E)) != MC_OK) return rc;
    if ((rc = upload(c, t.xs_T, &d.xs_T)) != MC_OK) return rc;
    if ((rc = upload(c, t.xs_E_modes, &d.xs_Em)) != MC_OK) return rc;
    if ((rc = upload(c, t.xs_T_modes, &d.xs_Tm)) != MC_OK) return rc;
    if ((rc = upload(c, t.xs_S, &d.xs_S)) != MC_OK) return rc;
    {
      // FP32 forms of the total's modes for fast-mode transport
      std::vector<float> ems(t.xs_E_modes.size()), tm(t.xs_T_modes.size());
      const size_t r = t.xs_rank;
      for (size_t i = 0; i < ems.size(); i++) ems[i] = static_cast<float>(t.xs_S[i % r] * t.xs_E_modes[i]);
      for (size_t i = 0; i < tm.size(); i++) tm[i] = static_cast<float>(t.xs_T_modes[i]);
      if ((rc = upload(c, ems, &d.xs_EmS_f)) != MC_OK) return rc;
      if ((rc = upload(c, tm, &d.xs_Tm_f)) != MC_OK) return rc;
    }
    if ((rc = upload(c, t.majorant.x, &d.maj_x)) != MC_OK) return rc;
    if ((rc = upload(c, t.majorant.y, &d.maj_y)) != MC_OK) return rc;
    if ((rc = build_pod(c, t.beta, d.beta)) != MC_OK) return rc;
    if ((rc = build_pod(c, t.alpha, d.alpha)) != MC_OK) return rc;
    bool fits = true;
    for (const auto& S : t.beta.S) fits &= S.size() <= static_cast<size_t>(mcd::kFastPodRank);
    for (const auto& S : t.alpha.S) fits &= S.size() <= static_cast<size_t>(mcd::kFastPodRank);
    d.fast_ok = fits ? 1 : 0;
    c->tsl_fast_ok.push_back(fits);
    libs.push_back(d);
  }
  c->dw.n_tsl = static_cast<int32_t>(libs.size());
  return upload(c, libs, &c->dw.tsl);
}

// Builds the flat device tables from the model (see mc_device.cuh for the
// layout).  Running sums are formed in the reference's summation order so
// that a table lookup equals the on-the-fly sum bit-for-bit.
int build_world(mc_ctx* c) {
  const mc::Model& m = c->model;
  DevWorld& w = c->dw;
  w = DevWorld{};
  w.n_surfaces = static_cast<int32_t>(m.surfaces.size());
  w.n_cells = static_cast<int32_t>(m.cells.size());
  w.n_materials = static_cast<int32_t>(m.materials.size());
  w.n_nuclides = static_cast<int32_t>(m.nuclides.size());
  w.n_types = 2;
  w.energy_mode = m.energy_mode;
  w.tracking = m.tracking;
  w.quirks = c->geometry_mode;
  w.G = static_cast<int32_t>(m.energy_mode == mc::kMultigroup ? m.groups : 0);

  std::vector<int32_t> surf_kind, surf_refl;
  std::vector<double> surf_p;
  for (const auto& s : m.surfaces) {
    surf_kind.push_back(s.kind);
    surf_refl.push_back(s.reflective);
    for (double v : s.p) surf_p.push_back(v);
  }
  std::vector<int32_t> cell_begin{0}, cell_surf, cell_mat, cell_field;
  std::vector<uint8_t> cell_within;
  for (const auto& cl : m.cells) {
    for (size_t k = 0; k < cl.surfaces.size(); k++) {
      cell_surf.push_back(cl.surfaces[k]);
      cell_within.push_back(cl.within[k]);
    }
    cell_begin.push_back(static_cast<int32_t>(cell_surf.size()));
    cell_mat.push_back(cl.material);
    cell_field.push_back(cl.temperature);
  }
  std::vector<double> field;
  for (const auto& f : m.fields) {
    const double v[8] = {static_cast<double>(f.linear), f.c, f.g[0], f.g[1], f.g[2], f.b, f.upper, f.lower};
    field.insert(field.end(), v, v + 8);
  }
  std::vector<double> mat_density, mat_afrac;
  std::vector<int32_t> mat_begin{0}, mat_nuc;
  int32_t max_nuc = 1;
  for (const auto& mt : m.materials) {
    mat_density.push_back(mt.number_density);
    for (size_t k = 0; k < mt.nuclides.size(); k++) {
      mat_nuc.push_back(mt.nuclides[k]);
      mat_afrac.push_back(mt.afrac[k]);
    }
    mat_begin.push_back(static_cast<int32_t>(mat_nuc.size()));
    max_nuc = std::max<int32_t>(max_nuc, static_cast<int32_t>(mt.nuclides.size()));
  }
  w.max_mat_nuc = max_nuc;

  int rc;
#define UP(vec, field_)                                  \
  if ((rc = upload(c, vec, &w.field_)) != MC_OK) return rc;
  UP(surf_kind, surf_kind)
  UP(surf_refl, surf_refl)
  UP(surf_p, surf_p)
  UP(cell_begin, cell_begin)
  UP(cell_surf, cell_surf)
  UP(cell_within, cell_within)
  UP(cell_mat, cell_mat)
  UP(cell_field, cell_field)
  UP(field, field)
  UP(mat_density, mat_density)
  UP(mat_begin, mat_begin)
  UP(mat_nuc, mat_nuc)
  UP(mat_afrac, mat_afrac)

  c->max_yield = 1;
  c->chi_last_min = HUGE_VAL;
  if (m.energy_mode == mc::kMultigroup) {
    const size_t G = m.groups, N = m.nuclides.size(), M = m.materials.size(), T = 2;
    std::vector<double> total(T * N * G, 0), rx(T * N * G * 3, 0), scat(T * N * G * G, 0), nubar(T * N * G, 0),
        chi(T * N * G * G, 0), nusigf(T * N * G, 0);
    double max_nubar = 0;
    for (size_t t = 0; t < T; t++) {
      for (size_t n = 0; n < N; n++) {
        const auto& nuc = m.nuclides[n];
        if (!nuc.present[t]) continue;
        const mc::MGData& d = nuc.mg[t];
        for (size_t g = 0; g < G; g++) {
          const size_t i = (t * N + n) * G + g;
          total[i] = d.total[g];
          double acc = 0;
          if (d.has_capture) acc = acc + d.capture[g];
          rx[i * 3 + 0] = acc;
          if (d.has_scatter) acc = acc + d.scatter[g];
          rx[i * 3 + 1] = acc;
          if (d.has_fission) acc = acc + d.fission[g];
          rx[i * 3 + 2] = acc;
          if (d.has_scatter) {
            double a = 0;
            for (size_t go = 0; go < G; go++) {
              a = a + d.scatter_prob[g * G + go];
              scat[i * G + go] = a;
            }
          }
          if (d.has_fission) {
            nubar[i] = d.nubar[g];
            nusigf[i] = d.nubar[g] * d.fission[g];
            max_nubar = std::max(max_nubar, d.nubar[g]);
            double a = 0;
            for (size_t go = 0; go < G; go++) {
              a = a + d.chi[g * G + go];
              chi[i * G + go] = a;
            }
            if (d.nubar[g] > 0) c->chi_last_min = std::min(c->chi_last_min, a);
          }
        }
      }
    }
    c->max_yield = static_cast<uint32_t>(std::floor(max_nubar)) + 1;
    std::vector<double> mtot(T * M * G, 0), mcdf(T * M * G * max_nuc, 0), mnsf(T * M * G, 0), msig(T * M * G, 0);
    for (size_t t = 0; t < T; t++) {
      for (size_t mi = 0; mi < M; mi++) {
        const auto& mt = m.materials[mi];
        for (size_t g = 0; g < G; g++) {
          // Material::GetMicroscopicTotal: accumulate afrac * sigma_t
          double acc = 0, nsf = 0;
          for (size_t k = 0; k < mt.nuclides.size(); k++) {
            const size_t i = (t * N + mt.nuclides[k]) * G + g;
            acc = acc + mt.afrac[k] * total[i];
            mcdf[((t * M + mi) * G + g) * max_nuc + k] = acc;
            nsf = nsf + mt.afrac[k] * nusigf[i];
          }
          mtot[(t * M + mi) * G + g] = acc;
          // SurfaceTracking: number_density * GetCollisionProbabilityDensity
          msig[(t * M + mi) * G + g] = mt.number_density * acc;
          mnsf[(t * M + mi) * G + g] = mt.number_density * nsf;
        }
      }
    }
    UP(msig, mat_mg_sigma)
    UP(total, mg_total)
    UP(rx, mg_rx_cdf)
    UP(scat, mg_scat_cdf)
    UP(nubar, mg_nubar)
    UP(chi, mg_chi_cdf)
    UP(nusigf, mg_nusigf)
    UP(mtot, mat_mg_total)
    UP(mcdf, mat_mg_nuc_cdf)
    UP(mnsf, mat_mg_nusigf)
    // FP32 copies (round to nearest) for the fast form
    auto f32 = [](const std::vector<double>& v) {
      std::vector<float> o(v.size());
      for (size_t i = 0; i < v.size(); i++) o[i] = static_cast<float>(v[i]);
      return o;
    };
    const std::vector<float> msig_f = f32(msig), mtot_f = f32(mtot), mcdf_f = f32(mcdf), total_f = f32(total),
                             rx_f = f32(rx), scat_f = f32(scat), nubar_f = f32(nubar);
    UP(msig_f, mat_mg_sigma_f)
    UP(mtot_f, mat_mg_total_f)
    UP(mcdf_f, mat_mg_nuc_cdf_f)
    UP(total_f, mg_total_f)
    UP(rx_f, mg_rx_cdf_f)
    UP(scat_f, mg_scat_cdf_f)
    UP(nubar_f, mg_nubar_f)
  }
  else {
    for (const auto& nuc : m.nuclides) {
      for (int t = 0; t < 2; t++) {
        if (!nuc.present[t]) continue;
        for (const auto& r : nuc.ce[t].reactions) {
          // the reference dereferences the empty optional
          // (src/ContinuousReaction.cpp:257-258)
          if (r.kind == mc::kFission && !r.has_nubar) return fail(c, MC_ERR_INPUT, "nuclide " + nuc.name + ": fission without nubar");
        }
      }
    }
    mc::CETables ct;
    try {
      ct = mc::build_ce_tables(m);
    }
    catch (const std::exception& e) {
      return fail(c, MC_ERR_INPUT, e.what());
    }
    c->max_yield = static_cast<uint32_t>(std::floor(ct.max_nubar)) + 1;
    c->ce_fast_reason = ct.fast_reason;
    if ((rc = build_tsl(c)) != MC_OK) return rc;
    mcd::DevCE& ce = w.ce;
    ce.nu = static_cast<int32_t>(ct.union_e.size());
    ce.n_buckets = ct.n_buckets;
    ce.shift = ct.shift;
    ce.fast_ok = ct.fast_ok ? 1 : 0;
    ce.kmax = ct.kmax;
    ce.key0 = ct.key0;
    std::vector<unsigned long long> ukey(ct.union_key.begin(), ct.union_key.end());
    if ((rc = upload(c, ukey, &ce.ukey)) != MC_OK) return rc;
    if ((rc = upload(c, ct.union_e, &ce.ue)) != MC_OK) return rc;
    if ((rc = upload(c, ct.bucket, &ce.bucket)) != MC_OK) return rc;
    if ((rc = upload(c, ct.tab_off, &ce.tab_off)) != MC_OK) return rc;
    if ((rc = upload(c, ct.tab_grid, &ce.tab_grid)) != MC_OK) return rc;
    if ((rc = upload(c, ct.tab_x, &ce.tab_x)) != MC_OK) return rc;
    if ((rc = upload(c, ct.tab_y, &ce.tab_y)) != MC_OK) return rc;
    if ((rc = upload(c, ct.umap, &ce.umap)) != MC_OK) return rc;
    if ((rc = upload(c, ct.nuc, &ce.nuc)) != MC_OK) return rc;
    if (ct.fast_ok) {
      if ((rc = upload(c, ct.union_inv, &ce.uinv)) != MC_OK) return rc;
      if ((rc = upload(c, ct.mat_ncdf, &ce.mat_ncdf)) != MC_OK) return rc;
      if ((rc = upload(c, ct.nuc_nubar, &ce.nuc_nubar)) != MC_OK) return rc;
      const float* fp = nullptr;
      if ((rc = upload(c, ct.mat_flight, &fp)) != MC_OK) return rc;
      ce.mat_flight = reinterpret_cast<const float2*>(fp);
      if ((rc = upload(c, ct.nuc_rx, &fp)) != MC_OK) return rc;
      ce.nuc_rx = reinterpret_cast<const float4*>(fp);
    }
  }

  // estimators
  std::vector<int32_t> est_kind, est_target, est_has_cos, est_bin_kind, est_nsens, est_sens;
  std::vector<uint64_t> est_offset, est_bound_off, est_size;
  std::vector<double> est_cos_dir, est_bin_par, est_bounds;
  uint64_t off = 0;
  for (const auto& e : m.estimators) {
    est_kind.push_back(e.kind);
    est_target.push_back(e.kind == mc::kCurrent ? e.surface : e.cell);
    est_offset.push_back(off);
    off += e.span();  // the estimator's bins, then each sensitivity's
    est_size.push_back(e.size());
    est_nsens.push_back(static_cast<int32_t>(e.sensitivities.size()));
    for (int k = 0; k < mcd::kMaxSens; k++)
      est_sens.push_back(k < static_cast<int>(e.sensitivities.size()) ? e.sensitivities[static_cast<size_t>(k)] : -1);
    est_has_cos.push_back(e.has_cosine ? 1 : 0);
    for (double v : e.cosine_dir) est_cos_dir.push_back(v);
    for (const mc::Bins1D* b : {&e.cosine, &e.energy}) {
      est_bin_kind.push_back(b->kind);
      const bool lin = b->kind == mc::kLinspace;
      const double par[6] = {static_cast<double>(b->n_bins), lin ? b->lower : b->log_lower,
                             lin ? b->upper : b->log_upper, lin ? b->width : b->log_width, b->base,
                             static_cast<double>(b->boundaries.size())};
      est_bin_par.insert(est_bin_par.end(), par, par + 6);
      est_bound_off.push_back(est_bounds.size());
      est_bounds.insert(est_bounds.end(), b->boundaries.begin(), b->boundaries.end());
    }
  }
  c->total_bins = off;
  w.n_est = static_cast<int32_t>(m.estimators.size());
  // multigroup: energy bin of each group number, by the reference formulas
  std::vector<int32_t> est_ebin_mg;
  std::vector<uint64_t> est_esize;
  for (const auto& e : m.estimators) {
    est_esize.push_back(e.energy.size());
    for (uint64_t g = 1; g <= std::max<uint64_t>(1, m.groups); g++)
      est_ebin_mg.push_back(static_cast<int32_t>(e.energy.index(static_cast<double>(g))));
  }
  UP(est_ebin_mg, est_ebin_mg)
  UP(est_esize, est_esize)
  // plane keys and box cells (exact fast paths, mc_device.cuh)
  std::vector<long long> surf_key;
  for (const auto& s : m.surfaces)
    surf_key.push_back(s.kind == mc::kPlaneX || s.kind == mc::kPlaneY || s.kind == mc::kPlaneZ ? mcd::dkey(s.p[0]) : 0);
  UP(surf_key, surf_key)
  std::vector<int32_t> cell_box;
  std::vector<mcd::BoxCell> boxes;
  for (const auto& cl : m.cells) {
    mcd::BoxCell bx{};
    bool ok = cl.surfaces.size() == 6;
    int seen[6] = {0, 0, 0, 0, 0, 0};
    for (size_t k = 0; ok && k < cl.surfaces.size(); k++) {
      const mc::Surface& s = m.surfaces[cl.surfaces[k]];
      const int axis = s.kind == mc::kPlaneX ? 0 : s.kind == mc::kPlaneY ? 1 : s.kind == mc::kPlaneZ ? 2 : -1;
      if (axis < 0) {
        ok = false;
        break;
      }
      // sense +1 (within = 0): the cell is above the plane -> low plane
      const int j = 2 * axis + (cl.within[k] ? 1 : 0);
      if (seen[j]++) ok = false;
      bx.c[j] = s.p[0];
      bx.key[j] = mcd::dkey(s.p[0]);
      bx.s[j] = cl.surfaces[k];
      bx.order[j] = static_cast<int32_t>(k);
    }
    for (int a = 0; ok && a < 3; a++) ok = bx.c[2 * a] < bx.c[2 * a + 1];
    if (ok) {
      cell_box.push_back(static_cast<int32_t>(boxes.size()));
      boxes.push_back(bx);
    }
    else {
      cell_box.push_back(-1);
    }
  }
  UP(cell_box, cell_box)
  {
    const mcd::BoxCell* dp = nullptr;
    if ((rc = upload(c, boxes, &dp)) != MC_OK) return rc;
    w.boxes = dp;
  }
  UP(est_kind, est_kind)
  UP(est_target, est_target)
  UP(est_offset, est_offset)
  UP(est_has_cos, est_has_cos)
  UP(est_cos_dir, est_cos_dir)
  UP(est_bin_kind, est_bin_kind)
  UP(est_bin_par, est_bin_par)
  UP(est_bound_off, est_bound_off)
  UP(est_bounds, est_bounds)
  UP(est_size, est_size)
  UP(est_nsens, est_nsens)
  UP(est_sens, est_sens)
  // perturbations: per material, the perturbations whose nuclide it holds
  // (TotalCrossSectionPerturbation::Stream, src/Perturbation.cpp:68-78)
  bool any_sens = false;
  for (const auto& e : m.estimators) any_sens = any_sens || !e.sensitivities.empty();
  w.n_pert = any_sens ? static_cast<int32_t>(m.perturbations.size()) : 0;  // nothing scores them otherwise
  std::vector<int32_t> mat_pert(std::max<size_t>(1, m.materials.size()), 0);
  for (size_t q = 0; q < m.perturbations.size(); q++)
    for (size_t i = 0; i < m.materials.size(); i++)
      for (int32_t n : m.materials[i].nuclides)
        if (n == m.perturbations[q].nuclide) mat_pert[i] |= 1 << q;
  UP(mat_pert, mat_pert)
#undef UP

  for (int i = 0; i < 3; i++) {
    w.src_pos[i] = m.source.position[i];
    w.src_dir[i] = m.source.dir[i];
  }
  w.src_dir_kind = m.source.direction;
  w.src_type = m.source.type;
  w.src_energy = m.energy_mode == mc::kMultigroup ? static_cast<double>(m.source.group) : m.source.energy;

  // run buffers
  void* p = nullptr;
  static_assert(sizeof(DevCounters) % 8 == 0, "the bank size follows the counters");
  if (cudaMalloc(&p, sizeof(DevCounters) + 64) != cudaSuccess) return fail(c, MC_ERR_OOM, "cudaMalloc counters");
  c->world_allocs.push_back(p);
  c->d_ctr = static_cast<DevCounters*>(p);
  c->d_total = reinterpret_cast<unsigned long long*>(c->d_ctr + 1);
  const size_t tb = std::max<uint64_t>(1, c->total_bins) * sizeof(double);
  if (cudaMalloc(&p, tb) != cudaSuccess) return fail(c, MC_ERR_OOM, "cudaMalloc tallies");
  c->world_allocs.push_back(p);
  c->d_sum = static_cast<double*>(p);
  if (cudaMalloc(&p, tb) != cudaSuccess) return fail(c, MC_ERR_OOM, "cudaMalloc tallies");
  c->world_allocs.push_back(p);
  c->d_sq = static_cast<double*>(p);
  CUDA_TRY(c, cudaMemsetAsync(c->d_sum, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_sq, 0, tb, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

bool check_ctx(mc_ctx* c, bool need_world = true) {
  if (!c) return false;
  if (need_world && !c->loaded) {
    c->err = "no problem loaded (call mc_load_xml first)";
    return false;
  }
  return true;
}

int pick_block(const mc_run_opts* o) {
  const int b = o && o->block_size > 0 ? o->block_size : 256;
  return std::min(256, std::max(32, (b / 32) * 32));
}

int grid_for(mc_ctx* c, int energy_mode, int rng, int block, bool keig, bool fast) {
  int per_sm = energy_mode == mc::kMultigroup
                   ? mcd::history_blocks_per_sm(energy_mode, rng, block, keig, fast, c->variant)
                   : mcd::history_blocks_per_sm_ce(c->dw, rng, block, keig, fast, c->variant);
  if (per_sm < 1) per_sm = 1;
  return per_sm * c->num_sms;
}

// one thread per history record for the fission-site kernels (most
// records hold no fission, so the latency of the others needs many threads)
int sites_grid(uint64_t n) { return static_cast<int>(std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, 1u << 20))); }

unsigned long long run_key(uint64_t seed, uint64_t cycle, uint64_t salt) {
  return mcd::splitmix64(seed * 0x9E3779B97F4A7C15ull + cycle * 0xD1B54A32D192ED03ull + salt);
}

// outcome of a run's counters as a status code
int counters_status(mc_ctx* c, const DevCounters& h) {
  if (h.lost) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "Point does not belong to any Cell. Please check that all space is either assigned a material "
                  "or void. (%llu particles lost; last at %.17g %.17g %.17g, cell %lld, history %llu)",
                  h.lost, h.lost_xyz[0], h.lost_xyz[1], h.lost_xyz[2], static_cast<long long>(h.pad[0]) - 1,
                  h.pad[1]);
    return fail(c, MC_ERR_LOST, buf);
  }
  if (h.overflow) return fail(c, MC_ERR_OVERFLOW, std::to_string(h.overflow) + " bank/stack/tally overflows");
  if (h.resample)
    return fail(c, MC_ERR_RESAMPLE, "Number of thermal scattering resamples exceeded limit: 10 (" +
                                         std::to_string(h.resample) + " times)");
  if (h.capped) return fail(c, MC_ERR_EVENT_CAP, std::to_string(h.capped) + " particles reached the event cap");
  return MC_OK;
}

// resolves MC_SCHEDULE_AUTO.  Measured on the 8-group two-zone problem the
// fused history schedule is faster than the event queues (the event kernels
// pay a launch and a state round trip per event), so AUTO picks it; the
// event schedule runs multigroup problems whose estimators fit the dense
// per-history scores, without perturbations, when asked for.
bool event_schedule_ok(const mc_ctx* c) {
  return c->model.energy_mode == mc::kMultigroup && c->total_bins <= mcd::kEvDenseBins &&
         c->model.perturbations.empty();
}

int resolve_schedule(mc_ctx* c, int requested) {
  const bool event_ok = event_schedule_ok(c);
  if (requested == MC_SCHEDULE_EVENT) return event_ok ? MC_SCHEDULE_EVENT : -1;
  if (requested == MC_SCHEDULE_AUTO && event_ok) return c->tuned_schedule;
  return MC_SCHEDULE_HISTORY;
}

// the collision-queue sort threshold of an event-schedule run (0: never)
unsigned event_sort_min(const mc_ctx* c) {
  if (c->sort_min_req == 0) return c->ev_sort_min;
  return c->sort_min_req == 0xFFFFFFFFu ? 0u : c->sort_min_req;
}

void count_launches(void* ctx, int n) { static_cast<mc_ctx*>(ctx)->launches += n; }

// event schedule: SoA store, queues, pending scores, fission records.
// Fixed-source secondaries take new store slots; when a chain needs more
// slots than the store holds the run is repeated with a larger store (every
// particle's stream is keyed by its own identity, not its slot, so the
// repeat draws the same numbers).
int run_event_once(mc_ctx* c, RunParams& rp, int rng, uint64_t cap);
int run_tq(mc_ctx* c, RunParams rp, int grid, int block);

int run_event(mc_ctx* c, RunParams& rp, int rng) {
  uint64_t cap = rp.keig ? rp.n : rp.n * 4 + 65536;
  for (int attempt = 0;; attempt++) {
    const int rc = run_event_once(c, rp, rng, cap);
    if (rc != MC_OK) return rc;
    if (rp.keig || attempt == 3) return MC_OK;
    unsigned long long overflow = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&overflow, &c->d_ctr->overflow, sizeof overflow, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (!overflow) return MC_OK;
    cap *= 4;
    CUDA_TRY(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), c->stream));
    if (rp.pend) CUDA_TRY(c, cudaMemsetAsync(rp.pend, 0, rp.n * rp.nb * sizeof(double), c->stream));
  }
}

int run_event_once(mc_ctx* c, RunParams& rp, int rng, uint64_t cap) {
  const uint64_t n = rp.n;
  mcd::EvParams ep{};
  ep.rp = rp;
  ep.capacity = static_cast<unsigned>(std::min<uint64_t>(cap, 0xffffffffull));
  if (cap >= 0x7fffffffull) return fail(c, MC_ERR_INPUT, "too many particles for the event schedule");
  // one allocation for the particle store: 6 f64 + E + 6 x u32 + u64 + u8
  const size_t bytes = cap * (8 * 7 + 4 * 6 + 8 + 1) + 256 * 16;
  char* base = static_cast<char*>(scratch(c, kEvState, bytes));
  auto* q = static_cast<int32_t*>(scratch(c, kEvQueues, cap * 4 * sizeof(int32_t)));
  auto* cnt = static_cast<unsigned*>(scratch(c, kEvCnt, 64 + 2 * mcd::kEvSortKeys * sizeof(unsigned)));
  if (!base || !q || !cnt) return fail(c, MC_ERR_OOM, "event-schedule buffers");
  size_t off = 0;
  auto take = [&](size_t each) {
    char* p = base + off;
    off += (cap * each + 255) / 256 * 256;
    return p;
  };
  ep.st.x = reinterpret_cast<double*>(take(8));
  ep.st.y = reinterpret_cast<double*>(take(8));
  ep.st.z = reinterpret_cast<double*>(take(8));
  ep.st.u = reinterpret_cast<double*>(take(8));
  ep.st.v = reinterpret_cast<double*>(take(8));
  ep.st.w = reinterpret_cast<double*>(take(8));
  ep.st.E = reinterpret_cast<double*>(take(8));
  ep.st.g = reinterpret_cast<int32_t*>(take(4));
  ep.st.cell = reinterpret_cast<int32_t*>(take(4));
  ep.st.skip = reinterpret_cast<int32_t*>(take(4));
  ep.st.nev = reinterpret_cast<uint32_t*>(take(4));
  ep.st.hist = reinterpret_cast<uint32_t*>(take(4));
  ep.st.rng = reinterpret_cast<uint32_t*>(take(4));
  ep.st.id = reinterpret_cast<unsigned long long*>(take(8));
  ep.st.tag = reinterpret_cast<uint8_t*>(take(1));
  ep.q_in = q;
  ep.q_out = q + cap;
  ep.q_coll = q + 2 * cap;
  ep.cnt = cnt;
  ep.q_sorted = q + 3 * cap;
  ep.sort_hist = cnt + 16;
  ep.sort_min = event_sort_min(c);
  const size_t keys = 2 * static_cast<size_t>(c->model.materials.size()) * static_cast<size_t>(c->model.groups);
  ep.sort_keys = ep.sort_min > 0 && keys <= static_cast<size_t>(mcd::kEvSortKeys) ? static_cast<int32_t>(keys) : 0;
  if (ep.sort_keys > 0) CUDA_TRY(c, cudaMemsetAsync(ep.sort_hist, 0, mcd::kEvSortKeys * sizeof(unsigned), c->stream));
  if (rp.hist_events) CUDA_TRY(c, cudaMemsetAsync(rp.hist_events, 0, n * 4, c->stream));
  mcd::EvLaunch L{};
  L.grid = c->num_sms * 8;
  L.check_every = 8;
  L.max_iterations = ((rp.max_events + 64) / L.check_every + 1) * L.check_every;
  const cudaError_t e = mcd::launch_event_mg(c->dw, ep, L, rng, c->stream, count_launches, c);
  if (e != cudaSuccess) return fail(c, MC_ERR_DEVICE, std::string("event transport: ") + cudaGetErrorString(e));
  return MC_OK;
}

// one transport launch over rp.n particles; returns elapsed device ms
// the main stream waits for the work on the side stream
int join_side(mc_ctx* c) {
  if (c->side_pending) {
    CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    c->side_pending = false;
    c->commit_pending[0] = c->commit_pending[1] = false;
  }
  return MC_OK;
}

// side_commit: the dense-score commit runs on the side stream, overlapping
// what the caller queues next on the main stream; join_side (or read_back)
// orders it before anything that reads the tallies or the score array.
int run_transport(mc_ctx* c, RunParams& rp, int rng, int block, double* ms, int schedule = MC_SCHEDULE_AUTO,
                  bool side_commit = false) {
  // dense per-history scores when the estimators are small (committed by
  // a separate kernel: per-history sums kept in shared memory instead were
  // measured slower, their commits contend on shared FP64 atomics)
  const bool dense = rp.score && c->total_bins > 0 && c->total_bins <= static_cast<uint64_t>(mcd::kDenseBins);
  const int pb = c->pend_next;
  if (dense && side_commit) {
    // only the commit that last read this run's score array must be done;
    // the other array's commit may still run beside this transport
    if (c->commit_pending[pb]) {
      CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_commit[pb], 0));
      c->commit_pending[pb] = false;
    }
  }
  else if (join_side(c) != MC_OK) {
    return MC_ERR_DEVICE;
  }
  CUDA_TRY(c, cudaMemsetAsync(c->d_ctr, 0, sizeof(DevCounters), c->stream));
  rp.ctr = c->d_ctr;
  rp.tally_sum = c->d_sum;
  rp.tally_sq = c->d_sq;
  rp.total_bins = c->total_bins;
  const bool keig = rp.keig != 0;
  const int sched = resolve_schedule(c, schedule);
  if (sched < 0) return fail(c, MC_ERR_INPUT, "the event schedule supports multigroup problems with at most 64 tally bins");
  c->last_schedule = sched;
  // fission records for k-eigenvalue cycles
  const uint64_t n = rp.n;
  rp.nb = dense ? static_cast<int32_t>(c->total_bins) : 0;
  const int pslot = pb == 0 ? kEvPend : kEvPend2;
  if (dense) c->pend_next = 1 - pb;
  rp.pend = rp.nb ? static_cast<double*>(scratch(c, pslot, n * rp.nb * sizeof(double))) : nullptr;
  rp.fis = keig ? static_cast<mcd::FissionRec*>(scratch(c, kEvFis, n * sizeof(mcd::FissionRec))) : nullptr;
  if ((rp.nb && !rp.pend) || (keig && !rp.fis)) return fail(c, MC_ERR_OOM, "score/fission buffers");
  CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
  // the commit kernel zeroes what it reads, so a dense array only needs a
  // memset when it is new or a previous run did not reach its commit
  const size_t pend_bytes = n * rp.nb * sizeof(double);
  if (rp.pend && (!c->pend_zero[pb] || c->pend_zero_bytes[pb] < pend_bytes)) {
    const size_t all = c->scratch[pslot].bytes;
    CUDA_TRY(c, cudaMemsetAsync(rp.pend, 0, all, c->stream));
    c->pend_zero_bytes[pb] = all;
  }
  if (rp.pend) c->pend_zero[pb] = false;  // dirty until the commit has run
  CUDA_TRY(c, cudaEventRecord(c->evk0, c->stream));
  if (sched == MC_SCHEDULE_EVENT) {
    const int rc = run_event(c, rp, rng);
    if (rc != MC_OK) return rc;
  }
  else {
    const int grid = grid_for(c, c->model.energy_mode, rng, block, keig, rp.fast != 0);
    c->last_grid = grid;
    c->last_block = block;
    if (rp.tq) {
      const int rc = run_tq(c, rp, grid, block);
      if (rc != MC_OK) return rc;
    }
    else {
      cudaError_t e;
      if (c->model.energy_mode == mc::kMultigroup)
        e = mcd::launch_history_mg(c->dw, rp, rng, grid, block, c->stream, c->variant);
      else e = mcd::launch_history_ce(c->dw, rp, rng, grid, block, c->stream, c->variant);
      if (e != cudaSuccess) return fail(c, MC_ERR_DEVICE, std::string("transport launch: ") + cudaGetErrorString(e));
      c->launches++;
    }
  }
  CUDA_TRY(c, cudaEventRecord(c->evk1, c->stream));
  if (keig && !rp.direct_sites) {  // direct: the sites are sampled into the bank later
    if (c->model.energy_mode == mc::kMultigroup)
      CUDA_TRY(c, mcd::launch_fission_sites_mg(c->dw, rp, rng, sites_grid(rp.n), c->stream));
    else CUDA_TRY(c, mcd::launch_fission_sites_ce(rp, rng, sites_grid(rp.n), c->stream));
    c->launches++;
  }
  if (rp.nb) {
    cudaStream_t cs = c->stream;
    if (side_commit) {
      CUDA_TRY(c, cudaEventRecord(c->ev_fork, c->stream));
      CUDA_TRY(c, cudaStreamWaitEvent(c->side, c->ev_fork, 0));
      cs = c->side;
    }
    CUDA_TRY(c, mcd::launch_commit_dense(rp, c->num_sms * 8, cs));
    c->launches++;
    c->pend_zero[pb] = true;
    if (side_commit) {
      CUDA_TRY(c, cudaEventRecord(c->ev_commit[pb], c->side));
      c->commit_pending[pb] = true;
      CUDA_TRY(c, cudaEventRecord(c->ev_join, c->side));
      c->side_pending = true;
    }
  }
  CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
  if (ms) {
    CUDA_TRY(c, cudaEventSynchronize(c->ev1));
    float f = 0;
    CUDA_TRY(c, cudaEventElapsedTime(&f, c->ev0, c->ev1));
    *ms = f;
    CUDA_TRY(c, cudaEventElapsedTime(&f, c->evk0, c->evk1));
    c->last_kernel_ms = f;
  }
  return MC_OK;
}

// Fixed source with the thermal-scatter queue: the source launch parks
// particles at thermal scatters; each round samples the parked rows with
// the surrogate (one tensor-core launch) and resumes them (one history
// launch), which may park them again.  Counts stay on the device, so the
// rounds need no host synchronisation; the last resume samples inline.
int run_tq(mc_ctx* c, RunParams rp, int grid, int block) {
  const uint64_t n = rp.n;
  const int mode = rp.tq_mode;  // 1 quantile surrogate, 2 guided, 3 plain POD queue
  const bool exact_q = mode >= 2;
  auto* A = static_cast<mcd::ParkRec*>(scratch(c, kParkA, n * sizeof(mcd::ParkRec)));
  auto* B = static_cast<mcd::ParkRec*>(scratch(c, kParkB, n * sizeof(mcd::ParkRec)));
  auto* qin = exact_q ? nullptr : static_cast<float4*>(scratch(c, kTqIn, n * sizeof(float4)));
  auto* qout = exact_q ? nullptr : static_cast<float2*>(scratch(c, kTqOut, n * sizeof(float2)));
  auto* rows = exact_q ? static_cast<mcd::GuideRow*>(scratch(c, kTqRows, n * sizeof(mcd::GuideRow))) : nullptr;
  auto* res = exact_q ? static_cast<mcd::GuideOut*>(scratch(c, kTqRes, n * sizeof(mcd::GuideOut))) : nullptr;
  auto* cnt = static_cast<unsigned long long*>(scratch(c, kTqCnt, 2 * (mcd::kTqRounds + 1) * 8));
  if (!A || !B || !cnt || (exact_q ? !(rows && res) : !(qin && qout)))
    return fail(c, MC_ERR_OOM, "thermal queue buffers");
  unsigned long long* heads = cnt + mcd::kTqRounds + 1;
  CUDA_TRY(c, cudaMemsetAsync(cnt, 0, 2 * (mcd::kTqRounds + 1) * 8, c->stream));
  rp.tq = 1;
  rp.tq_tsl = mode == 1 ? c->mlp_tsl : (c->guide_tsl >= 0 ? c->guide_tsl : 0);
  // the POD-exact queue forms sample what the inline sampler would: its
  // FP32 form in fast mode when the library's ranks allow it, else FP64
  rp.tq_fast = rp.fast && c->tsl_fast_ok[static_cast<size_t>(rp.tq_tsl)] ? 1 : 0;
  rp.tq_rows = rows;
  rp.tq_res = res;
  rp.tq_box[0] = std::exp(c->mlp_box.logE0);
  rp.tq_box[1] = std::exp(c->mlp_box.logE1);
  rp.tq_box[2] = c->mlp_box.T0;
  rp.tq_box[3] = c->mlp_box.T1;
  rp.park_cap = n;
  rp.tq_in = qin;
  rp.tq_out = qout;
  rp.head = nullptr;
  rp.n_resume = nullptr;
  rp.park_in = nullptr;
  rp.park_out = A;
  rp.park_count = cnt;
  cudaError_t e = mcd::launch_history_ce_tq(c->dw, rp, grid, block, c->stream);
  if (e != cudaSuccess) return fail(c, MC_ERR_DEVICE, std::string("transport launch: ") + cudaGetErrorString(e));
  c->launches++;
  for (int r = 0; r < mcd::kTqRounds; r++) {
    mcd::ParkRec* in = r % 2 == 0 ? A : B;
    mcd::ParkRec* out = r % 2 == 0 ? B : A;
    if (mode == 2)
      e = mcd::launch_sample_tsl_guided_queue(c->dw.tsl + rp.tq_tsl, c->guide, c->guide_box, rp.tq_fast != 0, rows,
                                              cnt + r, n, rp.run_key, res, c->num_sms, c->stream);
    else if (mode == 3)
      e = mcd::launch_sample_tsl_pod_queue(c->dw.tsl + rp.tq_tsl, rp.tq_fast != 0, rows, cnt + r, n, rp.run_key,
                                           res, c->num_sms, c->stream);
    else
      e = mcd::launch_sample_tsl_mlp_queue(c->mlp[0], c->mlp[1], c->mlp_box, qin, cnt + r, n, qout, c->num_sms,
                                           c->stream);
    if (e != cudaSuccess) return fail(c, MC_ERR_DEVICE, std::string("thermal sampler launch: ") + cudaGetErrorString(e));
    rp.tq = r + 1 < mcd::kTqRounds ? 1 : 0;
    rp.head = heads + r;
    rp.n_resume = cnt + r;
    rp.park_in = in;
    rp.park_out = out;
    rp.park_count = cnt + r + 1;
    e = mcd::launch_history_ce_tq(c->dw, rp, grid, block, c->stream);
    if (e != cudaSuccess) return fail(c, MC_ERR_DEVICE, std::string("transport launch: ") + cudaGetErrorString(e));
    c->launches += 2;
  }
  return MC_OK;
}

// Fission sites go straight into the compacted bank (no per-history slots)
// when each record's site count is known before sampling and a CTA's sites
// fit its shared-memory stage.  Continuous energy: always (the sites take
// the incident energy).  Multigroup: Philox streams and every chi cdf a
// fission draws from ending above the largest uniform the stream draws
// (1 - 2^-24 in the FP32 form, 1 - 2^-52 in the FP64 form; a minstd uniform
// can round to 1).
// 1: direct, 0: slots, -1: MC_BANK_DIRECT asked for where it does not apply.
int bank_direct(const mc_ctx* c, int rng, bool fast, int path) {
  if (path == MC_BANK_SLOTS) return 0;
  const bool counts_known = c->model.energy_mode != mc::kMultigroup ||
                            (rng == MC_RNG_PHILOX && c->chi_last_min > (fast ? 1.0 - 0x1p-24 : 1.0 - 0x1p-52));
  const bool ok = counts_known && mcd::sites_out_fits(c->max_yield);
  if (path == MC_BANK_DIRECT) return ok ? 1 : -1;
  return ok ? 1 : 0;
}

// writes a pending resampled k-eigenvalue source into scratch kSrc
int materialize_source(mc_ctx* c) {
  auto& k = c->keig;
  if (!k.src_pending) return MC_OK;
  k.src_pending = false;
  CUDA_TRY(c, mcd::launch_resample(static_cast<const Site*>(c->scratch[kBank].p),
                                   c->d_total, k.n, k.src_key,
                                   static_cast<Site*>(c->scratch[kSrc].p), c->stream));
  c->launches++;
  return MC_OK;
}

// The cycle's fission sites as a compacted bank in history order.  Slot
// path: the slot kernel has run; a scan of its counts places each history's
// sites and a compaction copies them into the device bank.  Direct path:
// counts from the fission records, their scan, then the sites sampled
// straight into `dest` (16-byte aligned page-locked host memory, `cap`
// sites) or else into the device bank.  *bank_out is the device bank (null
// when the sites went to `dest`); the size stays on the device (d_total,
// after the counters) unless read_size, which reads it into *m_out.
int emit_bank(mc_ctx* c, const RunParams& rp, int rng, Site* dest, uint64_t cap, Site** bank_out, uint64_t* m_out,
              bool read_size = true) {
  // the bank about to be written may still hold a pending source
  if (materialize_source(c) != MC_OK) return MC_ERR_DEVICE;
  const uint64_t n = rp.n;
  auto* count = static_cast<uint32_t*>(c->scratch[kCount].p);
  auto* offsets = static_cast<unsigned long long*>(scratch(c, kOffsets, n * 8));
  auto* sums = static_cast<unsigned long long*>(scratch(c, kScanSums, ((n + 1023) / 1024 + 1) * 8));
  unsigned long long* total = c->d_total;
  Site* bank = dest ? nullptr : static_cast<Site*>(scratch(c, kBank, n * c->max_yield * sizeof(Site)));
  if (!offsets || !sums || !total || (!dest && !bank)) return fail(c, MC_ERR_OOM, "bank scratch allocation failed");
  if (rp.direct_sites) {
    RunParams q = rp;
    q.ctr = c->d_ctr;
    q.bank_count = count;
    CUDA_TRY(c, mcd::launch_direct_bank_scan(q, offsets, sums, total, c->stream));
    const uint64_t qcap = dest ? cap : n * c->max_yield;
    if (c->model.energy_mode == mc::kMultigroup)
      CUDA_TRY(c, mcd::launch_fission_sites_out_mg(c->dw, q, offsets, total, qcap, dest ? dest : bank, c->stream));
    else CUDA_TRY(c, mcd::launch_fission_sites_out_ce(q, rng, offsets, total, qcap, dest ? dest : bank, c->stream));
    c->launches += 4;
  }
  else {
    auto* slots = static_cast<Site*>(c->scratch[kSlots].p);
    CUDA_TRY(c, mcd::launch_bank_scan(count, n, offsets, sums, total, c->stream));
    CUDA_TRY(c, mcd::launch_bank_compact(slots, count, offsets, n, c->max_yield, bank, c->stream));
    c->launches += 4;
  }
  unsigned long long m = 0;
  if (read_size) {
    CUDA_TRY(c, cudaMemcpyAsync(&m, total, 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  }
  *bank_out = bank;
  *m_out = m;
  return MC_OK;
}

// bank size (when m) and counters, read back with one synchronisation
int read_back(mc_ctx* c, uint64_t* m, DevCounters* h) {
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  // the counters and the bank size that follows them, in one copy
  auto* hc = reinterpret_cast<DevCounters*>(static_cast<char*>(c->h_small) + 64);
  CUDA_TRY(c, cudaMemcpyAsync(hc, c->d_ctr, sizeof(DevCounters) + (m ? 8 : 0), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (m) *m = *reinterpret_cast<const unsigned long long*>(hc + 1);
  *h = *hc;
  return MC_OK;
}

}  // namespace

extern "C" {

int mc_version(void) { return 1; }

int mc_create(mc_ctx** out, int device) {
  if (!out) return MC_ERR_INPUT;
  *out = nullptr;
  auto* c = new (std::nothrow) mc_ctx();
  if (!c) return MC_ERR_OOM;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return MC_ERR_DEVICE;
  }
  c->own_stream = true;
  if (cudaMallocHost(&c->h_small, 512) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) {
    if (c->h_small) cudaFreeHost(c->h_small);
    cudaStreamDestroy(c->stream);
    delete c;
    return MC_ERR_OOM;
  }
  cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->ev_commit[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->ev_commit[1], cudaEventDisableTiming);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaEventCreate(&c->ev0);
  cudaEventCreate(&c->ev1);
  cudaEventCreate(&c->evk0);
  cudaEventCreate(&c->evk1);
  *out = c;
  return MC_OK;
}

void mc_destroy(mc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_world(c);
  for (auto& b : c->scratch)
    if (b.p) cudaFree(b.p);
  for (void* p : c->mlp_allocs) cudaFree(p);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->evk0) cudaEventDestroy(c->evk0);
  if (c->evk1) cudaEventDestroy(c->evk1);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  if (c->h_small) cudaFreeHost(c->h_small);
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  for (cudaEvent_t e : c->ev_commit)
    if (e) cudaEventDestroy(e);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int mc_last_error(const mc_ctx* c, char* buf, size_t n) {
  if (!c || !buf || n == 0) return MC_ERR_INPUT;
  std::strncpy(buf, c->err.c_str(), n - 1);
  buf[n - 1] = 0;
  return MC_OK;
}

int mc_set_stream(mc_ctx* c, void* s) {
  if (!c) return MC_ERR_INPUT;
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->own_stream = false;
  c->stream = static_cast<cudaStream_t>(s);
  return MC_OK;
}

int mc_load_xml(mc_ctx* c, const char* xml_text, const char* base_dir) {
  if (!c || !xml_text) return MC_ERR_INPUT;
  cudaSetDevice(c->device);
  free_world(c);
  try {
    c->model = mc::load_model(xml_text, base_dir ? base_dir : "");
  }
  catch (const std::exception& e) {
    return fail(c, MC_ERR_INPUT, e.what());
  }
  {
    const mc::Model& m = c->model;
    bool sens = false;
    for (const auto& e : m.estimators) {
      if (e.sensitivities.size() > static_cast<size_t>(mcd::kMaxSens))
        return fail(c, MC_ERR_INPUT, "more than 4 sensitivities on one estimator");
      sens = sens || !e.sensitivities.empty();
    }
    if (m.perturbations.size() > static_cast<size_t>(mcd::kMaxPert))
      return fail(c, MC_ERR_INPUT, "more than 4 perturbations");
    // the reference's k-eigenvalue workers never give particles their
    // indirect effects (only FixedSource calls Particle::SetPerturbations,
    // src/FixedSource.cpp:63-65), so a sensitivity there has nothing to score
    if (sens && m.problem == mc::kKEigenvalue)
      return fail(c, MC_ERR_INPUT, "sensitivities are scored in fixed-source problems only");
  }
  const int rc = build_world(c);
  if (rc != MC_OK) {
    free_world(c);
    return rc;
  }
  c->loaded = true;
  return MC_OK;
}

int mc_set_geometry_mode(mc_ctx* c, int32_t mode) {
  if (!c) return MC_ERR_INPUT;
  if (mode != MC_GEOMETRY_ROBUST && mode != MC_GEOMETRY_REFERENCE) return fail(c, MC_ERR_INPUT, "unknown geometry mode");
  c->geometry_mode = mode;
  c->dw.quirks = mode;
  return MC_OK;
}

int mc_problem_info_get(mc_ctx* c, mc_problem_info* out) {
  if (!check_ctx(c) || !out) return MC_ERR_STATE;
  const mc::Model& m = c->model;
  std::memset(out, 0, sizeof *out);
  out->problem = m.problem;
  out->energy_mode = m.energy_mode;
  out->tracking = m.tracking;
  out->n_cells = static_cast<int32_t>(m.cells.size());
  out->n_surfaces = static_cast<int32_t>(m.surfaces.size());
  out->n_materials = static_cast<int32_t>(m.materials.size());
  out->n_nuclides = static_cast<int32_t>(m.nuclides.size());
  out->groups = static_cast<int32_t>(m.groups);
  out->n_estimators = static_cast<int32_t>(m.estimators.size());
  out->n_tsl = static_cast<int32_t>(m.tsl.size());
  out->histories = m.histories;
  out->seed = m.seed;
  out->inactive = static_cast<uint32_t>(m.inactive);
  out->active = static_cast<uint32_t>(m.active);
  out->total_bins = c->total_bins;
  out->max_yield = c->max_yield;
  out->n_perturbations = static_cast<int32_t>(m.perturbations.size());
  return MC_OK;
}

int mc_estimator_info_get(mc_ctx* c, int32_t index, mc_estimator_info* out) {
  if (!check_ctx(c) || !out) return MC_ERR_STATE;
  if (index < 0 || index >= static_cast<int32_t>(c->model.estimators.size()))
    return fail(c, MC_ERR_INPUT, "estimator index out of range");
  std::memset(out, 0, sizeof *out);
  uint64_t off = 0;
  for (int32_t i = 0; i < index; i++) off += c->model.estimators[i].span();
  const auto& e = c->model.estimators[index];
  std::strncpy(out->name, e.name.c_str(), sizeof(out->name) - 1);
  out->kind = e.kind;
  out->target = e.kind == mc::kCurrent ? e.surface : e.cell;
  out->offset = off;
  out->n_bins = e.size();
  out->cosine_bins = e.cosine.size();
  out->energy_bins = e.energy.size();
  out->n_sensitivities = static_cast<int32_t>(e.sensitivities.size());
  for (size_t k = 0; k < e.sensitivities.size() && k < 4; k++) out->sensitivity[k] = e.sensitivities[k];
  return MC_OK;
}

int mc_object_name(mc_ctx* c, int32_t kind, int32_t index, char* buf, size_t n) {
  if (!check_ctx(c) || !buf || n == 0) return MC_ERR_STATE;
  const mc::Model& m = c->model;
  std::string s;
  try {
    if (kind == 0) s = m.cells.at(index).name;
    else if (kind == 1) s = m.surfaces.at(index).name;
    else if (kind == 2) s = m.materials.at(index).name;
    else if (kind == 3) s = m.nuclides.at(index).name;
    else if (kind == 4) s = m.perturbations.at(index).name;
    else return fail(c, MC_ERR_INPUT, "unknown object kind");
  }
  catch (const std::exception&) {
    return fail(c, MC_ERR_INPUT, "object index out of range");
  }
  std::strncpy(buf, s.c_str(), n - 1);
  buf[n - 1] = 0;
  return MC_OK;
}

int mc_run_fixed_source(mc_ctx* c, const mc_run_opts* o, mc_tally_out* out) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  cudaSetDevice(c->device);
  const uint64_t n = o && o->histories ? o->histories : c->model.histories;
  const uint64_t seed = o && o->seed ? o->seed : c->model.seed;
  const int rng = o ? o->rng : 0;
  if (rng != MC_RNG_PHILOX && rng != MC_RNG_MINSTD) return fail(c, MC_ERR_INPUT, "unknown rng mode");
  const int block = pick_block(o);
  if (o && o->variant > 0) c->variant = std::min(o->variant - 1, mcd::history_variants() - 1);
  c->sort_min_req = o ? o->queue_sort_min : 0;
  RunParams rp{};
  rp.n = n;
  rp.seed = seed;
  rp.run_key = run_key(seed, 0, 0x46495845ull);
  rp.max_events = o && o->max_events ? o->max_events : 1000000u;
  rp.keig = 0;
  rp.score = 1;
  rp.fast = (o && o->fast_math && rng == MC_RNG_PHILOX) ? 1 : 0;
  rp.from_bank = 0;
  rp.ref_source_seeds = 1;
  rp.max_yield = c->max_yield;
  if (o && (o->thermal == MC_THERMAL_SURROGATE || o->thermal == MC_THERMAL_GUIDED ||
            o->thermal == MC_THERMAL_POD_QUEUE)) {
    if (c->model.energy_mode != mc::kContinuous || rng != MC_RNG_PHILOX)
      return fail(c, MC_ERR_INPUT, "the thermal-scatter queue needs a continuous-energy problem and Philox streams");
    if (o->thermal == MC_THERMAL_SURROGATE && c->mlp_tsl < 0)
      return fail(c, MC_ERR_STATE, "no trained surrogate (mc_train_surrogate)");
    if (o->thermal == MC_THERMAL_GUIDED && c->guide_tsl < 0)
      return fail(c, MC_ERR_STATE, "no trained guide network (mc_train_surrogate_guide)");
    if (o->thermal != MC_THERMAL_SURROGATE && c->dw.n_tsl == 0)
      return fail(c, MC_ERR_INPUT, "the problem has no thermal scattering library");
    if (!c->model.perturbations.empty())
      return fail(c, MC_ERR_INPUT, "the thermal-scatter queue does not carry indirect effects");
    rp.tq = 1;  // run_transport takes the queue form
    rp.tq_mode = o->thermal == MC_THERMAL_SURROGATE ? 1 : (o->thermal == MC_THERMAL_GUIDED ? 2 : 3);
  }
  else if (o && o->thermal != MC_THERMAL_POD) {
    return fail(c, MC_ERR_INPUT, "unknown thermal sampler");
  }
  if (out && out->history_events) {
    rp.hist_events = static_cast<uint32_t*>(scratch(c, kHistEvents, n * 4));
    if (!rp.hist_events) return fail(c, MC_ERR_OOM, "history buffer");
  }
  if (out && out->history_fate) {
    rp.hist_fate = static_cast<int8_t*>(scratch(c, kHistFate, n));
    if (!rp.hist_fate) return fail(c, MC_ERR_OOM, "history buffer");
  }
  const size_t tb = std::max<uint64_t>(1, c->total_bins) * sizeof(double);
  CUDA_TRY(c, cudaMemsetAsync(c->d_sum, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_sq, 0, tb, c->stream));
  double ms = 0;
  const uint64_t l0 = c->launches;
  int rc = run_transport(c, rp, rng, block, &ms, o ? o->schedule : 0);
  if (rc != MC_OK) return rc;
  DevCounters h{};
  CUDA_TRY(c, cudaMemcpyAsync(&h, c->d_ctr, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  if (out) {
    if (out->sum) CUDA_TRY(c, cudaMemcpyAsync(out->sum, c->d_sum, c->total_bins * 8, cudaMemcpyDeviceToHost, c->stream));
    if (out->sum_sq) CUDA_TRY(c, cudaMemcpyAsync(out->sum_sq, c->d_sq, c->total_bins * 8, cudaMemcpyDeviceToHost, c->stream));
    if (out->history_events)
      CUDA_TRY(c, cudaMemcpyAsync(out->history_events, rp.hist_events, n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (out->history_fate)
      CUDA_TRY(c, cudaMemcpyAsync(out->history_fate, rp.hist_fate, n, cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (out) {
    out->histories = n;
    out->events = h.events;
    out->secondaries = h.secondaries;
    out->lost = h.lost;
    out->capped = h.capped;
    out->overflow = h.overflow;
    out->resample_failures = h.resample;
    out->transport_ms = ms;
    out->kernel_ms = c->last_kernel_ms;
    out->launches = c->launches - l0;
  }
  return counters_status(c, h);
}

int mc_keig_begin(mc_ctx* c, const mc_run_opts* o) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  cudaSetDevice(c->device);
  auto& k = c->keig;
  k = decltype(c->keig){};
  k.n = o && o->histories ? o->histories : c->model.histories;
  k.seed = o && o->seed ? o->seed : c->model.seed;
  k.inactive = o && (o->inactive || o->active) ? o->inactive : static_cast<uint32_t>(c->model.inactive);
  k.act = o && (o->inactive || o->active) ? o->active : static_cast<uint32_t>(c->model.active);
  k.rng = o ? o->rng : 0;
  k.fast = (o && o->fast_math && k.rng == MC_RNG_PHILOX) ? 1 : 0;
  k.block = pick_block(o);
  k.schedule = o ? o->schedule : 0;
  k.max_events = o && o->max_events ? o->max_events : 1000000u;
  k.bank_path = o ? o->bank_path : MC_BANK_AUTO;
  k.launches0 = c->launches;
  // tune on the second inactive cycle unless the caller fixed the block
  // size, the variant or the schedule
  c->tune_pending = !(o && (o->block_size > 0 || o->variant > 0)) && k.inactive > 0 &&
                    k.schedule == MC_SCHEDULE_AUTO;
  c->sort_min_req = o ? o->queue_sort_min : 0;
  if (o && o->variant > 0) c->variant = std::min(o->variant - 1, mcd::history_variants() - 1);
  if (k.rng != MC_RNG_PHILOX && k.rng != MC_RNG_MINSTD) return fail(c, MC_ERR_INPUT, "unknown rng mode");
  if (k.n == 0) return fail(c, MC_ERR_INPUT, "no histories");
  if (k.bank_path < MC_BANK_AUTO || k.bank_path > MC_BANK_DIRECT) return fail(c, MC_ERR_INPUT, "unknown bank path");
  if (bank_direct(c, k.rng, k.fast != 0, k.bank_path) < 0)
    return fail(c, MC_ERR_INPUT, "the direct bank path needs (multigroup) Philox streams and chi cdfs that end "
                                 "above every threshold the stream draws");
  if (!scratch(c, kSrc, k.n * sizeof(Site)) || !scratch(c, kSlots, k.n * c->max_yield * sizeof(Site)) ||
      !scratch(c, kCount, k.n * 4) || !scratch(c, kOffsets, k.n * 8) || !scratch(c, kBank, k.n * c->max_yield * sizeof(Site)))
    return fail(c, MC_ERR_OOM, "k-eigenvalue bank allocation failed");
  // the two dense per-history score arrays of the active cycles, zeroed
  // here so that no cycle allocates
  if (c->total_bins > 0 && c->total_bins <= static_cast<uint64_t>(mcd::kDenseBins)) {
    for (int b = 0; b < 2; b++) {
      const int slot = b == 0 ? kEvPend : kEvPend2;
      const size_t bytes = k.n * c->total_bins * sizeof(double);
      if (c->scratch[slot].bytes < bytes || !c->pend_zero[b]) {
        if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
        void* pp = scratch(c, slot, bytes);
        if (!pp) return fail(c, MC_ERR_OOM, "score buffers");
        CUDA_TRY(c, cudaMemsetAsync(pp, 0, c->scratch[slot].bytes, c->stream));
        c->pend_zero[b] = true;
        c->pend_zero_bytes[b] = c->scratch[slot].bytes;
      }
    }
  }
  // mc_keig_cycles' per-cycle records and timing events for the longer of
  // the two phases, so that its calls neither allocate nor create events
  const uint32_t phase = std::max<uint32_t>({k.inactive, k.act, 1u});
  if (!scratch(c, kCycleRec, 3 * sizeof(double) * phase + sizeof(DevCounters)))
    return fail(c, MC_ERR_OOM, "cycle records");
  while (c->ev_pool.size() < 4 * static_cast<size_t>(phase)) {
    cudaEvent_t e = nullptr;
    CUDA_TRY(c, cudaEventCreate(&e));
    c->ev_pool.push_back(e);
  }
  const size_t tb = std::max<uint64_t>(1, c->total_bins) * sizeof(double);
  CUDA_TRY(c, cudaMemsetAsync(c->d_sum, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_sq, 0, tb, c->stream));
  k.active = true;
  return MC_OK;
}

}  // extern "C"

namespace {
// the run parameters of the k-eigenvalue cycle about to run
RunParams keig_params(mc_ctx* c, int32_t active) {
  auto& k = c->keig;
  RunParams rp{};
  rp.n = k.n;
  rp.seed = k.seed;
  rp.cycle = k.cycle;
  rp.run_key = run_key(k.seed, k.cycle, 0x4b454947ull);
  rp.max_events = k.max_events;
  rp.keig = 1;
  rp.score = active ? 1 : 0;
  rp.fast = k.fast;
  rp.from_bank = k.cycle > 0 ? 1 : 0;
  rp.ref_source_seeds = 0;  // cycle 0: Source::Sample(1..N) (src/KEigenvalue.cpp:31-33)
  rp.minstd_base = k.seed + static_cast<unsigned long long>(k.cycle) * k.n;
  rp.max_yield = c->max_yield;
  rp.src = static_cast<const Site*>(c->scratch[kSrc].p);
  if (k.src_pending) {
    rp.resample_bank = static_cast<const Site*>(c->scratch[kBank].p);
    rp.resample_m = c->d_total;
    rp.resample_key = k.src_key;
  }
  rp.bank = static_cast<Site*>(c->scratch[kSlots].p);
  rp.bank_count = static_cast<uint32_t*>(c->scratch[kCount].p);
  rp.direct_sites = bank_direct(c, k.rng, k.fast != 0, k.bank_path) > 0 ? 1 : 0;
  return rp;
}

// the autotuner runs in this cycle
bool keig_tunes(const mc_ctx* c, int32_t active) {
  return !active && c->tune_pending && (c->keig.cycle >= 1 || c->keig.inactive < 2);
}
}  // namespace

extern "C" {

int mc_keig_cycle(mc_ctx* c, int32_t active, double* kout) {
  if (!check_ctx(c) || !c->keig.active) return fail(c, MC_ERR_STATE, "mc_keig_begin not called");
  auto& k = c->keig;
  RunParams rp = keig_params(c, active);
  // the autotuner waits for the second inactive cycle when there is one:
  // the first cycle's source (Source::Sample) is not yet the fission
  // source the later cycles transport
  if (keig_tunes(c, active)) {
    // Autotuner: every candidate transports this (inactive, unscored)
    // cycle, twice, interleaved, keeping each candidate's shorter time of
    // its transport kernels.  Candidates: the history schedule's occupancy
    // variants at blocks of 256 and 128 threads, and -- where the event
    // schedule serves the problem -- the event schedule with collision
    // queues unsorted and sorted (threshold 2^15).  All draw the same
    // numbers and give the same results; only the timing differs.
    c->tune_pending = false;
    struct Candidate {
      int schedule, variant, block;
      unsigned sort_min;
    };
    std::vector<Candidate> cand;
    const int nv = mcd::history_variants();
    for (int b : {256, 128})
      for (int v = 0; v < nv; v++) cand.push_back({MC_SCHEDULE_HISTORY, v, b, 0});
    if (event_schedule_ok(c)) {
      cand.push_back({MC_SCHEDULE_EVENT, 0, 256, 0});
      cand.push_back({MC_SCHEDULE_EVENT, 0, 256, 1u << 15});
    }
    const int nc = std::min<int>(static_cast<int>(cand.size()), 16);
    for (int i = 0; i < 16; i++) c->tune_ms[i] = i < nc ? 1e300 : 0;
    const unsigned req = c->sort_min_req;
    c->sort_min_req = 0;
    for (int pass = 0; pass < 2; pass++) {
      for (int i = 0; i < nc; i++) {
        c->variant = cand[i].variant;
        c->ev_sort_min = cand[i].sort_min;
        double t = 0;
        const int rc = run_transport(c, rp, k.rng, cand[i].block, &t, cand[i].schedule);
        if (rc != MC_OK) return rc;
        c->tune_ms[i] = std::min(c->tune_ms[i], c->last_kernel_ms);
      }
    }
    c->sort_min_req = req;
    int best = 0;
    for (int i = 1; i < nc; i++)
      if (c->tune_ms[i] < c->tune_ms[best]) best = i;
    // The tuning cycle is an early one (its source has not converged) and
    // one cycle's time carries about 1 % of noise: the high-occupancy
    // variants, which spill, have timed fastest there and then run 10-15 %
    // slower in the converged cycles.  So the default -- occupancy variant
    // 1 at 256 threads -- is kept unless a candidate beats it by more than
    // kTuneMargin.
    constexpr double kTuneMargin = 0.03;
    const int def = 1;  // {history, variant 1, 256 threads}
    if (def < nc && cand[def].schedule == MC_SCHEDULE_HISTORY && cand[def].variant == 1 && cand[def].block == 256 &&
        c->tune_ms[best] > (1.0 - kTuneMargin) * c->tune_ms[def])
      best = def;
    c->tuned_schedule = cand[best].schedule;
    c->variant = cand[best].variant;
    c->ev_sort_min = cand[best].sort_min;
    c->tuned_block = cand[best].block;
    k.block = cand[best].block;
  }
  // transport, bank and read-back with one synchronisation; the cycle's
  // timing events have completed by then
  int rc = run_transport(c, rp, k.rng, k.block, nullptr, k.schedule, /*side_commit=*/true);
  if (rc != MC_OK) return rc;
  k.src_pending = false;  // read by the transport, which precedes any write of the bank
  Site* bank = nullptr;
  uint64_t m = 0;
  rc = emit_bank(c, rp, k.rng, nullptr, 0, &bank, &m, /*read_size=*/false);
  if (rc != MC_OK) return rc;
  DevCounters h{};
  rc = read_back(c, &m, &h);
  if (rc != MC_OK) return rc;
  float f = 0;
  CUDA_TRY(c, cudaEventElapsedTime(&f, c->ev0, c->ev1));
  k.transport_ms += f;
  CUDA_TRY(c, cudaEventElapsedTime(&f, c->evk0, c->evk1));
  c->last_kernel_ms = f;
  k.kernel_ms += f;
  k.events += h.events;
  k.lost += h.lost;
  k.capped += h.capped;
  k.overflow += h.overflow;
  const double kc = static_cast<double>(m) / static_cast<double>(k.n);
  k.k.push_back(kc);
  k.ktl.push_back(h.k_tracklength / static_cast<double>(k.n));
  k.bank.push_back(m);
  if (kout) *kout = kc;
  if (m == 0) return fail(c, MC_ERR_INPUT, "fission bank is empty: the source died out");
  // next cycle's source: resampled from this bank as the next transport
  // reads it (the same draw as the resampling kernel)
  if (bank != c->scratch[kBank].p) return fail(c, MC_ERR_STATE, "fission bank outside its buffer");
  k.src_pending = true;
  k.src_key = run_key(k.seed, k.cycle, 0x52455341ull);
  k.cycle++;
  return counters_status(c, h);
}

int mc_keig_cycles(mc_ctx* c, uint32_t ncyc, int32_t active, double* kout) {
  if (!check_ctx(c) || !c->keig.active) return fail(c, MC_ERR_STATE, "mc_keig_begin not called");
  auto& k = c->keig;
  uint32_t done = 0;
  int status = MC_OK;  // the first non-fatal status (lost, overflow, cap, resample) of the cycles run
  // the first cycle (its source is Source::Sample's) and a tuning cycle run
  // on their own
  while (done < ncyc && (k.cycle == 0 || keig_tunes(c, active))) {
    const int rc = mc_keig_cycle(c, active, kout ? kout + done : nullptr);
    if (rc == MC_ERR_DEVICE || rc == MC_ERR_OOM || rc == MC_ERR_STATE || rc == MC_ERR_INPUT) return rc;
    if (rc != MC_OK && status == MC_OK) status = rc;
    done++;
  }
  const uint32_t m = ncyc - done;
  if (m == 0) return status;
  if (k.rng != MC_RNG_PHILOX && k.rng != MC_RNG_MINSTD) return fail(c, MC_ERR_STATE, "unknown rng mode");
  CUDA_TRY(c, cudaSetDevice(c->device));
  // per cycle (k, M, k_tracklength), then the counters of all m cycles
  const size_t rec_bytes = 3 * sizeof(double) * m;
  auto* rec = static_cast<double*>(scratch(c, kCycleRec, rec_bytes + sizeof(DevCounters)));
  if (!rec) return fail(c, MC_ERR_OOM, "cycle records");
  auto* acc = reinterpret_cast<DevCounters*>(reinterpret_cast<char*>(rec) + rec_bytes);
  CUDA_TRY(c, cudaMemsetAsync(acc, 0, sizeof(DevCounters), c->stream));
  while (c->ev_pool.size() < 4 * static_cast<size_t>(m)) {
    cudaEvent_t e = nullptr;
    CUDA_TRY(c, cudaEventCreate(&e));
    c->ev_pool.push_back(e);
  }
  cudaEvent_t keep[4] = {c->ev0, c->ev1, c->evk0, c->evk1};
  auto restore = [&]() {
    c->ev0 = keep[0];
    c->ev1 = keep[1];
    c->evk0 = keep[2];
    c->evk1 = keep[3];
  };
  for (uint32_t i = 0; i < m; i++) {
    RunParams rp = keig_params(c, active);
    // this cycle's timing events (read after the one synchronisation)
    c->ev0 = c->ev_pool[4 * i];
    c->ev1 = c->ev_pool[4 * i + 1];
    c->evk0 = c->ev_pool[4 * i + 2];
    c->evk1 = c->ev_pool[4 * i + 3];
    int rc = run_transport(c, rp, k.rng, k.block, nullptr, k.schedule, /*side_commit=*/true);
    restore();
    if (rc != MC_OK) return rc;
    k.src_pending = false;
    Site* bank = nullptr;
    uint64_t mm = 0;
    rc = emit_bank(c, rp, k.rng, nullptr, 0, &bank, &mm, /*read_size=*/false);
    if (rc != MC_OK) return rc;
    if (bank != c->scratch[kBank].p) return fail(c, MC_ERR_STATE, "fission bank outside its buffer");
    CUDA_TRY(c, mcd::launch_keig_record(c->d_ctr, c->d_total, k.n, rec + 3 * i, acc, c->stream));
    c->launches++;
    // the next cycle draws its sources from this bank (an empty bank is
    // reported below; the next transport then reads only entry 0)
    k.src_pending = true;
    k.src_key = run_key(k.seed, k.cycle, 0x52455341ull);
    k.cycle++;
  }
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  std::vector<double> h(3 * static_cast<size_t>(m));
  DevCounters tot{};
  CUDA_TRY(c, cudaMemcpyAsync(h.data(), rec, rec_bytes, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(&tot, acc, sizeof tot, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  for (uint32_t i = 0; i < m; i++) {
    float f = 0;
    CUDA_TRY(c, cudaEventElapsedTime(&f, c->ev_pool[4 * i], c->ev_pool[4 * i + 1]));
    k.transport_ms += f;
    CUDA_TRY(c, cudaEventElapsedTime(&f, c->ev_pool[4 * i + 2], c->ev_pool[4 * i + 3]));
    c->last_kernel_ms = f;
    k.kernel_ms += f;
    k.k.push_back(h[3 * i]);
    k.bank.push_back(static_cast<uint64_t>(h[3 * i + 1]));
    k.ktl.push_back(h[3 * i + 2]);
    if (kout) kout[done + i] = h[3 * i];
    if (h[3 * i + 1] == 0) break;  // the source died out: later cycles are void
  }
  k.events += tot.events;
  k.lost += tot.lost;
  k.capped += tot.capped;
  k.overflow += tot.overflow;
  if (tot.next) return fail(c, MC_ERR_INPUT, "fission bank is empty: the source died out");
  if (status != MC_OK) return status;
  return counters_status(c, tot);
}

int mc_keig_status(mc_ctx* c, mc_keig_out* out) {
  if (!check_ctx(c) || !c->keig.active) return fail(c, MC_ERR_STATE, "mc_keig_begin not called");
  auto& k = c->keig;
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (out) {
    const size_t nc = k.k.size();
    if (out->k_cycle) std::copy(k.k.begin(), k.k.end(), out->k_cycle);
    if (out->bank_size) std::copy(k.bank.begin(), k.bank.end(), out->bank_size);
    if (out->sum) CUDA_TRY(c, cudaMemcpy(out->sum, c->d_sum, c->total_bins * 8, cudaMemcpyDeviceToHost));
    if (out->sum_sq) CUDA_TRY(c, cudaMemcpy(out->sum_sq, c->d_sq, c->total_bins * 8, cudaMemcpyDeviceToHost));
    double s = 0, s2 = 0, st = 0;
    size_t na = 0;
    for (size_t i = k.inactive; i < nc; i++) {
      s += k.k[i];
      s2 += k.k[i] * k.k[i];
      st += k.ktl[i];
      na++;
    }
    out->k_mean = na ? s / na : 0;
    out->k_std = na > 1 ? std::sqrt(std::max(0.0, (s2 - s * s / na) / (na - 1)) / na) : 0;
    out->k_tracklength_mean = na ? st / na : 0;
    out->events = k.events;
    out->lost = k.lost;
    out->capped = k.capped;
    out->overflow = k.overflow;
    out->transport_ms = k.transport_ms;
    out->kernel_ms = k.kernel_ms;
    out->launches = c->launches - k.launches0;
  }
  return MC_OK;
}

int mc_schedule_info(mc_ctx* c, int32_t* schedule, int32_t* variant, int32_t* grid, int32_t* block, double* tune_ms,
                     int32_t n) {
  if (!c) return MC_ERR_INPUT;
  if (schedule) *schedule = c->last_schedule;
  if (variant) *variant = c->variant;
  if (grid) *grid = c->last_grid;
  if (block) *block = c->last_block;
  if (tune_ms)
    for (int32_t i = 0; i < n && i < 16; i++) tune_ms[i] = c->tune_ms[i];
  return MC_OK;
}

int mc_keig_end(mc_ctx* c, mc_keig_out* out) {
  const int rc = mc_keig_status(c, out);
  if (rc != MC_OK) return rc;
  c->keig.active = false;
  return MC_OK;
}

// ---- checkpoint / resume of a k-eigenvalue run -----------------------------
// Between cycles a run is fully described by its options, the cycle number,
// the per-cycle k / bank-size history, the counters, the tallies and the
// next cycle's source bank: every random stream of a later cycle is keyed by
// (seed, cycle) (Philox) or seeded from seed + cycle * n (minstd), so nothing
// else carries over.

namespace {

constexpr char kCkptMagic[8] = {'M', 'C', 'K', 'E', 'I', 'G', '1', 0};

struct CkptHeader {
  char magic[8];
  uint64_t n, seed, total_bins, max_yield, fingerprint;
  uint32_t inactive, act, cycle, max_events;
  int32_t rng, fast, block, schedule;
  uint64_t events, lost, capped, overflow;
  double transport_ms, kernel_ms;
  uint64_t ncycles;
};
static_assert(offsetof(CkptHeader, cycle) == 56, "the Python reader expects the cycle number at byte 56");

// FNV-1a over the problem's shape and names: a checkpoint resumes only into
// the problem it was taken from
uint64_t model_fingerprint(const mc::Model& m) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&h](const void* p, size_t n) {
    const auto* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 1099511628211ull;
  };
  const int64_t dims[] = {m.energy_mode, static_cast<int64_t>(m.groups), static_cast<int64_t>(m.cells.size()),
                          static_cast<int64_t>(m.surfaces.size()), static_cast<int64_t>(m.materials.size()),
                          static_cast<int64_t>(m.nuclides.size()), static_cast<int64_t>(m.estimators.size()),
                          static_cast<int64_t>(m.total_bins()), m.problem, m.tracking};
  mix(dims, sizeof dims);
  for (const auto& x : m.cells) mix(x.name.data(), x.name.size() + 1);
  for (const auto& x : m.materials) {
    mix(x.name.data(), x.name.size() + 1);
    mix(&x.number_density, sizeof x.number_density);
  }
  for (const auto& x : m.nuclides) mix(x.name.data(), x.name.size() + 1);
  for (const auto& x : m.estimators) mix(x.name.data(), x.name.size() + 1);
  return h;
}

}  // namespace

int mc_keig_checkpoint(mc_ctx* c, void* buf, uint64_t cap, uint64_t* size) {
  if (!check_ctx(c) || !c->keig.active) return fail(c, MC_ERR_STATE, "no k-eigenvalue run in progress");
  auto& k = c->keig;
  const uint64_t nc = k.k.size();
  const uint64_t tb = c->total_bins;
  const uint64_t bytes = sizeof(CkptHeader) + nc * (8 + 8 + 8) + 2 * tb * 8 + k.n * sizeof(Site);
  if (size) *size = bytes;
  if (!buf) return MC_OK;
  if (cap < bytes) return fail(c, MC_ERR_OVERFLOW, "checkpoint buffer too small");
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  CkptHeader h{};
  std::memcpy(h.magic, kCkptMagic, 8);
  h.n = k.n;
  h.seed = k.seed;
  h.total_bins = tb;
  h.max_yield = c->max_yield;
  h.fingerprint = model_fingerprint(c->model);
  h.inactive = k.inactive;
  h.act = k.act;
  h.cycle = k.cycle;
  h.max_events = k.max_events;
  h.rng = k.rng;
  h.fast = k.fast;
  h.block = k.block;
  h.schedule = k.schedule;
  h.events = k.events;
  h.lost = k.lost;
  h.capped = k.capped;
  h.overflow = k.overflow;
  h.transport_ms = k.transport_ms;
  h.kernel_ms = k.kernel_ms;
  h.ncycles = nc;
  auto* out = static_cast<char*>(buf);
  std::memcpy(out, &h, sizeof h);
  out += sizeof h;
  std::memcpy(out, k.k.data(), nc * 8);
  out += nc * 8;
  std::memcpy(out, k.ktl.data(), nc * 8);
  out += nc * 8;
  std::memcpy(out, k.bank.data(), nc * 8);
  out += nc * 8;
  CUDA_TRY(c, cudaMemcpyAsync(out, c->d_sum, tb * 8, cudaMemcpyDeviceToHost, c->stream));
  out += tb * 8;
  CUDA_TRY(c, cudaMemcpyAsync(out, c->d_sq, tb * 8, cudaMemcpyDeviceToHost, c->stream));
  out += tb * 8;
  if (materialize_source(c) != MC_OK) return MC_ERR_DEVICE;
  CUDA_TRY(c, cudaMemcpyAsync(out, c->scratch[kSrc].p, k.n * sizeof(Site), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_keig_resume(mc_ctx* c, const void* buf, uint64_t size) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (!buf || size < sizeof(CkptHeader)) return fail(c, MC_ERR_INPUT, "checkpoint too short");
  CkptHeader h;
  std::memcpy(&h, buf, sizeof h);
  if (std::memcmp(h.magic, kCkptMagic, 8) != 0) return fail(c, MC_ERR_INPUT, "not a k-eigenvalue checkpoint");
  const uint64_t bytes = sizeof(CkptHeader) + h.ncycles * 24 + 2 * h.total_bins * 8 + h.n * sizeof(Site);
  if (h.n == 0 || h.ncycles != h.cycle || size != bytes) return fail(c, MC_ERR_INPUT, "corrupt checkpoint");
  if (h.fingerprint != model_fingerprint(c->model) || h.total_bins != c->total_bins || h.max_yield != c->max_yield)
    return fail(c, MC_ERR_INPUT, "checkpoint belongs to another problem");
  cudaSetDevice(c->device);
  auto& k = c->keig;
  k = decltype(c->keig){};
  k.n = h.n;
  k.seed = h.seed;
  k.inactive = h.inactive;
  k.act = h.act;
  k.cycle = h.cycle;
  k.max_events = h.max_events;
  k.rng = h.rng;
  k.fast = h.fast;
  k.block = h.block;
  k.schedule = h.schedule;
  k.events = h.events;
  k.lost = h.lost;
  k.capped = h.capped;
  k.overflow = h.overflow;
  k.transport_ms = h.transport_ms;
  k.kernel_ms = h.kernel_ms;
  k.launches0 = c->launches;
  const char* in = static_cast<const char*>(buf) + sizeof h;
  k.k.assign(reinterpret_cast<const double*>(in), reinterpret_cast<const double*>(in) + h.ncycles);
  in += h.ncycles * 8;
  k.ktl.assign(reinterpret_cast<const double*>(in), reinterpret_cast<const double*>(in) + h.ncycles);
  in += h.ncycles * 8;
  k.bank.assign(reinterpret_cast<const uint64_t*>(in), reinterpret_cast<const uint64_t*>(in) + h.ncycles);
  in += h.ncycles * 8;
  // the variants give identical results, so the resumed run keeps the
  // current one rather than tuning again
  c->tune_pending = false;
  if (!scratch(c, kSrc, k.n * sizeof(Site)) || !scratch(c, kSlots, k.n * c->max_yield * sizeof(Site)) ||
      !scratch(c, kCount, k.n * 4) || !scratch(c, kOffsets, k.n * 8) || !scratch(c, kBank, k.n * c->max_yield * sizeof(Site)))
    return fail(c, MC_ERR_OOM, "k-eigenvalue bank allocation failed");
  const size_t tb = std::max<uint64_t>(1, c->total_bins) * sizeof(double);
  CUDA_TRY(c, cudaMemsetAsync(c->d_sum, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_sq, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(c->d_sum, in, h.total_bins * 8, cudaMemcpyHostToDevice, c->stream));
  in += h.total_bins * 8;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_sq, in, h.total_bins * 8, cudaMemcpyHostToDevice, c->stream));
  in += h.total_bins * 8;
  CUDA_TRY(c, cudaMemcpyAsync(c->scratch[kSrc].p, in, k.n * sizeof(Site), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  k.active = true;
  return MC_OK;
}

int mc_run_keigenvalue(mc_ctx* c, const mc_run_opts* o, mc_keig_out* out) {
  int rc = mc_keig_begin(c, o);
  if (rc != MC_OK) return rc;
  int status = MC_OK;
  // the inactive cycles, then the active ones, each phase with one host
  // synchronisation (mc_keig_cycles)
  for (int phase = 0; phase < 2; phase++) {
    const uint32_t n = phase == 0 ? c->keig.inactive : c->keig.act;
    if (n == 0) continue;
    rc = mc_keig_cycles(c, n, phase, nullptr);
    if (rc == MC_ERR_DEVICE || rc == MC_ERR_OOM || rc == MC_ERR_STATE || (rc == MC_ERR_INPUT)) {
      mc_keig_end(c, out);
      return rc;
    }
    if (rc != MC_OK && status == MC_OK) status = rc;
  }
  rc = mc_keig_end(c, out);
  return rc != MC_OK ? rc : status;
}

int mc_transport_bank(mc_ctx* c, const mc_site* sites, uint64_t n, const mc_run_opts* o, mc_site* fission_sites,
                      uint64_t cap, uint64_t* n_out) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  const int rng = o ? o->rng : MC_RNG_PHILOX;
  if (rng != MC_RNG_PHILOX && rng != MC_RNG_MINSTD) return fail(c, MC_ERR_INPUT, "unknown rng mode");
  if (n == 0) {
    if (n_out) *n_out = 0;
    return MC_OK;
  }
  if (!sites) return fail(c, MC_ERR_INPUT, "sites is NULL");
  const int path = o ? o->bank_path : MC_BANK_AUTO;
  if (path < MC_BANK_AUTO || path > MC_BANK_DIRECT) return fail(c, MC_ERR_INPUT, "unknown bank path");
  const bool fast = o && o->fast_math && rng == MC_RNG_PHILOX;
  const int direct = bank_direct(c, rng, fast, path);
  if (direct < 0)
    return fail(c, MC_ERR_INPUT, "the direct bank path needs (multigroup) Philox streams and chi cdfs that end "
                                 "above every threshold the stream draws");
  cudaSetDevice(c->device);
  if ((!direct && !scratch(c, kSlots, n * c->max_yield * sizeof(Site))) || !scratch(c, kCount, n * 4))
    return fail(c, MC_ERR_OOM, "bank allocation failed");
  // Sites in page-locked host memory are read in place by the transport
  // kernel (each site once, coalesced, when its history starts), so the
  // host-to-device transfer overlaps the transport instead of preceding it;
  // pageable memory is copied first.
  c->sort_min_req = o ? o->queue_sort_min : 0;
  const Site* src = nullptr;
  cudaPointerAttributes pa{};
  if (cudaPointerGetAttributes(&pa, sites) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer) {
    src = static_cast<const Site*>(pa.devicePointer);
  }
  else {
    (void)cudaGetLastError();
    auto* dst = static_cast<Site*>(scratch(c, kSrc, n * sizeof(Site)));
    if (!dst) return fail(c, MC_ERR_OOM, "bank allocation failed");
    CUDA_TRY(c, cudaMemcpyAsync(dst, sites, n * sizeof(Site), cudaMemcpyHostToDevice, c->stream));
    src = dst;
  }
  RunParams rp{};
  rp.n = n;
  rp.seed = c->model.seed;
  rp.run_key = run_key(c->model.seed, 0, 0x42414e4bull);
  rp.max_events = o && o->max_events ? o->max_events : 1000000u;
  rp.keig = 1;
  rp.score = 1;
  rp.fast = (o && o->fast_math && rng == MC_RNG_PHILOX) ? 1 : 0;
  rp.from_bank = 1;
  rp.minstd_base = 0;  // each site's own key seeds its stream
  rp.max_yield = c->max_yield;
  rp.src = src;
  rp.bank = static_cast<Site*>(c->scratch[kSlots].p);
  rp.bank_count = static_cast<uint32_t*>(c->scratch[kCount].p);
  rp.direct_sites = direct;
  int rc = run_transport(c, rp, rng, pick_block(o), nullptr, o ? o->schedule : MC_SCHEDULE_AUTO,
                         /*side_commit=*/true);
  if (rc != MC_OK) return rc;
  // Page-locked output (16-byte aligned) is written in place over the
  // chip-to-chip link with coalesced 16-byte stores, by the direct site
  // kernel or by a copy kernel after the compaction, and the bank size stays
  // on the device until the one read-back; pageable output gets a copy after
  // the size is read.  (A compaction kernel writing into host memory one site
  // per thread measured slower: its scattered 64-byte writes cross the link
  // one site at a time.)
  Site* out_mapped = nullptr;
  if (fission_sites && cap) {
    cudaPointerAttributes oa{};
    if (cudaPointerGetAttributes(&oa, fission_sites) == cudaSuccess && oa.type == cudaMemoryTypeHost &&
        oa.devicePointer && reinterpret_cast<uintptr_t>(oa.devicePointer) % 16 == 0)
      out_mapped = static_cast<Site*>(oa.devicePointer);
    else
      (void)cudaGetLastError();
  }
  Site* bank = nullptr;
  uint64_t m = 0;
  rc = emit_bank(c, rp, rng, direct ? out_mapped : nullptr, cap, &bank, &m, /*read_size=*/out_mapped == nullptr);
  if (rc != MC_OK) return rc;
  if (out_mapped && bank) {
    k_copy_bank_out<<<c->num_sms * 8, 256, 0, c->stream>>>(
        reinterpret_cast<const uint4*>(bank), c->d_total, cap,
        reinterpret_cast<uint4*>(out_mapped));
    CUDA_TRY(c, cudaGetLastError());
    c->launches++;
  }
  else if (!out_mapped && fission_sites && cap) {
    CUDA_TRY(c, cudaMemcpyAsync(fission_sites, bank, std::min(m, cap) * sizeof(Site), cudaMemcpyDeviceToHost, c->stream));
  }
  DevCounters h{};
  rc = read_back(c, out_mapped ? &m : nullptr, &h);
  if (rc != MC_OK) return rc;
  if (n_out) *n_out = m;
  if (m > cap) return fail(c, MC_ERR_OVERFLOW, "fission bank larger than the output capacity");
  return counters_status(c, h);
}

int mc_tallies_reset(mc_ctx* c) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  const size_t tb = std::max<uint64_t>(1, c->total_bins) * sizeof(double);
  CUDA_TRY(c, cudaMemsetAsync(c->d_sum, 0, tb, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_sq, 0, tb, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_tallies_get(mc_ctx* c, double* sum, double* sum_sq) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  if (sum) CUDA_TRY(c, cudaMemcpyAsync(sum, c->d_sum, c->total_bins * 8, cudaMemcpyDeviceToHost, c->stream));
  if (sum_sq) CUDA_TRY(c, cudaMemcpyAsync(sum_sq, c->d_sq, c->total_bins * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

// ---- probes --------------------------------------------------------------

int mc_find_cell(mc_ctx* c, const double* xyz, uint64_t n, int32_t* cell) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (n == 0) return MC_OK;
  if (!xyz || !cell) return fail(c, MC_ERR_INPUT, "null argument");
  auto* dx = static_cast<double*>(scratch(c, kProbeIn, n * 24));
  auto* dc = static_cast<int32_t*>(scratch(c, kProbeOut, n * 4));
  if (!dx || !dc) return fail(c, MC_ERR_OOM, "probe buffers");
  CUDA_TRY(c, cudaMemcpyAsync(dx, xyz, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_find_cell(c->dw, dx, n, dc, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(cell, dc, n * 4, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_nearest_surface(mc_ctx* c, const int32_t* cell, const double* xyz, const double* uvw, uint64_t n,
                       int32_t* surf, double* dist) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (n == 0) return MC_OK;
  if (!cell || !xyz || !uvw || !surf || !dist) return fail(c, MC_ERR_INPUT, "null argument");
  auto* in = static_cast<char*>(scratch(c, kProbeIn, n * (24 + 24 + 4)));
  auto* outp = static_cast<char*>(scratch(c, kProbeOut, n * (4 + 8)));
  if (!in || !outp) return fail(c, MC_ERR_OOM, "probe buffers");
  auto* dxyz = reinterpret_cast<double*>(in);
  auto* duvw = reinterpret_cast<double*>(in + n * 24);
  auto* dcell = reinterpret_cast<int32_t*>(in + n * 48);
  auto* ddist = reinterpret_cast<double*>(outp);
  auto* dsurf = reinterpret_cast<int32_t*>(outp + n * 8);
  CUDA_TRY(c, cudaMemcpyAsync(dxyz, xyz, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(duvw, uvw, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dcell, cell, n * 4, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_nearest_surface(c->dw, dcell, dxyz, duvw, n, dsurf, ddist, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(surf, dsurf, n * 4, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(dist, ddist, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_surface_distance(mc_ctx* c, int32_t s, const double* xyz, const double* uvw, uint64_t n, double* dist) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (s < 0 || s >= c->dw.n_surfaces) return fail(c, MC_ERR_INPUT, "surface index out of range");
  if (n == 0) return MC_OK;
  if (!xyz || !uvw || !dist) return fail(c, MC_ERR_INPUT, "null argument");
  auto* in = static_cast<double*>(scratch(c, kProbeIn, n * 48));
  auto* outp = static_cast<double*>(scratch(c, kProbeOut, n * 8));
  if (!in || !outp) return fail(c, MC_ERR_OOM, "probe buffers");
  CUDA_TRY(c, cudaMemcpyAsync(in, xyz, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(in + 3 * n, uvw, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_surface_distance(c->dw, s, in, in + 3 * n, n, outp, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(dist, outp, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_surface_contains(mc_ctx* c, int32_t s, const double* xyz, uint64_t n, int8_t* contains) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (s < 0 || s >= c->dw.n_surfaces) return fail(c, MC_ERR_INPUT, "surface index out of range");
  if (n == 0) return MC_OK;
  if (!xyz || !contains) return fail(c, MC_ERR_INPUT, "null argument");
  auto* in = static_cast<double*>(scratch(c, kProbeIn, n * 24));
  auto* outp = static_cast<int8_t*>(scratch(c, kProbeOut, n));
  if (!in || !outp) return fail(c, MC_ERR_OOM, "probe buffers");
  CUDA_TRY(c, cudaMemcpyAsync(in, xyz, n * 24, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_surface_contains(c->dw, s, in, n, outp, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(contains, outp, n, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_material_xs(mc_ctx* c, int32_t cell, const double* xyz, const double* energy, uint64_t n, double* total,
                   double* majorant) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (cell < 0 || cell >= c->dw.n_cells) return fail(c, MC_ERR_INPUT, "cell index out of range");
  if (n == 0) return MC_OK;
  if (!energy || !total || !majorant) return fail(c, MC_ERR_INPUT, "null argument");
  if (c->dw.cell_mat == nullptr || c->model.cells[static_cast<size_t>(cell)].material < 0)
    return fail(c, MC_ERR_INPUT, "cell has no material");
  // continuous-energy cross sections depend on the temperature at the point
  const bool ce = c->model.energy_mode != mc::kMultigroup;
  auto* in = static_cast<double*>(scratch(c, kProbeIn, n * (ce ? 32 : 8)));
  auto* outp = static_cast<double*>(scratch(c, kProbeOut, n * 16));
  if (!in || !outp) return fail(c, MC_ERR_OOM, "probe buffers");
  CUDA_TRY(c, cudaMemcpyAsync(in, energy, n * 8, cudaMemcpyHostToDevice, c->stream));
  if (ce) {
    if (xyz) CUDA_TRY(c, cudaMemcpyAsync(in + n, xyz, n * 24, cudaMemcpyHostToDevice, c->stream));
    else CUDA_TRY(c, cudaMemsetAsync(in + n, 0, n * 24, c->stream));
    CUDA_TRY(c, mcd::launch_material_xs_ce(c->dw, cell, in, in + n, n, outp, outp + n, c->stream));
  }
  else {
    CUDA_TRY(c, mcd::launch_material_xs_mg(c->dw, cell, in, n, outp, outp + n, c->stream));
  }
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(total, outp, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(majorant, outp + n, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

namespace {
void copy_text(const std::string& t, char* buf, size_t n, size_t* needed) {
  if (needed) *needed = t.size();
  if (buf && n) {
    const size_t k = std::min(n - 1, t.size());
    std::memcpy(buf, t.data(), k);
    buf[k] = 0;
  }
}
}  // namespace

int mc_output_text(mc_ctx* c, const double* sum, const double* sum_sq, uint64_t batchsize, double total_weight,
                   char* buf, size_t n, size_t* needed) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if ((!sum || !sum_sq) && c->total_bins) return fail(c, MC_ERR_INPUT, "null argument");
  if (!(total_weight > 0)) return fail(c, MC_ERR_INPUT, "total weight must be positive");
  copy_text(mc::format_output(c->model, sum, sum_sq, total_weight, batchsize), buf, n, needed);
  return MC_OK;
}

int mc_output_format(const char* xml_text, const char* base_dir, const double* sum, const double* sum_sq,
                     uint64_t batchsize, double total_weight, char* buf, size_t n, size_t* needed) {
  if (!xml_text || !(total_weight > 0)) return MC_ERR_INPUT;
  try {
    const mc::Model m = mc::load_model(xml_text, base_dir ? base_dir : "");
    if (m.total_bins() && (!sum || !sum_sq)) return MC_ERR_INPUT;
    copy_text(mc::format_output(m, sum, sum_sq, total_weight, batchsize), buf, n, needed);
  }
  catch (const std::exception& e) {
    copy_text(e.what(), buf, n, needed);
    return MC_ERR_INPUT;
  }
  return MC_OK;
}

int mc_energy_index(mc_ctx* c, int32_t nuclide, const double* energy, uint64_t n, int64_t* upper_index) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (c->model.energy_mode != mc::kContinuous) return fail(c, MC_ERR_INPUT, "not a continuous-energy problem");
  if (nuclide < 0 || nuclide >= c->dw.n_nuclides || !c->model.nuclides[static_cast<size_t>(nuclide)].present[0])
    return fail(c, MC_ERR_INPUT, "nuclide index out of range or without neutron data");
  if (n == 0) return MC_OK;
  if (!energy || !upper_index) return fail(c, MC_ERR_INPUT, "null argument");
  auto* in = static_cast<double*>(scratch(c, kProbeIn, n * 8));
  auto* outp = static_cast<long long*>(scratch(c, kProbeOut, n * 48));
  if (!in || !outp) return fail(c, MC_ERR_OOM, "probe buffers");
  CUDA_TRY(c, cudaMemcpyAsync(in, energy, n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_energy_index(c->dw, nuclide, in, n, outp, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(upper_index, outp, n * 48, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

}  // extern "C"

namespace {

// ---- MLP surrogate: device buffers ------------------------------------------
template <class T>
T* mlp_alloc(mc_ctx* c, size_t n) {
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)) != cudaSuccess) return nullptr;
  c->mlp_allocs.push_back(p);
  return static_cast<T*>(p);
}

bool mlp_net_alloc(mc_ctx* c, mcd::MlpNet& n) {
  if (n.p) return true;
  using bf = __nv_bfloat16;
  const size_t W = mcd::kMlpWidth;
  n.p = mlp_alloc<float>(c, mcd::kMlpParams);
  n.g = mlp_alloc<float>(c, mcd::kMlpParams);
  n.m = mlp_alloc<float>(c, mcd::kMlpParams);
  n.v = mlp_alloc<float>(c, mcd::kMlpParams);
  n.W1 = mlp_alloc<__half>(c, W * mcd::kMlpIn);
  n.W2 = mlp_alloc<__half>(c, W * W);
  n.W3 = mlp_alloc<__half>(c, W * W);
  n.W2t = mlp_alloc<bf>(c, W * W);
  n.W3t = mlp_alloc<bf>(c, W * W);
  return n.p && n.g && n.m && n.v && n.W1 && n.W2 && n.W3 && n.W2t && n.W3t;
}

bool mlp_batch_alloc(mc_ctx* c, int B) {
  if (c->mlp_batch_cap >= B) {
    c->mlp_batch.B = B;
    return true;
  }
  using bf = __nv_bfloat16;
  mcd::MlpBatch& b = c->mlp_batch;
  const size_t n = static_cast<size_t>(B), W = mcd::kMlpWidth;
  b.X = mlp_alloc<__half>(c, n * mcd::kMlpIn);
  b.Xt = mlp_alloc<bf>(c, n * mcd::kMlpIn);
  b.y = mlp_alloc<float>(c, n);
  b.Z1 = mlp_alloc<float>(c, n * W);
  b.Z2 = mlp_alloc<float>(c, n * W);
  b.Z3 = mlp_alloc<float>(c, n * W);
  b.H1 = mlp_alloc<__half>(c, n * W);
  b.H2 = mlp_alloc<__half>(c, n * W);
  b.H1t = mlp_alloc<bf>(c, n * W);
  b.H2t = mlp_alloc<bf>(c, n * W);
  b.dZ3 = mlp_alloc<bf>(c, n * W);
  b.dZ2 = mlp_alloc<bf>(c, n * W);
  b.dZ3t = mlp_alloc<bf>(c, n * W);
  b.dZ2t = mlp_alloc<bf>(c, n * W);
  b.dZ1t = mlp_alloc<bf>(c, n * W);
  b.loss = mlp_alloc<float>(c, 1);
  if (!(b.X && b.Xt && b.y && b.Z1 && b.Z2 && b.Z3 && b.H1 && b.H2 && b.H1t && b.H2t && b.dZ3 && b.dZ2 && b.dZ3t &&
        b.dZ2t && b.dZ1t && b.loss))
    return false;
  c->mlp_batch_cap = B;
  b.B = B;
  return true;
}

// a tensor-core wait that gave up leaves a flag; report and clear it
int mlp_check(mc_ctx* c) {
  int h = 0;
  CUDA_TRY(c, cudaMemcpy(&h, mcd::mlp_error_flag(), sizeof h, cudaMemcpyDeviceToHost));
  if (h) {
    const int z = 0;
    cudaMemcpy(mcd::mlp_error_flag(), &z, sizeof z, cudaMemcpyHostToDevice);
    return fail(c, MC_ERR_TIMEOUT, "a tensor-core product did not complete in time");
  }
  return MC_OK;
}

// PyTorch-style initialisation U(-1/sqrt(fan_in), 1/sqrt(fan_in))
std::vector<float> mlp_init_params(uint64_t seed, int used_inputs) {
  std::vector<float> p(mcd::kMlpParams, 0.0f);
  uint64_t st = seed;
  auto uni = [&](float a) {
    st = mcd::splitmix64(st);
    return a * (2.0f * static_cast<float>((st >> 11) * (1.0 / 9007199254740992.0)) - 1.0f);
  };
  const float a1 = 1.0f / std::sqrt(static_cast<float>(used_inputs)), a = 1.0f / std::sqrt(128.0f);
  for (int o = 0; o < mcd::kMlpWidth; o++)
    for (int i = 0; i < used_inputs; i++) {
      // input i and its residual (slot 8 + i, scaled by 2048) start as one input
      const float wi = uni(a1);
      p[mcd::kMlpW1 + o * mcd::kMlpIn + i] = wi;
      p[mcd::kMlpW1 + o * mcd::kMlpIn + 8 + i] = wi / 2048.0f;
    }
  for (int i = 0; i < mcd::kMlpWidth; i++) p[mcd::kMlpB1 + i] = uni(a1);
  for (int i = 0; i < mcd::kMlpWidth * mcd::kMlpWidth; i++) {
    p[mcd::kMlpW2 + i] = uni(a);
    p[mcd::kMlpW3 + i] = uni(a);
  }
  for (int i = 0; i < mcd::kMlpWidth; i++) {
    p[mcd::kMlpB2 + i] = uni(a);
    p[mcd::kMlpB3 + i] = uni(a);
    p[mcd::kMlpW4 + i] = uni(a);
  }
  p[mcd::kMlpB4] = 0.5f;
  return p;
}

// one network trained on (X, y) by Adam with a cosine-decayed rate; returns
// the mean squared error over the last 5 % of the steps.  The step number,
// each step's learning rate and Adam's bias corrections live on the device,
// so after an eager first step (which also sets the products' launch
// attributes) one captured CUDA graph of kGraphSteps steps is replayed;
// the steps left over run eagerly with the same device state.
int mlp_train(mc_ctx* c, mcd::MlpNet& net, const __half* X, const float* y, uint64_t n, int used_inputs,
              const mc_train_desc& d, uint64_t key, double* loss_out) {
  constexpr uint32_t kGraphSteps = 8;
  const std::vector<float> p0 = mlp_init_params(key, used_inputs);
  CUDA_TRY(c, cudaMemcpyAsync(net.p, p0.data(), p0.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(net.m, 0, mcd::kMlpParams * sizeof(float), c->stream));
  CUDA_TRY(c, cudaMemsetAsync(net.v, 0, mcd::kMlpParams * sizeof(float), c->stream));
  CUDA_TRY(c, mcd::mlp_refresh_weights(net, c->stream));
  // the step state and the per-step losses live for this call only
  // (cudaFree waits for the device, so an early return frees them safely)
  struct CallBuffers {
    std::vector<void*> p;
    ~CallBuffers() {
      for (void* q : p) cudaFree(q);
    }
    void* get(size_t bytes) {
      void* q = nullptr;
      if (cudaMalloc(&q, std::max<size_t>(16, bytes)) != cudaSuccess) return nullptr;
      p.push_back(q);
      return q;
    }
  } bufs;
  auto* losses = static_cast<float*>(bufs.get(d.steps * sizeof(float)));
  auto* sched = static_cast<float*>(bufs.get(3ull * d.steps * sizeof(float)));
  auto* step = static_cast<int*>(bufs.get(sizeof(int)));
  if (!losses || !sched || !step) return fail(c, MC_ERR_OOM, "surrogate training buffers");
  std::vector<float> hs(3ull * d.steps);
  for (uint32_t t = 1; t <= d.steps; t++) {
    const double frac = static_cast<double>(t) / d.steps;
    hs[3 * (t - 1)] = static_cast<float>(d.lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(M_PI * frac))));
    hs[3 * (t - 1) + 1] = 1.0f / (1.0f - powf(0.9f, static_cast<float>(t)));
    hs[3 * (t - 1) + 2] = 1.0f / (1.0f - powf(0.999f, static_cast<float>(t)));
  }
  const int one = 1;
  CUDA_TRY(c, cudaMemcpyAsync(sched, hs.data(), hs.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(step, &one, sizeof one, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(losses, 0, d.steps * sizeof(float), c->stream));
  mcd::MlpBatch b = c->mlp_batch;
  b.loss = losses;
  const mcd::StepState st{step, sched};
  auto one_step = [&](cudaStream_t s) -> cudaError_t {
    cudaError_t e;
    if ((e = mcd::launch_mlp_gather(X, y, n, key, 0, b, s, step)) != cudaSuccess) return e;
    if ((e = mcd::mlp_forward_backward(net, b, s, st)) != cudaSuccess) return e;
    return mcd::mlp_adam(net, st, s);
  };
  CUDA_TRY(c, one_step(c->stream));
  uint32_t done = 1;
  c->launches += 12;
  const uint32_t reps = (d.steps - done) / kGraphSteps;
  if (reps > 0) {
    // the capture runs on a stream of its own (the context's stream may be
    // the legacy default stream, which cannot be captured), ordered after
    // the work queued so far and before what follows by events
    cudaStream_t cs = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto release = [&]() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
      if (cs) cudaStreamDestroy(cs);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    // a capture that cannot be made (nothing has run yet) leaves the steps
    // to the eager loop below
    bool captured = false;
    if (e == cudaSuccess && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      cudaError_t ce = cudaSuccess;
      for (uint32_t k = 0; k < kGraphSteps && ce == cudaSuccess; k++) ce = one_step(cs);
      const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
      captured = ce == cudaSuccess && ee == cudaSuccess && graph &&
                 cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
      (void)cudaGetLastError();
    }
    if (e == cudaSuccess && !captured) {
      release();
      cs = nullptr;
      ev[0] = ev[1] = nullptr;
      graph = nullptr;
      exec = nullptr;
    }
    else if (e == cudaSuccess) {
      e = cudaEventRecord(ev[0], c->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev[0], 0);
    }
    if (exec) {
      for (uint32_t r = 0; r < reps && e == cudaSuccess; r++) {
        e = cudaGraphLaunch(exec, cs);
        done += kGraphSteps;
        c->launches += 12 * kGraphSteps;
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev[1], cs);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, ev[1], 0);
    }
    if (e != cudaSuccess) {
      if (cs) cudaStreamSynchronize(cs);
      release();
      return fail(c, MC_ERR_DEVICE, std::string("surrogate training graph: ") + cudaGetErrorString(e));
    }
    // the stream and graph go once the replays have run
    if (cs) CUDA_TRY(c, cudaStreamSynchronize(cs));
    release();
  }
  for (; done < d.steps; done++) {
    CUDA_TRY(c, one_step(c->stream));
    c->launches += 12;
  }
  std::vector<float> h(d.steps);
  CUDA_TRY(c, cudaMemcpyAsync(h.data(), losses, d.steps * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  const uint32_t tail = std::max<uint32_t>(1, d.steps / 20);
  double acc = 0;
  for (uint32_t i = d.steps - tail; i < d.steps; i++) acc += h[i];
  *loss_out = acc / tail / d.batch;
  return mlp_check(c);
}

int sample_tsl_mlp(mc_ctx* c, int32_t tsl, const double* E, const double* T, uint64_t n, uint64_t seed, int32_t,
                   double* beta, double* alpha, uint64_t* failures) {
  if (c->mlp_tsl != tsl) return fail(c, MC_ERR_STATE, "the MLP surrogate is not trained for this library");
  auto* d_fail = static_cast<unsigned long long*>(scratch(c, kTslFail, sizeof(unsigned long long)));
  if (!d_fail) return fail(c, MC_ERR_OOM, "sampler counters");
  CUDA_TRY(c, cudaMemsetAsync(d_fail, 0, sizeof(unsigned long long), c->stream));
  CUDA_TRY(c, mcd::launch_sample_tsl_mlp(c->dw.tsl + tsl, c->mlp[0], c->mlp[1], c->mlp_box, E, T, n,
                                         run_key(seed, 0, 0x4D4C5053ull), beta, alpha, d_fail, c->num_sms,
                                         c->stream));
  c->launches++;
  unsigned long long h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, d_fail, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (failures) *failures = h;
  return mlp_check(c);
}

// the sampler on device arrays; `method` as mc_sample_tsl
int sample_tsl_device(mc_ctx* c, int32_t tsl, const double* E, const double* T, uint64_t n, uint64_t seed,
                      int32_t method, double* beta, double* alpha, uint64_t* failures) {
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  const int base = method & 0xF;
  if (base == MC_TSL_MLP) return sample_tsl_mlp(c, tsl, E, T, n, seed, method, beta, alpha, failures);
  if (base == MC_TSL_GUIDED) {
    if (c->guide_tsl != tsl) return fail(c, MC_ERR_STATE, "the guide network is not trained for this library");
    const bool gfast = (method & MC_TSL_FAST) != 0;
    if (gfast && !c->tsl_fast_ok[static_cast<size_t>(tsl)])
      return fail(c, MC_ERR_INPUT, "the FP32 POD form supports ranks up to " + std::to_string(mcd::kFastPodRank));
    auto* d_fail = static_cast<unsigned long long*>(scratch(c, kTslFail, sizeof(unsigned long long)));
    if (!d_fail) return fail(c, MC_ERR_OOM, "sampler counters");
    CUDA_TRY(c, cudaMemsetAsync(d_fail, 0, sizeof(unsigned long long), c->stream));
    // the POD sampler's stream keys (Philox), so that the samples are its own
    CUDA_TRY(c, mcd::launch_sample_tsl_guided(c->dw.tsl + tsl, c->guide, c->guide_box, gfast, E, T, n,
                                              run_key(seed, 0, 0x54534C00ull), beta, alpha, d_fail, c->num_sms,
                                              c->stream));
    c->launches++;
    unsigned long long h = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&h, d_fail, sizeof h, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (failures) *failures = h;
    return mlp_check(c);
  }
  if (base != MC_TSL_POD) return fail(c, MC_ERR_INPUT, "unknown thermal scattering method");
  const bool philox = (method & MC_TSL_PHILOX) != 0;
  const bool fast = (method & MC_TSL_FAST) != 0;
  if (fast && !c->model.tsl[static_cast<size_t>(tsl)].beta.S.empty()) {
    const mc::TSLData& t = c->model.tsl[static_cast<size_t>(tsl)];
    for (const auto* set : {&t.beta, &t.alpha})
      for (const auto& S : set->S)
        if (S.size() > static_cast<size_t>(mcd::kFastPodRank))
          return fail(c, MC_ERR_INPUT, "the FP32 POD form supports ranks up to " + std::to_string(mcd::kFastPodRank));
  }
  auto* d_fail = static_cast<unsigned long long*>(scratch(c, kTslFail, sizeof(unsigned long long)));
  if (!d_fail) return fail(c, MC_ERR_OOM, "sampler counters");
  CUDA_TRY(c, cudaMemsetAsync(d_fail, 0, sizeof(unsigned long long), c->stream));
  CUDA_TRY(c, mcd::launch_sample_tsl(c->dw.tsl + tsl, fast, philox ? 0 : 1, E, T, n, seed,
                                     run_key(seed, 0, 0x54534C00ull), beta, alpha, d_fail, c->stream));
  c->launches++;
  unsigned long long h = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&h, d_fail, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (failures) *failures = h;
  return MC_OK;
}

}  // namespace

extern "C" {

int mc_train_surrogate(mc_ctx* c, int32_t tsl, const mc_train_desc* desc, mc_train_out* out) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  if (!desc) return fail(c, MC_ERR_INPUT, "null argument");
  CUDA_TRY(c, cudaSetDevice(c->device));
  mc_train_desc d = *desc;
  if (!d.conditions) d.conditions = 8192;
  if (!d.samples_per_condition) d.samples_per_condition = 1024;
  if (!d.batch) d.batch = 8192;
  if (!d.steps) d.steps = 4000;
  if (!(d.lr > 0)) d.lr = 2e-3f;
  const uint32_t K = d.samples_per_condition;
  if (K < 2 || K > 1024 || (K & (K - 1))) return fail(c, MC_ERR_INPUT, "samples_per_condition: a power of two <= 1024");
  if (d.batch % 128 || d.batch > (1u << 20)) return fail(c, MC_ERR_INPUT, "batch: a multiple of 128 up to 2^20");
  const mc::TSLData& t = c->model.tsl[static_cast<size_t>(tsl)];
  if (!(d.E_min > 0 && d.E_min < d.E_max && d.E_max < t.cutoff_energy()))
    return fail(c, MC_ERR_INPUT, "energy box must lie inside (0, cutoff energy)");
  if (!(d.T_min > 0 && d.T_min < d.T_max)) return fail(c, MC_ERR_INPUT, "temperature box");
  mcd::MlpBox box;
  box.logE0 = std::log(d.E_min);
  box.logE1 = std::log(d.E_max);
  box.T0 = d.T_min;
  box.T1 = d.T_max;
  box.beta_cutoff = t.beta_cutoff;
  box.awr = t.awr;
  box.beta_scale = std::log1p(std::max(t.beta_cutoff, d.E_max / (mcd::kBoltzmann * d.T_min)));
  if (!mlp_net_alloc(c, c->mlp[0]) || !mlp_net_alloc(c, c->mlp[1]) || !mlp_batch_alloc(c, static_cast<int>(d.batch)))
    return fail(c, MC_ERR_OOM, "surrogate buffers");
  const uint64_t Nc = d.conditions, N = Nc * K;
  // data buffers (freed at the end)
  std::vector<void*> tmp;
  auto dalloc = [&](size_t bytes) -> void* {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
    tmp.push_back(p);
    return p;
  };
  auto release = [&]() {
    cudaStreamSynchronize(c->stream);
    for (void* p : tmp) cudaFree(p);
  };
  auto* Ec = static_cast<double*>(dalloc(Nc * 8));
  auto* Tc = static_cast<double*>(dalloc(Nc * 8));
  auto* bc = static_cast<double*>(dalloc(Nc * 8));
  auto* Ex = static_cast<double*>(dalloc(N * 8));
  auto* Tx = static_cast<double*>(dalloc(N * 8));
  auto* U = static_cast<double*>(dalloc(N * 8));
  auto* bx = static_cast<double*>(dalloc(N * 8));
  auto* sx = static_cast<double*>(dalloc(N * 8));
  auto* X = static_cast<__half*>(dalloc(N * mcd::kMlpIn * 2));
  auto* y = static_cast<float*>(dalloc(N * 4));
  auto* d_fail = static_cast<unsigned long long*>(dalloc(8));
  if (!(Ec && Tc && bc && Ex && Tx && U && bx && sx && X && y && d_fail)) {
    release();
    return fail(c, MC_ERR_OOM, "surrogate training data");
  }
  // conditions: E log-uniform, T uniform in the box
  std::vector<double> he(Nc), ht(Nc);
  uint64_t st = d.seed * 0x9E3779B97F4A7C15ull + 12345;
  for (uint64_t i = 0; i < Nc; i++) {
    st = mcd::splitmix64(st);
    const double a = (st >> 11) * (1.0 / 9007199254740992.0);
    st = mcd::splitmix64(st);
    const double b = (st >> 11) * (1.0 / 9007199254740992.0);
    he[i] = std::exp(box.logE0 + a * (box.logE1 - box.logE0));
    ht[i] = d.T_min + b * (d.T_max - d.T_min);
  }
  int rc = MC_OK;
  mc_train_out o{};
  double loss_b = 0, loss_a = 0;
  do {
    cudaError_t e;
#define TRY_CUDA(expr)                                                                    \
  if ((e = (expr)) != cudaSuccess) {                                                      \
    rc = fail(c, MC_ERR_DEVICE, std::string(#expr) + ": " + cudaGetErrorString(e));       \
    break;                                                                                \
  }
    TRY_CUDA(cudaEventRecord(c->ev0, c->stream));
    TRY_CUDA(cudaMemcpyAsync(Ec, he.data(), Nc * 8, cudaMemcpyHostToDevice, c->stream));
    TRY_CUDA(cudaMemcpyAsync(Tc, ht.data(), Nc * 8, cudaMemcpyHostToDevice, c->stream));
    TRY_CUDA(cudaMemsetAsync(d_fail, 0, 8, c->stream));
    TRY_CUDA(mcd::launch_expand(Ec, N, static_cast<int>(K), Ex, c->stream));
    TRY_CUDA(mcd::launch_expand(Tc, N, static_cast<int>(K), Tx, c->stream));
    TRY_CUDA(mcd::launch_quantile_u(U, N, static_cast<int>(K), c->stream));
    // beta network: sorted POD draws per condition
    TRY_CUDA(mcd::launch_tsl_beta_draws(c->dw.tsl + tsl, Ex, Tx, N, run_key(d.seed, 1, 0x4D4C4231ull), sx, d_fail,
                                        c->stream));
    TRY_CUDA(mcd::launch_segment_sort(sx, Nc, static_cast<int>(K), c->stream));
    TRY_CUDA(mcd::launch_mlp_features_beta(box, Ex, Tx, U, sx, N, X, y, c->stream));
    TRY_CUDA(cudaEventRecord(c->ev1, c->stream));
    TRY_CUDA(cudaEventSynchronize(c->ev1));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.data_ms += ms;
    TRY_CUDA(cudaEventRecord(c->ev0, c->stream));
    if ((rc = mlp_train(c, c->mlp[0], X, y, N, 7, d, run_key(d.seed, 2, 0x4D4C4231ull), &loss_b)) != MC_OK) break;
    TRY_CUDA(cudaEventRecord(c->ev1, c->stream));
    TRY_CUDA(cudaEventSynchronize(c->ev1));
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.train_ms += ms;
    // alpha network: one beta per condition, sorted alpha draws given it
    TRY_CUDA(cudaEventRecord(c->ev0, c->stream));
    TRY_CUDA(mcd::launch_tsl_beta_draws(c->dw.tsl + tsl, Ec, Tc, Nc, run_key(d.seed, 3, 0x4D4C4132ull), bc, d_fail,
                                        c->stream));
    TRY_CUDA(mcd::launch_expand(bc, N, static_cast<int>(K), bx, c->stream));
    TRY_CUDA(mcd::launch_tsl_alpha_draws(c->dw.tsl + tsl, Ex, Tx, bx, N, run_key(d.seed, 4, 0x4D4C4132ull), sx,
                                         d_fail, c->stream));
    TRY_CUDA(mcd::launch_segment_sort(sx, Nc, static_cast<int>(K), c->stream));
    TRY_CUDA(mcd::launch_mlp_features_alpha(box, Ex, Tx, bx, U, sx, N, X, y, c->stream));
    TRY_CUDA(cudaEventRecord(c->ev1, c->stream));
    TRY_CUDA(cudaEventSynchronize(c->ev1));
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.data_ms += ms;
    TRY_CUDA(cudaEventRecord(c->ev0, c->stream));
    if ((rc = mlp_train(c, c->mlp[1], X, y, N, 7, d, run_key(d.seed, 5, 0x4D4C4132ull), &loss_a)) != MC_OK) break;
    TRY_CUDA(cudaEventRecord(c->ev1, c->stream));
    TRY_CUDA(cudaEventSynchronize(c->ev1));
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.train_ms += ms;
    unsigned long long f = 0;
    TRY_CUDA(cudaMemcpy(&f, d_fail, 8, cudaMemcpyDeviceToHost));
    o.failures = f;
#undef TRY_CUDA
  } while (false);
  c->launches += 12;
  release();
  if (rc != MC_OK) return rc;
  c->mlp_box = box;
  c->mlp_tsl = tsl;
  o.loss_beta = loss_b;
  o.loss_alpha = loss_a;
  o.samples = N;
  if (out) *out = o;
  return MC_OK;
}

// The guide network of the guided sampler: rows from the FP32 POD sampler
// (per sample: (E, T) drawn in the box, SampleBeta, SampleAlpha's beta grid
// choice, then for both kinematic bounds the features and the grid position
// where find_cdf's bisection ends), then the same training loop as the
// surrogate networks.  desc->conditions * desc->samples_per_condition
// samples make twice as many rows.
int mc_train_surrogate_guide(mc_ctx* c, int32_t tsl, const mc_train_desc* desc, mc_train_out* out) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  if (!desc) return fail(c, MC_ERR_INPUT, "null argument");
  if (!c->tsl_fast_ok[static_cast<size_t>(tsl)])
    return fail(c, MC_ERR_INPUT, "the guided sampler needs the FP32 POD form (ranks up to 32)");
  CUDA_TRY(c, cudaSetDevice(c->device));
  mc_train_desc d = *desc;
  if (!d.conditions) d.conditions = 8192;
  if (!d.samples_per_condition) d.samples_per_condition = 256;
  if (!d.batch) d.batch = 8192;
  if (!d.steps) d.steps = 4000;
  if (!(d.lr > 0)) d.lr = 2e-3f;
  if (d.batch % 128 || d.batch > (1u << 20)) return fail(c, MC_ERR_INPUT, "batch: a multiple of 128 up to 2^20");
  const mc::TSLData& t = c->model.tsl[static_cast<size_t>(tsl)];
  if (!(d.E_min > 0 && d.E_min < d.E_max && d.E_max < t.cutoff_energy()))
    return fail(c, MC_ERR_INPUT, "energy box must lie inside (0, cutoff energy)");
  if (!(d.T_min > 0 && d.T_min < d.T_max)) return fail(c, MC_ERR_INPUT, "temperature box");
  mcd::MlpBox box;
  box.logE0 = std::log(d.E_min);
  box.logE1 = std::log(d.E_max);
  box.T0 = d.T_min;
  box.T1 = d.T_max;
  box.beta_cutoff = t.beta_cutoff;
  box.awr = t.awr;
  box.beta_scale = std::log1p(std::max(t.beta_cutoff, d.E_max / (mcd::kBoltzmann * d.T_min)));
  if (!mlp_net_alloc(c, c->guide) || !mlp_batch_alloc(c, static_cast<int>(d.batch)))
    return fail(c, MC_ERR_OOM, "guide network buffers");
  const uint64_t N = d.conditions * d.samples_per_condition, rows = 2 * N;
  __half* X = nullptr;
  float* y = nullptr;
  unsigned long long* d_fail = nullptr;
  if (cudaMalloc(&X, rows * mcd::kMlpIn * sizeof(__half)) != cudaSuccess ||
      cudaMalloc(&y, rows * sizeof(float)) != cudaSuccess || cudaMalloc(&d_fail, 8) != cudaSuccess) {
    cudaFree(X);
    cudaFree(y);
    cudaFree(d_fail);
    return fail(c, MC_ERR_OOM, "guide training data");
  }
  mc_train_out o{};
  double loss = 0;
  int rc = MC_OK;
  do {
    cudaError_t e;
    if ((e = cudaEventRecord(c->ev0, c->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(d_fail, 0, 8, c->stream)) != cudaSuccess ||
        (e = mcd::launch_guide_data(c->dw.tsl + tsl, box, run_key(d.seed, 1, 0x47554944ull), N, X, y, d_fail,
                                    c->stream)) != cudaSuccess ||
        (e = cudaEventRecord(c->ev1, c->stream)) != cudaSuccess || (e = cudaEventSynchronize(c->ev1)) != cudaSuccess) {
      rc = fail(c, MC_ERR_DEVICE, std::string("guide training data: ") + cudaGetErrorString(e));
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.data_ms = ms;
    CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    if ((rc = mlp_train(c, c->guide, X, y, rows, 7, d, run_key(d.seed, 2, 0x47554944ull), &loss)) != MC_OK) break;
    CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    CUDA_TRY(c, cudaEventSynchronize(c->ev1));
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    o.train_ms = ms;
    unsigned long long f = 0;
    CUDA_TRY(c, cudaMemcpy(&f, d_fail, 8, cudaMemcpyDeviceToHost));
    o.failures = f;
  } while (false);
  c->launches += 2;
  cudaStreamSynchronize(c->stream);
  cudaFree(X);
  cudaFree(y);
  cudaFree(d_fail);
  if (rc != MC_OK) return rc;
  c->guide_box = box;
  c->guide_tsl = tsl;
  o.loss_alpha = loss;  // the guide's loss (one network)
  o.samples = rows;
  if (out) *out = o;
  return MC_OK;
}

int mc_surrogate_get(mc_ctx* c, float* beta_params, float* alpha_params, mc_train_desc* box) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (c->mlp_tsl < 0) return fail(c, MC_ERR_STATE, "no trained surrogate");
  CUDA_TRY(c, cudaSetDevice(c->device));
  if (beta_params)
    CUDA_TRY(c, cudaMemcpy(beta_params, c->mlp[0].p, mcd::kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  if (alpha_params)
    CUDA_TRY(c, cudaMemcpy(alpha_params, c->mlp[1].p, mcd::kMlpParams * sizeof(float), cudaMemcpyDeviceToHost));
  if (box) {
    *box = mc_train_desc{};
    box->E_min = std::exp(c->mlp_box.logE0);
    box->E_max = std::exp(c->mlp_box.logE1);
    box->T_min = c->mlp_box.T0;
    box->T_max = c->mlp_box.T1;
  }
  return MC_OK;
}

int mc_surrogate_set(mc_ctx* c, int32_t tsl, const mc_train_desc* box, const float* beta_params,
                     const float* alpha_params) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  if (!box || !beta_params || !alpha_params) return fail(c, MC_ERR_INPUT, "null argument");
  if (!(box->E_min > 0 && box->E_min < box->E_max && box->T_min > 0 && box->T_min < box->T_max))
    return fail(c, MC_ERR_INPUT, "box");
  CUDA_TRY(c, cudaSetDevice(c->device));
  if (!mlp_net_alloc(c, c->mlp[0]) || !mlp_net_alloc(c, c->mlp[1])) return fail(c, MC_ERR_OOM, "surrogate buffers");
  const mc::TSLData& t = c->model.tsl[static_cast<size_t>(tsl)];
  mcd::MlpBox b;
  b.logE0 = std::log(box->E_min);
  b.logE1 = std::log(box->E_max);
  b.T0 = box->T_min;
  b.T1 = box->T_max;
  b.beta_cutoff = t.beta_cutoff;
  b.awr = t.awr;
  b.beta_scale = std::log1p(std::max(t.beta_cutoff, box->E_max / (mcd::kBoltzmann * box->T_min)));
  CUDA_TRY(c, cudaMemcpy(c->mlp[0].p, beta_params, mcd::kMlpParams * sizeof(float), cudaMemcpyHostToDevice));
  CUDA_TRY(c, cudaMemcpy(c->mlp[1].p, alpha_params, mcd::kMlpParams * sizeof(float), cudaMemcpyHostToDevice));
  CUDA_TRY(c, mcd::mlp_refresh_weights(c->mlp[0], c->stream));
  CUDA_TRY(c, mcd::mlp_refresh_weights(c->mlp[1], c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->mlp_box = b;
  c->mlp_tsl = tsl;
  return MC_OK;
}

int mc_surrogate_grad(mc_ctx* c, const float* params, const float* x, const float* y, uint64_t n, float* grad,
                      float* loss, float* out) {
  if (!c) return MC_ERR_STATE;
  if (!params || !x || !y || !grad) return fail(c, MC_ERR_INPUT, "null argument");
  if (n == 0 || n % 128 || n > (1u << 20)) return fail(c, MC_ERR_INPUT, "n: a multiple of 128 up to 2^20");
  CUDA_TRY(c, cudaSetDevice(c->device));
  if (!mlp_net_alloc(c, c->mlp_scratch) || !mlp_batch_alloc(c, static_cast<int>(n)))
    return fail(c, MC_ERR_OOM, "surrogate buffers");
  mcd::MlpBatch b = c->mlp_batch;
  b.B = static_cast<int>(n);
  // forward input in FP16, its transpose (weight gradients) in BF16
  std::vector<__half> hx(n * mcd::kMlpIn);
  std::vector<__nv_bfloat16> hxt(n * mcd::kMlpIn);
  for (uint64_t r = 0; r < n; r++)
    for (int f = 0; f < mcd::kMlpIn; f++) {
      hx[r * mcd::kMlpIn + f] = __float2half_rn(x[r * mcd::kMlpIn + f]);
      hxt[f * n + r] = __float2bfloat16_rn(__half2float(hx[r * mcd::kMlpIn + f]));
    }
  const mcd::MlpNet& net = c->mlp_scratch;
  CUDA_TRY(c, cudaMemcpyAsync(net.p, params, mcd::kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(b.X, hx.data(), hx.size() * 2, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(b.Xt, hxt.data(), hxt.size() * 2, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(b.y, y, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::mlp_refresh_weights(net, c->stream));
  CUDA_TRY(c, mcd::mlp_forward_backward(net, b, c->stream));
  c->launches += 10;
  CUDA_TRY(c, cudaMemcpyAsync(grad, net.g, mcd::kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  float hl = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&hl, b.loss, sizeof hl, cudaMemcpyDeviceToHost, c->stream));
  if (out) {
    float* d_out = reinterpret_cast<float*>(b.Z2);  // free after the backward pass
    CUDA_TRY(c, mcd::mlp_forward(net, b, d_out, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (loss) *loss = hl;
  return mlp_check(c);
}

int mc_sample_tsl_device(mc_ctx* c, int32_t tsl, const double* energy, const double* temperature, uint64_t n,
                         uint64_t seed, int32_t method, double* beta, double* alpha, uint64_t* failures) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (n == 0) return MC_OK;
  if (!energy || !temperature || !beta || !alpha) return fail(c, MC_ERR_INPUT, "null argument");
  CUDA_TRY(c, cudaSetDevice(c->device));
  return sample_tsl_device(c, tsl, energy, temperature, n, seed, method, beta, alpha, failures);
}

int mc_sample_tsl(mc_ctx* c, int32_t tsl, const double* energy, const double* temperature, uint64_t n, uint64_t seed,
                  int32_t method, double* beta, double* alpha, uint64_t* failures) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (n == 0) return MC_OK;
  if (!energy || !temperature || !beta || !alpha) return fail(c, MC_ERR_INPUT, "null argument");
  CUDA_TRY(c, cudaSetDevice(c->device));
  auto* buf = static_cast<double*>(scratch(c, kProbeIn, n * 32));
  if (!buf) return fail(c, MC_ERR_OOM, "sampler buffers");
  CUDA_TRY(c, cudaMemcpyAsync(buf, energy, n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(buf + n, temperature, n * 8, cudaMemcpyHostToDevice, c->stream));
  const int rc = sample_tsl_device(c, tsl, buf, buf + n, n, seed, method, buf + 2 * n, buf + 3 * n, failures);
  if (rc != MC_OK) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(beta, buf + 2 * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(alpha, buf + 3 * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_tsl_total(mc_ctx* c, int32_t tsl, const double* energy, const double* temperature, uint64_t n, double* xs) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  if (n == 0) return MC_OK;
  if (!energy || !temperature || !xs) return fail(c, MC_ERR_INPUT, "null argument");
  CUDA_TRY(c, cudaSetDevice(c->device));
  auto* buf = static_cast<double*>(scratch(c, kProbeIn, n * 24));
  if (!buf) return fail(c, MC_ERR_OOM, "buffers");
  CUDA_TRY(c, cudaMemcpyAsync(buf, energy, n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(buf + n, temperature, n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_tsl_total(c->dw.tsl + tsl, buf, buf + n, n, buf + 2 * n, c->stream));
  c->launches++;
  CUDA_TRY(c, cudaMemcpyAsync(xs, buf + 2 * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return MC_OK;
}

int mc_tsl_group_transfer(mc_ctx* c, int32_t tsl, const double* energy, const double* temperature, uint32_t rows,
                          uint64_t n, const double* bounds, uint32_t groups, uint64_t seed, int32_t method,
                          double* probs, uint64_t* failures) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (tsl < 0 || tsl >= c->dw.n_tsl) return fail(c, MC_ERR_INPUT, "thermal scattering library index out of range");
  if (rows == 0) return MC_OK;
  if (!energy || !temperature || !bounds || !probs) return fail(c, MC_ERR_INPUT, "null argument");
  if (groups < 1 || groups > static_cast<uint32_t>(mcd::kMaxTransferGroups))
    return fail(c, MC_ERR_INPUT, "groups must be 1.." + std::to_string(mcd::kMaxTransferGroups));
  if (n == 0 || n > (1ull << 26)) return fail(c, MC_ERR_INPUT, "samples per row must be 1..2^26");
  for (uint32_t g = 0; g < groups; g++)
    if (!(bounds[g] > bounds[g + 1])) return fail(c, MC_ERR_INPUT, "group boundaries must be descending");
  CUDA_TRY(c, cudaSetDevice(c->device));
  // rows per chunk: about 2^24 samples (E, T, beta, alpha: 512 MB) at a time
  const uint64_t per_chunk =
      std::max<uint64_t>(1, std::min<uint64_t>({static_cast<uint64_t>(rows), 65535ull, std::max<uint64_t>(1, (1ull << 24) / n)}));
  const size_t row_bytes = (2 * static_cast<size_t>(rows) + groups + 1) * 8 + static_cast<size_t>(rows) * groups * 8;
  auto* rb = static_cast<double*>(scratch(c, kGroupRows, row_bytes));
  auto* sb = static_cast<double*>(scratch(c, kGroupSamples, per_chunk * n * 32));
  if (!rb || !sb) return fail(c, MC_ERR_OOM, "thermal group transfer buffers");
  double* d_E = rb;
  double* d_T = rb + rows;
  double* d_bounds = rb + 2 * static_cast<size_t>(rows);
  auto* d_counts = reinterpret_cast<unsigned long long*>(d_bounds + groups + 1);
  CUDA_TRY(c, cudaMemcpyAsync(d_E, energy, rows * 8ull, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(d_T, temperature, rows * 8ull, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(d_bounds, bounds, (groups + 1) * 8ull, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(d_counts, 0, static_cast<size_t>(rows) * groups * 8, c->stream));
  uint64_t fails = 0;
  for (uint64_t r0 = 0, chunk = 0; r0 < rows; r0 += per_chunk, chunk++) {
    const unsigned nr = static_cast<unsigned>(std::min<uint64_t>(per_chunk, rows - r0));
    const uint64_t m = nr * n;
    double* E = sb;
    double* T = sb + m;
    double* beta = sb + 2 * m;
    double* alpha = sb + 3 * m;
    CUDA_TRY(c, mcd::launch_expand_rows(d_E + r0, d_T + r0, nr, n, E, T, c->stream));
    c->launches++;
    // every chunk its own streams
    uint64_t f = 0;
    const int rc = sample_tsl_device(c, tsl, E, T, m, seed ^ (chunk * 0x9E3779B97F4A7C15ull), method, beta, alpha, &f);
    if (rc != MC_OK) return rc;
    fails += f;
    CUDA_TRY(c, mcd::launch_group_bins(beta, nr, n, d_E + r0, d_T + r0, d_bounds, static_cast<int>(groups),
                                       d_counts + r0 * groups, c->stream));
    c->launches++;
  }
  std::vector<unsigned long long> counts(static_cast<size_t>(rows) * groups);
  CUDA_TRY(c, cudaMemcpyAsync(counts.data(), d_counts, counts.size() * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  for (uint32_t r = 0; r < rows; r++) {
    unsigned long long tot = 0;
    for (uint32_t g = 0; g < groups; g++) tot += counts[static_cast<size_t>(r) * groups + g];
    for (uint32_t g = 0; g < groups; g++)
      probs[static_cast<size_t>(r) * groups + g] =
          tot ? static_cast<double>(counts[static_cast<size_t>(r) * groups + g]) / static_cast<double>(tot) : 0.0;
  }
  if (failures) *failures = fails;
  return MC_OK;
}

int mc_pod_svd(mc_ctx* c, const double* A, uint64_t m, uint64_t n, double* U, double* S, double* V,
               uint32_t* sweeps) {
  if (!check_ctx(c, false)) return MC_ERR_STATE;
  if (!A || !U || !S || !V) return fail(c, MC_ERR_INPUT, "null argument");
  if (n == 0 || m < n) return fail(c, MC_ERR_INPUT, "mc_pod_svd: needs m >= n >= 1");
  if (n > (1u << 16) || m > (1ull << 31) || m * n > (1ull << 30))
    return fail(c, MC_ERR_INPUT, "mc_pod_svd: at most 2^16 columns, 2^31 rows and 2^30 entries");
  for (uint64_t k = 0; k < m * n; k++)
    if (!std::isfinite(A[k])) return fail(c, MC_ERR_INPUT, "mc_pod_svd: the matrix holds a non-finite value");
  CUDA_TRY(c, cudaSetDevice(c->device));
  auto* dA = static_cast<double*>(scratch(c, kPodA, m * n * 8));
  auto* dV = static_cast<double*>(scratch(c, kPodV, (n * n + n + 1) * 8));
  if (!dA || !dV) return fail(c, MC_ERR_OOM, "mc_pod_svd buffers");
  double* dS = dV + n * n;
  auto* d_rot = reinterpret_cast<unsigned*>(dS + n);
  const int mi = static_cast<int>(m), ni = static_cast<int>(n);
  CUDA_TRY(c, cudaMemcpyAsync(dA, A, m * n * 8, cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(c, mcd::launch_jacobi_init(dV, ni, c->stream));
  // a pair counts as orthogonal when |a_i . a_j| <= sqrt(m) eps |a_i| |a_j|
  const double tol = std::sqrt(static_cast<double>(m)) * 2.220446049250313e-16;
  constexpr uint32_t kMaxSweeps = 60;
  uint32_t done = 0;
  unsigned rot = 1;
  while (rot && done < kMaxSweeps) {
    CUDA_TRY(c, cudaMemsetAsync(d_rot, 0, sizeof(unsigned), c->stream));
    CUDA_TRY(c, mcd::launch_jacobi_sweep(dA, dV, mi, ni, tol, d_rot, c->stream));
    c->launches += static_cast<uint64_t>(ni + (ni & 1) - 1);
    CUDA_TRY(c, cudaMemcpyAsync(&rot, d_rot, sizeof rot, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    done++;
  }
  if (rot) return fail(c, MC_ERR_INPUT, "mc_pod_svd: no convergence in " + std::to_string(kMaxSweeps) + " sweeps");
  CUDA_TRY(c, mcd::launch_column_norms(dA, mi, ni, dS, c->stream));
  c->launches++;
  std::vector<double> hA(m * n), hV(n * n), hS(n);
  CUDA_TRY(c, cudaMemcpyAsync(hA.data(), dA, m * n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(hV.data(), dV, n * n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(hS.data(), dS, n * 8, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  // descending singular values (ties keep column order); U's columns
  // normalised, zero where the singular value is zero
  std::vector<uint64_t> order(n);
  for (uint64_t k = 0; k < n; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return hS[a] > hS[b]; });
  for (uint64_t k = 0; k < n; k++) {
    const uint64_t j = order[k];
    S[k] = hS[j];
    const double inv = hS[j] > 0.0 ? 1.0 / hS[j] : 0.0;
    for (uint64_t r = 0; r < m; r++) U[k * m + r] = hA[j * m + r] * inv;
    for (uint64_t r = 0; r < n; r++) V[k * n + r] = hV[j * n + r];
  }
  if (sweeps) *sweeps = done;
  return MC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Bank transport without allocation.
//
// Some callers cannot allocate device memory at the time they transport a
// bank: host applications that fix their device-memory budget at start-up
// and forbid allocation afterwards (for example a coupled multiphysics code
// whose own pool owns the GPU's memory), or code that runs where the device
// allocator must not be entered.  For them, mc_transport_bank_noalloc runs
// the same kernels as mc_transport_bank, but all of its scratch memory --
// run counters, fission records, per-history site slots, scan sums -- lives
// in the fixed array below, which every GPU that loads this library holds
// until the process exits.  The caller passes its own device buffers for the
// input sites and the output bank.  The call waits for its work before it
// returns: it reads the bank size and the run counters back to the host.

namespace {

constexpr uint64_t kNoAllocMaxHistories = 16384;  // sites per call
constexpr uint32_t kNoAllocMaxYield = 4;           // secondaries per fission
constexpr size_t kNoAllocCounters = 256;
constexpr size_t kNoAllocFission = kNoAllocMaxHistories * sizeof(mcd::FissionRec);
constexpr size_t kNoAllocSlots = kNoAllocMaxHistories * kNoAllocMaxYield * sizeof(Site);
constexpr size_t kNoAllocCount = kNoAllocMaxHistories * sizeof(uint32_t);
constexpr size_t kNoAllocOffsets = kNoAllocMaxHistories * sizeof(unsigned long long);
constexpr size_t kNoAllocSums = 64 * sizeof(unsigned long long);  // scan block sums + total
constexpr size_t kNoAllocBytes =
    kNoAllocCounters + kNoAllocFission + kNoAllocSlots + kNoAllocCount + kNoAllocOffsets + kNoAllocSums;  // 5.3 MB

static_assert(sizeof(DevCounters) <= kNoAllocCounters, "counter block");
static_assert(kNoAllocFission % 256 == 0 && kNoAllocSlots % 256 == 0 && kNoAllocCount % 256 == 0 &&
                  kNoAllocOffsets % 256 == 0,
              "sub-buffers keep 256-byte alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// device address of g_noalloc_scratch for each device, found once under the
// mutex (two host threads may make their first call on a device together)
constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};
std::mutex g_noalloc_mutex;

// the caller's buffer as a device address: device or managed memory as is,
// page-locked host memory through its device mapping; anything else
// (pageable host memory) is refused
bool device_view(const void* p, void** out) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
    *out = a.devicePointer ? a.devicePointer : const_cast<void*>(p);
    return true;
  }
  if (a.type == cudaMemoryTypeHost && a.devicePointer) {
    *out = a.devicePointer;
    return true;
  }
  return false;
}

}  // namespace

extern "C" int mc_transport_bank_noalloc(mc_ctx* c, const mc_site* d_sites, uint64_t n, const mc_run_opts* o,
                                         mc_site* d_fission_sites, uint64_t cap, uint64_t* n_out) {
  if (!check_ctx(c)) return MC_ERR_STATE;
  if (n_out) *n_out = 0;
  if (n == 0) return MC_OK;
  if (!d_sites) return fail(c, MC_ERR_INPUT, "sites is NULL");
  if (n > kNoAllocMaxHistories)
    return fail(c, MC_ERR_INPUT, "mc_transport_bank_noalloc: " + std::to_string(n) + " sites exceed the limit of " +
                                     std::to_string(kNoAllocMaxHistories) + " per call");
  if (c->max_yield > kNoAllocMaxYield)
    return fail(c, MC_ERR_INPUT, "mc_transport_bank_noalloc: up to " + std::to_string(kNoAllocMaxYield - 1) +
                                     " mean secondaries per fission are supported (this problem allows " +
                                     std::to_string(c->max_yield - 1) + ")");
  if (c->model.energy_mode != mc::kMultigroup)
    return fail(c, MC_ERR_INPUT, "mc_transport_bank_noalloc: multigroup problems only");
  const int rng = o ? o->rng : MC_RNG_PHILOX;
  if (rng != MC_RNG_PHILOX && rng != MC_RNG_MINSTD) return fail(c, MC_ERR_INPUT, "unknown rng mode");
  if (c->device < 0 || c->device >= kMaxDevices) return fail(c, MC_ERR_INPUT, "device index out of range");
  CUDA_TRY(c, cudaSetDevice(c->device));
  // a dense-score commit that an earlier call left on the side stream
  // must be ordered before this call's tally updates
  if (join_side(c) != MC_OK) return MC_ERR_DEVICE;
  void* in_dev = nullptr;
  void* out_dev = nullptr;
  if (!device_view(d_sites, &in_dev))
    return fail(c, MC_ERR_INPUT, "mc_transport_bank_noalloc: sites is not device or page-locked memory");
  if (d_fission_sites && cap && !device_view(d_fission_sites, &out_dev))
    return fail(c, MC_ERR_INPUT, "mc_transport_bank_noalloc: fission_sites is not device or page-locked memory");
  // set-up, once per device with that device current: the host-side symbol
  // is not a device address, so ask the runtime for the array's address
  char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[c->device]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return fail(c, MC_ERR_DEVICE,
                    std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
      g_noalloc_addr[c->device] = p;
    }
    base = static_cast<char*>(g_noalloc_addr[c->device]);
  }
  auto* ctr = reinterpret_cast<DevCounters*>(base);
  auto* fis = reinterpret_cast<mcd::FissionRec*>(base + kNoAllocCounters);
  auto* slots = reinterpret_cast<Site*>(base + kNoAllocCounters + kNoAllocFission);
  auto* count = reinterpret_cast<uint32_t*>(base + kNoAllocCounters + kNoAllocFission + kNoAllocSlots);
  auto* offsets =
      reinterpret_cast<unsigned long long*>(base + kNoAllocCounters + kNoAllocFission + kNoAllocSlots + kNoAllocCount);
  auto* sums = reinterpret_cast<unsigned long long*>(base + kNoAllocCounters + kNoAllocFission + kNoAllocSlots +
                                                     kNoAllocCount + kNoAllocOffsets);
  auto* total = sums + 48;  // after at most 16 block sums

  // the array keeps the previous call's contents: the counters must start
  // at zero; fission records and counts are rewritten for every history
  CUDA_TRY(c, cudaMemsetAsync(ctr, 0, sizeof(DevCounters), c->stream));
  RunParams rp{};
  rp.n = n;
  rp.seed = c->model.seed;
  rp.run_key = run_key(c->model.seed, 0, 0x42414e4bull);
  rp.max_events = o && o->max_events ? o->max_events : 1000000u;
  rp.keig = 1;
  rp.score = 1;
  rp.fast = (o && o->fast_math && rng == MC_RNG_PHILOX) ? 1 : 0;
  rp.from_bank = 1;
  rp.minstd_base = 0;
  rp.max_yield = kNoAllocMaxYield;
  rp.src = static_cast<const Site*>(in_dev);
  rp.bank = slots;
  rp.bank_count = count;
  rp.ctr = ctr;
  rp.tally_sum = c->d_sum;
  rp.tally_sq = c->d_sq;
  rp.total_bins = c->total_bins;
  rp.nb = 0;  // scores go through the per-history list, no dense array
  rp.pend = nullptr;
  rp.fis = fis;
  const int block = pick_block(o);
  const int grid = grid_for(c, c->model.energy_mode, rng, block, true, rp.fast != 0);
  CUDA_TRY(c, mcd::launch_history_mg(c->dw, rp, rng, grid, block, c->stream, c->variant));
  CUDA_TRY(c, mcd::launch_fission_sites_mg(c->dw, rp, rng, sites_grid(rp.n), c->stream));
  CUDA_TRY(c, mcd::launch_bank_scan(count, n, offsets, sums, total, c->stream));
  if (out_dev) {
    k_compact_capped<<<static_cast<unsigned>((n + 255) / 256), 256, 0, c->stream>>>(
        slots, count, offsets, n, kNoAllocMaxYield, static_cast<Site*>(out_dev), cap);
    CUDA_TRY(c, cudaGetLastError());
  }
  c->launches += 6;
  unsigned long long m = 0;
  DevCounters h{};
  CUDA_TRY(c, cudaMemcpyAsync(&m, total, sizeof m, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemcpyAsync(&h, ctr, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  if (n_out) *n_out = m;
  if (m > cap) return fail(c, MC_ERR_OVERFLOW, "fission bank larger than the output capacity");
  return counters_status(c, h);
}

// ---------------------------------------------------------------------------
// Batched problems (layout and device bookkeeping in mc_batch.cu).  Each
// problem is loaded into its own context (world tables on the device); the
// batch uploads their DevWorld descriptors and run parameters as arrays.

struct mc_batch {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  std::vector<mc_ctx*> probs;
  std::vector<uint64_t> hist, seeds;
};

namespace {

int bfail(mc_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define BATCH_TRY(b, expr)                                                                            \
  do {                                                                                                \
    const cudaError_t e_ = (expr);                                                                    \
    if (e_ != cudaSuccess) return bfail((b), MC_ERR_DEVICE, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// device allocations of one mc_batch_run, freed on every exit path
struct BatchMem {
  std::vector<void*> ptrs;
  ~BatchMem() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
};

// CTAs of the transport grid, proportional to each problem's histories
// (at least one each); block_problem[b] and block_first[p]
void batch_blocks(const std::vector<uint64_t>& hist, int grid_target, std::vector<uint32_t>& block_problem,
                  std::vector<uint32_t>& block_first) {
  uint64_t N = 0;
  for (uint64_t h : hist) N += h;
  block_problem.clear();
  block_first.assign(1, 0);
  for (size_t p = 0; p < hist.size(); p++) {
    const double share = static_cast<double>(grid_target) * static_cast<double>(hist[p]) / static_cast<double>(N);
    const uint64_t need = (hist[p] + 255) / 256;  // no more CTAs than 256-history chunks
    const uint32_t nb = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(need, static_cast<uint64_t>(share + 0.5))));
    for (uint32_t i = 0; i < nb; i++) block_problem.push_back(static_cast<uint32_t>(p));
    block_first.push_back(static_cast<uint32_t>(block_problem.size()));
  }
}

}  // namespace

extern "C" {

int mc_batch_create(mc_batch** out, int device) {
  if (!out) return MC_ERR_INPUT;
  *out = nullptr;
  auto* b = new (std::nothrow) mc_batch();
  if (!b) return MC_ERR_OOM;
  b->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return MC_ERR_DEVICE;
  }
  b->own_stream = true;
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, device);
  *out = b;
  return MC_OK;
}

void mc_batch_destroy(mc_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (mc_ctx* c : b->probs) mc_destroy(c);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int mc_batch_set_stream(mc_batch* b, void* s) {
  if (!b) return MC_ERR_INPUT;
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  b->own_stream = false;
  b->stream = static_cast<cudaStream_t>(s);
  return MC_OK;
}

int mc_batch_last_error(mc_batch* b, char* buf, size_t n) {
  if (!b || !buf || n == 0) return MC_ERR_INPUT;
  std::strncpy(buf, b->err.c_str(), n - 1);
  buf[n - 1] = 0;
  return MC_OK;
}

int mc_batch_add(mc_batch* b, const char* xml_text, const char* base_dir, uint64_t histories, uint64_t seed) {
  if (!b || !xml_text) return MC_ERR_INPUT;
  mc_ctx* c = nullptr;
  int rc = mc_create(&c, b->device);
  if (rc != MC_OK) return bfail(b, rc, "context creation failed");
  rc = mc_load_xml(c, xml_text, base_dir);
  if (rc != MC_OK) {
    b->err = c->err;
    mc_destroy(c);
    return rc;
  }
  if (c->model.energy_mode != mc::kMultigroup) {
    mc_destroy(c);
    return bfail(b, MC_ERR_INPUT, "batched problems are multigroup");
  }
  const uint64_t h = histories ? histories : c->model.histories;
  if (h == 0) {
    mc_destroy(c);
    return bfail(b, MC_ERR_INPUT, "no histories");
  }
  b->probs.push_back(c);
  b->hist.push_back(h);
  b->seeds.push_back(seed ? seed : c->model.seed);
  return static_cast<int>(b->probs.size() - 1);
}

int mc_batch_run(mc_batch* b, const mc_batch_opts* o, mc_batch_out* out) {
  if (!b || !o) return MC_ERR_INPUT;
  if (b->probs.empty()) return bfail(b, MC_ERR_STATE, "no problems added");
  const uint32_t cycles = o->inactive + o->active;
  if (cycles == 0) return bfail(b, MC_ERR_INPUT, "no cycles");
  BATCH_TRY(b, cudaSetDevice(b->device));
  const int P = static_cast<int>(b->probs.size());
  std::vector<unsigned long long> off(P + 1, 0);
  for (int p = 0; p < P; p++) off[p + 1] = off[p] + b->hist[p];
  const unsigned long long N = off[P];
  uint32_t max_yield = 1;
  for (mc_ctx* c : b->probs) max_yield = std::max(max_yield, c->max_yield);
  // fission sites straight into the bank when every problem's counts are
  // known before sampling (bank_direct) and a CTA's sites fit its stage
  if (o->bank_path < MC_BANK_AUTO || o->bank_path > MC_BANK_DIRECT)
    return bfail(b, MC_ERR_INPUT, "unknown bank path");
  bool direct = o->bank_path != MC_BANK_SLOTS && mcd::sites_out_fits(max_yield);
  for (mc_ctx* c : b->probs) direct = direct && bank_direct(c, MC_RNG_PHILOX, o->fast_math != 0, MC_BANK_AUTO) > 0;
  if (o->bank_path == MC_BANK_DIRECT && !direct)
    return bfail(b, MC_ERR_INPUT, "the direct bank path needs chi cdfs that end above every threshold the stream draws");
  if (direct) BATCH_TRY(b, mcd::sites_out_batch_prepare(max_yield));
  BatchMem mem;
  auto* d_worlds = mem.get<DevWorld>(P);
  auto* d_rps = mem.get<RunParams>(P);
  auto* d_ctr = mem.get<DevCounters>(P);
  auto* d_off = mem.get<unsigned long long>(P + 1);
  auto* d_seeds = mem.get<unsigned long long>(P);
  auto* d_start = mem.get<unsigned long long>(P);
  auto* d_M = mem.get<unsigned long long>(P);
  auto* d_k = mem.get<double>(static_cast<size_t>(P) * cycles);
  auto* d_stats = mem.get<unsigned long long>(4 * static_cast<size_t>(P));
  auto* d_cycle = mem.get<uint32_t>(1);
  auto* d_died = mem.get<int>(1);
  auto* src0 = mem.get<Site>(N);
  auto* src1 = mem.get<Site>(N);
  auto* fis = mem.get<mcd::FissionRec>(N);
  auto* slots = direct ? nullptr : mem.get<Site>(N * max_yield);
  auto* count = mem.get<uint32_t>(N);
  auto* offsets = mem.get<unsigned long long>(N);
  auto* sums = mem.get<unsigned long long>((N + 1023) / 1024 + 1);
  auto* total = mem.get<unsigned long long>(1);
  auto* bank = mem.get<Site>(N * max_yield);
  if (!(d_worlds && d_rps && d_ctr && d_off && d_seeds && d_start && d_M && d_k && d_stats && d_cycle && d_died &&
        src0 && src1 && fis && (direct || slots) && count && offsets && sums && total && bank))
    return bfail(b, MC_ERR_OOM, "batch buffers");
  std::vector<DevWorld> worlds(P);
  std::vector<RunParams> rps(P);
  for (int p = 0; p < P; p++) {
    mc_ctx* c = b->probs[p];
    worlds[p] = c->dw;
    RunParams& rp = rps[p];
    rp = RunParams{};
    rp.n = b->hist[p];
    rp.seed = b->seeds[p];
    rp.max_events = o->max_events ? o->max_events : 1000000u;
    rp.keig = 1;
    rp.score = 0;
    rp.fast = o->fast_math ? 1 : 0;
    rp.max_yield = max_yield;
    rp.bank = direct ? nullptr : slots + off[p] * max_yield;
    rp.bank_count = count + off[p];
    rp.total_bins = 0;
    rp.ctr = d_ctr + p;
    rp.fis = fis + off[p];
  }
  cudaStream_t s = b->stream;
  BATCH_TRY(b, cudaMemcpyAsync(d_worlds, worlds.data(), P * sizeof(DevWorld), cudaMemcpyHostToDevice, s));
  BATCH_TRY(b, cudaMemcpyAsync(d_rps, rps.data(), P * sizeof(RunParams), cudaMemcpyHostToDevice, s));
  BATCH_TRY(b, cudaMemcpyAsync(d_off, off.data(), (P + 1) * 8, cudaMemcpyHostToDevice, s));
  BATCH_TRY(b, cudaMemcpyAsync(d_seeds, b->seeds.data(), P * 8, cudaMemcpyHostToDevice, s));
  BATCH_TRY(b, cudaMemsetAsync(d_stats, 0, 4 * P * 8, s));
  BATCH_TRY(b, cudaMemsetAsync(d_cycle, 0, 4, s));
  BATCH_TRY(b, cudaMemsetAsync(d_died, 0, 4, s));
  mcd::BatchCycle bc{P, static_cast<int>(cycles), N, d_off, d_seeds, d_rps, d_ctr, d_start, d_M, d_k, d_stats,
                     d_cycle, d_died};
  mc_batch_out res{};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  struct EvGuard {
    cudaEvent_t a, b;
    ~EvGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } evg{e0, e1};
  // block tables per variant; autotune on cycle 0's transport
  std::vector<uint32_t> bp, bf;
  auto* d_bp = mem.get<uint32_t>(static_cast<size_t>(b->num_sms) * 8 + P);
  auto* d_bf = mem.get<uint32_t>(P + 1);
  if (!d_bp || !d_bf) return bfail(b, MC_ERR_OOM, "batch block tables");
  auto set_blocks = [&](int v) -> int {
    const int per_sm = std::max(1, std::min(8, mcd::history_batch_blocks_per_sm(v)));
    batch_blocks(b->hist, per_sm * b->num_sms, bp, bf);
    BATCH_TRY(b, cudaMemcpyAsync(d_bp, bp.data(), bp.size() * 4, cudaMemcpyHostToDevice, s));
    BATCH_TRY(b, cudaMemcpyAsync(d_bf, bf.data(), bf.size() * 4, cudaMemcpyHostToDevice, s));
    return MC_OK;
  };
  int variant = o->variant > 0 ? std::min(o->variant - 1, mcd::history_variants() - 1) : -1;
  if (variant < 0) {
    double best = 1e300;
    for (int v = 0; v < mcd::history_variants() && v < 8; v++) {
      int rc = set_blocks(v);
      if (rc != MC_OK) return rc;
      BATCH_TRY(b, mcd::launch_batch_begin(bc, src0, s));
      BATCH_TRY(b, cudaEventRecord(e0, s));
      BATCH_TRY(b, mcd::launch_history_mg_batch(d_worlds, d_rps, d_bp, static_cast<int>(bp.size()), P, s, v));
      BATCH_TRY(b, cudaEventRecord(e1, s));
      BATCH_TRY(b, cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      res.tune_ms[v] = ms;
      res.launches += 2;
      if (ms < best) {
        best = ms;
        variant = v;
      }
    }
  }
  {
    const int rc = set_blocks(variant);
    if (rc != MC_OK) return rc;
  }
  const int grid = static_cast<int>(bp.size());
  // the direct path's count kernel sees the concatenated records as one run
  // (max_yield bounds every problem's yield, so no count is cut)
  RunParams all{};
  all.n = N;
  all.fis = fis;
  all.bank_count = count;
  all.max_yield = max_yield;
  all.ctr = d_ctr;
  // one cycle's launches; `from` holds this cycle's sources, `to` the next
  auto cycle_launches = [&](const Site* from, Site* to) -> cudaError_t {
    cudaError_t e;
    if ((e = mcd::launch_batch_begin(bc, from, s)) != cudaSuccess) return e;
    if ((e = mcd::launch_history_mg_batch(d_worlds, d_rps, d_bp, grid, P, s, variant)) != cudaSuccess) return e;
    if (direct) {
      if ((e = mcd::launch_direct_bank_scan(all, offsets, sums, total, s)) != cudaSuccess) return e;
      if ((e = mcd::launch_fission_sites_out_mg_batch(d_worlds, d_rps, d_off, P, N, max_yield, o->fast_math != 0,
                                                      fis, count, offsets, total, bank, s)) != cudaSuccess)
        return e;
    }
    else {
      if ((e = mcd::launch_fission_sites_mg_batch(d_worlds, d_rps, d_bp, d_bf, grid, s)) != cudaSuccess) return e;
      if ((e = mcd::launch_bank_scan(count, N, offsets, sums, total, s)) != cudaSuccess) return e;
      if ((e = mcd::launch_bank_compact(slots, count, offsets, N, max_yield, bank, s)) != cudaSuccess) return e;
    }
    if ((e = mcd::launch_batch_tally(bc, offsets, total, s)) != cudaSuccess) return e;
    return mcd::launch_batch_resample(bc, bank, to, s);
  };
  const int kLaunchesPerCycle = direct ? 9 : 10;  // begin, transport, bank (4 or 5), tally, resample (2)
  BATCH_TRY(b, cudaMemsetAsync(d_cycle, 0, 4, s));
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  struct GraphGuard {
    cudaGraphExec_t* e;
    ~GraphGuard() {
      for (int i = 0; i < 2; i++)
        if (e[i]) cudaGraphExecDestroy(e[i]);
    }
  } gg{exec};
  const bool graph = !o->no_graph;
  if (graph) {
    for (int parity = 0; parity < 2; parity++) {
      cudaGraph_t g = nullptr;
      BATCH_TRY(b, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const cudaError_t ce = parity == 0 ? cycle_launches(src0, src1) : cycle_launches(src1, src0);
      const cudaError_t ee = cudaStreamEndCapture(s, &g);
      if (ce != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(b, MC_ERR_DEVICE, std::string("graph capture: ") + cudaGetErrorString(ce != cudaSuccess ? ce : ee));
      }
      const cudaError_t ie = cudaGraphInstantiate(&exec[parity], g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return bfail(b, MC_ERR_DEVICE, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    }
  }
  cudaEvent_t em;  // start of the active cycles
  BATCH_TRY(b, cudaEventCreate(&em));
  struct EvGuard1 {
    cudaEvent_t e;
    ~EvGuard1() { cudaEventDestroy(e); }
  } evm{em};
  BATCH_TRY(b, cudaEventRecord(e0, s));
  for (uint32_t cyc = 0; cyc < cycles; cyc++) {
    if (cyc == o->inactive) BATCH_TRY(b, cudaEventRecord(em, s));
    if (graph) {
      BATCH_TRY(b, cudaGraphLaunch(exec[cyc & 1], s));
      res.launches += 1;
    }
    else {
      BATCH_TRY(b, (cyc & 1) ? cycle_launches(src1, src0) : cycle_launches(src0, src1));
      res.launches += kLaunchesPerCycle;
    }
  }
  BATCH_TRY(b, cudaEventRecord(e1, s));
  BATCH_TRY(b, cudaEventSynchronize(e1));
  float ms = 0, ms_active = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (o->active > 0) cudaEventElapsedTime(&ms_active, em, e1);
  std::vector<double> k(static_cast<size_t>(P) * cycles);
  std::vector<unsigned long long> stats(4 * static_cast<size_t>(P));
  int died = 0;
  BATCH_TRY(b, cudaMemcpy(k.data(), d_k, k.size() * 8, cudaMemcpyDeviceToHost));
  BATCH_TRY(b, cudaMemcpy(stats.data(), d_stats, stats.size() * 8, cudaMemcpyDeviceToHost));
  BATCH_TRY(b, cudaMemcpy(&died, d_died, 4, cudaMemcpyDeviceToHost));
  res.transport_ms = ms;
  res.active_ms = ms_active;
  res.histories = N * cycles;
  res.variant = variant;
  res.graph = graph ? 1 : 0;
  for (int p = 0; p < P; p++) {
    res.events += stats[4 * p];
    res.lost += stats[4 * p + 1];
    res.capped += stats[4 * p + 2];
    res.overflow += stats[4 * p + 3];
  }
  if (out) {
    double* kc = out->k_cycle;
    double* km = out->k_mean;
    double* ks = out->k_std;
    *out = res;
    out->k_cycle = kc;
    out->k_mean = km;
    out->k_std = ks;
    if (kc) std::copy(k.begin(), k.end(), kc);
    for (int p = 0; p < P; p++) {
      double sm = 0, s2 = 0;
      for (uint32_t c = o->inactive; c < cycles; c++) {
        const double v = k[static_cast<size_t>(p) * cycles + c];
        sm += v;
        s2 += v * v;
      }
      const double na = o->active;
      if (km) km[p] = na ? sm / na : 0;
      if (ks) ks[p] = na > 1 ? std::sqrt(std::max(0.0, (s2 - sm * sm / na) / (na - 1)) / na) : 0;
    }
  }
  if (died) return bfail(b, MC_ERR_INPUT, "a problem's fission bank is empty: its source died out");
  if (res.lost) return bfail(b, MC_ERR_LOST, std::to_string(res.lost) + " particles lost");
  if (res.overflow) return bfail(b, MC_ERR_OVERFLOW, std::to_string(res.overflow) + " bank overflows");
  if (res.capped) return bfail(b, MC_ERR_EVENT_CAP, std::to_string(res.capped) + " particles reached the event cap");
  return MC_OK;
}

}  // extern "C"
