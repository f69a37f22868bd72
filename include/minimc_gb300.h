/*
 * minimc_gb300 — C ABI of the GB300 particle-history engine.
 *
 * The reference (minimc v0.5.1) has no FFI layer.  Its extension points are
 * C++ abstract classes, and the per-particle transport call
 *
 *     Bank TransportMethod::Transport(Particle&, EstimatorSetProxy&,
 *                                     const World&) const noexcept
 *     (src/TransportMethod.hpp:42-43)
 *
 * cannot be batched, so this library drops in one level up, where
 * Driver::Solve() (src/Driver.hpp:30) runs every history.  Each entry point
 * below names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns MC_OK (0) or a negative MC_ERR_* code; no C++
 *     exception crosses this boundary.  mc_last_error() returns the message,
 *     which uses the reference's exception text where the reference has one.
 *   - One mc_ctx per host thread.  A context owns all device memory it uses;
 *     calls are ordered on the context's stream and synchronous on return
 *     unless stated otherwise.
 *   - Host pointers are plain arrays; nothing here takes or returns a torch
 *     type.  Lengths are element counts.
 *   - Groups are numbered 1..G with 1 the fastest group, as in the reference
 *     (src/BasicTypes.hpp:17-21).  Energies are in MeV.
 */
#ifndef MINIMC_GB300_H
#define MINIMC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MC_OK 0
#define MC_ERR_INPUT (-1)      /* bad problem input or argument           */
#define MC_ERR_OOM (-2)        /* device allocation failed                */
#define MC_ERR_DEVICE (-3)     /* CUDA runtime error                      */
#define MC_ERR_TIMEOUT (-4)    /* a bounded device wait ran out           */
#define MC_ERR_LOST (-5)       /* a particle left every cell              */
#define MC_ERR_RESAMPLE (-6)   /* thermal-scattering resample limit hit   */
#define MC_ERR_STATE (-7)      /* call out of order (e.g. no problem)     */
#define MC_ERR_OVERFLOW (-8)   /* bank, stack or per-history tally full   */
#define MC_ERR_EVENT_CAP (-9)  /* a particle reached the event cap        */

/* ---- options ------------------------------------------------------------ */
/* Random-number streams.
 * MC_RNG_PHILOX: counter-based Philox4x32-10 stream per history (default).
 * MC_RNG_MINSTD: the reference's own streams: std::minstd_rand per particle,
 *   seeded exactly as src/Source.cpp:143-154 and src/Particle.cpp:96-100 do,
 *   consumed through the C++ standard's generate_canonical, so a history
 *   follows the same random walk as the reference's. */
#define MC_RNG_PHILOX 0
#define MC_RNG_MINSTD 1
/* Thermal scattering in fixed-source transport: the POD sampler inside the
 * history kernel, or the trained MLP surrogate (mc_train_surrogate) run as a
 * batched tensor-core launch over a queue of the particles that reach a
 * thermal scatter of its library inside its trained (E, T) box (Philox
 * streams, continuous energy); outside the box the POD sampler serves. */
#define MC_THERMAL_POD 0
#define MC_THERMAL_SURROGATE 1
/* The guided sampler on the same queue: the trained guide network
 * (mc_train_surrogate_guide) predicts where SampleAlpha's CDF search ends,
 * the POD reconstructions confirm it, so every thermal scatter draws exactly
 * the POD sampler's (beta, alpha) from the particle's own stream -- its FP32
 * form with fast_math, its exact FP64 form without -- and the transport
 * gives the same histories as MC_THERMAL_POD, for less work (Philox
 * streams, continuous energy). */
#define MC_THERMAL_GUIDED 2
/* The POD sampler run as a batched launch over the same queue, without the
 * network (the guided form's ablation; same histories). */
#define MC_THERMAL_POD_QUEUE 3

/* How the event loop is scheduled on the device. */
#define MC_SCHEDULE_AUTO 0     /* autotuner's choice                      */
#define MC_SCHEDULE_HISTORY 1  /* fused kernel, one history per thread,
                                  dead lanes refilled from the queue      */
#define MC_SCHEDULE_EVENT 2    /* event kernels over compacted queues     */

/* How k-eigenvalue fission sites reach the compacted bank.  Both paths give
 * the same bank, site for site. */
#define MC_BANK_AUTO 0    /* direct where it applies, else slots          */
#define MC_BANK_SLOTS 1   /* per-history slots, a scan, then a compaction */
#define MC_BANK_DIRECT 2  /* counts known before sampling (continuous
                             energy always; multigroup with Philox streams
                             and every chi cdf ending above the largest
                             uniform drawn): a scan, then the sites sampled
                             straight into their bank positions;
                             MC_ERR_INPUT where that does not hold        */

typedef struct mc_ctx mc_ctx;

typedef struct {
  uint64_t histories;   /* 0: the problem's <histories>                  */
  uint64_t seed;        /* 0: the problem's <seed> (default 1)           */
  uint32_t inactive;    /* k-eigenvalue: 0 and active==0 -> from problem */
  uint32_t active;
  int32_t rng;          /* MC_RNG_*                                      */
  int32_t schedule;     /* MC_SCHEDULE_*                                 */
  uint32_t max_events;  /* per-particle event cap; 0 -> 1000000          */
  int32_t block_size;   /* 0 -> autotuned                                */
  int32_t fast_math;    /* 1: FP32 sampling arithmetic (Philox only);
                           geometry and positions stay FP64            */
  int32_t variant;      /* history-kernel variant + 1; 0 -> autotuned   */
  int32_t thermal;      /* MC_THERMAL_*: thermal scattering sampler      */
  int32_t bank_path;    /* MC_BANK_*: k-eigenvalue fission-site path     */
  uint32_t queue_sort_min; /* event schedule: sort a step's collision queue
                           by (type, material, group) when it holds at
                           least this many particles; 0 -> the value the
                           autotuner chose (never before it has run);
                           0xFFFFFFFF -> never                          */
  int32_t reserved[3];
} mc_run_opts;

/* A particle in a bank: the state that Bank/Particle carry between
 * Transport calls (src/Particle.hpp:104-131).  64 bytes. */
typedef struct {
  double x, y, z;   /* position, cm                                      */
  double u, v, w;   /* direction cosines                                 */
  double energy;    /* MeV, or the group number for multigroup problems  */
  uint64_t key;     /* RNG seed (minstd) or stream key (Philox)          */
} mc_site;

typedef struct {
  int32_t problem;      /* 0 fixed source, 1 k-eigenvalue                */
  int32_t energy_mode;  /* 0 multigroup, 1 continuous energy             */
  int32_t tracking;     /* 0 surface, 1 cell delta                       */
  int32_t n_cells, n_surfaces, n_materials, n_nuclides;
  int32_t groups;
  int32_t n_estimators;
  int32_t n_tsl;
  uint64_t histories, seed;
  uint32_t inactive, active;
  uint64_t total_bins;  /* estimator and sensitivity bins               */
  uint32_t max_yield;   /* upper bound on secondaries per fission       */
  int32_t n_perturbations;  /* total cross-section perturbations (<= 4) */
  int32_t reserved[6];
} mc_problem_info;

/* An estimator's bins, then those of each of its sensitivity estimators
 * (Estimator::sensitivities, src/Estimator.cpp:76-90; same bins,
 * src/Scorable.cpp:22-29): sensitivity k scores into
 * [offset + n_bins * (k + 1), offset + n_bins * (k + 2)). */
typedef struct {
  char name[64];
  int32_t kind;         /* 0 current, 1 track length                    */
  int32_t target;       /* surface (current) or cell (track length)     */
  uint64_t offset;      /* first bin in the flattened tally arrays      */
  uint64_t n_bins;
  uint64_t cosine_bins, energy_bins;
  int32_t n_sensitivities;  /* <= 4                                      */
  int32_t sensitivity[4];   /* perturbation index of each sensitivity    */
  int32_t reserved;
} mc_estimator_info;

/* Per-run results.  sum/sum_sq are caller-owned host arrays of
 * mc_problem_info.total_bins doubles (may be NULL).  They receive, per bin,
 * the sum over histories of each history's score and of its square, which is
 * what Scorable keeps (src/Scorable.cpp:101-106). */
typedef struct {
  double* sum;
  double* sum_sq;
  uint32_t* history_events;  /* optional [histories]: events per history   */
  int8_t* history_fate;      /* optional [histories]: last event of the
                                source particle (Particle::Event order)   */
  uint64_t histories;
  uint64_t events;           /* collisions + crossings (+ virtual)         */
  uint64_t secondaries;      /* particles banked                           */
  uint64_t lost, capped, overflow, resample_failures;
  double transport_ms;       /* device time of the transport kernels       */
  uint64_t launches;         /* kernels launched                           */
  double kernel_ms;          /* device time of the main transport kernel    */
  double reserved[3];
} mc_tally_out;

/* k-eigenvalue results.  k_cycle: caller-owned [inactive+active]; tallies
 * are accumulated over active cycles, one history per source particle. */
typedef struct {
  double* k_cycle;
  uint64_t* bank_size;       /* optional [inactive+active]                  */
  double* sum;
  double* sum_sq;
  double k_mean, k_std;      /* over active cycles                          */
  double k_tracklength_mean; /* track-length estimate over active cycles    */
  uint64_t events, lost, capped, overflow;
  double transport_ms;       /* transport kernels + site/score kernels      */
  uint64_t launches;
  double kernel_ms;          /* device time of the main transport kernel(s) */
  double reserved[3];
} mc_keig_out;

/* ---- context ------------------------------------------------------------ */
int mc_create(mc_ctx** out, int device);
void mc_destroy(mc_ctx* ctx);
/* Copies the last error message (NUL-terminated, truncated to n). */
int mc_last_error(const mc_ctx* ctx, char* buf, size_t n);
/* Runs subsequent work on a caller stream (cudaStream_t as void*). */
int mc_set_stream(mc_ctx* ctx, void* cuda_stream);
int mc_version(void);

/* ---- problem ------------------------------------------------------------ */
/* Driver::Create(path) (src/Driver.cpp:18-35) + World(root)
 * (src/World.cpp:20-24): parses the XML text, builds the world, nuclear
 * data, source and estimators, and uploads them.  Relative data-file paths
 * resolve against base_dir (NULL or "" = current directory). */
int mc_load_xml(mc_ctx* ctx, const char* xml_text, const char* base_dir);
int mc_problem_info_get(mc_ctx* ctx, mc_problem_info* out);

/* Geometry semantics (applies to later runs and probes of this context).
 * MC_GEOMETRY_ROBUST (default): after a surface crossing the crossed
 *   surface's side follows the direction of travel and that surface is
 *   ignored until the next collision, so a grazing particle cannot stay on a
 *   surface and leave the geometry; CylinderX::Contains compares rho^2 with
 *   r^2.
 * MC_GEOMETRY_REFERENCE: the reference's exact semantics -- relocation by a
 *   point test after a 10*DBL_EPSILON nudge (src/TransportMethod.cpp:68-72)
 *   and CylinderX::Contains comparing sqrt(rho^2) with r^2
 *   (src/CSGSurface.cpp:173). */
#define MC_GEOMETRY_ROBUST 0
#define MC_GEOMETRY_REFERENCE 1
int mc_set_geometry_mode(mc_ctx* ctx, int32_t mode);
int mc_estimator_info_get(mc_ctx* ctx, int32_t index, mc_estimator_info* out);
/* Name of cell/surface/material/nuclide/perturbation by index (kind 0-4). */
int mc_object_name(mc_ctx* ctx, int32_t kind, int32_t index, char* buf, size_t n);

/* ---- solvers ------------------------------------------------------------ */
/* FixedSource::Solve (src/FixedSource.cpp:22-77): histories i = 0..n-1 start
 * from Source::Sample(seed + i); secondaries are transported within their
 * history; tallies are committed per history. */
int mc_run_fixed_source(mc_ctx* ctx, const mc_run_opts* opts, mc_tally_out* out);

/* KEigenvalue::Solve (src/KEigenvalue.cpp:36-84; a stub in the reference,
 * completed here): cycle 0 starts from Source::Sample(1..N); each cycle
 * transports N particles, banks fission sites (Multigroup::Fission /
 * ContinuousFission::Interact), sets k_cycle = sites/N and draws the next N
 * sources uniformly from the bank. */
int mc_run_keigenvalue(mc_ctx* ctx, const mc_run_opts* opts, mc_keig_out* out);

/* Cycle-by-cycle form of mc_run_keigenvalue, for callers that drive the
 * cycle loop.  begin samples the initial source; cycle transports the
 * current source and prepares the next one (k of the cycle in *k); end
 * fills out. */
int mc_keig_begin(mc_ctx* ctx, const mc_run_opts* opts);
int mc_keig_cycle(mc_ctx* ctx, int32_t active, double* k);
/* n cycles (all active or all inactive) with one host synchronisation at
 * the end: each cycle's bank size, k and counters stay on the device until
 * then, and each cycle draws its sources from the previous bank in place.
 * The same k per cycle and tallies as n calls of mc_keig_cycle; k (NULL or
 * n values) receives them.  The first cycle and an autotuning cycle run on
 * their own. */
int mc_keig_cycles(mc_ctx* ctx, uint32_t n, int32_t active, double* k);
int mc_keig_end(mc_ctx* ctx, mc_keig_out* out);
/* Running totals of the cycles run so far (events, transport_ms, launches,
 * counters); k_cycle/bank_size/sum/sum_sq are filled when non-NULL. */
int mc_keig_status(mc_ctx* ctx, mc_keig_out* out);

/* Checkpoint / resume between cycles (no reference counterpart: the
 * reference's k-eigenvalue Solve is a stub, src/KEigenvalue.cpp:36-62).
 * The checkpoint holds the run options, the cycle number, per-cycle k and
 * bank sizes, counters, tallies and the next cycle's source bank; every
 * later random stream is keyed by (seed, cycle), so a run resumed from it
 * (in this or another context holding the same problem) gives results
 * identical to one that did not stop.  mc_keig_checkpoint writes *size
 * bytes into buf (pass buf = NULL to query the size); mc_keig_resume
 * replaces mc_keig_begin and continues with mc_keig_cycle / mc_keig_end. */
int mc_keig_checkpoint(mc_ctx* ctx, void* buf, uint64_t cap, uint64_t* size);
int mc_keig_resume(mc_ctx* ctx, const void* buf, uint64_t size);

/* What the last transport ran: schedule (MC_SCHEDULE_*), the autotuned
 * history-kernel variant, grid and block, and the kernel times the tuner
 * measured per candidate (tune_ms: n entries, may be NULL): the history
 * schedule's five occupancy variants at block 256, then at block 128, then
 * (multigroup problems the event schedule serves) the event schedule with
 * unsorted and with sorted collision queues.  With MC_SCHEDULE_AUTO and no
 * fixed block size or variant, the tuner runs on the second inactive
 * k-eigenvalue cycle and keeps the fastest candidate (schedule, block,
 * variant, queue-sort threshold); it has no counterpart in the reference. */
int mc_schedule_info(mc_ctx* ctx, int32_t* schedule, int32_t* variant, int32_t* grid, int32_t* block,
                     double* tune_ms, int32_t n);

/* Batched Particle::Transport (src/Particle.cpp:42-44) over a host bank:
 * copies n sites in, transports each until it dies, and copies the fission
 * sites they banked (Particle::MoveSecondariesTo, src/Particle.cpp:102-104)
 * back, ordered by source index.  *n_out receives the number of sites;
 * MC_ERR_OVERFLOW if it exceeds cap (the first cap sites are returned).
 * keys of the input sites seed each particle's stream; opts (may be NULL)
 * selects rng, fast_math, schedule and max_events.  Tallies are
 * accumulated into the context's estimators (see mc_tallies_get). */
int mc_transport_bank(mc_ctx* ctx, const mc_site* sites, uint64_t n, const mc_run_opts* opts,
                      mc_site* fission_sites, uint64_t cap, uint64_t* n_out);
/* mc_transport_bank for callers that cannot allocate device memory when
 * they transport: applications that fix their device-memory budget at
 * start-up and forbid allocation afterwards (e.g. a coupled code whose own
 * pool owns the GPU's memory), or code that runs where the device allocator
 * must not be entered.  No counterpart in the reference.  sites and
 * fission_sites are caller-owned DEVICE (or managed, or page-locked host)
 * pointers; pageable host memory is refused with MC_ERR_INPUT.  *n_out
 * (host) gets the number of sites banked; at most cap are written, and
 * MC_ERR_OVERFLOW is returned when the bank was larger.  Allocates nothing:
 * its scratch is a fixed 5.3 MB array that every GPU loading this library
 * holds until exit.  Limits: n <= 16384 sites per call, multigroup problems
 * whose fissions bank at most 4 sites; larger calls fail with MC_ERR_INPUT.
 * The first call on a device looks the array's address up (and loads the
 * kernels): make it before any stream capture.  The address is kept for
 * the life of the process, so a device reset invalidates it.  The call
 * waits for its work before returning (it reads the bank size and the run
 * counters back to the host).  All calls share the array, so calls that
 * overlap on the GPU (other streams, other contexts on the same device)
 * race; serialize them.  Tallies accumulate into the context's estimators
 * as with mc_transport_bank. */
int mc_transport_bank_noalloc(mc_ctx* ctx, const mc_site* sites, uint64_t n, const mc_run_opts* opts,
                              mc_site* fission_sites, uint64_t cap, uint64_t* n_out);
int mc_tallies_reset(mc_ctx* ctx);
int mc_tallies_get(mc_ctx* ctx, double* sum, double* sum_sq);

/* ---- deterministic kernels, for parity checks --------------------------- */
/* World::FindCellContaining (src/World.cpp:26-37): first cell in XML order
 * containing each point; -1 where the reference throws. xyz: [n][3]. */
int mc_find_cell(mc_ctx* ctx, const double* xyz, uint64_t n, int32_t* cell);
/* Cell::NearestSurface (src/Cell.cpp:37-51). */
int mc_nearest_surface(mc_ctx* ctx, const int32_t* cell, const double* xyz, const double* uvw,
                       uint64_t n, int32_t* surface, double* distance);
/* CSGSurface::Distance / Contains (src/CSGSurface.cpp:71-174). */
int mc_surface_distance(mc_ctx* ctx, int32_t surface, const double* xyz, const double* uvw,
                        uint64_t n, double* distance);
int mc_surface_contains(mc_ctx* ctx, int32_t surface, const double* xyz, uint64_t n,
                        int8_t* contains);
/* Material::GetMicroscopicTotal / GetMicroscopicMajorant (src/Material.cpp:41-61)
 * for a neutron in `cell` at xyz with the given energy (MeV or group). */
int mc_material_xs(mc_ctx* ctx, int32_t cell, const double* xyz, const double* energy,
                   uint64_t n, double* total, double* majorant);
/* ContinuousMap::at bracket (src/ContinuousMap.hpp:21-56): for each energy,
 * the std::map::upper_bound position in each table of a continuous-energy
 * nuclide (neutron data), found through the unionized grid.
 * upper_index: [n][6] -- total, the reactions in input order, then the nubar
 * tables of the fission reactions; -1 past the last table. */
int mc_energy_index(mc_ctx* ctx, int32_t nuclide, const double* energy, uint64_t n,
                    int64_t* upper_index);

/* ---- thermal scattering (ThermalScattering.cpp) --------------------------- */
#define MC_TSL_POD 0      /* POD reconstruction, SampleBeta/SampleAlpha     */
#define MC_TSL_MLP 1      /* MLP surrogate (POD outside the trained box)    */
#define MC_TSL_GUIDED 2   /* guided POD: the POD sampler's samples for the
                             same Philox streams (the FP32 form with
                             MC_TSL_FAST, else the exact FP64 form), CDF
                             searches started where the guide network
                             predicts (Philox streams always)              */
#define MC_TSL_PHILOX 0x10 /* flag: Philox streams keyed by seed, counter i;
                              without it sample i draws from minstd seeded
                              seed + i, as the reference would            */
#define MC_TSL_FAST 0x20  /* flag: FP32 POD reconstruction (see DESIGN)     */
/* ThermalScattering::Scatter (src/ThermalScattering.cpp:159-171) at the
 * sampler level: for each (E,T) draws beta then alpha.  `method` is
 * MC_TSL_POD or MC_TSL_MLP, or'ed with the flags.  Failures (resample
 * limit) leave NaN and are counted in *failures.  Host arrays. */
int mc_sample_tsl(mc_ctx* ctx, int32_t tsl, const double* energy, const double* temperature,
                  uint64_t n, uint64_t seed, int32_t method, double* beta, double* alpha,
                  uint64_t* failures);
/* The same on device arrays of the context's device (stream-ordered on the
 * context's stream, synchronous on return).  No reference counterpart: the
 * reference samples one scatter at a time inside Particle::Transport. */
int mc_sample_tsl_device(mc_ctx* ctx, int32_t tsl, const double* energy, const double* temperature,
                         uint64_t n, uint64_t seed, int32_t method, double* beta, double* alpha,
                         uint64_t* failures);
/* ---- MLP surrogate of the thermal scattering sampler ----------------------
 * No reference counterpart: the reference samples thermal scattering from
 * its POD tables only.  Two networks (16 inputs, three hidden layers of 128
 * with SiLU, one output; BF16 tensor-core products, FP32 master weights)
 * map (E, T, u) to the quantile position of beta in [-E/kT, beta_cutoff],
 * and (E, T, beta, u) to that of alpha between its kinematic bounds.  They
 * are trained on the device from POD samples (`conditions` random (E, T)
 * pairs in the box, `samples_per_condition` POD draws each, sorted into
 * empirical quantiles) with Adam.  Sampling with MC_TSL_MLP outside the
 * trained box falls back to the POD sampler. */
typedef struct mc_train_desc {
  double E_min, E_max;          /* trained incident-energy box (MeV)        */
  double T_min, T_max;          /* and temperature box (K)                  */
  uint64_t conditions;          /* (E, T) pairs; 0 -> 8192                  */
  uint32_t samples_per_condition; /* power of two <= 1024; 0 -> 1024        */
  uint32_t batch;               /* multiple of 128; 0 -> 8192               */
  uint32_t steps;               /* Adam steps per network; 0 -> 4000        */
  float lr;                     /* 0 -> 2e-3 (cosine-decayed to 1 %)        */
  uint64_t seed;
  uint64_t reserved[4];
} mc_train_desc;
typedef struct mc_train_out {
  double loss_beta, loss_alpha; /* mean squared quantile error, last 5 %    */
  double data_ms, train_ms;     /* device time: POD data, training          */
  uint64_t samples;             /* training samples per network             */
  uint64_t failures;            /* POD draws that hit the resample limit    */
  uint64_t reserved[4];
} mc_train_out;
#define MC_MLP_PARAMS 35329     /* FP32 parameters per network              */
int mc_train_surrogate(mc_ctx* ctx, int32_t tsl, const mc_train_desc* desc, mc_train_out* out);
/* The guide network of the guided sampler (MC_TSL_GUIDED, MC_THERMAL_GUIDED;
 * no reference counterpart): the same architecture, trained on the device to
 * predict the CDF-grid position where ThermalScattering::SampleAlpha's
 * find_cdf bisection ends (src/ThermalScattering.cpp:395-421) for each
 * kinematic bound, from the bound, |beta| of the chosen grid point and T.
 * Rows come from the FP32 POD sampler in the (E, T) box:
 * conditions * samples_per_condition samples (defaults 8192 * 256), two
 * rows each.  out->loss_alpha receives the guide's mean squared error. */
int mc_train_surrogate_guide(mc_ctx* ctx, int32_t tsl, const mc_train_desc* desc, mc_train_out* out);
/* Trained weights and box (net 0: beta, 1: alpha; MC_MLP_PARAMS floats each). */
int mc_surrogate_get(mc_ctx* ctx, float* beta_params, float* alpha_params, mc_train_desc* box);
int mc_surrogate_set(mc_ctx* ctx, int32_t tsl, const mc_train_desc* box, const float* beta_params,
                     const float* alpha_params);
/* One forward and backward pass of a network with the given parameters on
 * host inputs x[n][16] and targets y[n] (n a multiple of 128): the gradient
 * of the mean squared error and the loss (for checking against a CPU
 * reference); `out` (optional) receives the forward outputs. */
int mc_surrogate_grad(mc_ctx* ctx, const float* params, const float* x, const float* y, uint64_t n,
                      float* grad, float* loss, float* out);

/* minimc's result file text (src/minimc.cpp:20-21): the batch size line, then
 * EstimatorSet::to_string (src/Estimator.cpp:48-56, 207-213;
 * src/Scorable.cpp:51-70; src/Bins.cpp:84-170) for the given per-bin sums
 * and sums of squares (estimator order, as mc_tally_out / mc_keig_out
 * return them) normalised by total_weight (the number of histories scored:
 * the batch size for a fixed-source run, batch size x active cycles for a
 * k-eigenvalue run).  Writes at most n bytes (NUL-terminated) into buf and
 * the full length into *needed. */
int mc_output_text(mc_ctx* ctx, const double* sum, const double* sum_sq, uint64_t batchsize, double total_weight,
                   char* buf, size_t n, size_t* needed);

/* The same text without a context or a device: parses the problem XML on
 * the host (data files relative to base_dir) and formats the given sums.
 * On an input error writes the message into buf and returns MC_ERR_INPUT. */
int mc_output_format(const char* xml_text, const char* base_dir, const double* sum, const double* sum_sq,
                     uint64_t batchsize, double total_weight, char* buf, size_t n, size_t* needed);

/* ---- batched problems -------------------------------------------------------
 * No reference counterpart: the reference runs one problem per process.
 * Many independent multigroup k-eigenvalue problems of uneven sizes run
 * together: one persistent transport launch per cycle serves all of them
 * (each CTA starts on one problem and, its queue drained, helps drain the
 * others'), one prefix sum, compaction and resampling over their
 * concatenated fission banks, and one cycle's launches are captured once
 * as a CUDA graph and replayed every cycle.  Per problem the k per cycle
 * equals mc_run_keigenvalue's with Philox streams and the same seed. */
typedef struct mc_batch mc_batch;
typedef struct mc_batch_opts {
  uint32_t inactive, active;  /* cycles                                      */
  int32_t fast_math;          /* FP32 sampling arithmetic                    */
  int32_t no_graph;           /* 1: launch the cycle's kernels one by one    */
  int32_t variant;            /* history-kernel variant + 1; 0: autotune     */
  uint32_t max_events;        /* per-particle event cap; 0 -> 1000000        */
  int32_t bank_path;          /* MC_BANK_*: fission-site path                */
  int32_t pad;
  uint64_t reserved[3];
} mc_batch_opts;
typedef struct mc_batch_out {
  double* k_cycle;            /* [problems][inactive + active] or NULL       */
  double* k_mean;             /* [problems] over active cycles, or NULL      */
  double* k_std;              /* [problems] standard error, or NULL          */
  double transport_ms;        /* device time of all cycles                   */
  double tune_ms[8];          /* autotuner: transport time per variant       */
  uint64_t histories;         /* all problems, all cycles                    */
  uint64_t events, lost, capped, overflow;
  uint64_t launches;          /* kernel launches (graph: one per cycle)      */
  int32_t variant;            /* chosen variant                              */
  int32_t graph;              /* 1 if the cycles ran as a CUDA graph         */
  double active_ms;           /* device time of the active cycles            */
  uint64_t reserved[3];
} mc_batch_out;
int mc_batch_create(mc_batch** out, int device);
void mc_batch_destroy(mc_batch* b);
int mc_batch_set_stream(mc_batch* b, void* cuda_stream);
/* adds a multigroup problem (its own XML); histories/seed 0 take the XML's.
 * Returns the problem's index (>= 0) or an error code. */
int mc_batch_add(mc_batch* b, const char* xml_text, const char* base_dir, uint64_t histories, uint64_t seed);
int mc_batch_run(mc_batch* b, const mc_batch_opts* opts, mc_batch_out* out);
int mc_batch_last_error(mc_batch* b, char* buf, size_t n);

/* Multigroup transfer of thermal scatters: for each of `rows` (energy MeV,
 * temperature K) pairs, n scatters are sampled on the device with `method`
 * (any mc_sample_tsl method: MC_TSL_MLP is the surrogate, MC_TSL_POD |
 * MC_TSL_PHILOX [| MC_TSL_FAST] the POD sampler), each outgoing energy
 * E' = E + beta k T formed as ThermalScattering::Scatter does
 * (src/ThermalScattering.cpp:159-171) and binned into the groups whose
 * boundaries (MeV, `groups` + 1 values, descending, group 1 the fastest)
 * are given: group g holds bounds[g] <= E' < bounds[g - 1]; energies above
 * the first bound count in group 1, below the last in the last group.
 * probs[r * groups + g] = the fraction of row r's binned samples in group
 * g + 1.  Samples whose resampling failed (NaN) are not binned; their
 * number is returned in *failures.  The samples stay on the device.
 * groups <= 64, n <= 2^26. */
int mc_tsl_group_transfer(mc_ctx* ctx, int32_t tsl, const double* energy, const double* temperature,
                          uint32_t rows, uint64_t n, const double* bounds, uint32_t groups, uint64_t seed,
                          int32_t method, double* probs, uint64_t* failures);

/* Thin SVD of the POD table pipeline's decomposition step (truncate /
 * adaptive_coarsen in the pipeline that writes the partition files the
 * reference reads in ThermalScattering.cpp:183-463; the pipeline's own source
 * is not in the reference, its call site is
 * scripts/tolerance_vs_spectrum_error/tolerance_vs_spectrum_error.py:16-41):
 * A = U diag(S) V^T for a column-major m x n host matrix, m >= n, in FP64 on
 * the device by one-sided Jacobi rotations.  Outputs (host): S[n] descending,
 * U m x n and V n x n column-major; a column of U whose singular value is 0
 * is zero.  *sweeps (may be NULL) = sweeps over the column pairs until one
 * made no rotation.  Needs no loaded problem.  n <= 2^16, m * n <= 2^30,
 * finite entries. */
int mc_pod_svd(mc_ctx* ctx, const double* A, uint64_t m, uint64_t n, double* U, double* S, double* V,
               uint32_t* sweeps);

/* ThermalScattering::GetTotal (src/ThermalScattering.cpp:111-157). */
int mc_tsl_total(mc_ctx* ctx, int32_t tsl, const double* energy, const double* temperature,
                 uint64_t n, double* xs);

#ifdef __cplusplus
}
#endif

#endif /* MINIMC_GB300_H */
