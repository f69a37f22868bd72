// Device-side world tables, geometry, random streams and physics.
//
// Geometry and anything a parity check compares bit-for-bit is written with
// explicit round-to-nearest intrinsics (__dadd_rn/__dmul_rn/__ddiv_rn), so
// the compiler cannot contract a*b+c into an FMA: the reference, built for
// x86-64 without FMA, rounds every product and sum separately.
#pragma once

#include "mc_ce_layout.h"

#include <cstdint>
#include <cuda_runtime.h>
#include <math_constants.h>

namespace mcd {

// ---------------------------------------------------------------------------
// constants (src/Constants.hpp)
constexpr double kPi = 3.14159265358979323846;
constexpr double kNudge = 10 * 2.220446049250313080847e-16;  // 10 * DBL_EPSILON
constexpr double kOnAxisTolerance = 0.9;
constexpr double kBoltzmann = 8.617333262145e-11;
constexpr double kNeutronMass = 1.045354912280858e-18;
constexpr int kResampleLimit = 10;

// Particle::Event (src/Particle.hpp:36-44) plus the reflection extension
enum Event : int32_t {
  kBirth = 0,
  kScatter = 1,
  kCapture = 2,
  kFission = 3,
  kSurfaceCross = 4,
  kLeak = 5,
  kVirtualCollision = 6,
  kReflect = 7,
  kLostEvent = 8,
};

enum SurfKind : int32_t { kSphere = 0, kPlaneX = 1, kPlaneY = 2, kPlaneZ = 3, kCylX = 4, kCylY = 5, kCylZ = 6 };

// error / counter slots shared by all kernels of a run
struct DevCounters {
  unsigned long long next;       // queue head for dynamic history assignment
  unsigned long long events;
  unsigned long long secondaries;
  unsigned long long lost;
  unsigned long long capped;
  unsigned long long overflow;
  unsigned long long resample;
  unsigned long long banked;     // fission sites banked (k-eigenvalue)
  double k_tracklength;          // sum of nu*Sigma_f*d over the cycle
  double lost_xyz[3];
  unsigned long long pad[4];
};

// A cell bounded by exactly one low and one high axis-aligned plane per axis.
// Per axis at most one of the two planes can be ahead of the particle, so
// Cell::NearestSurface needs three distances instead of six.
struct BoxCell {
  double c[6];      // plane positions: x lo, x hi, y lo, y hi, z lo, z hi
  long long key[6]; // their order-preserving integer keys
  int32_t s[6];     // surface indices
  int32_t order[6]; // position of each plane in the cell's surface list
};

// Continuous-energy tables (built by mc_ce_tables.cpp; lookups in mc_ce.cuh).
struct DevCE {
  int32_t nu;                         // union grid points
  int32_t n_buckets;
  int32_t shift;                      // bucket = (key(E) - key0) >> shift
  int32_t fast_ok;                    // FP32 union tables valid
  int32_t kmax;                       // row length of mat_ncdf
  int32_t pad;
  unsigned long long key0;
  const unsigned long long* ukey;     // [nu] union energies as integer keys
  const double* ue;                   // [nu] union energies
  const uint32_t* bucket;             // [n_buckets + 1]
  const uint32_t* tab_off;            // [n_tables + 1]
  const int32_t* tab_grid;            // [n_tables]
  const double* tab_x;
  const double* tab_y;
  const uint32_t* umap;               // [n_grids][nu + 1]
  const mc::CENuclideDesc* nuc;       // [2][n_nuclides]
  const float* uinv;                  // [nu]
  const float2* mat_flight;           // [2][M][nu]
  const float* mat_ncdf;              // [2][M][nu][kmax]
  const float4* nuc_rx;               // [2][N][nu]
  const float* nuc_nubar;             // [2][N][nu]
};

// One set of POD partitions of a thermal scattering library
// (src/ThermalScattering.hpp:58-97): beta partitions (grid = incident
// energies) or alpha partitions (grid = betas).  Per partition p the tables
// are concatenated; offsets index them.
struct DevPOD {
  int32_t n_parts;
  int32_t n_grid;             // concatenated grid length
  const double* grid;         // [n_grid] Es or betas, increasing
  const uint32_t* ends;       // [n_parts] one past each partition's last grid index
  const int32_t* nF;          // [n_parts] CDF values
  const int32_t* rank;        // [n_parts]
  const int32_t* nT;          // [n_parts] temperatures
  const uint32_t* F_off;      // [n_parts] into F
  const double* F;
  const uint32_t* cdf_off;    // [n_parts] into cdf ([nF][rank])
  const double* cdf;
  const float* cs;            // [.] S[o] * cdf[F][o] in FP32 (fast form), same offsets as cdf
  const uint32_t* S_off;      // [n_parts] into S
  const double* S;
  const uint32_t* T_off;      // [n_parts] into T
  const double* T;
  const uint32_t* g_off;      // [n_parts] into g ([grid][nT][rank])
  const double* g;
  const float* gf;            // g in FP32 (fast form), same offsets
  // [n_grid] bit 0 where the FP32 reconstruction of the grid point's inverse
  // CDF rises along F at every tabulated temperature by more than its
  // rounding bound (so it rises at every temperature between them too), bit
  // 1 the same for the exact FP64 reconstruction: a search over it may
  // start anywhere and still find upper_bound's answer
  const uint8_t* mono;
};

struct DevTSL {
  double beta_cutoff, alpha_cutoff, awr, cutoff_energy;
  int32_t xs_nE, xs_nT, xs_rank, maj_n;
  int32_t fast_ok;            // every partition's rank fits the FP32 form
  int32_t pad;
  const double* xs_E;         // [xs_nE]
  const double* xs_T;         // [xs_nT]
  const double* xs_Em;        // [xs_nE][xs_rank]
  const double* xs_Tm;        // [xs_nT][xs_rank]
  const double* xs_S;         // [xs_rank]
  const float* xs_EmS_f;      // [xs_nE][xs_rank] S[o] * Em[E][o] in FP32 (fast-mode totals)
  const float* xs_Tm_f;       // [xs_nT][xs_rank]
  const double* maj_x;        // majorant ContinuousMap
  const double* maj_y;
  DevPOD beta, alpha;
};

// A parked thermal scatter as the batched POD-exact samplers read it (the
// guided sampler and the plain POD queue): incident energy, temperature and
// the particle's own Philox stream position; and what they return: (beta,
// alpha), the stream position after their draws, and whether the sampler
// stayed within the resample limits.
struct GuideRow {
  double E, T;
  unsigned long long rng_id;
  uint32_t rng_pos, rng_tag;
};
struct GuideOut {
  double beta, alpha;
  uint32_t rng_pos;
  int32_t ok;
};

constexpr int kMaxPert = 4;  // perturbations per problem
constexpr int kMaxSens = 4;  // sensitivities per estimator

// Flattened world, passed to kernels by value.
struct DevWorld {
  int32_t n_surfaces, n_cells, n_materials, n_nuclides, n_types;
  int32_t energy_mode, tracking, quirks, G, max_mat_nuc;
  // surfaces
  const int32_t* surf_kind;
  const int32_t* surf_refl;
  const double* surf_p;  // [n][4]
  // cells
  const int32_t* cell_begin;  // [n_cells+1]
  const int32_t* cell_surf;
  const uint8_t* cell_within;
  const int32_t* cell_mat;
  const int32_t* cell_field;
  const double* field;  // [nf][8]: linear, c, g0, g1, g2, b, upper, lower
  // materials
  const double* mat_density;
  const int32_t* mat_begin;
  const int32_t* mat_nuc;
  const double* mat_afrac;
  // multigroup tables, all indexed by particle type first
  const double* mg_total;     // [T][N][G]
  const double* mg_rx_cdf;    // [T][N][G][3] running sums capture, scatter, fission
  const double* mg_scat_cdf;  // [T][N][G][G] running sums over outgoing group
  const double* mg_nubar;     // [T][N][G]
  const double* mg_chi_cdf;   // [T][N][G][G]
  const double* mg_nusigf;    // [T][N][G] nubar * fission (track-length k)
  const double* mat_mg_total;    // [T][M][G]  Σ afrac * total, reference order
  const double* mat_mg_nuc_cdf;  // [T][M][G][max_mat_nuc] running sums
  const double* mat_mg_nusigf;   // [T][M][G]  N * Σ afrac * nu * sigma_f (macroscopic)
  // estimators
  int32_t n_est;
  const int32_t* est_kind;     // 0 current, 1 track length
  const int32_t* est_target;   // surface or cell
  const uint64_t* est_offset;  // first bin
  const int32_t* est_has_cos;
  const double* est_cos_dir;   // [n_est][3]
  const int32_t* est_bin_kind; // [n_est][2] cosine, energy
  const double* est_bin_par;   // [n_est][2][6]: n_bins, lower/log_lower, upper/log_upper, width/log_width, base, nbounds
  const uint64_t* est_bound_off;  // [n_est][2] offset into est_bounds
  const double* est_bounds;
  const int32_t* est_ebin_mg;     // [n_est][G] energy bin of each group (multigroup)
  const uint64_t* est_esize;      // [n_est] number of energy bins
  // perturbations (TotalCrossSectionPerturbation) and sensitivity estimators
  int32_t n_pert;                 // <= kMaxPert
  const int32_t* mat_pert;        // [n_materials] bit k: the material holds perturbation k's nuclide
  const int32_t* est_nsens;       // [n_est] sensitivities of each estimator
  const int32_t* est_sens;        // [n_est][kMaxSens] their perturbation indices
  const uint64_t* est_size;       // [n_est] bins of an estimator (and of each of its sensitivities)
  // fast paths (all exact)
  const long long* surf_key;      // [n] order-preserving integer key of a plane's position
  const int32_t* cell_box;        // [n_cells] index into boxes, or -1
  const struct BoxCell* boxes;
  const double* mat_mg_sigma;     // [T][M][G] number_density * microscopic total
  // FP32 copies for the fast form (Philox streams, FP32 sampling
  // arithmetic): flight lengths, nuclide / reaction / outgoing-group
  // thresholds and fission yields are drawn against these
  const float* mat_mg_sigma_f;    // [T][M][G]
  const float* mat_mg_total_f;    // [T][M][G]
  const float* mat_mg_nuc_cdf_f;  // [T][M][G][max_mat_nuc]
  const float* mg_total_f;        // [T][N][G]
  const float* mg_rx_cdf_f;       // [T][N][G][3]
  const float* mg_scat_cdf_f;     // [T][N][G][G]
  const float* mg_nubar_f;        // [T][N][G]
  DevCE ce;                       // continuous energy
  int32_t n_tsl;
  const DevTSL* tsl;              // [n_tsl] thermal scattering libraries
  // source (src/Source.cpp)
  double src_pos[3];
  double src_dir[3];
  int32_t src_dir_kind;  // 0 constant, 1 isotropic, 2 isotropic flux
  int32_t src_type;
  double src_energy;     // MeV or group
};

// ---------------------------------------------------------------------------
// arithmetic without contraction
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// Point::Dot (src/Point.cpp:51-53): (x*rx + y*ry) + z*rz
__device__ __forceinline__ double dot3(double x, double y, double z, double a, double b, double c) {
  return dadd(dadd(dmul(x, a), dmul(y, b)), dmul(z, c));
}

// Order-preserving integer key of a double: for non-NaN a, b,
// a < b  <=>  dkey(a) < dkey(b) (signed).  -0.0 maps to the key of +0.0, so
// equal values get equal keys.  Comparing keys runs on the integer pipe,
// which on this part issues 32x more operations per clock than FP64.
__host__ __device__ __forceinline__ long long dkey(double v) {
#ifdef __CUDA_ARCH__
  long long b = __double_as_longlong(v);
#else
  long long b;
  __builtin_memcpy(&b, &v, sizeof b);
#endif
  if (b == static_cast<long long>(0x8000000000000000ull)) b = 0;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

// threshold comparisons of non-negative doubles (running sums of cross
// sections and probabilities): the IEEE bit patterns order like the values
__device__ __forceinline__ long long nonneg_bits(double v) { return __double_as_longlong(v); }

// ---------------------------------------------------------------------------
// random streams

// std::minstd_rand (a = 48271, m = 2^31 - 1) consumed through the C++
// standard's generate_canonical<double, 53>: two draws, S = g1' + g2'*R,
// result S / R^2 with R = 2^31 - 2 and g' = g - 1.
struct MinstdRng {
  uint32_t x;
  __device__ __forceinline__ static uint32_t seed_state(unsigned long long s) {
    const uint32_t r = static_cast<uint32_t>(s % 2147483647ull);
    return r == 0 ? 1u : r;
  }
  __device__ __forceinline__ void seed(unsigned long long s) { x = seed_state(s); }
  __device__ __forceinline__ uint32_t next() {
    x = static_cast<uint32_t>((static_cast<unsigned long long>(x) * 48271ull) % 2147483647ull);
    return x;
  }
  __device__ __forceinline__ double u01() {
    const double r = 2147483646.0;
    double sum = static_cast<double>(next() - 1u);
    sum = dadd(sum, dmul(static_cast<double>(next() - 1u), r));
    const double tmp = dmul(r, r);
    double ret = ddiv(sum, tmp);
    if (ret >= 1.0) ret = 0.99999999999999988898;  // nextafter(1, 0)
    return ret;
  }
  __device__ __forceinline__ float u01f() { return static_cast<float>(u01()); }
  // key for a child particle: the reference seeds secondaries with rng()
  __device__ __forceinline__ unsigned long long child_key() { return next(); }
  __device__ __forceinline__ uint32_t save() const { return x; }
  __device__ __forceinline__ void restore(unsigned long long, unsigned long long, uint32_t, uint32_t packed) {
    x = packed;
  }
};

// Philox4x32-10 round function (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11): 10 rounds over a 4x32 counter with a
// 2x32 key; multipliers and Weyl key increments from that paper.
__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const unsigned long long p0 = 0xD2511F53ull * c[0];
    const unsigned long long p1 = 0xCD9E8D57ull * c[2];
    const uint32_t hi0 = static_cast<uint32_t>(p0 >> 32), lo0 = static_cast<uint32_t>(p0);
    const uint32_t hi1 = static_cast<uint32_t>(p1 >> 32), lo1 = static_cast<uint32_t>(p1);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

// One Philox block as an out-of-line function: a stream's refill is reached
// from every draw site of the transport kernels, and inlining its 10 rounds
// at each of them makes the kernels large enough to miss the instruction
// cache; arguments and result stay in registers.
static __device__ __noinline__ uint4 philox_block(uint32_t ctr, uint32_t h0, uint32_t h1, uint32_t tag, uint32_t k0,
                                                  uint32_t k1) {
  uint32_t c[4] = {ctr, h0, h1, tag};
  philox4x32_10(c, k0, k1);
  return make_uint4(c[0], c[1], c[2], c[3]);
}

// Counter-based stream of one particle: key = the run (seed, cycle), counter
// = (block index, particle id lo, particle id hi, tag).  Primaries use
// their history index as id and tag 0; secondaries use 64 bits drawn from
// their parent and tag 1.
struct PhiloxRng {
  uint32_t k0, k1, h0, h1, tag;
  uint32_t ctr;
  uint32_t buf[4];
  int32_t idx;
  __device__ __forceinline__ void init(unsigned long long run_key, unsigned long long id, uint32_t t) {
    k0 = static_cast<uint32_t>(run_key);
    k1 = static_cast<uint32_t>(run_key >> 32);
    h0 = static_cast<uint32_t>(id);
    h1 = static_cast<uint32_t>(id >> 32);
    tag = t;
    ctr = 0;
    idx = 4;
  }
  __device__ __forceinline__ void refill() {
    const uint4 b = philox_block(ctr++, h0, h1, tag, k0, k1);
    buf[0] = b.x;
    buf[1] = b.y;
    buf[2] = b.z;
    buf[3] = b.w;
    idx = 0;
  }
  __device__ __forceinline__ uint32_t next() {
    if (idx >= 4) refill();
    return buf[idx++];
  }
  // uniform in [0, 1) on the 2^-52 lattice: 52 random mantissa bits under
  // the exponent of 1.0 give [1, 2); one FP64 subtraction shifts it down
  __device__ __forceinline__ double u01() {
    const uint32_t hi = next(), lo = next();
    return __hiloint2double(static_cast<int>(0x3FF00000u | (hi >> 12)), static_cast<int>(lo)) - 1.0;
  }
  // uniform in [2^-24, 1 - 2^-24]: 23 random bits plus a half step, exact in
  // FP32 (24 bits plus the half step would round the top value up to 1.0)
  __device__ __forceinline__ float u01f() { return (static_cast<float>(next() >> 9) + 0.5f) * (1.0f / 8388608.0f); }
  __device__ __forceinline__ unsigned long long child_key() {
    const unsigned long long lo = next();
    return lo | (static_cast<unsigned long long>(next()) << 32);
  }
  // Position in the stream as one word (block counter, index in block), so
  // that a particle resumed in another kernel draws exactly the numbers it
  // would have drawn without the break.
  __device__ __forceinline__ uint32_t save() const { return (ctr << 3) | static_cast<uint32_t>(idx); }
  __device__ __forceinline__ void restore(unsigned long long run_key, unsigned long long id, uint32_t t,
                                          uint32_t packed) {
    init(run_key, id, t);
    ctr = packed >> 3;
    idx = static_cast<int32_t>(packed & 7u);
    if (idx < 4) {
      uint32_t c[4] = {ctr - 1, h0, h1, tag};
      philox4x32_10(c, k0, k1);
      buf[0] = c[0];
      buf[1] = c[1];
      buf[2] = c[2];
      buf[3] = c[3];
    }
  }
};

// ---------------------------------------------------------------------------
// surfaces (src/CSGSurface.cpp)

// CSGSurface::SolveQuadratic (src/CSGSurface.cpp:71-97)
__device__ __forceinline__ double solve_quadratic(double a, double b, double c) {
  const double disc = dsub(dmul(b, b), dmul(dmul(4.0, a), c));
  if (disc <= 0) return CUDART_INF;
  const double sq = __dsqrt_rn(disc);
  const double two_a = dmul(2.0, a), two_c = dmul(2.0, c);
  const double lesser = b > 0 ? ddiv(dsub(-b, sq), two_a) : ddiv(two_c, dadd(-b, sq));
  const double greater = b > 0 ? ddiv(two_c, dsub(-b, sq)) : ddiv(dadd(-b, sq), two_a);
  if (lesser > 0) return lesser;
  if (greater > 0) return greater;
  return CUDART_INF;
}

// Distance to the cylinder r^2 = |p|^2 - (p.w)^2 about a coordinate axis.
// (CylinderX::Distance, src/CSGSurface.cpp:148-162; y/z axes by symmetry)
__device__ __forceinline__ double cylinder_distance(double px, double py, double pz, double dx, double dy, double dz,
                                                    int axis, double r) {
  const double pp = dot3(px, py, pz, px, py, pz);
  const double ax = axis == 0, ay = axis == 1, az = axis == 2;
  const double pw = dot3(px, py, pz, ax, ay, az);
  const double dw = dot3(dx, dy, dz, ax, ay, az);
  const double pd = dot3(px, py, pz, dx, dy, dz);
  return solve_quadratic(dsub(1.0, dmul(dw, dw)), dmul(2.0, dsub(pd, dmul(pw, dw))),
                         dsub(dsub(pp, dmul(pw, pw)), dmul(r, r)));
}

__device__ __forceinline__ double plane_distance(double pos, double dir, double c) {
  // PlaneX::Distance (src/CSGSurface.cpp:125-134): v = c - p.x, d = v / u
  const double d = ddiv(dsub(c, pos), dir);
  return d > 0 ? d : CUDART_INF;
}

__device__ __forceinline__ double surface_distance(const DevWorld& w, int s, double x, double y, double z, double u,
                                                   double v, double ww) {
  const double* p = w.surf_p + 4 * s;
  switch (__ldg(w.surf_kind + s)) {
  case kPlaneX: return plane_distance(x, u, __ldg(p));
  case kPlaneY: return plane_distance(y, v, __ldg(p));
  case kPlaneZ: return plane_distance(z, ww, __ldg(p));
  case kSphere: {
    // Sphere::Distance (src/CSGSurface.cpp:107-111)
    const double ox = dsub(x, __ldg(p)), oy = dsub(y, __ldg(p + 1)), oz = dsub(z, __ldg(p + 2));
    const double r = __ldg(p + 3);
    return solve_quadratic(1.0, dmul(2.0, dot3(ox, oy, oz, u, v, ww)), dsub(dot3(ox, oy, oz, ox, oy, oz), dmul(r, r)));
  }
  case kCylX: return cylinder_distance(x, y, z, u, v, ww, 0, __ldg(p));
  case kCylY: return cylinder_distance(x, y, z, u, v, ww, 1, __ldg(p));
  default: return cylinder_distance(x, y, z, u, v, ww, 2, __ldg(p));
  }
}

// a point with the order-preserving keys of its coordinates
struct PointK {
  double x, y, z;
  long long kx, ky, kz;
  __device__ __forceinline__ PointK(double x_, double y_, double z_)
      : x(x_), y(y_), z(z_), kx(dkey(x_)), ky(dkey(y_)), kz(dkey(z_)) {}
};

// CSGSurface::Contains: true on the negative side; on-surface is positive.
// Planes compare integer keys (x < c  <=>  key(x) < key(c)).
__device__ __forceinline__ bool surface_contains(const DevWorld& w, int s, const PointK& q) {
  const double* p = w.surf_p + 4 * s;
  const double x = q.x, y = q.y, z = q.z;
  switch (__ldg(w.surf_kind + s)) {
  case kPlaneX: return q.kx < __ldg(w.surf_key + s);
  case kPlaneY: return q.ky < __ldg(w.surf_key + s);
  case kPlaneZ: return q.kz < __ldg(w.surf_key + s);
  case kSphere: {
    const double ox = dsub(x, __ldg(p)), oy = dsub(y, __ldg(p + 1)), oz = dsub(z, __ldg(p + 2));
    const double r = __ldg(p + 3);
    return dot3(ox, oy, oz, ox, oy, oz) < dmul(r, r);
  }
  default: {
    const int axis = __ldg(w.surf_kind + s) - kCylX;
    const double pp = dot3(x, y, z, x, y, z);
    const double pw = dot3(x, y, z, axis == 0, axis == 1, axis == 2);
    const double r = __ldg(p);
    const double rho2 = dsub(pp, dmul(pw, pw));
    // CylinderX::Contains (src/CSGSurface.cpp:164-174) compares sqrt(rho^2)
    // with r^2; quirks=1 keeps that, quirks=0 compares rho^2 with r^2.
    return w.quirks ? __dsqrt_rn(rho2) < dmul(r, r) : rho2 < dmul(r, r);
  }
  }
}

__device__ __forceinline__ bool surface_contains(const DevWorld& w, int s, double x, double y, double z) {
  return surface_contains(w, s, PointK(x, y, z));
}

// Cell::Contains (src/Cell.cpp:27-35)
__device__ __forceinline__ bool cell_contains(const DevWorld& w, int c, const PointK& q) {
  const int b = __ldg(w.cell_begin + c), e = __ldg(w.cell_begin + c + 1);
  for (int k = b; k < e; k++) {
    const bool inside = surface_contains(w, __ldg(w.cell_surf + k), q);
    if (inside != (__ldg(w.cell_within + k) != 0)) return false;
  }
  return true;
}

// World::FindCellContaining (src/World.cpp:26-37): first match in XML order
__device__ __forceinline__ int find_cell(const DevWorld& w, double x, double y, double z) {
  const PointK q(x, y, z);
  for (int c = 0; c < w.n_cells; c++)
    if (cell_contains(w, c, q)) return c;
  return -1;
}

// Cell::NearestSurface for a box cell: per axis only the plane ahead can have
// a positive distance -- the high plane when moving up (the low one if the
// point is below it), the low plane when moving down (the high one if above
// it) -- so one exact division per axis.  Ties keep the reference's order:
// the earliest surface in the cell's list wins, and with every distance
// infinite the cell's first surface is returned.
// sign tests on the integer pipe (NaN never reaches them)
__device__ __forceinline__ bool dpos(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool dneg(double x) {
  const long long b = __double_as_longlong(x);
  return b < 0 && b != static_cast<long long>(0x8000000000000000ull);
}

// The three candidate distances are ordered with FP32 quotients first
// (relative error < 4e-7); when the nearest is ahead of the next by more
// than 4e-6 relative, only its exact FP64 distance is needed.  Near ties,
// tiny or unusable FP32 values fall back to all exact divisions, so the
// result always equals the exact computation.
// c / d without a division, for the Philox fast form's plane distances:
// the FP32 reciprocal of d refined by one Newton-Raphson step (relative
// error about 2^-46), the quotient, and one residual correction
// q + r (c - d q), which leaves it within an ulp or two of the correctly
// rounded quotient.  df is d in FP32 and must be a normal number.
__device__ __forceinline__ double quot_nr(double c, double d, float df) {
  const double r0 = static_cast<double>(__frcp_rn(df));
  const double r1 = __fma_rn(r0, __fma_rn(-d, r0, 1.0), r0);
  const double q0 = __dmul_rn(c, r1);
  return __fma_rn(r1, __fma_rn(-d, q0, c), q0);
}

__device__ __forceinline__ int nearest_surface_box(const DevWorld& w, int box, int c, const double* pos,
                                                   const double* dir, const float* dirf, double& dist, int skip,
                                                   bool fast_div) {
  const BoxCell& B = w.boxes[box];
  int cj[3];
  double cv[3];
  float tf[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double p = pos[a], d = dir[a];
    const long long kp = dkey(p);
    const bool hi = dpos(d) ? !(kp < __ldg(&B.key[2 * a])) : (kp > __ldg(&B.key[2 * a + 1]));
    int j = 2 * a + (hi ? 1 : 0);
    // the skipped surface reads as infinitely far; the axis' other plane
    // then is the only candidate
    if (__ldg(&B.s[j]) == skip) j ^= 1;
    cj[a] = j;
    // PlaneX::Distance: v = c - p, positive iff v and d have the same sign
    const double v = dsub(__ldg(&B.c[j]), p);
    cv[a] = v;
    const bool ahead = __ldg(&B.s[j]) != skip && ((dpos(v) && dpos(d)) || (dneg(v) && dneg(d)));
    tf[a] = ahead ? fabsf(__fdiv_rn(__double2float_rn(v), dirf[a])) : CUDART_INF_F;
  }
  int a0 = 0;
  if (tf[1] < tf[a0]) a0 = 1;
  if (tf[2] < tf[a0]) a0 = 2;
  float second = CUDART_INF_F;
#pragma unroll
  for (int a = 0; a < 3; a++)
    if (a != a0) second = fminf(second, tf[a]);
  if (tf[a0] < CUDART_INF_F && tf[a0] > 1e-30f && !(second <= __fmul_rn(tf[a0], 1.000004f))) {
    const double t = fast_div && fabsf(dirf[a0]) >= 1.17549435e-38f ? quot_nr(cv[a0], dir[a0], dirf[a0])
                                                                    : ddiv(cv[a0], dir[a0]);
    if (t > 0 && t < CUDART_INF) {
      dist = t;
      return __ldg(&B.s[cj[a0]]);
    }
  }
  // exact path: every candidate divided, reference tie-breaking
  int best_s = __ldg(w.cell_surf + __ldg(w.cell_begin + c));
  int best_o = 0x7fffffff;
  double bd = CUDART_INF;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const int j = cj[a];
    const int s = __ldg(&B.s[j]);
    const int o = __ldg(&B.order[j]);
    double t = CUDART_INF;
    if (s != skip) {
      const double q = ddiv(cv[a], dir[a]);
      t = q > 0 ? q : CUDART_INF;
    }
    if (t < bd || (t == bd && t != CUDART_INF && o < best_o)) {
      bd = t;
      best_s = s;
      best_o = o;
    }
  }
  dist = bd;
  return best_s;
}

// Cell::NearestSurface (src/Cell.cpp:37-51): first surface (in the cell's
// surface order) with the least distance.  `skip` (robust crossing, see
// below) is a surface the particle has just left and is moving away from;
// it is treated as infinitely far.
__device__ __forceinline__ int nearest_surface_general(const DevWorld& w, int c, double x, double y, double z,
                                                       double u, double v, double ww, double& dist, int skip);

// The same with the direction also given in FP32 (the box cells' preselection
// reads it; callers that keep it avoid three conversions per event).
// fast_div (Philox fast form only): a box cell's plane distance by quot_nr.
__device__ __forceinline__ int nearest_surface(const DevWorld& w, int c, double x, double y, double z, double u,
                                               double v, double ww, float fu, float fv, float fw, double& dist,
                                               int skip = -1, bool fast_div = false) {
  const int box = __ldg(w.cell_box + c);
  if (box >= 0) {
    const double pos[3] = {x, y, z}, dir[3] = {u, v, ww};
    const float dirf[3] = {fu, fv, fw};
    return nearest_surface_box(w, box, c, pos, dir, dirf, dist, skip, fast_div);
  }
  return nearest_surface_general(w, c, x, y, z, u, v, ww, dist, skip);
}

__device__ __forceinline__ int nearest_surface(const DevWorld& w, int c, double x, double y, double z, double u,
                                               double v, double ww, double& dist, int skip = -1,
                                               bool fast_div = false) {
  return nearest_surface(w, c, x, y, z, u, v, ww, __double2float_rn(u), __double2float_rn(v), __double2float_rn(ww),
                         dist, skip, fast_div);
}

__device__ __forceinline__ int nearest_surface_general(const DevWorld& w, int c, double x, double y, double z,
                                                       double u, double v, double ww, double& dist, int skip) {
  const int b = __ldg(w.cell_begin + c), e = __ldg(w.cell_begin + c + 1);
  int best = -1;
  double bd = CUDART_INF;
  for (int k = b; k < e; k++) {
    const int s = __ldg(w.cell_surf + k);
    const double d = s == skip ? CUDART_INF : surface_distance(w, s, x, y, z, u, v, ww);
    if (best < 0 || d < bd) {
      best = s;
      bd = d;
    }
  }
  dist = bd;
  return best;
}

// Robust crossing.  The reference relocates a particle after a crossing by
// moving it a fixed 10*DBL_EPSILON cm past the surface and testing the point
// (src/TransportMethod.cpp:68-72).  Where a coordinate's ulp exceeds that
// nudge times the direction component, the point stays on (or before) the
// surface, the particle is put back into the cell it was leaving, and the
// surface then reads as infinitely far, so the particle can leave the
// geometry without ever crossing.  In robust mode the crossed surface's side
// is taken from the direction of travel instead of the point test, and the
// surface is skipped until the next collision.

// true if moving along (u,v,w) at (x,y,z) goes to the positive side of s
__device__ __forceinline__ bool moving_positive(const DevWorld& w, int s, double x, double y, double z, double u,
                                                double v, double ww) {
  const double* p = w.surf_p + 4 * s;
  switch (__ldg(w.surf_kind + s)) {
  case kPlaneX: return u > 0;
  case kPlaneY: return v > 0;
  case kPlaneZ: return ww > 0;
  case kSphere: return dot3(dsub(x, __ldg(p)), dsub(y, __ldg(p + 1)), dsub(z, __ldg(p + 2)), u, v, ww) > 0;
  case kCylX: return dadd(dmul(y, v), dmul(z, ww)) > 0;
  case kCylY: return dadd(dmul(x, u), dmul(z, ww)) > 0;
  default: return dadd(dmul(x, u), dmul(y, v)) > 0;
  }
}

// World::FindCellContaining with the crossed surface's side forced
__device__ __forceinline__ int find_cell_crossing(const DevWorld& w, double x, double y, double z, int crossed,
                                                  bool to_positive) {
  const PointK q(x, y, z);
  for (int c = 0; c < w.n_cells; c++) {
    const int b = __ldg(w.cell_begin + c), e = __ldg(w.cell_begin + c + 1);
    bool in = true;
    for (int k = b; k < e && in; k++) {
      const int s = __ldg(w.cell_surf + k);
      const bool inside = s == crossed ? !to_positive : surface_contains(w, s, q);
      in = inside == (__ldg(w.cell_within + k) != 0);
    }
    if (in) return c;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// directions (src/Point.cpp:90-121)

// Direction(RNG&): mu = U(-1, 1), phi = U(0, 2 pi)
template <class Rng>
__device__ __forceinline__ void isotropic(Rng& rng, double& u, double& v, double& w) {
  u = dadd(dmul(rng.u01(), 2.0), -1.0);
  const double st = __dsqrt_rn(dsub(1.0, dmul(u, u)));
  const double phi = dadd(dmul(rng.u01(), 2 * kPi), 0.0);
  double s, c;
  sincos(phi, &s, &c);
  v = dmul(st, c);
  w = dmul(st, s);
}

// isotropic direction with FP32 trigonometry, renormalized in FP64 by one
// Newton step (fast-math streams only)
// Every FP32 operation is an explicit round-to-nearest intrinsic or a
// hardware approximation (__sincosf), so the result is the same in every
// kernel that inlines it whatever the compiler contracts elsewhere.
template <class Rng>
__device__ __forceinline__ void isotropic_fast(Rng& rng, double& u, double& v, double& w) {
  const float mu = __fmaf_rn(2.0f, rng.u01f(), -1.0f);
  float s, c;
  // phi in [-pi, pi): the hardware sine/cosine is accurate to ~2^-21 there
  __sincosf(__fmul_rn(__fsub_rn(rng.u01f(), 0.5f), 6.28318530717958647692f), &s, &c);
  const float st = __fsqrt_rn(fmaxf(0.0f, __fmaf_rn(-mu, mu, 1.0f)));
  // unit to FP32 precision (|d|^2 = 1 +- 1e-7); plane distances do not
  // depend on the norm and the robust crossing tolerates the ~1e-7 relative
  // path-length error on curved surfaces
  u = mu;
  v = __fmul_rn(st, c);
  w = __fmul_rn(st, s);
}

// the same, also returning the direction's FP32 values (exactly the
// FP64 ones rounded back: they were FP32 numbers)
template <class Rng>
__device__ __forceinline__ void isotropic_fast(Rng& rng, double& u, double& v, double& w, float& fu, float& fv,
                                               float& fw) {
  const float mu = __fmaf_rn(2.0f, rng.u01f(), -1.0f);
  float s, c;
  __sincosf(__fmul_rn(__fsub_rn(rng.u01f(), 0.5f), 6.28318530717958647692f), &s, &c);
  const float st = __fsqrt_rn(fmaxf(0.0f, __fmaf_rn(-mu, mu, 1.0f)));
  fu = mu;
  fv = __fmul_rn(st, c);
  fw = __fmul_rn(st, s);
  u = fu;
  v = fv;
  w = fw;
}

// exponential flight length in FP32: -log(U) / sigma (U in (0,1))
__device__ __forceinline__ double flight_fast(float u, double sigma) {
  return static_cast<double>(__fdiv_rn(-__logf(u), __double2float_rn(sigma)));
}

// the same on an FP32 table (fast form)
__device__ __forceinline__ int cdf_first_above_f(const float* cdf, int n, float threshold) {
  const int t = __float_as_int(threshold);
  for (int k = 0; k < n; k++)
    if (__float_as_int(__ldg(cdf + k)) > t) return k;
  return -1;
}

// exponential flight length from an FP32 macroscopic total
__device__ __forceinline__ double flight_fast_f(float u, float sigma) {
  return static_cast<double>(__fdiv_rn(-__logf(u), sigma));
}

// first k in [0, n) with cdf[k] > threshold (both non-negative), or -1;
// the comparison runs on the integer pipe (IEEE order of non-negative values)
__device__ __forceinline__ int cdf_first_above(const double* cdf, int n, double threshold) {
  const long long t = nonneg_bits(threshold);
  for (int k = 0; k < n; k++)
    if (__double_as_longlong(__ldg(cdf + k)) > t) return k;
  return -1;
}

// directions in FP32 (fast form): Direction(d, mu, phi) with phi drawn as
// (U - 1/2) 2 pi, normalized in FP32
__device__ __forceinline__ void rotate_f(float& dx, float& dy, float& dz, float mu, float uphi) {
  const bool off_x = dx <= 0.9f && dx > -0.9f;
  float ux, uy, uz;
  if (off_x) {  // d x (1, 0, 0)
    ux = 0.0f;
    uy = dz;
    uz = -dy;
  }
  else {  // d x (0, 1, 0)
    ux = -dz;
    uy = 0.0f;
    uz = dx;
  }
  const float ru = __frsqrt_rn(__fmaf_rn(ux, ux, __fmaf_rn(uy, uy, __fmul_rn(uz, uz))));
  ux = __fmul_rn(ux, ru);
  uy = __fmul_rn(uy, ru);
  uz = __fmul_rn(uz, ru);
  // v = d x u
  const float vx = __fsub_rn(__fmul_rn(dy, uz), __fmul_rn(dz, uy));
  const float vy = __fsub_rn(__fmul_rn(dz, ux), __fmul_rn(dx, uz));
  const float vz = __fsub_rn(__fmul_rn(dx, uy), __fmul_rn(dy, ux));
  float s, c;
  __sincosf(__fmul_rn(__fsub_rn(uphi, 0.5f), 6.28318530717958647692f), &s, &c);
  const float st = __fsqrt_rn(fmaxf(0.0f, __fmaf_rn(-mu, mu, 1.0f)));
  const float a = __fmul_rn(st, c), b = __fmul_rn(st, s);
  const float rx = __fmaf_rn(a, ux, __fmaf_rn(b, vx, __fmul_rn(mu, dx)));
  const float ry = __fmaf_rn(a, uy, __fmaf_rn(b, vy, __fmul_rn(mu, dy)));
  const float rz = __fmaf_rn(a, uz, __fmaf_rn(b, vz, __fmul_rn(mu, dz)));
  const float rn = __frsqrt_rn(__fmaf_rn(rx, rx, __fmaf_rn(ry, ry, __fmul_rn(rz, rz))));
  dx = __fmul_rn(rx, rn);
  dy = __fmul_rn(ry, rn);
  dz = __fmul_rn(rz, rn);
}


// Direction(d, mu, phi) (src/Point.cpp:98-121), normalized on assignment
__device__ __forceinline__ void rotate(double& dx, double& dy, double& dz, double mu, double phi) {
  const bool off_x = dx <= kOnAxisTolerance && dx > -kOnAxisTolerance;
  const double ax = off_x ? 1.0 : 0.0, ay = off_x ? 0.0 : 1.0, az = 0.0;
  // u = normalize(d x axis)
  double ux = dsub(dmul(dy, az), dmul(dz, ay));
  double uy = dsub(dmul(dz, ax), dmul(dx, az));
  double uz = dsub(dmul(dx, ay), dmul(dy, ax));
  double n = __dsqrt_rn(dot3(ux, uy, uz, ux, uy, uz));
  ux = ddiv(ux, n);
  uy = ddiv(uy, n);
  uz = ddiv(uz, n);
  // v = normalize(d x u)
  double vx = dsub(dmul(dy, uz), dmul(dz, uy));
  double vy = dsub(dmul(dz, ux), dmul(dx, uz));
  double vz = dsub(dmul(dx, uy), dmul(dy, ux));
  n = __dsqrt_rn(dot3(vx, vy, vz, vx, vy, vz));
  vx = ddiv(vx, n);
  vy = ddiv(vy, n);
  vz = ddiv(vz, n);
  const double smu = __dsqrt_rn(dsub(1.0, dmul(mu, mu)));
  double sp, cp;
  sincos(phi, &sp, &cp);
  const double a = dmul(smu, cp), bb = dmul(smu, sp);
  double rx = dadd(dadd(dmul(a, ux), dmul(bb, vx)), dmul(mu, dx));
  double ry = dadd(dadd(dmul(a, uy), dmul(bb, vy)), dmul(mu, dy));
  double rz = dadd(dadd(dmul(a, uz), dmul(bb, vz)), dmul(mu, dz));
  n = __dsqrt_rn(dot3(rx, ry, rz, rx, ry, rz));
  dx = ddiv(rx, n);
  dy = ddiv(ry, n);
  dz = ddiv(rz, n);
}

// ---------------------------------------------------------------------------
// bins (src/Bins.cpp)
__device__ __forceinline__ uint64_t bin_index(const DevWorld& w, int e, int dim, double val) {
  const int kind = __ldg(w.est_bin_kind + 2 * e + dim);
  const double* par = w.est_bin_par + (2 * e + dim) * 6;
  if (kind == 1) {  // linspace
    const double lo = __ldg(par + 1), hi = __ldg(par + 2), width = __ldg(par + 3);
    const uint64_t nb = static_cast<uint64_t>(__ldg(par));
    if (val < lo) return 0;
    if (val >= hi) return nb - 1;
    return static_cast<uint64_t>(dadd(ddiv(dsub(val, lo), width), 1.0));
  }
  if (kind == 2) {  // logspace
    const double lo = __ldg(par + 1), hi = __ldg(par + 2), width = __ldg(par + 3), base = __ldg(par + 4);
    const uint64_t nb = static_cast<uint64_t>(__ldg(par));
    const double lv = ddiv(log(val), log(base));
    if (lv < lo) return 0;
    if (lv >= hi) return nb - 1;
    return static_cast<uint64_t>(dadd(ddiv(dsub(lv, lo), width), 1.0));
  }
  if (kind == 3) {  // boundaries: upper_bound
    const double* bnd = w.est_bounds + __ldg(w.est_bound_off + 2 * e + dim);
    uint64_t lo = 0, n = static_cast<uint64_t>(__ldg(par + 5));
    while (n > 0) {
      const uint64_t half = n >> 1;
      if (!(val < __ldg(bnd + lo + half))) {
        lo += half + 1;
        n -= half + 1;
      }
      else {
        n = half;
      }
    }
    return lo;
  }
  return 0;
}

// ParticleBins::GetIndex (src/Bins.cpp:196-204)
__device__ __forceinline__ uint64_t particle_bin(const DevWorld& w, int e, double u, double v, double ww,
                                                 double energy) {
  uint64_t ci = 0;
  if (__ldg(w.est_has_cos + e)) {
    const double* d = w.est_cos_dir + 3 * e;
    ci = bin_index(w, e, 0, dot3(__ldg(d), __ldg(d + 1), __ldg(d + 2), u, v, ww));
  }
  const uint64_t ei = bin_index(w, e, 1, energy);
  const double* epar = w.est_bin_par + (2 * e + 1) * 6;
  const int ek = __ldg(w.est_bin_kind + 2 * e + 1);
  const uint64_t esize = ek == 0 ? 1 : (ek == 3 ? static_cast<uint64_t>(__ldg(epar + 5)) + 1 : static_cast<uint64_t>(__ldg(epar)));
  return esize * ci + ei;
}

// multigroup form: the energy value is the group number, whose bin is
// tabulated per group on the host with the same formulas
__device__ __forceinline__ uint64_t particle_bin_mg(const DevWorld& w, int e, double u, double v, double ww, int g) {
  uint64_t ci = 0;
  if (__ldg(w.est_has_cos + e)) {
    const double* d = w.est_cos_dir + 3 * e;
    ci = bin_index(w, e, 0, dot3(__ldg(d), __ldg(d + 1), __ldg(d + 2), u, v, ww));
  }
  return __ldg(w.est_esize + e) * ci + static_cast<uint64_t>(__ldg(w.est_ebin_mg + e * w.G + g));
}

// Per-history pending scores (ScorableProxy::pending_scores,
// src/Scorable.hpp:82-86): a short list of (bin, score).
template <int N>
struct Pending {
  uint32_t bin[N];
  double score[N];
  int n;
  bool overflow;
  __device__ __forceinline__ void clear() {
    n = 0;
    overflow = false;
  }
  __device__ __forceinline__ void add(uint32_t b, double s) {
    for (int i = 0; i < n; i++) {
      if (bin[i] == b) {
        score[i] += s;
        return;
      }
    }
    if (n < N) {
      bin[n] = b;
      score[n] = s;
      n++;
    }
    else {
      overflow = true;
    }
  }
};

}  // namespace mcd
