// Thermal scattering (src/ThermalScattering.cpp) on the device:
//   GetTotal / EvaluateInelastic      :111-157, :260-269
//   BetaPartition/AlphaPartition::Evaluate  :183-256
//   SampleBeta / SampleAlpha / Scatter      :159-171, :271-463
//
// Two forms of the POD reconstruction:
//   exact: FP64 with the reference's operation order (bit-for-bit with the
//          reference's arithmetic for the same random numbers);
//   fast:  the temperature interpolation is applied to the mode vector
//          once per sample (G_T = G_lo + w (G_hi - G_lo)), after which each
//          reconstruction is one rank-r FP32 dot product with the
//          precomputed S * CDF_modes row.  Linear interpolation commutes
//          with the sum, so this is the same function rounded in FP32.
// The sampling logic (grid choice, bisection, endpoints, resampling, the
// alpha interpolation factor as the reference writes it) is shared.
#pragma once

#include "mc_device.cuh"

#include <type_traits>

namespace mcd {

constexpr int kTslResampleLimit = 10;  // constants::beta/alpha_resample_limit
constexpr int kFastPodRank = 32;       // fast form: mode vector in registers

// std::upper_bound on a sorted array (libstdc++'s bisection); the
// comparisons run on order-preserving integer keys (the same outcome as the
// FP64 comparison for every value, on the integer pipe)
__device__ __forceinline__ int upper_index(const double* v, int n, double x) {
  // a NaN compares false with every element
  if ((__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll) return n;
  const long long kx = dkey(x);
  int first = 0, len = n;
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (kx < dkey(__ldg(v + mid))) {
      len = half;
    }
    else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  return first;
}

// one partition at one temperature: the temperature bracket of
// Evaluate (T >= T_max uses the top interval, T < T_min both ends at the
// first point)
struct PodAt {
  int part, r, nT, lo, hi, nF;
  double T, Tl, Th;
  const double* S;
  const double* cdf;
  const double* g;
  const double* F;
  const float* cs;
  const float* gf;
};

__device__ __forceinline__ PodAt pod_at(const DevPOD& P, int part, double T) {
  PodAt c;
  c.part = part;
  c.r = __ldg(P.rank + part);
  c.nT = __ldg(P.nT + part);
  c.nF = __ldg(P.nF + part);
  const double* Ts = P.T + __ldg(P.T_off + part);
  const int cand = upper_index(Ts, c.nT, T);
  const bool above = cand == c.nT;
  c.hi = above ? cand - 1 : cand;
  c.lo = c.hi == 0 ? c.hi : c.hi - 1;
  c.T = T;
  c.Tl = __ldg(Ts + c.lo);
  c.Th = __ldg(Ts + c.hi);
  c.S = P.S + __ldg(P.S_off + part);
  c.cdf = P.cdf + __ldg(P.cdf_off + part);
  c.cs = P.cs + __ldg(P.cdf_off + part);
  c.g = P.g + __ldg(P.g_off + part);
  c.gf = P.gf + __ldg(P.g_off + part);
  c.F = P.F + __ldg(P.F_off + part);
  return c;
}

// Evaluate(cdf_i, g_i, T), exact form
__device__ __forceinline__ double pod_eval(const PodAt& c, int cdf_i, int g_i) {
  const double* C = c.cdf + static_cast<size_t>(cdf_i) * c.r;
  const double* Gh = c.g + (static_cast<size_t>(g_i) * c.nT + c.hi) * c.r;
  const double* Gl = c.g + (static_cast<size_t>(g_i) * c.nT + c.lo) * c.r;
  double vh = 0, vl = 0;
  for (int o = 0; o < c.r; o++) {
    const double sc = dmul(__ldg(c.S + o), __ldg(C + o));
    vh = dadd(vh, dmul(sc, __ldg(Gh + o)));
    vl = dadd(vl, dmul(sc, __ldg(Gl + o)));
  }
  return dadd(vl, dmul(ddiv(dsub(vh, vl), dsub(c.Th, c.Tl)), dsub(c.T, c.Tl)));
}

// fast form: the mode vector of grid point g_i interpolated to T
struct PodVec {
  float v[kFastPodRank];
};
__device__ __forceinline__ void pod_vec(const PodAt& c, int g_i, PodVec& out) {
  const float* Gh = c.gf + (static_cast<size_t>(g_i) * c.nT + c.hi) * c.r;
  const float* Gl = c.gf + (static_cast<size_t>(g_i) * c.nT + c.lo) * c.r;
  const float w = static_cast<float>(ddiv(dsub(c.T, c.Tl), dsub(c.Th, c.Tl)));
#pragma unroll
  for (int o = 0; o < kFastPodRank; o++) {
    if (o < c.r) {
      const float l = __ldg(Gl + o);
      out.v[o] = __fmaf_rn(w, __fsub_rn(__ldg(Gh + o), l), l);
    }
    else {
      out.v[o] = 0.0f;
    }
  }
}
__device__ __forceinline__ double pod_eval_fast(const PodAt& c, const PodVec& gv, int cdf_i) {
  const float* C = c.cs + static_cast<size_t>(cdf_i) * c.r;
  float acc = 0.0f;
#pragma unroll
  for (int o = 0; o < kFastPodRank; o++)
    if (o < c.r) acc = __fmaf_rn(__ldg(C + o), gv.v[o], acc);
  return static_cast<double>(acc);
}

// Arithmetic around the reconstructions: the reference's FP64 operations in
// the exact form; FP32 in the fast form (the reconstructions there are FP32
// already), with FP32 uniforms from Philox streams.
template <bool FAST>
__device__ __forceinline__ double sdiv(double a, double b) {
  if constexpr (FAST) return static_cast<double>(__fdiv_rn(__double2float_rn(a), __double2float_rn(b)));
  else return ddiv(a, b);
}
template <bool FAST>
__device__ __forceinline__ double ssqrt(double a) {
  if constexpr (FAST) return static_cast<double>(__fsqrt_rn(__double2float_rn(a)));
  else return __dsqrt_rn(a);
}
template <bool FAST, class Rng>
__device__ __forceinline__ double su01(Rng& rng) {
  if constexpr (FAST && std::is_same_v<Rng, PhiloxRng>) return static_cast<double>(rng.u01f());
  else return rng.u01();
}

// partition holding global grid index i (upper_bound over the ends)
__device__ __forceinline__ int pod_partition(const DevPOD& P, int i, int& local) {
  int ps = 0;
  while (ps < P.n_parts && static_cast<int>(__ldg(P.ends + ps)) <= i) ps++;
  local = ps == 0 ? i : i - static_cast<int>(__ldg(P.ends + ps - 1));
  return ps;
}

template <bool FAST>
struct PodEval {
  PodAt c;
  PodVec gv;
  int g_i;
  __device__ __forceinline__ void init(const DevPOD& P, int part, int local, double T) {
    c = pod_at(P, part, T);
    g_i = local;
    if constexpr (FAST) pod_vec(c, local, gv);
  }
  __device__ __forceinline__ double operator()(int cdf_i) const {
    if constexpr (FAST) return pod_eval_fast(c, gv, cdf_i);
    else return pod_eval(c, cdf_i, g_i);
  }
  // fast form: the reconstruction in FP32, without the conversion
  __device__ __forceinline__ float f32(int cdf_i) const {
    const float* C = c.cs + static_cast<size_t>(cdf_i) * c.r;
    float acc = 0.0f;
#pragma unroll
    for (int o = 0; o < kFastPodRank; o++)
      if (o < c.r) acc = __fmaf_rn(__ldg(C + o), gv.v[o], acc);
    return acc;
  }
};

// ThermalScattering::EvaluateInelastic
__device__ __forceinline__ double tsl_inelastic(const DevTSL& t, int E_i, int T_i) {
  const int r = t.xs_rank;
  double acc = 0;
  for (int o = 0; o < r; o++)
    acc = dadd(acc, dmul(dmul(__ldg(t.xs_S + o), __ldg(t.xs_Em + E_i * r + o)), __ldg(t.xs_Tm + T_i * r + o)));
  return acc;
}

// ThermalScattering::GetTotal
__device__ __forceinline__ double tsl_total(const DevTSL& t, double E, double T) {
  const int E_hi_i = upper_index(t.xs_E, t.xs_nE, E);
  if (E_hi_i == t.xs_nE) return CUDART_NAN;  // E at or above the cutoff (asserted by the reference)
  const bool below_E_min = E_hi_i == 0;
  const int E_lo_i = below_E_min ? E_hi_i : E_hi_i - 1;
  const int cand = upper_index(t.xs_T, t.xs_nT, T);
  const bool above_T_max = cand == t.xs_nT;
  const int T_hi_i = above_T_max ? cand - 1 : cand;
  const bool below_T_min = T_hi_i == 0;
  const int T_lo_i = below_T_min ? T_hi_i : T_hi_i - 1;
  const double a = tsl_inelastic(t, E_lo_i, T_lo_i), b = tsl_inelastic(t, E_lo_i, T_hi_i);
  const double c = tsl_inelastic(t, E_hi_i, T_lo_i), d = tsl_inelastic(t, E_hi_i, T_hi_i);
  const double E_lo = __ldg(t.xs_E + E_lo_i), E_hi = __ldg(t.xs_E + E_hi_i);
  const double r_E = below_E_min ? 1.0 : ddiv(dsub(E, E_lo), dsub(E_hi, E_lo));
  const double xs_T_lo = dadd(a, dmul(r_E, dsub(c, a)));
  const double xs_T_hi = dadd(b, dmul(r_E, dsub(d, b)));
  const double T_lo = __ldg(t.xs_T + T_lo_i), T_hi = __ldg(t.xs_T + T_hi_i);
  const double r_T = below_T_min ? 1.0 : above_T_max ? 0.0 : ddiv(dsub(T, T_lo), dsub(T_hi, T_lo));
  return dadd(xs_T_lo, dmul(r_T, dsub(xs_T_hi, xs_T_lo)));
}

// GetTotal's form for fast-mode transport: the same brackets and weights,
// the rank sums in FP32
__device__ __forceinline__ float tsl_inelastic_f(const DevTSL& t, int E_i, int T_i) {
  const int r = t.xs_rank;
  const float* a = t.xs_EmS_f + static_cast<size_t>(E_i) * r;
  const float* b = t.xs_Tm_f + static_cast<size_t>(T_i) * r;
  float acc = 0.0f;
  for (int o = 0; o < r; o++) acc = fmaf(__ldg(a + o), __ldg(b + o), acc);
  return acc;
}

__device__ __forceinline__ double tsl_total_fast(const DevTSL& t, double E, double T) {
  const int E_hi_i = upper_index(t.xs_E, t.xs_nE, E);
  if (E_hi_i == t.xs_nE) return CUDART_NAN;
  const bool below_E_min = E_hi_i == 0;
  const int E_lo_i = below_E_min ? E_hi_i : E_hi_i - 1;
  const int cand = upper_index(t.xs_T, t.xs_nT, T);
  const bool above_T_max = cand == t.xs_nT;
  const int T_hi_i = above_T_max ? cand - 1 : cand;
  const bool below_T_min = T_hi_i == 0;
  const int T_lo_i = below_T_min ? T_hi_i : T_hi_i - 1;
  const float a = tsl_inelastic_f(t, E_lo_i, T_lo_i), b = tsl_inelastic_f(t, E_lo_i, T_hi_i);
  const float c = tsl_inelastic_f(t, E_hi_i, T_lo_i), d = tsl_inelastic_f(t, E_hi_i, T_hi_i);
  const double E_lo = __ldg(t.xs_E + E_lo_i), E_hi = __ldg(t.xs_E + E_hi_i);
  const float r_E = below_E_min ? 1.0f : __fdiv_rn(__double2float_rn(E - E_lo), __double2float_rn(E_hi - E_lo));
  const float lo = fmaf(r_E, c - a, a), hi = fmaf(r_E, d - b, b);
  const double T_lo = __ldg(t.xs_T + T_lo_i), T_hi = __ldg(t.xs_T + T_hi_i);
  const float r_T = below_T_min  ? 1.0f
                    : above_T_max ? 0.0f
                                  : __fdiv_rn(__double2float_rn(T - T_lo), __double2float_rn(T_hi - T_lo));
  return static_cast<double>(fmaf(r_T, hi - lo, lo));
}

// ThermalScattering::GetMajorant: ContinuousMap::at on the majorant table
__device__ __forceinline__ double tsl_majorant(const DevTSL& t, double E) {
  const int hi = upper_index(t.maj_x, t.maj_n, E);
  if (hi == t.maj_n) return __ldg(t.maj_y + t.maj_n - 1);
  if (hi == 0) return __ldg(t.maj_y);
  const double k_hi = __ldg(t.maj_x + hi), v_hi = __ldg(t.maj_y + hi);
  const double k_lo = __ldg(t.maj_x + hi - 1), v_lo = __ldg(t.maj_y + hi - 1);
  return dadd(v_lo, dmul(ddiv(dsub(v_hi, v_lo), dsub(k_hi, k_lo)), dsub(E, k_lo)));
}

// ThermalScattering::SampleBeta; false past the resample limit (the
// reference throws)
template <bool FAST, class Rng>
__device__ __forceinline__ bool tsl_sample_beta(const DevTSL& t, Rng& rng, double E, double T, double& beta) {
  const DevPOD& P = t.beta;
  const int n = P.n_grid;
  const int E_hi_i = upper_index(P.grid, n, E);
  if (E_hi_i == n) return false;  // E at or above the cutoff (asserted by the reference)
  const double r = E_hi_i != 0 ? sdiv<FAST>(dsub(E, __ldg(P.grid + E_hi_i - 1)),
                                            dsub(__ldg(P.grid + E_hi_i), __ldg(P.grid + E_hi_i - 1)))
                               : 1.0;
  const int E_s_i = r <= su01<FAST>(rng) ? E_hi_i - 1 : E_hi_i;
  const double E_s = __ldg(P.grid + E_s_i);
  int local;
  const int ps = pod_partition(P, E_s_i, local);
  PodEval<FAST> ev;
  ev.init(P, ps, local, T);
  const int nF = ev.c.nF;
  const double kT = dmul(kBoltzmann, T);
  for (int res = 0; res < kTslResampleLimit; res++) {
    const double F = su01<FAST>(rng);
    const int F_hi_i = upper_index(ev.c.F, nF, F);
    const double F_lo = F_hi_i != 0 ? __ldg(ev.c.F + F_hi_i - 1) : 0.0;
    const double F_hi = F_hi_i != nF ? __ldg(ev.c.F + F_hi_i) : 1.0;
    const double b_lo = F_hi_i != 0 ? ev(F_hi_i - 1) : sdiv<FAST>(-E_s, kT);
    const double b_hi = F_hi_i != nF ? ev(F_hi_i) : t.beta_cutoff;
    const double b_prime = dadd(b_lo, dmul(sdiv<FAST>(dsub(F, F_lo), dsub(F_hi, F_lo)), dsub(b_hi, b_lo)));
    const double b_min = sdiv<FAST>(-E, kT);
    if (b_min <= b_prime) {
      beta = b_prime;
      return true;
    }
  }
  return false;
}

// (sqrt(E) -+ sqrt(E + b kT))^2 / (A kT): alpha bounds at beta b
template <bool FAST>
__device__ __forceinline__ void alpha_bounds(double sqrt_E, double E, double b, double T, double akT, double& a_min,
                                             double& a_max) {
  const double s = ssqrt<FAST>(dadd(E, dmul(dmul(b, kBoltzmann), T)));
  const double lo = dsub(sqrt_E, s), hi = dadd(sqrt_E, s);
  a_min = sdiv<FAST>(dmul(lo, lo), akT);
  a_max = sdiv<FAST>(dmul(hi, hi), akT);
}

// ThermalScattering::SampleAlpha (src/ThermalScattering.cpp:340-463), in
// three steps so that a batched sampler can replace the CDF search between
// them: alpha_begin (beta grid choice, kinematic bounds, partition), the
// find_cdf of the two bounds, alpha_end (the resampling loop)
template <bool FAST>
struct AlphaCtx {
  double b, E, T;
  double sqrt_E, akT;
  double b_s, b_s_a_min, b_s_a_max;
  int b_s_i, nF;
  const double* Fs;
  PodEval<FAST> ev;
};

// everything of SampleAlpha that follows from the chosen beta grid point
// b_s_i (no random draw), so a sampler may rebuild it after other work
template <bool FAST>
__device__ __forceinline__ void alpha_setup(const DevTSL& t, double b, double E, double T, int b_s_i,
                                            AlphaCtx<FAST>& x) {
  const DevPOD& P = t.alpha;
  const int sgn_b = (0 < b) - (b < 0);
  x.b = b;
  x.E = E;
  x.T = T;
  x.b_s_i = b_s_i;
  x.b_s = static_cast<double>(sgn_b) * __ldg(P.grid + b_s_i);
  x.sqrt_E = ssqrt<FAST>(E);
  x.akT = dmul(dmul(t.awr, kBoltzmann), T);
  alpha_bounds<FAST>(x.sqrt_E, E, x.b_s, T, x.akT, x.b_s_a_min, x.b_s_a_max);
  int local;
  const int ps = pod_partition(P, b_s_i, local);
  x.ev.init(P, ps, local, T);
  x.nF = x.ev.c.nF;
  x.Fs = x.ev.c.F;
}

template <bool FAST, class Rng>
__device__ __forceinline__ bool alpha_begin(const DevTSL& t, Rng& rng, double b, double E, double T, AlphaCtx<FAST>& x) {
  const DevPOD& P = t.alpha;
  const double abs_b = fabs(b);
  const int sgn_b = (0 < b) - (b < 0);
  const int n = P.n_grid;
  const int b_hi_i = upper_index(P.grid, n, abs_b);
  if (b_hi_i == n) return false;  // betas.at() throws in the reference
  const double kT = dmul(kBoltzmann, T);
  const double g_hi = __ldg(P.grid + b_hi_i);
  const bool snap_to_lower = (sgn_b == 1 && t.beta_cutoff <= g_hi) || (sgn_b == -1 && -g_hi < sdiv<FAST>(-E, kT));
  const bool snap_to_min = b_hi_i == 0;
  double r;
  if (snap_to_lower) r = 0.0;
  else if (snap_to_min) r = 1.0;
  else {
    // as written in the reference (src/ThermalScattering.cpp:363-365): the
    // division binds before the subtraction
    const double g_lo = __ldg(P.grid + b_hi_i - 1);
    r = dsub(abs_b, sdiv<FAST>(g_lo, dsub(g_hi, g_lo)));
  }
  const int b_s_i = r <= su01<FAST>(rng) ? b_hi_i - 1 : b_hi_i;
  if (b_s_i < 0) return false;  // snapped below the first beta: betas.at() throws in the reference
  alpha_setup<FAST>(t, b, E, T, b_s_i, x);
  return true;
}

// find_cdf's search: std::upper_bound over CDF indices with a < Evaluate(i)
// (the fast form compares in FP32: its reconstructions are FP32 values)
template <bool FAST>
__device__ __forceinline__ bool cdf_pred(const AlphaCtx<FAST>& x, double a, float af, int i) {
  if constexpr (FAST) return af < x.ev.f32(i);
  else return a < x.ev(i);
}

template <bool FAST>
__device__ __forceinline__ int cdf_upper_bisect(const AlphaCtx<FAST>& x, double a) {
  int first = 0, len = x.nF;
  const float af = __double2float_rn(a);
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (cdf_pred(x, a, af, mid)) {
      len = half;
    }
    else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  return first;
}

// The same index from a starting guess i0 (a learned prediction): probe
// i0 and its neighbour, walk away from them with doubling steps until the
// answer is bracketed, then bisect the bracket.  For a non-decreasing
// sequence of reconstructions (the POD pipeline removes CDFs that are not)
// this is exactly upper_bound's answer, with 2 evaluations when the guess
// is right instead of log2(nF).
template <bool FAST>
__device__ __forceinline__ int cdf_upper_guided(const AlphaCtx<FAST>& x, double a, int i0) {
  const int nF = x.nF;
  const float af = __double2float_rn(a);
  int lo, hi;  // answer in [lo, hi]: pred false below lo, pred(hi) true or hi == nF
  const int g = i0 < 0 ? 0 : (i0 > nF ? nF : i0);
  if (g < nF && !cdf_pred(x, a, af, g)) {
    lo = g + 1;
    hi = nF;
    for (int step = 1; lo < nF;) {
      const int j = g + step < nF ? g + step : nF - 1;
      if (cdf_pred(x, a, af, j)) {
        hi = j;
        break;
      }
      lo = j + 1;
      if (j == nF - 1) break;
      step <<= 1;
    }
  }
  else {
    hi = g;
    lo = 0;
    for (int step = 1; hi > 0;) {
      const int j = g - step > 0 ? g - step : 0;
      if (!cdf_pred(x, a, af, j)) {
        lo = j + 1;
        break;
      }
      hi = j;
      if (j == 0) break;
      step <<= 1;
    }
  }
  // bisect [lo, hi): hi is known to satisfy the predicate (or be nF)
  int first = lo, len = hi - lo;
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (cdf_pred(x, a, af, mid)) {
      len = half;
    }
    else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  return first;
}

// The last two reconstructions a search evaluated, (index, value): the
// guided search's confirming probes are the bracket that cdf_at reads, so
// keeping them saves two reconstructions per bound (the values are the
// same ones cdf_at would compute).
struct Probes {
  int i0 = -1, i1 = -1;
  double v0 = 0, v1 = 0;
  __device__ __forceinline__ void put(int i, double v) {
    i1 = i0;
    v1 = v0;
    i0 = i;
    v0 = v;
  }
  __device__ __forceinline__ bool get(int i, double& v) const {
    if (i == i0) {
      v = v0;
      return true;
    }
    if (i == i1) {
      v = v1;
      return true;
    }
    return false;
  }
};

// cdf_pred, keeping the reconstruction it evaluates
template <bool FAST>
__device__ __forceinline__ bool cdf_pred_kept(const AlphaCtx<FAST>& x, double a, float af, int i, Probes& pr) {
  if constexpr (FAST) {
    const float v = x.ev.f32(i);
    pr.put(i, static_cast<double>(v));
    return af < v;
  }
  else {
    const double v = x.ev(i);
    pr.put(i, v);
    return a < v;
  }
}

// cdf_upper_guided, keeping its last two reconstructions in pr
template <bool FAST>
__device__ __forceinline__ int cdf_upper_guided_kept(const AlphaCtx<FAST>& x, double a, int i0, Probes& pr) {
  const int nF = x.nF;
  const float af = __double2float_rn(a);
  int lo, hi;
  const int g = i0 < 0 ? 0 : (i0 > nF ? nF : i0);
  if (g < nF && !cdf_pred_kept(x, a, af, g, pr)) {
    lo = g + 1;
    hi = nF;
    for (int step = 1; lo < nF;) {
      const int j = g + step < nF ? g + step : nF - 1;
      if (cdf_pred_kept(x, a, af, j, pr)) {
        hi = j;
        break;
      }
      lo = j + 1;
      if (j == nF - 1) break;
      step <<= 1;
    }
  }
  else {
    hi = g;
    lo = 0;
    for (int step = 1; hi > 0;) {
      const int j = g - step > 0 ? g - step : 0;
      if (!cdf_pred_kept(x, a, af, j, pr)) {
        lo = j + 1;
        break;
      }
      hi = j;
      if (j == 0) break;
      step <<= 1;
    }
  }
  int first = lo, len = hi - lo;
  while (len > 0) {
    const int half = len >> 1, mid = first + half;
    if (cdf_pred_kept(x, a, af, mid, pr)) {
      len = half;
    }
    else {
      first = mid + 1;
      len -= half + 1;
    }
  }
  return first;
}

// the CDF value of `a` from its bracket (assuming a histogram PDF)
template <bool FAST>
__device__ __forceinline__ double cdf_at(const DevTSL& t, const AlphaCtx<FAST>& x, double a, int F_a_hi_i) {
  const int nF = x.nF;
  const double F_a_lo = F_a_hi_i != 0 ? __ldg(x.Fs + F_a_hi_i - 1) : 0.0;
  const double F_a_hi = F_a_hi_i != nF ? __ldg(x.Fs + F_a_hi_i) : 1.0;
  const double a_lo = F_a_hi_i != 0 ? x.ev(F_a_hi_i - 1) : 0.0;
  const double a_hi = F_a_hi_i != nF ? x.ev(F_a_hi_i) : t.alpha_cutoff;
  return dadd(F_a_lo, sdiv<FAST>(dmul(dsub(a, a_lo), dsub(F_a_hi, F_a_lo)), dsub(a_hi, a_lo)));
}

// cdf_at with the bracket's reconstructions taken from pr where it holds them
template <bool FAST>
__device__ __forceinline__ double cdf_at_kept(const DevTSL& t, const AlphaCtx<FAST>& x, double a, int F_a_hi_i,
                                              const Probes& pr) {
  const int nF = x.nF;
  const double F_a_lo = F_a_hi_i != 0 ? __ldg(x.Fs + F_a_hi_i - 1) : 0.0;
  const double F_a_hi = F_a_hi_i != nF ? __ldg(x.Fs + F_a_hi_i) : 1.0;
  double a_lo = 0.0, a_hi = t.alpha_cutoff;
  if (F_a_hi_i != 0 && !pr.get(F_a_hi_i - 1, a_lo)) a_lo = x.ev(F_a_hi_i - 1);
  if (F_a_hi_i != nF && !pr.get(F_a_hi_i, a_hi)) a_hi = x.ev(F_a_hi_i);
  return dadd(F_a_lo, sdiv<FAST>(dmul(dsub(a, a_lo), dsub(F_a_hi, F_a_lo)), dsub(a_hi, a_lo)));
}

// the fractional index position of `a` in [0, 1]: (upper index + where a
// falls in its bracket) / (nF + 1) -- what the guide network learns
template <bool FAST>
__device__ __forceinline__ float cdf_position(const DevTSL& t, const AlphaCtx<FAST>& x, double a, int F_a_hi_i) {
  const int nF = x.nF;
  const double a_lo = F_a_hi_i != 0 ? x.ev(F_a_hi_i - 1) : 0.0;
  const double a_hi = F_a_hi_i != nF ? x.ev(F_a_hi_i) : t.alpha_cutoff;
  float th = static_cast<float>((a - a_lo) / (a_hi - a_lo));
  th = th == th ? fminf(0.999f, fmaxf(0.0f, th)) : 0.5f;
  return (static_cast<float>(F_a_hi_i) + th) / static_cast<float>(nF + 1);
}

template <bool FAST, class Rng>
__device__ __forceinline__ bool alpha_end(const DevTSL& t, Rng& rng, const AlphaCtx<FAST>& x, double F_min,
                                          double F_max, double& alpha) {
  const int nF = x.nF;
  const double* Fs = x.Fs;
  for (int res = 0; res < kTslResampleLimit; res++) {
    const double F = dadd(F_min, dmul(su01<FAST>(rng), dsub(F_max, F_min)));
    const int F_hi_i = upper_index(Fs, nF, F);
    const double F_lo = F_hi_i != 0 ? __ldg(Fs + F_hi_i - 1) : 0.0;
    const double F_hi = F_hi_i != nF ? __ldg(Fs + F_hi_i) : 1.0;
    const double a_lo = F_hi_i != 0 ? x.ev(F_hi_i - 1) : 0.0;
    const double a_hi = F_hi_i != nF ? x.ev(F_hi_i) : t.alpha_cutoff;
    const double a_prime = dadd(a_lo, dmul(sdiv<FAST>(dsub(F, F_lo), dsub(F_hi, F_lo)), dsub(a_hi, a_lo)));
    if (x.b_s_a_min < a_prime && a_prime < x.b_s_a_max) {
      double b_a_min, b_a_max;
      alpha_bounds<FAST>(x.sqrt_E, x.E, x.b, x.T, x.akT, b_a_min, b_a_max);
      alpha = dadd(b_a_min, sdiv<FAST>(dmul(dsub(a_prime, x.b_s_a_min), dsub(b_a_max, b_a_min)),
                                       dsub(x.b_s_a_max, x.b_s_a_min)));
      return true;
    }
  }
  return false;
}

// ThermalScattering::SampleAlpha
template <bool FAST, class Rng>
__device__ __forceinline__ bool tsl_sample_alpha(const DevTSL& t, Rng& rng, double b, double E, double T,
                                                 double& alpha) {
  AlphaCtx<FAST> x;
  if (!alpha_begin<FAST>(t, rng, b, E, T, x)) return false;
  const double F_min = cdf_at<FAST>(t, x, x.b_s_a_min, cdf_upper_bisect<FAST>(x, x.b_s_a_min));
  const double F_max = cdf_at<FAST>(t, x, x.b_s_a_max, cdf_upper_bisect<FAST>(x, x.b_s_a_max));
  return alpha_end<FAST>(t, rng, x, F_min, F_max, alpha);
}

// ThermalScattering::Scatter: beta, alpha -> E', mu; Particle::Scatter
// rotates the direction by mu with a fresh azimuth
// Scatter's kinematics for a sampled (beta, alpha): E' = E + beta kT and the
// cosine, then Particle::Scatter's rotation with a fresh azimuth
template <bool FAST, class Rng>
__device__ __forceinline__ void tsl_apply(const DevTSL& t, Rng& rng, double T, double beta, double alpha, double& E,
                                          double& du, double& dv, double& dw) {
  const double E_p = dadd(E, dmul(dmul(beta, kBoltzmann), T));
  if constexpr (FAST && std::is_same_v<Rng, PhiloxRng>) {
    // E' and mu from the sampled pair, the direction in FP32
    const float mu = fminf(1.0f, fmaxf(-1.0f, __fdiv_rn(__double2float_rn(dsub(dadd(E, E_p),
                                                                                  dmul(dmul(dmul(alpha, t.awr),
                                                                                            kBoltzmann), T))),
                                                         __fmul_rn(2.0f, __fsqrt_rn(__double2float_rn(dmul(E, E_p)))))));
    float dx = static_cast<float>(du), dy = static_cast<float>(dv), dz = static_cast<float>(dw);
    rotate_f(dx, dy, dz, mu, rng.u01f());
    du = dx;
    dv = dy;
    dw = dz;
  }
  else {
    const double mu = ddiv(dsub(dadd(E, E_p), dmul(dmul(dmul(alpha, t.awr), kBoltzmann), T)),
                           dmul(2.0, __dsqrt_rn(dmul(E, E_p))));
    const double phi = dmul(2 * kPi, rng.u01());
    rotate(du, dv, dw, mu, phi);
  }
  E = E_p;
}

template <bool FAST, class Rng>
__device__ __forceinline__ bool tsl_scatter_body(const DevTSL& t, Rng& rng, double T, double& E, double& du, double& dv,
                                            double& dw) {
  double beta, alpha;
  if (!tsl_sample_beta<FAST>(t, rng, E, T, beta)) return false;
  if (!tsl_sample_alpha<FAST>(t, rng, beta, E, T, alpha)) return false;
  tsl_apply<FAST>(t, rng, T, beta, alpha, E, du, dv, dw);
  return true;
}

template <bool FAST, class Rng>
__device__ __forceinline__ bool tsl_scatter(const DevTSL& t, Rng& rng, double T, double& E, double& du, double& dv,
                                            double& dw) {
  return tsl_scatter_body<FAST>(t, rng, T, E, du, dv, dw);
}

}  // namespace mcd
