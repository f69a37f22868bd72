// Continuous-energy physics on the device:
//   ContinuousMap::at                 src/ContinuousMap.hpp:21-39
//   Continuous::GetTotal/GetMajorant  src/Continuous.cpp:26-58
//   ContinuousReaction cross sections src/ContinuousReaction.cpp:45-120
//   free-gas elastic scattering       src/ContinuousReaction.cpp:119-189
//   free-gas cross-section adjustment src/ContinuousReaction.cpp:205-237
//
// Two forms share one energy search:
//   exact: each table's own energies and values in FP64, the reference's
//          formulas and rounding (bit-for-bit with the reference's
//          arithmetic for the same random numbers);
//   fast:  FP32 tables on the unionized grid (see mc_ce_tables.hpp), FP32
//          free-gas kinematics; statistically equivalent.
#pragma once

#include "mc_device.cuh"
#include "mc_tsl.cuh"

namespace mcd {

// ---------------------------------------------------------------------------
// energy search: j = upper_bound(union, E), exactly as std::map::upper_bound
// orders doubles.  Positive doubles compare like their bit patterns, so the
// search runs on integers from a bucket of the key.
__device__ __forceinline__ int ce_search(const DevCE& ce, double E) {
  const int nu = ce.nu;
  if (!(E < __ldg(ce.ue + nu - 1))) return nu;  // at or past the end, or NaN
  if (E < __ldg(ce.ue)) return 0;
  const unsigned long long k = static_cast<unsigned long long>(__double_as_longlong(E));
  const unsigned b = static_cast<unsigned>((k - ce.key0) >> ce.shift);
  unsigned lo = __ldg(ce.bucket + b), hi = __ldg(ce.bucket + b + 1);
  while (lo < hi) {
    const unsigned mid = (lo + hi) >> 1;
    if (__ldg(ce.ukey + mid) > k) hi = mid;
    else lo = mid + 1;
  }
  return static_cast<int>(lo);
}

// upper_bound position of union point j in table `tab`'s own energies
__device__ __forceinline__ uint32_t ce_table_index(const DevCE& ce, int tab, int j) {
  return __ldg(ce.umap + static_cast<size_t>(__ldg(ce.tab_grid + tab)) * (ce.nu + 1) + j) ;
}

// ContinuousMap::at with the reference's rounding
__device__ __forceinline__ double ce_table_at(const DevCE& ce, int tab, int j, double E) {
  const uint32_t off = __ldg(ce.tab_off + tab);
  const uint32_t len = __ldg(ce.tab_off + tab + 1) - off;
  const uint32_t hi = ce_table_index(ce, tab, j);
  if (hi == len) return __ldg(ce.tab_y + off + len - 1);
  if (hi == 0) return __ldg(ce.tab_y + off);
  const double k_hi = __ldg(ce.tab_x + off + hi), v_hi = __ldg(ce.tab_y + off + hi);
  const double k_lo = __ldg(ce.tab_x + off + hi - 1), v_lo = __ldg(ce.tab_y + off + hi - 1);
  return dadd(v_lo, dmul(ddiv(dsub(v_hi, v_lo), dsub(k_hi, k_lo)), dsub(E, k_lo)));
}

// ScalarField::at at a point of the cell, and the field's upper bound
// (src/ScalarField.cpp:41-59)
__device__ __forceinline__ double cell_temperature(const DevWorld& w, int cell, double x, double y, double z) {
  const double* f = w.field + 8 * __ldg(w.cell_field + cell);
  if (__ldg(f) == 0) return __ldg(f + 1);
  return dadd(dadd(dadd(dmul(__ldg(f + 2), x), dmul(__ldg(f + 3), y)), dmul(__ldg(f + 4), z)), __ldg(f + 5));
}
__device__ __forceinline__ double cell_temperature_max(const DevWorld& w, int cell) {
  return __ldg(w.field + 8 * __ldg(w.cell_field + cell) + 6);
}

// ContinuousEvaluation::IsValid: signed relative difference below 1 %
__device__ __forceinline__ bool ce_valid(double evaluated, double requested) {
  return ddiv(dsub(requested, evaluated), evaluated) < 0.01;
}

// ContinuousScatter::IsFreeGasScatteringValid
__device__ __forceinline__ bool ce_free_gas_valid(double awr, int type, double E, double T) {
  if (type != 0) return false;
  if (awr <= 1.0) return true;
  return E < ddiv(dmul(dmul(500.0, kBoltzmann), T), awr);
}

// ContinuousScatter::GetFreeGasScatterAdjustment
__device__ __forceinline__ double ce_free_gas_adjustment(double awr, double E, double T) {
  if (T == 0) return 1.0;
  const double x = __dsqrt_rn(ddiv(E, dmul(kBoltzmann, T)));
  const double arg = dmul(dmul(awr, x), x);
  return dadd(dmul(dadd(1.0, ddiv(1.0, dmul(2.0, arg))), erf(__dsqrt_rn(arg))),
              ddiv(exp(-arg), __dsqrt_rn(dmul(kPi, arg))));
}

__device__ __forceinline__ const mc::CENuclideDesc& ce_desc(const DevWorld& w, int type, int nuc) {
  return w.ce.nuc[type * w.n_nuclides + nuc];
}

// ThermalScattering::IsValid: a library on reaction k, a neutron below the
// library's cutoff energy
__device__ __forceinline__ bool ce_tsl_valid(const DevWorld& w, const mc::CENuclideDesc& d, int k, int type, double E) {
  const int t = d.rx_tsl[k];
  return t >= 0 && type == 0 && E < w.tsl[t].cutoff_energy;
}

// ThermalScattering::GetTotal is a pure function of (library, E, T) and the
// history loop asks for it several times per event (flight, nuclide choice,
// reaction choice) at the same arguments: one value per particle is kept.
// The reference recomputes it; the memo returns the identical double.
// In fast mode (Philox streams, FP32 sampling arithmetic) the memo also
// selects the FP32 rank sums.
struct TslMemo {
  int t = -1;
  bool fast32 = false;
  double E = 0, T = 0, v = 0;
};

__device__ __forceinline__ double tsl_total_memo(const DevWorld& w, int ti, double E, double T, TslMemo* memo) {
  if (memo && memo->t == ti && memo->E == E && memo->T == T) return memo->v;
  const double v = memo && memo->fast32 ? tsl_total_fast(w.tsl[ti], E, T) : tsl_total(w.tsl[ti], E, T);
  if (memo) {
    memo->t = ti;
    memo->E = E;
    memo->T = T;
    memo->v = v;
  }
  return v;
}

// ContinuousReaction::GetCrossSection (majorant = false) or GetMajorant
// (majorant = true).  T is the temperature the free-gas rules use (the
// particle's, or the cell's maximum for majorants); T_pos is the particle's
// (thermal scattering totals).
__device__ __forceinline__ double ce_reaction_xs(const DevWorld& w, const mc::CENuclideDesc& d, int k, int type,
                                                 int j, double E, double T, double T_pos, bool majorant,
                                                 TslMemo* memo = nullptr) {
  if (d.rx_kind[k] == 1 && ce_tsl_valid(w, d, k, type, E)) {
    if (majorant) return tsl_majorant(w.tsl[d.rx_tsl[k]], E);
    return tsl_total_memo(w, d.rx_tsl[k], E, T_pos, memo);
  }
  const double xs = ce_table_at(w.ce, d.rx_table[k], j, E);
  if (d.rx_kind[k] != 1) return xs;
  if (ce_valid(d.rx_T[k], T)) return xs;
  if (ce_free_gas_valid(d.awr, type, E, T))
    return dmul(ddiv(xs, ce_free_gas_adjustment(d.awr, E, d.rx_T[k])), ce_free_gas_adjustment(d.awr, E, T));
  return xs;
}

// Continuous::GetTotal / GetMajorant (src/Continuous.cpp:26-58)
__device__ __forceinline__ double ce_nuclide_total(const DevWorld& w, const mc::CENuclideDesc& d, int type, int j,
                                                   double E, double T, double T_pos, bool majorant,
                                                   TslMemo* memo = nullptr) {
  bool modifies = false;  // Continuous::ReactionsModifyTotal
  for (int k = 0; k < d.n_rx; k++) modifies |= d.rx_kind[k] == 1 && ce_tsl_valid(w, d, k, type, E);
  if (!modifies && ce_valid(d.total_T, T)) return ce_table_at(w.ce, d.total, j, E);
  double acc = 0;
  for (int k = 0; k < d.n_rx; k++) acc = dadd(acc, ce_reaction_xs(w, d, k, type, j, E, T, T_pos, majorant, memo));
  return acc;
}

// Material::GetMicroscopicTotal (or Majorant) in the reference's summation
// order
__device__ __forceinline__ double ce_material_micro(const DevWorld& w, int mat, int type, int j, double E, double T,
                                                    double T_pos, bool majorant, TslMemo* memo = nullptr) {
  const int nb = __ldg(w.mat_begin + mat), ne = __ldg(w.mat_begin + mat + 1);
  double acc = 0;
  for (int i = nb; i < ne; i++)
    acc = dadd(acc, dmul(__ldg(w.mat_afrac + i), ce_nuclide_total(w, ce_desc(w, type, __ldg(w.mat_nuc + i)), type, j,
                                                                  E, T, T_pos, majorant, memo)));
  return acc;
}

// sum of afrac * nubar * sigma_f (track-length k, an extension)
__device__ __forceinline__ double ce_material_nusigf(const DevWorld& w, int mat, int type, int j, double E) {
  const int nb = __ldg(w.mat_begin + mat), ne = __ldg(w.mat_begin + mat + 1);
  double acc = 0;
  for (int i = nb; i < ne; i++) {
    const mc::CENuclideDesc& d = ce_desc(w, type, __ldg(w.mat_nuc + i));
    for (int k = 0; k < d.n_rx; k++) {
      if (d.rx_kind[k] == 2 && d.rx_nubar[k] >= 0)
        acc = dadd(acc, dmul(__ldg(w.mat_afrac + i),
                             dmul(ce_table_at(w.ce, d.rx_nubar[k], j, E), ce_table_at(w.ce, d.rx_table[k], j, E))));
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// FP32 union tables: the bracket [jl, jh] and weight of E, snapped at both
// ends like ContinuousMap::at
struct UnionPos {
  int jl, jh;
  float f;
};
__device__ __forceinline__ UnionPos ce_union_pos(const DevCE& ce, int j, double E) {
  UnionPos u;
  if (j <= 0 || j >= ce.nu) {
    u.jl = u.jh = j <= 0 ? 0 : ce.nu - 1;
    u.f = 0.0f;
  }
  else {
    u.jl = j - 1;
    u.jh = j;
    u.f = __fmul_rn(__double2float_rn(dsub(E, __ldg(ce.ue + j - 1))), __ldg(ce.uinv + j));
  }
  return u;
}
__device__ __forceinline__ float lerpf(float lo, float hi, float f) { return __fmaf_rn(f, __fsub_rn(hi, lo), lo); }

// ---------------------------------------------------------------------------
// free-gas elastic scattering (ContinuousScatter::Interact without a thermal
// scattering library).  The target speed x (in units of 1/beta) and the
// cosine mu between neutron and target velocities are sampled by rejection
// (MCNP's C49/C61 mixture, OpenMC eq. 75), the collision is elastic and
// isotropic in the centre-of-mass frame, and Particle::Scatter rotates the
// flight direction by the lab cosine with a fresh azimuth.
// Returns false if the rejection loop gave up (never in practice).
constexpr int kFreeGasTries = 1000;

template <class Rng>
__device__ __forceinline__ bool free_gas_exact(Rng& rng, double awr, double T, double& E, double& du, double& dv,
                                               double& dw) {
  const double m_n = kNeutronMass;
  const double s_n = __dsqrt_rn(ddiv(dmul(2.0, E), m_n));
  const double vnx = dmul(du, s_n), vny = dmul(dv, s_n), vnz = dmul(dw, s_n);
  const double beta = __dsqrt_rn(ddiv(dmul(awr, m_n), dmul(dmul(2.0, kBoltzmann), T)));
  const double y = dmul(beta, s_n);
  const double branch = ddiv(2.0, dadd(dmul(__dsqrt_rn(kPi), y), 2.0));
  double x = 0, mu = 0;
  bool ok = false;
  for (int it = 0; it < kFreeGasTries; it++) {
    const double xi_1 = rng.u01();
    const double xi_2 = rng.u01();
    if (rng.u01() < branch) {
      x = __dsqrt_rn(-log(dmul(xi_1, xi_2)));
    }
    else {
      const double xi_3 = rng.u01();
      const double z = cos(ddiv(dmul(kPi, xi_3), 2.0));
      x = __dsqrt_rn(dsub(-log(xi_1), dmul(dmul(log(xi_2), z), z)));
    }
    mu = dsub(dmul(2.0, rng.u01()), 1.0);
    const double acc = ddiv(__dsqrt_rn(dsub(dadd(dmul(x, x), dmul(y, y)), dmul(dmul(dmul(2.0, x), y), mu))), dadd(x, y));
    if (!(rng.u01() >= acc)) {
      ok = true;
      break;
    }
  }
  const double s_T = ddiv(x, beta);
  const double phi = dmul(2 * kPi, rng.u01());
  double tx = du, ty = dv, tz = dw;
  rotate(tx, ty, tz, mu, phi);
  tx = dmul(tx, s_T);
  ty = dmul(ty, s_T);
  tz = dmul(tz, s_T);
  const double den = dadd(1.0, awr);
  const double cmx = ddiv(dadd(vnx, dmul(tx, awr)), den);
  const double cmy = ddiv(dadd(vny, dmul(ty, awr)), den);
  const double cmz = ddiv(dadd(vnz, dmul(tz, awr)), den);
  const double Vx = dsub(vnx, cmx), Vy = dsub(vny, cmy), Vz = dsub(vnz, cmz);
  const double mu_cm = dsub(dmul(2.0, rng.u01()), 1.0);
  const double phi_cm = dmul(2 * kPi, rng.u01());
  const double Vn = __dsqrt_rn(dot3(Vx, Vy, Vz, Vx, Vy, Vz));
  double ex = ddiv(Vx, Vn), ey = ddiv(Vy, Vn), ez = ddiv(Vz, Vn);
  rotate(ex, ey, ez, mu_cm, phi_cm);
  const double px = dadd(dmul(ex, Vn), cmx), py = dadd(dmul(ey, Vn), cmy), pz = dadd(dmul(ez, Vn), cmz);
  const double E_prime = dmul(dmul(0.5, m_n), dot3(px, py, pz, px, py, pz));
  const double pn = __dsqrt_rn(dot3(px, py, pz, px, py, pz));
  const double mu_lab = dot3(du, dv, dw, ddiv(px, pn), ddiv(py, pn), ddiv(pz, pn));
  const double phi_lab = dmul(2 * kPi, rng.u01());
  rotate(du, dv, dw, mu_lab, phi_lab);
  E = E_prime;
  return ok;
}

template <class Rng>
__device__ __forceinline__ bool free_gas_fast(Rng& rng, float awr, float T, double& E, double& du, double& dv,
                                              double& dw) {
  constexpr float m_n = 1.045354912280858e-18f;
  constexpr float two_over_m = static_cast<float>(2.0 / 1.045354912280858e-18);
  constexpr float two_k = static_cast<float>(2.0 * 8.617333262145e-11);
  float dx = static_cast<float>(du), dy = static_cast<float>(dv), dz = static_cast<float>(dw);
  const float s_n = __fsqrt_rn(__fmul_rn(static_cast<float>(E), two_over_m));
  const float beta = __fsqrt_rn(__fdiv_rn(__fmul_rn(awr, m_n), __fmul_rn(two_k, T)));
  const float y = __fmul_rn(beta, s_n);
  const float branch = __fdiv_rn(2.0f, __fmaf_rn(1.77245385090551603f, y, 2.0f));
  float x = 0.0f, mu = 0.0f;
  bool ok = false;
  for (int it = 0; it < kFreeGasTries; it++) {
    const float xi_1 = rng.u01f();
    const float xi_2 = rng.u01f();
    if (rng.u01f() < branch) {
      x = __fsqrt_rn(fmaxf(0.0f, -logf(__fmul_rn(xi_1, xi_2))));
    }
    else {
      const float z = __cosf(__fmul_rn(1.57079632679489662f, rng.u01f()));
      x = __fsqrt_rn(fmaxf(0.0f, __fsub_rn(-logf(xi_1), __fmul_rn(__fmul_rn(logf(xi_2), z), z))));
    }
    mu = __fmaf_rn(2.0f, rng.u01f(), -1.0f);
    const float rel = __fsqrt_rn(fmaxf(0.0f, __fsub_rn(__fmaf_rn(x, x, __fmul_rn(y, y)), __fmul_rn(__fmul_rn(2.0f, x), __fmul_rn(y, mu)))));
    if (rng.u01f() < __fdiv_rn(rel, __fadd_rn(x, y))) {
      ok = true;
      break;
    }
  }
  const float s_T = __fdiv_rn(x, beta);
  float tx = dx, ty = dy, tz = dz;
  rotate_f(tx, ty, tz, mu, rng.u01f());
  const float inv = __frcp_rn(__fadd_rn(1.0f, awr));
  const float vnx = __fmul_rn(dx, s_n), vny = __fmul_rn(dy, s_n), vnz = __fmul_rn(dz, s_n);
  const float ta = __fmul_rn(s_T, awr);
  const float cmx = __fmul_rn(__fmaf_rn(tx, ta, vnx), inv);
  const float cmy = __fmul_rn(__fmaf_rn(ty, ta, vny), inv);
  const float cmz = __fmul_rn(__fmaf_rn(tz, ta, vnz), inv);
  const float Vx = __fsub_rn(vnx, cmx), Vy = __fsub_rn(vny, cmy), Vz = __fsub_rn(vnz, cmz);
  const float Vn = __fsqrt_rn(__fmaf_rn(Vx, Vx, __fmaf_rn(Vy, Vy, __fmul_rn(Vz, Vz))));
  const float rV = __frcp_rn(Vn);
  float ex = __fmul_rn(Vx, rV), ey = __fmul_rn(Vy, rV), ez = __fmul_rn(Vz, rV);
  const float mu_cm = __fmaf_rn(2.0f, rng.u01f(), -1.0f);
  const float u_phi_cm = rng.u01f();
  rotate_f(ex, ey, ez, mu_cm, u_phi_cm);
  const float px = __fmaf_rn(ex, Vn, cmx), py = __fmaf_rn(ey, Vn, cmy), pz = __fmaf_rn(ez, Vn, cmz);
  const float p2 = __fmaf_rn(px, px, __fmaf_rn(py, py, __fmul_rn(pz, pz)));
  const float mu_lab = fminf(1.0f, fmaxf(-1.0f, __fmul_rn(__fmaf_rn(dx, px, __fmaf_rn(dy, py, __fmul_rn(dz, pz))), __frsqrt_rn(p2))));
  rotate_f(dx, dy, dz, mu_lab, rng.u01f());
  E = static_cast<double>(__fmul_rn(__fmul_rn(0.5f, m_n), p2));
  du = dx;
  dv = dy;
  dw = dz;
  return ok;
}

}  // namespace mcd
