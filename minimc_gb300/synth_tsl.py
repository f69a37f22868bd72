"""Seeded synthetic thermal scattering library in the reference's POD layout.

The reference samples thermal inelastic scattering from proper orthogonal
decompositions (POD) of inverse CDFs (src/ThermalScattering.cpp:183-463),
produced by a Python pipeline that is not part of the repository, from ENDF
data that is not present either.  This module builds the same kind of
tables from an analytic scattering law:

    S_sym(alpha, beta; T) = sum_k w_k exp(-(alpha - |beta|)^2 / (4 alpha tau_k) - |beta| / 2)
                                     / sqrt(4 pi alpha tau_k)

the short-collision-time form of a free gas (tau = 1) plus an
effective-temperature component (Debye-like harmonic oscillator,
tau(T) = x coth(x), x = theta / 2T).  S_sym is symmetric in beta and the
physical law S(alpha, beta) = exp(-beta / 2) S_sym obeys detailed balance;
for tau = 1 it is the free-gas law exactly.  From it:

  * beta partitions: for incident energies E (split into contiguous ranges)
    and temperatures T, the inverse CDF of the beta marginal
    p(beta | E, T) ~ int_{alpha_min}^{alpha_max} S dalpha on
    [-E / kT, beta_cutoff], at interior CDF values F; the matrix
    [F] x [(E, T)] is truncated to rank r by SVD:
    CDF_modes [F][r], S [r], E_T_modes [E][T][r];
  * alpha partitions: for |beta| grid values and T, the inverse CDF of
    p(alpha | beta, T) ~ S_sym on [0, alpha_cutoff]; rank r:
    CDF_modes [F][r], S [r], beta_T_modes [beta][T][r];
  * total inelastic cross section sigma(E, T) =
    sigma_b A kT / (4 E) int int S dalpha dbeta, rank-r POD:
    total_E [E][r], total_S [r], total_T [T][r]; and a majorant
    1.05 * max_T sigma(E, T) on the same energies.

Axes of the order level are 0..r-1, as pandas writes them.  Every table is a
``.mctab`` file (see synth_ce.write_table).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import pod
from .synth_ce import write_table

KB = 8.617333262145e-11  # MeV / K
EV = 1e-6


def tau_of(T, theta: float = 1000.0):
    x = theta / (2.0 * np.asarray(T, dtype=np.float64))
    return x / np.tanh(x)


def s_sym(alpha, beta, T, weights=(0.6, 0.4), theta: float = 1000.0):
    """Symmetric scattering law (broadcasting)."""
    alpha = np.maximum(np.asarray(alpha, dtype=np.float64), 1e-300)
    beta = np.asarray(beta, dtype=np.float64)
    ab = np.abs(beta)
    out = 0.0
    for w, tau in zip(weights, (1.0, tau_of(T, theta))):
        out = out + w * np.exp(-(alpha - ab) ** 2 / (4 * alpha * tau) - ab / 2) / np.sqrt(4 * np.pi * alpha * tau)
    return out


def _alpha_bounds(E, beta, T, awr):
    kT = KB * T
    ep = np.maximum(E + beta * kT, 0.0)
    a_min = (np.sqrt(E) - np.sqrt(ep)) ** 2 / (awr * kT)
    a_max = (np.sqrt(E) + np.sqrt(ep)) ** 2 / (awr * kT)
    return a_min, a_max


def _int_alpha(a_lo, a_hi, beta, T, n=64):
    """int_{a_lo}^{a_hi} S_sym dalpha by Gauss-Legendre in s = sqrt(alpha)
    (the integrand 2 s S_sym is smooth at alpha = 0)."""
    x, w = np.polynomial.legendre.leggauss(n)
    s_lo, s_hi = np.sqrt(a_lo)[..., None], np.sqrt(a_hi)[..., None]
    s = 0.5 * (s_hi - s_lo) * x + 0.5 * (s_hi + s_lo)
    f = 2 * s * s_sym(s * s, np.asarray(beta)[..., None], np.asarray(T)[..., None])
    return 0.5 * (s_hi - s_lo)[..., 0] * (f * w).sum(-1)


def beta_marginal_cdf(E, T, awr, beta_cutoff, n_beta=1500):
    """beta grid on [-E/kT, beta_cutoff] and the CDF of p(beta | E, T)."""
    b = np.linspace(-E / (KB * T), beta_cutoff, n_beta)
    a_min, a_max = _alpha_bounds(E, b, T, awr)
    pdf = np.exp(-b / 2) * _int_alpha(a_min, a_max, b, np.full_like(b, T))
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (pdf[1:] + pdf[:-1]) * np.diff(b))])
    return b, cdf, cdf[-1]


def alpha_conditional_cdf(beta, T, alpha_cutoff, n_s=2000):
    """alpha grid on [0, alpha_cutoff] and the CDF of p(alpha | beta, T)."""
    s = np.linspace(0.0, np.sqrt(alpha_cutoff), n_s)
    f = 2 * s * s_sym(s * s, beta, T)
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (f[1:] + f[:-1]) * np.diff(s))])
    return s * s, cdf / cdf[-1]


def _inverse(x, cdf, F):
    """Inverse of a tabulated non-decreasing CDF at F (linear)."""
    keep = np.concatenate([[True], np.diff(cdf) > 0])
    return np.interp(F, cdf[keep], x[keep])




def cdf_grid(n):
    """Interior CDF values, denser in both tails."""
    t = (np.arange(n) + 0.5) / n
    return 0.5 * (1 - np.cos(np.pi * t))


def beta_table(Es, Ts, awr: float, beta_cutoff: float, n_F: int, sigma_b: float):
    """The full beta inverse-CDF table [F][E][T] and the total inelastic
    cross section [E][T] of the analytic law."""
    Fb = cdf_grid(n_F)
    beta_inv = np.zeros((n_F, len(Es), len(Ts)))
    xs = np.zeros((len(Es), len(Ts)))
    for i, E in enumerate(Es):
        for j, T in enumerate(Ts):
            b, cdf, tot = beta_marginal_cdf(E, T, awr, beta_cutoff)
            beta_inv[:, i, j] = _inverse(b, cdf / tot, Fb)
            xs[i, j] = sigma_b * awr * KB * T / (4 * E) * tot
    return pod.Table(Fb, np.asarray(Es, np.float64), np.asarray(Ts, np.float64), beta_inv), xs


def alpha_table(betas, Ts, alpha_cutoff: float, n_F: int):
    """The full alpha inverse-CDF table [F][|beta|][T] of the analytic law."""
    Fa = cdf_grid(n_F)
    alpha_inv = np.zeros((n_F, len(betas), len(Ts)))
    for k, b in enumerate(betas):
        for j, T in enumerate(Ts):
            a, cdf = alpha_conditional_cdf(b, T, alpha_cutoff)
            alpha_inv[:, k, j] = _inverse(a, cdf, Fa)
    return pod.Table(Fa, np.asarray(betas, np.float64), np.asarray(Ts, np.float64), alpha_inv)


def write_tsl(directory: Path, prefix: str = "tsl", awr: float = 0.999167339, sigma_b: float = 80.0,
              temperatures=None, n_E: int = 80, E_min: float = 1e-5 * EV, E_cutoff: float = 4.0 * EV,
              n_beta_grid: int = 300, beta_cutoff: float = 20.0, n_F_beta: int = 120, n_F_alpha: int = 160,
              rank: int = 30, partitions: int = 4, xs_rank: int = 10, rel_tol: float | None = None,
              device: str | None = "numpy") -> dict:
    """Writes the tables; returns the <tsl> attributes and partition files.
    Partitions are equal splits of the outer grids, truncated to `rank`, or,
    with `rel_tol`, the POD pipeline's adaptive ranks (minimc_gb300.pod)
    with non-monotone CDFs removed."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    Ts = np.asarray(temperatures if temperatures is not None else np.linspace(283.6, 623.6, 18), dtype=np.float64)
    Es = np.geomspace(E_min, E_cutoff, n_E)
    # alpha range needed at the highest energy and beta, lowest temperature
    a_max = (np.sqrt(E_cutoff) + np.sqrt(E_cutoff + beta_cutoff * KB * Ts.max())) ** 2 / (awr * KB * Ts.min())
    alpha_cutoff = float(1.25 * a_max)
    # alpha conditionals on a |beta| grid reaching the largest downscatter
    # (-beta up to E_cutoff / kT_min) and the upscatter cutoff
    beta_top = 1.02 * max(beta_cutoff, E_cutoff / (KB * Ts.min()))
    betas = np.concatenate([[1e-3], np.geomspace(1e-2, beta_top, n_beta_grid - 1)])

    def decompose(table):
        cuts = [len(a) for a in np.array_split(np.arange(len(table.outer)), partitions)]
        parts = pod.split(table, np.cumsum(cuts)[:-1])
        if rel_tol is not None:
            return pod.adaptive_coarsen(parts, rel_frobenius_norm_tol=rel_tol, device=device)
        return [pod.truncate(p, rank, device) for p in parts]

    bt, xs = beta_table(Es, Ts, awr, beta_cutoff, n_F_beta, sigma_b)
    at = alpha_table(betas, Ts, alpha_cutoff, n_F_alpha)
    files = {"beta": pod.write_partitions(decompose(bt), directory, prefix, "beta"),
             "alpha": pod.write_partitions(decompose(at), directory, prefix, "alpha")}

    # ---- total inelastic cross section and majorant
    U, S, Vt = np.linalg.svd(xs, full_matrices=False)
    r = min(xs_rank, len(S))
    U, S, V = U[:, :r], S[:r], Vt[:r].T
    tot = {"E": f"{prefix}-total-E.mctab", "S": f"{prefix}-total-S.mctab", "T": f"{prefix}-total-T.mctab",
           "majorant": f"{prefix}-majorant.mctab"}
    write_table(directory / tot["E"], [Es, np.arange(r, dtype=np.float64)], U)
    write_table(directory / tot["S"], [np.arange(r, dtype=np.float64)], S)
    write_table(directory / tot["T"], [Ts, np.arange(r, dtype=np.float64)], V)
    write_table(directory / tot["majorant"], [Es], 1.05 * xs.max(axis=1))
    return {"files": files, "total": tot, "beta_cutoff": beta_cutoff, "alpha_cutoff": alpha_cutoff,
            "awr": awr, "Es": Es, "Ts": Ts, "betas": betas, "xs": xs}


def tsl_xml(t: dict, indent: str = "          ") -> str:
    """The <tsl> node for a scatter reaction."""
    lines = [f'{indent}<tsl majorant="{t["total"]["majorant"]}" total_T="{t["total"]["T"]}"',
             f'{indent}     total_S="{t["total"]["S"]}" total_E="{t["total"]["E"]}"',
             f'{indent}     beta_cutoff="{t["beta_cutoff"]!r}" alpha_cutoff="{t["alpha_cutoff"]!r}">',
             f"{indent}  <beta_partitions>"]
    for f in t["files"]["beta"]:
        lines.append(f'{indent}    <partition CDF="{f["CDF"]}" S="{f["S"]}" E_T="{f["E_T"]}"/>')
    lines.append(f"{indent}  </beta_partitions>")
    lines.append(f"{indent}  <alpha_partitions>")
    for f in t["files"]["alpha"]:
        lines.append(f'{indent}    <partition CDF="{f["CDF"]}" S="{f["S"]}" beta_T="{f["beta_T"]}"/>')
    lines.append(f"{indent}  </alpha_partitions>")
    lines.append(f"{indent}</tsl>")
    return "\n".join(lines)


def moderator_nuclide(directory: Path, name: str = "Hmod", awr: float = 0.999167339, capture: float = 0.3,
                      elastic: float = 20.0) -> dict:
    """Continuous-energy tables of the bound nuclide (flat capture and
    elastic; below the library's cutoff the thermal library replaces the
    elastic cross section)."""
    from .synth_ce import write_flat_nuclide

    return write_flat_nuclide(directory, name, awr, capture=capture, scatter=elastic,
                              energies=np.geomspace(1e-11, 20.0, 64))


def broomstick_xml(tsl: dict, nuc: dict, histories: int = 100_000, energy: float = 1.0 * EV,
                   temperature: float = 450.0, radius: float = 0.01, cosine_bins: int = 200,
                   energy_bins: int = 200, aden: float = 0.066854, name: str = "Hmod") -> str:
    """Fixed-source broomstick: a thin cylinderx of moderator between planes
    at -+0.5e12 cm, a monoenergetic pencil beam along +x from the origin;
    the current through the cylinder is binned in cosine to +x and in
    outgoing energy (0 to 2.5 E, linear)."""
    sc = (f'        <scatter>\n          <xs file="{nuc["elastic"]}" temperature="293.6"/>\n'
          + tsl_xml(tsl, indent="          ") + "\n        </scatter>")
    nucxml = (f'    <nuclide name="{name}" awr="{nuc["awr"]!r}">\n      <neutron>\n'
              f'        <total file="{nuc["total"]}" temperature="293.6"/>\n'
              f'        <capture file="{nuc["capture"]}" temperature="293.6"/>\n{sc}\n      </neutron>\n    </nuclide>')
    est = (f'  <current name="leakage" surface="cylinder">\n    <bins>\n'
           f'      <cosine u="1.0" v="0.0" w="0.0">\n        <linspace bins="{cosine_bins}" min="-1.0" max="1.0"/>\n'
           f'      </cosine>\n      <energy>\n'
           f'        <linspace bins="{energy_bins}" min="0.0" max="{2.5 * energy!r}"/>\n'
           f"      </energy>\n    </bins>\n  </current>")
    return ("<minimc>\n<general>\n  <particles>neutron</particles>\n"
            f"  <histories>{histories}</histories>\n  <threads>1</threads>\n  <chunksize>1000</chunksize>\n"
            "  <seed>1</seed>\n</general>\n"
            "<nuclides>\n  <continuous>\n" + nucxml + "\n  </continuous>\n</nuclides>\n"
            f'<materials>\n  <material name="mod" aden="{aden!r}">\n    <nuclide name="{name}" afrac="1.0"/>\n'
            "  </material>\n</materials>\n"
            f'<surfaces>\n  <cylinderx name="cylinder" r="{radius!r}"/>\n'
            '  <planex name="left-plane" x="-0.5e12"/>\n  <planex name="right-plane" x="0.5e12"/>\n</surfaces>\n'
            "<cells>\n"
            '  <void>\n    <surface name="left-plane" sense="-1"/>\n  </void>\n'
            '  <void>\n    <surface name="right-plane" sense="+1"/>\n  </void>\n'
            '  <void>\n    <surface name="cylinder" sense="+1"/>\n    <surface name="left-plane" sense="+1"/>\n'
            '    <surface name="right-plane" sense="-1"/>\n  </void>\n'
            '  <cell name="broomstick" material="mod">\n    <surface name="cylinder" sense="-1"/>\n'
            '    <surface name="left-plane" sense="+1"/>\n    <surface name="right-plane" sense="-1"/>\n  </cell>\n'
            "</cells>\n"
            "<problemtype>\n  <fixedsource>\n"
            '    <position>\n      <constant x="0" y="0" z="0"/>\n    </position>\n'
            '    <direction>\n      <constant x="1" y="0" z="0"/>\n    </direction>\n'
            f'    <energy>\n      <constant energy="{energy!r}"/>\n    </energy>\n'
            '    <particletype>\n      <constant type="neutron"/>\n    </particletype>\n'
            "  </fixedsource>\n</problemtype>\n"
            f'<temperature>\n  <constant c="{temperature!r}"/>\n</temperature>\n'
            f"<estimators>\n{est}\n</estimators>\n</minimc>\n")


def continuous_temperature_slab_xml(tsl: dict, nuc: dict, histories: int = 100_000, energy: float = 0.56 * EV,
                                    thickness: float = 4.33, t_lower: float = 300.0, t_upper: float = 600.0,
                                    energy_bins: int = 60, aden: float = 0.066854, name: str = "Hmod",
                                    seed: int = 1) -> str:
    """The shape of the reference's continuous-temperature benchmark: a
    slab of the bound moderator between planex -1e-6 and `thickness` cm,
    cell delta tracking (the thermal library's majorant bounds the flights),
    a linear temperature field rising from t_lower at x = 0 to t_upper at the
    far face, a monoenergetic pencil beam along +x from the origin, and the
    current through the far face binned in energy (log-spaced boundaries)."""
    sc = (f'        <scatter>\n          <xs file="{nuc["elastic"]}" temperature="293.6"/>\n'
          + tsl_xml(tsl, indent="          ") + "\n        </scatter>")
    nucxml = (f'    <nuclide name="{name}" awr="{nuc["awr"]!r}">\n      <neutron>\n'
              f'        <total file="{nuc["total"]}" temperature="293.6"/>\n'
              f'        <capture file="{nuc["capture"]}" temperature="293.6"/>\n{sc}\n      </neutron>\n    </nuclide>')
    edges = " ".join(repr(float(x)) for x in np.geomspace(1e-11, 2.5e-6, energy_bins + 1))
    gradient = (t_upper - t_lower) / thickness
    return ("<minimc>\n<general>\n  <particles>neutron</particles>\n"
            f"  <histories>{histories}</histories>\n  <threads>1</threads>\n  <chunksize>1000</chunksize>\n"
            f"  <seed>{seed}</seed>\n  <tracking>cell delta</tracking>\n</general>\n"
            "<nuclides>\n  <continuous>\n" + nucxml + "\n  </continuous>\n</nuclides>\n"
            f'<materials>\n  <material name="mod" aden="{aden!r}">\n    <nuclide name="{name}" afrac="1.0"/>\n'
            "  </material>\n</materials>\n"
            f'<surfaces>\n  <planex name="near" x="-1e-06"/>\n  <planex name="far" x="{thickness!r}"/>\n</surfaces>\n'
            "<cells>\n"
            '  <void>\n    <surface name="near" sense="-1"/>\n  </void>\n'
            '  <cell name="slab" material="mod">\n    <surface name="near" sense="+1"/>\n'
            '    <surface name="far" sense="-1"/>\n  </cell>\n'
            '  <void>\n    <surface name="far" sense="+1"/>\n  </void>\n'
            "</cells>\n"
            "<problemtype>\n  <fixedsource>\n"
            '    <position>\n      <constant x="0" y="0" z="0"/>\n    </position>\n'
            '    <direction>\n      <constant x="1" y="0" z="0"/>\n    </direction>\n'
            f'    <energy>\n      <constant energy="{energy!r}"/>\n    </energy>\n'
            '    <particletype>\n      <constant type="neutron"/>\n    </particletype>\n'
            "  </fixedsource>\n</problemtype>\n"
            f'<temperature>\n  <linear>\n    <bounds lower="{t_lower!r}" upper="{t_upper!r}"/>\n'
            f'    <intercept b="{t_lower!r}"/>\n    <gradient x="{gradient!r}" y="0" z="0"/>\n  </linear>\n'
            "</temperature>\n"
            f'<estimators>\n  <current name="leakage" surface="far">\n    <bins>\n      <energy>\n'
            f"        <boundaries>{edges}</boundaries>\n      </energy>\n    </bins>\n  </current>\n"
            "</estimators>\n</minimc>\n")
