"""POD table pipeline for thermal scattering libraries.

The reference samples thermal inelastic scattering from proper orthogonal
decompositions of inverse CDFs (src/ThermalScattering.cpp:183-463).  The
tables are produced outside the reference by a pipeline whose source is not
part of the repository; its steps appear at one call site
(scripts/tolerance_vs_spectrum_error/tolerance_vs_spectrum_error.py:16-41):
split the full table along the incident-energy level, truncate each
partition to a rank, remove non-monotone CDFs, and coarsen adaptively to a
relative Frobenius-norm tolerance.  This module builds those steps from
their names and the layout the reference reads:

* a table is the inverse-CDF matrix M[F][(g, T)] of one partition kind --
  rows are interior CDF values F, columns the outer grid (incident energy
  E for beta tables, |beta| for alpha tables) times the temperatures T;
* ``split`` cuts the outer grid into contiguous partitions;
* ``truncate`` is the rank-r SVD M = CDF_modes diag(S) outer_T_modes^T
  (the layout of the partition files: CDF [F][r], S [r], outer_T [g][T][r]);
* ``remove_nonmonotonic_cdfs`` drops the outer grid points whose
  reconstructed inverse CDF decreases in F at any temperature (the
  reference's bisection and interpolation assume non-decreasing values);
* ``adaptive_coarsen`` chooses for every partition the least rank whose
  relative Frobenius error is within a tolerance (from the singular
  values, sum_{k>r} S_k^2 <= tol^2 sum_k S_k^2), optionally from complete
  decompositions made once for a sweep over tolerances.

The decompositions run on the GPU when one is present: a one-sided Jacobi
SVD in FP64 (minimc_gb300/csrc/mc_pod.cu, C ABI mc_pod_svd), with LAPACK
on hosts without one; the results are written as ``.mctab`` files
(synth_ce.write_table) named like synth_tsl's.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .synth_ce import write_table


@dataclass
class Table:
    """Inverse-CDF matrix of one partition kind: values[F][g][T]."""
    F: np.ndarray       # interior CDF values (rows)
    outer: np.ndarray   # outer grid: E (beta tables) or |beta| (alpha tables)
    T: np.ndarray       # temperatures
    values: np.ndarray  # [len(F)][len(outer)][len(T)]

    def matrix(self) -> np.ndarray:
        return self.values.reshape(len(self.F), -1)


@dataclass
class Pod:
    """Rank-r POD of one partition: M ~ cdf diag(S) outer_T^T."""
    F: np.ndarray
    outer: np.ndarray
    T: np.ndarray
    cdf: np.ndarray       # [F][r]
    S: np.ndarray         # [r]
    outer_T: np.ndarray   # [outer][T][r]
    full_S: np.ndarray = field(default_factory=lambda: np.zeros(0))  # all singular values of the partition

    @property
    def rank(self) -> int:
        return len(self.S)

    def reconstruct(self) -> np.ndarray:
        """values[F][outer][T] of the truncated decomposition."""
        r = self.rank
        V = self.outer_T.reshape(-1, r)
        return ((self.cdf * self.S) @ V.T).reshape(len(self.F), len(self.outer), len(self.T))

    def rel_frobenius_error(self) -> float:
        """||M - M_r||_F / ||M||_F from the singular values."""
        tot = float(np.sum(self.full_S ** 2))
        return float(np.sqrt(max(0.0, tot - float(np.sum(self.S ** 2))) / tot)) if tot > 0 else 0.0


_SVD_CTX = None


def _device_svd(M: np.ndarray):
    """Thin SVD on the GPU: the project's one-sided Jacobi kernel
    (Context.pod_svd, C ABI mc_pod_svd), FP64."""
    global _SVD_CTX
    if _SVD_CTX is None:
        from .engine import Context

        _SVD_CTX = Context(0)
    U, S, Vh, _ = _SVD_CTX.pod_svd(M)
    return U, S, Vh


def _gpu_present() -> bool:
    try:
        import torch

        return bool(torch.cuda.is_available())
    except ImportError:
        return False


def _svd(M: np.ndarray, device: str | None):
    """Thin SVD in FP64: device "cuda" runs the project's Jacobi kernel on
    the GPU, "numpy" LAPACK on the host; None picks the GPU when one is
    present."""
    if device is None:
        device = "cuda" if _gpu_present() else "numpy"
    if device == "cuda":
        return _device_svd(M)
    if device == "numpy":
        return np.linalg.svd(M, full_matrices=False)
    raise ValueError(f"unknown SVD device {device!r} (\"cuda\" or \"numpy\")")


def split(table: Table, boundaries) -> list[Table]:
    """Contiguous partitions of the outer grid, cut before each index in
    `boundaries` (the call site passes [95, 235, 500] for four partitions)."""
    cuts = [0] + [int(b) for b in boundaries] + [len(table.outer)]
    if any(b <= a for a, b in zip(cuts, cuts[1:])):
        raise ValueError(f"partition boundaries must increase within 1..{len(table.outer) - 1}: {boundaries}")
    return [Table(table.F, table.outer[a:b], table.T, table.values[:, a:b, :]) for a, b in zip(cuts, cuts[1:])]


def truncate(table: Table, rank: int, device: str | None = None) -> Pod:
    """Rank-`rank` POD of one partition (the SVD, cut after `rank` modes)."""
    U, S, Vh = _svd(table.matrix(), device)
    r = max(1, min(int(rank), len(S)))
    V = Vh[:r].T.reshape(len(table.outer), len(table.T), r)
    return Pod(table.F, table.outer, table.T, U[:, :r].copy(), S[:r].copy(), V.copy(), S.copy())


def remove_nonmonotonic_cdfs(pod: Pod, tol: float = 0.0) -> Pod:
    """Drops the outer grid points whose reconstructed inverse CDF decreases
    (by more than `tol`) between consecutive F at some temperature."""
    R = pod.reconstruct()
    bad = (np.diff(R, axis=0) < -tol).any(axis=(0, 2))
    if not bad.any():
        return pod
    keep = ~bad
    if not keep.any():
        raise ValueError("every CDF of the partition is non-monotone at this rank")
    return Pod(pod.F, pod.outer[keep], pod.T, pod.cdf, pod.S, pod.outer_T[keep], pod.full_S)


def rank_for_tolerance(singular_values: np.ndarray, rel_frobenius_norm_tol: float) -> int:
    """Least r with sqrt(sum_{k>=r} S_k^2 / sum S_k^2) <= tol."""
    s2 = np.asarray(singular_values, np.float64) ** 2
    tot = s2.sum()
    if tot == 0:
        return 1
    tail = np.concatenate([np.cumsum(s2[::-1])[::-1], [0.0]])  # tail[r] = sum_{k>=r}
    ok = np.nonzero(np.sqrt(tail / tot) <= rel_frobenius_norm_tol)[0]
    return max(1, int(ok[0]))


def adaptive_coarsen(partitions: list[Table], previous: list[Pod] | None = None,
                     rel_frobenius_norm_tol: float = 1e-3, device: str | None = None,
                     monotone: bool = True) -> list[Pod]:
    """For every partition the least-rank POD within the relative Frobenius
    tolerance (its non-monotone CDFs removed when `monotone`); `previous`
    (full_decompositions of the same partitions) supplies the complete
    SVDs, so a sweep over tolerances decomposes each partition once."""
    out = []
    for i, part in enumerate(partitions):
        if previous is not None and i < len(previous) and len(previous[i].full_S) and \
                np.array_equal(previous[i].outer, part.outer) and previous[i].rank == len(previous[i].full_S):
            full = previous[i]
        else:
            full = truncate(part, len(part.F) * len(part.outer) * len(part.T), device)
        r = rank_for_tolerance(full.full_S, rel_frobenius_norm_tol)
        pod = Pod(full.F, full.outer, full.T, full.cdf[:, :r].copy(), full.S[:r].copy(),
                  full.outer_T[:, :, :r].copy(), full.full_S)
        out.append(remove_nonmonotonic_cdfs(pod) if monotone else pod)
    return out


def full_decompositions(partitions: list[Table], device: str | None = None) -> list[Pod]:
    """Every partition's complete SVD (the starting point for sweeps)."""
    return [truncate(p, len(p.F) * len(p.outer) * len(p.T), device) for p in partitions]


def write_partitions(pods: list[Pod], directory, prefix: str, kind: str) -> list[dict]:
    """Partition files in the reference's layout; kind "beta" writes
    CDF / S / E_T, kind "alpha" CDF / S / beta_T.  Returns the file names
    per partition (the <partition .../> attributes)."""
    directory = Path(directory)
    directory.mkdir(parents=True, exist_ok=True)
    outer_key = {"beta": "E_T", "alpha": "beta_T"}[kind]
    files = []
    for p, pod in enumerate(pods):
        r = pod.rank
        order = np.arange(r, dtype=np.float64)
        names = {k: f"{prefix}-{kind}{p}-{k}.mctab" for k in ("CDF", "S", outer_key)}
        write_table(directory / names["CDF"], [pod.F, order], pod.cdf)
        write_table(directory / names["S"], [order], pod.S)
        write_table(directory / names[outer_key], [pod.outer, pod.T, order], pod.outer_T)
        files.append(names)
    return files
