"""SOS-AO-MP2 Laplace term around the device Z builder (host side, FP64).

Restates what megalochem's mpmod::compute does around its Z builder
(src/mp/mp_compute.cpp:40-392):
  * the Laplace interval [2(e_lumo - e_homo), 2(e_max - e_min)] and the
    minimax points (alpha_t, omega_t) (:64-91, chem_gb300.laplace);
  * per point the scaled coefficients C_o e^{+alpha e_i / 2} and
    C_v e^{-alpha e_a / 2} (:240-266);
  * their pseudo-densities in the orthogonalised basis,
    omega^{1/4} (L_S^-1 C)(L_S^-1 C)^T with S = L_S L_S^T (:167-176, :268-281),
    a pivoted incomplete Cholesky decomposition of each (:283-329,
    src/math/linalg/piv_cd.cpp) and the factors back in the AO basis,
    L = L_S L_ortho, so that L L^T = omega^{1/4} C C^T;
  * Z_t from the ll_full builder (both factors; src/mp/z_full.cpp:427-620),
    here the device batch gbjk_mp2_*;
  * e_t = tr(Z_t V^-1 Z_t V^-1), summed over the points (:361-381); the
    reference reports the sum as "Final MP2 energy" and c_os times it as the
    scaled energy (:384-389), with the sign as printed there (positive).
The random-orbital inputs of the MP2 workload (orthonormal in the S metric,
orbital energies drawn uniformly) are made by `random_orbitals`.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

from .laplace import laplace_points


def random_orbitals(S, nocc, seed, eps_occ=(-20.0, -0.3), eps_vir=(0.1, 50.0)):
    """Orbitals C (nbf x nbf, C^T S C = 1) from a seeded random orthogonal
    matrix, and sorted orbital energies drawn uniformly from the given ranges.
    Returns (C_occ, C_vir, e_occ, e_vir)."""
    rng = np.random.default_rng(seed)
    n = S.shape[0]
    s, U = np.linalg.eigh(S)
    Xs = U @ np.diag(s ** -0.5) @ U.T
    Q, R = np.linalg.qr(rng.standard_normal((n, n)))
    Q = Q * np.sign(np.diag(R))
    Cm = Xs @ Q
    e_o = np.sort(rng.uniform(eps_occ[0], eps_occ[1], nocc))
    e_v = np.sort(rng.uniform(eps_vir[0], eps_vir[1], n - nocc))
    return Cm[:, :nocc].copy(), Cm[:, nocc:].copy(), e_o, e_v


def laplace_interval(e_occ, e_vir):
    """(ymin, ymax) = (2(e_lumo - e_homo), 2(e_max - e_min)) (mp_compute.cpp:64-69)."""
    return 2.0 * (e_vir[0] - e_occ[-1]), 2.0 * (e_vir[-1] - e_occ[0])


def pivoted_cholesky(A, thresh=None, max_rank=None, reorder_eps=None):
    """Pivoted incomplete Cholesky A ~ L L^T (src/math/linalg/piv_cd.cpp:152-420).

    Step I takes the largest remaining diagonal |U_jj| as pivot; a negative
    pivot above the threshold is an error; the decomposition stops when the
    pivot falls below `thresh` (default N * eps * max|diag|, :281) or at
    `max_rank`.  Returns L (N x rank) in the original row order.  With
    reorder_eps, the columns are sorted by the centre of their rows above
    reorder_eps (pivinc_cd::reorder_and_reduce, :27-142); L L^T does not
    depend on the column order."""
    A = np.asarray(A, dtype=float)
    N = A.shape[0]
    d = np.diag(A).copy()  # diagonal of the remaining Schur complement
    if thresh is None:
        thresh = N * np.finfo(float).eps * np.max(np.abs(d))
    kmax = N if max_rank is None else min(N, int(max_rank))
    L = np.zeros((N, kmax))
    for k in range(kmax):
        j = int(np.argmax(np.abs(d)))
        piv = d[j]
        if piv < 0.0 and abs(piv) > thresh:
            raise ValueError("Negative Pivot element. CD not possible.")
        if abs(piv) < thresh:
            L = L[:, :k]
            break
        # column j of the Schur complement, scaled by 1/sqrt(pivot)
        col = (A[:, j] - L[:, :k] @ L[j, :k]) / np.sqrt(piv)
        col[j] = np.sqrt(piv)
        L[:, k] = col
        d = d - col * col
        d[j] = 0.0
    if reorder_eps is not None and L.shape[1] > 1:
        pos = np.empty(L.shape[1])
        for c in range(L.shape[1]):
            rows = np.nonzero(L[:, c] > reorder_eps)[0]
            pos[c] = N - 1 if rows.size == 0 else 0.5 * (rows[0] + rows[-1])
        L = L[:, np.argsort(pos, kind="stable")]
    return L


@dataclass
class LaplaceFactors:
    alpha: np.ndarray
    omega: np.ndarray
    err: float
    Lo: list = field(default_factory=list)   # per point, nbf x rank_o
    Lv: list = field(default_factory=list)   # per point, nbf x rank_v
    Po: list = field(default_factory=list)   # per point pseudo-densities (AO)
    Pv: list = field(default_factory=list)


def laplace_factors(C_occ, C_vir, e_occ, e_vir, S, nlap, keep_densities=False):
    """Per Laplace point the AO-basis Cholesky factors Lo_t, Lv_t with
    Lo Lo^T = omega^{1/4} C_o' C_o'^T and Lv Lv^T = omega^{1/4} C_v' C_v'^T."""
    ymin, ymax = laplace_interval(e_occ, e_vir)
    alpha, omega, err = laplace_points(nlap, ymin, ymax)
    Ls = np.linalg.cholesky(S)
    Ls_inv = sla.solve_triangular(Ls, np.eye(len(S)), lower=True)
    out = LaplaceFactors(alpha, omega, err)
    for a, w in zip(alpha, omega):
        co = C_occ * np.exp(0.5 * e_occ * a)
        cv = C_vir * np.exp(-0.5 * e_vir * a)
        f = w ** 0.25
        for c, dst in ((co, out.Lo), (cv, out.Lv)):
            cort = Ls_inv @ c
            P_ortho = f * (cort @ cort.T)
            dst.append(Ls @ pivoted_cholesky(P_ortho))
        if keep_densities:
            out.Po.append(f * (co @ co.T))
            out.Pv.append(f * (cv @ cv.T))
    return out


def sos_mp2_laplace(engine, factors: LaplaceFactors, c_os=1.3):
    """Laplace sum on the device: e_t per point, their sum (megalochem's
    "Final MP2 energy") and c_os times it."""
    e, _ = engine.mp2_laplace(factors.Lo, factors.Lv)
    tot = float(np.sum(e))
    return {"points": e, "energy": tot, "scaled": c_os * tot}
