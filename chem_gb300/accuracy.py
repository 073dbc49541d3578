"""Accuracy yardsticks for the metric step of DF-J (host, extended precision).

DF-J needs h = V^-1 g for the Coulomb metric V (src/fock/jkdf.cpp:137-141).
megalochem forms it with the explicit inverse V^-1 = L^-T L^-1
(src/ints/aoloader.cpp:14-32); the engine also offers the Cholesky route
h = L^-T (L^-1 g).  With cond(V) ~ 1e7 the two FP64 routes differ far above
the 1e-8 Eh target, so the question which one is right needs a solution of
V h = g that is exact for the given FP64 V and g.  This module gets it by
iterative refinement with exactly computed residuals:

  * every product V_ij h_j is split exactly into p + e (Dekker's product
    with Veltkamp splitting), and r_i = g_i - sum_j (p_ij + e_ij) is
    summed with math.fsum, so the residual is correctly rounded;
  * h is carried as a sum of FP64 vectors h_0 + d_1 + d_2 + ...; each
    correction d_k solves V d_k = r_{k-1} with the FP64 Cholesky factor.
Each step shrinks the error by about cond(V) * 2^-53, so three steps give
the exact solution far beyond FP64 resolution.  Energies gᵀh are summed the
same way.  Where numpy's longdouble is IEEE quadruple precision (aarch64),
the residuals can instead be formed in quad arithmetic, which is much faster
for naux in the thousands.  No GPU; used by the tests and the bench's
accuracy report.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg as sla

_SPLIT = 134217729.0  # 2^27 + 1


def _split(a):
    c = _SPLIT * a
    hi = c - (c - a)
    return hi, a - hi


def two_prod(a, b):
    """a * b = p + e exactly, elementwise (no overflow assumed)."""
    p = a * b
    ah, al = _split(a)
    bh, bl = _split(b)
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def exact_dot(x, parts):
    """sum_i x_i * sum_k parts[k]_i, correctly rounded."""
    terms = []
    for h in parts:
        p, e = two_prod(np.asarray(x, float), np.asarray(h, float))
        terms.append(p)
        terms.append(e)
    return math.fsum(np.concatenate(terms).tolist())


def exact_residual(V, g, parts):
    """r = g - V (sum_k parts[k]), each entry correctly rounded."""
    n = len(g)
    r = np.empty(n)
    for i in range(n):
        terms = [np.array([g[i]])]
        for h in parts:
            p, e = two_prod(V[i], h)
            terms.append(-p)
            terms.append(-e)
        r[i] = math.fsum(np.concatenate(terms).tolist())
    return r


def quad_residual(V, g, parts):
    """r = g - V (sum_k parts[k]) in IEEE quadruple precision (numpy
    longdouble where it has a 113-bit significand, as on aarch64), rounded
    to FP64 at the end.  Its error, ~2^-113 of the terms, is far below what
    refinement needs for cond(V) ~ 1e7."""
    ld = np.longdouble
    Vq = V.astype(ld)
    h = np.zeros(len(g), ld)
    for p in parts:
        h += p.astype(ld)
    return (g.astype(ld) - Vq @ h).astype(np.float64)


def have_quad():
    return np.finfo(np.longdouble).nmant >= 112


def refined_solve(V, g, steps=3, residual=None):
    """The solution of V h = g as a list of FP64 vectors whose exact sum
    is h to far beyond FP64 resolution (iterative refinement with exact
    residuals: correctly rounded sums, or quadruple precision where numpy
    has it and residual="quad").  Returns (parts, residual norm after the
    last step)."""
    res = quad_residual if residual == "quad" else exact_residual
    cf = sla.cho_factor(V, lower=True)
    parts = [sla.cho_solve(cf, g)]
    r = None
    for _ in range(steps):
        r = res(V, g, parts)
        parts.append(sla.cho_solve(cf, r))
    r = res(V, g, parts)
    return parts, float(np.abs(r).max())


def panel_g(layout, B, Ptot):
    """g_X = sum_{mu nu} (X|mu nu) Ptot_{mu nu} over the panel layout (FP64)."""
    boff = layout.boff
    cols = layout.column_map()
    g = np.zeros(layout.naux)
    for I in range(layout.nblk):
        K = int(layout.panel_K[I])
        if K == 0:
            continue
        b = int(layout.bsizes[I])
        pan = B[layout.panel_off[I]:layout.panel_off[I] + b * layout.naux * K].reshape(
            b, layout.naux, K)
        g += np.einsum("mxk,mk->x", pan, Ptot[boff[I]:boff[I + 1]][:, cols[I]])
    return g


def panel_j(layout, B, h):
    """J_{mu nu} = sum_X (X|mu nu) h_X over the panel layout (FP64)."""
    n = layout.nbf
    boff = layout.boff
    cols = layout.column_map()
    J = np.zeros((n, n))
    for I in range(layout.nblk):
        K = int(layout.panel_K[I])
        if K == 0:
            continue
        b = int(layout.bsizes[I])
        pan = B[layout.panel_off[I]:layout.panel_off[I] + b * layout.naux * K].reshape(
            b, layout.naux, K)
        J[boff[I]:boff[I + 1], cols[I]] = np.einsum("mxk,x->mk", pan, h)
    return J


def coulomb_routes(V, Linv, Vinv, g, residual=None):
    """Coulomb energy E_J = 1/2 gᵀV⁻¹g (Eh, for g from P_tot = 2 P_alpha)
    exactly and on the two FP64 routes, plus each route's h and the exact h
    rounded to FP64.  Linv is the lower-triangular L^-1 with V = L Lᵀ.
    residual="quad" refines with quadruple-precision residuals (fast where
    numpy's longdouble is IEEE quad); the default sums exactly."""
    parts, res = refined_solve(V, g, residual=residual)
    e_exact = 0.5 * exact_dot(g, parts)
    h_exact = np.sum(parts, axis=0)  # rounded to FP64
    h_vinv = Vinv @ g
    y = np.tril(Linv) @ g
    h_chol = np.tril(Linv).T @ y
    return {
        "E_exact": e_exact,
        "residual_max": res,
        "dE_vinv": 0.5 * float(g @ h_vinv) - e_exact,
        "dE_cholesky": 0.5 * float(y @ y) - e_exact,
        "h_exact": h_exact,
        "h_vinv": h_vinv,
        "h_cholesky": h_chol,
    }


def j_energy_vs_exact(P_alpha, J, e_exact):
    """Coulomb energy of a built J against the exact one: sum P_alpha J -
    1/2 gᵀV⁻¹g (J from P_tot = 2 P_alpha)."""
    return float(np.sum(P_alpha * J)) - e_exact
