"""Seeded synthetic block-sparse DF-K workload (nbf 4000, naux 12000,
nocc 600 at full size): AO block sizes drawn uniformly from
{5, 9, 14, 18, 30, 40} until they sum to nbf (the last block truncated);
block pair (I, J) kept with probability exp(-|I-J|/L), L set by bisection
for the requested fraction of kept elements (symmetric pattern, diagonal
always kept); tensor entries N(0,1) exp(-|I-J|/(2L)), symmetric in (mu, nu),
generated on the device (gbjk_upload_b_synthetic) and treated as
pre-fitted; occupied coefficients a QR-orthonormalised Gaussian matrix."""
from __future__ import annotations

import numpy as np

from .layout import build_layout

SIZES = (5, 9, 14, 18, 30, 40)


def block_sizes(total, rng):
    out = []
    while sum(out) < total:
        out.append(int(rng.choice(SIZES)))
    out[-1] -= sum(out) - total
    return np.array(out, np.int64)


def synthetic_layout(nbf, naux, density=0.10, seed=20261203):
    rng = np.random.default_rng(seed)
    bs = block_sizes(nbf, rng)
    nb = len(bs)
    u = rng.random((nb, nb))
    u = np.triu(u) + np.triu(u, 1).T  # one draw per unordered pair
    dist = np.abs(np.arange(nb)[:, None] - np.arange(nb)[None, :])
    w = np.outer(bs, bs).astype(float)

    def frac(L):
        keep = (u < np.exp(-dist / L)) | (dist == 0)
        return float(w[keep].sum()) / float(nbf) ** 2, keep

    lo, hi = 1e-3, float(nb)
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        f, _ = frac(mid)
        if f < density:
            lo = mid
        else:
            hi = mid
    L = 0.5 * (lo + hi)
    _, keep = frac(L)
    layout = build_layout(bs, [naux], lambda I, J: np.array([keep[I, J]]))
    return layout, L


def occupied(nbf, nocc, seed=20261203):
    rng = np.random.default_rng(seed + 1)
    return np.ascontiguousarray(np.linalg.qr(rng.standard_normal((nbf, nocc)))[0])
