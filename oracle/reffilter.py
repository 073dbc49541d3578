"""megalochem's intermediate block filters in DF-J and DF-MO-K, restated in
numpy — TEST INFRASTRUCTURE ONLY (used by tests/ to measure what the
filters change; the product path never imports it).

megalochem filters more than the result matrices.  In fock::DF_J::compute_J
(src/fock/jkdf.cpp:69-190) and fock::DFMO_K::compute_K (:221-462), with
eps = dbcsr::global::filter_eps (the input's block_threshold):

  F1  P_tot's (I, J) blocks at eps                         (jkdf.cpp:100)
  F2  g = (X|MN) P_MN after every nu batch, aux blocks, eps (:124)
  F3  h = g V^-1, aux blocks, eps                          (:137-141)
  F4  J's second pass, (I, J) blocks, eps / nbatches_b     (:166)
  F5  HT1 = (X|MN) C_Mi, (A, o, J) blocks, eps / nbatches_b (:364)
  F6  HT2 = L^-T fit, (A, o, J) blocks, eps                 (:387)
  F7  K accumulated over occupied x auxiliary batches, (I, J) blocks
      after every batch, eps / nbatches_x                   (:419)

Each filter drops the blocks whose Frobenius norm is below its threshold,
as dbcsr::tensor::filter and the .filter() of a contraction do after the
product is formed (src/dbcsrx/dbcsr_tensor.hpp:678-688,
dbcsr_tensor_ops.hpp:128-137).  DBCSR's additional on-the-fly skipping of
block products with small norm products inside the multiplication is not
restated; it removes at most what the result filter of the same
contraction would.

Blocks: AO and auxiliary atom blocks (ao_split_method "atomic"); occupied
blocks split_range(nocc, mo_split) (src/desc/molecule.hpp:177-193).
Batches: make_blk_bounds (src/dbcsrx/dbcsr_btensor.hpp:35-95): a batch
closes at the first block where the running size reaches
ibatch * (total / nbatches).  The defaults below are megalochem's HF input
defaults (src/megalochem_driver.cpp:69, 91-93): mo_split 10, nbatches_b 4,
nbatches_x 4, occ_nbatches 2.
"""
from __future__ import annotations

import numpy as np


def split_range(n, split):
    """Block sizes of n items in blocks of `split` (src/desc/molecule.hpp:177)."""
    nb = n // split + (1 if n % split else 0)
    out = [split] * nb
    if n % split:
        out[-1] = n % split
    return out


def blk_bounds(sizes, nbatches):
    """[first, last] block index of each batch (make_blk_bounds without a
    block map: consecutive blocks are different centres)."""
    sizes = list(sizes)
    nb = len(sizes)
    nbatches = min(nbatches, nb)
    per = sum(sizes) / nbatches
    out, first, cur, ib = [], 0, 0, 1
    for i, s in enumerate(sizes):
        cur += s
        if cur >= ib * per:
            out.append((first, i))
            first = i + 1
            ib += 1
    return out


def _offsets(sizes):
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)


def _filter_blocks(M, roff, coff, eps):
    """Zero the (I, J) blocks of a matrix with Frobenius norm < eps."""
    for I in range(len(roff) - 1):
        for J in range(len(coff) - 1):
            blk = M[roff[I]:roff[I + 1], coff[J]:coff[J + 1]]
            if np.sqrt(np.sum(blk * blk)) < eps:
                blk[...] = 0.0


def _filter_vec(v, off, eps):
    for A in range(len(off) - 1):
        seg = v[off[A]:off[A + 1]]
        if np.sqrt(np.sum(seg * seg)) < eps:
            seg[...] = 0.0


def _panels(layout, B):
    out = []
    for I in range(layout.nblk):
        K = int(layout.panel_K[I])
        b = int(layout.bsizes[I])
        out.append(B[layout.panel_off[I]:layout.panel_off[I] + b * layout.naux * K].reshape(
            b, layout.naux, K) if K else None)
    return out


def _col_blocks(layout):
    """Per panel I: the AO block J of every panel column."""
    boff = layout.boff
    out = []
    for I in range(layout.nblk):
        cols = []
        for J in layout.nbr[I]:
            cols += [J] * int(boff[J + 1] - boff[J])
        out.append(np.array(cols, np.int64))
    return out


def filtered_j(layout, B, Vinv, Ptot, eps, nbatches_b=4):
    """DF-J with megalochem's filters F1-F4 (FP64, numpy)."""
    boff, aoff = layout.boff, layout.aoff
    cmap = layout.column_map()
    cblk = _col_blocks(layout)
    pans = _panels(layout, B)
    P = np.array(Ptot, float)
    _filter_blocks(P, boff, boff, eps)  # F1
    g = np.zeros(layout.naux)
    for (j0, j1) in blk_bounds(layout.bsizes, nbatches_b):
        for I in range(layout.nblk):
            if pans[I] is None:
                continue
            sel = (cblk[I] >= j0) & (cblk[I] <= j1)
            if not sel.any():
                continue
            Pg = P[boff[I]:boff[I + 1]][:, cmap[I][sel]]
            g += np.einsum("mxk,mk->x", pans[I][:, :, sel], Pg)
        _filter_vec(g, aoff, eps)  # F2
    h = Vinv @ g
    _filter_vec(h, aoff, eps)  # F3
    n = layout.nbf
    J = np.zeros((n, n))
    for I in range(layout.nblk):
        if pans[I] is not None:
            J[boff[I]:boff[I + 1], cmap[I]] = np.einsum("mxk,x->mk", pans[I], h)
    # the nu batches write disjoint column blocks, so one pass filters all
    _filter_blocks(J, boff, boff, eps / len(blk_bounds(layout.bsizes, nbatches_b)))  # F4
    return J


def filtered_dfmo_k(layout, B, Linv, Cocc, eps, nbatches_b=4, nbatches_x=4, occ_nbatches=2,
                    mo_split=10):
    """DF-MO K with megalochem's filters F5-F7 (FP64, numpy); returns the
    negated K as the builder does."""
    boff, aoff = layout.boff, layout.aoff
    cmap = layout.column_map()
    pans = _panels(layout, B)
    n, naux = layout.nbf, layout.naux
    nocc = Cocc.shape[1]
    osz = split_range(nocc, mo_split)
    ooff = _offsets(osz)
    # HT1[N][X][i] = sum_M (X|N M) C_Mi   (panel N-rows, contracted over columns)
    H = np.zeros((n, naux, nocc))
    for I in range(layout.nblk):
        if pans[I] is not None:
            H[boff[I]:boff[I + 1]] = np.einsum("mxk,ki->mxi", pans[I], Cocc[cmap[I]])
    nb_b = len(blk_bounds(layout.bsizes, nbatches_b))
    _filter_ht(H, boff, aoff, ooff, eps / nb_b)  # F5
    # HT2[N][Y][i] = sum_X L^-1[Y][X] HT1[N][X][i]
    Lt = np.tril(Linv)
    H2 = np.einsum("yx,nxi->nyi", Lt, H, optimize=True)
    del H
    _filter_ht(H2, boff, aoff, ooff, eps)  # F6
    K = np.zeros((n, n))
    xb = blk_bounds(layout.asizes, nbatches_x)
    ob = blk_bounds(osz, occ_nbatches)
    for (o0, o1) in ob:
        i0, i1 = ooff[o0], ooff[o1 + 1]
        for (a0, a1) in xb:
            y0, y1 = aoff[a0], aoff[a1 + 1]
            T = H2[:, y0:y1, i0:i1].reshape(n, -1)
            K += T @ T.T
            _filter_blocks(K, boff, boff, eps / len(xb))  # F7
    return -K


def _filter_ht(H, boff, aoff, ooff, eps):
    for J in range(len(boff) - 1):
        for A in range(len(aoff) - 1):
            blk = H[boff[J]:boff[J + 1], aoff[A]:aoff[A + 1]]
            nrm2 = np.einsum("nyi,nyi->i", blk, blk)
            for o in range(len(ooff) - 1):
                if np.sqrt(nrm2[ooff[o]:ooff[o + 1]].sum()) < eps:
                    blk[:, :, ooff[o]:ooff[o + 1]] = 0.0
