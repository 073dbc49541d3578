"""Block-sparse layout of the 3-center tensor B = (X|mu nu) in HBM.

Screening follows megalochem: a block triple (A, I, J) (auxiliary atom block
A, AO atom blocks I, J) is kept when
    float(||Z_IJ||_F * ||Z_A||_F) > eps
with Z the shell-level Schwarz factors and ||.||_F the Frobenius norm over the
shells of the block (src/ints/screening.cpp:23-30,
src/dbcsrx/dbcsr_conversions.hpp:564-601, src/ints/aofactory.cpp:52-137).

Storage ("panels"): for every AO block I the kept partner blocks
nbr(I) = {J : some A kept for (I, J)} are concatenated along a column index
k, giving K_I = sum_{J in nbr(I)} b_J columns, and panel I is the dense array
    P_I[mu][X][k]     mu < b_I, X < naux, k < K_I        (FP64, row-major)
Screened (A, I, J) blocks are stored as zeros.  Both (I, J) and (J, I) are
stored, so the half transform of panel I is one dense GEMM
(b_I*naux x K_I) x (K_I x nocc) whose output rows land contiguously in the
half-transformed tensor H[mu][X][i].
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class PanelLayout:
    nblk: int
    nablk: int
    bsizes: np.ndarray  # AO block sizes
    asizes: np.ndarray  # auxiliary block sizes
    naux: int
    pair_I: np.ndarray  # kept block pairs, I <= J
    pair_J: np.ndarray
    keep: np.ndarray  # [npairs, nablk] uint8
    nbr: list  # nbr[I] = sorted kept partner blocks
    panel_K: np.ndarray  # K_I
    panel_off: np.ndarray  # element offset of panel I
    col_IJ: np.ndarray  # column offset of J in panel I, per pair
    col_JI: np.ndarray  # column offset of I in panel J, per pair
    col_of: dict  # (I, J) -> column offset of J in panel I

    @property
    def nbf(self):
        return int(self.bsizes.sum())

    @property
    def boff(self):
        return np.concatenate([[0], np.cumsum(self.bsizes)]).astype(np.int64)

    @property
    def aoff(self):
        return np.concatenate([[0], np.cumsum(self.asizes)]).astype(np.int64)

    @property
    def nnz(self):
        return int(self.panel_off[-1] + self.bsizes[-1] * self.naux * self.panel_K[-1]) \
            if self.nblk else 0

    @property
    def npairs(self):
        return len(self.pair_I)

    def kept_block_fraction(self):
        """Fraction of (I, J) AO block pairs kept (both orders counted)."""
        return float(self.panel_K @ self.bsizes) / float(self.nbf) ** 2

    def column_map(self):
        """For each panel I, the AO index of every column k (int64 array)."""
        boff = self.boff
        out = []
        for I in range(self.nblk):
            cols = [np.arange(boff[J], boff[J + 1]) for J in self.nbr[I]]
            out.append(np.concatenate(cols) if cols else np.zeros(0, np.int64))
        return out

    def to_dense(self, B):
        """Dense (naux, nbf, nbf) tensor from the panel array (tests only)."""
        boff = self.boff
        T = np.zeros((self.naux, self.nbf, self.nbf))
        for I in range(self.nblk):
            bI, KI = int(self.bsizes[I]), int(self.panel_K[I])
            P = B[self.panel_off[I]:self.panel_off[I] + bI * self.naux * KI].reshape(bI, self.naux, KI)
            for J in self.nbr[I]:
                c = self.col_of[(I, J)]
                bJ = int(self.bsizes[J])
                T[:, boff[I]:boff[I + 1], boff[J]:boff[J + 1]] = P[:, :, c:c + bJ].transpose(1, 0, 2)
        return T


def block_norms(values, groups):
    """Frobenius norm of `values` summed within index groups (offsets)."""
    return np.array([np.sqrt(np.sum(values[groups[i]:groups[i + 1]] ** 2))
                     for i in range(len(groups) - 1)])


def build_layout(bsizes, asizes, keep_fn) -> PanelLayout:
    """Generic constructor from a block-triple predicate keep_fn(I, J) -> bool
    mask over auxiliary blocks (length nablk)."""
    bsizes = np.asarray(bsizes, np.int64)
    asizes = np.asarray(asizes, np.int64)
    nblk, nablk = len(bsizes), len(asizes)
    naux = int(asizes.sum())
    pI, pJ, keeps = [], [], []
    nbr = [[] for _ in range(nblk)]
    for I in range(nblk):
        for J in range(I, nblk):
            m = np.asarray(keep_fn(I, J), bool)
            if m.any():
                pI.append(I)
                pJ.append(J)
                keeps.append(m.astype(np.uint8))
                nbr[I].append(J)
                if J != I:
                    nbr[J].append(I)
    for I in range(nblk):
        nbr[I].sort()
    col_of = {}
    K = np.zeros(nblk, np.int64)
    for I in range(nblk):
        c = 0
        for J in nbr[I]:
            col_of[(I, J)] = c
            c += int(bsizes[J])
        K[I] = c
    off = np.zeros(nblk, np.int64)
    acc = 0
    for I in range(nblk):
        off[I] = acc
        acc += int(bsizes[I]) * naux * int(K[I])
    col_IJ = np.array([col_of[(i, j)] for i, j in zip(pI, pJ)], np.int32)
    col_JI = np.array([col_of[(j, i)] for i, j in zip(pI, pJ)], np.int32)
    keep = np.array(keeps, np.uint8).reshape(len(pI), nablk)
    return PanelLayout(nblk, nablk, bsizes, asizes, naux, np.array(pI, np.int32),
                       np.array(pJ, np.int32), keep, nbr, K, off, col_IJ, col_JI, col_of)


def schwarz_layout(mol, Zmn, zx, eps) -> PanelLayout:
    """Layout from shell-level Schwarz factors with megalochem's block test."""
    bas, aux = mol.basis, mol.dfbasis
    so = bas.block_shell_off
    ao = aux.block_shell_off
    nb = bas.nblk
    nmn = np.zeros((nb, nb))
    for I in range(nb):
        for J in range(nb):
            nmn[I, J] = np.sqrt(np.sum(Zmn[so[I]:so[I + 1], so[J]:so[J + 1]] ** 2))
    nx = block_norms(zx, ao)

    def keep(I, J):
        return np.float32(nmn[I, J] * nx) > eps

    return build_layout(bas.block_sizes, aux.block_sizes, keep)
