"""Minimal closed-shell DF-HF SCF driver (FP64) around the J/K builders.

Restates the parts of megalochem's hf::hfmod the configs need:
  * Loewdin orthogonaliser X = S^-1/2 (src/math/linalg/orthogonalizer.cpp:14-45);
  * form_fock: F = H + J + K_A with J from P_tot = 2 P_A and K_A already
    negated (src/hf/hfscf.cpp:228-276);
  * energy E = sum P_A (H + F) + E_nuc (src/hf/hfscf.cpp:278-296);
  * error matrix FPS - SPF (AO basis) and its RMS sqrt(sum e^2 / nbf^2);
    converged when the RMS falls below the threshold after the first
    iteration (src/hf/hfscf.cpp:298-324, :381-384, :430);
  * DIIS extrapolation on the Fock matrices (src/math/solvers/diis.hpp:43-234);
  * diagonalisation X^T F X and P = C_occ C_occ^T (src/hf/hfdiagfock.cpp:20-102).
The guess is the core Hamiltonian (megalochem's default SAD guess runs an
atomic UHF with exact J/K; the converged RHF state is the same).
Diagonalisation, DIIS and the energy stay FP64 on the host; J and K come
from the device engine.  With a split-precision engine the driver switches
to the FP64 path once the DIIS error falls below `switch_thresh`.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class SCFResult:
    energy: float
    converged: bool
    iterations: int
    C: np.ndarray
    eps: np.ndarray
    P: np.ndarray
    F: np.ndarray
    history: list = field(default_factory=list)
    audit: list = field(default_factory=list)


class DIIS:
    """Pulay DIIS over (F, error) pairs (src/math/solvers/diis.hpp:43-234)."""

    def __init__(self, max_vecs=8):
        self.max_vecs = max_vecs
        self.F, self.E = [], []

    def push(self, F, err):
        self.F.append(F.copy())
        self.E.append(err.copy())
        if len(self.F) > self.max_vecs:
            self.F.pop(0)
            self.E.pop(0)

    def extrapolate(self):
        n = len(self.F)
        if n < 2:
            return self.F[-1]
        Bm = -np.ones((n + 1, n + 1))
        Bm[n, n] = 0.0
        for i in range(n):
            for j in range(n):
                Bm[i, j] = np.sum(self.E[i] * self.E[j])
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        c = np.linalg.lstsq(Bm, rhs, rcond=None)[0][:n]
        return sum(ci * Fi for ci, Fi in zip(c, self.F))


def fp64_switch(engine, jmode="cholesky"):
    """Switch callback for run_rhf: moves a split-precision engine to the
    FP64 path with J on the given route ("cholesky", or "vinv" for the
    reference's explicit V^-1)."""
    def sw():
        engine.set_precision("fp64")
        engine.set_jmode(jmode)
    return sw


def run_rhf(S, Hcore, enuc, nocc, jk, conv=1e-8, max_iter=100, diis_start=0, max_vecs=8,
            switch=None, switch_thresh=1e-5, log=None, audit=None):
    """jk(P_alpha, C_occ) -> (J, K_alpha) with K already negated; conv is the
    RMS threshold of the error matrix (megalochem's scf_thresh).
    switch(): called once when the DIIS RMS error falls below switch_thresh
    (moves a split-precision engine to FP64, e.g. fp64_switch(engine)).
    audit(P_alpha, C_occ, J, K) -> dict: called on every build's result
    (e.g. its deviation from an FP64 build at the same density); the dicts
    are returned in SCFResult.audit, one per iteration."""
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    F = Hcore.copy()
    diis = DIIS(max_vecs)
    E_old = 0.0
    hist = []
    audits = []
    switched = switch is None
    for it in range(max_iter):
        Fo = X.T @ F @ X
        e, Cp = np.linalg.eigh(Fo)
        Cm = X @ Cp
        Cocc = Cm[:, :nocc]
        P = Cocc @ Cocc.T
        J, K = jk(P, Cocc)
        if audit is not None:
            audits.append(audit(P, Cocc, J, K))
        F_new = Hcore + J + K
        E = float(np.sum(P * (Hcore + F_new)) + enuc)
        err = F_new @ P @ S - S @ P @ F_new
        rms = float(np.sqrt(np.mean(err ** 2)))
        hist.append((it, E, E - E_old, rms))
        if log:
            log(f"iter {it:3d}  E {E:.12f}  dE {E - E_old:.3e}  rms {rms:.3e}")
        if not switched and rms < switch_thresh:
            switch()
            switched = True
            E_old = E
            F = F_new
            continue
        if it > 0 and rms < conv and switched:
            return SCFResult(E, True, it + 1, Cm, e, P, F_new, hist, audits)
        E_old = E
        if it >= diis_start:
            diis.push(F_new, err)
            F = diis.extrapolate()
        else:
            F = F_new
    return SCFResult(E, False, max_iter, Cm, e, P, F_new, hist, audits)


def run_rhf_device(engine, S, Hcore, enuc, nocc, kmethod="dfmo", conv=1e-8, max_iter=100,
                   max_vecs=8, switch=None, switch_thresh=1e-5, log=None, audit=None):
    """The same SCF as run_rhf with each iteration's device work in CUDA
    graphs (JKEngine.scf_*): P = C C^T, the Fock build, F = H + J + K, the
    energy, the error matrix FPS - SPF with its RMS and the DIIS overlaps
    run on the GPU (one graph), and the DIIS combination with X F X (a
    second graph).  The host solves the DIIS system and diagonalises in
    FP64, as megalochem does (src/hf/hfscf.cpp:386-459).  DIIS keeps the
    last max_vecs (F, error) pairs in device ring slots.
    audit(P_alpha, C_occ, J, K) -> dict is called on every build (it
    downloads J and K)."""
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    engine.scf_begin(Hcore, S, X, nocc, max_vecs)
    Bm = np.zeros((max_vecs, max_vecs))
    order = []  # ring slots in use, oldest first
    nxt = 0
    Fo = X.T @ Hcore @ X
    E_old = 0.0
    hist, audits = [], []
    switched = switch is None
    try:
        for it in range(max_iter):
            e, Cp = np.linalg.eigh(Fo)
            Cm = X @ Cp
            Cocc = np.ascontiguousarray(Cm[:, :nocc])
            slot = nxt % max_vecs
            E_el, rms, ov = engine.scf_build(Cocc, slot, kmethod)
            E = E_el + enuc
            if audit is not None:
                _, J, K = engine.scf_read(slot, jk=True)
                audits.append(audit(Cocc @ Cocc.T, Cocc, J, K))
            hist.append((it, E, E - E_old, rms))
            if log:
                log(f"iter {it:3d}  E {E:.12f}  dE {E - E_old:.3e}  rms {rms:.3e}")
            if not switched and rms < switch_thresh:
                # as run_rhf: the switch iteration's F is used as it is and
                # not kept for DIIS (its ring slot is reused next)
                switch()
                switched = True
                E_old = E
                c = np.zeros(max_vecs)
                c[slot] = 1.0
                Fo = engine.scf_extrapolate(c)
                continue
            if it > 0 and rms < conv and switched:
                F = engine.scf_read(slot)
                return SCFResult(E, True, it + 1, Cm, e, Cocc @ Cocc.T, F, hist, audits)
            E_old = E
            nxt += 1
            if slot in order:
                order.remove(slot)
            order.append(slot)
            Bm[slot, :] = ov
            Bm[:, slot] = ov
            c = np.zeros(max_vecs)
            if len(order) < 2:
                c[slot] = 1.0
            else:
                n = len(order)
                Bs = -np.ones((n + 1, n + 1))
                Bs[n, n] = 0.0
                Bs[:n, :n] = Bm[np.ix_(order, order)]
                rhs = np.zeros(n + 1)
                rhs[n] = -1.0
                c[order] = np.linalg.lstsq(Bs, rhs, rcond=None)[0][:n]
            Fo = engine.scf_extrapolate(c)
        F = engine.scf_read(slot)
        return SCFResult(E, False, max_iter, Cm, e, Cocc @ Cocc.T, F, hist, audits)
    finally:
        engine.scf_end()
