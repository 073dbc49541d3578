"""Per-molecule setup of the DF Fock build (host side, runs once).

Restates the integral requests and setup megalochem performs before its SCF
loop (src/hf/hfscf.cpp:131-221, src/ints/aoloader.cpp:34-398):
  * S, T, V one-electron matrices and H = T + V;
  * Coulomb metric V_XY, its Cholesky factor L (V = L L^T), L^-1 and
    V^-1 = L^-T L^-1 (src/ints/aoloader.cpp:14-32, src/math/linalg/LLT.cpp);
  * Schwarz factors and the screened panel layout (chem_gb300.layout);
  * the 3-center tensor in panel form.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla

from . import ints
from .layout import PanelLayout, schwarz_layout
from .molecule import Molecule


@dataclass
class DFSystem:
    mol: Molecule
    eps: float
    layout: PanelLayout
    B: np.ndarray
    V: np.ndarray
    Linv: np.ndarray
    Vinv: np.ndarray
    S: np.ndarray = None
    Hcore: np.ndarray = None
    timings: dict = field(default_factory=dict)

    @property
    def nbf(self):
        return self.layout.nbf

    @property
    def naux(self):
        return self.layout.naux

    @property
    def nocc(self):
        return self.mol.nocc


def metric_factors(V):
    """L^-1 (lower) and V^-1 = L^-T L^-1 from the Cholesky factor of V."""
    L = np.linalg.cholesky(V)
    Linv = sla.solve_triangular(L, np.eye(len(V)), lower=True)
    Vinv = Linv.T @ Linv
    return Linv, Vinv


def build_dfsystem(mol: Molecule, eps=1e-10, one_electron=True, nthreads=0,
                   device_ints=False) -> DFSystem:
    """device_ints: leave the 3-center tensor to the device engine
    (B = ("device_ints", mol), computed by gbjk_upload_b_eri3c when the J/K
    engine is created) instead of computing it on the host."""
    t = {}
    t0 = time.perf_counter()
    Zmn, zx = ints.schwarz(mol, nthreads)
    layout = schwarz_layout(mol, Zmn, zx, eps)
    t["schwarz"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    B = ("device_ints", mol) if device_ints else ints.eri3c_panels(mol, layout, nthreads)
    t["eri3c"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    V = ints.coulomb_metric(mol, nthreads)
    Linv, Vinv = metric_factors(V)
    t["metric"] = time.perf_counter() - t0
    S = Hc = None
    if one_electron:
        S = ints.one_electron(mol, "overlap", nthreads)
        Hc = ints.one_electron(mol, "kinetic", nthreads) + ints.one_electron(mol, "nuclear", nthreads)
    return DFSystem(mol, eps, layout, B, V, Linv, Vinv, S, Hc, t)
