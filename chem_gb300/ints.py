"""Python side of the host integral engine (libgbints.so, include/gbints.h).

Builds the inputs of the DF Fock build once per molecule, as megalochem's
ints::aoloader::compute does (src/ints/aoloader.cpp:34-398): one-electron
matrices, the Coulomb metric, Schwarz factors, and the Schwarz-screened
3-center tensor laid out as atom-block panels (chem_gb300.layout).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .molecule import Basis, Molecule

_LIBDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(_LIBDIR, "libgbints.so")
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: run __graft_entry__.build() first")
        L = C.CDLL(path)
        L.gbints_basis_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, _ip, _ip, _dp, _dp, _dp]
        L.gbints_basis_destroy.argtypes = [C.c_void_p]
        L.gbints_basis_nbf.argtypes = [C.c_void_p]
        L.gbints_one_electron.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, C.c_int]
        L.gbints_coulomb_2c.argtypes = [C.c_void_p, _dp, C.c_int]
        L.gbints_eri4c.argtypes = [C.c_void_p, _dp, C.c_int]
        L.gbints_schwarz_pairs.argtypes = [C.c_void_p, _dp, C.c_int]
        L.gbints_schwarz_aux.argtypes = [C.c_void_p, _dp, C.c_int]
        L.gbints_basis_shells.argtypes = [C.c_void_p, _ip, _ip, _ip, _dp, _dp, _dp]
        L.gbints_sph_coeffs.argtypes = [C.c_int, _dp]
        L.gbints_eri3c_panels.argtypes = [
            C.c_void_p, C.c_void_p, C.c_int, _ip, C.c_int, _ip, C.c_int, _ip, _ip,
            C.POINTER(C.c_ubyte), C.POINTER(C.c_longlong), _ip, _ip, _ip, _dp, C.c_int]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what} failed with status {rc}")


class BasisHandle:
    """Owns a gbints_basis for one Basis."""

    def __init__(self, basis: Basis):
        L = lib()
        ls = np.array([s.l for s in basis.shells], np.int32)
        npr = np.array([len(s.alpha) for s in basis.shells], np.int32)
        cen = np.ascontiguousarray(np.array([s.center for s in basis.shells], float).reshape(-1))
        al = np.ascontiguousarray(np.concatenate([s.alpha for s in basis.shells]))
        co = np.ascontiguousarray(np.concatenate([s.coef for s in basis.shells]))
        h = C.c_void_p()
        _check(L.gbints_basis_create(C.byref(h), len(ls), _p(ls, _ip), _p(npr, _ip), _p(cen),
                                     _p(al), _p(co)), "gbints_basis_create")
        self.h = h
        self.nbf = L.gbints_basis_nbf(h)
        self.nshell = len(ls)
        assert self.nbf == basis.nbf

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.gbints_basis_destroy(self.h)
            self.h = None


def one_electron(mol: Molecule, which: str, nthreads=0):
    code = {"overlap": 0, "kinetic": 1, "nuclear": 2}[which]
    bh = BasisHandle(mol.basis)
    M = np.zeros((bh.nbf, bh.nbf))
    Z = mol.charges.copy()
    xyz = np.ascontiguousarray(mol.coords.reshape(-1))
    _check(lib().gbints_one_electron(bh.h, code, len(Z), _p(Z), _p(xyz), _p(M), nthreads),
           "gbints_one_electron")
    return M


def coulomb_metric(mol: Molecule, nthreads=0):
    bh = BasisHandle(mol.dfbasis)
    M = np.zeros((bh.nbf, bh.nbf))
    _check(lib().gbints_coulomb_2c(bh.h, _p(M), nthreads), "gbints_coulomb_2c")
    return M


def eri4c(mol: Molecule, nthreads=0):
    bh = BasisHandle(mol.basis)
    n = bh.nbf
    out = np.zeros((n, n, n, n))
    _check(lib().gbints_eri4c(bh.h, _p(out), nthreads), "gbints_eri4c")
    return out


def schwarz(mol: Molecule, nthreads=0):
    """Shell-level Schwarz factors (AO pairs, auxiliary shells)."""
    bh = BasisHandle(mol.basis)
    ah = BasisHandle(mol.dfbasis)
    Z = np.zeros((bh.nshell, bh.nshell))
    z = np.zeros(ah.nshell)
    _check(lib().gbints_schwarz_pairs(bh.h, _p(Z), nthreads), "gbints_schwarz_pairs")
    _check(lib().gbints_schwarz_aux(ah.h, _p(z), nthreads), "gbints_schwarz_aux")
    return Z, z


def eri3c_panels(mol: Molecule, layout, nthreads=0):
    """Fill the panel array of `layout` (chem_gb300.layout.PanelLayout)."""
    bh = BasisHandle(mol.basis)
    ah = BasisHandle(mol.dfbasis)
    B = np.zeros(layout.nnz, float)
    boff = np.ascontiguousarray(mol.basis.block_shell_off, np.int32)
    aoff = np.ascontiguousarray(mol.dfbasis.block_shell_off, np.int32)
    pI = np.ascontiguousarray(layout.pair_I, np.int32)
    pJ = np.ascontiguousarray(layout.pair_J, np.int32)
    keep = np.ascontiguousarray(layout.keep, np.uint8)
    poff = np.ascontiguousarray(layout.panel_off, np.int64)
    pK = np.ascontiguousarray(layout.panel_K, np.int32)
    cij = np.ascontiguousarray(layout.col_IJ, np.int32)
    cji = np.ascontiguousarray(layout.col_JI, np.int32)
    _check(lib().gbints_eri3c_panels(
        bh.h, ah.h, layout.nblk, _p(boff, _ip), layout.nablk, _p(aoff, _ip), len(pI),
        _p(pI, _ip), _p(pJ, _ip), _p(keep, C.POINTER(C.c_ubyte)), _p(poff, C.POINTER(C.c_longlong)),
        _p(pK, _ip), _p(cij, _ip), _p(cji, _ip), _p(B), nthreads), "gbints_eri3c_panels")
    return B


def shell_arrays(basis: Basis):
    """Normalised shell data of a basis as the host engine uses it (for the
    device integral engine): dict of l, nprim, bf_off, centers, alpha, coef."""
    bh = BasisHandle(basis)
    n = bh.nshell
    npr = sum(len(s.alpha) for s in basis.shells)
    out = {"l": np.zeros(n, np.int32), "nprim": np.zeros(n, np.int32),
           "bf_off": np.zeros(n, np.int32), "centers": np.zeros(3 * n),
           "alpha": np.zeros(npr), "coef": np.zeros(npr)}
    _check(lib().gbints_basis_shells(bh.h, _p(out["l"], _ip), _p(out["nprim"], _ip),
                                     _p(out["bf_off"], _ip), _p(out["centers"]),
                                     _p(out["alpha"]), _p(out["coef"])), "gbints_basis_shells")
    return out


def sph_tables(lmax=3):
    """Concatenated cartesian -> spherical tables for l = 0..lmax."""
    parts = []
    for l in range(lmax + 1):
        t = np.zeros((2 * l + 1) * (l + 1) * (l + 2) // 2)
        _check(lib().gbints_sph_coeffs(l, _p(t)), "gbints_sph_coeffs")
        parts.append(t)
    return np.concatenate(parts)
