"""Python wrapper of the CPU oracle (dfjk_oracle.c) — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm use this module, as the checker or the timed CPU baseline.  The product
path (chem_gb300) never imports it.

Parity unpinned: megalochem's J/K path cannot be built here (DBCSR, libcint,
MPI, ScaLAPACK and HDF5 are absent) and it ships no golden outputs.  The C
restatement is cross-checked against `dense_*` below, an independent numpy
einsum of the same formulas over the dense tensor.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
SO = os.path.join(BUILD, "libdfjk_oracle.so")

_lib = None


class OracleLayout(C.Structure):
    _fields_ = [
        ("nbf", C.c_int), ("naux", C.c_int), ("nblk", C.c_int),
        ("blk_off", C.POINTER(C.c_int)), ("panel_K", C.POINTER(C.c_int)),
        ("panel_off", C.POINTER(C.c_longlong)), ("colmap_off", C.POINTER(C.c_int)),
        ("colmap", C.POINTER(C.c_int)),
    ]


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "dfjk_oracle.c")
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                               "-std=c11", src, "-o", SO, "-lm"])
    return SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(SO)
        dp = C.POINTER(C.c_double)
        lp = C.POINTER(OracleLayout)
        L.oracle_df_j.argtypes = [lp, dp, dp, dp, dp, C.c_double]
        L.oracle_df_j_chol.argtypes = [lp, dp, dp, dp, dp, C.c_double]
        L.oracle_dfmo_k.argtypes = [lp, dp, dp, dp, C.c_int, dp, C.c_double, C.c_longlong]
        L.oracle_dfmo_k_batched.argtypes = [lp, dp, dp, C.c_int, dp, C.c_double, C.c_int,
                                            C.c_longlong, C.c_longlong]
        L.oracle_dfk_occ_batched.argtypes = [lp, dp, dp, C.c_int, dp, C.c_int, dp, C.c_double,
                                             C.c_int, C.c_longlong, C.c_longlong]
        L.oracle_dflmo_k.argtypes = [lp, dp, dp, dp, C.c_int, dp, C.c_double, C.c_longlong]
        L.oracle_dfao_k.argtypes = [lp, dp, dp, dp, dp, C.c_double, C.c_longlong]
        L.oracle_half_transform.argtypes = [lp, dp, dp, C.c_int, dp]
        L.oracle_filter.argtypes = [lp, dp, C.c_double]
        L.oracle_prefit.argtypes = [lp, dp, dp, C.c_int, dp]
        L.oracle_dflmo_k_asym.argtypes = [lp, dp, dp, dp, dp, C.c_int, dp, C.c_double,
                                          C.c_longlong]
        L.oracle_mp2_ll_point.argtypes = [lp, dp, dp, C.c_int, dp, C.c_int, C.c_longlong,
                                          C.c_int, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """Holds a layout and the panel array; computes J/K on the CPU."""

    def __init__(self, layout, B):
        self.layout = layout
        self.B = np.ascontiguousarray(B, float)
        cm = layout.column_map()
        self._blk_off = np.ascontiguousarray(layout.boff, np.int32)
        self._K = np.ascontiguousarray(layout.panel_K, np.int32)
        self._poff = np.ascontiguousarray(layout.panel_off, np.int64)
        self._cmoff = np.ascontiguousarray(np.concatenate([[0], np.cumsum([len(c) for c in cm])]),
                                           np.int32)
        self._cm = np.ascontiguousarray(np.concatenate(cm) if cm else np.zeros(0), np.int32)
        self.L = OracleLayout(layout.nbf, layout.naux, layout.nblk,
                              self._blk_off.ctypes.data_as(C.POINTER(C.c_int)),
                              self._K.ctypes.data_as(C.POINTER(C.c_int)),
                              self._poff.ctypes.data_as(C.POINTER(C.c_longlong)),
                              self._cmoff.ctypes.data_as(C.POINTER(C.c_int)),
                              self._cm.ctypes.data_as(C.POINTER(C.c_int)))

    def df_j(self, Vinv, Ptot, eps=0.0):
        n = self.layout.nbf
        J = np.zeros((n, n))
        lib().oracle_df_j(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Vinv)),
                          _dp(np.ascontiguousarray(Ptot)), _dp(J), eps)
        return J

    def df_j_chol(self, Linv, Ptot, eps=0.0):
        n = self.layout.nbf
        J = np.zeros((n, n))
        lib().oracle_df_j_chol(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Linv)),
                               _dp(np.ascontiguousarray(Ptot)), _dp(J), eps)
        return J

    def dfmo_k(self, Linv, Cocc, eps=0.0, kchunk=0):
        """kchunk: length of the in-order partial sums of the exchange
        contraction (0 = one sum); the device path's value comes from
        chem_gb300.fock.k_split_plan."""
        n = self.layout.nbf
        K = np.zeros((n, n))
        Cocc = np.ascontiguousarray(Cocc, float)
        lp = None if Linv is None else _dp(np.ascontiguousarray(Linv))
        rc = lib().oracle_dfmo_k(C.byref(self.L), _dp(self.B), lp,
                                 _dp(Cocc), Cocc.shape[1], _dp(K), eps, int(kchunk))
        if rc:
            raise MemoryError("oracle_dfmo_k")
        return K

    def dfmo_k_batched(self, Cocc, xb, kc_full, kc_last, eps=0.0):
        """DF-MO K of a pre-fitted tensor summed in auxiliary batches of xb
        rows (the device's batched FP64 order)."""
        C_ = np.ascontiguousarray(Cocc, float)
        K = np.empty((self.layout.nbf, self.layout.nbf))
        rc = lib().oracle_dfmo_k_batched(C.byref(self.L), _dp(self.B), _dp(C_), C_.shape[1],
                                         _dp(K), eps, int(xb), int(kc_full), int(kc_last))
        if rc:
            raise RuntimeError(f"oracle_dfmo_k_batched failed ({rc})")
        return K

    def dfk_occ_batched(self, M, Cocc, ob, kc_full, kc_last, eps=0.0, lmo=False):
        """DF-MO (M = L^-1) or DF-LMO (M = V^-1, lmo=True) K summed in
        occupied batches of ob orbitals (the device's batched FP64 order)."""
        C_ = np.ascontiguousarray(Cocc, float)
        K = np.empty((self.layout.nbf, self.layout.nbf))
        rc = lib().oracle_dfk_occ_batched(C.byref(self.L), _dp(self.B),
                                          _dp(np.ascontiguousarray(M, float)), int(lmo), _dp(C_),
                                          C_.shape[1], _dp(K), eps, int(ob), int(kc_full),
                                          int(kc_last))
        if rc:
            raise RuntimeError(f"oracle_dfk_occ_batched failed ({rc})")
        return K

    def dflmo_k(self, Vinv, Cocc, eps=0.0, kchunk=0):
        n = self.layout.nbf
        K = np.zeros((n, n))
        Cocc = np.ascontiguousarray(Cocc, float)
        rc = lib().oracle_dflmo_k(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Vinv)),
                                  _dp(Cocc), Cocc.shape[1], _dp(K), eps, int(kchunk))
        if rc:
            raise MemoryError("oracle_dflmo_k")
        return K

    def dfao_k(self, Vinv, P, eps=0.0, kchunk=0):
        """kchunk: in-order partial sums of the exchange over t = (X, S)
        (the device path uses chem_gb300.fock.k_split_plan(nbf, naux, nbf))."""
        n = self.layout.nbf
        K = np.zeros((n, n))
        rc = lib().oracle_dfao_k(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Vinv)),
                                 _dp(np.ascontiguousarray(P)), _dp(K), eps, int(kchunk))
        if rc:
            raise MemoryError("oracle_dfao_k")
        return K

    def dflmo_k_asym(self, Vinv, U, Vt, eps=0.0, kchunk=0):
        """Non-symmetric DF-LMO K from left U (nbf x nocc) and right Vt
        (nocc x nbf) coefficients."""
        n = self.layout.nbf
        K = np.zeros((n, n))
        U = np.ascontiguousarray(U, float)
        V = np.ascontiguousarray(np.asarray(Vt, float).T)
        rc = lib().oracle_dflmo_k_asym(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Vinv)),
                                       _dp(U), _dp(V), U.shape[1], _dp(K), eps, int(kchunk))
        if rc:
            raise MemoryError("oracle_dflmo_k_asym")
        return K

    def half_transform(self, Cocc):
        n, naux = self.layout.nbf, self.layout.naux
        Cocc = np.ascontiguousarray(Cocc, float)
        H = np.zeros((n, naux, Cocc.shape[1]))
        lib().oracle_half_transform(C.byref(self.L), _dp(self.B), _dp(Cocc), Cocc.shape[1], _dp(H))
        return H

    def prefit(self, Linv, nx=0):
        """L^-1 B per panel in the device's lower-triangular GEMM order; only
        the first nx auxiliary rows when nx > 0 (the rest stay zero)."""
        Bf = np.zeros_like(self.B)
        lib().oracle_prefit(C.byref(self.L), _dp(self.B), _dp(np.ascontiguousarray(Linv)),
                            int(nx), _dp(Bf))
        return Bf

    def mp2_ll_point(self, Bfit, Lo, Lv, kchunk=0, nx=0):
        """(Z~, e) of one Laplace point (ll_full builder) on the prefitted
        tensor, in the device path's padded layouts and summation order.
        nx > 0 restricts to the first nx auxiliary functions."""
        n = self.layout.nbf
        ro, rv = Lo.shape[1], Lv.shape[1]
        hld, vld = ro + (ro & 1), rv + (rv & 1)
        lo = np.zeros((n, hld)); lo[:, :ro] = Lo
        lv = np.zeros((n, vld)); lv[:, :rv] = Lv
        m = nx if 0 < nx < self.layout.naux else self.layout.naux
        Z = np.zeros((m, m))
        e = C.c_double()
        rc = lib().oracle_mp2_ll_point(C.byref(self.L), _dp(np.ascontiguousarray(Bfit)), _dp(lo),
                                       hld, _dp(lv), vld, int(kchunk), int(nx), _dp(Z),
                                       C.byref(e))
        if rc:
            raise MemoryError("oracle_mp2_ll_point")
        return Z, e.value

    def filter(self, M, eps):
        M = np.ascontiguousarray(M, float).copy()
        lib().oracle_filter(C.byref(self.L), _dp(M), eps)
        return M


# --- independent dense restatements (numpy einsum) -------------------------

def dense_j(T, Vinv, Ptot):
    g = np.einsum("xmn,mn->x", T, Ptot)
    return np.einsum("x,xmn->mn", Vinv @ g, T)


def dense_dfmo_k(T, Linv, Cocc):
    H = np.einsum("xmn,mi->xin", T, Cocc)
    H2 = np.einsum("yx,xin->yin", Linv, H)
    return -np.einsum("xim,xin->mn", H2, H2)


def dense_dflmo_k(T, Vinv, Cocc):
    H = np.einsum("xmn,ni->xmi", T, Cocc)
    Hf = np.einsum("xy,ymi->xmi", Vinv, H)
    return -np.einsum("xmi,xni->nm", H, Hf)


def dense_dfao_k(T, Vinv, P):
    cbar = np.einsum("xmn,nl->xml", T, P)
    c = np.einsum("xy,yns->xns", Vinv, T)
    return -np.einsum("xns,xms->mn", c, cbar)


# --- SOS-AO-MP2 Laplace term (dense numpy restatements) -------------------

def dense_mp2_ll(T, Vinv, Lo, Lv):
    """ll_full route (src/mp/z_full.cpp:427-620): B_xov = Lo^T (X|mn) Lv,
    Z = B_xov B_xov^T, e = tr(Z V^-1 Z V^-1) (mp_compute.cpp:361-381)."""
    W = np.einsum("mi,xmn,na->xia", Lo, T, Lv, optimize=True)
    Z = np.einsum("xia,yia->xy", W, W, optimize=True)
    Zt = Z @ Vinv
    return Z, float(np.sum(Zt * Zt.T))


def dense_mp2_llmp(T, Vinv, Lo, Pv, pair_mask):
    """llmp_full route, megalochem's default Z builder (z_full.cpp:69-397):
    B = Lo^T (X|mn), B2 = B Pv, B3 = Lo B2 kept on the screened shell-pair
    pattern, Z(X,Y) = sum_mn B3(X,m,n) (Y|mn)."""
    B1 = np.einsum("mi,xmn->xin", Lo, T, optimize=True)
    B2 = np.einsum("Nn,xin->xiN", Pv, B1, optimize=True)
    B3 = np.einsum("Mi,xiN->xMN", Lo, B2, optimize=True) * pair_mask[None]
    Z = np.einsum("xmn,ymn->xy", B3, T, optimize=True)
    Zt = Z @ Vinv
    return Z, float(np.sum(Zt * Zt.T))


def dense_sos_mp2(T, Vinv, C_occ, C_vir, e_occ, e_vir):
    """sum_{ijab} (ia|jb)^2 / (e_a + e_b - e_i - e_j) with DF integrals: the
    quantity the Laplace sum of e_t approximates."""
    Bia = np.einsum("xmn,mi,na->xia", T, C_occ, C_vir, optimize=True)
    Lc = np.linalg.cholesky(Vinv)
    Q = np.einsum("xy,xia->yia", Lc, Bia, optimize=True)
    iajb = np.einsum("yia,yjb->iajb", Q, Q, optimize=True)
    den = (e_vir[None, :, None, None] + e_vir[None, None, None, :]
           - e_occ[:, None, None, None] - e_occ[None, None, :, None])
    return float(np.sum(iajb ** 2 / den))


def dense_dflmo_k_asym(T, Vinv, U, Vt):
    Hu = np.einsum("xmn,ni->xmi", T, U)
    Hv = np.einsum("xmn,in->xmi", T, Vt)
    Hf = np.einsum("xy,ymi->xmi", Vinv, Hv)
    return -np.einsum("xmi,xni->mn", Hu, Hf)
