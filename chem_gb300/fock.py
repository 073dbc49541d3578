"""J/K builders over the GB300 engine (libgbjk.so, include/gbjk.h).

Mirrors megalochem's builder interface (src/fock/jkbuilder.hpp:62-210):
abstract J and K classes with set_density_alpha/beta, set_coeff_alpha/beta,
set_sym, set_SAD, init(), compute_J()/compute_K(), get_J()/get_K_A()/get_K_B(),
and factories create_j()/create_k() keyed by the same method strings
("dfao" for J; "dfmo", "dflmo" for K).  Errors raise RuntimeError with the
engine's message, as the reference throws std::runtime_error.

All arithmetic runs in the CUDA library; this module only moves host arrays
across the C ABI.  There is no CPU fallback: without the built library (or a
GPU) every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_LIBDIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")
_lib = None

GBJK_FP64 = 0
GBJK_SPLIT_BF16 = 1
KMETHODS = {"dfmo": 0, "dflmo": 1}  # coefficient-based; "dfao" takes the density
JMETHODS = ("dfao",)
STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT",
          5: "NOT_CONVERGED", 6: "NOT_READY"}


class GbjkShells(C.Structure):
    _fields_ = [("nshell", C.c_int), ("l", C.POINTER(C.c_int)), ("nprim", C.POINTER(C.c_int)),
                ("bf_off", C.POINTER(C.c_int)), ("centers", C.POINTER(C.c_double)),
                ("alpha", C.POINTER(C.c_double)), ("coef", C.POINTER(C.c_double))]


class GbjkTunables(C.Structure):
    _fields_ = [("fp64_ht_tn", C.c_int), ("fp64_k_tile", C.c_int), ("fp64_kchunk", C.c_longlong),
                ("split_ksplit", C.c_int), ("overlap_sms", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class GbjkDesc(C.Structure):
    _fields_ = [("nbf", C.c_int), ("naux", C.c_int), ("nblk", C.c_int),
                ("blk_size", C.POINTER(C.c_int)), ("panel_K", C.POINTER(C.c_int)),
                ("colmap", C.POINTER(C.c_int)), ("filter_eps", C.c_double), ("device", C.c_int)]


def lib_path():
    return os.path.join(_LIBDIR, "libgbjk.so")


def lib():
    """Load libgbjk.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(f"{path} missing: the CUDA engine is not built "
                               "(run __graft_entry__.build())")
        L = C.CDLL(path)
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.gbjk_create.argtypes = [C.POINTER(vp), C.POINTER(GbjkDesc)]
        L.gbjk_destroy.argtypes = [vp]
        L.gbjk_last_error.argtypes = [vp]
        L.gbjk_last_error.restype = C.c_char_p
        L.gbjk_upload_b.argtypes = [vp, dp]
        L.gbjk_upload_metric.argtypes = [vp, dp, dp]
        L.gbjk_set_precision.argtypes = [vp, C.c_int, C.c_int]
        L.gbjk_set_jmode.argtypes = [vp, C.c_int]
        L.gbjk_set_overlap.argtypes = [vp, C.c_int]
        L.gbjk_test_split_stall.argtypes = [vp, C.c_int, C.c_double]
        L.gbjk_scf_begin.argtypes = [vp, dp, dp, dp, C.c_int, C.c_int]
        L.gbjk_scf_build.argtypes = [vp, C.c_int, dp, C.c_int, dp]
        L.gbjk_scf_extrapolate.argtypes = [vp, dp, dp]
        L.gbjk_scf_read.argtypes = [vp, C.c_int, dp, dp, dp]
        L.gbjk_scf_end.argtypes = [vp]
        L.gbjk_get_overlap.argtypes = [vp]
        L.gbjk_get_overlap.restype = C.c_int
        L.gbjk_set_split_fuse.argtypes = [vp, C.c_int]
        L.gbjk_get_split_fuse.argtypes = [vp]
        L.gbjk_get_split_fuse.restype = C.c_int
        L.gbjk_set_fitted.argtypes = [vp, C.c_int]
        L.gbjk_set_aux_batch.argtypes = [vp, C.c_int]
        L.gbjk_set_occ_batch.argtypes = [vp, C.c_int]
        L.gbjk_upload_b_synthetic.argtypes = [vp, C.c_ulonglong, C.c_double]
        L.gbjk_download_b.argtypes = [vp, dp]
        ip = C.POINTER(C.c_int)
        L.gbjk_upload_b_eri3c.argtypes = [vp, C.POINTER(GbjkShells), C.POINTER(GbjkShells), dp,
                                          ip, C.c_int, ip, C.c_int, ip, ip,
                                          C.POINTER(C.c_ubyte), ip, ip]
        L.gbjk_compute_j.argtypes = [vp, dp, dp]
        L.gbjk_compute_k.argtypes = [vp, C.c_int, dp, C.c_int, dp]
        L.gbjk_compute_jk.argtypes = [vp, C.c_int, dp, dp, C.c_int, dp, dp]
        L.gbjk_compute_k_ao.argtypes = [vp, dp, dp]
        L.gbjk_compute_k_lmo_asym.argtypes = [vp, dp, dp, C.c_int, dp]
        L.gbjk_compute_k_ao_dev.argtypes = [vp, C.c_void_p, C.c_void_p]
        L.gbjk_compute_jk_dev.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p]
        L.gbjk_synchronize.argtypes = [vp]
        L.gbjk_capture_graph.argtypes = [vp, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_void_p, C.c_void_p]
        L.gbjk_launch_graph.argtypes = [vp]
        L.gbjk_host_alloc.argtypes = [C.c_size_t]
        L.gbjk_host_alloc.restype = C.c_void_p
        L.gbjk_host_free.argtypes = [C.c_void_p]
        L.gbjk_stream.argtypes = [vp]
        L.gbjk_stream.restype = C.c_void_p
        L.gbjk_device_bytes.argtypes = [vp]
        L.gbjk_device_bytes.restype = C.c_size_t
        L.gbjk_kernel_launches.argtypes = [vp]
        L.gbjk_kernel_launches.restype = C.c_int64
        L.gbjk_k_split_plan.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_longlong)]
        tp = C.POINTER(GbjkTunables)
        L.gbjk_tune_plan.argtypes = [C.c_int, C.c_int, C.c_int, tp, tp, C.POINTER(C.c_int)]
        L.gbjk_set_tunables.argtypes = [vp, tp]
        L.gbjk_get_tunables.argtypes = [vp, tp]
        L.gbjk_tune_signature.argtypes = [vp, C.c_int, C.c_int, C.c_char_p, C.c_size_t]
        L.gbjk_tune_cache_lookup.argtypes = [C.c_char_p, C.c_char_p, tp]
        L.gbjk_tune_cache_store.argtypes = [C.c_char_p, C.c_char_p, tp]
        L.gbjk_autotune.argtypes = [vp, C.c_int, dp, dp, C.c_int, C.c_int, C.c_char_p,
                                    C.c_char_p, C.c_size_t]
        L.gbjk_profile.argtypes = [vp, C.c_int]
        L.gbjk_profile_read.argtypes = [vp, C.c_int, C.POINTER(C.c_char_p), dp,
                                        C.POINTER(C.c_int64)]
        ip, dpp = C.POINTER(C.c_int), C.POINTER(dp)
        L.gbjk_mp2_set_factors.argtypes = [vp, C.c_int, ip, dpp, ip, dpp]
        L.gbjk_mp2_compute_dev.argtypes = [vp]
        L.gbjk_mp2_read.argtypes = [vp, dp, dp]
        L.gbjk_mp2_laplace.argtypes = [vp, C.c_int, ip, dpp, ip, dpp, dp, dp]
        L.gbjk_mp2_release.argtypes = [vp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def tune_plan(nbf, naux, nocc, **req):
    """Effective FP64 launch choices (dict) and the exchange's number of k
    parts for a problem and requested tunables (gbjk_tune_plan; no GPU)."""
    r = GbjkTunables(**req)
    e = GbjkTunables()
    ks = C.c_int()
    if lib().gbjk_tune_plan(nbf, naux, nocc, C.byref(r), C.byref(e), C.byref(ks)) != 0:
        raise RuntimeError("gbjk_tune_plan: invalid arguments")
    return e.as_dict(), ks.value


def tune_cache_lookup(path, sig):
    t = GbjkTunables()
    rc = lib().gbjk_tune_cache_lookup(path.encode(), sig.encode(), C.byref(t))
    return t.as_dict() if rc == 0 else None


def tune_cache_store(path, sig, **tun):
    if lib().gbjk_tune_cache_store(path.encode(), sig.encode(), C.byref(GbjkTunables(**tun))):
        raise RuntimeError("gbjk_tune_cache_store failed")


def k_split_plan(nbf, naux, nocc):
    """(ksplit, kchunk) of the device exchange contraction (gbjk_k_split_plan)."""
    ks = C.c_int()
    kc = C.c_longlong()
    if lib().gbjk_k_split_plan(nbf, naux, nocc, C.byref(ks), C.byref(kc)) != 0:
        raise RuntimeError("gbjk_k_split_plan: invalid arguments")
    return ks.value, kc.value


class _PinnedBuffer:
    """Page-locked host bytes from gbjk_host_alloc, freed with the last array
    that views them."""

    def __init__(self, nbytes):
        self.ptr = lib().gbjk_host_alloc(max(1, nbytes))
        if not self.ptr:
            raise MemoryError(f"gbjk_host_alloc of {nbytes} bytes failed")
        self.__array_interface__ = {"shape": (nbytes,), "typestr": "|u1",
                                    "data": (self.ptr, False), "version": 3}

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and _lib is not None:  # at interpreter exit the library may be gone
            _lib.gbjk_host_free(ptr)


def host_array(shape, dtype=np.float64):
    """A numpy array in page-locked host memory (gbjk_host_alloc): inputs and
    outputs of the host-buffer calls in this memory are copied by DMA."""
    dt = np.dtype(dtype)
    shape = (shape,) if np.isscalar(shape) else tuple(int(d) for d in shape)
    nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
    return np.asarray(_PinnedBuffer(nbytes))[:nbytes].view(dt).reshape(shape)


class JKEngine:
    """One gbjk context: the resident 3-center tensor and metric of a molecule."""

    def __init__(self, layout, B, Linv, Vinv, eps=0.0, device=0, precision=GBJK_FP64,
                 nslices=0, fitted=False, synthetic=None, aux_batch=0):
        """B: host panel array, or None with synthetic=(seed, decay) to
        generate it on the device.  fitted: B already is L^-1 B (Linv and
        Vinv may be None).  aux_batch: split path auxiliary batch rows."""
        L = lib()
        self.layout = layout
        self.nbf, self.naux = layout.nbf, layout.naux
        cm = layout.column_map()
        self._bs = np.ascontiguousarray(layout.bsizes, np.int32)
        self._K = np.ascontiguousarray(layout.panel_K, np.int32)
        self._cm = np.ascontiguousarray(np.concatenate(cm), np.int32)
        desc = GbjkDesc(self.nbf, self.naux, layout.nblk,
                        self._bs.ctypes.data_as(C.POINTER(C.c_int)),
                        self._K.ctypes.data_as(C.POINTER(C.c_int)),
                        self._cm.ctypes.data_as(C.POINTER(C.c_int)), float(eps), int(device))
        h = C.c_void_p()
        rc = L.gbjk_create(C.byref(h), C.byref(desc))
        if rc != 0:
            raise RuntimeError(f"gbjk_create failed: {STATUS.get(rc, rc)}")
        self.h = h
        if fitted:
            self._check(L.gbjk_set_fitted(h, 1), "gbjk_set_fitted")
        if aux_batch:
            self._check(L.gbjk_set_aux_batch(h, int(aux_batch)), "gbjk_set_aux_batch")
        if isinstance(B, tuple) and B and B[0] == "device_ints":
            self.upload_b_device_ints(B[1])
        elif B is None:
            if synthetic is None:
                raise ValueError("B or synthetic=(seed, decay) is required")
            seed, decay = synthetic
            self._check(L.gbjk_upload_b_synthetic(h, int(seed), float(decay)),
                        "gbjk_upload_b_synthetic")
        else:
            B = np.ascontiguousarray(B, float)
            if B.size != layout.nnz:
                raise ValueError("B does not match the layout")
            self._check(L.gbjk_upload_b(h, _dp(B)), "gbjk_upload_b")
        if Linv is not None:
            self._check(L.gbjk_upload_metric(h, _dp(np.ascontiguousarray(Linv, float)),
                                             _dp(np.ascontiguousarray(Vinv, float))),
                        "gbjk_upload_metric")
        self.set_precision(precision, nslices)

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().gbjk_last_error(self.h).decode()
            raise RuntimeError(f"{what}: {STATUS.get(rc, rc)}: {msg}")

    def set_precision(self, precision, nslices=0):
        if isinstance(precision, str):
            precision = {"fp64": GBJK_FP64, "split": GBJK_SPLIT_BF16,
                         "split_bf16": GBJK_SPLIT_BF16}[precision]
        self._check(lib().gbjk_set_precision(self.h, int(precision), int(nslices)),
                    "gbjk_set_precision")
        self.precision = precision

    def download_b(self):
        B = np.empty(self.layout.nnz)
        self._check(lib().gbjk_download_b(self.h, _dp(B)), "gbjk_download_b")
        return B

    def set_tunables(self, **tun):
        """Launch choices (gbjk_tunables fields; omitted or 0 = built-in rule)."""
        self._check(lib().gbjk_set_tunables(self.h, C.byref(GbjkTunables(**tun))),
                    "gbjk_set_tunables")

    def get_tunables(self):
        """The launch choices in effect at the last build."""
        t = GbjkTunables()
        self._check(lib().gbjk_get_tunables(self.h, C.byref(t)), "gbjk_get_tunables")
        return t.as_dict()

    def tune_signature(self, kmethod="dfmo", nocc=None):
        buf = C.create_string_buffer(768)
        self._check(lib().gbjk_tune_signature(self.h, KMETHODS[kmethod], int(nocc), buf, 768),
                    "gbjk_tune_signature")
        return buf.value.decode()

    def autotune(self, Ptot, Cocc, kmethod="dfmo", reps=3, cache=None):
        """Time candidate launch configurations of one Fock build at the
        engine's precision and keep the fastest (gbjk_autotune); with a
        cache file holding this problem's signature the recorded choice is
        adopted without timing.  Returns the report as a dict."""
        import json
        P = np.ascontiguousarray(Ptot, dtype=np.float64)
        Cm = np.ascontiguousarray(Cocc, dtype=np.float64)
        buf = C.create_string_buffer(1 << 16)
        self._check(lib().gbjk_autotune(self.h, KMETHODS[kmethod], _dp(P), _dp(Cm), Cm.shape[1],
                                        int(reps), cache.encode() if cache else None, buf,
                                        1 << 16), "gbjk_autotune")
        return json.loads(buf.value.decode())

    # --- SCF iteration on the device (gbjk_scf_*) ---------------------------
    def scf_begin(self, H, S, X, nocc, max_diis=8):
        """Upload H, S and the symmetric orthogonaliser X for the device SCF
        iteration; max_diis ring slots for Fock and error matrices."""
        self._scf_nslots = int(max_diis)
        a = [np.ascontiguousarray(m, dtype=np.float64) for m in (H, S, X)]
        self._check(lib().gbjk_scf_begin(self.h, _dp(a[0]), _dp(a[1]), _dp(a[2]), int(nocc),
                                         int(max_diis)), "gbjk_scf_begin")

    def scf_build(self, Cocc, slot, kmethod="dfmo"):
        """One SCF build on the device from C_occ: returns (E_el, rms,
        overlaps of the new error matrix with every ring slot)."""
        Cm = np.ascontiguousarray(Cocc, dtype=np.float64)
        out = np.empty(2 + self._scf_nslots)
        self._check(lib().gbjk_scf_build(self.h, KMETHODS[kmethod], _dp(Cm), int(slot), _dp(out)),
                    "gbjk_scf_build")
        return float(out[0]), float(out[1]), out[2:].copy()

    def scf_extrapolate(self, coef):
        """Fo = X (sum_j coef[j] F_j) X from the ring (device)."""
        c = np.zeros(self._scf_nslots)
        c[:len(coef)] = coef
        Fo = np.empty((self.nbf, self.nbf))
        self._check(lib().gbjk_scf_extrapolate(self.h, _dp(c), _dp(Fo)), "gbjk_scf_extrapolate")
        return Fo

    def scf_read(self, slot, jk=False):
        """F of a ring slot (and J, K of the last build when jk)."""
        F = np.empty((self.nbf, self.nbf))
        J = np.empty_like(F) if jk else None
        K = np.empty_like(F) if jk else None
        self._check(lib().gbjk_scf_read(self.h, int(slot), _dp(F), _dp(J) if jk else None,
                                        _dp(K) if jk else None), "gbjk_scf_read")
        return (F, J, K) if jk else F

    def scf_end(self):
        self._check(lib().gbjk_scf_end(self.h), "gbjk_scf_end")

    def test_split_stall(self, item, wait_ms=5.0):
        """Failure-detection test hook (gbjk_test_split_stall): item >= 0
        makes the split GEMM stop producing at that work item, so the
        bounded waits run out and builds report TIMEOUT; -1 restores."""
        self._check(lib().gbjk_test_split_stall(self.h, int(item), float(wait_ms)),
                    "gbjk_test_split_stall")

    def set_occ_batch(self, cols):
        """FP64 K in occupied batches of `cols` orbitals (0: all at once)."""
        self._check(lib().gbjk_set_occ_batch(self.h, int(cols)), "gbjk_set_occ_batch")

    def set_overlap(self, sms):
        """SMs the mixed-path exchange leaves to the concurrent J column
        sums on a second stream (0, default: none, the J blocks co-reside
        with the exchange CTAs; -1: phases in order on one stream)."""
        self._check(lib().gbjk_set_overlap(self.h, int(sms)), "gbjk_set_overlap")

    def get_overlap(self):
        return int(lib().gbjk_get_overlap(self.h))

    def set_split_fuse(self, on):
        """Mixed-path exchange digits: cut in the half-transform epilogue
        with one exponent per (AO function, 32 auxiliary indices) (True), or
        from an FP64 H with one exponent per AO function (False, default)."""
        self._check(lib().gbjk_set_split_fuse(self.h, 1 if on else 0), "gbjk_set_split_fuse")

    def get_split_fuse(self):
        return bool(lib().gbjk_get_split_fuse(self.h))

    def set_jmode(self, jmode):
        """'vinv' (reference route, default) or 'cholesky'."""
        code = {"vinv": 0, "cholesky": 1}[jmode]
        self._check(lib().gbjk_set_jmode(self.h, code), "gbjk_set_jmode")

    def compute_jk(self, Ptot=None, Cocc=None, kmethod="dfmo", out=None):
        """J from the total density and K from the occupied coefficients
        (gbjk_compute_jk).  `out=(J, K)` writes into caller-owned
        C-contiguous float64 nbf x nbf arrays, e.g. from host_array(), whose
        page-locked memory the copies reach by DMA."""
        n = self.nbf
        if out is not None:
            J, K = out
            for a, want in ((J, Ptot is not None), (K, Cocc is not None)):
                if want and (a is None or a.shape != (n, n) or a.dtype != np.float64
                             or not a.flags.c_contiguous or not a.flags.writeable):
                    raise ValueError("out arrays must be writable C-contiguous float64 nbf x nbf")
            J = J if Ptot is not None else None
            K = K if Cocc is not None else None
        else:
            J = np.empty((n, n)) if Ptot is not None else None
            K = np.empty((n, n)) if Cocc is not None else None
        P = np.ascontiguousarray(Ptot, float) if Ptot is not None else None
        Cm = np.ascontiguousarray(Cocc, float) if Cocc is not None else None
        nocc = Cm.shape[1] if Cm is not None else 0
        self._check(lib().gbjk_compute_jk(
            self.h, KMETHODS[kmethod], _dp(P) if P is not None else None,
            _dp(Cm) if Cm is not None else None, nocc,
            _dp(J) if J is not None else None, _dp(K) if K is not None else None),
            "gbjk_compute_jk")
        return J, K

    def upload_b_device_ints(self, mol):
        """Compute the 3-center tensor on the device (gbjk_upload_b_eri3c)
        for molecule `mol` on this engine's layout."""
        from . import ints
        lay = self.layout
        keep_alive = []

        def shells(basis):
            d = ints.shell_arrays(basis)
            keep_alive.append(d)
            ptr = lambda a, t: a.ctypes.data_as(C.POINTER(t))
            return GbjkShells(len(d["l"]), ptr(d["l"], C.c_int), ptr(d["nprim"], C.c_int),
                              ptr(d["bf_off"], C.c_int), ptr(d["centers"], C.c_double),
                              ptr(d["alpha"], C.c_double), ptr(d["coef"], C.c_double))
        ao, ax = shells(mol.basis), shells(mol.dfbasis)
        sph = ints.sph_tables(3)
        arr = {k: np.ascontiguousarray(v, np.int32) for k, v in (
            ("boff", mol.basis.block_shell_off), ("aoff", mol.dfbasis.block_shell_off),
            ("pI", lay.pair_I), ("pJ", lay.pair_J), ("cij", lay.col_IJ), ("cji", lay.col_JI))}
        keep = np.ascontiguousarray(lay.keep, np.uint8)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
        self._check(lib().gbjk_upload_b_eri3c(
            self.h, C.byref(ao), C.byref(ax), _dp(sph), ip(arr["boff"]), lay.nablk,
            ip(arr["aoff"]), len(arr["pI"]), ip(arr["pI"]), ip(arr["pJ"]),
            keep.ctypes.data_as(C.POINTER(C.c_ubyte)), ip(arr["cij"]), ip(arr["cji"])),
            "gbjk_upload_b_eri3c")

    def compute_k_ao(self, P):
        """DF-AO K (gbjk_compute_k_ao) from the alpha density P; K negated."""
        P = np.ascontiguousarray(P, float)
        K = np.zeros((self.nbf, self.nbf))
        self._check(lib().gbjk_compute_k_ao(self.h, _dp(P), _dp(K)), "gbjk_compute_k_ao")
        return K

    def compute_k_lmo_asym(self, U, Vt):
        """Non-symmetric DF-LMO K (gbjk_compute_k_lmo_asym): U nbf x nocc,
        Vt nocc x nbf; K negated."""
        U = np.ascontiguousarray(U, float)
        Vt = np.ascontiguousarray(Vt, float)
        if U.shape[0] != self.nbf or Vt.shape != (U.shape[1], self.nbf):
            raise ValueError("U must be nbf x nocc and Vt nocc x nbf")
        K = np.zeros((self.nbf, self.nbf))
        self._check(lib().gbjk_compute_k_lmo_asym(self.h, _dp(U), _dp(Vt), U.shape[1], _dp(K)),
                    "gbjk_compute_k_lmo_asym")
        return K

    def compute_k_ao_dev(self, dP, dK):
        self._check(lib().gbjk_compute_k_ao_dev(self.h, dP, dK), "gbjk_compute_k_ao_dev")

    def compute_jk_dev(self, dP, dC, nocc, dJ, dK, kmethod="dfmo"):
        """Device pointers (ints); ordered on the engine stream, no sync."""
        self._check(lib().gbjk_compute_jk_dev(self.h, KMETHODS[kmethod], dP, dC, int(nocc),
                                              dJ, dK), "gbjk_compute_jk_dev")

    def capture_graph(self, dP, dC, nocc, dJ, dK, kmethod="dfmo"):
        """Capture one device-pointer build as a CUDA graph (see gbjk.h)."""
        self._check(lib().gbjk_capture_graph(self.h, KMETHODS[kmethod], dP, dC, int(nocc),
                                             dJ, dK), "gbjk_capture_graph")

    def launch_graph(self):
        self._check(lib().gbjk_launch_graph(self.h), "gbjk_launch_graph")

    def synchronize(self):
        self._check(lib().gbjk_synchronize(self.h), "gbjk_synchronize")

    @property
    def stream(self):
        return lib().gbjk_stream(self.h)

    @property
    def device_bytes(self):
        return int(lib().gbjk_device_bytes(self.h))

    @property
    def kernel_launches(self):
        return int(lib().gbjk_kernel_launches(self.h))

    def profile(self, enable=True):
        self._check(lib().gbjk_profile(self.h, int(enable)), "gbjk_profile")

    # --- SOS-AO-MP2 Laplace batch (gbjk_mp2_*) ------------------------------
    def mp2_set_factors(self, Lo, Lv):
        """Lo, Lv: per Laplace point, the occupied (nbf x r_t) and virtual
        (nbf x rv_t) Cholesky factors of the pseudo-densities."""
        if len(Lo) != len(Lv) or not Lo:
            raise ValueError("need one occupied and one virtual factor per point")
        lo = [np.ascontiguousarray(a, float) for a in Lo]
        lv = [np.ascontiguousarray(a, float) for a in Lv]
        for a in lo + lv:
            if a.ndim != 2 or a.shape[0] != self.nbf:
                raise ValueError("factors must be nbf x rank")
        n = len(lo)
        ro = np.array([a.shape[1] for a in lo], np.int32)
        rv = np.array([a.shape[1] for a in lv], np.int32)
        dpp = C.POINTER(C.c_double) * n
        plo, plv = dpp(*[_dp(a) for a in lo]), dpp(*[_dp(a) for a in lv])
        self._check(lib().gbjk_mp2_set_factors(self.h, n, ro.ctypes.data_as(C.POINTER(C.c_int)), plo,
                                               rv.ctypes.data_as(C.POINTER(C.c_int)), plv),
                    "gbjk_mp2_set_factors")
        self._mp2_npts = n

    def mp2_compute_dev(self):
        self._check(lib().gbjk_mp2_compute_dev(self.h), "gbjk_mp2_compute_dev")

    def mp2_read(self, want_z=False):
        """(e_t per point, Z~_t stacked or None)."""
        n = self._mp2_npts
        e = np.zeros(n)
        Z = np.zeros((n, self.naux, self.naux)) if want_z else None
        self._check(lib().gbjk_mp2_read(self.h, _dp(e), _dp(Z) if want_z else None),
                    "gbjk_mp2_read")
        return e, Z

    def mp2_laplace(self, Lo, Lv, want_z=False):
        self.mp2_set_factors(Lo, Lv)
        self.mp2_compute_dev()
        return self.mp2_read(want_z)

    def mp2_release(self):
        self._check(lib().gbjk_mp2_release(self.h), "gbjk_mp2_release")

    def profile_read(self):
        out = {}
        i = 0
        name = C.c_char_p()
        ms = C.c_double()
        n = C.c_int64()
        while lib().gbjk_profile_read(self.h, i, C.byref(name), C.byref(ms), C.byref(n)):
            out[name.value.decode()] = (ms.value, n.value)
            i += 1
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().gbjk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --- builder classes with the reference's interface ------------------------

class JK_common:
    def __init__(self, engine: JKEngine):
        self.engine = engine
        self.m_p_A = self.m_p_B = self.m_c_A = self.m_c_B = None
        self.m_sym = True
        self.m_SAD_iter = False
        self.m_SAD_rank = 0

    def set_density_alpha(self, P):
        self.m_p_A = P

    def set_density_beta(self, P):
        self.m_p_B = P

    def set_coeff_alpha(self, Cm):
        self.m_c_A = Cm

    def set_coeff_beta(self, Cm):
        self.m_c_B = Cm

    def set_sym(self, sym):
        self.m_sym = bool(sym)

    def set_SAD(self, sad, rank):
        self.m_SAD_iter, self.m_SAD_rank = bool(sad), int(rank)


class J(JK_common):
    def init(self):
        self.m_J = None

    def get_J(self):
        return self.m_J


class K(JK_common):
    def init(self):
        self.m_K_A = self.m_K_B = None

    def get_K_A(self):
        return self.m_K_A

    def get_K_B(self):
        return self.m_K_B


class DF_J(J):
    """fock::DF_J (src/fock/jkdf.cpp:13-190): P_tot = 2 P_A (RHF) or P_A + P_B."""

    def compute_J(self):
        if self.m_p_A is None:
            raise RuntimeError("DF_J: density not set")
        Ptot = 2.0 * self.m_p_A if self.m_p_B is None else self.m_p_A + self.m_p_B
        self.m_J, _ = self.engine.compute_jk(Ptot=Ptot)


class _DFK(K):
    kmethod = "dfmo"

    def compute_K(self):
        if self.m_c_A is None:
            raise RuntimeError(f"{type(self).__name__}: coefficients not set")
        _, self.m_K_A = self.engine.compute_jk(Cocc=self.m_c_A, kmethod=self.kmethod)
        if self.m_c_B is not None:
            _, self.m_K_B = self.engine.compute_jk(Cocc=self.m_c_B, kmethod=self.kmethod)


class DFMO_K(_DFK):
    """fock::DFMO_K (src/fock/jkdf.cpp:192-462)."""
    kmethod = "dfmo"


class DFLMO_K(_DFK):
    """fock::DFLMO_K (src/fock/jkdf.cpp:861-1323): the symmetric branch from
    set_coeff_alpha, or with set_sym(False) the non-symmetric one from
    set_coeff_left_alpha (nbf x nocc) and set_coeff_right_alpha (nocc x nbf),
    as the ADC matrix-vector products call it."""
    kmethod = "dflmo"

    def set_coeff_left_alpha(self, U):
        self.m_u_A = U

    def set_coeff_right_alpha(self, Vt):
        self.m_v_A = Vt

    def compute_K(self):
        if self.m_sym:
            return super().compute_K()
        if getattr(self, "m_u_A", None) is None or getattr(self, "m_v_A", None) is None:
            raise RuntimeError("DFLMO_K: left/right coefficients not set")
        self.m_K_A = self.engine.compute_k_lmo_asym(self.m_u_A, self.m_v_A)


class DFAO_K(K):
    """fock::DFAO_K (src/fock/jkdf.cpp:464-648): K from the alpha (and beta)
    density with the fitting coefficients V^-1 (X|mn)."""

    def compute_K(self):
        if self.m_p_A is None:
            raise RuntimeError("DFAO_K: density not set")
        self.m_K_A = self.engine.compute_k_ao(self.m_p_A)
        self.m_K_B = None if self.m_p_B is None else self.engine.compute_k_ao(self.m_p_B)


def create_j(engine: JKEngine, method="dfao") -> J:
    """fock::create_j (src/fock/jkbuilder.hpp:621-690)."""
    if method not in JMETHODS:
        raise RuntimeError("Invalid jmethod")
    return DF_J(engine)


def create_k(engine: JKEngine, method="dfmo") -> K:
    """fock::create_k (src/fock/jkbuilder.hpp:698-841)."""
    if method == "dfmo":
        return DFMO_K(engine)
    if method == "dflmo":
        return DFLMO_K(engine)
    if method in ("dfao", "dfmem"):
        # fock::DFMEM_K (src/fock/jkdf.cpp:650-859) forms the same exchange
        # as DFAO_K with the fit on the other factor:
        #   K = -sum_{X,s} (X|ns) [V^-1 (X|mr) P_rs]  =  -(B^T V^-1 B P)
        # so both names select the DF-AO builder
        return DFAO_K(engine)
    if method == "dfrobust":
        # fock::DFROBUST_K needs the PARI metric; with the Coulomb metric
        # the reference refuses it (src/fock/jkbuilder.hpp:598-603)
        raise RuntimeError("Cannot use robust k for method other than PARI")
    raise RuntimeError("Invalid kmethod")
