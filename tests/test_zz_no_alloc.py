"""gbjk_compute_j_noalloc: DF-J for callers that cannot allocate device
memory (a host framework that owns all GPU memory through its own pool).
Compared, through the C ABI, with the context-based gbjk_compute_jk on two
calls in a row with different densities; both run the same kernels in the
same order, so the tolerance is 0 (bit for bit), as in the other FP64
parity tests.  The second call must leave the device's free memory
unchanged (it allocates nothing).

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case():
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(10)  # has Schwarz-screened block pairs
    return build_dfsystem(molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit"), eps=1e-10)


def test_noalloc_matches_context_path():
    import torch
    from chem_gb300 import fock
    from chem_gb300.fock import GbjkDesc, JKEngine

    ds = _case()
    L = fock.lib()
    f = L.gbjk_compute_j_noalloc
    f.argtypes = [C.POINTER(GbjkDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    lay = ds.layout
    bs = np.ascontiguousarray(lay.bsizes, np.int32)
    pk = np.ascontiguousarray(lay.panel_K, np.int32)
    cm = np.ascontiguousarray(np.concatenate(lay.column_map()), np.int32)
    desc = GbjkDesc(lay.nbf, lay.naux, lay.nblk, bs.ctypes.data_as(C.POINTER(C.c_int)),
                    pk.ctypes.data_as(C.POINTER(C.c_int)), None, 1e-10, 0)
    dev = torch.device("cuda", 0)
    d_cm = torch.from_numpy(cm).to(dev)
    d_B = torch.from_numpy(ds.B).to(dev)
    d_V = torch.from_numpy(np.ascontiguousarray(ds.Vinv)).to(dev)
    d_J = torch.empty((lay.nbf, lay.nbf), dtype=torch.float64, device=dev)
    eng = JKEngine(lay, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    rng = np.random.default_rng(2024)
    for call in range(2):
        Cm = np.linalg.qr(rng.standard_normal((lay.nbf, lay.nbf)))[0][:, :ds.nocc]
        Ptot = np.ascontiguousarray(2.0 * Cm @ Cm.T)
        d_P = torch.from_numpy(Ptot).to(dev)
        d_J.fill_(float("nan"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(dev)[0]
        err = C.create_string_buffer(256)
        rc = f(C.byref(desc), d_cm.data_ptr(), d_B.data_ptr(), d_V.data_ptr(), d_P.data_ptr(),
               d_J.data_ptr(), None, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        if call == 1:  # after the first call's one-time set-up: no device memory taken
            assert torch.cuda.mem_get_info(dev)[0] == free0
        J_ref, _ = eng.compute_jk(Ptot, None)
        J = d_J.cpu().numpy()
        assert np.array_equal(J, J_ref), f"call {call}: max diff {np.abs(J - J_ref).max()}"
    # a problem whose scratch exceeds the 16 MiB array is rejected on the
    # host before any launch (nbf*naux alone is 24 MB here)
    bs_big = np.array([3000], np.int32)
    pk_big = np.array([3000], np.int32)
    big = GbjkDesc(3000, 1000, 1, bs_big.ctypes.data_as(C.POINTER(C.c_int)),
                   pk_big.ctypes.data_as(C.POINTER(C.c_int)), None, 0.0, 0)
    err = C.create_string_buffer(256)
    rc = f(C.byref(big), d_cm.data_ptr(), d_B.data_ptr(), d_V.data_ptr(), d_P.data_ptr(),
           d_J.data_ptr(), None, err, 256)
    assert rc == 1 and b"limit" in err.value
    # grids with nbf rows beyond the launch limit are rejected the same way
    bs_wide = np.array([70000], np.int32)
    pk_wide = np.array([0], np.int32)
    wide = GbjkDesc(70000, 8, 1, bs_wide.ctypes.data_as(C.POINTER(C.c_int)),
                    pk_wide.ctypes.data_as(C.POINTER(C.c_int)), None, 0.0, 0)
    rc = f(C.byref(wide), d_cm.data_ptr(), d_B.data_ptr(), d_V.data_ptr(), d_P.data_ptr(),
           d_J.data_ptr(), None, err, 256)
    assert rc == 1 and b"65535" in err.value
    eng.close()


def test_noalloc_call_captured_in_a_graph():
    """A captured call holds only launches and memsets (the per-block layout
    travels as a by-value kernel argument): replaying the graph after a new
    density is copied into the same buffer gives the context path's J for
    that density, bit for bit."""
    import torch
    from chem_gb300 import fock
    from chem_gb300.fock import GbjkDesc, JKEngine

    ds = _case()
    L = fock.lib()
    f = L.gbjk_compute_j_noalloc
    f.argtypes = [C.POINTER(GbjkDesc), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    lay = ds.layout
    bs = np.ascontiguousarray(lay.bsizes, np.int32)
    pk = np.ascontiguousarray(lay.panel_K, np.int32)
    cm = np.ascontiguousarray(np.concatenate(lay.column_map()), np.int32)
    desc = GbjkDesc(lay.nbf, lay.naux, lay.nblk, bs.ctypes.data_as(C.POINTER(C.c_int)),
                    pk.ctypes.data_as(C.POINTER(C.c_int)), None, 1e-10, 0)
    dev = torch.device("cuda", 0)
    d_cm = torch.from_numpy(cm).to(dev)
    d_B = torch.from_numpy(ds.B).to(dev)
    d_V = torch.from_numpy(np.ascontiguousarray(ds.Vinv)).to(dev)
    d_J = torch.empty((lay.nbf, lay.nbf), dtype=torch.float64, device=dev)
    d_P = torch.empty((lay.nbf, lay.nbf), dtype=torch.float64, device=dev)
    eng = JKEngine(lay, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    rng = np.random.default_rng(7)

    def density():
        Cm = np.linalg.qr(rng.standard_normal((lay.nbf, lay.nbf)))[0][:, :ds.nocc]
        return np.ascontiguousarray(2.0 * Cm @ Cm.T)

    err = C.create_string_buffer(256)
    P0 = density()
    d_P.copy_(torch.from_numpy(P0))
    side = torch.cuda.Stream(dev)
    # a direct call first (the one-time address look-up happens outside capture)
    with torch.cuda.stream(side):
        rc = f(C.byref(desc), d_cm.data_ptr(), d_B.data_ptr(), d_V.data_ptr(), d_P.data_ptr(),
               d_J.data_ptr(), C.c_void_p(side.cuda_stream), err, 256)
    assert rc == 0, err.value.decode()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        rc = f(C.byref(desc), d_cm.data_ptr(), d_B.data_ptr(), d_V.data_ptr(), d_P.data_ptr(),
               d_J.data_ptr(), C.c_void_p(side.cuda_stream), err, 256)
    assert rc == 0, err.value.decode()
    for _ in range(2):
        Pn = density()
        d_P.copy_(torch.from_numpy(Pn))
        d_J.fill_(float("nan"))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        J_ref, _ = eng.compute_jk(Pn, None)
        assert np.array_equal(d_J.cpu().numpy(), J_ref)
    eng.close()
