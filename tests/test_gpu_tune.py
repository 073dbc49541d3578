"""Autotuner on the GPU: every FP64 candidate stays bit-identical to the
oracle (which follows the published k parts of the exchange), the timed
search picks a configuration and records it, and a second engine adopts the
cached choice without timing."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _orbitals(ds, seed=3):
    rng = np.random.default_rng(seed)
    return np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc]


@pytest.mark.parametrize("sysname", ["water", "butane"])
def test_fp64_bitwise_for_every_candidate(sysname, request):
    ds = request.getfixturevalue(sysname)
    C = np.ascontiguousarray(_orbitals(ds))
    P = C @ C.T
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    orc = Oracle(ds.layout, ds.B)
    Jr = orc.df_j(ds.Vinv, 2 * P, 1e-10)
    eng.compute_jk(2 * P, C)
    base = eng.get_tunables()["fp64_kchunk"]
    checked = 0
    for tn in (1, 16, 32, 64):
        for kt in (1, 64):
            for kc in (max(16, base // 2), base, 2 * base):
                eng.set_tunables(fp64_ht_tn=tn, fp64_k_tile=kt, fp64_kchunk=kc)
                J, K = eng.compute_jk(2 * P, C)
                eff = eng.get_tunables()
                assert (eff["fp64_ht_tn"], eff["fp64_k_tile"]) == (tn, kt)
                Kr = orc.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=eff["fp64_kchunk"])
                assert np.array_equal(J, Jr), (tn, kt, kc)
                assert np.array_equal(K, Kr), (tn, kt, kc)
                checked += 1
    eng.close()
    assert checked == 24


@pytest.mark.parametrize("precision", ["split", "fp64"])
def test_autotune_and_cache(precision, butane, tmp_path):
    ds = butane
    C = np.ascontiguousarray(_orbitals(ds))
    P = C @ C.T
    cache = str(tmp_path / "tune.txt")
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=precision)
    rep = eng.autotune(2 * P, C, reps=2, cache=cache)
    assert rep["source"] == "timed" and len(rep["candidates"]) >= 4
    assert all(c["ms"] > 0 for c in rep["candidates"])
    # the choice is a measured candidate, replaced only by one at least
    # 0.5 % faster, so within that margin of the fastest
    fastest = min(c["ms"] for c in rep["candidates"])
    assert any(c["ms"] == rep["best_ms"] for c in rep["candidates"])
    assert fastest <= rep["best_ms"] <= fastest / (1 - 0.005) + 1e-12
    J1, K1 = eng.compute_jk(2 * P, C)
    chosen = rep["chosen"]
    eng.close()
    e2 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=precision)
    rep2 = e2.autotune(2 * P, C, reps=0, cache=cache)
    assert rep2["source"] == "cache" and rep2["chosen"] == chosen
    J2, K2 = e2.compute_jk(2 * P, C)
    e2.close()
    # same choice, same bits
    assert np.array_equal(J1, J2) and np.array_equal(K1, K2)
    # a signature not in the cache with reps = 0 is refused
    e3 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=precision)
    with pytest.raises(RuntimeError):
        e3.autotune(2 * P, C, kmethod="dflmo", reps=0, cache=cache)
    e3.close()


def test_split_overlap_modes_same_bits(decane):
    """The mixed build's J column sums on a second stream co-resident with
    the exchange (default, 0), beside an exchange that leaves 8 SMs, and in
    order on one stream (-1), through direct calls and a captured graph:
    the same bits every time."""
    import torch
    ds = decane
    C = np.ascontiguousarray(_orbitals(ds))
    P = C @ C.T
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    assert eng.get_overlap() == 0
    ref = None
    for mode in (0, -1, 8, 0):
        eng.set_overlap(mode)
        assert eng.get_overlap() == mode
        J, K = eng.compute_jk(2 * P, C)
        if ref is None:
            ref = (J, K)
        assert np.array_equal(J, ref[0]) and np.array_equal(K, ref[1]), mode
    dev = torch.device("cuda", 0)
    dP = torch.from_numpy(2 * P).to(dev)
    dC = torch.from_numpy(C).to(dev)
    dJ = torch.empty((ds.nbf, ds.nbf), dtype=torch.float64, device=dev)
    dK = torch.empty_like(dJ)
    for mode in (0, -1):
        eng.set_overlap(mode)
        eng.capture_graph(dP.data_ptr(), dC.data_ptr(), ds.nocc, dJ.data_ptr(), dK.data_ptr())
        eng.launch_graph()
        eng.launch_graph()
        eng.synchronize()
        assert np.array_equal(dJ.cpu().numpy(), ref[0]), mode
        assert np.array_equal(dK.cpu().numpy(), ref[1]), mode
    with pytest.raises(RuntimeError):
        eng.set_overlap(-2)
    eng.close()
