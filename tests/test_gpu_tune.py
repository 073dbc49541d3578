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
    assert rep["best_ms"] == min(c["ms"] for c in rep["candidates"])
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
