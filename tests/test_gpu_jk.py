"""FP64 device path against the CPU oracle, through the C ABI.

The oracle and the kernels share one summation order per contraction, so
J and K must agree bit for bit (tolerance 0); the config-1 bar of 1e-12 max
abs is asserted as well.  Marked gpu: needs a GB300."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine, create_j, create_k, k_split_plan
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _orbitals(ds, seed=11):
    rng = np.random.default_rng(seed)
    return np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc]


def _engine(ds, eps=1e-10):
    return JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=eps)


@pytest.mark.parametrize("sysname", ["water", "butane", "decane"])
@pytest.mark.parametrize("kmethod", ["dfmo", "dflmo"])
def test_fp64_bitwise_vs_oracle(sysname, kmethod, request):
    ds = request.getfixturevalue(sysname)
    eng = _engine(ds)
    O = Oracle(ds.layout, ds.B)
    C = _orbitals(ds)
    P = C @ C.T
    J, K = eng.compute_jk(2 * P, C, kmethod)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nocc)[1]
    Jr = O.df_j(ds.Vinv, 2 * P, 1e-10)
    if kmethod == "dfmo":
        Kr = O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc)
    else:
        Kr = O.dflmo_k(ds.Vinv, C, 1e-10, kchunk=kc)
    assert np.abs(J - Jr).max() <= 1e-12
    assert np.abs(K - Kr).max() <= 1e-12
    assert np.array_equal(J, Jr)
    assert np.array_equal(K, Kr)
    if sysname == "decane":
        # screened block pairs exist and come back as exact zeros
        assert ds.layout.kept_block_fraction() < 1.0
        I, Jb = next((i, j) for i in range(ds.layout.nblk) for j in range(ds.layout.nblk)
                     if j not in ds.layout.nbr[i])
        bo = ds.layout.boff
        assert not J[bo[I]:bo[I + 1], bo[Jb]:bo[Jb + 1]].any()


def test_deterministic_and_builders(water):
    ds = water
    eng = _engine(ds)
    C = _orbitals(ds, 5)
    P = C @ C.T
    j = create_j(eng, "dfao")
    j.set_density_alpha(P)
    j.init()
    j.compute_J()
    k = create_k(eng, "dfmo")
    k.set_coeff_alpha(C)
    k.init()
    k.compute_K()
    J2, K2 = eng.compute_jk(2 * P, C)
    assert np.array_equal(j.get_J(), J2)
    assert np.array_equal(k.get_K_A(), K2)
    with pytest.raises(RuntimeError):
        create_k(eng, "nope")


def test_nocc_change_and_errors(butane):
    ds = butane
    eng = _engine(ds)
    O = Oracle(ds.layout, ds.B)
    for nocc in (3, ds.nocc, 1):
        C = _orbitals(ds)[:, :nocc]
        _, K = eng.compute_jk(None, C)
        kc = k_split_plan(ds.nbf, ds.naux, nocc)[1]
        assert np.array_equal(K, O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc))
    with pytest.raises(RuntimeError):
        eng.compute_jk(None, np.zeros((ds.nbf, 0)))


def test_empty_filter_eps_zero(water):
    ds = water
    eng = _engine(ds, eps=0.0)
    O = Oracle(ds.layout, ds.B)
    C = _orbitals(ds)
    J, K = eng.compute_jk(2 * C @ C.T, C)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nocc)[1]
    assert np.array_equal(J, O.df_j(ds.Vinv, 2 * C @ C.T, 0.0))
    assert np.array_equal(K, O.dfmo_k(np.tril(ds.Linv), C, 0.0, kchunk=kc))


@pytest.mark.parametrize("sysname", ["water", "butane", "decane"])
def test_fp64_cholesky_route_bitwise(sysname, request):
    ds = request.getfixturevalue(sysname)
    eng = _engine(ds)
    eng.set_jmode("cholesky")
    O = Oracle(ds.layout, ds.B)
    C = _orbitals(ds)
    P = C @ C.T
    J, _ = eng.compute_jk(2 * P, None)
    Jr = O.df_j_chol(np.tril(ds.Linv), 2 * P, 1e-10)
    assert np.array_equal(J, Jr)
    eng.close()


def test_fp64_bitwise_vs_oracle_c20h42():
    """The benchmark molecule itself (nbf 490, naux 2366, 66 % of block pairs
    kept): FP64 J and K bit for bit against the oracle."""
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(20)
    ds = build_dfsystem(molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit"), eps=1e-10)
    eng = _engine(ds)
    C = _orbitals(ds, 3)
    P = C @ C.T
    J, K = eng.compute_jk(2 * P, C, "dfmo")
    eng.close()
    O = Oracle(ds.layout, ds.B)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nocc)[1]
    assert np.array_equal(J, O.df_j(ds.Vinv, 2 * P, 1e-10))
    assert np.array_equal(K, O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc))


@pytest.mark.parametrize("sysname,ob", [("water", 3), ("butane", 8), ("decane", 16)])
@pytest.mark.parametrize("kmethod", ["dfmo", "dflmo"])
def test_fp64_occupied_batches_match_oracle(sysname, ob, kmethod, request):
    """FP64 K with the occupied orbitals in batches (megalochem's
    occ_nbatches): bit for bit the oracle's batched order, within rounding
    of the unbatched K."""
    from chem_gb300.fock import JKEngine, tune_plan
    from oracle.oracle import Oracle
    ds = request.getfixturevalue(sysname)
    rng = np.random.default_rng(12)
    C = np.ascontiguousarray(np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc])
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    _, K0 = eng.compute_jk(None, C, kmethod)
    eng.set_occ_batch(ob)
    _, K1 = eng.compute_jk(None, C, kmethod)
    eng.close()
    olast = ds.nocc - (-(-ds.nocc // ob) - 1) * ob
    kc_full = tune_plan(ds.nbf, ds.naux, ob)[0]["fp64_kchunk"]
    kc_last = tune_plan(ds.nbf, ds.naux, olast)[0]["fp64_kchunk"]
    M = np.tril(ds.Linv) if kmethod == "dfmo" else ds.Vinv
    Kr = Oracle(ds.layout, ds.B).dfk_occ_batched(M, C, ob, kc_full, kc_last, 1e-10,
                                                  lmo=kmethod == "dflmo")
    assert np.array_equal(K1, Kr), np.abs(K1 - Kr).max()
    assert np.abs(K1 - K0).max() <= 1e-12 * max(1.0, np.abs(K0).max())
