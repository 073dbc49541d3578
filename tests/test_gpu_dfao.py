"""DF-AO exchange on the GPU (gbjk_compute_k_ao): the FP64 path (fitting
coefficients V^-1 (X|mn), the reference route) against the CPU oracle bit
for bit; both paths against DF-MO K of the same density (P = C C^T gives the
same K); the builder interface (create_k("dfao"))."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _density(ds, seed=3):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((ds.nbf, ds.nbf))
    s, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(s ** -0.5) @ U.T
    _, V = np.linalg.eigh(X.T @ (ds.Hcore + 0.01 * (M + M.T)) @ X)
    C = np.ascontiguousarray((X @ V)[:, :ds.nocc])
    return C, C @ C.T


def _engine(ds, precision):
    from chem_gb300.fock import JKEngine
    return JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=0.0, precision=precision)


@pytest.mark.parametrize("sysname", ["water", "decane"])
def test_dfao_fp64_matches_oracle_bitwise(sysname, request):
    from chem_gb300.fock import k_split_plan
    from oracle.oracle import Oracle
    ds = request.getfixturevalue(sysname)
    _, P = _density(ds)
    eng = _engine(ds, "fp64")
    K = eng.compute_k_ao(P)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nbf)[1]
    Kr = Oracle(ds.layout, ds.B).dfao_k(ds.Vinv, P, 0.0, kchunk=kc)
    assert np.array_equal(K, Kr), np.abs(K - Kr).max()
    eng.close()


@pytest.mark.parametrize("sysname", ["water", "decane"])
def test_dfao_matches_dfmo(sysname, request):
    ds = request.getfixturevalue(sysname)
    C, P = _density(ds)
    e64 = _engine(ds, "fp64")
    _, Kmo = e64.compute_jk(Cocc=C)
    Kao = e64.compute_k_ao(P)
    e64.close()
    assert np.abs(Kao - Kmo).max() <= 1e-9 * max(1.0, np.abs(Kmo).max())
    es = _engine(ds, "split")
    Ks = es.compute_k_ao(P)
    assert np.abs(Ks - Ks.T).max() == 0.0
    assert np.abs(Ks - Kmo).max() <= 1e-9 * max(1.0, np.abs(Kmo).max())
    es.close()


def test_dfao_builder_interface(water):
    from chem_gb300.fock import create_k
    ds = water
    C, P = _density(ds)
    eng = _engine(ds, "split")
    k = create_k(eng, "dfao")
    k.init()
    k.set_density_alpha(P)
    k.compute_K()
    _, Kmo = eng.compute_jk(Cocc=C)
    assert np.abs(k.get_K_A() - Kmo).max() <= 1e-9
    assert k.get_K_B() is None
    eng.close()


@pytest.mark.parametrize("sysname", ["water", "decane"])
def test_dflmo_asym_fp64_bitwise_and_split(sysname, request):
    """Non-symmetric DF-LMO K (ADC-style left/right coefficients)."""
    from chem_gb300.fock import k_split_plan
    from oracle.oracle import Oracle
    ds = request.getfixturevalue(sysname)
    rng = np.random.default_rng(9)
    C, _ = _density(ds)
    U = C + 0.1 * rng.standard_normal(C.shape)
    Vt = (C + 0.1 * rng.standard_normal(C.shape)).T.copy()
    e64 = _engine(ds, "fp64")
    K64 = e64.compute_k_lmo_asym(U, Vt)
    e64.close()
    kc = k_split_plan(ds.nbf, ds.naux, U.shape[1])[1]
    Kr = Oracle(ds.layout, ds.B).dflmo_k_asym(ds.Vinv, U, Vt, 0.0, kchunk=kc)
    assert np.array_equal(K64, Kr), np.abs(K64 - Kr).max()
    es = _engine(ds, "split")
    Ks = es.compute_k_lmo_asym(U, Vt)
    es.close()
    assert np.abs(Ks - K64).max() <= 1e-9 * max(1.0, np.abs(K64).max())
    assert np.abs(K64 - K64.T).max() > 1e-6  # genuinely non-symmetric


def test_dflmo_builder_nonsymmetric(water):
    from chem_gb300.fock import create_k
    ds = water
    C, _ = _density(ds)
    eng = _engine(ds, "split")
    k = create_k(eng, "dflmo")
    k.init()
    k.set_sym(False)
    k.set_coeff_left_alpha(C)
    k.set_coeff_right_alpha(C.T)
    k.compute_K()
    _, Kmo = eng.compute_jk(Cocc=C)
    assert np.abs(k.get_K_A() - Kmo).max() <= 1e-9
    eng.close()
