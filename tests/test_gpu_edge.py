"""Edge cases of the device paths: one occupied orbital, a fully screened
block pair (ragged panels), odd strides, and repeated calls with changing
nocc — FP64 against the oracle bit for bit, split against FP64."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine, k_split_plan
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def h2_far():
    """Two H2 molecules 40 Angstrom apart: nocc 2, AO block pairs across the
    gap are screened out, so panels are ragged (K_I = 10 of 20)."""
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    xyz = np.array([[0, 0, 0], [0, 0, 0.74], [40, 0, 0], [40, 0, 0.74]], float)
    mol = molecule_from_angstrom(["H", "H", "H", "H"], xyz, "cc-pvdz", "cc-pvdz-jkfit")
    return build_dfsystem(mol, eps=1e-10)


def test_ragged_panels_and_single_orbital(h2_far):
    ds = h2_far
    assert ds.layout.kept_block_fraction() < 1.0
    O = Oracle(ds.layout, ds.B)
    rng = np.random.default_rng(1)
    for nocc in (1, 2, 1):  # nocc changes between calls: plans are rebuilt
        C = np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :nocc]
        P = C @ C.T
        e64 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
        J, K = e64.compute_jk(2 * P, C)
        kc = k_split_plan(ds.nbf, ds.naux, nocc)[1]
        assert np.array_equal(J, O.df_j(ds.Vinv, 2 * P, 1e-10))
        assert np.array_equal(K, O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc))
        e64.set_jmode("cholesky")
        Jc, _ = e64.compute_jk(2 * P, None)
        e64.close()
        es = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
        Js, Ks = es.compute_jk(2 * P, C)
        es.close()
        assert np.abs(Ks - K).max() <= 1e-10
        # the mixed J follows the Cholesky route of the metric; against the
        # V^-1 route it may differ by that route's own rounding as well
        assert np.abs(Js - Jc).max() <= 1e-9
        assert np.abs(Js - J).max() <= np.abs(Jc - J).max() + 1e-9
        # J of a screened block pair is an exact zero in both paths (K is
        # not: delocalised orbitals couple the two molecules)
        bo = ds.layout.boff
        assert not J[bo[0]:bo[1], bo[2]:bo[3]].any() and not Js[bo[0]:bo[1], bo[2]:bo[3]].any()
        assert np.abs(K[bo[0]:bo[1], bo[2]:bo[3]]).max() > 1e-6


def test_engine_reuse_across_nocc(water):
    ds = water
    es = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    rng = np.random.default_rng(2)
    for nocc in (5, 3, 5, 7):
        C = np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :nocc]
        _, K1 = es.compute_jk(None, C)
        _, K2 = es.compute_jk(None, C)
        assert np.array_equal(K1, K2)  # deterministic after re-planning
        e64 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
        _, K64 = e64.compute_jk(None, C)
        e64.close()
        assert np.abs(K1 - K64).max() <= 1e-10
    es.close()
