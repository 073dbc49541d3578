"""3-center integrals on the device (gbjk_upload_b_eri3c) against the host
engine: same panels to rounding, screened blocks exactly zero, and the
J/K built on them agree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mol(kind, n, dfbasis):
    from chem_gb300 import geometry
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(n) if kind == "alkane" else geometry.water()
    return molecule_from_angstrom(s, x, "cc-pvdz", dfbasis)


def _screened_mask(lay):
    """Panel-layout mask of the entries of kept AO block pairs whose
    auxiliary block the Schwarz test screened out."""
    m = np.zeros(lay.nnz, bool)
    aoff = lay.aoff
    for p in range(lay.npairs):
        I, J = int(lay.pair_I[p]), int(lay.pair_J[p])
        for A in np.flatnonzero(lay.keep[p] == 0):
            for P, Q, col in ((I, J, lay.col_IJ[p]), (J, I, lay.col_JI[p])):
                bP, KP, bQ = int(lay.bsizes[P]), int(lay.panel_K[P]), int(lay.bsizes[Q])
                v = m[lay.panel_off[P]:lay.panel_off[P] + bP * lay.naux * KP].reshape(
                    bP, lay.naux, KP)
                v[:, aoff[A]:aoff[A + 1], col:col + bQ] = True
    return m


# (kind, n, auxiliary basis, Schwarz threshold).  At 1e-10 the Schwarz test
# drops whole AO block pairs only (the panels do not store them); the
# butane case at 0.1 also screens auxiliary blocks out of two kept AO pairs.
@pytest.mark.parametrize("kind,n,dfbasis,seps", [("water", 0, "cc-pvdz-jkfit", 1e-10),
                                                 ("alkane", 4, "cc-pvdz-jkfit", 1e-10),
                                                 ("alkane", 2, "cc-pvdz-ri", 1e-10),
                                                 ("alkane", 10, "cc-pvdz-jkfit", 1e-10),
                                                 ("alkane", 4, "cc-pvdz-jkfit", 0.1)])
def test_device_eri3c_matches_host(kind, n, dfbasis, seps):
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.fock import JKEngine
    mol = _mol(kind, n, dfbasis)
    ds = build_dfsystem(mol, eps=seps)
    eng = JKEngine(ds.layout, ("device_ints", mol), np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    Bd = eng.download_b()
    scale = np.abs(ds.B).max()
    assert np.abs(Bd - ds.B).max() <= 1e-13 * scale
    # entries of auxiliary blocks screened out for a kept AO block pair are
    # exactly zero on both
    screened = _screened_mask(ds.layout)
    assert screened.any() == (seps > 1e-3)
    assert not Bd[screened].any() and not ds.B[screened].any()
    # a Fock build on the device tensor matches the host-tensor one
    rng = np.random.default_rng(0)
    C = np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc]
    J1, K1 = eng.compute_jk(2 * C @ C.T, C)
    eng.close()
    e2 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    J2, K2 = e2.compute_jk(2 * C @ C.T, C)
    e2.close()
    # rounding-level tensor differences pass through V^-1 (cond ~1e6 here)
    assert np.abs(J1 - J2).max() <= 1e-8 and np.abs(K1 - K2).max() <= 1e-10
