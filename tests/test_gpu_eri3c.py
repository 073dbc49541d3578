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


@pytest.mark.parametrize("kind,n,dfbasis", [("water", 0, "cc-pvdz-jkfit"),
                                            ("alkane", 4, "cc-pvdz-jkfit"),
                                            ("alkane", 2, "cc-pvdz-ri"),
                                            ("alkane", 10, "cc-pvdz-jkfit")])
def test_device_eri3c_matches_host(kind, n, dfbasis):
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.fock import JKEngine
    mol = _mol(kind, n, dfbasis)
    ds = build_dfsystem(mol, eps=1e-10)
    eng = JKEngine(ds.layout, ("device_ints", mol), np.tril(ds.Linv), ds.Vinv, eps=ds.eps)
    Bd = eng.download_b()
    scale = np.abs(ds.B).max()
    assert np.abs(Bd - ds.B).max() <= 1e-13 * scale
    assert np.array_equal(Bd == 0.0, ds.B == 0.0) or np.abs(Bd[ds.B == 0.0]).max() <= 1e-15 * scale
    # a Fock build on the device tensor matches the host-tensor one
    rng = np.random.default_rng(0)
    C = np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc]
    J1, K1 = eng.compute_jk(2 * C @ C.T, C)
    eng.close()
    e2 = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps)
    J2, K2 = e2.compute_jk(2 * C @ C.T, C)
    e2.close()
    # rounding-level tensor differences pass through V^-1 (cond ~1e6 here)
    assert np.abs(J1 - J2).max() <= 1e-8 and np.abs(K1 - K2).max() <= 1e-10
