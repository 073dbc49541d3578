"""SOS-AO-MP2 Laplace batch on the GPU (gbjk_mp2_*): the FP64 path against
the CPU oracle bit for bit, the split-precision path against the FP64 path,
and the batch against single-point evaluations."""
import numpy as np
import pytest

from chem_gb300 import mp2

pytestmark = pytest.mark.gpu


def _system(n_carbon, seed, nlap=8):
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(n_carbon)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-ri")
    ds = build_dfsystem(mol, eps=1e-10)
    Co, Cv, eo, ev = mp2.random_orbitals(ds.S, ds.nocc, seed=seed)
    f = mp2.laplace_factors(Co, Cv, eo, ev, ds.S, nlap)
    return ds, f


@pytest.fixture(scope="module")
def ethane():
    return _system(2, 11)


@pytest.fixture(scope="module")
def decane():
    return _system(10, 12)


def _engine(ds, precision):
    from chem_gb300.fock import JKEngine
    return JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, precision=precision)


@pytest.mark.parametrize("sysname", ["ethane", "decane"])
def test_mp2_fp64_matches_oracle_bitwise(sysname, request):
    from oracle import oracle as O
    ds, f = request.getfixturevalue(sysname)
    eng = _engine(ds, "fp64")
    e, Z = eng.mp2_laplace(f.Lo, f.Lv, want_z=True)
    orc = O.Oracle(ds.layout, ds.B)
    Bf = orc.prefit(np.tril(ds.Linv))
    for t in range(len(f.Lo)):
        Zo, eo = orc.mp2_ll_point(Bf, f.Lo[t], f.Lv[t])
        assert np.array_equal(Z[t], Zo), (t, np.abs(Z[t] - Zo).max())
        assert e[t] == eo
    assert eng.kernel_launches > 0
    eng.close()


def test_mp2_split_matches_fp64(decane):
    ds, f = decane
    e64, Z64 = _engine(ds, "fp64").mp2_laplace(f.Lo, f.Lv, want_z=True)
    eng = _engine(ds, "split")
    es, Zs = eng.mp2_laplace(f.Lo, f.Lv, want_z=True)
    # three chained split products (39-bit digits, one exponent per operand
    # row): steep points, whose factors span many decades, lose most; the
    # Laplace sum stays far inside the 1e-8 Eh target
    for t in range(len(f.Lo)):
        assert np.abs(Zs[t] - Z64[t]).max() <= 1e-8 * np.abs(Z64[t]).max(), t
    assert np.all(np.abs(es - e64) <= 1e-8 * e64)
    assert abs(es.sum() - e64.sum()) < 1e-10
    # a second evaluation of the same factors is bitwise identical
    es2, Zs2 = eng.mp2_laplace(f.Lo, f.Lv, want_z=True)
    assert np.array_equal(es2, es) and np.array_equal(Zs2, Zs)
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_mp2_batch_equals_single_points(ethane, precision):
    ds, f = ethane
    eng = _engine(ds, precision)
    e_all, _ = eng.mp2_laplace(f.Lo, f.Lv)
    for t in (0, 3, 7):
        e1, _ = eng.mp2_laplace([f.Lo[t]], [f.Lv[t]])
        if precision == "fp64":
            assert e1[0] == e_all[t]
        else:  # the split-K partition of Z depends on the batch size
            assert abs(e1[0] - e_all[t]) <= 1e-12 * e_all[t]
    eng.close()


def test_mp2_rejects_bad_factors(ethane):
    ds, f = ethane
    eng = _engine(ds, "split")
    with pytest.raises(ValueError):
        eng.mp2_set_factors(f.Lo, f.Lv[:-1])
    with pytest.raises(ValueError):
        eng.mp2_set_factors([f.Lo[0][:-1]], [f.Lv[0]])
    with pytest.raises(RuntimeError):
        eng.mp2_compute_dev()  # nothing planned yet
    eng.close()
