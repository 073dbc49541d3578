"""SOS-AO-MP2 Laplace term on the CPU: the minimax restatement against the
published error table, the pivoted Cholesky decomposition, and the MP2 oracle
against two independent dense restatements (megalochem's ll_full and default
llmp_full Z builders) and against the exact SOS sum it approximates."""
import json
import os

import numpy as np
import pytest

from chem_gb300 import laplace, mp2

HERE = os.path.dirname(os.path.abspath(__file__))


def _table():
    return json.load(open(os.path.join(HERE, "golden", "minimax_errors.json")))["entries"]


@pytest.mark.parametrize("k", [8])
def test_minimax_k8_matches_published_errors(k):
    # every tabulated interval for the quadrature size of the MP2 workload
    rows = [e for e in _table() if e["k"] == k]
    assert len(rows) >= 20
    for e in rows:
        _, _, err = laplace.minimax_unit(e["k"], e["R"])
        assert abs(err - e["err"]) / e["err"] < 2e-3, (e, err)


def test_minimax_other_sizes_match_published_errors():
    rows = [e for e in _table() if e["R"] in (100, 1000) and e["k"] != 8]
    assert len(rows) >= 8
    for e in rows:
        _, _, err = laplace.minimax_unit(e["k"], e["R"])
        assert abs(err - e["err"]) / e["err"] < 2e-3, (e, err)


def test_laplace_points_equioscillate_on_the_interval():
    ymin, ymax = 0.8, 140.0
    a, w, err = laplace.laplace_points(8, ymin, ymax)
    assert np.all(a > 0) and np.all(w > 0) and np.all(np.diff(a) > 0)
    y = np.exp(np.linspace(np.log(ymin), np.log(ymax), 200001))
    dev = np.exp(-np.outer(y, a)) @ w - 1.0 / y
    assert np.max(np.abs(dev)) <= err * (1 + 1e-6)
    assert np.max(np.abs(dev)) >= err * (1 - 1e-6)
    # alternation: 2k+1 = 17 sign-alternating extrema of size err
    big = np.abs(dev) > 0.999 * err
    signs = np.sign(dev[big])
    assert 1 + np.count_nonzero(np.diff(signs) != 0) == 17


def test_laplace_rejects_bad_interval():
    with pytest.raises(ValueError):
        laplace.laplace_points(8, 1.0, 0.5)
    with pytest.raises(ValueError):
        laplace.minimax_unit(0, 10.0)


def test_pivoted_cholesky_rank_and_reconstruction():
    rng = np.random.default_rng(3)
    G = rng.standard_normal((20, 7))
    A = G @ G.T
    L = mp2.pivoted_cholesky(A)
    assert L.shape == (20, 7)
    assert np.abs(L @ L.T - A).max() < 1e-12 * np.abs(A).max()
    Lr = mp2.pivoted_cholesky(A, reorder_eps=1e-10)
    assert np.abs(Lr @ Lr.T - A).max() < 1e-12 * np.abs(A).max()
    assert mp2.pivoted_cholesky(A, max_rank=3).shape == (20, 3)
    with pytest.raises(ValueError):
        mp2.pivoted_cholesky(-A)


def test_random_orbitals_are_orthonormal():
    rng = np.random.default_rng(0)
    M = rng.standard_normal((12, 12))
    S = M @ M.T + 12 * np.eye(12)
    Co, Cv, eo, ev = mp2.random_orbitals(S, 4, seed=5)
    Cm = np.hstack([Co, Cv])
    assert np.abs(Cm.T @ S @ Cm - np.eye(12)).max() < 1e-12
    assert eo.shape == (4,) and ev.shape == (8,)
    assert np.all(np.diff(eo) >= 0) and eo.min() >= -20 and eo.max() <= -0.3
    assert np.all(np.diff(ev) >= 0) and ev.min() >= 0.1 and ev.max() <= 50


@pytest.fixture(scope="module")
def ethane_ri():
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(2)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-ri")
    ds = build_dfsystem(mol, eps=1e-10)
    Co, Cv, eo, ev = mp2.random_orbitals(ds.S, ds.nocc, seed=11)
    f = mp2.laplace_factors(Co, Cv, eo, ev, ds.S, 8, keep_densities=True)
    return ds, (Co, Cv, eo, ev), f


def test_pseudo_density_factors(ethane_ri):
    ds, _, f = ethane_ri
    for t in range(8):
        assert np.abs(f.Lo[t] @ f.Lo[t].T - f.Po[t]).max() < 1e-11 * np.abs(f.Po[t]).max()
        assert np.abs(f.Lv[t] @ f.Lv[t].T - f.Pv[t]).max() < 1e-11 * np.abs(f.Pv[t]).max()
        assert f.Lo[t].shape[1] == ds.nocc


def test_mp2_oracle_matches_dense_routes(ethane_ri):
    from oracle import oracle as O
    ds, (Co, Cv, eo, ev), f = ethane_ri
    T = ds.layout.to_dense(ds.B)
    orc = O.Oracle(ds.layout, ds.B)
    Bf = orc.prefit(np.tril(ds.Linv))
    # screened shell-pair pattern of the tensor (the retained sparsity of
    # the llmp_full builder's third transform)
    pm = np.zeros((ds.nbf, ds.nbf))
    for I, cols in enumerate(ds.layout.column_map()):
        pm[ds.layout.boff[I]:ds.layout.boff[I + 1], cols] = 1
    Linv = np.tril(ds.Linv)
    tot = 0.0
    for t in range(8):
        Zll, ell = O.dense_mp2_ll(T, ds.Vinv, f.Lo[t], f.Lv[t])
        _, emp = O.dense_mp2_llmp(T, ds.Vinv, f.Lo[t], f.Pv[t], pm)
        Zo, eo_t = orc.mp2_ll_point(Bf, f.Lo[t], f.Lv[t])
        assert abs(emp - ell) <= 1e-10 * ell
        assert abs(eo_t - ell) <= 1e-10 * ell
        # the oracle's Z is the fitted L^-1 Z L^-T
        Zf = Linv @ Zll @ Linv.T
        assert np.abs(Zo - Zf).max() <= 1e-10 * np.abs(Zf).max()
        tot += eo_t
    exact = O.dense_sos_mp2(T, ds.Vinv, Co, Cv, eo, ev)
    # the Laplace sum approximates sum (ia|jb)^2 / D to the minimax error
    assert abs(tot - exact) / exact < 1e-6


def test_mp2_oracle_aux_subset_is_a_prefix(ethane_ri):
    # nx restricts to the first nx auxiliary functions (the CPU timing sample)
    from oracle import oracle as O
    ds, _, f = ethane_ri
    orc = O.Oracle(ds.layout, ds.B)
    Bf = orc.prefit(np.tril(ds.Linv))
    Bs = orc.prefit(np.tril(ds.Linv), nx=40)
    Z, _ = orc.mp2_ll_point(Bf, f.Lo[0], f.Lv[0])
    Zs, es = orc.mp2_ll_point(Bs, f.Lo[0], f.Lv[0], nx=40)
    assert np.array_equal(Zs, Z[:40, :40])
    assert es == pytest.approx(float(np.sum(Zs * Zs)), rel=1e-13)
