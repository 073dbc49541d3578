"""megalochem's intermediate block filters (oracle/reffilter.py) against the
result-only filtering this engine applies.

At the configs' block threshold (1e-10) the intermediate filters of
fock::DF_J / fock::DFMO_K (P_tot, g, h, HT1, HT2 and K per batch;
src/fock/jkdf.cpp:100,124,137-141,166,364,387,419) change nothing that
matters: measured on n-C20H42 max|dK| 1.3e-13, max|dJ| 0, dE 2e-17 Eh; the
test below checks the same on decane.  At thresholds of 1e-8 and above they
do act (C20H42, 1e-8: max|dK| 7.5e-9, dE 2e-10 Eh against result-only
filtering)."""
import numpy as np

from oracle import reffilter


def _core(ds):
    sv, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(sv ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
    return np.ascontiguousarray((X @ Cp)[:, :ds.nocc])


def test_split_range_and_batch_bounds():
    assert reffilter.split_range(81, 10) == [10] * 8 + [1]
    assert reffilter.split_range(20, 10) == [10, 10]
    sizes = [14, 5, 5, 5, 14, 5, 5, 14, 5, 5, 5]
    b = reffilter.blk_bounds(sizes, 4)
    assert len(b) == 4 and b[0][0] == 0 and b[-1][1] == len(sizes) - 1
    assert all(b[i][1] + 1 == b[i + 1][0] for i in range(3))
    # a batch closes at the first block where the running size reaches
    # ibatch * total / nbatches
    per = sum(sizes) / 4
    for i, (f, l) in enumerate(b[:-1]):
        assert sum(sizes[:l + 1]) >= (i + 1) * per > sum(sizes[:l])
    assert reffilter.blk_bounds([5, 5], 4) == [(0, 0), (1, 1)]


def test_filters_off_match_dense(water):
    from oracle.oracle import dense_dfmo_k, dense_j
    ds = water
    C = _core(ds)
    P = C @ C.T
    T = ds.layout.to_dense(ds.B)
    J = reffilter.filtered_j(ds.layout, ds.B, ds.Vinv, 2 * P, 0.0)
    K = reffilter.filtered_dfmo_k(ds.layout, ds.B, ds.Linv, C, 0.0)
    assert np.abs(J - dense_j(T, ds.Vinv, 2 * P)).max() <= 1e-9
    assert np.abs(K - dense_dfmo_k(T, np.tril(ds.Linv), C)).max() <= 1e-12


def test_intermediate_filters_immaterial_at_config_threshold(decane):
    from oracle.oracle import Oracle
    ds = decane
    C = _core(ds)
    P = C @ C.T
    orc = Oracle(ds.layout, ds.B)
    J0 = reffilter.filtered_j(ds.layout, ds.B, ds.Vinv, 2 * P, 0.0)
    K0 = reffilter.filtered_dfmo_k(ds.layout, ds.B, ds.Linv, C, 0.0)
    eps = 1e-10
    Jr = reffilter.filtered_j(ds.layout, ds.B, ds.Vinv, 2 * P, eps)
    Kr = reffilter.filtered_dfmo_k(ds.layout, ds.B, ds.Linv, C, eps)
    Jf, Kf = orc.filter(J0, eps), orc.filter(K0, eps)  # this engine: results only
    assert np.abs(Jr - Jf).max() <= 1e-12
    assert np.abs(Kr - Kf).max() <= 1e-12
    assert abs(np.sum(P * ((Jr - Jf) + (Kr - Kf)))) <= 1e-12
    # at a coarse threshold the intermediate filters do act
    Kc = reffilter.filtered_dfmo_k(ds.layout, ds.B, ds.Linv, C, 1e-6)
    assert np.abs(Kc - orc.filter(K0, 1e-6)).max() > 1e-9
