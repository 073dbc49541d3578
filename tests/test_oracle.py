"""CPU oracle (oracle/dfjk_oracle.c) against an independent dense einsum of
the reference's formulas, physics identities, and the filter semantics."""
import numpy as np
import pytest

from oracle.oracle import Oracle, dense_dfao_k, dense_dflmo_k, dense_dfmo_k, dense_j


def _orbitals(ds, seed=3):
    rng = np.random.default_rng(seed)
    Q = np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0]
    return Q[:, :ds.nocc]


@pytest.mark.parametrize("sysname", ["water", "butane"])
def test_oracle_vs_dense(sysname, request):
    ds = request.getfixturevalue(sysname)
    T = ds.layout.to_dense(ds.B)
    O = Oracle(ds.layout, ds.B)
    C = _orbitals(ds)
    P = C @ C.T
    # different summation orders: agreement to ~1e-11 relative (the metric
    # inverse amplifies rounding in g by its condition number)
    J = O.df_j(ds.Vinv, 2 * P)
    assert np.abs(J - dense_j(T, ds.Vinv, 2 * P)).max() < 1e-9 * np.abs(J).max()
    K = O.dfmo_k(ds.Linv, C)
    assert np.abs(K - dense_dfmo_k(T, ds.Linv, C)).max() < 1e-11 * np.abs(K).max()
    K2 = O.dflmo_k(ds.Vinv, C)
    assert np.abs(K2 - dense_dflmo_k(T, ds.Vinv, C)).max() < 1e-9 * np.abs(K).max()
    # chunked exchange sums (the device's plan) agree to rounding
    K4 = O.dfmo_k(ds.Linv, C, kchunk=96)
    assert np.abs(K4 - K).max() < 1e-13 * np.abs(K).max()
    if sysname == "water":
        K3 = O.dfao_k(ds.Vinv, P)
        assert np.abs(K3 - dense_dfao_k(T, ds.Vinv, P)).max() < 1e-11
        assert np.abs(K3 - K).max() < 1e-9


def test_identities(water):
    ds = water
    O = Oracle(ds.layout, ds.B)
    C = _orbitals(ds)
    P = C @ C.T
    J = O.df_j(ds.Vinv, 2 * P)
    K = O.dfmo_k(ds.Linv, C)
    # J, K symmetric; K negative semidefinite
    assert np.abs(J - J.T).max() < 1e-13
    assert np.abs(K - K.T).max() < 1e-13
    assert np.linalg.eigvalsh(K).max() < 1e-10
    # tr(P J) = g^T V^-1 g with g = B : P_tot
    T = ds.layout.to_dense(ds.B)
    g = np.einsum("xmn,mn->x", T, 2 * P)
    assert abs(np.sum(2 * P * J) - g @ ds.Vinv @ g) < 1e-9 * abs(g @ ds.Vinv @ g)
    # DF-MO and DF-LMO agree (L^-T L^-1 = V^-1)
    assert np.abs(K - O.dflmo_k(ds.Vinv, C)).max() < 1e-9


def test_filter_drops_small_blocks(butane):
    ds = butane
    O = Oracle(ds.layout, ds.B)
    M = np.ones((ds.nbf, ds.nbf))
    bo = ds.layout.boff
    M[bo[0]:bo[1], bo[2]:bo[3]] = 1e-9
    F = O.filter(M, 1e-6)
    assert np.all(F[bo[0]:bo[1], bo[2]:bo[3]] == 0)
    assert np.all(F[bo[1]:bo[2], :] == 1)


def test_layout_screening(butane):
    L = butane.layout
    assert L.to_dense(butane.B).shape == (L.naux, L.nbf, L.nbf)
    # kept pattern symmetric, diagonal blocks always kept
    for I in range(L.nblk):
        assert I in L.nbr[I]
        for J in L.nbr[I]:
            assert I in L.nbr[J]
    assert L.nnz == sum(int(L.bsizes[I]) * L.naux * int(L.panel_K[I]) for I in range(L.nblk))


def test_dflmo_asym_oracle_matches_dense(water):
    import numpy as np
    from oracle.oracle import Oracle, dense_dflmo_k_asym
    ds = water
    rng = np.random.default_rng(5)
    U = rng.standard_normal((ds.nbf, 4))
    Vt = rng.standard_normal((4, ds.nbf))
    T = ds.layout.to_dense(ds.B)
    K = Oracle(ds.layout, ds.B).dflmo_k_asym(ds.Vinv, U, Vt)
    Kd = dense_dflmo_k_asym(T, ds.Vinv, U, Vt)
    assert np.abs(K - Kd).max() < 1e-11 * np.abs(Kd).max()
    # U = V gives the symmetric branch's K (which is stored as K_nm, so its
    # transpose matches operation for operation)
    Ks = Oracle(ds.layout, ds.B).dflmo_k(ds.Vinv, U)
    Ka = Oracle(ds.layout, ds.B).dflmo_k_asym(ds.Vinv, U, U.T)
    assert np.array_equal(Ks.T, Ka)
