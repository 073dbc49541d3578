"""Which FP64 route of DF-J's metric step is right.

fock::DF_J multiplies g by the explicit inverse V^-1 = L^-T L^-1
(src/fock/jkdf.cpp:137-141, src/ints/aoloader.cpp:14-32); the engine's
Cholesky route applies L^-1 and then L^-T.  Both are compared with the
solution of V h = g that is exact for the same FP64 V and g (iterative
refinement with correctly rounded residuals, chem_gb300.accuracy), at a
core-guess density.  The oracle restates each device route operation for
operation (the device equals it bit for bit), so its J is the device's J.

Measured here: butane (cond V 6.7e6) V^-1 route -8.0e-8 Eh, Cholesky route
-5e-13 Eh; decane (cond V 1.6e7) 3.0e-7 Eh against 2.3e-11 Eh.  The
explicit inverse therefore carries an FP64 error 60x above the 1e-8 Eh
accuracy target on its own, while the Cholesky route is exact to ~1e-11 Eh.
"""
import numpy as np
import pytest


def _core_density(ds):
    sv, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(sv ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
    C = (X @ Cp)[:, :ds.nocc]
    return C @ C.T


def test_refined_solve_is_exact():
    """The refinement reaches a residual far below FP64 resolution and is
    independent of the starting solve (a 1e-6 perturbed start converges to
    the same energy)."""
    from chem_gb300 import accuracy
    rng = np.random.default_rng(3)
    n = 60
    Q = np.linalg.qr(rng.standard_normal((n, n)))[0]
    V = Q @ np.diag(np.logspace(0, -7, n)) @ Q.T  # cond 1e7, SPD
    V = 0.5 * (V + V.T)
    g = rng.standard_normal(n)
    parts, res = accuracy.refined_solve(V, g)
    assert res < 1e-25
    e1 = accuracy.exact_dot(g, parts)
    parts2 = [parts[0] * (1 + 1e-6)]
    for _ in range(4):
        r = accuracy.exact_residual(V, g, parts2)
        parts2.append(np.linalg.solve(V, r))
    e2 = accuracy.exact_dot(g, parts2)
    assert abs(e1 - e2) <= 1e-12 * abs(e1)


@pytest.mark.parametrize("fixture,vinv_min", [("butane", 2e-8), ("decane", 1e-7)])
def test_cholesky_route_is_exact_vinv_route_is_not(fixture, vinv_min, request):
    from chem_gb300 import accuracy
    from oracle.oracle import Oracle
    ds = request.getfixturevalue(fixture)
    P = _core_density(ds)
    g = accuracy.panel_g(ds.layout, ds.B, 2.0 * P)
    r = accuracy.coulomb_routes(ds.V, ds.Linv, ds.Vinv, g)
    assert r["residual_max"] < 1e-20
    orc = Oracle(ds.layout, ds.B)
    J_vinv = orc.df_j(ds.Vinv, 2.0 * P, 0.0)            # the device's reference route
    J_chol = orc.df_j_chol(np.tril(ds.Linv), 2.0 * P, 0.0)  # the device's Cholesky route
    J_exact = accuracy.panel_j(ds.layout, ds.B, r["h_exact"])
    dE_vinv = accuracy.j_energy_vs_exact(P, J_vinv, r["E_exact"])
    dE_chol = accuracy.j_energy_vs_exact(P, J_chol, r["E_exact"])
    # the Cholesky route is exact to ~1e-11 Eh; the explicit inverse is not
    assert abs(dE_chol) <= 1e-10
    assert abs(dE_vinv) >= vinv_min
    assert abs(dE_vinv) >= 100 * abs(dE_chol)
    dj_chol = np.abs(J_chol - J_exact).max()
    dj_vinv = np.abs(J_vinv - J_exact).max()
    assert dj_chol <= 1e-10 and dj_vinv >= 10 * dj_chol


@pytest.mark.skipif(not __import__("chem_gb300.accuracy", fromlist=["x"]).have_quad(),
                    reason="numpy longdouble is not IEEE quadruple precision here")
def test_quad_residual_matches_exact_sums():
    """Where numpy's longdouble is IEEE quad (aarch64), the faster quad
    residuals give the same refined energy as the exactly summed ones."""
    from chem_gb300 import accuracy
    rng = np.random.default_rng(5)
    n = 80
    Q = np.linalg.qr(rng.standard_normal((n, n)))[0]
    V = Q @ np.diag(np.logspace(0, -7, n)) @ Q.T
    V = 0.5 * (V + V.T)
    g = rng.standard_normal(n)
    pe, _ = accuracy.refined_solve(V, g)
    pq, res = accuracy.refined_solve(V, g, residual="quad")
    assert res < 1e-25
    e1, e2 = accuracy.exact_dot(g, pe), accuracy.exact_dot(g, pq)
    assert abs(e1 - e2) <= 1e-14 * abs(e1)
