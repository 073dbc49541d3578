"""Split-precision (BF16 digit slices on tcgen05 tensor cores) K path against
the FP64 oracle.  Tolerances are the configs' bars: max|dK| <= 1e-9 and, for
SCF energies, |dE| <= 1e-8 Eh against the FP64 path.  In the mixed mode
J's density contraction also runs on the tensor cores (max|dJ| <= 1e-9);
a J-only call takes the FP64 path."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine, k_split_plan
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _core_orbitals(ds):
    s, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(s ** -0.5) @ U.T
    e, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
    return np.ascontiguousarray((X @ Cp)[:, :ds.nocc])


@pytest.mark.parametrize("sysname", ["water", "butane", "decane"])
def test_split_k_vs_oracle(sysname, request):
    ds = request.getfixturevalue(sysname)
    C = _core_orbitals(ds)
    P = C @ C.T
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    J, K = eng.compute_jk(2 * P, C, "dfmo")
    O = Oracle(ds.layout, ds.B)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nocc)[1]
    Kr = O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc)
    Jr = O.df_j(ds.Vinv, 2 * P, 1e-10)
    dK = np.abs(K - Kr).max()
    print(f"{sysname}: max|dK| = {dK:.3e}  max|K| = {np.abs(Kr).max():.3f}")
    # mixed-mode J: density contracted on the tensor cores against L^-1 B,
    # then one FP64 pass over L^-1 B (no V^-1 in the path).  Its split error
    # is measured against the same Cholesky-route formula in FP64; the
    # V^-1-route FP64 J carries its own ~1e-9 rounding noise (cond(V) ~ 1e7)
    T = ds.layout.to_dense(ds.B)
    Bt = np.einsum("yx,xmn->ymn", np.tril(ds.Linv), T)
    Jc = np.einsum("y,ymn->mn", np.einsum("ymn,mn->y", Bt, 2 * P), Bt)
    dJ = np.abs(J - Jc).max()
    print(f"{sysname}: max|dJ| = {dJ:.3e} (Cholesky route), "
          f"{np.abs(J - Jr).max():.3e} (V^-1 route)  max|J| = {np.abs(Jr).max():.3f}")
    assert dK <= 1e-9
    assert dJ <= 1e-9
    # against the V^-1 route: no farther than that route's own rounding
    # noise (|Jc - Jr|, ~1e-8 for decane) plus the split error
    assert np.abs(J - Jr).max() <= np.abs(Jc - Jr).max() + 1e-9
    # and against the device FP64 path on the Cholesky route
    eng.set_precision("fp64")
    eng.set_jmode("cholesky")
    J64c, _ = eng.compute_jk(2 * P, None)
    assert np.abs(J - J64c).max() <= 1e-9
    eng.set_jmode("vinv")
    eng.set_precision("split")
    # J alone (no coefficients) takes the FP64 path: identical to the oracle
    Jalone, _ = eng.compute_jk(2 * P, None)
    assert np.array_equal(Jalone, Jr)
    # repeated builds are deterministic
    _, K2 = eng.compute_jk(None, C, "dfmo")
    assert np.array_equal(K, K2)
    eng.close()


@pytest.mark.parametrize("sysname", ["butane", "decane"])
def test_split_fuse_modes(sysname, request):
    """Both digit cuts of the half transform H: from an FP64 H with one
    exponent per AO function (default), and in the half-transform epilogue
    with one exponent per (AO function, 32 auxiliary indices) and a
    segmented exchange.  Each is within the K bar of the oracle; the density
    partials of J come from the same integers, so J is the same bits."""
    ds = request.getfixturevalue(sysname)
    C = _core_orbitals(ds)
    P = C @ C.T
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    assert not eng.get_split_fuse()
    J0, K0 = eng.compute_jk(2 * P, C, "dfmo")
    eng.set_split_fuse(True)
    assert eng.get_split_fuse()
    J1, K1 = eng.compute_jk(2 * P, C, "dfmo")
    eng.set_split_fuse(False)
    eng.set_split_fuse(True)
    J2, K2 = eng.compute_jk(2 * P, C, "dfmo")
    eng.close()
    O = Oracle(ds.layout, ds.B)
    kc = k_split_plan(ds.nbf, ds.naux, ds.nocc)[1]
    Kr = O.dfmo_k(np.tril(ds.Linv), C, 1e-10, kchunk=kc)
    d1, d0 = np.abs(K1 - Kr).max(), np.abs(K0 - Kr).max()
    print(f"{sysname}: max|dK| fused {d1:.3e}, unfused {d0:.3e}")
    assert d1 <= 1e-9 and d0 <= 1e-9
    assert np.array_equal(J1, J0)
    assert np.array_equal(K1, K2) and np.array_equal(J1, J2)
    assert np.abs(K1 - K1.T).max() == 0.0


@pytest.mark.parametrize("aux_batch", [0, 200])
def test_split_k_block_filter(aux_batch, decane):
    """The mixed path's K block filter (after the last split-K reduction,
    unbatched and auxiliary-batched) is the oracle's block filter applied to
    the unfiltered mixed K, bit for bit, at a threshold where it acts."""
    ds = decane
    C = _core_orbitals(ds)
    out = {}
    for eps in (0.0, 1e-6):
        eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=eps, precision="split",
                       aux_batch=aux_batch)
        _, out[eps] = eng.compute_jk(None, C, "dfmo")
        eng.close()
    Kf = Oracle(ds.layout, ds.B).filter(out[0.0], 1e-6)
    assert (Kf == 0).sum() > (out[0.0] == 0).sum()  # the filter acts here
    assert np.array_equal(out[1e-6], Kf)


def test_split_scf_energy(water):
    from chem_gb300.scf import run_rhf
    ds = water
    res = {}
    for prec in ("fp64", "split"):
        eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=prec)

        def jk(P, C):
            return eng.compute_jk(2 * P, C, "dfmo")

        r = run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=1e-10)
        assert r.converged
        res[prec] = r.energy
        eng.close()
    assert abs(res["split"] - res["fp64"]) <= 1e-8
