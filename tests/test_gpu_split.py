"""Split-precision (BF16 digit slices on tcgen05 tensor cores) K path against
the FP64 oracle.  Tolerances are the configs' bars: max|dK| <= 1e-9 and, for
SCF energies, |dE| <= 1e-8 Eh against the FP64 path.  J stays FP64 in the
mixed mode and must be bit-identical to the plain path."""
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
    assert dK <= 1e-9
    assert np.array_equal(J, Jr)
    # repeated builds are deterministic
    _, K2 = eng.compute_jk(None, C, "dfmo")
    assert np.array_equal(K, K2)
    eng.close()


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
