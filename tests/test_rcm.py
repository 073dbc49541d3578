"""megalochem's default atom reordering (chem_gb300.molecule.rcm_order,
restating src/math/other/rcm.hpp as src/megalochem_driver.cpp:380-399
applies it): a valid permutation that narrows the connectivity band of a
shuffled molecule, and a DF-HF energy independent of the atom order."""
import numpy as np

from chem_gb300 import geometry
from chem_gb300.molecule import BOHR_PER_ANGSTROM, molecule_from_angstrom, rcm_order


def _band(X, cutoff=5.0):
    d = np.sqrt(((X[:, None] - X[None]) ** 2).sum(-1))
    i, j = np.nonzero(d < cutoff)
    return int(np.abs(i - j).max())


def test_rcm_is_a_permutation_and_narrows_the_band():
    s, x = geometry.alkane(6)
    X = np.asarray(x) * BOHR_PER_ANGSTROM
    rng = np.random.default_rng(4)
    Xs = X[rng.permutation(len(X))]
    o = rcm_order(Xs)
    assert sorted(o) == list(range(len(X)))
    assert _band(Xs[o]) < _band(Xs)
    # deterministic, and independent of where the atoms sit in space
    assert rcm_order(Xs) == o
    assert rcm_order(Xs + 3.0) == o
    # water: the reference's rule starts from one hydrogen of the most
    # distant pair and ends (after the reversal) with the other
    sw, xw = geometry.water()
    ow = rcm_order(np.asarray(xw) * BOHR_PER_ANGSTROM)
    assert [sw[i] for i in ow] == ["H", "O", "H"]


def test_energy_independent_of_atom_order():
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.scf import run_rhf
    from oracle.oracle import Oracle
    s, x = geometry.water()
    E = []
    for reorder in (False, True):
        ds = build_dfsystem(molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit",
                                                   reorder=reorder), eps=1e-10)
        O = Oracle(ds.layout, ds.B)
        Linv = np.tril(ds.Linv)

        # J on the Cholesky route: the explicit V^-1 adds order-dependent
        # rounding of ~5e-10 Eh even for water
        def jk(Pa, Ca):
            return O.df_j_chol(Linv, 2.0 * Pa, ds.eps), O.dfmo_k(Linv, Ca, ds.eps)

        r = run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=1e-9)
        assert r.converged
        E.append(r.energy)
    assert abs(E[0] - E[1]) <= 1e-10
