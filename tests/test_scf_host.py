"""The DF-HF SCF driver (chem_gb300/scf.py) on the CPU, with the oracle's
J and K as its Fock builder: it converges water (cc-pVDZ / cc-pVDZ-jkfit)
to the DF-HF energy, and the precision switch fires once."""
import numpy as np

from chem_gb300.scf import run_rhf


def test_scf_driver_with_oracle_jk(water):
    from oracle.oracle import Oracle
    ds = water
    O = Oracle(ds.layout, ds.B)
    Linv = np.tril(ds.Linv)
    calls = []

    def jk(Pa, Ca):
        return O.df_j(ds.Vinv, 2.0 * Pa, ds.eps), O.dfmo_k(Linv, Ca, ds.eps)

    def switch():
        calls.append(1)

    r = run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=1e-8,
                switch=switch)
    assert r.converged
    assert abs(r.energy - (-76.026747)) < 2e-6, r.energy
    assert calls == [1]
    # the same run again repeats the energy and iteration count exactly
    r2 = run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=1e-8,
                 switch=switch)
    assert r2.energy == r.energy and r2.iterations == r.iterations
    # without the switch the driver converges to the same energy
    r3 = run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=1e-8)
    assert r3.converged and abs(r3.energy - r.energy) < 1e-8
