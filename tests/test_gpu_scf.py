"""Full DF-HF SCF through the device engine (decane, cc-pVDZ/cc-pVDZ-jkfit).

* FP64 on the reference route (explicit V^-1, as fock::DF_J) and on the
  Cholesky route; the two differ by the conditioning error of V^-1.
* Mixed precision switching to FP64 (Cholesky route) once the DIIS error is
  below 1e-5: converges to the FP64 Cholesky energy within 1e-8 Eh.
* Mixed precision throughout: within 1e-8 Eh of the FP64 Cholesky energy."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine
from chem_gb300.scf import run_rhf

pytestmark = pytest.mark.gpu


def _scf(ds, eng, switch=None, conv=1e-9):
    def jk(P, C):
        return eng.compute_jk(2 * P, C, "dfmo")
    return run_rhf(ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, jk, conv=conv,
                   switch=switch)


def test_scf_mixed_vs_fp64(decane):
    ds = decane
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)
    r_ref = _scf(ds, eng)
    eng.set_jmode("cholesky")
    r_chol = _scf(ds, eng)
    eng.set_precision("split")
    r_mix = _scf(ds, eng)

    def to_fp64():
        eng.set_precision("fp64")

    eng.set_precision("split")
    r_sw = _scf(ds, eng, switch=to_fp64)
    eng.close()
    for r in (r_ref, r_chol, r_mix, r_sw):
        assert r.converged
    print(f"E fp64 V^-1 route  {r_ref.energy:.12f} ({r_ref.iterations} it)")
    print(f"E fp64 Cholesky    {r_chol.energy:.12f} ({r_chol.iterations} it)")
    print(f"E mixed            {r_mix.energy:.12f} ({r_mix.iterations} it)")
    print(f"E mixed -> fp64    {r_sw.energy:.12f} ({r_sw.iterations} it)")
    assert abs(r_mix.energy - r_chol.energy) <= 1e-8
    assert abs(r_sw.energy - r_chol.energy) <= 1e-8
    assert abs(r_ref.energy - r_chol.energy) <= 1e-6
