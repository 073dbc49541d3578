"""The SCF iteration on the device (gbjk_scf_*: P = C C^T, the Fock build,
F = H + J + K, the energy, FPS - SPF with its RMS and the DIIS overlaps in
one CUDA graph; the DIIS combination and X F X in another) against the host
SCF driver with the same engine: same converged energies and iteration
counts on decane, FP64 (Cholesky route) and mixed precision switching to
FP64."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine
from chem_gb300.scf import fp64_switch, run_rhf, run_rhf_device

pytestmark = pytest.mark.gpu


def test_device_scf_matches_host_scf(decane):
    ds = decane
    enuc = ds.mol.nuclear_repulsion()
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10)

    def jk(P, C):
        return eng.compute_jk(2 * P, C, "dfmo")

    res = {}
    for mode in ("fp64", "mixed"):
        for where in ("host", "device"):
            eng.set_jmode("cholesky")
            eng.set_precision("fp64" if mode == "fp64" else "split")
            sw = fp64_switch(eng, "cholesky") if mode == "mixed" else None
            if where == "host":
                r = run_rhf(ds.S, ds.Hcore, enuc, ds.nocc, jk, conv=1e-9, switch=sw)
            else:
                r = run_rhf_device(eng, ds.S, ds.Hcore, enuc, ds.nocc, conv=1e-9, switch=sw)
            assert r.converged
            res[(mode, where)] = r
            print(f"{mode:6s} {where:6s} E {r.energy:.12f} ({r.iterations} it)")
    # the device F of the last build equals H + J + K of a host build at P
    eng.set_precision("fp64")
    r = res[("fp64", "device")]
    J, K = jk(r.P, r.C[:, :ds.nocc])
    assert np.abs(r.F - (ds.Hcore + J + K)).max() <= 1e-11
    eng.close()
    for mode in ("fp64", "mixed"):
        h, d = res[(mode, "host")], res[(mode, "device")]
        assert abs(h.energy - d.energy) <= 1e-9
        assert abs(h.iterations - d.iterations) <= 2
    assert abs(res[("mixed", "device")].energy - res[("fp64", "host")].energy) <= 1e-8


def test_device_scf_audit_and_graph_reuse(water):
    ds = water
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    eng.set_jmode("cholesky")
    n0 = eng.kernel_launches

    def audit(P, C, J, K):
        eng.set_precision("fp64")
        J64, K64 = eng.compute_jk(2 * P, C)
        eng.set_precision("split")
        return float(np.abs(K - K64).max())

    r = run_rhf_device(eng, ds.S, ds.Hcore, ds.mol.nuclear_repulsion(), ds.nocc, conv=1e-9,
                       audit=audit)
    assert r.converged and len(r.audit) == r.iterations
    assert max(r.audit) <= 1e-9
    assert eng.kernel_launches > n0
    eng.close()
