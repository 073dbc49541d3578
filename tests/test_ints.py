"""Host integral engine: known-answer tests.

megalochem computes its integrals with libcint, which it does not vendor, and
ships no integral fixtures.  The engine is pinned instead to published
values: T. D. Crawford's "Programming Projects" #3 (water, STO-3G, the
Szabo-Ostlund geometry) lists S, T, V, (00|00) and the converged RHF energy
-74.942079928192 Eh for the psi4 STO-3G set used below.
"""
import json
import os

import mpmath
import numpy as np
import pytest

from chem_gb300 import ints
from chem_gb300.molecule import Molecule, molecule_from_angstrom

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def crawford_water():
    with open(os.path.join(GOLDEN, "crawford_h2o_sto3g.json")) as f:
        g = json.load(f)
    mol = Molecule(["O", "H", "H"], np.array(g["geometry_bohr"]), "sto-3g", "cc-pvdz-jkfit")
    # psi4's STO-3G digits (BSE carries more digits for the same set)
    sh = mol.basis.shells
    for s, (alpha, coef) in zip(sh, g["shells"]):
        s.alpha = np.array(alpha)
        s.coef = np.array(coef)
    return mol, g


def rhf_exact(mol, S, H, eri, conv=1e-12):
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    F = H.copy()
    E_old = 0.0
    for _ in range(300):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        Co = (X @ Cp)[:, :mol.nocc]
        P = Co @ Co.T
        J = np.einsum("mnls,ls->mn", eri, P)
        K = np.einsum("mlns,ls->mn", eri, P)
        F = H + 2 * J - K
        E = np.sum(P * (H + F)) + mol.nuclear_repulsion()
        if abs(E - E_old) < conv:
            return E
        E_old = E
    raise AssertionError("no convergence")


def test_crawford_components():
    mol, g = crawford_water()
    S = ints.one_electron(mol, "overlap")
    T = ints.one_electron(mol, "kinetic")
    V = ints.one_electron(mol, "nuclear")
    eri = ints.eri4c(mol)
    assert abs(mol.nuclear_repulsion() - g["enuc"]) < 1e-12
    assert abs(S[0, 1] - g["S01"]) < 1e-13
    assert abs(T[0, 0] - g["T00"]) < 1e-12
    assert abs(V[0, 0] - g["V00"]) < 1e-12
    assert abs(eri[0, 0, 0, 0] - g["eri0000"]) < 1e-12
    # 8-fold permutational symmetry
    assert np.allclose(eri, eri.transpose(1, 0, 2, 3), atol=1e-14)
    assert np.allclose(eri, eri.transpose(2, 3, 0, 1), atol=1e-14)


def test_crawford_scf_energy():
    mol, g = crawford_water()
    S = ints.one_electron(mol, "overlap")
    H = ints.one_electron(mol, "kinetic") + ints.one_electron(mol, "nuclear")
    E = rhf_exact(mol, S, H, ints.eri4c(mol))
    assert abs(E - g["escf"]) < 1e-10


def test_normalisation_all_shells():
    # one atom of each element: every contracted spherical function has norm 1
    for basis in ["cc-pvdz", "cc-pvdz-jkfit", "cc-pvdz-ri"]:
        mol = Molecule(["C", "O", "H"], np.array([[0, 0, 0], [0, 0, 20.0], [0, 20.0, 0]]),
                       basis, "cc-pvdz-jkfit")
        S = ints.one_electron(mol, "overlap")
        assert np.allclose(np.diag(S), 1.0, atol=1e-12), basis
        # functions of one shell are orthonormal
        off = 0
        for s in mol.basis.shells:
            blk = S[off:off + s.size, off:off + s.size]
            assert np.allclose(blk, np.eye(s.size), atol=1e-12)
            off += s.size


def test_boys_against_mpmath():
    # (ss|ss) with primitive s functions tests F_0; the 2c integral (s|s)
    # between unnormalised-by-hand single primitives has the closed form
    # (a|b) = 2 pi^{5/2} / (a b sqrt(a+b)) F_0(a b/(a+b) R^2) N_a N_b
    a, b = 0.8, 1.7
    # T = 0.544 R^2: 0, 0.05, 2.2, 10.1 (Taylor grid), 20.3, 30.6, 122 (asymptotic)
    for R in [0.0, 0.3, 2.0, 4.3, 6.11, 7.5, 15.0]:
        mol = Molecule(["H", "H"], np.array([[0, 0, 0], [0, 0, R + 1e-300]]), "sto-3g",
                       "cc-pvdz-jkfit")
        mol.dfbasis.shells = mol.dfbasis.shells[:1]
        sh0 = mol.dfbasis.shells[0]
        sh0.alpha = np.array([a])
        sh0.coef = np.array([1.0])
        import copy
        sh1 = copy.deepcopy(sh0)
        sh1.alpha = np.array([b])
        sh1.center = np.array([0, 0, R])
        mol.dfbasis.shells = [sh0, sh1]
        mol.dfbasis.block_shell_off = np.array([0, 1, 2], np.int32)
        mol.dfbasis.block_sizes = np.array([1, 1])
        M = ints.coulomb_metric(mol)
        mp = mpmath.mp
        mp.dps = 30
        T = mp.mpf(a * b / (a + b) * R * R)
        F0 = mp.sqrt(mp.pi / T) / 2 * mp.erf(mp.sqrt(T)) if T > 0 else mp.mpf(1)
        Na = (2 * mp.mpf(a) / mp.pi) ** mp.mpf(0.75)
        Nb = (2 * mp.mpf(b) / mp.pi) ** mp.mpf(0.75)
        ref = 2 * mp.pi ** 2.5 / (a * b * mp.sqrt(a + b)) * F0 * Na * Nb
        assert abs(M[0, 1] - float(ref)) < 1e-13 * max(1.0, abs(float(ref)))


def test_rotation_invariance_3c_norms():
    # the Frobenius norm of every (X-shell | mu-shell nu-shell) block is
    # invariant under a rigid rotation: checks d/f solid harmonics
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300 import geometry
    s, x = geometry.water()
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    R = R @ np.array([[1, 0, 0], [0, np.cos(0.4), -np.sin(0.4)], [0, np.sin(0.4), np.cos(0.4)]])
    d1 = build_dfsystem(molecule_from_angstrom(s, x), eps=0.0, one_electron=False)
    d2 = build_dfsystem(molecule_from_angstrom(s, x @ R.T), eps=0.0, one_electron=False)
    T1 = d1.layout.to_dense(d1.B)
    T2 = d2.layout.to_dense(d2.B)
    so = d1.mol.basis.shell_bf_offsets()
    sx = d1.mol.dfbasis.shell_bf_offsets()
    for a in range(len(so) - 1):
        for b in range(len(so) - 1):
            for c in range(0, len(sx) - 1, 3):
                n1 = np.linalg.norm(T1[sx[c]:sx[c + 1], so[a]:so[a + 1], so[b]:so[b + 1]])
                n2 = np.linalg.norm(T2[sx[c]:sx[c + 1], so[a]:so[a + 1], so[b]:so[b + 1]])
                assert abs(n1 - n2) < 1e-11 * max(1, n1)
    # metric eigenvalues are rotation invariant too
    assert np.allclose(np.linalg.eigvalsh(d1.V), np.linalg.eigvalsh(d2.V), rtol=1e-11, atol=1e-12)
