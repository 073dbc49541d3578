"""Atoms, basis sets and atom blocks for the DF Fock build.

Mirrors megalochem's descriptors:
  * basis JSON reading (Basis Set Exchange format), general contractions
    split into one shell per coefficient column with zero coefficients
    dropped, sp shells split into s and p (src/desc/basis.cpp:173-276);
  * "atomic" clustering: all shells of one atom form one block
    (src/desc/basis.cpp:52-82), which sets the block sizes the kernels see;
  * geometry in angstrom converted with 0.529177210671212
    (src/utils/constants.hpp, src/megalochem_driver.cpp:358-378).
Atom order is kept as given (megalochem reorders atoms by reverse
Cuthill-McKee by default, src/megalochem_driver.cpp:380-399; the generators
in geometry.py already emit chain-ordered atoms).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field

import numpy as np

BOHR_PER_ANGSTROM = 1.0 / 0.529177210671212
SYMBOL_Z = {"H": 1, "He": 2, "C": 6, "N": 7, "O": 8}
BASIS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis")


@dataclass
class Shell:
    l: int
    atom: int
    center: np.ndarray
    alpha: np.ndarray
    coef: np.ndarray

    @property
    def size(self):
        return 2 * self.l + 1


def read_atom_basis(name: str, symbols):
    """Per-element shell lists (exponents, coefficients) from a BSE JSON file
    (src/desc/basis.cpp:173-276)."""
    path = os.path.join(BASIS_DIR, name.lower() + ".json")
    if not os.path.exists(path):
        raise RuntimeError(f"Could not find basis {name}")
    with open(path) as f:
        data = json.load(f)["elements"]
    out = {}
    for s in set(symbols):
        z = str(SYMBOL_Z[s])
        shells = []
        for sh in data[z]["electron_shells"]:
            alpha = np.array([float(x) for x in sh["exponents"]])
            ams = sh["angular_momentum"]
            if len(ams) == 1:
                for col in sh["coefficients"]:
                    c = np.array([float(x) for x in col])
                    keep = np.abs(c) > np.finfo(float).eps
                    shells.append((ams[0], alpha[keep], c[keep]))
            else:
                for l, col in zip(ams, sh["coefficients"]):
                    shells.append((l, alpha.copy(), np.array([float(x) for x in col])))
        out[s] = shells
    return out


@dataclass
class Basis:
    name: str
    shells: list
    block_shell_off: np.ndarray  # shell range of each atom block
    block_sizes: np.ndarray  # functions per atom block
    block_atom: np.ndarray

    @property
    def nbf(self):
        return int(self.block_sizes.sum())

    @property
    def nshell(self):
        return len(self.shells)

    @property
    def nblk(self):
        return len(self.block_sizes)

    @property
    def block_offsets(self):
        return np.concatenate([[0], np.cumsum(self.block_sizes)]).astype(np.int64)

    def shell_bf_offsets(self):
        return np.concatenate([[0], np.cumsum([s.size for s in self.shells])]).astype(np.int64)


def make_basis(name: str, symbols, coords_bohr) -> Basis:
    """Shells for every atom, atomic clustering (src/desc/basis.cpp:52-82)."""
    table = read_atom_basis(name, symbols)
    shells = []
    blk_off = [0]
    blk_sizes = []
    for ia, s in enumerate(symbols):
        n = 0
        for (l, a, c) in table[s]:
            shells.append(Shell(l, ia, np.asarray(coords_bohr[ia], float), a, c))
            n += 2 * l + 1
        blk_off.append(len(shells))
        blk_sizes.append(n)
    return Basis(name, shells, np.array(blk_off, np.int32), np.array(blk_sizes, np.int64),
                 np.arange(len(symbols)))


@dataclass
class Molecule:
    symbols: list
    coords: np.ndarray  # bohr, natom x 3
    basis_name: str
    dfbasis_name: str
    charge: int = 0
    basis: Basis = field(init=False)
    dfbasis: Basis = field(init=False)

    def __post_init__(self):
        self.coords = np.asarray(self.coords, float).reshape(-1, 3)
        self.basis = make_basis(self.basis_name, self.symbols, self.coords)
        self.dfbasis = make_basis(self.dfbasis_name, self.symbols, self.coords)

    @property
    def charges(self):
        return np.array([SYMBOL_Z[s] for s in self.symbols], float)

    @property
    def nelectron(self):
        return int(self.charges.sum()) - self.charge

    @property
    def nocc(self):
        ne = self.nelectron
        if ne % 2:
            raise ValueError("closed-shell RHF needs an even electron count")
        return ne // 2

    def nuclear_repulsion(self):
        Z = self.charges
        R = self.coords
        e = 0.0
        for i in range(len(Z)):
            for j in range(i):
                e += Z[i] * Z[j] / np.linalg.norm(R[i] - R[j])
        return e


def rcm_order(coords_bohr, cutoff=5.0):
    """megalochem's atom reordering (math::rcm, src/math/other/rcm.hpp,
    applied by default in src/megalochem_driver.cpp:380-399 with a 5 bohr
    cutoff): atoms closer than `cutoff` are connected; each breadth-first
    sweep starts from one atom of the most distant pair that still has an
    atom outside the order (the one with fewer neighbours, or the one not
    yet placed), neighbours are queued by decreasing degree (ties keep the
    index order, as the reference's sort does for fewer than 17 neighbours),
    and the final order is reversed.  Returns the new atom order: atom i of
    the reordered molecule is atom order[i] of the input."""
    X = np.asarray(coords_bohr, float)
    n = len(X)
    d = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    con = d < cutoff
    deg = con.sum(1) - 1
    iu = np.triu_indices(n, 1)
    placed = np.zeros(n, bool)
    R = []

    def neighbours(p):
        nb = [i for i in range(n) if con[p, i] and i != p]
        return sorted(nb, key=lambda i: -deg[i])  # stable: ties keep index order

    while len(R) < n:
        free = ~(placed[iu[0]] & placed[iu[1]])
        dv = np.where(free, d[iu], 0.0)
        k = int(np.argmax(dv))  # first pair of the row-major scan at the maximum
        n1, n2 = int(iu[0][k]), int(iu[1][k])
        p = n2 if ((deg[n1] > deg[n2] or placed[n1]) and not placed[n2]) else n1
        R.append(p)
        placed[p] = True
        queue = list(neighbours(p))
        while queue:
            q = queue.pop(0)
            if placed[q]:
                continue
            R.append(q)
            placed[q] = True
            queue.extend(neighbours(q))
    return R[::-1]


def molecule_from_angstrom(symbols, coords_ang, basis="cc-pvdz", dfbasis="cc-pvdz-jkfit",
                           charge=0, reorder=False) -> Molecule:
    """reorder=True applies megalochem's default atom reordering (rcm_order)
    so that atom blocks, and so J and K element by element, come in the
    reference's order; the generators here emit chain order."""
    sym = list(symbols)
    X = np.asarray(coords_ang, float) * BOHR_PER_ANGSTROM
    if reorder:
        order = rcm_order(X)
        sym = [sym[i] for i in order]
        X = X[order]
    return Molecule(sym, X, basis, dfbasis, charge)
