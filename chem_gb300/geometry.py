"""Molecule generators for the DF Fock-build workloads.

* water: the geometry of megalochem's examples/h2o.json (angstrom);
* linear all-trans alkanes C_nH_{2n+2} from a seed-free rule: C-C 1.54 A,
  C-H 1.09 A, tetrahedral angles, planar zig-zag backbone, CH2 hydrogens in
  the plane perpendicular to the backbone, terminal CH3 groups staggered;
* water clusters (H2O)_k: O atoms on a 2.8 A cubic lattice with +-0.2 A
  uniform jitter and randomly oriented water molecules of the h2o.json shape.
Atoms are emitted in chain order (each heavy atom followed by its hydrogens),
which keeps the atom-block sparsity pattern banded.
"""
from __future__ import annotations

import numpy as np

WATER_SYMBOLS = ["O", "H", "H"]
WATER_ANGSTROM = np.array([
    [0.00000, 0.00000, 0.11779],
    [0.00000, 0.75545, -0.47116],
    [0.00000, -0.75545, -0.47116],
])

CC = 1.54
CH = 1.09
TET = np.arccos(-1.0 / 3.0)  # 109.4712 degrees


def alkane(n: int):
    """n-C_nH_{2n+2}: returns (symbols, coords in angstrom).

    Carbon i sits at (i*dx, (i%2)*dy, 0) with dx = CC sin(T/2), dy = CC cos(T/2)
    so every C-C-C angle is tetrahedral (T).  The two hydrogens of a carbon lie
    in the plane perpendicular to the backbone plane, pointing away from the
    neighbours at half the tetrahedral angle; each terminal carbon carries a
    third hydrogen where the next carbon of the zig-zag would be (staggered).
    """
    if n < 1:
        raise ValueError("n >= 1")
    half = TET / 2.0
    dx, dy = CC * np.sin(half), CC * np.cos(half)

    def cpos(i):
        return np.array([i * dx, (i % 2) * dy, 0.0])

    sym, xyz = [], []
    for i in range(n):
        c = cpos(i)
        sym.append("C")
        xyz.append(c)
        if n == 1:
            for d in np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float):
                sym.append("H")
                xyz.append(c + CH * d / np.linalg.norm(d))
            continue
        up = -1.0 if i % 2 == 0 else 1.0  # away from the neighbours
        for s in (1.0, -1.0):
            d = np.array([0.0, up * np.cos(half), s * np.sin(half)])
            sym.append("H")
            xyz.append(c + CH * d)
        if i == 0 or i == n - 1:
            ghost = cpos(-1) if i == 0 else cpos(n)
            d = ghost - c
            sym.append("H")
            xyz.append(c + CH * d / np.linalg.norm(d))
    return sym, np.array(xyz)


def water():
    return list(WATER_SYMBOLS), WATER_ANGSTROM.copy()


def water_cluster(k: int, rng: np.random.Generator, spacing=2.8, jitter=0.2):
    """(H2O)_k with O on a cubic lattice, uniform jitter, random orientation."""
    side = int(np.ceil(k ** (1.0 / 3.0)))
    sites = [(i, j, l) for i in range(side) for j in range(side) for l in range(side)][:k]
    o_ref = WATER_ANGSTROM[0]
    sym, xyz = [], []
    for s in sites:
        o = np.array(s, float) * spacing + rng.uniform(-jitter, jitter, 3)
        # random rotation from a normalised Gaussian quaternion
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        a, b, c, d = q
        R = np.array([
            [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
            [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
            [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
        ])
        for sy, p in zip(WATER_SYMBOLS, WATER_ANGSTROM):
            sym.append(sy)
            xyz.append(o + R @ (p - o_ref))
    return sym, np.array(xyz)
