import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from chem_gb300 import build
    build.build_all()
    from oracle import oracle
    oracle.build()
    yield


@pytest.fixture(scope="session")
def water():
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.water()
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    return build_dfsystem(mol, eps=1e-10)


@pytest.fixture(scope="session")
def butane():
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(4)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    return build_dfsystem(mol, eps=1e-10)


@pytest.fixture(scope="session")
def decane():
    """n-C10H22: the smallest alkane here with Schwarz-screened block pairs
    (96.5 % of AO block pairs kept)."""
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(10)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    return build_dfsystem(mol, eps=1e-10)


@pytest.fixture(scope="session")
def c20h42():
    """n-C20H42, the benchmark molecule (nbf 490, naux 2366, nocc 81)."""
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(20)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    return build_dfsystem(mol, eps=1e-10)
