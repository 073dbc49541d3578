"""The C-ABI libraries load and export every symbol their headers declare;
argument checks that need no GPU reject bad input."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gb(?:jk|ints)_[a-z0-9_]+)\s*\(", src)))


@pytest.mark.parametrize("header,lib", [("gbjk.h", "libgbjk.so"), ("gbints.h", "libgbints.so")])
def test_exports(header, lib):
    names = declared(header)
    assert names
    so = C.CDLL(os.path.join(ROOT, "chem_gb300", "lib", lib))
    for n in names:
        assert hasattr(so, n), f"{lib} does not export {n}"


def test_create_rejects_bad_desc():
    from chem_gb300 import fock
    L = fock.lib()
    h = C.c_void_p()
    assert L.gbjk_create(C.byref(h), None) == 1
    bs = (C.c_int * 2)(3, 2)
    K = (C.c_int * 2)(5, 5)
    cm = (C.c_int * 10)(*range(5), *range(5))
    # block sizes sum (5) != nbf (6)
    d = fock.GbjkDesc(6, 10, 2, bs, K, cm, 0.0, 0)
    assert L.gbjk_create(C.byref(h), C.byref(d)) == 1
    # column index out of range
    cm2 = (C.c_int * 10)(*range(5), 0, 1, 2, 3, 9)
    d = fock.GbjkDesc(5, 10, 2, bs, K, cm2, 0.0, 0)
    assert L.gbjk_create(C.byref(h), C.byref(d)) == 1
    assert L.gbjk_set_precision(None, 0, 0) == 1
    assert L.gbjk_compute_j(None, None, None) == 1


def test_product_has_no_oracle_import():
    # the product package must never route through the CPU oracle
    pkg = os.path.join(ROOT, "chem_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in re.sub(r"#.*|\"\"\"[\s\S]*?\"\"\"", "", src), f


def test_k_split_plan_covers_the_sum_in_aligned_chunks():
    # gbjk_k_split_plan needs no GPU: the chunks are multiples of 16, cover
    # the naux*nocc terms exactly once, hold at least 64 terms when split,
    # and split further for small exchange matrices (fewer output tiles)
    from chem_gb300.fock import k_split_plan
    for nbf, naux, nocc in [(24, 116, 5), (106, 510, 17), (490, 2366, 81), (970, 4686, 161),
                            (4000, 12000, 600), (7, 3, 1)]:
        ks, kc = k_split_plan(nbf, naux, nocc)
        kdim = naux * nocc
        assert ks >= 1 and kc % 16 == 0
        assert (ks - 1) * kc < kdim <= ks * kc
        assert ks == 1 or kc >= 64
    # water: one 64 x 64 output tile, 580 terms, still spread over parts
    assert k_split_plan(24, 116, 5)[0] > 1
    with pytest.raises(RuntimeError):
        k_split_plan(0, 116, 5)
