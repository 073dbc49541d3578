"""Synthetic pre-fitted DF-K workload at a reduced size (nbf 400, naux 1200,
nocc 60): device-generated tensor, FP64 path bit-exact against the oracle on
the downloaded tensor, split path (unbatched and auxiliary-batched with a
short last batch, both digit cuts of H) within 1e-11 of max|K| of FP64."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine, k_split_plan
from chem_gb300.synthetic import occupied, synthetic_layout
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def test_synthetic_fp64_split_batched():
    nbf, naux, nocc = 400, 1200, 60
    layout, decay = synthetic_layout(nbf, naux, seed=7)
    C = occupied(nbf, nocc, seed=7)
    syn = (1234, decay)
    e64 = JKEngine(layout, None, None, None, fitted=True, synthetic=syn)
    _, K64 = e64.compute_jk(None, C)
    B = e64.download_b()
    e64.close()
    kc = k_split_plan(nbf, naux, nocc)[1]
    Kr = Oracle(layout, B).dfmo_k(None, C, 0.0, kchunk=kc)
    assert np.array_equal(K64, Kr)
    scale = np.abs(K64).max()
    for fuse in (True, False):
        for batch in (0, 256):
            es = JKEngine(layout, None, None, None, fitted=True, synthetic=syn,
                          precision="split", aux_batch=batch)
            es.set_split_fuse(fuse)
            _, Ks = es.compute_jk(None, C)
            # a second build on the same buffers gives the same bits (the
            # short last batch reuses H slots the full batches wrote)
            _, Ks2 = es.compute_jk(None, C)
            es.close()
            assert np.array_equal(Ks, Ks2)
            d = np.abs(Ks - K64).max()
            print(f"fuse {fuse} aux batch {batch}: max|dK| = {d:.3e} of max|K| = {scale:.3e}")
            assert d <= 1e-11 * scale
            assert np.abs(Ks - Ks.T).max() == 0.0


def test_synthetic_fp64_batched_matches_oracle():
    """FP64 exchange of the pre-fitted tensor in auxiliary batches (the path
    that lets the full 153 GB workload run in FP64): bit for bit the
    oracle's batched order, and within rounding of the unbatched FP64 K."""
    from chem_gb300.fock import tune_plan
    nbf, naux, nocc = 400, 1200, 60
    layout, decay = synthetic_layout(nbf, naux, seed=7)
    C = occupied(nbf, nocc, seed=7)
    syn = (1234, decay)
    e64 = JKEngine(layout, None, None, None, fitted=True, synthetic=syn)
    _, K64 = e64.compute_jk(None, C)
    B = e64.download_b()
    e64.close()
    for batch in (256, 300):  # 300 rounds down to 288: batches of 288, last 48
        eb = JKEngine(layout, None, None, None, fitted=True, synthetic=syn, aux_batch=batch)
        _, Kb = eb.compute_jk(None, C)
        _, Kb2 = eb.compute_jk(None, C)
        eb.close()
        xb = batch & ~31
        xlast = naux - (-(-naux // xb) - 1) * xb
        kc_full = tune_plan(nbf, xb, nocc)[0]["fp64_kchunk"]
        kc_last = tune_plan(nbf, xlast, nocc)[0]["fp64_kchunk"]
        Kr = Oracle(layout, B).dfmo_k_batched(C, xb, kc_full, kc_last)
        assert np.array_equal(Kb, Kr), (batch, np.abs(Kb - Kr).max())
        assert np.array_equal(Kb, Kb2)
        assert np.abs(Kb - K64).max() <= 1e-12 * np.abs(K64).max()
