"""Failure detection in the split-precision GEMM without a GPU fault: the
test hook makes the producer stop issuing operand copies at one work item,
so the consumers' bounded mbarrier waits (a few ms here) run out.  The
build must return TIMEOUT rather than hang, every CTA waits for its own
copies and MMAs before exiting, and the context stays usable: the next
build (hook off) gives the same bits as before, since the error flag is
cleared at the start of every build."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("item", [0, 5])
def test_split_wait_times_out_and_context_recovers(butane, item):
    ds = butane
    rng = np.random.default_rng(1)
    C = np.ascontiguousarray(np.linalg.qr(rng.standard_normal((ds.nbf, ds.nbf)))[0][:, :ds.nocc])
    P = C @ C.T
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    J0, K0 = eng.compute_jk(2 * P, C)
    eng.test_split_stall(item, wait_ms=5.0)
    with pytest.raises(RuntimeError, match="TIMEOUT"):
        eng.compute_jk(2 * P, C)
    eng.test_split_stall(-1)
    J1, K1 = eng.compute_jk(2 * P, C)
    J2, K2 = eng.compute_jk(2 * P, C)  # replays the captured build
    eng.close()
    assert np.array_equal(J0, J1) and np.array_equal(K0, K1)
    assert np.array_equal(J1, J2) and np.array_equal(K1, K2)
