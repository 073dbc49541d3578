"""A Fock build captured as a CUDA graph replays to the same bits as the
direct call, for new input contents behind the same device pointers."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_graph_replay_matches_direct(precision, decane):
    import torch
    ds = decane
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=precision)
    dev = torch.device("cuda", 0)
    n, nocc = ds.nbf, ds.nocc
    rng = np.random.default_rng(5)
    Cs = [np.linalg.qr(rng.standard_normal((n, n)))[0][:, :nocc] for _ in range(2)]
    dP = torch.empty((n, n), dtype=torch.float64, device=dev)
    dC = torch.empty((n, nocc), dtype=torch.float64, device=dev)
    dJ = torch.empty((n, n), dtype=torch.float64, device=dev)
    dK = torch.empty((n, n), dtype=torch.float64, device=dev)
    dP.copy_(torch.from_numpy(2 * Cs[0] @ Cs[0].T))
    dC.copy_(torch.from_numpy(np.ascontiguousarray(Cs[0])))
    torch.cuda.synchronize()
    eng.capture_graph(dP.data_ptr(), dC.data_ptr(), nocc, dJ.data_ptr(), dK.data_ptr())
    for Cm in Cs:
        dP.copy_(torch.from_numpy(2 * Cm @ Cm.T))
        dC.copy_(torch.from_numpy(np.ascontiguousarray(Cm)))
        torch.cuda.synchronize()
        eng.launch_graph()
        eng.synchronize()
        Jg, Kg = dJ.cpu().numpy(), dK.cpu().numpy()
        J, K = eng.compute_jk(2 * Cm @ Cm.T, Cm)
        assert np.array_equal(Jg, J)
        assert np.array_equal(Kg, K)
    eng.close()
