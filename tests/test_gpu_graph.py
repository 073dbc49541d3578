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


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_host_calls_replay_their_graph(precision, decane):
    # gbjk_compute_jk captures each argument shape on its first call and
    # replays it afterwards: every call, in any order of shapes, gives the
    # bits of the direct device-pointer build
    import torch
    from chem_gb300.fock import host_array
    ds = decane
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision=precision)
    dev = torch.device("cuda", 0)
    n = ds.nbf
    rng = np.random.default_rng(9)
    Q = np.linalg.qr(rng.standard_normal((n, n)))[0]

    def direct(P, Cm, want_j=True, want_k=True):
        dP = torch.from_numpy(P).to(dev)
        dC = torch.from_numpy(np.ascontiguousarray(Cm)).to(dev)
        dJ = torch.empty((n, n), dtype=torch.float64, device=dev)
        dK = torch.empty((n, n), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        eng.compute_jk_dev(dP.data_ptr() if want_j else None, dC.data_ptr() if want_k else None,
                           Cm.shape[1] if want_k else 0, dJ.data_ptr() if want_j else None,
                           dK.data_ptr() if want_k else None)
        eng.synchronize()
        return dJ.cpu().numpy(), dK.cpu().numpy()

    out = (host_array((n, n)), host_array((n, n)))
    for nocc in (ds.nocc, ds.nocc, ds.nocc - 3, ds.nocc):
        Cm = Q[:, :nocc] * (1.0 + 0.01 * nocc)
        P = 2 * Cm @ Cm.T
        Jd, Kd = direct(P, Cm)
        # J alone takes the FP64 J route, K alone the K launches only
        Jo, _ = direct(P, Cm, want_k=False)
        _, Ko = direct(P, Cm, want_j=False)
        for _ in range(3):
            J, K = eng.compute_jk(P, Cm)
            assert np.array_equal(J, Jd) and np.array_equal(K, Kd)
            Jp, Kp = eng.compute_jk(P, Cm, out=out)
            assert Jp is out[0] and np.array_equal(Jp, Jd) and np.array_equal(Kp, Kd)
            J1, K1 = eng.compute_jk(P, None)
            assert K1 is None and np.array_equal(J1, Jo)
            J2, K2 = eng.compute_jk(None, Cm)
            assert J2 is None and np.array_equal(K2, Ko)
    eng.close()


def test_captured_build_goes_stale_on_state_change(decane):
    import torch
    ds = decane
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=1e-10, precision="split")
    dev = torch.device("cuda", 0)
    n, nocc = ds.nbf, ds.nocc
    rng = np.random.default_rng(4)
    Cm = np.linalg.qr(rng.standard_normal((n, n)))[0][:, :nocc]
    dP = torch.from_numpy(2 * Cm @ Cm.T).to(dev)
    dC = torch.from_numpy(np.ascontiguousarray(Cm)).to(dev)
    dJ = torch.empty((n, n), dtype=torch.float64, device=dev)
    dK = torch.empty((n, n), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    eng.capture_graph(dP.data_ptr(), dC.data_ptr(), nocc, dJ.data_ptr(), dK.data_ptr())
    eng.launch_graph()
    eng.synchronize()
    # a build with another nocc replaces the coefficient workspaces the graph
    # reads: the captured build is refused, not replayed on freed memory
    eng.compute_jk(None, Cm[:, :-2])
    with pytest.raises(RuntimeError, match="NOT_READY"):
        eng.launch_graph()
    eng.capture_graph(dP.data_ptr(), dC.data_ptr(), nocc, dJ.data_ptr(), dK.data_ptr())
    eng.launch_graph()
    eng.synchronize()
    eng.set_precision("fp64")
    with pytest.raises(RuntimeError, match="NOT_READY"):
        eng.launch_graph()
    eng.close()
