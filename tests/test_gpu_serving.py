"""Continuous batching on the GPU: every request served in the mix (several
molecules in flight on their own streams, engines evicted under a tight HBM
budget) is bit-identical to the same build served alone."""
import numpy as np
import pytest

from chem_gb300.fock import JKEngine
from chem_gb300.serving import FockServer, Request, footprint_bytes, make_system_factory

pytestmark = pytest.mark.gpu

MOLS = [("water", 1), ("water", 2), ("alkane", 3), ("alkane", 4), ("water", 3)]


def test_mix_equals_solo():
    factories = {f"{k}{n}": make_system_factory(k, n) for k, n in MOLS}
    systems = {key: f() for key, f in factories.items()}
    # solo results: a fresh engine per molecule, nothing else on the GPU
    solo = {}
    for key, (ds, P, C) in systems.items():
        eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, precision="split")
        solo[key] = eng.compute_jk(2.0 * P, C)
        eng.close()
    fps = sorted(footprint_bytes(ds.layout, ds.nocc) for ds, _, _ in systems.values())
    budget = fps[-1] + fps[-2]  # at most two molecules resident: forces eviction
    rng = np.random.default_rng(0)
    keys = list(systems)
    reqs = [Request(i, keys[int(rng.integers(len(keys)))], 0.002 * i,
                    (lambda k: (lambda: systems[k]))(keys[int(rng.integers(len(keys)))]))
            for i in range(40)]
    for q in reqs:  # make the factory match the key
        q.make_system = (lambda k: (lambda: systems[k]))(q.key)
    srv = FockServer(budget_bytes=budget, slots=4, precision="split", drop_host_tensor=False)
    done = srv.run(reqs)
    srv.close()
    assert all(q.error is None for q in done), [q.error for q in done if q.error]
    assert srv.max_used <= budget
    for q in done:
        Js, Ks = solo[q.key]
        assert np.array_equal(q.J, Js) and np.array_equal(q.K, Ks), q.key
