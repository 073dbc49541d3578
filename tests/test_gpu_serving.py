"""Continuous batching on the GPU: every request served in the mix (several
molecules in flight on their own streams, engines evicted under a tight HBM
budget) is bit-identical to the same build served alone."""
import time

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


def test_mix_equals_solo_with_device_setup():
    # host and device integral workers share the set-up queue: every result
    # equals the solo build of the same molecule set up by the same route
    mols = [("water", 2), ("alkane", 3), ("alkane", 4), ("water", 3), ("alkane", 5)]
    host = {f"{k}{n}": make_system_factory(k, n)() for k, n in mols}
    dev = {f"{k}{n}": make_system_factory(k, n, device_ints=True)() for k, n in mols}
    keys = list(host)

    def host_setup(k):  # the host integrals take a while, as they do
        def f():
            time.sleep(0.3)
            return host[k]
        return f

    reqs = []
    for i in range(30):
        key = keys[i % len(keys)]
        reqs.append(Request(i, key, 0.001 * i, host_setup(key),
                            cost=float(host[key][0].nbf) ** 3,
                            make_system_device=(lambda k: (lambda: dev[k]))(key)))
    fps = sorted(footprint_bytes(ds.layout, ds.nocc) for ds, _, _ in host.values())
    srv = FockServer(budget_bytes=fps[-1] + fps[-2], slots=3, precision="split",
                     drop_host_tensor=False, device_setup=True)
    done = srv.run(reqs)
    srv.close()
    assert all(q.error is None for q in done), [q.error for q in done if q.error]
    routes = {q.key: q.route for q in done}
    assert "device" in routes.values()
    for key, route in routes.items():
        ds, P, C = (dev if route == "device" else host)[key]
        eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, precision="split")
        Js, Ks = eng.compute_jk(2.0 * P, C)
        eng.close()
        for q in done:
            if q.key == key:
                assert q.route == route
                assert np.array_equal(q.J, Js) and np.array_equal(q.K, Ks), (key, route)
