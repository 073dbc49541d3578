"""Admission, eviction and accounting of the Fock-build server, with a fake
engine (no GPU): every admitted engine fits the HBM budget, idle engines
are evicted least-recently-used, and every request is served."""
import threading
import time

import numpy as np

from chem_gb300.layout import build_layout
from chem_gb300.serving import FockServer, Request, footprint_bytes


class _DS:
    def __init__(self, nbf, naux, nocc):
        bs = [nbf // 2, nbf - nbf // 2]
        self.layout = build_layout(bs, [naux], lambda I, J: np.ones(1, bool))
        self.nocc = nocc
        self.eps = 0.0


class _FakeEngine:
    live = 0
    peak = 0
    lock = threading.Lock()

    def __init__(self, ds):
        self.n = ds.layout.nbf
        with _FakeEngine.lock:
            _FakeEngine.live += 1
            _FakeEngine.peak = max(_FakeEngine.peak, _FakeEngine.live)

    def compute_jk(self, P, C):
        time.sleep(0.002)
        return P * 0 + 1.0, P * 0 - 1.0

    def close(self):
        with _FakeEngine.lock:
            _FakeEngine.live -= 1


def test_admission_and_eviction():
    sizes = {"a": (40, 200, 5), "b": (60, 300, 7), "c": (80, 400, 9)}
    systems = {k: (_DS(*v), np.eye(v[0]), np.ones((v[0], v[2]))) for k, v in sizes.items()}
    fps = {k: footprint_bytes(s[0].layout, s[0].nocc) for k, s in systems.items()}
    budget = fps["c"] + fps["b"]  # never all three at once
    srv = FockServer(budget_bytes=budget, slots=3, engine_factory=_FakeEngine)
    reqs = []
    for i in range(30):
        key = "abc"[i % 3]
        reqs.append(Request(i, key, 0.001 * i, lambda k=key: systems[k]))
    done = srv.run(reqs, realtime=True)
    srv.close()
    assert all(q.error is None for q in done)
    assert all(np.all(q.J == 1.0) and np.all(q.K == -1.0) for q in done)
    assert srv.max_used <= budget
    assert _FakeEngine.peak <= 2
    assert any(e[0] == "evict" for e in srv.log)
    assert all(q.latency is not None and q.latency >= 0 for q in done)


def test_oversized_request_is_an_error_not_a_hang():
    ds = _DS(40, 200, 5)
    srv = FockServer(budget_bytes=1000, slots=1, engine_factory=_FakeEngine)
    done = srv.run([Request(0, "x", 0.0, lambda: (ds, np.eye(40), np.ones((40, 5))))])
    srv.close()
    assert done[0].error and "budget" in done[0].error


def test_requests_of_a_resident_molecule_are_served_together():
    # budget for one molecule at a time; requests alternate a, b, a, b, ...
    # and all arrive before any set-up ends: each molecule is admitted once
    sizes = {"a": (40, 200, 5), "b": (44, 220, 5)}
    systems = {k: (_DS(*v), np.eye(v[0]), np.ones((v[0], v[2]))) for k, v in sizes.items()}
    need = max(footprint_bytes(s[0].layout, s[0].nocc) for s in systems.values())

    def slow(k):
        time.sleep(0.05)
        return systems[k]

    srv = FockServer(budget_bytes=need, slots=2, engine_factory=_FakeEngine)
    reqs = [Request(i, "ab"[i % 2], 0.0, lambda k="ab"[i % 2]: slow(k)) for i in range(12)]
    done = srv.run(reqs, realtime=False)
    srv.close()
    assert all(q.error is None for q in done)
    admits = [e for e in srv.log if e[0] == "admit"]
    assert len(admits) == 2, srv.log
    assert srv.max_used <= need


def test_no_double_admission_with_many_slots():
    ds = _DS(40, 200, 5)
    created = []

    def factory(d):
        created.append(1)
        return _FakeEngine(d)

    srv = FockServer(budget_bytes=10 * footprint_bytes(ds.layout, ds.nocc), slots=4,
                     engine_factory=factory)
    reqs = [Request(i, "x", 0.0, lambda: (ds, np.eye(40), np.ones((40, 5)))) for i in range(16)]
    done = srv.run(reqs, realtime=False)
    srv.close()
    assert all(q.error is None for q in done)
    assert len(created) == 1


def test_setup_runs_shortest_job_first_and_failures_do_not_hang():
    order = []
    ds = _DS(40, 200, 5)

    def make(key, delay=0.02):
        def f():
            time.sleep(delay)
            order.append(key)
            if key == "bad":
                raise ValueError("no basis")
            return ds, np.eye(40), np.ones((40, 5))
        return f

    srv = FockServer(budget_bytes=10 * footprint_bytes(ds.layout, ds.nocc), slots=2,
                     engine_factory=_FakeEngine)
    reqs = [Request(0, "first", 0.0, make("first", 0.2), cost=0.5),
            Request(1, "big", 0.0, make("big"), cost=9.0),
            Request(2, "bad", 0.0, make("bad"), cost=1.0),
            Request(3, "small", 0.0, make("small"), cost=2.0),
            Request(4, "small", 0.0, make("small"), cost=2.0)]
    done = srv.run(reqs, realtime=False)
    srv.close()
    # cheapest first, whatever the pipeline had queued when it started
    assert order == ["first", "bad", "small", "big"]
    assert done[2].error and "set-up failed" in done[2].error
    assert all(q.error is None for q in done if q.key != "bad")
    assert all(q.t_done is not None for q in done)


def test_device_setup_worker_shares_the_queue():
    # two set-up workers (host integrals, device integrals) drain one queue;
    # each molecule keeps the route it was set up by, also when its engine
    # is evicted and admitted again
    created = []

    def factory(ds):
        created.append((ds.key, ds.B))
        return _FakeEngine(ds)

    def make(key, n, device):
        def f():
            time.sleep(0.02)
            d = _DS(n, 200, 5)
            d.key = key
            d.B = ("device_ints", key) if device else np.zeros(4)
            return d, np.eye(n), np.ones((n, 5))
        return f

    sizes = {f"m{i}": 40 + 2 * i for i in range(8)}
    fp = max(footprint_bytes(_DS(n, 200, 5).layout, 5) for n in sizes.values())
    reqs = []
    for i in range(32):
        key = f"m{i % 8}"
        n = sizes[key]
        reqs.append(Request(i, key, 0.0, make(key, n, False), cost=float(n),
                            make_system_device=make(key, n, True)))
    srv = FockServer(budget_bytes=3 * fp, slots=2, engine_factory=factory, device_setup=True,
                     drop_host_tensor=True)
    done = srv.run(reqs, realtime=False)
    srv.close()
    assert all(q.error is None for q in done), [q.error for q in done if q.error]
    routes = {}
    for q in done:
        assert q.route in ("host", "device")
        assert routes.setdefault(q.key, q.route) == q.route
    assert set(routes.values()) == {"host", "device"}
    assert srv.max_used <= 3 * fp
    assert any(e[0] == "evict" for e in srv.log)
    for key, B in created:
        assert isinstance(B, tuple) == (routes[key] == "device"), (key, B)


def test_true_up_charges_measured_bytes_both_ways():
    """After an engine's first build its reservation becomes its measured
    device bytes (plus 2 % and 16 MiB): an estimate that was too high is
    released, one that was too low is charged in full."""
    from chem_gb300.serving import _Resident

    class _Eng:
        def __init__(self, nbytes):
            self.device_bytes = nbytes

    srv = FockServer(budget_bytes=1 << 40, slots=1, engine_factory=_FakeEngine)
    for est, actual in ((10 << 30, 4 << 30), (4 << 30, 9 << 30)):
        r = _Resident(_Eng(actual), est)
        srv._used = est
        srv._true_up(r)
        want = int(actual * 1.02) + (16 << 20)
        assert r.nbytes == want and srv._used == want and r.measured
    srv.close()
