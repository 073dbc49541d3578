"""Continuous-batching Fock-build server on one GPU.

A request asks for the Fock-build contractions (J, K) of one molecule at one
density.  The server keeps every admitted molecule resident on the device as
a J/K engine (its 3-center tensor, metric factors, digit slices and
workspaces) and serves requests as they arrive:

* set-up — the host integrals of a molecule not seen before run on a CPU
  pipeline (one job at a time, each using all host threads), shortest
  estimated job first (a request's `cost` hint; arrival order without one),
  except that a job waiting longer than `max_setup_wait` goes first; with
  `device_setup`, a second worker takes jobs from the same queue and sets
  its molecule up with the 3-center integrals computed on the GPU
  (gbjk_upload_b_eri3c) while it admits the engine, so host and device
  integrals run side by side (the route taken is recorded on the request);
* admission — a molecule's engine is created when its device footprint fits
  the HBM budget; idle engines are evicted to make room, first those with
  no requests waiting (least-recently-used first), then any idle one;
* scheduling — a free GPU slot takes the earliest waiting request whose
  molecule is resident and idle, else the earliest request of a molecule
  that is neither resident nor being admitted; so the requests of a
  resident molecule are served together before it is evicted;
* execution — GPU slots are host threads, each issuing builds on its own
  engine's CUDA stream; a molecule's builds are serialised on its engine.
  Builds of different molecules are in flight together, but the split
  GEMMs of a large molecule take every SM (one CTA per SM, 216 KB of shared
  memory), so they run one after another; the streams overlap only the
  small kernels, copies and host work around them.
Every build runs the same deterministic kernels whatever else is in flight,
so a result in the mix is bit-identical to the same request served alone.

megalochem has no serving layer; its SCF loop calls the builders in-process
(src/hf/hfscf.cpp:241-259).  This module is the multi-request caller of the
same boundary.
"""
from __future__ import annotations

import bisect
import threading
import time
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    key: str             # molecule identity
    arrival: float       # seconds after the start of the run
    make_system: object  # callable() -> (DFSystem, P_alpha, C_occ)
    cost: float = None   # relative set-up cost estimate (shortest job first)
    # callable() -> the same without the host 3-center tensor (B left to the
    # device engine); used by the device set-up worker
    make_system_device: object = None
    route: str = None    # "host" or "device": how the molecule was set up
    t_setup_done: float = None
    t_admitted: float = None
    t_done: float = None
    J: np.ndarray = None
    K: np.ndarray = None
    error: str = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def footprint_bytes(layout, nocc, precision="split"):
    """Device bytes a J/K engine will hold for this molecule (estimate used
    for admission; the engine's own gbjk_device_bytes is recorded after)."""
    nnz, nbf, naux = layout.nnz, layout.nbf, layout.naux
    b = 8 * nnz + 2 * 8 * naux * naux           # B, L^-1, V^-1
    b += 8 * (nbf * nbf * 4 + nbf * naux)       # P, J, K, partials
    if precision == "split":
        b += 8 * nnz + 11 * nnz                 # L^-1 B (FP64) + digit slices (padded)
        b += 6.1 * nnz                          # J's compact copy (6 B, rows padded)
        b += 8 * nbf * naux * (nocc + 1)        # fitted half transform
        b += 11 * nbf * naux * (nocc + 1)       # its digits
        b += 8 * nbf * nbf * 64                 # split-K partials (upper bound)
    else:
        b += 2 * 8 * nbf * naux * nocc + 8 * nbf * nbf * 64
    return int(b * 1.05) + (64 << 20)


class _Resident:
    def __init__(self, engine, nbytes):
        self.engine = engine
        self.nbytes = nbytes
        self.lock = threading.Lock()
        self.busy = 0
        self.measured = False


class FockServer:
    """Serves Request objects; see the module docstring."""

    def __init__(self, budget_bytes=150e9, slots=4, precision="split", device=0,
                 engine_factory=None, clock=time.perf_counter, drop_host_tensor=True,
                 max_host_bytes=48e9, progress=None, max_setup_wait=60.0,
                 device_setup=False):
        self.budget = int(budget_bytes)
        self.device_setup = device_setup
        self._routes = {}                # key -> "host" | "device"
        self.drop_host_tensor = drop_host_tensor
        self.max_host_bytes = int(max_host_bytes)
        self.progress = progress  # callable(done, total) after each request
        self.max_setup_wait = max_setup_wait
        self._host_pending = 0
        self._host_bytes = {}
        self.slots = slots
        self.precision = precision
        self.device = device
        self.clock = clock
        self._engine_factory = engine_factory or self._make_engine
        self._cv = threading.Condition()
        self._resident = OrderedDict()   # key -> _Resident (LRU order)
        self._used = 0
        self._systems = {}               # key -> (ds, P, C) once set up
        self._setup_waiters = {}         # key -> requests waiting for its set-up
        self._setup_jobs = []            # (request, submit time) of pending set-ups
        self._setup_done = set()         # keys set up (or failed)
        self._submitted_all = False
        self._ready = []                 # sorted list of (arrival, rid, request)
        self._waiting = {}               # key -> requests submitted, not yet taken
        self._admitting = set()          # keys whose engine a slot is creating
        self._taken = 0
        self.max_used = 0
        self.builds = 0
        self.log = []

    # -- engines -------------------------------------------------------------
    def _make_engine(self, ds):
        from .fock import JKEngine
        return JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps,
                        device=self.device, precision=self.precision)

    def _evict_for(self, need):
        """Evict idle engines until `need` bytes fit; caller holds _cv.  First
        pass: molecules with no waiting request (LRU first); second pass: any
        idle molecule (LRU first)."""
        for any_idle in (False, True):
            for key in list(self._resident.keys()):
                if self._used + need <= self.budget:
                    return True
                r = self._resident[key]
                if r.busy or (not any_idle and self._waiting.get(key, 0) > 0):
                    continue
                del self._resident[key]
                self._used -= r.nbytes
                r.engine.close()
                self.log.append(("evict", key))
        return self._used + need <= self.budget

    def _take(self):
        """Next request for a free slot (caller holds _cv): (request, resident
        engine reserved for it, or None when the slot must admit it)."""
        for i, (_, _, q) in enumerate(self._ready):
            r = self._resident.get(q.key)
            if r is not None and r.busy == 0:
                del self._ready[i]
                r.busy += 1
                self._resident.move_to_end(q.key)
                self._waiting[q.key] -= 1
                self._taken += 1
                return q, r
        for i, (_, _, q) in enumerate(self._ready):
            if q.key not in self._resident and q.key not in self._admitting:
                del self._ready[i]
                self._admitting.add(q.key)
                self._waiting[q.key] -= 1
                self._taken += 1
                return q, None
        return None, None

    def _acquire(self, req):
        """Admit the request's molecule (its key is in _admitting): block until
        its footprint fits, then create the engine, reserved for the request."""
        try:
            return self._admit(req)
        finally:
            with self._cv:
                self._admitting.discard(req.key)
                self._cv.notify_all()

    def _admit(self, req):
        ds, _, _ = self._systems[req.key]
        need = footprint_bytes(ds.layout, ds.nocc, self.precision)
        if need > self.budget:
            raise RuntimeError(f"molecule {req.key} needs {need / 1e9:.1f} GB > budget")
        with self._cv:
            while True:
                if self._evict_for(need):
                    self._used += need
                    self.max_used = max(self.max_used, self._used)
                    break
                self._cv.wait()
        try:
            return self._create(req, need)
        except BaseException:
            with self._cv:
                self._used -= need
                self._cv.notify_all()
            raise

    def _create(self, req, need):
        ds = self._systems[req.key][0]
        if getattr(ds, "B", 1) is None:
            # the host copy was dropped when an earlier engine took it: set
            # the molecule up again (only after an eviction)
            self._systems[req.key] = req.make_system()
            ds = self._systems[req.key][0]
            with self._cv:
                self._host_bytes[req.key] = int(ds.B.nbytes)
                self._host_pending += int(ds.B.nbytes)
        eng = self._engine_factory(ds)
        if self.drop_host_tensor and isinstance(getattr(ds, "B", None), np.ndarray):
            ds.B = None  # the engine holds the device copy
            with self._cv:
                self._host_pending -= self._host_bytes.pop(req.key, 0)
                self._cv.notify_all()
        r = _Resident(eng, need)
        r.busy = 1
        with self._cv:
            self._resident[req.key] = r
            self.log.append(("admit", req.key))
            self._cv.notify_all()
        return r

    def _true_up(self, r):
        """After an engine's first build (all its buffers allocated), replace
        the admission estimate by its measured device bytes, in either
        direction (an estimate that was too low is charged in full)."""
        r.measured = True
        actual = getattr(r.engine, "device_bytes", None)
        if actual is None:
            return
        actual = int(actual * 1.02) + (16 << 20)
        if actual != r.nbytes:
            with self._cv:
                self._used += actual - r.nbytes
                self.max_used = max(self.max_used, self._used)
                r.nbytes = actual
                self._cv.notify_all()

    def _release(self, r):
        with self._cv:
            r.busy -= 1
            self._cv.notify_all()

    # -- request flow ----------------------------------------------------------
    def _setup(self, req):
        # back-pressure: the set-up pipeline pauses while the host tensors of
        # molecules set up but not yet resident exceed max_host_bytes
        with self._cv:
            while self._host_pending > self.max_host_bytes:
                self._cv.wait(0.1)
        if req.key not in self._systems:
            sysm = req.make_system()
            nb = int(getattr(getattr(sysm[0], "B", None), "nbytes", 0) or 0)
            with self._cv:
                self._systems[req.key] = sysm
                self._host_pending += nb
                self._host_bytes[req.key] = nb

    def _setup_device(self, req):
        """Device route: the host part of the set-up (screening, metric) on
        this thread, then admission of the molecule's engine, whose
        3-center tensor the GPU computes; the engine becomes resident and
        idle, ready for the molecule's requests."""
        if req.key not in self._systems:
            sysm = req.make_system_device()
            with self._cv:
                self._systems[req.key] = sysm
        ds = self._systems[req.key][0]
        need = footprint_bytes(ds.layout, ds.nocc, self.precision)
        if need > self.budget:
            raise RuntimeError(f"molecule {req.key} needs {need / 1e9:.1f} GB > budget")
        with self._cv:
            self._admitting.add(req.key)
            while not self._evict_for(need):
                self._cv.wait()
            self._used += need
            self.max_used = max(self.max_used, self._used)
        try:
            eng = self._engine_factory(ds)
        except BaseException:
            with self._cv:
                self._used -= need
                self._admitting.discard(req.key)
                self._cv.notify_all()
            raise
        with self._cv:
            self._resident[req.key] = _Resident(eng, need)
            self._admitting.discard(req.key)
            self.log.append(("admit", req.key))
            self._cv.notify_all()

    def _on_setup(self, req, t0):
        req.t_setup_done = self.clock() - t0
        with self._cv:
            bisect.insort(self._ready, (req.arrival, req.rid, req), key=lambda e: (e[0], e[1]))
            self._cv.notify_all()

    def _worker(self, t0, total):
        while True:
            with self._cv:
                while True:
                    req, r = self._take()
                    if req is not None or self._taken >= total:
                        break
                    self._cv.wait(0.05)
            if req is None:
                return
            try:
                if r is None:
                    r = self._acquire(req)
                try:
                    req.t_admitted = self.clock() - t0
                    ds, P, C = self._systems[req.key]
                    with r.lock:   # one build at a time per engine (its stream)
                        req.J, req.K = r.engine.compute_jk(2.0 * P, C)
                        if not r.measured:
                            self._true_up(r)
                finally:
                    self._release(r)
            except Exception as e:  # recorded, the server keeps serving
                req.error = str(e)
            req.t_done = self.clock() - t0
            with self._cv:
                self._done += 1
                self.builds += req.error is None
                done = self._done
                self._cv.notify_all()
            if self.progress:
                self.progress(done, total)

    def _next_setup(self, now):
        """Pick the next set-up job (caller holds _cv): the oldest one if it
        has waited longer than max_setup_wait, else the cheapest."""
        jobs = self._setup_jobs
        i_old = min(range(len(jobs)), key=lambda i: jobs[i][1])
        if now - jobs[i_old][1] > self.max_setup_wait:
            return jobs.pop(i_old)[0]
        i = min(range(len(jobs)), key=lambda i: (jobs[i][0].cost if jobs[i][0].cost is not None
                                                 else 0.0, jobs[i][1]))
        return jobs.pop(i)[0]

    def _setup_loop(self, t0, total, route="host"):
        while True:
            with self._cv:
                while not self._setup_jobs and not self._submitted_all:
                    self._cv.wait(0.05)
                if not self._setup_jobs:
                    return
                req = self._next_setup(self.clock())
            how = "device" if route == "device" and req.make_system_device is not None else "host"
            with self._cv:
                self._routes[req.key] = how
            err = None
            try:
                if how == "device":
                    self._setup_device(req)
                else:
                    self._setup(req)
            except Exception as e:  # recorded on every request of the molecule
                err = f"set-up failed: {e}"
            with self._cv:
                self._setup_done.add(req.key)
                waiters = self._setup_waiters.pop(req.key, [])
            for q in waiters:
                q.route = how
                if err is None:
                    self._on_setup(q, t0)
                else:
                    self._fail(q, err, t0, total)

    def _fail(self, req, err, t0, total):
        req.error = err
        req.t_done = self.clock() - t0
        with self._cv:
            self._waiting[req.key] -= 1
            self._taken += 1
            self._done += 1
            done = self._done
            self._cv.notify_all()
        if self.progress:
            self.progress(done, total)

    def _submit(self, req, t0, total):
        with self._cv:
            if req.key in self._setup_done:
                ok = req.key in self._systems
            else:
                first = req.key not in self._setup_waiters
                self._setup_waiters.setdefault(req.key, []).append(req)
                if first:
                    self._setup_jobs.append((req, self.clock()))
                    self._cv.notify_all()
                return
        req.route = self._routes.get(req.key)
        if ok:
            self._on_setup(req, t0)
        else:
            self._fail(req, "set-up failed earlier", t0, total)

    def run(self, requests, realtime=True):
        """Serve `requests` (arrival times relative to now); returns them."""
        reqs = sorted(requests, key=lambda q: q.arrival)
        self._done = 0
        self._taken = 0
        self._submitted_all = False
        for q in reqs:
            self._waiting[q.key] = self._waiting.get(q.key, 0) + 1
        t0 = self.clock()
        workers = [threading.Thread(target=self._worker, args=(t0, len(reqs)), daemon=True)
                   for _ in range(self.slots)]
        setups = [threading.Thread(target=self._setup_loop, args=(t0, len(reqs)), daemon=True)]
        if self.device_setup:
            setups.append(threading.Thread(target=self._setup_loop,
                                           args=(t0, len(reqs), "device"), daemon=True))
        for w in workers + setups:
            w.start()
        for req in reqs:
            if realtime:
                delay = req.arrival - (self.clock() - t0)
                if delay > 0:
                    time.sleep(delay)
            self._submit(req, t0, len(reqs))
        with self._cv:
            self._submitted_all = True
            self._cv.notify_all()
        for w in setups + workers:
            w.join()
        return reqs

    def close(self):
        with self._cv:
            for r in self._resident.values():
                r.engine.close()
            self._resident.clear()
            self._used = 0


def latency_stats(requests):
    lat = np.array([q.latency for q in requests if q.error is None])
    if lat.size == 0:
        return {}
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max()), "n": int(lat.size)}


def make_system_factory(kind, size, eps=1e-10, basis="cc-pvdz", dfbasis="cc-pvdz-jkfit",
                        device_ints=False):
    """Callable building (DFSystem, P_alpha, C_occ) for an alkane C_nH_{2n+2}
    (kind 'alkane', size n) or a water cluster (kind 'water', size k) at the
    core-guess density.  Water-cluster geometries are seeded by k, so
    requests of one cluster size share the molecule (and its set-up).  With
    device_ints the 3-center tensor is left to the device engine."""
    def make():
        from . import geometry
        from .dfsystem import build_dfsystem
        from .molecule import molecule_from_angstrom
        if kind == "alkane":
            s, x = geometry.alkane(size)
        else:
            s, x = geometry.water_cluster(size, np.random.default_rng(1000 + size))
        ds = build_dfsystem(molecule_from_angstrom(s, x, basis, dfbasis), eps=eps,
                            device_ints=device_ints)
        sv, U = np.linalg.eigh(ds.S)
        X = U @ np.diag(sv ** -0.5) @ U.T
        _, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
        C = np.ascontiguousarray((X @ Cp)[:, :ds.nocc])
        return ds, C @ C.T, C
    return make


def poisson_requests(n, rate, seed, alkane=(4, 40), water=(2, 32)):
    """n requests with exponential inter-arrival times (rate per second);
    each is an alkane C_nH_{2n+2} (n uniform in `alkane`) or a water
    cluster (k uniform in `water`), half and half."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        if rng.random() < 0.5:
            size = int(rng.integers(alkane[0], alkane[1] + 1))
            kind = "alkane"
        else:
            size = int(rng.integers(water[0], water[1] + 1))
            kind = "water"
        # set-up cost grows ~ nbf^3 (3-center integrals with screening)
        nbf = 24 * size + 10 if kind == "alkane" else 24 * size
        out.append(Request(rid, f"{kind}{size}", t, make_system_factory(kind, size),
                           cost=float(nbf) ** 3,
                           make_system_device=make_system_factory(kind, size, device_ints=True)))
    return out
