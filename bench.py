"""Benchmark: DF Fock builds (J + K) per second on one GB300.

Workload (default): n-C20H42, cc-pVDZ / cc-pVDZ-jkfit, atom blocks, Schwarz
1e-10 (nbf 490, naux 2366, nocc 81), 3-center tensor resident in HBM; one
step = one Fock build (DF-J + DF-MO-K) at the core-guess density.  The
tensor (3 GB) is larger than L2, so no extra flush runs between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|split]
  python bench.py --impl reference ...   # CPU restatement on the host cores

N > 1 (torchrun): replicas only; every rank builds on its own GPU, the time
is the max over ranks and the value the sum of builds/s.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Fock builds/s (DF-J + DF-K)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 Fock builds, about half a second "
                         "of device time; 10 for the other workloads and the reference arm)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="split", choices=["fp64", "split"])
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--alkane", type=int, default=20)
    ap.add_argument("--kmethod", default="dfmo")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scf", action="store_true")
    ap.add_argument("--no-dfao", action="store_true")
    ap.add_argument("--no-water", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the compact synthetic DF-K, C40H82 MP2 and serving blocks")
    ap.add_argument("--tune-reps", type=int, default=10,
                    help="timed builds per autotuner candidate (0: built-in launch rules)")
    ap.add_argument("--device-setup", action="store_true",
                    help="serving: add a set-up worker that computes the 3-center "
                         "integrals on the GPU")
    ap.add_argument("--workload", default="fock", choices=["fock", "serving", "synthetic", "mp2"])
    ap.add_argument("--mp2-alkane", type=int, default=40)
    ap.add_argument("--mp2-points", type=int, default=8)
    ap.add_argument("--syn-nbf", type=int, default=4000)
    ap.add_argument("--syn-naux", type=int, default=12000)
    ap.add_argument("--syn-nocc", type=int, default=600)
    ap.add_argument("--syn-batch", type=int, default=1000)
    ap.add_argument("--syn-fp64-full", action="store_true",
                    help="also one FP64 build at full size (minutes) for split vs FP64")
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--alkane-max", type=int, default=40)
    ap.add_argument("--water-max", type=int, default=32)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 200 if args.workload == "fock" and args.impl == "ours" else 10
    return args


def setup(nC):
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.molecule import molecule_from_angstrom
    s, x = geometry.alkane(nC)
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    t0 = time.perf_counter()
    ds = build_dfsystem(mol, eps=1e-10)
    tset = time.perf_counter() - t0
    Cocc = core_guess(ds, mol.nocc)
    P = Cocc @ Cocc.T
    return mol, ds, Cocc, P, tset


def workload_config(ds, mol, nC, precision, world):
    return {
        "workload": f"C{nC}H{2 * nC + 2} DF-HF Fock build, cc-pVDZ/cc-pVDZ-jkfit, atom blocks, "
                    f"Schwarz 1e-10",
        "nbf": ds.nbf, "naux": ds.naux, "nocc": mol.nocc, "nnz_B": ds.layout.nnz,
        "kept_block_pairs": round(ds.layout.kept_block_fraction(), 4),
        "precision": precision, "kmethod": "dfmo", "jmethod": "dfao",
        "l2_flush": "none: resident 3-center tensor (%.2f GB) exceeds L2" % (ds.layout.nnz * 8e-9),
        "launch": "whole build replayed as one CUDA graph",
        "parallelism": f"replicas x{world}",
    }


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx),
                                      "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.1)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def max_over_ranks(x, world, device=None):
    """Replicas: each rank times its own copy of the workload; the job's time
    is the slowest rank's (all-reduce MAX; NCCL on the GPUs, any backend the
    process group was started with)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_per_step, world):
    """Whole-job throughput of `world` replicas (builds/s over all ranks)."""
    return world * 1e3 / ms_per_step


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], d.get("bf16_tflops_sustained"), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


def core_guess(ds, nocc):
    """Core-guess orbitals: H diagonalised in the Loewdin basis."""
    sv, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(sv ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
    return np.ascontiguousarray((X @ Cp)[:, :nocc])


def run_water(dev, reps=2000):
    """Water DF-HF Fock build (cc-pVDZ / cc-pVDZ-jkfit; nbf 24, naux 116,
    nocc 5): launch-bound, so the latency of one build replayed as a CUDA
    graph is the figure, beside the host-buffer call, the CPU oracle and the
    FP64 path's agreement with the oracle."""
    import torch
    from chem_gb300 import geometry
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.fock import JKEngine, host_array
    from chem_gb300.molecule import molecule_from_angstrom
    from oracle.oracle import Oracle
    s, x = geometry.water()
    mol = molecule_from_angstrom(s, x, "cc-pvdz", "cc-pvdz-jkfit")
    ds = build_dfsystem(mol, eps=1e-10)
    C = core_guess(ds, mol.nocc)
    Pt = 2.0 * C @ C.T
    n = ds.nbf
    O = Oracle(ds.layout, ds.B)
    t0 = time.perf_counter()
    for _ in range(20):
        Jo = O.df_j(ds.Vinv, Pt, ds.eps)
        Ko = O.dfmo_k(np.tril(ds.Linv), C, ds.eps)
    cpu_us = (time.perf_counter() - t0) / 20 * 1e6
    res = {"workload": "H2O DF-HF Fock build, cc-pVDZ/cc-pVDZ-jkfit, atom blocks, Schwarz 1e-10",
           "nbf": n, "naux": ds.naux, "nocc": mol.nocc, "cpu_oracle_us": cpu_us,
           "cpu_oracle_threads": os.cpu_count()}
    for prec in ("fp64", "split"):
        eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, precision=prec)
        st = torch.cuda.ExternalStream(eng.stream, device=dev)
        dP = torch.from_numpy(Pt).to(dev)
        dC = torch.from_numpy(C).to(dev)
        dJ = torch.empty((n, n), dtype=torch.float64, device=dev)
        dK = torch.empty((n, n), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        eng.capture_graph(dP.data_ptr(), dC.data_ptr(), mol.nocc, dJ.data_ptr(), dK.data_ptr())
        for _ in range(20):
            eng.launch_graph()
        eng.synchronize()
        l0 = eng.kernel_launches
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            eng.launch_graph()
        e1.record(st)
        eng.synchronize()
        res[f"{prec}_graph_us"] = e0.elapsed_time(e1) / reps * 1e3
        res[f"{prec}_launches_per_build"] = (eng.kernel_launches - l0) // reps
        Ph, Ch = host_array((n, n)), host_array(C.shape)
        Ph[...], Ch[...] = Pt, C
        out = (host_array((n, n)), host_array((n, n)))
        for _ in range(20):
            eng.compute_jk(Ph, Ch, out=out)
        t0 = time.perf_counter()
        for _ in range(reps // 4):
            eng.compute_jk(Ph, Ch, out=out)
        res[f"{prec}_e2e_us"] = (time.perf_counter() - t0) / (reps // 4) * 1e6
        if prec == "fp64":
            res["fp64_max_abs_dJ_vs_oracle"] = float(np.abs(out[0] - Jo).max())
            res["fp64_max_abs_dK_vs_oracle"] = float(np.abs(out[1] - Ko).max())
        else:
            res["split_max_abs_dK_vs_oracle"] = float(np.abs(out[1] - Ko).max())
        eng.close()
    return res


def cpu_reference_build(ds, Cocc, P, kchunk, want=False):
    """One Fock build with the CPU oracle on all host threads: seconds, and
    with want=True also (J, K)."""
    from oracle.oracle import Oracle
    O = Oracle(ds.layout, ds.B)
    t0 = time.perf_counter()
    J = O.df_j(ds.Vinv, 2.0 * P, ds.eps)
    K = O.dfmo_k(np.tril(ds.Linv), Cocc, ds.eps, kchunk=kchunk)
    t = time.perf_counter() - t0
    return (t, J, K) if want else t


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mol, ds, Cocc, P, _ = setup(args.alkane)
    ncores = os.cpu_count()
    times = []
    for i in range(args.warmup + args.steps):
        t = cpu_reference_build(ds, Cocc, P, 0)
        if i >= args.warmup:
            times.append(t)
    tot = sum(times)
    val = len(times) / tot
    cfg = workload_config(ds, mol, args.alkane, "fp64", 1)
    print(json.dumps({
        "metric": METRIC, "value": val, "unit": "builds/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / len(times), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic molecule (seed-free alkane rule)",
        "config": cfg,
        "cpu_baseline": {"value": val, "unit": "builds/s", "cores": ncores, "kind": "port",
                         "sample": "full Fock build (DF-J + DF-MO-K) per step, C restatement, "
                                   f"OpenMP on {ncores} threads"},
        "e2e": {"value": val, "unit": "builds/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


def run_serving(args):
    """Continuous-batching serving run: Poisson arrivals of Fock-build
    requests over alkanes and water clusters (chem_gb300.serving)."""
    import torch
    from chem_gb300.serving import FockServer, latency_stats, poisson_requests
    torch.cuda.set_device(0)
    reqs = poisson_requests(args.requests, args.rate, seed=20261203,
                            alkane=(4, args.alkane_max), water=(2, args.water_max))
    t_start = time.perf_counter()

    def progress(done, total):
        if done % 32 == 0 or done == total:
            print(f"serving: {done}/{total} requests done at {time.perf_counter() - t_start:.1f} s",
                  file=sys.stderr, flush=True)

    srv = FockServer(budget_bytes=args.budget_gb * 1e9, slots=args.slots,
                     precision=args.precision, progress=progress,
                     device_setup=args.device_setup)
    t0 = time.perf_counter()
    with ClockSampler(0) as clk:
        done = srv.run(reqs)
    wall = time.perf_counter() - t0
    srv.close()
    ok = [q for q in done if q.error is None]
    svc = np.array([q.t_done - max(q.arrival, q.t_setup_done) for q in ok])
    t_first = min(q.t_admitted for q in ok)
    t_last = max(q.t_done for q in ok)
    return {
        "metric": "Fock builds/s (serving)", "value": len(ok) / (t_last - t_first),
        "unit": "builds/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 in/out; bf16 digit slices on tcgen05",
        "data": "synthetic molecules: alkanes and seeded water clusters",
        "config": {"workload": f"serving: {args.requests} requests, Poisson {args.rate}/s, "
                               f"alkanes C4..C{args.alkane_max}, (H2O)2..{args.water_max}, "
                               "cc-pVDZ/cc-pVDZ-jkfit", "budget_gb": args.budget_gb,
                   "slots": args.slots, "precision": args.precision,
                   "distinct_molecules": len(set(q.key for q in reqs)),
                   "setup": "host and device integral workers on one queue"
                            if args.device_setup else "host integrals"},
        "setup_routes": {r: len({q.key for q in done if q.route == r}) for r in ("host", "device")},
        "latency_arrival_to_result": latency_stats(ok),
        "latency_service": {"p50_s": float(np.percentile(svc, 50)),
                            "p99_s": float(np.percentile(svc, 99)),
                            "definition": "result time minus the later of arrival and "
                                          "the end of the molecule's host set-up"},
        "served": len(ok), "errors": len(done) - len(ok), "wall_s": wall,
        "peak_reserved_gb": srv.max_used / 1e9,
        "evictions": sum(1 for e in srv.log if e[0] == "evict"),
        "clocks": clk.summary(),
    }


def run_synthetic(args):
    """Synthetic pre-fitted block-sparse DF-K (chem_gb300.synthetic): the
    full-size tensor (153 GB FP64) is generated on the device and the split
    path streams the auxiliary index in batches; FP64 and the CPU oracle are
    compared on a reduced size of the same construction."""
    import torch
    from chem_gb300.fock import JKEngine, k_split_plan
    from chem_gb300.synthetic import occupied, synthetic_layout
    torch.cuda.set_device(0)
    nbf, naux, nocc = args.syn_nbf, args.syn_naux, args.syn_nocc
    layout, decay = synthetic_layout(nbf, naux)
    C = occupied(nbf, nocc)
    eng = JKEngine(layout, None, None, None, fitted=True, synthetic=(20261203, decay),
                   precision="split", aux_batch=args.syn_batch)
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", 0))
    dC = torch.from_numpy(C).cuda()
    dK = torch.empty((nbf, nbf), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for _ in range(max(1, args.warmup)):
        eng.compute_jk_dev(0, dC.data_ptr(), nocc, 0, dK.data_ptr())
    eng.synchronize()
    l0 = eng.kernel_launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            eng.compute_jk_dev(0, dC.data_ptr(), nocc, 0, dK.data_ptr())
        e1.record(stream)
        eng.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    K = dK.cpu().numpy()
    dev_gb = eng.device_bytes / 1e9
    eng.profile(True)
    eng.compute_jk_dev(0, dC.data_ptr(), nocc, 0, dK.data_ptr())
    eng.synchronize()
    prof = {k: v[0] for k, v in eng.profile_read().items() if v[1]}
    eng.close()
    full64 = None
    if args.syn_fp64_full:
        # the same tensor regenerated for an FP64 engine (auxiliary batches)
        e64 = JKEngine(layout, None, None, None, fitted=True, synthetic=(20261203, decay),
                       precision="fp64", aux_batch=args.syn_batch)
        s64 = torch.cuda.ExternalStream(e64.stream, device=torch.device("cuda", 0))
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(s64)
        e64.compute_jk_dev(0, dC.data_ptr(), nocc, 0, dK.data_ptr())
        f1.record(s64)
        e64.synchronize()
        t64f = f0.elapsed_time(f1) * 1e-3
        K64f = dK.cpu().numpy()
        full64 = {"fp64_gpu_s_per_build": t64f, "speedup_split": t64f / (ms * 1e-3),
                  "max_abs_dK_split_vs_fp64": float(np.abs(K - K64f).max()),
                  "max_abs_K": float(np.abs(K64f).max()),
                  "device_gb_fp64": e64.device_bytes / 1e9,
                  "note": "one FP64 build, pre-fitted tensor, exchange in auxiliary batches"}
        e64.close()
        del K64f
    hbm, bf16, _, src = peaks()
    f_ht = 15 * 2.0 * nocc * layout.nnz
    f_k = 15 * 1.0 * naux * nocc * nbf * (nbf + 1)
    # reduced size: split vs FP64 vs CPU oracle on the same construction
    rn, ra, ro = nbf // 5, naux // 5, nocc // 5
    rl, rdec = synthetic_layout(rn, ra)
    rC = occupied(rn, ro)
    e64 = JKEngine(rl, None, None, None, fitted=True, synthetic=(20261203, rdec))
    t0 = time.perf_counter()
    _, K64 = e64.compute_jk(None, rC)
    t64 = time.perf_counter() - t0
    B = e64.download_b()
    e64.close()
    es = JKEngine(rl, None, None, None, fitted=True, synthetic=(20261203, rdec), precision="split",
                  aux_batch=ra // 4)
    _, Ks = es.compute_jk(None, rC)
    es.close()
    from oracle.oracle import Oracle
    t0 = time.perf_counter()
    Kr = Oracle(rl, B).dfmo_k(None, rC, 0.0, kchunk=k_split_plan(rn, ra, ro)[1])
    tcpu = time.perf_counter() - t0
    return {
        "metric": "DF-K builds/s (synthetic block-sparse)", "value": 1e3 / ms, "unit": "builds/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 in/out; bf16 digit slices on tcgen05",
        "data": "seeded synthetic tensor generated on the device",
        "config": {"workload": "synthetic DF-K", "nbf": nbf, "naux": naux, "nocc": nocc,
                   "nnz_B": layout.nnz, "tensor_gb_fp64": layout.nnz * 8e-9,
                   "kept_fraction": layout.kept_block_fraction(), "decay_blocks": decay,
                   "aux_batch": args.syn_batch, "device_gb": dev_gb},
        "phases_ms": prof,
        "tensor_tflops": {"half_transform": f_ht / (prof.get("split_gemm_ht", 1e9) * 1e-3) / 1e12,
                          "exchange": f_k / (prof.get("split_gemm_k", 1e9) * 1e-3) / 1e12,
                          "peak_bf16": bf16, "peak_source": src},
        "K_symmetric_max_asym": float(np.abs(K - K.T).max()),
        "K_trace": float(np.trace(K)),
        "full_size_fp64": full64,
        "reduced": {"nbf": rn, "naux": ra, "nocc": ro, "max_abs_dK_split_vs_fp64":
                    float(np.abs(Ks - K64).max()), "max_abs_K": float(np.abs(K64).max()),
                    "fp64_gpu_s": t64, "fp64_bitwise_vs_oracle": bool(np.array_equal(K64, Kr)),
                    "cpu_oracle_s": tcpu, "cpu_cores": os.cpu_count()},
        "clocks": clk.summary(),
    }


def run_mp2(args):
    """SOS-AO-MP2 Laplace batch (ll_full Z builder, all quadrature points in
    one launch per contraction) on n-C40H82, cc-pVDZ/cc-pVDZ-ri, with random
    S-orthonormal orbitals and uniform orbital energies; split precision
    timed, FP64 GPU compared once, the CPU oracle timed on a sample."""
    import torch
    from chem_gb300 import geometry, mp2
    from chem_gb300.dfsystem import build_dfsystem
    from chem_gb300.fock import JKEngine
    from chem_gb300.molecule import molecule_from_angstrom
    torch.cuda.set_device(0)
    nC, npts = args.mp2_alkane, args.mp2_points
    t0 = time.perf_counter()
    sym, xyz = geometry.alkane(nC)
    mol = molecule_from_angstrom(sym, xyz, "cc-pvdz", "cc-pvdz-ri")
    ds = build_dfsystem(mol, eps=1e-10)
    t_ints = time.perf_counter() - t0
    Co, Cv, eo, ev = mp2.random_orbitals(ds.S, ds.nocc, seed=20261203)
    t0 = time.perf_counter()
    fac = mp2.laplace_factors(Co, Cv, eo, ev, ds.S, npts)
    t_fac = time.perf_counter() - t0
    ro = [a.shape[1] for a in fac.Lo]
    rv = [a.shape[1] for a in fac.Lv]
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, precision="split")
    stream = torch.cuda.ExternalStream(eng.stream, device=torch.device("cuda", 0))
    eng.mp2_set_factors(fac.Lo, fac.Lv)
    for _ in range(max(3, args.warmup)):
        eng.mp2_compute_dev()
    eng.mp2_read()
    l0 = eng.kernel_launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            eng.mp2_compute_dev()
        ev1.record(stream)
        e_split, _ = eng.mp2_read()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = (eng.kernel_launches - l0) / args.steps
    # end to end through the public call: host factors in, energies out
    te = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        e_e2e, _ = eng.mp2_laplace(fac.Lo, fac.Lv)
        te.append(time.perf_counter() - t1)
    hld, vld = max(ro) + (max(ro) & 1), max(rv) + (max(rv) & 1)
    h2d = 8 * npts * ds.nbf * (hld + vld)
    eng.profile(True)
    eng.mp2_compute_dev()
    eng.mp2_read()
    prof = {k: v[0] for k, v in eng.profile_read().items() if k.startswith("mp2") and v[1]}
    eng.profile(False)
    _, Zs = eng.mp2_read(want_z=True)
    dev_gb = eng.device_bytes / 1e9
    # FP64 GPU path, once
    if args.no_fp64_compare:
        e64, t64, dz, zmax = e_split, float("nan"), float("nan"), float(np.abs(Zs).max())
    else:
        eng.set_precision("fp64")
        t1 = time.perf_counter()
        e64, Z64 = eng.mp2_laplace(fac.Lo, fac.Lv, want_z=True)
        t64 = time.perf_counter() - t1
        dz = float(max(np.abs(Zs[t] - Z64[t]).max() for t in range(npts)))
        zmax = float(max(np.abs(Z64[t]).max() for t in range(npts)))
        del Z64
    eng.close()
    del Zs
    # algorithmic FLOPs per evaluation (FP64-equivalent products x 2)
    nnz, nbf, naux = ds.layout.nnz, ds.nbf, ds.naux
    f_t1 = sum(2.0 * r * nnz for r in ro)
    f_t2 = sum(2.0 * naux * r * nbf * v for r, v in zip(ro, rv))
    f_z = sum(1.0 * naux * (naux + 1) * r * v for r, v in zip(ro, rv))
    hbm, bf16, _, src = peaks()
    tf = {k: 15 * f / (prof[p] * 1e-3) / 1e12 for k, f, p in
          (("t1", f_t1, "mp2_t1"), ("t2", f_t2, "mp2_t2"), ("z", f_z, "mp2_z")) if p in prof}
    dom = max(("mp2_t1", "mp2_t2", "mp2_z"), key=lambda p: prof.get(p, 0.0))
    dom_tf = tf[{"mp2_t1": "t1", "mp2_t2": "t2", "mp2_z": "z"}[dom]]
    # CPU oracle on a sample: one point, the first nx auxiliary functions;
    # per point t(nx) = b nx + c nx^2 (transforms linear, Z quadratic in nx)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle.oracle import Oracle
        orc = Oracle(ds.layout, ds.B)
        ts = {}
        for nx in (256, 512):
            Bf = orc.prefit(np.tril(ds.Linv), nx=nx)
            t1 = time.perf_counter()
            orc.mp2_ll_point(Bf, fac.Lo[0], fac.Lv[0], nx=nx)
            ts[nx] = time.perf_counter() - t1
            del Bf
        c = (ts[512] / 512 - ts[256] / 256) / 256
        b = ts[256] / 256 - c * 256
        t_eval = npts * max(b * naux + c * naux * naux, ts[512] * naux / 512)
        cpu = {"value": 1.0 / t_eval, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"C oracle (ll_full Z builder, OpenMP), 1 point, first 256 and 512 of "
                         f"{naux} aux functions: {ts[256]:.2f} s, {ts[512]:.2f} s; full "
                         f"evaluation = {npts} x (b naux + c naux^2)"}
    return {
        "metric": f"SOS-MP2 Laplace evaluations/s ({npts} points)", "value": 1e3 / ms,
        "unit": "evals/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 in/out; bf16 digit slices on tcgen05",
        "data": "seed-free alkane geometry; random S-orthonormal orbitals, uniform orbital energies",
        "config": {"workload": f"SOS-AO-MP2 Laplace Z batch, C{nC}H{2 * nC + 2}, "
                               "cc-pVDZ/cc-pVDZ-ri, ll_full Z builder",
                   "nbf": nbf, "naux": naux, "nocc": ds.nocc, "points": npts,
                   "rank_occ": ro, "rank_vir": rv, "nnz_B": nnz, "device_gb": dev_gb,
                   "laplace_alpha": fac.alpha.tolist(), "laplace_omega": fac.omega.tolist(),
                   "laplace_max_err": fac.err, "inputs_vs_l2": "intermediates of 30+ GB per "
                   "contraction, far larger than L2"},
        "energy": {"split": float(e_split.sum()),
                   "fp64": None if args.no_fp64_compare else float(e64.sum()),
                   "abs_dE": None if args.no_fp64_compare else float(abs(e_split.sum() - e64.sum())),
                   "max_abs_de_point": None if args.no_fp64_compare else
                   float(np.abs(e_split - e64).max()),
                   "max_abs_dZ": None if args.no_fp64_compare else dz, "max_abs_Z": zmax,
                   "scaled_c_os_1.3": 1.3 * float(e_split.sum()),
                   "e2e_matches_device": bool(np.array_equal(e_e2e, e_split))},
        "fp64_gpu": None if args.no_fp64_compare else
        {"s_per_eval": t64, "speedup_split": t64 / (ms * 1e-3)},
        "phases_ms": prof,
        "tensor_tflops_bf16_pipe": tf,
        "roofline": {"bound": "tensor", "kernel": dom, "achieved": dom_tf, "peak": bf16,
                     "unit": "TFLOP/s", "frac": dom_tf / bf16, "traffic": None,
                     "peak_source": src, "note": "15 BF16 digit products per FP64-equivalent "
                     "product; achieved = 15 x algorithmic FLOPs of the phase / its CUDA-event time"},
        "e2e": {"value": len(te) / sum(te), "unit": "evals/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8 * npts},
        "cpu_baseline": cpu, "gpu_launches": launches,
        "setup_s": {"integrals": t_ints, "laplace_and_cholesky": t_fac},
        "clocks": clk.summary(),
    }


def other_configs(args):
    """Compact runs of the other configs, so that the default bench line
    records them; each is guarded, so a failure is recorded and the line
    still prints.  Synthetic DF-K at full size (nbf 4000, naux 12000, nocc
    600; split path, two timed builds; FP64 and the oracle at the reduced
    size); C40H82 SOS-MP2 with 8 Laplace points (split path, three timed
    evaluations; the FP64 comparison and the CPU sample are left to
    --workload mp2); serving on a 64-request sample of the serving
    workload's distribution with smaller molecules (C4..C12, (H2O)2..8)."""
    import copy
    res = {}
    runs = (
        ("synthetic_dfk", run_synthetic, dict(steps=2, warmup=1)),
        ("sos_mp2_c40h82", run_mp2, dict(steps=3, warmup=3, no_fp64_compare=True,
                                          no_cpu_baseline=True)),
        ("serving_sample", run_serving, dict(requests=64, rate=20.0, alkane_max=12,
                                             water_max=8, precision="split")),
    )
    for name, fn, kw in runs:
        a = copy.copy(args)
        for k, v in kw.items():
            setattr(a, k, v)
        t0 = time.perf_counter()
        try:
            r = fn(a)
            r["wall_s_block"] = round(time.perf_counter() - t0, 1)
            res[name] = r
        except Exception as e:  # recorded in the line, the bench goes on
            res[name] = {"error": str(e)[:300]}
    return res


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload in ("serving", "mp2", "synthetic"):
        run = {"serving": run_serving, "mp2": run_mp2, "synthetic": run_synthetic}[args.workload]
        print(json.dumps(run(args)), flush=True)
        return
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from chem_gb300 import accuracy
    from chem_gb300.fock import JKEngine, host_array, k_split_plan

    mol, ds, Cocc, P, tset = setup(args.alkane)
    eng = JKEngine(ds.layout, ds.B, np.tril(ds.Linv), ds.Vinv, eps=ds.eps, device=local,
                   precision=args.precision)
    dev = torch.device("cuda", local)
    dP = torch.from_numpy(2.0 * P).to(dev)
    dC = torch.from_numpy(Cocc).to(dev)
    n = ds.nbf
    dJ = torch.empty((n, n), dtype=torch.float64, device=dev)
    dK = torch.empty((n, n), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)

    # launch choices of this problem picked by the autotuner (timed here,
    # no cache file), then the whole Fock build (all launches, memsets) is
    # one CUDA graph
    tune = eng.autotune(2.0 * P, Cocc, args.kmethod, reps=args.tune_reps) if args.tune_reps \
        else {"chosen": "built-in rules", "best_ms": None, "candidates": []}
    eng.capture_graph(dP.data_ptr(), dC.data_ptr(), mol.nocc, dJ.data_ptr(), dK.data_ptr(),
                      args.kmethod)

    def step():
        eng.launch_graph()

    for _ in range(max(3, args.warmup)):
        step()
    eng.synchronize()

    # timed region: device-resident inputs, CUDA events on the engine stream
    launches0 = eng.kernel_launches
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        eng.synchronize()
    torch.cuda.synchronize()
    launches = eng.kernel_launches - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, dev)
    value = replica_value(ms, world)

    # per-phase device time (CUDA events around every launch), same builds
    # issued directly rather than through the graph
    eng.profile(True)
    for _ in range(args.steps):
        eng.compute_jk_dev(dP.data_ptr(), dC.data_ptr(), mol.nocc, dJ.data_ptr(), dK.data_ptr(),
                           args.kmethod)
    eng.synchronize()
    prof = eng.profile_read()
    eng.profile(False)

    # end to end through the public host API: H2D of P and C, D2H of J and
    # K, from and into page-locked host arrays (fock.host_array)
    Ph = host_array((ds.nbf, ds.nbf))
    Ph[...] = 2.0 * P
    Ch = host_array(Cocc.shape)
    Ch[...] = Cocc
    out = (host_array((ds.nbf, ds.nbf)), host_array((ds.nbf, ds.nbf)))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(max(3, args.warmup)):  # the first call captures its graph
        eng.compute_jk(Ph, Ch, args.kmethod, out=out)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        Jh, Kh = eng.compute_jk(Ph, Ch, args.kmethod, out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)

    # roofline of the dominant phase
    hbm, bf16, bf16s, src = peaks()
    top = max(prof.items(), key=lambda kv: kv[1][0])
    name, (tms, nl) = top
    per_launch_ms = tms / max(1, nl)
    nbf, naux, nocc, nnz = ds.nbf, ds.naux, mol.nocc, ds.layout.nnz
    pairs = 15  # BF16 digit-pair products per FP64 product (5 digits, s+t <= 4)
    flops64 = {
        "half_transform": 2.0 * nocc * nnz,
        "fit": 2.0 * naux * naux * nbf * nocc / 2.0,  # lower-triangular L^-1
        "k_gemm": 1.0 * naux * nocc * nbf * (nbf + 1),
        "split_gemm_ht": 2.0 * nocc * nnz,
        "split_gemm_k": 1.0 * naux * nocc * nbf * (nbf + 1),
    }
    roof = None
    if name.startswith("split_gemm"):
        f = pairs * flops64[name]
        ach = f / (per_launch_ms * 1e-3) / 1e12
        # DRAM bytes per launch of the half transform, read+write, from one
        # ncu capture of the same kernel on n-C14H30 / cc-pVDZ-jkfit
        # (1.757 GB read + 0.254 GB written for 1.66175e8 tensor elements),
        # scaled by the tensor elements of this workload
        traffic = 2.0115e9 / 1.66175e8 * nnz if name == "split_gemm_ht" else None
        tensor = {"achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                  "peak_source": f"{src} (MEASURED_PEAKS.json bf16_tflops, burst)",
                  "algorithmic_flops_per_launch": f,
                  "flops_definition": "15 BF16 digit-pair products x 2*M*N*K of the unpadded "
                                      "FP64 product (M*N*K = nocc*nnz(B) for the half "
                                      "transform)"}
        roof = {"kernel": "k_split_gemm (" + name + ")", "bound": "tensor", "achieved": ach,
                "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16, "traffic": traffic,
                "traffic_source": "ncu capture on C14H30 scaled by tensor elements",
                "peak_source": tensor["peak_source"], "algorithmic_flops_per_launch": f,
                "flops_definition": tensor["flops_definition"],
                "fp64_equivalent_tflops": flops64[name] / (per_launch_ms * 1e-3) / 1e12,
                "ms_per_launch": per_launch_ms}
        if name == "split_gemm_ht":
            # algorithmic bytes of one launch: the digit slices of L^-1 B
            # (five BF16 digits per tensor element, read once), H written
            # (five BF16 digits per element over auxiliary groups of 32 when
            # the digits are cut in the epilogue, else FP64), the density-row
            # partials (FP64), and the digit slices of C and of the density
            # rows per panel
            lay = ds.layout
            cdig = sum(10.0 * int(k) * (nocc + int(b)) for k, b in zip(lay.panel_K, lay.bsizes))
            if eng.get_split_fuse():
                hbytes = 10.0 * nbf * (-(-naux // 32) * 32) * nocc
            else:
                hbytes = 8.0 * nbf * naux * nocc
            byts = 10.0 * nnz + hbytes + 8.0 * nbf * naux + cdig
            ai, ridge = f / byts, bf16 * 1e12 / (hbm * 1e9)
            if ai < ridge:  # below the ridge point: HBM bounds the launch
                achb = byts / (per_launch_ms * 1e-3) / 1e9
                roof.update({"bound": "hbm", "achieved": achb, "peak": hbm, "unit": "GB/s",
                             "frac": achb / hbm, "peak_source": f"{src} (MEASURED_PEAKS.json "
                                                               "hbm_gbs)",
                             "algorithmic_bytes_per_launch": byts,
                             "bytes_definition": "10 B per tensor element (digit slices of "
                                                 "L^-1 B) + H written (10 B digits per "
                                                 "element, auxiliary index padded to 32; 8 B "
                                                 "FP64 unfused) + 8 B per density partial + "
                                                 "digit slices of C and the density rows",
                             "arithmetic_intensity_flop_per_byte": ai,
                             "ridge_flop_per_byte": ridge, "tensor_pipe": tensor})
    elif name in flops64:
        fp64_peak = 1250.0  # GB300 nominal FP64 (GFLOP/s), not in MEASURED_PEAKS.json
        ach = flops64[name] / (per_launch_ms * 1e-3) / 1e12
        roof = {"kernel": name, "bound": "fp64", "achieved": ach, "peak": fp64_peak / 1e3,
                "unit": "TFLOP/s", "frac": ach / (fp64_peak / 1e3), "traffic": None,
                "peak_source": "nominal FP64 1.25 TFLOP/s (MEASURED_PEAKS.json has no FP64 figure)",
                "algorithmic_flops_per_launch": flops64[name], "ms_per_launch": per_launch_ms}
    elif name in ("j_rowdot", "j_colsum"):
        # the mixed path's column sums read the 6-byte compact copy of L^-1 B
        byts = nnz * (6.0 if args.precision == "split" and name == "j_colsum" else 8.0)
        ach = byts / (per_launch_ms * 1e-3) / 1e9
        roof = {"kernel": name, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                "frac": ach / hbm, "traffic": None, "peak_source": src,
                "algorithmic_bytes_per_launch": byts, "ms_per_launch": per_launch_ms}

    # FP64 GPU path beside it: speed and accuracy deltas
    fp64 = None
    if args.precision == "split" and not args.no_fp64_compare:
        Jm, Km = eng.compute_jk(Ph, Cocc, args.kmethod)
        eng.set_precision("fp64")
        tune64 = eng.autotune(2.0 * P, Cocc, args.kmethod, reps=1) if args.tune_reps \
            else {"chosen": "built-in rules", "best_ms": None, "candidates": []}
        eng.compute_jk(Ph, Cocc, args.kmethod)
        nst = max(2, min(args.steps, 5))
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(nst):
            eng.compute_jk_dev(dP.data_ptr(), dC.data_ptr(), mol.nocc, dJ.data_ptr(),
                               dK.data_ptr(), args.kmethod)
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1) / nst
        Jf, Kf = eng.compute_jk(Ph, Cocc, args.kmethod)
        Jf, Kf = Jf.copy(), Kf.copy()
        eng.set_jmode("cholesky")
        Jfc, _ = eng.compute_jk(Ph, None, args.kmethod)
        eng.set_jmode("vinv")
        eng.set_precision(args.precision)
        # Coulomb energy of each route against the exactly refined solve of
        # V h = g (quadruple-precision residuals where numpy has them)
        cexact = None
        if accuracy.have_quad():
            g = accuracy.panel_g(ds.layout, ds.B, 2.0 * P)
            cr = accuracy.coulomb_routes(ds.V, ds.Linv, ds.Vinv, g, residual="quad")
            cexact = {"E_J_exact_Eh": cr["E_exact"],
                      "mixed": accuracy.j_energy_vs_exact(P, Jm, cr["E_exact"]),
                      "fp64_vinv_route": accuracy.j_energy_vs_exact(P, Jf, cr["E_exact"]),
                      "fp64_cholesky_route": accuracy.j_energy_vs_exact(P, Jfc, cr["E_exact"]),
                      "definition": "sum P_alpha J - 1/2 g^T V^-1 g, the exact solve by "
                                    "iterative refinement with quadruple-precision residuals"}
        fp64 = {"value": world * 1e3 / ms64, "unit": "builds/s", "ms_per_step": ms64,
                "autotune": {"chosen": tune64["chosen"], "best_ms": tune64["best_ms"],
                             "candidates": len(tune64["candidates"])},
                "steps": nst,
                "speedup_mixed_over_fp64": ms64 / ms,
                "max_abs_dK": float(np.abs(Km - Kf).max()),
                "max_abs_dJ": float(np.abs(Jm - Jf).max()),
                "dE_Eh": float(np.sum(P * ((Jm - Jf) + (Km - Kf)))),
                "dE_K_Eh": float(np.sum(P * (Km - Kf))),
                "max_abs_dJ_vs_fp64_cholesky": float(np.abs(Jm - Jfc).max()),
                "dE_vs_fp64_cholesky_Eh": float(np.sum(P * ((Jm - Jfc) + (Km - Kf)))),
                "coulomb_energy_vs_exact_Eh": cexact,
                "fp64_route_note": "fp64 J uses the explicit V^-1 of fock::DF_J; for this "
                                   "metric (cond ~2e7) that route itself errs by ~1e-6 Eh in "
                                   "the Coulomb energy, the Cholesky route by ~1e-10 Eh",
                "dE_definition": "sum P_alpha ((J + K)_mixed - (J + K)_fp64): energy change "
                                 "of one Fock build at the bench density (E = sum P_alpha "
                                 "(H + F), F = H + J + K)"}

    # DF-AO K (the reference example's K builder) at the same density: split
    # and FP64 build times, and agreement with DF-MO K of the same density
    dfao = None
    if args.precision == "split" and not args.no_dfao:
        Pa = np.ascontiguousarray(P)
        dPa = torch.from_numpy(Pa).to(dev)
        dKa = torch.empty((n, n), dtype=torch.float64, device=dev)
        res = {}
        for prec in ("split", "fp64"):
            eng.set_precision(prec)
            eng.compute_k_ao_dev(dPa.data_ptr(), dKa.data_ptr())  # plan, fitting, warm-up
            eng.synchronize()
            nst = 3 if prec == "fp64" else max(3, args.steps)
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            for _ in range(nst):
                eng.compute_k_ao_dev(dPa.data_ptr(), dKa.data_ptr())
            a1.record(stream)
            eng.synchronize()
            res[prec] = (a0.elapsed_time(a1) / nst, dKa.cpu().numpy())
        eng.set_precision("fp64")
        _, Kmo64 = eng.compute_jk(None, Cocc, "dfmo")
        eng.set_precision(args.precision)
        dfao = {"split_ms": res["split"][0], "fp64_ms": res["fp64"][0],
                "speedup": res["fp64"][0] / res["split"][0],
                "max_abs_dK_split_vs_fp64_dfmo": float(np.abs(res["split"][1] - Kmo64).max()),
                "max_abs_dK_fp64_dfao_vs_fp64_dfmo": float(np.abs(res["fp64"][1] - Kmo64).max()),
                "dE_K_split_vs_fp64_Eh": float(np.sum(P * (res["split"][1] - res["fp64"][1])))}

    # non-symmetric DF-LMO K (the ADC caller's left/right coefficients):
    # split and FP64 call times through the host-buffer entry point; a
    # failure here is recorded and does not stop the bench line
    asym = None
    if args.precision == "split" and not args.no_dfao:
        try:
            rng = np.random.default_rng(9)
            U = Cocc + 0.1 * rng.standard_normal(Cocc.shape)
            Vt = np.ascontiguousarray((Cocc + 0.1 * rng.standard_normal(Cocc.shape)).T)
            res, Ka = {}, {}
            for prec, nst in (("split", 10), ("fp64", 3)):
                eng.set_precision(prec)
                Ka[prec] = eng.compute_k_lmo_asym(U, Vt)  # plans and warm-up
                t0 = time.perf_counter()
                for _ in range(nst):
                    eng.compute_k_lmo_asym(U, Vt)
                res[prec + "_ms"] = (time.perf_counter() - t0) / nst * 1e3
            eng.set_precision(args.precision)
            asym = dict(res, speedup=res["fp64_ms"] / res["split_ms"],
                        max_abs_dK_split_vs_fp64=float(np.abs(Ka["split"] - Ka["fp64"]).max()),
                        max_abs_K=float(np.abs(Ka["fp64"]).max()),
                        timing="host wall clock per gbjk_compute_k_lmo_asym call "
                               "(host buffers in and out)")
        except Exception as e:  # recorded in the line, the bench goes on
            eng.set_precision(args.precision)
            asym = {"error": str(e)[:300]}

    # full DF-HF SCF (the config's SCF comparison): FP64 on the reference
    # route, FP64 on the Cholesky route, mixed precision switching to FP64
    # (Cholesky route) once the DIIS error is below 1e-5
    scf = None
    if not args.no_scf:
        from chem_gb300.scf import fp64_switch, run_rhf

        def jk(Pa, Ca):
            return eng.compute_jk(2.0 * Pa, Ca, args.kmethod)

        def run(prec, jmode, switch_route=None, audit=None, max_vecs=8):
            eng.set_precision(prec)
            eng.set_jmode(jmode)
            sw = fp64_switch(eng, switch_route) if switch_route else None
            t0 = time.perf_counter()
            r = run_rhf(ds.S, ds.Hcore, mol.nuclear_repulsion(), mol.nocc, jk, conv=1e-8,
                        switch=sw, audit=audit, max_vecs=max_vecs)
            return r, time.perf_counter() - t0

        def e_exact_metric(r):
            # energy of a converged state with J on the Cholesky route
            eng.set_precision("fp64")
            eng.set_jmode("cholesky")
            J, K = jk(r.P, r.C[:, :mol.nocc])
            return float(np.sum(r.P * (2 * ds.Hcore + J + K)) + mol.nuclear_repulsion())

        def rec(r, t, **kw):
            return dict({"E": r.energy, "iterations": r.iterations, "seconds": round(t, 2),
                         "converged": r.converged}, **kw)

        def audit(Pa, Ca, J, K):
            # every mixed build against an FP64 (Cholesky route) build at the
            # same density
            eng.set_precision("fp64")
            eng.set_jmode("cholesky")
            J64, K64 = jk(Pa, Ca)
            eng.set_precision("split")
            return (float(np.abs(K - K64).max()), float(np.sum(Pa * ((J - J64) + (K - K64)))))

        r_ref, t_ref = run("fp64", "vinv")
        r_chol, t_chol = run("fp64", "cholesky")
        r_mix, t_mix = run("split", "cholesky", "cholesky")
        r_mixv, t_mixv = run("split", "cholesky", "vinv")
        r_pure, t_pure = run("split", "cholesky")
        # the same mixed SCF with each iteration's device work in CUDA graphs
        from chem_gb300.scf import run_rhf_device
        eng.set_precision("split")
        eng.set_jmode("cholesky")
        run_rhf_device(eng, ds.S, ds.Hcore, mol.nuclear_repulsion(), mol.nocc, kmethod=args.kmethod,
                       conv=1e-8, max_iter=3)  # captures the graphs
        t0 = time.perf_counter()
        r_dev = run_rhf_device(eng, ds.S, ds.Hcore, mol.nuclear_repulsion(), mol.nocc,
                               kmethod=args.kmethod, conv=1e-8)
        t_dev = time.perf_counter() - t0
        eng.set_precision("split")
        eng.set_jmode("cholesky")
        t0 = time.perf_counter()
        r_devsw = run_rhf_device(eng, ds.S, ds.Hcore, mol.nuclear_repulsion(), mol.nocc,
                                 kmethod=args.kmethod, conv=1e-8,
                                 switch=fp64_switch(eng, "cholesky"))
        t_devsw = time.perf_counter() - t0
        r_aud, _ = run("split", "cholesky", audit=audit)
        r_ref6, t_ref6 = run("fp64", "vinv", max_vecs=6)
        ec = {"fp64_vinv_route": e_exact_metric(r_ref),
              "fp64_vinv_route_diis6": e_exact_metric(r_ref6),
              "mixed_then_fp64_vinv": e_exact_metric(r_mixv)}
        eng.set_precision(args.precision)
        eng.set_jmode("vinv")
        sw_note = "FP64 once the DIIS RMS error < 1e-5"
        scf = {"conv_rms": 1e-8,
               "fp64_vinv_route": rec(r_ref, t_ref),
               "fp64_cholesky_route": rec(r_chol, t_chol),
               "mixed_then_fp64_cholesky": rec(r_mix, t_mix, switch=sw_note + ", Cholesky route"),
               "mixed_then_fp64_vinv": rec(r_mixv, t_mixv, switch=sw_note + ", V^-1 route"),
               "mixed_only": rec(r_pure, t_pure),
               "mixed_only_device_graphs": rec(r_dev, t_dev, note="P = C C^T, Fock build, "
                                               "F = H + J + K, energy, FPS - SPF, RMS and DIIS "
                                               "overlaps in one CUDA graph; DIIS combination "
                                               "and X F X in a second; FP64 eigh on the host"),
               "mixed_then_fp64_cholesky_device_graphs": rec(r_devsw, t_devsw),
               "dE_mixed_only_device_vs_fp64_cholesky": r_dev.energy - r_chol.energy,
               "dE_mixed_only_vs_fp64_cholesky": r_pure.energy - r_chol.energy,
               "dE_mixed_then_fp64_cholesky_vs_fp64_cholesky": r_mix.energy - r_chol.energy,
               "dE_mixed_then_fp64_vinv_vs_fp64_vinv": r_mixv.energy - r_ref.energy,
               "dE_fp64_vinv_vs_cholesky": r_ref.energy - r_chol.energy,
               "fp64_vinv_route_diis6": rec(r_ref6, t_ref6),
               "vinv_route_restart_spread_Eh": r_ref6.energy - r_ref.energy,
               "vinv_route_states_exact_metric_E": ec,
               "vinv_route_note": "the V^-1 route's converged energy carries the explicit "
                                  "inverse's rounding noise, different for every SCF "
                                  "trajectory (see the restart spread); its converged "
                                  "states are compared by their exact-metric energies",
               "mixed_only_per_build_vs_fp64_cholesky": {
                   "max_abs_dK": [a[0] for a in r_aud.audit],
                   "dE_Eh": [a[1] for a in r_aud.audit],
                   "worst_max_abs_dK": max(a[0] for a in r_aud.audit),
                   "worst_abs_dE_Eh": max(abs(a[1]) for a in r_aud.audit)}}

    out = {
        "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 in/out; bf16 digit slices x5 on tcgen05, exact int64 recombination"
                 if args.precision == "split" else "f64",
        "data": "synthetic molecule (seed-free alkane rule), host-computed integrals",
        "config": dict(workload_config(ds, mol, args.alkane, args.precision, world),
                       h_digits="cut in the half-transform epilogue, exponent per (AO function, "
                                "32 auxiliary indices)" if eng.get_split_fuse()
                       else "separate pass over FP64 H, exponent per AO function"
                       if args.precision == "split" else None,
                       autotune={"chosen": tune["chosen"], "best_ms": tune["best_ms"],
                                 "candidates": [(c["effective"], round(c["ms"], 4))
                                                for c in tune["candidates"]]}),
        "e2e": {"value": world * 1e3 / e2e_ms, "unit": "builds/s",
                "h2d_bytes_per_step": int(Ph.nbytes + Ch.nbytes),
                "d2h_bytes_per_step": int(2 * n * n * 8), "host_memory": "page-locked"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "fp64_gpu": fp64,
        "dfao_k": dfao,
        "adc_asym_k": asym,
        "scf": scf,
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in prof.items() if v[1]},
        "clocks": clk.summary(),
        "setup_s": {"integrals_host": round(tset, 2)},
    }
    if rank == 0 and not args.no_water:
        out["water"] = run_water(dev)
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle sums the exchange in the k parts the FP64 device build
        # used (the autotuner's choice, or the built-in plan)
        kc = eng.get_tunables()["fp64_kchunk"] if fp64 is not None else \
            k_split_plan(nbf, naux, nocc)[1]
        tcpu, Jo, Ko = cpu_reference_build(ds, Cocc, P, kc, want=True)
        if fp64 is not None and args.kmethod == "dfmo":
            # the FP64 device path against the CPU oracle on the same inputs
            fp64["oracle_max_abs_dJ"] = float(np.abs(Jf - Jo).max())
            fp64["oracle_max_abs_dK"] = float(np.abs(Kf - Ko).max())
            fp64["bitwise_vs_oracle"] = bool(np.array_equal(Jf, Jo) and np.array_equal(Kf, Ko))
        out["cpu_baseline"] = {"value": 1.0 / tcpu, "unit": "builds/s", "cores": os.cpu_count(),
                               "kind": "port",
                               "sample": "one full Fock build (DF-J + DF-MO-K), C restatement, "
                                         f"OpenMP on {os.cpu_count()} threads"}
    eng.close()
    if rank == 0 and not args.no_configs:
        out["other_configs"] = other_configs(args)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
