"""Benchmark: 3D Crank-Nicolson steps/s at a 1e-10 FP64 residual on one GB300.

Workload: the 3D heterostructure (160 x 160 x 320 elements, degree 3, five C0
interfaces along z, N = 8 847 477 coefficients), field along z, dt = 0.5 a.u.,
synthetic data (tdsez_gb300.workloads.heterostructure). One step = one CN
stage solve (M + i dt/2 H_E) X = M psi to ||b - A X|| <= 1e-10 ||b|| in FP64
(FGMRES) plus psi <- 2X - psi.

Arms (same workload, same stopping rule):
  value      FP64 FGMRES with double-float applies, FP32 fast-diagonalisation
             preconditioner (--pc fdm, default), initial guess x0 = P^-1 b
  mixed_mg   FP64 FGMRES, FP32 geometric B-spline multigrid (mixed_mg_exact_coarse:
             the same with the coarsest level solved by its exact FDM inverse)
  plain_mg   the plain GPU multigrid form: the same multigrid in FP64
e2e: the same steps through the C ABI with the state in pinned host memory,
copied host->device before and device->host after every step.
cpu_baseline / --impl reference: the reference's GMRES(30) + ILU(0) CPU
method restated in C (oracle/cn_bjilu.c, OpenMP over the host cores) on a
reduced grid, scaled by the coefficient count.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D CN steps/sec at 1e-10 residual: learned+mixed vs plain GPU MG, one GB300"
UNIT = "steps/s"
RTOL = 1e-10


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_init():
    """Replicas: one process per GPU (torchrun env), NCCL on GPUs, gloo without."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_kernel(fn, reps, stream):
    """Average duration (s) of fn() launched reps times, CUDA events on stream."""
    import torch
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    s.record(stream)
    for _ in range(reps):
        fn()
    e.record(stream)
    torch.cuda.synchronize()
    return s.elapsed_time(e) / 1e3 / reps


def batch_scan(args):
    """Intensity / carrier-envelope-phase scan of independent 2D soft-core
    runs (V = -1/sqrt(x^2 + y^2 + 1) on [-100, 100]^2, field along x, CN
    dt = 0.05): grids and degrees drawn per run with the seeded generator,
    E0 log-uniform in [0.01, 0.1], CEP uniform in [0, 2 pi). The runs are
    stepped one after another, then together (BatchPropagator: own streams,
    host thread pool); reported as run-steps per second."""
    import math as _m
    import numpy as np
    import torch
    from tdsez_gb300 import _lib
    from tdsez_gb300.operators import Operator, Physics
    from tdsez_gb300.propagator import BatchPropagator, Propagator
    from tdsez_gb300.space import Space, uniform_knots
    torch.cuda.set_device(0)
    _lib.load()
    rng = np.random.default_rng(20261203)
    T = 4 * 2 * _m.pi / 0.057
    runs = []
    for r in range(args.batch_scan):
        nel = int(rng.integers(args.scan_min_el, args.scan_max_el + 1))
        p = int(rng.integers(3, 6))
        E0 = 10 ** rng.uniform(-2, -1)
        phi = rng.uniform(0, 2 * _m.pi)
        S = Space([uniform_knots(nel, -100.0, 100.0, p)] * 2, p, p + 1)
        ph = Physics(charge=-1.0, mass=1.0, coupled=(0,), softcore=[(1.0, 0.0, 0.0, 0.0, 1.0)])
        op = Operator(S, ph)
        field = (lambda E0, phi: (lambda t: [E0 * _m.sin(_m.pi * t / T) ** 2 * _m.sin(0.057 * t + phi)]))(E0, phi)
        psi = op.separable_state([lambda x: np.exp(-x * x / 2.0)] * 2)
        runs.append((S, op, field, psi, nel, p))
    def make():
        return [Propagator(op, "cn", field=f, pc=args.scan_pc, precision="fp32", rtol=1e-10, outer="df")
                for (S, op, f, psi, nel, p) in runs]
    dt = 0.05
    steps = args.steps
    # serial
    Ps = make()
    st = [r[3].clone() for r in runs]
    for G, x in zip(Ps, st):
        G.step(x, 0.0, dt)
    torch.cuda.synchronize()
    t0 = time.time()
    for k in range(1, steps + 1):
        for G, x in zip(Ps, st):
            G.step(x, k * dt, dt)
    torch.cuda.synchronize()
    t_serial = time.time() - t0
    # batched
    Pb = make()
    B = BatchPropagator(Pb, threads=args.scan_threads)
    sb = [r[3].clone() for r in runs]
    B.step(sb, 0.0, dt)
    torch.cuda.synchronize()
    t0 = time.time()
    for k in range(1, steps + 1):
        B.step(sb, k * dt, dt)
    torch.cuda.synchronize()
    t_batch = time.time() - t0
    n = len(runs)
    its = sum(G.stats()["its"] for G in Pb) / max(1, sum(G.stats()["solves"] for G in Pb))
    print(json.dumps({"metric": "batched 2D soft-core scan, CN run-steps/s", "value": n * steps / t_batch,
                      "unit": "run-steps/s", "serial": n * steps / t_serial, "speedup": t_serial / t_batch,
                      "preconditioner": args.scan_pc, "its_per_solve": its,
                      "runs": n, "steps": steps, "threads": args.scan_threads,
                      "grids": sorted(set(int(r[4]) for r in runs)), "degrees": sorted(set(int(r[5]) for r in runs)),
                      "ndof_total": int(sum(r[0].ndof for r in runs)),
                      "note": "host wall clock around K steps after one warm-up step; grids drawn in "
                              "[%d, %d]^2 elements" % (args.scan_min_el, args.scan_max_el)}))


def run_tdz(args):
    import torch
    from tdsez_gb300 import _lib, build as _build
    from tdsez_gb300.operators import Operator
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.workloads import heterostructure

    rank, world = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    _build.build()
    lib = _lib.load()
    w = heterostructure()
    S = Space(w.knots, w.p, w.nq)
    op = Operator(S, w.phys)
    psi0 = op.separable_state(w.packet)
    N = S.ndof
    stream = torch.cuda.current_stream()
    sid = stream.cuda_stream
    dt = w.dt
    mg = dict(pc="mg", rtol=RTOL, mg_smooth=args.mg_smooth, mg_coarse_its=args.mg_coarse_its,
              mg_levels=args.mg_levels)
    if args.apply_only:
        return apply_only(args, op, S, psi0, stream)
    if args.precond_only:
        return precond_only(args, op, S, psi0, stream, w)

    # ---- headline arm: FP64 FGMRES, FP32 preconditioner (fast diagonalisation)
    t_setup = time.time()
    G = Propagator(op, "cn", field=w.field, precision="fp32", pc=args.pc, rtol=args.rtol, outer=args.outer,
                   guess_order=args.guess_order, relaxed=args.relaxed == "on")
    t_setup = time.time() - t_setup
    psi = psi0.clone()
    t = 0.0
    for i in range(args.warmup):
        G.step(psi, t, dt)
        t += dt
    torch.cuda.synchronize()
    st0 = G.stats()
    l0 = lib.tdz_launch_count()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for i in range(args.steps):
            G.step(psi, t, dt)
            t += dt
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    elapsed = allmax(ev0.elapsed_time(ev1) / 1e3, world)
    launches = lib.tdz_launch_count() - l0
    st1 = G.stats()
    its_per_step = (st1["its"] - st0["its"]) / max(1, args.steps)
    value = world * args.steps / elapsed

    # ---- the 1e-10 claim, checked: one more step of the same solver right
    # after the timed region; its stage system (M + i dt/2 H_E) X = M psi_n
    # is re-evaluated with the native FP64 apply (not the double-float one the
    # solver uses), X = (psi_{n+1} + psi_n) / 2
    from tdsez_gb300 import _lib as L
    true_rres, solver_rres = true_residual(G, op, psi, t, dt, w)
    t += dt

    # ---- roofline of the dominant kernel: the fused stage apply
    c = [w.phys.sign * e for e in w.field(t - 0.5 * dt)]
    op.set_stage(1.0, 0.5j * dt, c)
    x32 = psi.to(torch.complex64)
    y32 = torch.empty_like(x32)
    y64 = torch.empty_like(psi)
    t32 = time_kernel(lambda: op.apply(L.TDZ_STAGE, x32, y32), 20, stream)
    t64 = time_kernel(lambda: op.apply(L.TDZ_STAGE, psi, y64), 10, stream)
    tdf = time_kernel(lambda: op.apply(L.TDZ_STAGE, psi, y64, df=True), 10, stream)
    pk = peaks()
    bytes32 = 16.0 * N          # x read + y written, complex FP32
    bytes64 = 32.0 * N
    ach32 = bytes32 / t32 / 1e9
    ach64 = bytes64 / t64 / 1e9

    def run_arm(precision, nsteps, **kw):
        Gp = Propagator(op, "cn", field=w.field, precision=precision, **kw)
        pp = psi0.clone()
        tp = 0.0
        for i in range(args.warmup):
            Gp.step(pp, tp, dt)
            tp += dt
        torch.cuda.synchronize()
        sp0 = Gp.stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(nsteps):
            Gp.step(pp, tp, dt)
            tp += dt
        e1.record(stream)
        torch.cuda.synchronize()
        tpl = e0.elapsed_time(e1) / 1e3
        sp1 = Gp.stats()
        return {"steps_per_s": nsteps / tpl, "its_per_step": (sp1["its"] - sp0["its"]) / nsteps, "steps": nsteps}

    mixed_mg = run_arm("fp32", args.mg_steps, outer=args.outer, **mg) if args.mg_steps > 0 else None
    # the same multigrid with the coarsest level solved exactly by its FDM
    # inverse (the role of the reference's coarse LU)
    exact_coarse = None
    if args.mg_steps > 0:
        exact_coarse = run_arm("fp32", args.mg_steps, outer=args.outer, mg_coarse="fdm", **mg)
        exact_coarse["what"] = "FP32 multigrid, coarsest level by the exact FDM inverse, in FP64 FGMRES"

    # ---- learned arm: FP32 multigrid with the learned coarse correction, its
    # network trained on the coarse right-hand sides of the run's own first
    # steps, beside the same hierarchy without the network
    learned = None
    if args.learned_steps > 0:
        learned = learned_arms(args, op, psi0, w, stream)

    # ---- plain GPU multigrid arm (FP64 throughout)
    plain = run_arm("fp64", args.plain_steps, **mg) if args.plain_steps > 0 else None

    # ---- e2e through the C ABI with host buffers
    host = psi.cpu().pin_memory()
    dev = torch.empty_like(psi)
    ke = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    ee0, ee1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ee0.record(stream)
    te = t
    for i in range(ke):
        dev.copy_(host, non_blocking=True)
        G.step(dev, te, dt)
        te += dt
        host.copy_(dev, non_blocking=True)
    ee1.record(stream)
    torch.cuda.synchronize()
    e2e = world * ke / allmax(ee0.elapsed_time(ee1) / 1e3, world)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("c128 (FP64 FGMRES, " + ("double-float" if args.outer == "df" else "FP64") + " applies) + c64 (FP32 "
                  + args.pc + " preconditioner)"),
        "data": "synthetic (seeded heterostructure, Gaussian packet)",
        "config": {"workload": "3D heterostructure CN, 160x160x320 el, p=3, 5 C0 interfaces, N=%d" % N,
                   "global_batch": world, "dt": dt, "rtol": args.rtol, "precond": args.pc + " (FP32) in FP64 FGMRES",
                   "outer_apply": {"df": "double-float (FP32 pairs)", "fp64": "native FP64"}[args.outer],
                   "guess_order": args.guess_order, "relaxed_arnoldi": args.relaxed,
                   "mg": {"smooth": args.mg_smooth, "coarse_its": args.mg_coarse_its, "levels": args.mg_levels},
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "working set > L2 (state alone 141.6 MB)"},
        "its_per_step": its_per_step,
        "true_rres_last": true_rres,
        "solver_rres_last": solver_rres,
        "true_rres_note": "||M psi_n - A X|| / ||M psi_n|| with A = M + i dt/2 H(t + dt/2) applied in native FP64, "
                          "X = (psi_n+1 + psi_n)/2, for the step taken right after the timed ones",
        "headline_arm": "FDM-preconditioned FGMRES (FP32 fast-diagonalisation inverse inside FP64 FGMRES, "
                        "double-float applies); no learned component",
        "precision_note": "FP64 storage; outer residual and right-hand-side applies in double-float arithmetic "
                          "(~48 bits, 1e-14 relative) rather than native FP64; Arnoldi apply in FP32 arithmetic "
                          "certified by the bound gamma |||A||| ||z||; preconditioner in FP32 with TF32 hi/lo "
                          "tensor-core transforms (no BF16x3)",
        "vs_plain_mg": (value / plain["steps_per_s"]) if plain else None,
        "mixed_mg": mixed_mg,
        "mixed_mg_exact_coarse": exact_coarse,
        "plain_mg": plain,
        "learned_mg": learned["learned"] if learned else None,
        "mixed_mg_same_levels": learned["plain"] if learned else None,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 16 * N, "d2h_bytes_per_step": 16 * N,
                "steps": ke},
        "gpu_launches": int(launches),
        # dominant kernel of the CN step (about half of it): the double-float stage apply on FP64
        # vectors, 32 algorithmic bytes per coefficient (x read, y written once). It is bound by the
        # FP32 pipes (double-float arithmetic), so its HBM fraction is low by construction; traffic is
        # dram read + write of one launch from the ncu capture in profiles/.
        "roofline": {"kernel": "k_apply3d_rb<dff> double-float stage apply (FGMRES residual)",
                     "bound": "hbm", "achieved": bytes64 / tdf / 1e9, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                     "frac": bytes64 / tdf / 1e9 / pk.get("hbm_gbs", 6800.0), "traffic": DF_APPLY_TRAFFIC,
                     "peak_source": "measured" if "hbm_gbs" in pk else "fallback",
                     "launch_us": tdf * 1e6, "bytes_per_launch": bytes64,
                     "limiter": "FP32 pipes: 12 FP32 instructions per double-float FMA (ncu: 70% issue, "
                                "55% FMA pipe)",
                     "fp32_apply": {"kernel": "k_apply3d_rb<float> (multigrid smoother and residual; latency-bound, "
                                              "ncu: 57% issue, 24% warps active)",
                                    "achieved": ach32, "frac": ach32 / pk.get("hbm_gbs", 6800.0),
                                    "launch_us": t32 * 1e6, "bytes_per_launch": bytes32},
                     "fp64_apply": {"kernel": "k_apply3d<double> (native FP64, not used by the step)",
                                    "achieved": ach64, "launch_us": t64 * 1e6, "bytes_per_launch": bytes64}},
        "clocks": clk.summary(),
        "setup_s": t_setup,
    }
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(N, dt, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


CPU_GRID = (16, 16, 32)
CPU_GRID2 = (20, 20, 40)
# dram__bytes_read.sum + dram__bytes_write.sum of one k_apply3d_rb<dff> CN stage apply on
# the 160x160x320 workload (ncu --set full, tile 32 x run 73;
# profiles/k_apply3d_rb_df_stage_heterostructure_160x160x320_p3.md). Writes still in L2
# when the launch ends are not counted; the halo re-reads of neighbouring tiles are.
DF_APPLY_TRAFFIC = 206.87e6 + 109.77e6


def learned_arms(args, op, psi0, w, stream):
    """CN steps with the FP32 multigrid (args.learned_levels levels, default
    coarse polynomial) in FP64 FGMRES, with and without the learned coarse
    correction. The network's training inputs are the coarsest right-hand
    sides of the V-cycles of the learned arm's own first
    args.learned_train_steps steps (untimed), then args.learned_steps steps are
    timed after args.warmup more; the plain arm takes the same steps."""
    import torch
    from tdsez_gb300.propagator import Propagator
    dt = w.dt
    kw = dict(pc="mg", precision="fp32", outer=args.outer, rtol=args.rtol, mg_smooth=args.mg_smooth,
              mg_coarse_its=args.mg_coarse_its, mg_levels=args.learned_levels)
    out = {}
    G = Propagator(op, "cn", field=w.field, mg_learned=True, **kw)
    G0 = Propagator(op, "cn", field=w.field, **kw)
    psi, psi_p = psi0.clone(), psi0.clone()
    t = 0.0
    G.record_coarse(args.learned_pairs)
    t0 = time.time()
    for _ in range(args.learned_train_steps):   # both arms take these steps (same guess history)
        G.step(psi, t, dt)
        G0.step(psi_p, t, dt)
        t += dt
    G.record_coarse(0)
    loss, pairs = G.train_coarse(epochs=args.learned_epochs, lr=1e-3)
    torch.cuda.synchronize()
    train_s = time.time() - t0
    t_start = t
    sps, its, _ = _timed_steps(G, psi, t_start, dt, args.warmup, args.learned_steps, stream)
    out["learned"] = {"steps_per_s": sps, "its_per_step": its, "levels": args.learned_levels,
                      "train_pairs": pairs, "train_loss": loss, "train_steps": args.learned_train_steps,
                      "train_epochs": args.learned_epochs, "train_s": train_s, "steps": args.learned_steps,
                      "what": "FP32 multigrid with the CNN coarse correction (BF16 weights) in FP64 FGMRES"}
    sps0, its0, _ = _timed_steps(G0, psi_p, t_start, dt, args.warmup, args.learned_steps, stream)
    out["plain"] = {"steps_per_s": sps0, "its_per_step": its0, "levels": args.learned_levels,
                    "steps": args.learned_steps, "what": "the same hierarchy without the network"}
    return out


def true_residual(G, op, psi, t, dt, w):
    """One CN step of propagator G from psi (in place), then the relative
    residual of its stage system with the native FP64 apply; returns (true,
    the solver's own estimate)."""
    import torch
    from tdsez_gb300 import _lib as L
    psi_n = psi.clone()
    G.step(psi, t, dt)
    solver_rres = G.stats()["last_rres"]
    X = 0.5 * (psi + psi_n)
    b = torch.empty_like(psi)
    op.apply(L.TDZ_MASS, psi_n, b)
    c = [w.phys.sign * e for e in w.field(t + 0.5 * dt)]
    op.set_stage(1.0, 0.5j * dt, c)
    ax = torch.empty_like(psi)
    op.apply(L.TDZ_STAGE, X, ax)
    r = torch.linalg.vector_norm(b - ax).item() / torch.linalg.vector_norm(b).item()
    del psi_n, X, b, ax
    return r, solver_rres


def apply_only(args, op, S, psi0, stream):
    """Time the fused stage apply alone (FP32 and FP64), args.steps launches
    each after 3 warm-up launches: the command profiled for the kernel."""
    import torch
    from tdsez_gb300 import _lib as L
    op.set_stage(1.0, 0.25j, [0.001])
    x32 = psi0.to(torch.complex64)
    y32 = torch.empty_like(x32)
    y64 = torch.empty_like(psi0)
    t32 = time_kernel(lambda: op.apply(L.TDZ_STAGE, x32, y32), args.steps, stream)
    t64 = time_kernel(lambda: op.apply(L.TDZ_STAGE, psi0, y64), max(1, args.steps // 4), stream)
    tdf = time_kernel(lambda: op.apply(L.TDZ_STAGE, psi0, y64, df=True), max(1, args.steps // 2), stream)
    N = S.ndof
    print(json.dumps({"apply_fp32_us": t32 * 1e6, "apply_fp32_gbs": 16.0 * N / t32 / 1e9,
                      "apply_fp64_us": t64 * 1e6, "apply_fp64_gbs": 32.0 * N / t64 / 1e9,
                      "apply_df_us": tdf * 1e6, "apply_df_gbs": 32.0 * N / tdf / 1e9, "N": N}))


def precond_only(args, op, S, psi0, stream, w):
    """Time one FDM preconditioner application (transforms + line solves) on
    the CN stage, args.steps applications after 3 warm-up ones; restart 2 keeps
    the device footprint small (the command profiled for the FDM kernels)."""
    import torch
    from tdsez_gb300.propagator import Solver
    op.set_stage(1.0, 0.5j * w.dt, [0.001])
    s = Solver(op, pc="fdm", precision="fp32", restart=2, rtol=1e-10)
    z = torch.empty_like(psi0)
    t = time_kernel(lambda: s.precondition(psi0, z), args.steps, stream)
    print(json.dumps({"fdm_apply_us": t * 1e6, "N": S.ndof}))


def cpu_baseline(n_full: int, dt: float, seconds: float):
    """The reference's CPU method restated (GMRES(30) + ILU(0) on the
    assembled FP64 CN matrix, preconditioner reused; the oracle's C port with
    OpenMP over every host core) on a reduced grid of the same workload,
    scaled to the full grid by the coefficient count. ILU(0) of the whole
    matrix (triangular solves on one thread, everything else threaded) is the
    fastest configuration on the host: one block-Jacobi block per thread, as
    on one MPI rank per core, needs 20x the iterations on this grid. Without
    a C compiler the scipy restatement (one core, SuperLU ILUTP) stands in."""
    from oracle.cpu_baseline import cn_steps, cn_steps_threads
    from tdsez_gb300.workloads import heterostructure
    w = heterostructure(nel=CPU_GRID, dt=dt)
    try:
        r = cn_steps_threads(w, seconds=seconds, threads=0, blocks=1)
        cores, how = r["threads"], "GMRES(30)+ILU(0), %d OpenMP threads (C port)" % r["threads"]
    except Exception as e:   # no gcc / OpenMP on this host
        r = cn_steps(w, seconds=seconds)
        cores, how = 1, "GMRES(30)+ILUTP, 1 core (scipy port; C port unavailable: %s)" % type(e).__name__
    out = {"value": r["steps_per_s"] * r["ndof"] / n_full, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "%d CN steps on %s elements (N=%d), %s at rtol 1e-10, %.1f s; extrapolated linearly by "
                     "N=%d/%d to the full grid (optimistic: the ILU(0)-GMRES iterations grow with N)"
           % (r["steps"], r["elements"], r["ndof"], how, r["seconds"], r["ndof"], n_full),
           "its_per_step": r["its_per_step"]}
    # a second, larger timed point shows how the iteration count and the
    # rate per coefficient move with N
    try:
        w2 = heterostructure(nel=CPU_GRID2, dt=dt)
        r2 = cn_steps_threads(w2, seconds=max(2.0, 0.5 * seconds), threads=0, blocks=1)
        out["larger_sample"] = {"elements": r2["elements"], "ndof": r2["ndof"], "steps": r2["steps"],
                                "steps_per_s": r2["steps_per_s"], "its_per_step": r2["its_per_step"],
                                "extrapolated_value": r2["steps_per_s"] * r2["ndof"] / n_full}
    except Exception as e:   # a host without the C port
        out["larger_sample"] = {"unavailable": type(e).__name__}
    return out


def _timed_steps(G, psi, t0, dt, warmup, steps, stream):
    """warmup untimed steps, then `steps` steps between CUDA events; returns
    (steps/s, Krylov its per stage solve, t after the steps)."""
    import torch
    t = t0
    for _ in range(warmup):
        G.step(psi, t, dt)
        t += dt
    torch.cuda.synchronize()
    s0 = G.stats()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        G.step(psi, t, dt)
        t += dt
    e1.record(stream)
    torch.cuda.synchronize()
    s1 = G.stats()
    el = e0.elapsed_time(e1) / 1e3
    return steps / el, (s1["its"] - s0["its"]) / max(1, s1["solves"] - s0["solves"]), t


def run_softcore(args):
    """The soft-core configurations at size (secondary lines, not the
    headline): cfg2, 2D soft-core hydrogen 512^2 elements p = 4, Pade(2,2)
    dt = 0.02 with a CAP of width 20 a.u. and t-SURFF on |x_d| = 80, ground
    state by the GPU eigensolver, FP32 multigrid inside FP64 FGMRES against
    the FP64 multigrid; cfg3, 3D soft-core atom 192^3 elements p = 4 with
    symmetric exponential knots, Magnus-4 dt = 0.02, 3-level multigrid in
    FP32 inside FP64 FGMRES. Steps are timed with CUDA events after
    --warmup untimed steps, starting at the pulse's peak."""
    import dataclasses
    import torch
    from tdsez_gb300 import _lib as L
    from tdsez_gb300 import build as _build
    from tdsez_gb300.eigen import bound_states
    from tdsez_gb300.operators import Operator
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    from tdsez_gb300.workloads import softcore2d, softcore3d
    torch.cuda.set_device(0)
    _build.build()
    L.load()
    stream = torch.cuda.current_stream()
    out = {"config": args.config, "unit": "steps/s", "data": "synthetic (seeded workload, ground state or packet)"}
    if args.config == "cfg2":
        w = softcore2d(nel=args.nel or 512)
        S = Space(w.knots, w.p, w.nq)
        op = Operator(S, w.phys)
        op0 = Operator(S, dataclasses.replace(w.phys, cap_kmin=None, bounds=()))
        torch.cuda.synchronize()
        tg = time.time()
        E, V, berr, solves = bound_states(op0, 1, target=-1.5, tol=1e-10, pc="mg", precision="fp32", rtol=1e-11,
                                          outer="df")
        torch.cuda.synchronize()
        out["ground_state"] = {"E0": E[0], "backward_error": berr[0], "inner_solves": solves,
                               "seconds": time.time() - tg}
        psi0 = V[0].clone()
        t0 = 0.5 * w.meta["T"]
        arms = {}
        for name, kw in (("fp32_mg_in_fp64", dict(pc="mg", precision="fp32", outer="df")),
                         ("fp64_mg", dict(pc="mg", precision="fp64", outer="fp64")),
                         # the FDM inverse of the separable part (kinetic and absorbing
                         # layers through complex axis pencils; the soft-core term and the
                         # field along x left to FGMRES)
                         ("fp32_fdm_in_fp64", dict(pc="fdm", precision="fp32", outer="df"))):
            G = Propagator(op, "pade22", field=w.field, rtol=args.rtol, **kw)
            psi = psi0.clone()
            sps, its, _ = _timed_steps(G, psi, t0, w.dt, args.warmup, args.steps if "fp32" in name else
                                       max(2, args.steps // 4), stream)
            arms[name] = {"steps_per_s": sps, "its_per_solve": its}
        ts = TSurff(S, 80.0, [(-2.0, 2.0, 128)] * 2, w.field, w.dt)
        ts.sample(t0, psi)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(10):
            ts.sample(t0 + (k + 1) * w.dt, psi)
        e1.record(stream)
        torch.cuda.synchronize()
        out.update({"workload": "2D soft-core 512^2 el p=4, Pade(2,2) dt=0.02, CAP 20 a.u., t-SURFF R=80",
                    "ndof": S.ndof, "arms": arms, "tsurff_sample_ms": e0.elapsed_time(e1) / 10,
                    "rtol": args.rtol})
    else:
        w = softcore3d(nel=args.nel or 192)
        S = Space(w.knots, w.p, w.nq)
        op = Operator(S, w.phys)
        psi = op.separable_state(w.packet)
        t0 = 0.5 * w.meta["T"]
        G = Propagator(op, "magnus4", field=w.field, rtol=args.rtol, pc="mg", precision="fp32", outer="df",
                       mg_levels=3)
        sps, its, _ = _timed_steps(G, psi, t0, w.dt, args.warmup, args.steps, stream)
        # the FDM inverse of the separable part (the soft-core term left to FGMRES)
        Gf = Propagator(op, "magnus4", field=w.field, rtol=args.rtol, pc="fdm", precision="fp32", outer="df")
        sps_f, its_f, _ = _timed_steps(Gf, psi, t0, w.dt, args.warmup, args.steps, stream)
        out["fdm_arm"] = {"steps_per_s": sps_f, "its_per_solve": its_f,
                          "what": "FP32 FDM inverse of the separable part in FP64 FGMRES"}
        op.set_stage(1.0, 0.01j, [0.001])
        x32 = psi.to(torch.complex64)
        y32 = torch.empty_like(x32)
        ta = time_kernel(lambda: op.apply(L.TDZ_STAGE, x32, y32), 5, stream)
        out.update({"workload": "3D soft-core 192^3 el p=4 symexp, Magnus-4 dt=0.02, 3-level MG (FP32) in FP64 FGMRES",
                    "ndof": S.ndof, "steps_per_s": sps, "its_per_solve": its, "rtol": args.rtol,
                    "fp32_stage_apply_us": ta * 1e6, "fp32_stage_apply_gbs": 16.0 * S.ndof / ta / 1e9})
    print(json.dumps(out))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n_full = 163 * 163 * 333
    cb = cpu_baseline(n_full, 0.5, args.cpu_seconds)
    v = cb["value"]
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "impl": "reference",
           "config": {"workload": "3D heterostructure CN, 160x160x320 el, p=3, 5 C0 interfaces, N=%d" % n_full},
           "cpu_baseline": {"kind": "port", "cores": cb["cores"], "sample": cb["sample"], "value": v},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference needs PETSc/SLEPc/PetIGA/MUMPS (absent); its CPU method is timed as the oracle port"}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tdz")
    ap.add_argument("--plain-steps", type=int, default=10)
    ap.add_argument("--mg-steps", type=int, default=10)
    ap.add_argument("--pc", default="fdm")
    ap.add_argument("--outer", default="df", choices=["df", "fp64"])
    ap.add_argument("--guess-order", type=int, default=-1)
    ap.add_argument("--rtol", type=float, default=RTOL)
    ap.add_argument("--relaxed", default="on", choices=["on", "off"])
    ap.add_argument("--apply-only", action="store_true")
    ap.add_argument("--precond-only", action="store_true")
    ap.add_argument("--batch-scan", type=int, default=0, help="runs of the batched 2D scan (0: headline bench)")
    ap.add_argument("--scan-min-el", type=int, default=128)
    ap.add_argument("--scan-pc", default="fdm", choices=["fdm", "mg"], help="preconditioner of the scan's runs")
    ap.add_argument("--scan-max-el", type=int, default=512)
    ap.add_argument("--scan-threads", type=int, default=16)
    ap.add_argument("--mg-smooth", type=int, default=8)
    ap.add_argument("--mg-coarse-its", type=int, default=12)
    ap.add_argument("--mg-levels", type=int, default=0)
    ap.add_argument("--learned-steps", type=int, default=10, help="timed steps of the learned arm (0: skip it)")
    ap.add_argument("--learned-levels", type=int, default=3)
    ap.add_argument("--learned-train-steps", type=int, default=6)
    ap.add_argument("--learned-pairs", type=int, default=64)
    ap.add_argument("--learned-epochs", type=int, default=40)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--config", default="cfg5", choices=["cfg5", "cfg2", "cfg3"],
                    help="cfg5: the headline heterostructure; cfg2 / cfg3: the soft-core configurations at size")
    ap.add_argument("--nel", type=int, default=0, help="elements per axis of cfg2 / cfg3 (0: the configuration's)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config in ("cfg2", "cfg3"):
        run_softcore(args)
    elif args.batch_scan > 0:
        batch_scan(args)
    else:
        run_tdz(args)


if __name__ == "__main__":
    main()
