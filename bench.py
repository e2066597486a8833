#!/usr/bin/env python
"""Benchmark: Heston options/sec of the batched FP64 ADI pricer on one GB300.

Workload (the batched configuration): 4096 Heston calls drawn from a seed,
uniform in K/S0 in [0.7, 1.3], T in [0.1, 2], r in [0, 0.08], kappa in [0.5, 5],
theta in [0.01, 0.16], sigma in [0.1, 1], rho in [-0.9, 0], v0 in [0.01, 0.16];
uneven grids nS in {64, 96, ..., 512}, nv in {32, 48, ..., 256}; nt = 200
(two implicit half-steps, then 199 Hundsdorfer-Verwer steps at
theta = 1/2 + sqrt(3)/6). One step = pricing the whole batch once: build every
option's operators on the device, reset the state to the payoff and run the
200 time steps (one CUDA graph), then read the prices. Inputs are synthetic
(there is no public dataset); state arrays (~1.4 GB) exceed L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Heston options/sec at <=1e-3 abs err: batched ADI vs plain ADI vs surrogate"
UNIT = "options/s"
HV_THETA = 0.5 + np.sqrt(3.0) / 6.0

# Algorithmic state traffic (bytes per grid point) and FP64 work (flops per
# grid point, an FMA counts 2) of one launch of each stage kernel. State
# traffic counts the stage's input and output grids once (operator
# coefficients, which stream at the same time, are not counted). Flops: spot
# and variance applies 3 FMA each, the mixed term 3 FMA for the shared row
# sums (x 10/8 for the tile halo) + 3 FMA + 1 MUL, the scheme combination
# 4-6; Thomas solves FMA + MUL forward and FMA backward (+1 for x - T).
# Algorithmic FLOPs of one surrogate forward per query and member, network
# 8 -> 256 x 4 -> 2 (the padding to 16 inputs and 128/16 outputs is not counted).
NET_FLOPS = 2.0 * (8 * 256 + 3 * 256 * 256 + 256 * 2)

# Algorithmic state bytes per grid point of each stage: the per-stage figures
# of the unit "one grid point x one time step" (FP64 state grids only; operator
# coefficients and Thomas factors are counted as cached). HV step = 144 B:
# Y0 16 (read V, write Y0) + Y1 24 + Y2 24 + corrector 32 (read Y0, Y2, V;
# write) + two corrector solves 24 each. Implicit step = 40 B: the mixed
# explicit part 16 + two solves 12 each. The fused kernels read and write more
# or less than these (KERNEL_IO_BYTES), but the roofline counts these.
STAGE_BYTES = {"explicit_hv0": 16, "explicit_hv3": 32, "spot_solve": 24, "var_solve_y2": 24,
               "var_solve_v": 24, "explicit_implicit": 16, "var_solve_implicit": 12,
               "spot_solve_implicit": 12}
HV_STEP_BYTES = 144
HV_STEP_STAGES = ["explicit_hv0", "spot_solve", "var_solve_y2", "explicit_hv3", "spot_solve",
                  "var_solve_v"]
# The state bytes each fused kernel itself reads and writes per point (its own
# input and output grids): the predictor reads V and writes F(V), W and F1 V.
KERNEL_IO_BYTES = {"explicit_hv0": 32, "explicit_hv3": 40, "spot_solve": 24, "var_solve_y2": 16,
                   "var_solve_v": 16, "explicit_implicit": 16, "var_solve_implicit": 16,
                   "spot_solve_implicit": 16}
# DRAM bytes per grid point per launch measured by ncu (--set full) on the
# 256-option cut of the batch workload (profiles/explicit_hv_batch256.md and
# profiles/line_solves_batch256.md); its state, operators and Thomas factors
# already exceed L2, and traffic grows with the points processed, so a full
# launch is this x points. The spot solve's figure includes its three Thomas
# factors per point and the forward sweep's result read back by the backward
# sweep, which the algorithmic state bytes leave out.
NCU_TRAFFIC_B_PER_POINT = {"explicit_hv0": 52.6, "explicit_hv3": 62.6, "spot_solve": 56.9}
# FP64 pipe work per grid point: FP64 instructions x 2, so that a pipe fully
# busy with DFMA (2 flops each; DMUL and DADD occupy it the same) reads as the
# DFMA peak that fdadi_fp64_probe measures. The mixed-term row sums are formed
# for 18 staged rows per 16-row tile: 3 x 18/16 = 3.375 instructions per point.
STAGE_FLOPS = {"explicit_hv0": 30.75, "explicit_hv3": 32.75, "spot_solve": 8, "var_solve_y2": 6,
               "var_solve_v": 6, "explicit_implicit": 12.75, "var_solve_implicit": 6,
               "spot_solve_implicit": 6}


def workload(n_options, seed, nt=200):
    """Seeded config: per option (params, nS, nv)."""
    rng = np.random.default_rng(seed)
    S0 = 100.0
    K = S0 * rng.uniform(0.7, 1.3, n_options)
    T = rng.uniform(0.1, 2.0, n_options)
    r = rng.uniform(0.0, 0.08, n_options)
    kappa = rng.uniform(0.5, 5.0, n_options)
    theta = rng.uniform(0.01, 0.16, n_options)
    sigma = rng.uniform(0.1, 1.0, n_options)
    rho = rng.uniform(-0.9, 0.0, n_options)
    v0 = rng.uniform(0.01, 0.16, n_options)
    nS = rng.choice(np.arange(64, 513, 32), n_options)
    nv = rng.choice(np.arange(32, 257, 16), n_options)
    # group equal grid sizes so neighbouring lines of the arena have equal length
    order = np.lexsort((nv, nS))
    cols = [K, T, r, kappa, theta, sigma, rho, v0, nS, nv]
    K, T, r, kappa, theta, sigma, rho, v0, nS, nv = [c[order] for c in cols]
    return dict(S0=S0, K=K, T=T, r=r, kappa=kappa, theta=theta, sigma=sigma, rho=rho, v0=v0,
                nS=nS.astype(np.int32), nv=nv.astype(np.int32), nt=nt)


def workload_large():
    """The large single-instance configuration: rho = -0.7, sigma = 0.5,
    K in {80, 100, 120} (one option each, run as one batch), 1024 x 512 grid,
    nt = 1000, HV theta = 1/2 + sqrt(3)/6 after two implicit half-steps."""
    K = np.array([80.0, 100.0, 120.0])
    n = K.size
    return dict(S0=100.0, K=K, T=np.ones(n), r=np.full(n, 0.06), kappa=np.ones(n),
                theta=np.full(n, 0.04), sigma=np.full(n, 0.5), rho=np.full(n, -0.7),
                v0=np.full(n, 0.04), nS=np.full(n, 1024, np.int32), nv=np.full(n, 512, np.int32),
                nt=1000)


def subset(w, idx):
    out = dict(w)
    for k, v in w.items():
        if isinstance(v, np.ndarray):
            out[k] = v[idx]
    return out


def _mesh_one(args):
    from fd_adi_gb300 import mesh
    S0, K, v0, nS, nv = args
    return mesh.heston_meshes(S0, K, v0, int(nS), int(nv), 8.0 * K, 5.0)


def meshes_for(w, idx=None):
    idx = range(len(w["K"])) if idx is None else idx
    jobs = [(w["S0"], w["K"][k], w["v0"][k], w["nS"][k], w["nv"][k]) for k in idx]
    if len(jobs) > 64:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
            return pool.map(_mesh_one, jobs, chunksize=32)
    return [_mesh_one(j) for j in jobs]


def params_of(w, idx=None):
    idx = range(len(w["K"])) if idx is None else idx
    return [(w["r"][k], w["kappa"][k], w["theta"][k], w["sigma"][k], w["rho"][k]) for k in idx]


def payoffs(w, meshes, idx=None):
    idx = list(range(len(w["K"])) if idx is None else idx)
    return [np.maximum(m[0][:, None] - w["K"][k], 0.0) * np.ones((1, m[1].size))
            for k, m in zip(idx, meshes)]


class Clocks(object):
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            try:
                pw.append(float(f[3]))
            except ValueError:
                pass
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_min_mhz": float(min(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "power_w": float(np.median(pw)) if pw else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def fp64_peak(torch, index=0, seconds=1.2):
    """FP64 FMA throughput of this device, measured with the library's probe:
    a full-occupancy DFMA loop (8 blocks of 256 threads per SM) with 1, 2, 4, 8
    and 16 independent chains per thread, each run for about `seconds` while
    nvidia-smi samples the SM clock. Returns the best rate (TFLOP/s) and the
    sweep: per chain count its rate, the median SM clock during it and the
    DFMA thread-instructions it retired per SM per clock cycle."""
    from fd_adi_gb300 import _lib
    dev = torch.cuda.current_device()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, threads = sms * 8, 256
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    flops = ctypes.c_double()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run(chains, iters):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.call("fdadi_fp64_probe", ctypes.c_void_p(out.data_ptr()), blocks, threads, iters,
                  chains, ctypes.byref(flops), st)
        e1.record()
        e1.synchronize()
        return flops.value, e0.elapsed_time(e1) * 1e-3

    sweep = {}
    best = 0.0
    for chains in (1, 2, 4, 8, 16):
        f, t = run(chains, 256)
        iters = max(256, int(256 * seconds / max(t, 1e-6)))
        iters = min(iters, 1 << 30)
        clk = Clocks(index)
        clk.start()
        time.sleep(0.25)
        f, t = run(chains, iters)
        c = clk.stop()
        rate = f / t
        mhz = c.get("sm_mhz")
        per_clk = (f / 2.0 / t / sms / (mhz * 1e6)) if mhz else None
        sweep[str(chains)] = {"tflops": round(rate / 1e12, 4), "seconds": round(t, 3),
                              "sm_mhz": mhz, "dfma_per_sm_per_clk": (round(per_clk, 3)
                                                                     if per_clk else None)}
        best = max(best, rate)
    return best / 1e12, sweep


def stage_times(batch, V, torch):
    """Average device time per launch of every stage kernel over one full
    run, launched stage by stage with CUDA events on the batch's stream."""
    from fd_adi_gb300 import _lib
    s = batch.struct
    seq = []
    for _ in range(s.implicit_steps):
        seq += ["explicit_implicit", "var_solve_implicit", "spot_solve_implicit"]
    for _ in range(s.n_steps):
        seq += ["explicit_hv0", "spot_solve", "var_solve_y2", "explicit_hv3", "spot_solve",
                "var_solve_v"]
    stream = batch.stream
    acc, cnt = {}, {}
    evs = []
    with torch.cuda.stream(stream):
        for name in seq:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.call("fdadi_heston_stage", ctypes.byref(s),
                      ctypes.c_void_p(batch.workspace.data_ptr()), batch.workspace_bytes,
                      ctypes.c_void_p(V.data_ptr()), _lib.STAGE[name],
                      ctypes.c_void_p(stream.cuda_stream))
            e1.record(stream)
            evs.append((name, e0, e1))
    stream.synchronize()
    for name, e0, e1 in evs:
        acc[name] = acc.get(name, 0.0) + e0.elapsed_time(e1)
        cnt[name] = cnt.get(name, 0) + 1
    return {k: (acc[k] / cnt[k], cnt[k], acc[k]) for k in acc}


def plain_vs_batched(torch, n_batch=2048):
    """The 150x150 option (nt=150: two implicit half-steps then Douglas 0.5):
    options/s of the per-operator engine (the reference's per-step call
    sequence, one option per launch chain) vs the fused batched engine."""
    from fd_adi_gb300 import HestonOption, HestonFiniteDifferenceEngine, mesh
    from fd_adi_gb300.batch import HestonBatch
    n, dt = 150, 1.0 / 150
    opt = HestonOption(spot=100., strike=100., interest_rate=0.06, volatility=0.2, tenor=1.0,
                       mean_reversion=1.0, mean_variance=0.04, vol_of_variance=0.2,
                       correlation=0.0)
    S, v = mesh.heston_meshes(100., 100., 0.04, 150, 150, 800., 5.)
    grid_host = np.maximum(S[:, None] - 100., 0) * np.ones((1, v.size))

    def plain_once():
        from fd_adi_gb300 import Grid
        F = HestonFiniteDifferenceEngine(opt, grid=Grid([S.copy(), v.copy()],
                                                        initializer=lambda *x: np.maximum(
                                                            x[0] - 100., 0)), fused=False)
        V = F._initial(None)
        F.solve_implicit_(2, dt * 0.5, V)
        F.solve_douglas_(n - 1, dt, V, 0.5)
        return float(V[F.idx].item())

    plain_once()
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        p_plain = plain_once()
    torch.cuda.synchronize()
    plain = reps / (time.perf_counter() - t0)
    b = HestonBatch([opt] * n_batch, [(S, v)] * n_batch, scheme="douglas", n_steps=n - 1, dt=dt,
                    theta=0.5, implicit_steps=2, implicit_dt_factor=0.5, graph=True, plan="auto")
    V0 = b.pack([grid_host] * n_batch)
    V = torch.empty_like(V0)
    idx = b.flat_index()
    out = torch.empty(n_batch, dtype=torch.float64, device="cuda")

    def batched_once():
        with torch.cuda.stream(b.stream):
            b._prepare()
            V.copy_(V0, non_blocking=True)
            b.run(V)
            b.gather(V, idx, out)

    batched_once()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(b.stream)
    for _ in range(reps):
        batched_once()
    e1.record(b.stream)
    torch.cuda.synchronize()
    batched = reps * n_batch / (e0.elapsed_time(e1) * 1e-3)
    p_batch = float(out[0].item())
    # the fused engine on one option at a time: one CUDA graph per option
    # (the same kernels as the batch, a batch of 1), timed on the device
    b1 = HestonBatch([opt], [(S, v)], scheme="douglas", n_steps=n - 1, dt=dt, theta=0.5,
                     implicit_steps=2, implicit_dt_factor=0.5, graph=True, plan="auto")
    V10 = b1.pack([grid_host])
    V1 = torch.empty_like(V10)
    idx1 = b1.flat_index()
    out1 = torch.empty(1, dtype=torch.float64, device="cuda")

    def single_once():
        with torch.cuda.stream(b1.stream):
            b1._prepare()
            V1.copy_(V10, non_blocking=True)
            b1.run(V1)
            b1.gather(V1, idx1, out1)

    for _ in range(3):
        single_once()
    torch.cuda.synchronize()
    reps1 = 20
    e0.record(b1.stream)
    for _ in range(reps1):
        single_once()
    e1.record(b1.stream)
    torch.cuda.synchronize()
    single = reps1 / (e0.elapsed_time(e1) * 1e-3)
    p_single = float(out1[0].item())
    return {"config": "150x150, nt=150, 2 implicit half-steps + Douglas theta=0.5",
            "plain_options_per_s": plain, "batched_options_per_s": batched,
            "ratio": batched / plain, "batch": n_batch, "plan": b.plan,
            "plain_note": "per-operator engine: the reference's per-step call sequence, about "
                          "a dozen small launches per step issued from Python through ctypes; "
                          "its time is mostly host launch overhead, not GPU work",
            "fused_single_options_per_s": single,
            "ratio_vs_fused_single": batched / single,
            "fused_single_note": "fused engine with a batch of 1 option: the operator build, "
                                 "then the time loop (%d launches) replayed from one CUDA "
                                 "graph per option (device-timed)" % b1.launches_per_run,
            "price_plain": p_plain, "price_batched": p_batch, "price_fused_single": p_single,
            "price_rel_diff": abs(p_plain - p_batch) / abs(p_plain),
            "price_rel_diff_single": abs(p_single - p_batch) / abs(p_batch)}


def run_gemm(args):
    """Ensemble forward of the surrogate network alone on --queries random
    inputs (4 members, 8-256x4-2): tensor-core GEMM throughput."""
    import torch
    from fd_adi_gb300 import _lib
    from fd_adi_gb300.surrogate import MLPEnsemble, LAYERS
    torch.cuda.set_device(0)
    _lib.load()
    dev = torch.device("cuda", 0)
    M = (args.queries // 128) * 128
    net = MLPEnsemble(members=4, seed=args.seed, device=dev)
    X = torch.zeros(M, 16)
    X[:, :8] = torch.rand(M, 8) * 2 - 1
    X = X.to(torch.bfloat16).to(dev)
    flops = NET_FLOPS * M * net.P
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        peak = float(json.load(f).get("bf16_tflops", 1901.1))
    out = {"workload": "surrogate ensemble forward", "queries": M, "peak": peak}
    # fused inference (one kernel, activations on chip), the layered inference
    # (hidden pre-activations not stored) and the training forward
    runs = (("fused_inference", lambda: net.infer(X, M)),
            ("inference", lambda: net.forward(X, M, keep_preact=False)),
            ("training", lambda: net.forward(X, M, keep_preact=True)))
    for name, fn in runs:
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        net.check()
        ms = e0.elapsed_time(e1) / args.steps
        ach = flops / (ms * 1e-3) / 1e12
        out[name] = {"ms": ms, "queries_per_s": M / (ms * 1e-3), "tflops": ach,
                     "frac": ach / peak}
    print(json.dumps(out))
    return 0


def run_surrogate(args):
    """Learned surrogate with ADI fallback (the surrogate configurations):
    training set of scrambled-Sobol draws in the batched box priced by the
    batched FP64 ADI at 256x128x200; a 4-member BF16 ensemble trained on the
    tensor cores (lr 1e-3 cosine, batch 8192); queries 95% inside the box and
    5% outside (T up to 5, sigma up to 2) priced by surrogate + fallback."""
    import multiprocessing as mp
    import torch
    from fd_adi_gb300 import _lib
    from fd_adi_gb300.surrogate import (Surrogate, adi_price, sobol_queries, BOX_LO, BOX_HI,
                                        MLPEnsemble, LAYERS, CoarseADI)
    torch.cuda.set_device(0)
    _lib.load()
    dev = torch.device("cuda", 0)
    grid = dict(nS=256, nv=128, nt=200)
    pool = mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1))
    t0 = time.perf_counter()
    Qtr = sobol_queries(args.train, seed=args.seed + 1)
    Qte = sobol_queries(args.test, seed=args.seed + 2)
    cached = None
    if args.train_cache:
        # training prices from an earlier run of the same pricer on the same
        # seeded draws; the held-out set is still priced (and timed) here
        d = np.load(args.train_cache)
        if d["ptr"].shape != (args.train,):
            raise SystemExit("--train-cache holds %d training prices, not %d"
                             % (d["ptr"].shape[0], args.train))
        ptr, dtr = d["ptr"], d["dtr"]
        cached = "training prices loaded (%d draws, seed %d); held-out priced live" % (
            args.train, args.seed + 1)
        t0 = time.perf_counter()
        n_priced = args.test
    else:
        ptr, dtr = adi_price(Qtr, pool=pool, **grid)
        n_priced = args.train + args.test
    pte, dte = adi_price(Qte, pool=pool, **grid)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    adi_rate = n_priced / t_data
    # the same data with the plain Black-Scholes control variate, for comparison
    alt = {}
    for cv in ([c for c in (0, 1, 2) if c != args.cv] if args.compare_cv else []):
        s_alt = Surrogate(members=4, seed=args.seed, device=dev, cv=cv)
        s_alt.fit(Qtr, ptr, dtr, epochs=args.epochs, batch=8192, lr=1e-3)
        pa = s_alt.predict(torch.as_tensor(Qte, device=dev))[0].cpu().numpy()
        alt["cv%d_heldout_rms_abs_err" % cv] = float(np.sqrt(np.mean((pa - pte) ** 2)))
        alt["cv%d_heldout_max_abs_err" % cv] = float(np.abs(pa - pte).max())
        del s_alt
    coarse = ctr = cte = None
    t_coarse = None
    if args.coarse:
        # two-level surrogate: the coarse-grid ADI prices of the training and
        # held-out draws (their control variate), priced and timed here
        nS_c, nv_c, nt_c = (int(x) for x in args.coarse.split("x"))
        coarse = CoarseADI(nS_c, nv_c, nt_c)
        t0 = time.perf_counter()
        ctr = coarse.price(Qtr)
        cte = coarse.price(Qte)
        torch.cuda.synchronize()
        t_coarse = time.perf_counter() - t0
        print("coarse prices: %.1f s" % t_coarse, file=sys.stderr, flush=True)
    sur = Surrogate(members=4, seed=args.seed, device=dev, cv=args.cv, coarse=coarse)
    t0 = time.perf_counter()
    sur.fit(Qtr, ptr, dtr, epochs=args.epochs, batch=8192, lr=1e-3, coarse=ctr)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    p, d, spread, fb, _ = sur.predict(torch.as_tensor(Qte, device=dev), coarse=cte)
    p = p.cpu().numpy()
    d = d.cpu().numpy()
    err = np.abs(p - pte)
    gate = None
    if args.gate:
        # the error gate, trained on the training draws' own errors and
        # calibrated on the first half of the held-out draws; evaluated on the
        # second half and on the served query sample below
        t0 = time.perf_counter()
        sur.fit_gate(Qtr, ptr, epochs=args.epochs, batch=8192, lr=1e-3, coarse=ctr)
        h = Qte.shape[0] // 2
        tau, cal_fb = sur.calibrate(Qte[:h], pte[:h], bar=1e-3, margin=args.gate_margin,
                                    coarse=None if cte is None else cte[:h])
        _, _, _, fbv, _ = sur.predict(torch.as_tensor(Qte[h:], device=dev),
                                      coarse=None if cte is None else cte[h:])
        fbv = fbv.cpu().numpy().astype(bool)
        ev = err[h:]
        gate = {"bar": 1e-3, "threshold_log10": tau, "margin_log10": args.gate_margin,
                "train_s": time.perf_counter() - t0,
                "calibration_fallback_fraction": cal_fb,
                "heldout_half_fallback_fraction": float(fbv.mean()),
                "heldout_half_served_max_abs_err": float(ev[~fbv].max()) if (~fbv).any()
                else None,
                "heldout_half_misses_caught": float(fbv[ev > 1e-3].mean())
                if (ev > 1e-3).any() else None}
    # queries: 95% in the box, 5% outside it
    rng = np.random.default_rng(args.seed + 3)
    nq = args.queries
    Q = sobol_queries(nq, seed=args.seed + 4)
    out = rng.random(nq) < 0.05
    Q[out, 2] = rng.uniform(0.1, 5.0, out.sum())
    Q[out, 6] = rng.uniform(0.1, 2.0, out.sum())
    def step():
        return sur.price(Q, pool=pool, **grid)

    def serve():
        # warm-up on the first 16,384 queries: graphs and plans are built
        # there, and a full warm-up pass would price every fallback twice
        for _ in range(args.warmup):
            sur.price(Q[:min(nq, 16384)], pool=pool, **grid)
        torch.cuda.synchronize()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            pq, dq, fbq = step()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        return nq / float(np.mean(times)), times, pq, dq, fbq

    if gate is not None:
        print("gate: %s" % json.dumps(gate), file=sys.stderr, flush=True)
    value, times, pq, dq, fbq = serve()
    print("served: %.1f options/s" % value, file=sys.stderr, flush=True)
    # accuracy of the served prices on a sample, against FP64 ADI
    ns = min(args.sample, nq)
    sidx = np.linspace(0, nq - 1, ns).astype(int)
    pref, _ = adi_price(Q[sidx], pool=pool, **grid)
    qerr = np.abs(pq[sidx] - pref)
    box_only = None
    if gate is not None:
        # the other operating point: the box gate alone
        tau = sur.gate_tau
        sur.gate_tau = None
        v2, t2, pq2, _, fbq2 = serve()
        sur.gate_tau = tau
        qerr2 = np.abs(pq2[sidx] - pref)
        box_only = {"options_per_s": v2, "query_fallback_fraction": float(fbq2.mean()),
                    "query_max_abs_err": float(qerr2.max()),
                    "query_rms_abs_err": float(np.sqrt(np.mean(qerr2 ** 2)))}
    # tensor pipe: one ensemble forward on the query batch, timed with events
    Qd = torch.as_tensor(Q, device=dev)
    M = (nq // 128) * 128
    X, _, _ = sur.feat(Qd[:M].contiguous())   # the network's cost is the same either way
    sur.net.infer(X, M)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        sur.net.infer(X, M)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / 5
    flops = NET_FLOPS * M * sur.net.P
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        peak = float(json.load(f).get("bf16_tflops", 1901.1))
    ach = flops / (fwd_ms * 1e-3) / 1e12
    pool.close()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(times)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network (fp32 accumulate) + f64 ADI fallback", "data": "synthetic",
            "config": {"workload": "surrogate + ADI fallback: %d queries (95%% in box, 5%% "
                                   "outside: T<=5, sigma<=2); 4-member BF16 MLP 8-256x4-2 "
                                   "trained on %d Sobol draws priced by FP64 ADI 256x128x200"
                                   % (nq, args.train),
                       "train": args.train, "test": args.test, "epochs": args.epochs,
                       "batch": 8192, "grid": "256x128x200 HV + Rannacher",
                       "parallelism": "dp1"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(Q.nbytes),
                    "d2h_bytes_per_step": int(nq * 8 * 3)},
            "roofline": {"bound": "tensor", "kernel": "mlp_infer_kernel (fused ensemble inference)",
                         "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                         "traffic": None, "peak_source": "measured (MEASURED_PEAKS.json burst)"},
            "surrogate": {"heldout_max_abs_err": float(err.max()),
                          "heldout_rms_abs_err": float(np.sqrt(np.mean(err ** 2))),
                          "heldout_delta_rms_err": float(np.sqrt(np.mean((d - dte) ** 2))),
                          "heldout_fallback_fraction": float(fb.float().mean().item()),
                          "query_fallback_fraction": float(fbq.mean()),
                          "query_max_abs_err": float(qerr.max()),
                          "query_rms_abs_err": float(np.sqrt(np.mean(qerr ** 2))),
                          "batched_adi_options_per_s": adi_rate,
                          "speedup_vs_batched_adi": value / adi_rate,
                          "control_variate": (("FP64 ADI on a %s grid (price), Black-Scholes "
                                               "at mean variance (delta)" % args.coarse)
                                              if args.coarse else
                                              "Black-Scholes at mean variance" if args.cv == 0
                                              else "Black-Scholes at mean variance + order-%d "
                                              "series in vol of variance (price), residual / "
                                              "(sigma sqrt T + 0.1)" % args.cv),
                          **alt,
                          "error_gate": gate,
                          "box_gate_only": box_only,
                          "coarse_adi": (None if coarse is None else
                                         {"grid": args.coarse, "price_s_train_and_test": t_coarse,
                                          "options_per_s": (Qtr.shape[0] + Qte.shape[0])
                                          / t_coarse}),
                          "adam_betas": list(sur.net.adam[:2]),
                          "train_data": cached or "priced in this run",
                          "data_gen_s": t_data, "train_s": t_train,
                          "forward_ms": fwd_ms}}
    print(json.dumps(line))
    return 0


def _ref_worker_init(barrier):
    """Pool initializer of the reference-engine workers: import the compiled
    reference, then wait until every worker has."""
    from oracle import ref_harness as H
    H._import()
    barrier.wait(timeout=600)


def _warm_job(job):
    """A short copy of a reference-engine job (a few time steps, no grid kept)
    for warming a worker."""
    j = list(job)
    j[8] = j[8] * 4 / j[11]   # T scaled with the steps, as cpu_baseline does
    j[11] = 4
    if len(j) > 12:
        j[12] = False
    return tuple(j)


def cpu_baseline(w, n_sample, nt_sample=None, want_results=False):
    """The reference CPU engine (compiled from its generated sources on this
    host, kind "reference") or, where it does not import, the C restatement
    of it (kind "port"), on all host cores (one single-threaded process per
    core, options spread over them), on n_sample options spread through the
    workload and, when nt_sample is given, only that many time steps of each.
    The sample's grid-point-step rate is converted to options of the
    workload's mean grid size. With want_results, also returns the sample's
    option indices, prices and final grids (for the parity check)."""
    n = len(w["K"])
    idx = sorted(set(np.linspace(0, n - 1, n_sample).astype(int).tolist()))
    nt = w["nt"]
    nrun = nt if nt_sample is None else nt_sample
    cores = os.cpu_count() or 1
    mean_pts = float(np.mean(w["nS"].astype(np.int64) * w["nv"])) * nt
    from oracle import ref_harness as H
    if H.available():
        import multiprocessing as mp
        for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
            os.environ[var] = "1"
        jobs = [(w["S0"], w["K"][k], w["r"][k], w["kappa"][k], w["theta"][k], w["sigma"][k],
                 w["rho"][k], w["v0"][k], w["T"][k] * nrun / nt, w["nS"][k], w["nv"][k], nrun,
                 want_results) for k in idx]
        workers = min(cores, len(jobs))
        ctx = mp.get_context("spawn")
        # every worker imports the reference engine and waits for the others
        # before it takes a job, so no import falls in the timed region
        with ctx.Pool(workers, initializer=_ref_worker_init,
                      initargs=(ctx.Barrier(workers),)) as pool:
            pool.map(H.price_option, [_warm_job(jobs[0])] * workers, chunksize=1)
            t0 = time.perf_counter()
            res = pool.map(H.price_option, jobs, chunksize=1)
            dt = time.perf_counter() - t0
        kind = "reference"
        what = "reference CPU engine (FiniteDifferenceEngine.pyx, compat build)"
        prices = [x[0] for x in res]
        grids = [x[3] for x in res]
    else:
        from oracle import oracle as O
        meshes = meshes_for(w, idx)
        V0 = payoffs(w, meshes, idx)
        scheds = [[("implicit", 2, w["T"][k] / nt / 2, 1.0),
                   ("hv", nrun - 1, w["T"][k] / nt, HV_THETA)] for k in idx]
        O.build()
        t0 = time.perf_counter()
        grids = O.heston_batch(meshes, params_of(w, idx), V0, scheds, nthreads=cores)
        dt = time.perf_counter() - t0
        kind = "port"
        what = "C restatement of the reference engine (oracle)"
        from fd_adi_gb300 import mesh as M
        prices = [float(g[M.price_index(m[0], m[1], w["S0"], w["v0"][k])])
                  for g, m, k in zip(grids, meshes, idx)]
    pts = float(sum(int(w["nS"][k]) * int(w["nv"][k]) for k in idx)) * nrun
    out = {"value": pts / dt / mean_pts, "unit": UNIT, "cores": min(cores, len(idx)),
           "kind": kind, "elapsed_s": dt,
           "sample": "%s: %d options spread through the %d-option workload, %d of %d time "
                     "steps (%.3g grid-point-steps) on %d cores in %.1f s = %.3g "
                     "grid-point-steps/s, scaled to the workload's mean option"
                     % (what, len(idx), n, nrun, nt, pts, min(cores, len(idx)), dt, pts / dt)}
    if want_results:
        return out, (idx, prices, grids)
    return out


def parity(batch, V, prices, sample):
    """The GPU's prices and final grids against the CPU engine's on the same
    options: max relative price difference, and max grid difference relative
    to each grid's max-norm (bars: 1e-10 and 1e-9)."""
    idx, ref_prices, ref_grids = sample
    got = prices.cpu().numpy()
    Vh = V.cpu().numpy()
    prel, grel = [], []
    for k, p, g in zip(idx, ref_prices, ref_grids):
        prel.append(abs(got[k] - p) / max(abs(p), 1e-300))
        if g is not None:
            mine = Vh[batch.p_off[k]:batch.p_off[k + 1]].reshape(batch.n0[k], batch.n1[k])
            grel.append(float(np.abs(mine - g).max() / max(np.abs(g).max(), 1e-300)))
    worst = sorted(range(len(idx)), key=lambda m: -prel[m])[:3]
    return {"n": len(idx), "max_price_rel": float(max(prel)),
            "max_grid_rel_on_sample": float(max(grel)) if grel else None,
            "worst": [{"option": int(idx[m]), "nS": int(batch.n0[idx[m]]),
                       "nv": int(batch.n1[idx[m]]), "price": float(ref_prices[m]),
                       "price_rel": float(prel[m])} for m in worst],
            "price_bar": 1e-10, "grid_bar": 1e-9,
            "ok": bool(max(prel) <= 1e-10 and (not grel or max(grel) <= 1e-9))}


def run_reference_bs(args):
    """The reference arm of the Black-Scholes workload: the reference CPU
    engine on a bounded sample of the same options, per step."""
    w = workload_bs(args.bs_options, args.seed)
    rates, elapsed = [], []
    for s in range(args.warmup + args.steps):
        cb, _, _ = bs_cpu_baseline(w, args.ref_sample)
        if s >= args.warmup:
            rates.append(cb["value"])
            elapsed.append(cb["elapsed_s"])
    value = float(np.mean(rates))
    cb["value"] = value
    line = {"metric": "Black-Scholes options/sec, batched FP64 ADI", "value": value,
            "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(elapsed)) * 1e3,
            "ms_per_workload_extrapolated": len(w["K"]) / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": "batched Black-Scholes calls, uneven meshes, HV nt=200 "
                                   "with Rannacher start", "options": len(w["K"]),
                       "nt": w["nt"], "nS": "uniform {64..512 step 32}", "seed": args.seed},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    if args.workload == "bs":
        return run_reference_bs(args)
    w = workload_large() if args.workload == "large" else workload(args.options, args.seed)
    rates, elapsed = [], []
    for s in range(args.warmup + args.steps):
        cb = cpu_baseline(w, args.ref_sample, 20 if args.workload == "large" else None)
        if s >= args.warmup:
            rates.append(cb["value"])
            elapsed.append(cb["elapsed_s"])
    value = float(np.mean(rates))
    cb["value"] = value
    # a step is the bounded sample (its wall time is measured); the whole
    # workload's time at this rate is reported beside it
    sample_ms = [x * 1e3 for x in elapsed]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(sample_ms)),
            "ms_per_workload_extrapolated": len(w["K"]) / value * 1e3,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": config_block(args, w),
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# Batched Black-Scholes (the 1-D engine): FP64 instructions per grid point per
# step of the fused kernel: HV 23 (first sweep: F V 3, + V 1, Le V 3, - 1,
# elimination 2; back substitution 1; second sweep: the difference 1, F D 3,
# - 1/2 F D 1, Le Y1 3, - 1, elimination 2; back substitution 1); an implicit
# step 3. State bytes per point per HV step, each array counted where the
# kernel reads or writes it (operator rows and factors counted as cached):
# V, Y0, D out of the first sweep (24), D in and Y1 out (16), V, Y1, Y0 in and
# D out (32), D in and V out (16).
BS_HV_INSTR, BS_IMPLICIT_INSTR, BS_HV_BYTES = 23, 3, 88


def workload_bs(n_options, seed, nt=200):
    """Seeded batched Black-Scholes calls: K/S0 in [0.7, 1.3], T in [0.1, 2],
    r in [0, 0.08], volatility in [0.1, 0.6]; nS uniform over {64, 96, ...,
    512}; meshes as the reference engine builds them (sinh to 1500 clustered at
    S0 = 100)."""
    rng = np.random.default_rng(seed)
    K = 100.0 * rng.uniform(0.7, 1.3, n_options)
    T = rng.uniform(0.1, 2.0, n_options)
    r = rng.uniform(0.0, 0.08, n_options)
    vol = rng.uniform(0.1, 0.6, n_options)
    nS = rng.choice(np.arange(64, 513, 32), n_options).astype(np.int32)
    return dict(S0=100.0, K=K, T=T, r=r, var=vol * vol, nS=nS, nt=nt)


def run_bs(args):
    """The batched Black-Scholes workload: price every option once per step
    (operators built, payoff, the whole schedule in one launch, prices read)."""
    import multiprocessing as mp
    import torch
    from fd_adi_gb300 import _lib, mesh as M
    from fd_adi_gb300.batch import BlackScholesBatch
    torch.cuda.set_device(0)
    _lib.load()
    n = args.bs_options
    w = workload_bs(n, args.seed)
    nt = w["nt"]
    mesh_of = {int(k): np.asarray(M.sinh_space(100.0, 1500.0, 7.0, int(k), force_exact=True))
               for k in np.unique(w["nS"])}
    meshes = [mesh_of[int(k)] for k in w["nS"]]
    params = np.stack([w["r"], w["var"]], axis=1)
    dts = w["T"] / nt
    batch = BlackScholesBatch([tuple(p) for p in params], meshes, scheme="hv", n_steps=nt - 1,
                              dt=dts, theta=HV_THETA, implicit_steps=2, implicit_dt_factor=0.5)
    K_dev = torch.tensor(w["K"], dtype=torch.float64, device="cuda")
    flat_idx = batch.flat_index([100.0] * n)
    prices = torch.empty(n, dtype=torch.float64, device="cuda")
    V = torch.empty(batch.total_points, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()

    def step_device():
        batch._prepare()
        batch.payoff(K_dev, V)
        batch.run(V)
        batch.gather(V, flat_idx, prices)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_device()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    # the run kernel alone (the whole schedule), events around its launch;
    # each prefetch depth once (the default choice is the batch's)
    def run_once():
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        batch.payoff(K_dev, V)
        r0.record(stream)
        batch.run(V)
        r1.record(stream)
        torch.cuda.synchronize()
        return r0.elapsed_time(r1)

    run_ms = run_once()
    by_pf = {}
    for pf in (2, 4, 8):
        batch.struct.prefetch = pf
        by_pf[str(pf)] = round(run_once(), 3)
    batch.struct.prefetch = 0
    # e2e: parameters in, prices out through the public call
    batch.price_calls(100.0, w["K"], params, dts)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        got = batch.price_calls(100.0, w["K"], params, dts)
    ms_e2e = (time.perf_counter() - t0) * 1e3 / args.steps
    if not np.array_equal(got, prices.cpu().numpy()):
        raise RuntimeError("price_calls differs from the device-resident step")
    P = batch.total_points
    instr = P * (2 * BS_IMPLICIT_INSTR + (nt - 1) * BS_HV_INSTR)
    fp64, probe = fp64_peak(torch, 0)
    fp_ach = 2.0 * instr / (run_ms * 1e-3) / 1e12
    hbm_peak, peak_src = measured_peaks()
    gbs = BS_HV_BYTES * P * (nt - 1) / (run_ms * 1e-3) / 1e9
    out = {"metric": "Black-Scholes options/sec, batched FP64 ADI", "value": n / (ms * 1e-3),
           "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "batched Black-Scholes calls, uneven meshes, HV nt=200 with "
                                  "Rannacher start", "options": n, "nt": nt,
                      "grid_points": int(P), "nS": "uniform {64..512 step 32}",
                      "mesh": "sinh_space(100, 1500, 7, nS, force_exact)",
                      "scheme": "2 implicit half-steps + 199 HV steps, theta=1/2+sqrt(3)/6",
                      "seed": args.seed, "parallelism": "dp1"},
           "e2e": {"value": n / (ms_e2e * 1e-3), "unit": UNIT, "ms_per_step": ms_e2e,
                   "h2d_bytes_per_step": int(batch.price_calls_h2d_bytes),
                   "d2h_bytes_per_step": 8 * n,
                   "api": "BlackScholesBatch.price_calls: host parameters in, host prices "
                          "out (meshes built on the host, pinned copies, operators, payoff, "
                          "one-launch schedule, read-out)"},
           "gpu_launches": 4 * args.steps,
           "grid_point_steps_per_s": float(P) * nt / (ms * 1e-3),
           "roofline": {"bound": "fp64", "kernel": "bs_run_kernel (whole schedule)",
                        "achieved": fp_ach, "peak": fp64, "unit": "TFLOP/s",
                        "frac": fp_ach / fp64, "launch_ms": run_ms,
                        "launch_ms_by_prefetch": by_pf,
                        "instructions_per_point_step": {"hv": BS_HV_INSTR,
                                                        "implicit": BS_IMPLICIT_INSTR},
                        "peak_source": "measured live: fdadi_fp64_probe",
                        "traffic": None,
                        "hbm": {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                                "frac": gbs / hbm_peak, "bytes_per_point_step": BS_HV_BYTES,
                                "peak_source": peak_src}},
           "fp64_probe": probe, "clocks": clk}
    if args.cpu_sample > 0:
        cb, idx, ref = bs_cpu_baseline(w, args.cpu_sample)
        got = prices.cpu().numpy()[idx]
        rel = np.abs(got - ref) / np.abs(ref)
        out["cpu_baseline"] = cb
        out["parity"] = {"n": len(idx), "max_price_rel": float(rel.max()), "price_bar": 1e-10,
                         "ok": bool(rel.max() <= 1e-10)}
    print(json.dumps(out))
    return 0


def bs_cpu_baseline(w, n_sample):
    """The reference CPU engine with blackscholes.py's operator (compat build,
    kind "reference") or, where it does not import, the C oracle (kind
    "port"), on n_sample options spread through the Black-Scholes workload,
    one single-threaded process per host core. Returns the baseline object,
    the sample's option indices and its prices."""
    import multiprocessing as mp
    from oracle import ref_harness as H
    from fd_adi_gb300 import mesh as M
    n = len(w["K"])
    nt = w["nt"]
    idx = sorted(set(np.linspace(0, n - 1, n_sample).astype(int).tolist()))
    cores = os.cpu_count() or 1
    if H.available():
        for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
            os.environ[var] = "1"
        jobs = [(100.0, w["K"][k], w["r"][k], w["var"][k], w["T"][k], int(w["nS"][k]), nt)
                for k in idx]
        workers = min(cores, len(jobs))
        ctx = mp.get_context("spawn")
        with ctx.Pool(workers, initializer=_ref_worker_init,
                      initargs=(ctx.Barrier(workers),)) as pool:
            pool.map(H.price_bs_option, [jobs[0]] * workers, chunksize=1)
            t0 = time.perf_counter()
            res = pool.map(H.price_bs_option, jobs, chunksize=4)
            el = time.perf_counter() - t0
        ref = np.array([x[0] for x in res])
        kind = "reference"
        what = "reference CPU engine (compat build) with blackscholes.py's operator"
    else:
        from oracle import oracle as O
        ref = []
        t0 = time.perf_counter()
        for k in idx:
            S = np.asarray(M.sinh_space(100.0, 1500.0, 7.0, int(w["nS"][k]), force_exact=True))
            dt = w["T"][k] / nt
            g = O.bs_solve(S, w["r"][k], w["var"][k], np.maximum(S - w["K"][k], 0.0),
                           [("implicit", 2, dt / 2, 1.0), ("hv", nt - 1, dt, HV_THETA)])
            ref.append(g[int(np.argmin(np.abs(S - 100.0)))])
        el = time.perf_counter() - t0
        ref = np.array(ref)
        cores = 1
        kind = "port"
        what = "C restatement of the reference engine (oracle), one core"
    used = min(cores, len(idx))
    mean_pts = float(np.mean(w["nS"]))
    pts = float(sum(int(w["nS"][k]) for k in idx)) * nt
    cb = {"value": pts / el / (mean_pts * nt), "unit": UNIT, "cores": used, "kind": kind,
          "elapsed_s": el,
          "sample": "%s: %d options spread through the %d-option workload on %d cores in "
                    "%.1f s, scaled to the workload's mean option"
                    % (what, len(idx), n, used, el)}
    return cb, idx, ref


def config_block(args, w):
    if args.workload == "large":
        return {"workload": "large single instance x3: K in {80,100,120}, 1024x512, nt=1000, "
                            "HV theta=1/2+sqrt(3)/6 with Rannacher start, rho=-0.7, sigma=0.5",
                "options_per_gpu": int(len(w["K"])), "nt": int(w["nt"]),
                "grid_points": int(np.sum(w["nS"].astype(np.int64) * w["nv"])),
                "l2": "state arrays larger than L2 (no flush needed)",
                "parallelism": "dp%d (options sharded, no collective)" % args.gpus}
    return {"workload": "batched Heston calls, uneven grids, HV nt=200 with Rannacher start",
            "options_per_gpu": int(len(w["K"])), "nt": int(w["nt"]),
            "grid_points": int(np.sum(w["nS"].astype(np.int64) * w["nv"])),
            "nS": "uniform {64..512 step 32}", "nv": "uniform {32..256 step 16}",
            "scheme": "2 implicit half-steps + 199 HV steps, theta=1/2+sqrt(3)/6",
            "seed": args.seed, "l2": "state arrays larger than L2 (no flush needed)",
            "parallelism": "dp%d (options sharded, no collective)" % args.gpus}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--options", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--ref-sample", type=int, default=32)
    ap.add_argument("--cpu-sample", type=int, default=32)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="line-solve launch plan from the size heuristic, not the autotuner")
    ap.add_argument("--plan", default=None,
                    help="launch plan as JSON (fdadi_heston_plan_t fields) instead of tuning")
    ap.add_argument("--workload", default="batch",
                    choices=["batch", "large", "surrogate", "gemm", "bs"])
    ap.add_argument("--bs-options", type=int, default=65536,
                    help="options of the batched Black-Scholes workload (--workload bs)")
    ap.add_argument("--train", type=int, default=1 << 17)
    ap.add_argument("--test", type=int, default=1 << 13)
    ap.add_argument("--queries", type=int, default=100000)
    ap.add_argument("--epochs", type=int, default=50)
    ap.add_argument("--sample", type=int, default=2000)
    ap.add_argument("--cv", type=int, default=0, choices=[0, 1, 2],
                    help="surrogate control variate: 0 Black-Scholes at the mean variance, "
                         "1 or 2 plus the vol-of-variance series to that order")
    ap.add_argument("--train-cache", default=None,
                    help="npz with the training set's ADI prices (ptr, dtr) from an earlier "
                         "run on the same seeds")
    ap.add_argument("--compare-cv", action="store_true",
                    help="also train on the same data with the other control variates")
    ap.add_argument("--gate", action="store_true",
                    help="surrogate: train and calibrate the error gate (served error <= 1e-3)")
    ap.add_argument("--gate-margin", type=float, default=0.05,
                    help="error gate: threshold margin below the calibration misses (log10)")
    ap.add_argument("--coarse", default=None,
                    help="surrogate: two-level variant, the coarse-ADI control variate's grid "
                         "as NSxNVxNT (e.g. 128x64x80)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "surrogate":
        return run_surrogate(args) if rank == 0 else 0
    if args.workload == "gemm":
        return run_gemm(args) if rank == 0 else 0
    if args.workload == "bs":
        return run_bs(args) if rank == 0 else 0

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from fd_adi_gb300 import _lib
    from fd_adi_gb300.batch import HestonBatch
    _lib.load()

    # weak scaling: the seeded workload has args.options options per rank and
    # is partitioned across ranks by work (no data-path collective)
    from fd_adi_gb300.shard import shard_of
    w_all = (workload_large() if args.workload == "large"
             else workload(args.options * world, args.seed))
    mine = shard_of(w_all["nS"].astype(np.int64) * w_all["nv"], rank, world)
    w = subset(w_all, mine)
    meshes = meshes_for(w)
    params = params_of(w)
    nt = w["nt"]
    dts = (w["T"] / nt).tolist()
    t_tune = time.perf_counter()
    batch = HestonBatch(params, meshes, scheme="hv", n_steps=nt - 1, dt=dts, theta=HV_THETA,
                        implicit_steps=2, implicit_dt_factor=0.5, graph=True,
                        plan=(json.loads(args.plan) if args.plan else
                              None if args.no_tune else "auto"))
    t_tune = time.perf_counter() - t_tune
    # device-resident inputs (value); e2e prices from the options' parameters
    V0_dev = batch.pack(payoffs(w, meshes))
    V = torch.empty_like(V0_dev)
    # the initial grids are the calls' payoffs, built on the device from the
    # strikes (checked once against the host-built grids)
    K_dev = torch.tensor(w["K"], dtype=torch.float64, device="cuda")
    batch._prepare()
    if not torch.equal(batch.payoff(K_dev, V), V0_dev):
        raise RuntimeError("device payoff differs from the host-built initial grids")
    flat_idx = batch.flat_index([(w["S0"], v0) for v0 in w["v0"]])
    prices = torch.empty(batch.n, dtype=torch.float64, device="cuda")
    stream = batch.stream
    # the batched host mesh generator (timed inside e2e) against the
    # per-option generators (untimed, above), once
    from fd_adi_gb300 import mesh as M
    sb, vb = M.heston_meshes_batch(w["S0"], w["K"], w["v0"], w["nS"], w["nv"], 8.0 * w["K"], 5.0)
    mesh_bitwise = bool(np.array_equal(sb, np.concatenate([m[0] for m in meshes])) and
                        np.array_equal(vb, np.concatenate([m[1] for m in meshes])))
    idx_b = batch.p_off[:-1] + M.price_index_batch(sb, vb, w["nS"], w["nv"], w["S0"], w["v0"])
    mesh_bitwise = mesh_bitwise and bool(np.array_equal(idx_b, flat_idx.cpu().numpy()))
    h_params = np.array(params, dtype=np.float64)
    h_dt = np.asarray(dts, dtype=np.float64)

    def step_device():
        with torch.cuda.stream(stream):
            batch._prepare()
            batch.payoff(K_dev, V)
            batch.run(V)
            batch.gather(V, flat_idx, prices)

    def step_e2e():
        # parameters in, prices out: host meshes and price indices, copies
        # from pinned memory, operators, payoff, time loop, gather, prices back
        return batch.price_calls(w["S0"], w["K"], w["v0"], h_params, h_dt, V=V)

    def steps_e2e(k):
        # the serving loop: k option sets through the pipelined call, each
        # set's host work overlapping the device's work on the set before
        return batch.price_calls_many([(w["S0"], w["K"], w["v0"], h_params, h_dt)] * k, V=V)

    def timed(fn, k):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        ms = e0.elapsed_time(e1) / k
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    ms = timed(step_device, args.steps)
    clk = clocks.stop()
    step_e2e()
    torch.cuda.synchronize()
    clocks_e2e = Clocks(local)
    clocks_e2e.start()
    time.sleep(0.3)
    ke = max(1, args.steps)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    steps_e2e(ke)
    torch.cuda.synchronize()
    ms_e2e = (time.perf_counter() - t_wall) * 1e3 / ke
    if world > 1:
        t = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t.item())
    clk_e2e = clocks_e2e.stop()
    # one unpipelined call: its host share shows in full
    t_single = time.perf_counter()
    step_e2e()
    t_single = (time.perf_counter() - t_single) * 1e3
    t_mesh = time.perf_counter()
    M.heston_meshes_batch(w["S0"], w["K"], w["v0"], w["nS"], w["nv"], 8.0 * w["K"], 5.0)
    t_mesh = (time.perf_counter() - t_mesh) * 1e3
    # the last step's final grids and prices, kept for the parity check (the
    # per-stage timing below advances V again)
    V_final = V.clone()
    prices_final = torch.as_tensor(batch.price_calls_last(), dtype=torch.float64)

    n_total = len(w_all["K"])
    value = n_total / (ms * 1e-3)
    e2e_value = n_total / (ms_e2e * 1e-3)
    h2d = batch.price_calls_h2d_bytes
    d2h = batch.n * 8
    # per step: the run, 4 prepare kernels, the payoff and the price gather
    launches = args.steps * (batch.launches_per_run + 4 + 2)

    out = None
    if rank == 0:
        P = batch.total_points
        st = stage_times(batch, V, torch)
        dom = max(st, key=lambda k: st[k][2])
        avg_ms = st[dom][0]
        hbm_peak, peak_src = measured_peaks()
        ach = STAGE_BYTES[dom] * P / (avg_ms * 1e-3) / 1e9
        fp64, probe = fp64_peak(torch, local)
        fp_ach = STAGE_FLOPS[dom] * P / (avg_ms * 1e-3) / 1e12
        pts_steps = float(P) * nt
        hv_step_ms = sum(st[k][0] for k in HV_STEP_STAGES if k in st)
        hv_step_gbs = HV_STEP_BYTES * P / (hv_step_ms * 1e-3) / 1e9
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64", "data": "synthetic", "config": config_block(args, w),
               "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
                       "api": "HestonBatch.price_calls_many: option parameters in (host "
                              "numpy), prices out (host); each step builds every option's "
                              "meshes and price indices on the host, copies meshes, "
                              "parameters, steps and strikes from pinned memory, rebuilds the "
                              "operators, runs and reads the prices back; step k+1's host "
                              "work overlaps step k's device work (wall clock, K steps)",
                       "host_mesh_ms": round(t_mesh, 2), "mesh_bitwise": mesh_bitwise,
                       "ms_single_call_unpipelined": round(t_single, 1),
                       "clocks": clk_e2e},
               "gpu_launches": int(launches),
               "grid_point_steps_per_s": pts_steps * world / (ms * 1e-3),
               # the dominant kernel is bound by the FP64 pipe: its FP64 work per
               # launch over its event-timed duration, against the live DFMA probe
               "roofline": {"bound": "fp64", "kernel": dom, "achieved": fp_ach, "peak": fp64,
                            "unit": "TFLOP/s", "frac": fp_ach / fp64,
                            "flops_per_point": STAGE_FLOPS[dom],
                            "flops_note": "2 x FP64 instructions per grid point (a DMUL or "
                                          "DADD holds the FP64 pipe like a DFMA)",
                            "peak_source": "measured live: fdadi_fp64_probe, best of 1-16 "
                                           "DFMA chains per thread, ~1.2 s each",
                            "traffic": (NCU_TRAFFIC_B_PER_POINT[dom] * P
                                        if dom in NCU_TRAFFIC_B_PER_POINT else None),
                            "traffic_source": "ncu dram__bytes_read+write per point (256-option "
                                              "capture) x points of this launch",
                            "avg_launch_ms": avg_ms, "launches": st[dom][1],
                            "points_per_launch": int(P),
                            # the same launch against HBM, by the algorithmic
                            # state bytes of this stage
                            "hbm": {"achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                                    "frac": ach / hbm_peak, "bytes_per_point": STAGE_BYTES[dom],
                                    "peak_source": peak_src},
                            # one whole HV step (six stage launches) at 144 B per point
                            "hv_step": {"ms": hv_step_ms, "bytes_per_point": HV_STEP_BYTES,
                                        "gbs": hv_step_gbs, "hbm_frac": hv_step_gbs / hbm_peak}},
               "fp64_probe": probe,
               "stage_ms": {k: round(v[0], 4) for k, v in st.items()},
               # per stage: algorithmic GB/s (state bytes per point x points /
               # launch time) against the HBM copy peak, and the FP64 pipe's share
               "stage_gbs": {k: round(STAGE_BYTES[k] * P / (v[0] * 1e-3) / 1e9, 1)
                             for k, v in st.items()},
               "stage_hbm_frac": {k: round(STAGE_BYTES[k] * P / (v[0] * 1e-3) / 1e9 / hbm_peak, 4)
                                  for k, v in st.items()},
               "stage_fp64_frac": {k: round(STAGE_FLOPS[k] * P / (v[0] * 1e-3) / 1e12 / fp64, 4)
                                   for k, v in st.items()},
               # DRAM traffic (ncu bytes per point x points / launch time)
               # against the HBM copy peak, where a traffic figure exists
               "stage_dram_frac": {k: round(NCU_TRAFFIC_B_PER_POINT[k] * P / (v[0] * 1e-3) / 1e9
                                            / hbm_peak, 4)
                                   for k, v in st.items() if k in NCU_TRAFFIC_B_PER_POINT},
               "plan": dict(batch.plan, tuned=not (args.no_tune or args.plan),
                            setup_s=round(t_tune, 2)),
               "clocks": clk}
        if args.cpu_sample > 0:
            full = args.workload != "large"
            cb = cpu_baseline(w, args.cpu_sample, None if full else 20, want_results=full)
            if full:
                cb, sample = cb
                out["parity"] = parity(batch, V_final, prices_final, sample)
            out["cpu_baseline"] = cb
        if not args.no_extras:
            out["plain_vs_batched"] = plain_vs_batched(torch)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
