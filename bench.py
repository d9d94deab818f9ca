#!/usr/bin/env python
"""Benchmark of the wtomo3d forward-modelling hot path on GB300.

Metric: solves/s at 96x96x64 (configuration 2: mixed-precision multifrontal
with FP64 refinement to relative residual <= 1e-8).  A step is one frequency
of the workload: assemble A(omega) on the GPU, factor it, and solve its 32
sources with refinement; value = solves / time with every input resident in
HBM, e2e = the same through the host-buffer C ABI (model upload, RHS upload
and solution download inside the timed region), resident = the rate of
solving the sources again on a resident factorisation (alone on the GPU).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs independent replicas (one per GPU, no collective): the path has no
exchange step; every rank factors its own frequency.
"""
import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s @96x96x64 mixed vs FP64 GPU at resid<=1e-8; serve p50/p99 ms"
# ncu capture (--set full) of one k_tc_gemm launch of the GEMM microbenchmark
# (f16 split): dram__bytes_read.sum + dram__bytes_write.sum, and the launch's
# algorithmic bytes (split operands once + C read and written once)
TC_CAPTURE = {"launch": "M=N=8192, K=512 (python -m wtomo3d_gb300.gemm_bench 8192 8192 512), k_tc_gemm<true>",
              "dram_bytes": 1.057372e9 + 0.487806e9, "algorithmic_bytes": 0.1007e9 + 2 * 0.5369e9}
FREQS = [0.5, 1.0, 1.5, 2.0]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev, path=None):
        import tempfile
        self.path = path or os.path.join(tempfile.gettempdir(), "wt3d_clocks_%d_%d.csv" % (dev, os.getpid()))
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        self.dev = dev
        self.p = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx = max(mx, float(c[2]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def plane_wave_sources(nrhs, seed=11):
    """Incidence uniform in [0, 30] degrees, back-azimuth uniform in [0, 360),
    seeded (configuration 2); all incident P waves."""
    rng = np.random.default_rng(seed)
    ain = np.radians(rng.uniform(0.0, 30.0, nrhs))
    ain = np.maximum(ain, np.radians(0.05))     # haskgrn divides by sin(ain)
    baz = np.radians(rng.uniform(0.0, 360.0, nrhs))
    return ain, baz


def workload_config(args, world=1):
    """The workload description shared by every arm (identical dicts)."""
    nrhs = args.nrhs
    nl = args.lanes
    return {"workload": "config2 %dx%dx%d: per frequency assemble A(omega), factor, solve 32 plane-wave sources "
                        "to relres <= tol" % tuple(args.dims), "h_m": 20.0,
            "pml_nodes": 10, "free_surface": True, "usemin": True,
            "model": "4 flat layers Vp 3000-6000, Vs=Vp/1.73, 5% Gaussian-correlated 200 m (seed 1), Gardner rho",
            "freqs_hz": FREQS, "sources_per_step": nrhs,
            "rhs": ("%d Haskell plane-wave P sources per frequency (incidence U[0,30] deg, back-azimuth U[0,360), "
                    "seed 11), scattered-field f = (A_bg - A) u0 against the unperturbed layered background" % nrhs),
            "tol": args.tol,
            "l2": "inputs larger than L2: the factors (74.7 GB complex64 at 96x96x64) are re-read every pass",
            "parallelism": "replicas" if world > 1 else "single GPU",
            "pipelining": "%d solver handles of the same grid, alternate frequencies from %d host threads: "
                          "one frequency's substitution passes overlap the next one's factorisation" % (nl, nl)}


def run_pipelined(n_steps, first, work, nlanes):
    """Runs steps first .. first+n_steps-1; step i on lane i % nlanes, one host
    thread per lane (the library releases the interpreter lock).  Lanes are
    separate solver handles of the same grid: their factorisations are
    serialised by the shared workspace, so one lane's substitution passes
    overlap the other lane's factorisation."""
    import threading
    out = [None] * n_steps
    errs = []

    def lane(l):
        try:
            for i in range(first, first + n_steps):
                if i % nlanes == l:
                    out[i - first] = work(l, i)
        except Exception as exc:   # re-raised below
            errs.append(exc)

    ths = [threading.Thread(target=lane, args=(l,)) for l in range(nlanes)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    if errs:
        raise errs[0]
    return out


def run_ours(args, rank, world, mixed_solutions):
    import ctypes
    import torch
    import wtomo3d_gb300 as wt
    from wtomo3d_gb300 import Grid, model, replicas

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wt.set_device(dev)
    nx, ny, nz = args.dims
    dx = 20.0
    g = Grid(nx, ny, nz, dx, pmld=10 * dx, fst=1, usemin=1)
    vp, vs, rho = model.layered_random(nx, ny, nz, dx, seed=1)
    vp0, vs0, rho0 = model.layered(nx, ny, nz)
    layers = wt.Layered1D(*model.layered1d(nz, dx))
    nrhs = args.nrhs
    ain, baz = plane_wave_sources(nrhs)
    # two lanes (handles) of the same grid, pipelined frequencies; the
    # factorisations' tensor-core GEMM leaves sm_reserve SMs to the other
    # lane's substitution passes
    nl = args.lanes
    wt.set_sm_reserve(args.sm_reserve if nl > 1 else 0)
    t0 = time.perf_counter()
    S = [wt.Solver(g, wt.PREC_MIXED) for _ in range(nl)]
    t_analyse = time.perf_counter() - t0
    dB, dX = [], []
    for s in S:
        s.set_model(vp, vs, rho)
        s.set_background(vp0, vs0, rho0)
        dB.append(torch.zeros((nrhs, g.n), dtype=torch.complex128, device="cuda"))   # n x nrhs column-major
        dX.append(torch.zeros_like(dB[-1]))
    stream = torch.cuda.ExternalStream(S[0].stream)

    def step(l, i):
        s = S[l]
        f = replicas.rank_frequency(i, rank, FREQS)
        s.factor(2 * np.pi * f)
        s.rhs_planewave(layers, ain, baz, d_F=dB[l].data_ptr())
        rr = s.solve_device(dB[l].data_ptr(), dX[l].data_ptr(), nrhs, tol=args.tol, maxit=30)
        st = s.stats()
        return dict(freq=f, relres=float(rr.max()), iters=s.last_iters, factor_ms=st["t_factor_ms"],
                    solve_ms=st["t_solve_ms"], assemble_ms=st["t_assemble_ms"],
                    launches=st["kernels_factor"] + st["kernels_solve"] + 4)   # + background, expansion, source

    run_pipelined(args.warmup, 0, step, nl)
    clocks = Clocks(dev, args.clocks_log)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    recs = run_pipelined(args.steps, args.warmup, step, nl)
    torch.cuda.synchronize()
    e1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = e0.elapsed_time(e1)
    launches = sum(r.pop("launches") for r in recs)
    ms = replicas.max_over_ranks(ms, world, "cuda")
    value = replicas.job_rate(world, nrhs * args.steps, ms / 1e3)

    # ---- end to end through the public API: host model, background and source
    # parameters in, solutions back to pinned host memory ----
    Xh = [torch.empty((nrhs, g.n), dtype=torch.complex128).pin_memory() for _ in range(nl)]
    host_models = [[torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).pin_memory()
                    for a in arrs] for arrs in ((vp, vs, rho), (vp0, vs0, rho0))]
    L = wt.lib()
    last_f = {}

    def e2e_step(l, i):
        s = S[l]
        f = replicas.rank_frequency(i, rank, FREQS)
        last_f[l] = f
        L.wt3d_set_model(s._h, *[ctypes.c_void_p(a.data_ptr()) for a in host_models[0]])
        L.wt3d_set_background(s._h, *[ctypes.c_void_p(a.data_ptr()) for a in host_models[1]])
        s.factor(2 * np.pi * f)
        s.rhs_planewave(layers, ain, baz, d_F=dB[l].data_ptr())
        s.solve_device(dB[l].data_ptr(), dX[l].data_ptr(), nrhs, tol=args.tol, maxit=30)   # returns synchronised
        s.memcpy(Xh[l].data_ptr(), dX[l].data_ptr(), Xh[l].numel() * 16)
        return None

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_pipelined(args.steps, args.warmup, e2e_step, nl)
    torch.cuda.synchronize()
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0, world, "cuda")
    e2e = replicas.job_rate(world, nrhs * args.steps, e2e_s)
    h2d = 2 * sum(a.nbytes for a in (vp, vs, rho)) + ain.nbytes + baz.nbytes
    d2h = Xh[0].numel() * 16

    # ---- (ii) resident-factor rate: each lane's last factorisation stays
    # resident and its right-hand sides are solved again, alone on the GPU
    # (with every SM: the reserve only serves overlapped lanes) ----
    wt.set_sm_reserve(0)
    resident = []
    for l in sorted(last_f):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rr = S[l].solve_device(dB[l].data_ptr(), dX[l].data_ptr(), nrhs, tol=args.tol, maxit=30)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        resident.append({"freq": last_f[l], "solves_per_s": nrhs / dt, "ms": 1e3 * dt, "passes": S[l].last_iters,
                         "relres": float(rr.max())})
        # the mixed-precision wavefields of this frequency, kept on the host for
        # the comparison with the FP64 GPU factorisation
        mixed_solutions[last_f[l]] = (dX[l].cpu().numpy(), rr.copy())
    # the FP64 leg's other frequencies, solved here by the mixed path too
    for f in getattr(args, "fp64_freqs", []) or []:
        if f not in mixed_solutions:
            S[0].factor(2 * np.pi * f)
            S[0].rhs_planewave(layers, ain, baz, d_F=dB[0].data_ptr())
            rr = S[0].solve_device(dB[0].data_ptr(), dX[0].data_ptr(), nrhs, tol=args.tol, maxit=30)
            mixed_solutions[f] = (dX[0].cpu().numpy(), rr.copy())
    s = S[0]

    # ---- roofline of the dominant kernel (one profiled factorisation) ----
    prof = s.profile_factor()
    sprof = s.profile_solve(nrhs)
    st = s.stats()
    pk, pk_src = peaks()
    gemm_ms = prof["gemm_tc_ms"] + prof["gemm_simt_ms"]
    gemm_tflops = prof["gemm_flops"] / (gemm_ms / 1e3) / 1e12
    peak = pk["bf16_tflops_sustained"]
    total_ms = sum(v for k, v in prof.items() if k.endswith("_ms"))
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 fronts (fp32 accumulate, f16-split tensor-core products) + f64 refinement", "data": "synthetic",
        "config": workload_config(args, world),
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "resident": resident,
        "gpu_launches": launches,
        "roofline": {"bound": "tensor", "kernel": "k_tc_gemm (tcgen05 f16-split front Schur/trailing updates)",
                     "achieved": gemm_tflops, "peak": peak, "unit": "TFLOP/s", "frac": gemm_tflops / peak,
                     "peak_source": "%s bf16_tflops_sustained" % pk_src,
                     "gemm_time_share": gemm_ms / total_ms,
                     # DRAM bytes of one captured launch of this kernel: a whole
                     # factorisation's DRAM capture takes several ncu passes, which
                     # the capture rules allow only on a small case
                     "traffic": TC_CAPTURE["dram_bytes"],
                     "traffic_launch": TC_CAPTURE["launch"],
                     "traffic_algorithmic": TC_CAPTURE["algorithmic_bytes"]},
        "steps_detail": recs,
        "factor": {"flops": st["factor_flops"], "entries": st["factor_entries"], "fronts": st["nfronts"],
                   "bytes": st["factor_bytes"], "analyse_s": t_analyse, "profile_ms": prof},
        "solve_pass_profile_ms": sprof,
        "clocks": ck,
    }
    # release torch's handles on the library stream before the handles (and
    # their streams) are destroyed
    del stream, e0, e1, dB, dX, Xh
    torch.cuda.synchronize()
    for h in S:
        h.close()
    wt.set_sm_reserve(0)
    return out


def assembly_rate(dims, reps=3):
    """Device assembly of A (complex128 CSR values) at 1 Hz on a grid, in HBM
    bytes per second: algorithmic bytes = nnz x 16 written + 3 x 4 bytes of
    model per node read + (n + 1) x 4 bytes of row pointers read."""
    import ctypes
    import torch
    import wtomo3d_gb300 as wt
    from wtomo3d_gb300 import Grid, model
    nx, ny, nz = dims
    g = Grid(nx, ny, nz, 20.0, pmld=(12 if nx >= 128 else 10) * 20.0, fst=1, usemin=1)
    # row pointers from the closed form: 3 rows per node of 3 * (3x3x3 box clipped) entries
    def cnt(n):
        c = np.full(n, 3)
        c[0] -= 1
        c[-1] -= 1
        return c
    cz, cx, cy = cnt(nz), cnt(nx), cnt(ny)
    per_node = 3 * (cz[:, None, None] * cx[None, :, None] * cy[None, None, :]).reshape(-1, order="F")
    rows = np.repeat(per_node, 3)
    irptr = np.zeros(3 * nx * ny * nz + 1, np.int32)
    irptr[1:] = np.cumsum(rows)
    nnz = int(irptr[-1])
    vp, vs, rho = [torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).cuda()
                   for a in model.layered_random(nx, ny, nz, 20.0, seed=1)]
    dir_ = torch.from_numpy(irptr).cuda()
    da = torch.empty(nnz, dtype=torch.complex128, device="cuda")
    st = torch.cuda.Stream()
    L = wt.lib()
    L.wt3d_assemble_device.argtypes = [ctypes.POINTER(Grid), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
    args = (ctypes.byref(g), ctypes.c_void_p(vp.data_ptr()), ctypes.c_void_p(vs.data_ptr()),
            ctypes.c_void_p(rho.data_ptr()), 2 * np.pi, 0.0, ctypes.c_void_p(dir_.data_ptr()),
            ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(st.cuda_stream))
    torch.cuda.synchronize()
    if L.wt3d_assemble_device(*args):
        raise RuntimeError(L.wt3d_last_error().decode())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        L.wt3d_assemble_device(*args)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    nbytes = nnz * 16 + nx * ny * nz * 12 + (3 * nx * ny * nz + 1) * 4
    pk, src = peaks()
    out = {"dims": list(dims), "nnz": nnz, "bytes": nbytes, "ms": ms, "gb_per_s": nbytes / ms / 1e6,
           "frac": nbytes / ms / 1e6 / pk["hbm_gbs"], "peak_source": "%s hbm_gbs" % src,
           "note": "includes the per-node Lame conversion of the model (one small kernel)"}
    del vp, vs, rho, dir_, da, st
    torch.cuda.synchronize()
    return out


def run_serve(args):
    """Serving loop (configuration 3): a seeded Poisson stream of requests over
    grids 48^3, 64^3 and 96x96x64 (weights 0.5/0.35/0.15), model seeds from a
    pool of 8, frequencies {0.5, 1, 1.5, 2} Hz, 1-64 sources (75% plane
    waves, 25% point forces); factorisations resident under a 120 GB budget
    with LRU eviction, right-hand sides batched per factorisation.  Latency =
    arrival to solution on the host."""
    from wtomo3d_gb300 import serve
    # two factorisation workspaces per grid: two keys of one grid factor at once
    be = serve.GpuBackend(dx=20.0, pml_nodes=10, tol=args.tol, maxit=30, workspaces_per_grid=2)
    grids = ((48, 48, 48), (64, 64, 64), (96, 96, 64))
    for g in grids:          # host analyses of the three grids, computed once per process
        be.bytes_needed((g, 0, 1.0))
    def one(stream, desc):
        srv = serve.Server(be, budget_bytes=120e9, max_batch=64, workers=4)
        try:
            summ = srv.run(stream, timeout_s=900)
        finally:
            srv.close()
        summ = {k: (float("%.4g" % v) if isinstance(v, float) else v) for k, v in summ.items()}
        summ.update({"workload": desc, "hit_rate": round(summ["hits"] / max(1, summ["requests"]), 3)})
        return summ

    out = one(serve.make_stream(args.serve_requests, rate_hz=args.serve_rate, seed=7, grids=grids),
              "config3 serving: Poisson %.2f req/s, %d requests (seed 7), grids 48^3/64^3/96x96x64 "
              "(0.5/0.35/0.15), model pool 8, f in {0.5,1,1.5,2} Hz, 1-64 sources (75%% plane, 25%% "
              "point), budget 120 GB resident factors, LRU, RHS batched per factor, 4 workers"
              % (args.serve_rate, args.serve_requests))
    if args.serve_reuse_requests > 0:
        # a stream whose keys recur, as in a survey where many shots share a
        # model and a frequency: 2 models, 2 frequencies, 64^3 and 96x96x64
        out["reuse"] = one(serve.make_stream(args.serve_reuse_requests, rate_hz=args.serve_reuse_rate, seed=8,
                                             grids=grids[1:], grid_weights=(0.6, 0.4), freqs=(1.0, 2.0),
                                             n_models=2),
                           "config3 serving, key reuse: Poisson %.2f req/s, %d requests (seed 8), grids "
                           "64^3/96x96x64 (0.6/0.4), model pool 2, f in {1,2} Hz, 1-64 sources, same budget "
                           "and batching" % (args.serve_reuse_rate, args.serve_reuse_requests))
    import wtomo3d_gb300 as wt
    wt.lib().wt3d_set_workspaces_per_grid(1)
    return out


def run_fp64_leg(args, mixed_solutions):
    """The FP64 GPU factorisation oracle on the same workload: complex128
    fronts (FP64 SIMT kernels) and the same FP64 refinement, one frequency per
    step, device-resident inputs.  Every frequency of args.fp64_freqs is
    factored once; its 32 wavefields are compared with the mixed-precision
    wavefields of the same frequency (err = max over sources of
    ||x_mixed - x_fp64|| / ||x_fp64||)."""
    import torch
    import wtomo3d_gb300 as wt
    from wtomo3d_gb300 import Grid, model
    nx, ny, nz = args.dims
    dx = 20.0
    g = Grid(nx, ny, nz, dx, pmld=10 * dx, fst=1, usemin=1)
    torch.cuda.empty_cache()
    s = wt.Solver(g, wt.PREC_FP64)
    s.set_model(*model.layered_random(nx, ny, nz, dx, seed=1))
    s.set_background(*model.layered(nx, ny, nz))
    layers = wt.Layered1D(*model.layered1d(nz, dx))
    ain, baz = plane_wave_sources(args.nrhs)
    dB = torch.zeros((args.nrhs, g.n), dtype=torch.complex128, device="cuda")
    dX = torch.zeros_like(dB)
    recs, errs = [], {}
    t_total = 0.0
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    try:
        for f in args.fp64_freqs:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.factor(2 * np.pi * f)
            s.rhs_planewave(layers, ain, baz, d_F=dB.data_ptr())
            rr = s.solve_device(dB.data_ptr(), dX.data_ptr(), args.nrhs, tol=args.tol, maxit=30)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            st = s.stats()
            t_total += dt
            rec = dict(freq=f, relres=float(rr.max()), iters=s.last_iters, factor_ms=st["t_factor_ms"],
                       solve_ms=st["t_solve_ms"], step_s=dt)
            if f in mixed_solutions:
                Xm, rrm = mixed_solutions[f]
                X64 = dX.cpu().numpy()
                e = np.linalg.norm(Xm - X64, axis=1) / np.linalg.norm(X64, axis=1)
                errs[f] = float(e.max())
                rec.update(err_vs_fp64=float(e.max()), err_vs_fp64_median=float(np.median(e)),
                           mixed_relres=float(rrm.max()))
            recs.append(rec)
    finally:
        ck = clocks.stop()
        del dB, dX
        torch.cuda.synchronize()
        st = s.stats()
        s.close()
    value = args.nrhs * len(args.fp64_freqs) / t_total
    return {"impl": "fp64-gpu-oracle", "value": value, "unit": "solves/s",
            "ms_per_step": 1e3 * t_total / len(args.fp64_freqs), "steps": len(args.fp64_freqs),
            "dtype": "c128 fronts (fp64) + f64 refinement", "factor_flops": st["factor_flops"],
            "note": "one frequency per step: factorisation + plane-wave sources + solves, inputs resident",
            "steps_detail": recs, "clocks": ck}, errs


def run_cpu(args, steps, warmup, workload=None):
    """The CPU port (oracle/cpu_baseline.py) over `steps` frequencies after
    `warmup` untimed ones: full single-thread assembly plus a sampled
    multifrontal factor and substitution per frequency."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cpu_baseline
    w = workload or cpu_baseline.Workload(tuple(args.dims))
    t_est, dets = 0.0, []
    try:
        for i in range(warmup + steps):
            v, det = w.step(FREQS[i % len(FREQS)], args.nrhs, args.cpu_budget, i)
            if i >= warmup:
                t_est += args.nrhs / v
                dets.append(det)
    finally:
        if workload is None:
            w.close()
    v = args.nrhs * steps / t_est
    sample = ("per frequency: the oracle's C assembly of the full %dx%dx%d operator (1 thread, timed in full) + "
              "the FP64 multifrontal (numpy/LAPACK) on a %.1f s sample of fronts from every level of its own "
              "nested-dissection tree, levels with at least one front per core at the single-core rate divided by "
              "the core count, the others with threaded BLAS; factor extrapolated by flops, one forward + backward "
              "substitution of the 32 sources by factor entries (an FP64 factor needs one pass for 1e-8)"
              % (tuple(args.dims) + (args.cpu_budget,)))
    agg = {k: float(np.mean([d[k] for d in dets])) for k in ("t_assemble_s", "t_factor_est_s", "t_solve_est_s")}
    agg.update(threads=w.threads, factor_flops=w.tree["flops"], factor_entries=w.tree["entries"], steps=steps)
    return v, {"value": v, "unit": "solves/s", "cores": w.threads, "kind": "port", "sample": sample,
               "detail": agg}


def run_general(dims, nrhs=8, seed=5):
    """The benchmark's operator (1 Hz, layered random model) through the
    general-pattern path: the grid handle (plane separators) against a handle
    of the same matrix under a random node permutation
    (wt3d_solver_create_csr: multilevel ordering on the host, then the same
    kernels).  Times are host wall clock around synchronous calls."""
    import scipy.sparse as sp
    import wtomo3d_gb300 as wt
    from wtomo3d_gb300 import Grid, model
    nx, ny, nz = dims
    g = Grid(nx, ny, nz, 20.0, pmld=200.0, fst=1)
    vp, vs, rho = model.layered_random(nx, ny, nz, 20.0, seed=1)
    om = 2 * np.pi * 1.0
    ir, jc = wt.pattern(nx, ny, nz, base=0)
    A = sp.csr_matrix((wt.assemble(g, vp, vs, rho, om), jc, ir), shape=(g.n, g.n))
    q = np.random.default_rng(seed).permutation(g.nnodes)
    perm = (3 * q[:, None] + np.arange(3)).reshape(-1)
    Ap = sp.csr_matrix(A[perm][:, perm])
    Ap.sort_indices()
    rng = np.random.default_rng(seed + 1)
    B = np.zeros((g.n, nrhs), complex)
    for j in range(nrhs):   # point forces away from the Dirichlet faces
        node = rng.integers(0, nz - 1) + nz * (rng.integers(1, nx - 1) + nx * rng.integers(1, ny - 1))
        B[3 * node + rng.integers(0, 3), j] = 1.0
    out, X = {"workload": "%dx%dx%d, 1 Hz, %d point forces, node-permuted operator" % (nx, ny, nz, nrhs)}, {}
    for name in ("grid", "general"):
        t0 = time.perf_counter()
        s = wt.Solver(g) if name == "grid" else wt.Solver.from_csr(Ap.indptr, Ap.indices)
        t1 = time.perf_counter()
        if name == "grid":
            s.set_model(vp, vs, rho)
            t2 = time.perf_counter()
            s.factor(om)
        else:
            a = np.ascontiguousarray(Ap.data)
            wt._check(wt.lib().wt3d_set_values_c128(s._h, wt._ptr(a)))
            t2 = time.perf_counter()
            wt._check(wt.lib().wt3d_factor_values(s._h))
        t3 = time.perf_counter()
        X[name] = s.solve(B if name == "grid" else B[perm], tol=1e-8)
        t4 = time.perf_counter()
        st = s.stats()
        out[name] = {"analysis_s": t1 - t0, "factor_s": t3 - t2, "solve_s": t4 - t3, "solves_per_s": nrhs / (t4 - t3),
                     "refinement_steps": s.last_iters, "relres_max": float(s.last_relres.max()),
                     "factor_entries": st["factor_entries"], "factor_flops": st["factor_flops"]}
        s.close()
    out["wavefield_rel_diff"] = float(np.linalg.norm(X["grid"][perm] - X["general"]) / np.linalg.norm(X["grid"]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dims", type=int, nargs=3, default=[96, 96, 64])
    ap.add_argument("--nrhs", type=int, default=32)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--cpu-budget", type=float, default=2.0, help="seconds of sampled fronts per CPU step")
    ap.add_argument("--no-c1", action="store_true", help="reference arm: skip the full 40^3 CPU factor and solve")
    ap.add_argument("--fp64-freqs", type=lambda t: [float(x) for x in t.split(",") if x],
                    default=[0.5], help="frequencies of the FP64 GPU factorisation leg (one factorisation takes "
                    "~6 min; 0.5 Hz is the frequency where the mixed solve needs GMRES; '' skips it)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--clocks-log", default=None, help="file for the nvidia-smi samples of the timed region")
    ap.add_argument("--lanes", type=int, default=2, help="pipelined solver handles (1 = sequential steps)")
    ap.add_argument("--sm-reserve", type=int, default=0, help="SMs the factorisation GEMM leaves to the other lane")
    ap.add_argument("--serve-requests", type=int, default=30)
    ap.add_argument("--serve-rate", type=float, default=0.3)
    ap.add_argument("--serve-reuse-requests", type=int, default=30)
    ap.add_argument("--serve-reuse-rate", type=float, default=0.5)
    ap.add_argument("--general-pattern", type=int, nargs=3, default=None, metavar=("NX", "NY", "NZ"),
                    help="only time the general-pattern path against the grid path at this size")
    args = ap.parse_args()
    if args.general_pattern:
        print(json.dumps({"general_pattern": run_general(tuple(args.general_pattern))}))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))

    if args.impl == "reference":
        # the CPU port on the host cores; rank 0 only, the other ranks exit
        if rank != 0:
            return
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import cpu_baseline
        t0 = time.perf_counter()
        w = cpu_baseline.Workload(tuple(args.dims))
        try:
            v, cb = run_cpu(args, args.steps, args.warmup, workload=w)
        finally:
            w.close()
        wall = time.perf_counter() - t0
        out = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": 1e3 * args.nrhs / v, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "impl": "reference", "dtype": "c128 (fp64)", "data": "synthetic",
               "config": workload_config(args, world), "cpu_baseline": cb,
               "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "note": ("the reference's STRUMPACK/MPI path cannot be built here (no Fortran compiler, STRUMPACK, "
                        "HDF5 or MPI; sources missing from its tree): its CPU port is timed instead, with each "
                        "frequency's factor and substitution extrapolated from a sample (ms_per_step is that "
                        "estimate; wall_s is the arm's own run time)"),
               "wall_s": wall}
        if not args.no_c1:
            out["c1_full"] = cpu_baseline.config1_full()
        print(json.dumps(out))
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    mixed_solutions = {}
    out = run_ours(args, rank, world, mixed_solutions)
    if rank == 0:
        # assembly throughput at the benchmark grid and at the largest grid
        # (128x128x96, 12-node PML), whose factors do not fit one GPU
        out["assembly"] = [assembly_rate(tuple(args.dims)), assembly_rate((128, 128, 96))]
    if rank == 0 and not args.no_serve:
        out["serve"] = run_serve(args)
    if rank == 0 and args.fp64_freqs:
        fp, errs = run_fp64_leg(args, mixed_solutions)
        out["fp64"] = fp
        out["mixed_over_fp64"] = out["value"] / fp["value"]
        if errs:
            out["err_vs_fp64"] = max(errs.values())
            out["err_vs_fp64_by_freq"] = {str(k): v for k, v in errs.items()}
    if rank == 0:
        if not args.no_cpu:
            v, cb = run_cpu(args, 1, 0)
            out["cpu_baseline"] = cb
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
