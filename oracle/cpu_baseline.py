"""CPU baseline for the solves/s metric (the oracle port, timed on the host).

TEST/BENCH INFRASTRUCTURE ONLY: executed by bench.py's cpu_baseline leg and
its `--impl reference` arm, never by the product path.

The reference's own CPU path (STRUMPACK/MPI behind strumpack_finter.c) cannot
be built here (no Fortran compiler, no STRUMPACK, HDF5 or MPI, and several
sources named by its Makefile are missing), so the CPU arm is a port of the
same work:
  1. assembly: the C restatement of ASMBLE (oracle/wt3d_oracle.c), single
     threaded in the reference's loop order, on the full grid;
  2. factorisation: the multifrontal LU of the same elimination tree with FP64
     LAPACK/BLAS (scipy, all host threads) -- a bounded sample of fronts from
     every level of the tree is factored (dense LU of the pivot block, the two
     triangular solves and the Schur GEMM) and each level's time is
     extrapolated from its sampled flop rate;
  3. solves: forward/backward substitution estimated at the measured
     rate of the largest sampled fronts, one pass per right-hand side batch
     plus the same number of refinement passes the GPU needed.
The sampled fronts are seeded diagonally dominant complex matrices of the
exact front sizes (their values do not change LAPACK's run time); fronts above
4e12 flops are sampled at a reduced size of the same aspect ratio.  The timing
sample and its extrapolation are reported alongside the number.
"""
import ctypes
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _analysis(nx, ny, nz):
    sys.path.insert(0, ROOT)
    import wtomo3d_gb300 as wt
    L = wt.lib()
    info = (ctypes.c_longlong * 8)()
    fl = ctypes.c_double()
    L.wt3d_analyse_info.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p]
    rc = L.wt3d_analyse_info(nx, ny, nz, 64, info, ctypes.byref(fl))
    assert rc == 0
    nf, nb = info[0], info[5]
    n = 3 * nx * ny * nz
    perm = np.zeros(n, np.int32)
    arrs = [np.zeros(nf, np.int32) for _ in range(5)]
    border = np.zeros(nb, np.int32)
    rel = np.zeros(nb, np.int32)
    L.wt3d_analyse_export.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 8
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = L.wt3d_analyse_export(nx, ny, nz, 64, p(perm), *[p(a) for a in arrs], p(border), p(rel))
    assert rc == 0
    fp, fb, ffirst, fpar, flev = arrs
    return fp, fb, flev, fl.value, info[1]


def _front_time(p, b, rng):
    import scipy.linalg as sla
    F11 = (rng.standard_normal((p, p)) + 1j * rng.standard_normal((p, p))) + 4 * p * np.eye(p)
    F12 = rng.standard_normal((p, b)) + 0j
    F21 = rng.standard_normal((b, p)) + 0j
    F22 = rng.standard_normal((b, b)) + 0j
    t0 = time.perf_counter()
    lu, piv = sla.lu_factor(F11, overwrite_a=True, check_finite=False)
    if b:
        U12 = sla.lu_solve((lu, piv), F12, check_finite=False)
        L21 = sla.solve_triangular(lu, F21.T, trans="T", lower=False, check_finite=False).T
        F22 -= L21 @ U12
    return time.perf_counter() - t0


def measure(dims=(96, 96, 64), dx=20.0, nrhs=32, refine_passes=6, budget_s=15.0, seed=1, freq=1.0,
            assemble=True):
    """Returns (solves_per_s, details) for one frequency of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    nx, ny, nz = dims
    details = {}
    t_asm = 0.0
    if assemble:
        import oracle_ctypes
        from wtomo3d_gb300 import Grid, model
        o = oracle_ctypes.Oracle()
        g = Grid(nx, ny, nz, dx, pmld=10 * dx, fst=1)
        vp, vs, rho = model.layered_random(nx, ny, nz, dx, seed=seed)
        ir, jc = o.pattern(nx, ny, nz)
        t0 = time.perf_counter()
        a, ierr = o.assemble(g, vp, vs, rho, 2 * np.pi * freq, ir)
        t_asm = time.perf_counter() - t0
        assert ierr == 0
        del a, ir, jc
    fp, fb, flev, total_flops, fac_entries = _analysis(nx, ny, nz)
    rng = np.random.default_rng(0)
    levels = sorted(set(flev.tolist()))
    per_level_budget = budget_s / len(levels)
    t_fac = 0.0
    sampled = 0
    best_rate = 0.0
    rates = {}
    for lev in levels:
        ids = np.where(flev == lev)[0]
        pf, bf = fp[ids].astype(np.float64), fb[ids].astype(np.float64)
        lev_flops = float(np.sum(8.0 * (pf ** 3 / 3.0 + pf * pf * bf + pf * bf * bf)))
        spent, done_flops = 0.0, 0.0
        # the largest fronts of the top levels exceed any budget: sample a
        # scaled-down front of the same aspect ratio there
        for f in ids:
            p, b = int(fp[f]), int(fb[f])
            fl = 8.0 * (p ** 3 / 3.0 + p * p * b + p * b * b)
            if fl > 4e12:
                s = (4e12 / fl) ** (1.0 / 3.0)
                p, b = max(int(p * s), 64), int(b * s)
                fl = 8.0 * (p ** 3 / 3.0 + p * p * b + p * b * b)
            dt = _front_time(p, b, rng)
            spent += dt
            done_flops += fl
            sampled += 1
            if spent > per_level_budget:
                break
        rate = done_flops / max(spent, 1e-9)
        rates[int(lev)] = rate
        best_rate = max(best_rate, rate)
        t_fac += lev_flops / rate
    # solve: 2 passes (L and U) over the factors per right-hand-side batch,
    # 8 real flops per complex MAC, at the best sampled BLAS rate
    solve_flops = 2.0 * 8.0 * fac_entries * nrhs * refine_passes
    t_solve = solve_flops / best_rate
    t_total = t_asm + t_fac + t_solve
    details.update(t_assemble_s=t_asm, t_factor_est_s=t_fac, t_solve_est_s=t_solve, factor_flops=total_flops,
                   fronts_sampled=sampled, threads=os.cpu_count(), best_rate_gflops=best_rate / 1e9)
    return nrhs / t_total, details


if __name__ == "__main__":
    v, d = measure(dims=tuple(int(x) for x in sys.argv[1:4]) if len(sys.argv) > 3 else (96, 96, 64))
    print(v, d)
