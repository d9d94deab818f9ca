"""CPU baseline for the solves/s metric: the oracle port, timed on the host.

TEST/BENCH INFRASTRUCTURE ONLY: executed by bench.py's cpu_baseline leg and
its `--impl reference` arm, never by the product path.  It loads only the
oracle's own library (oracle/_build/libwt3d_oracle.so) and numpy/scipy: no
part of the product library.

The reference's own CPU path (STRUMPACK/MPI behind strumpack_finter.c) cannot
be built here (no Fortran compiler, no STRUMPACK, HDF5 or MPI, and several
sources named by its Makefile are missing), so the CPU arm is a port of the
same work:
  1. assembly: the C restatement of ASMBLE (oracle/wt3d_oracle.c, pinned bit
     for bit to the reference's statements), single threaded in the
     reference's loop order, on the full grid -- timed in full;
  2. factorisation and solves: the FP64 multifrontal LU of
     oracle/cpu_multifrontal.py (LAPACK/BLAS on every host thread) over its
     own nested-dissection tree.  At the benchmark grid a whole factorisation
     takes tens of minutes, so each step times a bounded sample of fronts from
     every level (dense LU of the pivot block, the two triangular solves and
     the Schur GEMM, then one forward and one backward substitution of the
     step's right-hand sides through the same front) and extrapolates each
     level by its sampled flop rate (factor) and entry rate (substitution);
  3. on the configuration-1 grid (40^3) the same multifrontal runs in full,
     factor and solve, and its measured time is set beside the estimate the
     sampling method gives for that grid.
An FP64 direct factorisation reaches the 1e-8 residual in one substitution
pass, which is what the estimate counts.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))
for _p in (HERE, ROOT, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import cpu_multifrontal as cmf  # noqa: E402


def threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class Workload:
    """The configuration-2 grid with its model, elimination tree and the
    oracle library, set up once."""

    def __init__(self, dims=(96, 96, 64), dx=20.0, seed=1):
        import oracle_ctypes
        from wtomo3d_gb300 import Grid, model
        self.dims = tuple(dims)
        nx, ny, nz = dims
        self.o = oracle_ctypes.Oracle()
        self.g = Grid(nx, ny, nz, dx, pmld=10 * dx, fst=1, usemin=1)
        self.model = model.layered_random(nx, ny, nz, dx, seed=seed)
        self.ir, self.jc = self.o.pattern(nx, ny, nz)
        t0 = time.perf_counter()
        self.tree = cmf.nd_tree(nx, ny, nz)
        self.t_tree = time.perf_counter() - t0
        self.threads = threads()
        self.serial = cmf.SerialSampler() if self.threads > 1 else None

    def close(self):
        if self.serial is not None:
            self.serial.close()
            self.serial = None

    def step(self, freq, nrhs, budget_s, seed):
        """One frequency: full single-thread assembly (timed) + sampled
        factor and substitution estimate.  Returns (solves_per_s, detail)."""
        t0 = time.perf_counter()
        a, ierr = self.o.assemble(self.g, *self.model, 2 * np.pi * freq, self.ir)
        t_asm = time.perf_counter() - t0
        assert ierr == 0
        del a
        t_fac, t_sol, det = cmf.sampled_rate(self.tree, nrhs, 1, budget_s, seed=seed, serial=self.serial,
                                             nthreads=self.threads)
        total = t_asm + t_fac + t_sol
        det.update(freq=freq, t_assemble_s=t_asm, t_factor_est_s=t_fac, t_solve_est_s=t_sol)
        return nrhs / total, det


def config1_full(budget_s=3.0):
    """Configuration 1 in full on the CPU: 40^3, h = 25 m, homogeneous
    (5000, 2887, 2700), 10-node PML on all faces, 1 Hz, vertical point force
    at the centre node; complex128 assembly (oracle), FP64 multifrontal factor
    and solve.  Also the sampled estimate of the same factor and solve, to
    show how far the extrapolation used at the benchmark grid is off."""
    import oracle_ctypes
    import scipy.sparse as sp
    from wtomo3d_gb300 import Grid, model
    o = oracle_ctypes.Oracle()
    n1 = 40
    g = Grid(n1, n1, n1, 25.0, pmld=250.0, fst=0, usemin=1)
    vp, vs, rho = model.homogeneous(n1, n1, n1)
    ir, jc = o.pattern(n1, n1, n1)
    t0 = time.perf_counter()
    a, ierr = o.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir)
    t_asm = time.perf_counter() - t0
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    c = (n1 - 1) * 25.0 / 2
    b = model.point_force(n1, n1, n1, 25.0, c, c, c, comp=2)
    t = cmf.nd_tree(n1, n1, n1)
    X, t_fac, t_sol = cmf.timed_full(A, t, b.reshape(-1, 1))
    relres = float(np.linalg.norm(b - A @ X[:, 0]) / np.linalg.norm(b))
    # the same estimate with the fronts run one after another (as timed_full
    # does) and with one front per core (as the benchmark-grid estimate does)
    e_fac1, e_sol1, _ = cmf.sampled_rate(t, 1, 1, budget_s, seed=3)
    ser = cmf.SerialSampler() if threads() > 1 else None
    try:
        e_fac, e_sol, _ = cmf.sampled_rate(t, 1, 1, budget_s, seed=3, serial=ser, nthreads=threads())
    finally:
        if ser is not None:
            ser.close()
    return {"grid": [n1, n1, n1], "t_assemble_s": t_asm, "t_factor_s": t_fac, "t_solve_s": t_sol,
            "relres": relres, "factor_flops": t["flops"], "factor_gflops": t["flops"] / t_fac / 1e9,
            "factor_entries": t["entries"], "estimate_sequential_t_factor_s": e_fac1,
            "estimate_sequential_t_solve_s": e_sol1, "estimate_t_factor_s": e_fac, "estimate_t_solve_s": e_sol,
            "sequential_estimate_over_measured_factor": e_fac1 / t_fac, "threads": threads()}


def measure(dims=(96, 96, 64), nrhs=32, budget_s=3.0, freq=1.0, seed=0, workload=None):
    """One sampled step (for the cpu_baseline leg of the GPU arm)."""
    w = workload or Workload(dims)
    try:
        v, det = w.step(freq, nrhs, budget_s, seed)
    finally:
        if workload is None:
            w.close()
    det.update(threads=threads(), factor_flops=w.tree["flops"], factor_entries=w.tree["entries"],
               t_tree_s=w.t_tree)
    return v, det


if __name__ == "__main__":
    print(measure(dims=tuple(int(x) for x in sys.argv[1:4]) if len(sys.argv) > 3 else (96, 96, 64)))
