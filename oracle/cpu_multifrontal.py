"""FP64 CPU multifrontal LU over a geometric nested dissection (TEST AND BENCH
INFRASTRUCTURE ONLY: the CPU baseline of bench.py and a checker in tests/).

The reference factors through STRUMPACK (strumpack_finter.c:32-117): a
multifrontal sparse LU over a METIS nested-dissection ordering, dense BLAS-3
front by front, threaded on the host.  STRUMPACK is not in the reference tree
and cannot be built here, so this module restates that method with numpy /
LAPACK (threaded BLAS on every host core):

  ordering   one-node coordinate planes bisect the longest axis of a box
             (a vertex separator of the 27-point graph: no stencil edge
             crosses it); boxes of at most `leaf` nodes, or too thin to cut,
             are leaves; nodes are numbered box by box in postorder, (y, x, z)
             loops inside a box;
  structure  the border of a front is every grid node in the one-node shell
             around the box of its subtree (all of them lie on ancestor
             separators, so all are numbered later), 3 dofs each;
  factor     per front: scatter the operator's entries, extend-add the
             children's Schur complements, partial pivoted LU of the pivot
             block, U12 = L11^-1 F12, L21 = F21 U11^-1, F22 -= L21 U12;
  solve      forward sweep leaves to root, backward sweep root to leaves,
             many right-hand sides at once.

Nothing here calls the product library.
"""
import os
import time

import numpy as np


def _shell_nodes(lo, hi, dims):
    """Grid nodes (x, y, z) in the one-node shell around box [lo, hi)."""
    elo = [max(l - 1, 0) for l in lo]
    ehi = [min(h + 1, d) for h, d in zip(hi, dims)]
    xs, ys, zs = (np.arange(a, b) for a, b in zip(elo, ehi))
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    inside = ((X >= lo[0]) & (X < hi[0]) & (Y >= lo[1]) & (Y < hi[1]) & (Z >= lo[2]) & (Z < hi[2]))
    return X[~inside], Y[~inside], Z[~inside]


def nd_tree(nx, ny, nz, leaf=64):
    """Nested-dissection fronts of the nx*ny*nz grid (3 dofs per node).

    Returns a dict: p, b, first, level, parent (per front, postorder),
    perm (new dof -> natural dof), border (concatenated new dof indices of
    every front's border, ascending per front), boff (offsets into border),
    flops (sum 8 (p^3/3 + p^2 b + p b^2)), entries (sum p^2 + 2 p b)."""
    dims = (nx, ny, nz)
    nn = nx * ny * nz
    newnode = np.full(nn, -1, np.int64)
    fronts = []           # (p, level, box lo, box hi, first node, children)
    counter = [0]

    def nid(x, y, z):
        return z + nz * (x + nx * y)

    def number(lo, hi):
        first = counter[0]
        ys, xs, zs = np.meshgrid(np.arange(lo[1], hi[1]), np.arange(lo[0], hi[0]), np.arange(lo[2], hi[2]),
                                 indexing="ij")
        g = nid(xs.ravel(), ys.ravel(), zs.ravel())
        newnode[g] = np.arange(first, first + len(g))
        counter[0] += len(g)
        return first, len(g)

    # explicit stack: (lo, hi, depth, state)
    def build(lo, hi, depth):
        ln = [h - l for l, h in zip(lo, hi)]
        ax = 0
        for a in (1, 2):
            if ln[a] > ln[ax]:
                ax = a
        vol = ln[0] * ln[1] * ln[2]
        if vol <= leaf or ln[ax] < 3:
            first, cnt = number(lo, hi)
            fronts.append([3 * cnt, depth, lo, hi, first, []])
            return len(fronts) - 1
        m = (lo[ax] + hi[ax]) // 2
        lo1, hi1 = list(lo), list(hi)
        hi1[ax] = m
        lo2, hi2 = list(lo), list(hi)
        lo2[ax] = m + 1
        c1 = build(lo1, hi1, depth + 1)
        c2 = build(lo2, hi2, depth + 1)
        slo, shi = list(lo), list(hi)
        slo[ax], shi[ax] = m, m + 1
        first, cnt = number(slo, shi)
        fronts.append([3 * cnt, depth, lo, hi, first, [c1, c2]])
        return len(fronts) - 1

    import sys
    old = sys.getrecursionlimit()
    sys.setrecursionlimit(max(old, 10000))
    try:
        build([0, 0, 0], [nx, ny, nz], 0)
    finally:
        sys.setrecursionlimit(old)
    nf = len(fronts)
    p = np.array([f[0] for f in fronts], np.int64)
    level = np.array([f[1] for f in fronts], np.int64)
    first = np.array([3 * f[4] for f in fronts], np.int64)
    parent = np.full(nf, -1, np.int64)
    for i, f in enumerate(fronts):
        for c in f[5]:
            parent[c] = i
    b = np.zeros(nf, np.int64)
    borders = []
    for i, f in enumerate(fronts):
        X, Y, Z = _shell_nodes(f[2], f[3], dims)
        w = np.sort(newnode[nid(X, Y, Z)])
        dof = (3 * w[:, None] + np.arange(3)[None, :]).ravel()
        borders.append(dof)
        b[i] = len(dof)
    boff = np.concatenate([[0], np.cumsum(b)])
    node_of_new = np.empty(nn, np.int64)
    node_of_new[newnode] = np.arange(nn)
    perm = (3 * node_of_new[:, None] + np.arange(3)[None, :]).ravel()
    pf, bf = p.astype(np.float64), b.astype(np.float64)
    return dict(p=p, b=b, first=first, level=level, parent=parent, perm=perm,
                border=np.concatenate(borders) if borders else np.zeros(0, np.int64), boff=boff,
                children=[f[5] for f in fronts],
                flops=float(np.sum(8.0 * (pf ** 3 / 3.0 + pf * pf * bf + pf * bf * bf))),
                entries=int(np.sum(p * p + 2 * p * b)))


def factor(A, t):
    """Multifrontal LU of the natural-order sparse matrix A (scipy CSR,
    complex128) over tree t.  Returns the list of per-front factors."""
    import scipy.linalg as sla
    perm = t["perm"]
    Ap = A[perm][:, perm].tocsr()
    nf = len(t["p"])
    upd = {}
    facs = []
    for f in range(nf):
        p, first = int(t["p"][f]), int(t["first"][f])
        bidx = t["border"][t["boff"][f]:t["boff"][f + 1]]
        idx = np.concatenate([np.arange(first, first + p), bidx])
        b = len(bidx)
        F = np.zeros((p + b, p + b), complex)
        F[:p, :] = Ap[first:first + p][:, idx].toarray()
        if b:
            F[p:, :p] = Ap[bidx][:, first:first + p].toarray()
        pos = {int(d): k for k, d in enumerate(idx)}
        for c in t["children"][f]:
            if c in upd:
                U, cb = upd.pop(c)
                rel = np.array([pos[int(d)] for d in cb])
                F[np.ix_(rel, rel)] += U
        lu, piv = sla.lu_factor(F[:p, :p], overwrite_a=True, check_finite=False)
        U12 = sla.lu_solve((lu, piv), F[:p, p:], check_finite=False) if b else np.zeros((p, 0), complex)
        L21 = F[p:, :p].copy()
        if b:
            upd[f] = (F[p:, p:] - L21 @ U12, bidx)
        facs.append((lu, piv, U12, L21, first, p, bidx))
    return facs


def solve(facs, t, B):
    """X = A^-1 B for the natural-order right-hand sides B (n x m)."""
    import scipy.linalg as sla
    perm = t["perm"]
    Y = np.array(B, complex, copy=True)[perm]
    for lu, piv, U12, L21, first, p, bidx in facs:
        z = sla.lu_solve((lu, piv), Y[first:first + p], check_finite=False)
        if len(bidx):
            Y[bidx] -= L21 @ z
        Y[first:first + p] = z
    for lu, piv, U12, L21, first, p, bidx in reversed(facs):
        if len(bidx):
            Y[first:first + p] -= U12 @ Y[bidx]
    X = np.empty_like(Y)
    X[perm] = Y
    return X


def timed_full(A, t, B):
    """Full factor and solve with wall times: (X, t_factor_s, t_solve_s)."""
    t0 = time.perf_counter()
    facs = factor(A, t)
    t1 = time.perf_counter()
    X = solve(facs, t, B)
    t2 = time.perf_counter()
    return X, t1 - t0, t2 - t1


def _front_factor_time(p, b, rng):
    """Dense work of one front of the given shape (values do not change
    LAPACK's run time): LU of the pivot block, the two triangular solves and
    the Schur update."""
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
    return time.perf_counter() - t0, (lu, piv, U12 if b else None, L21 if b else None)


def _front_solve_time(p, b, fac, m, rng):
    """One forward and one backward substitution of m right-hand sides
    through a front: the triangular solves with its pivot block and the two
    border products."""
    import scipy.linalg as sla
    lu, piv, U12, L21 = fac
    Y = rng.standard_normal((p, m)) + 1j * rng.standard_normal((p, m))
    Yb = rng.standard_normal((b, m)) + 1j * rng.standard_normal((b, m))
    t0 = time.perf_counter()
    z = sla.lu_solve((lu, piv), Y, check_finite=False)
    if b:
        Yb -= L21 @ z
        z -= U12 @ Yb
    return time.perf_counter() - t0


def sample_fronts(shapes, nrhs, budget_s, max_front_flops, seed):
    """Factors and substitutes fronts of the given (p, b) shapes, in order,
    until budget_s is spent.  Fronts above max_front_flops are replaced by a
    smaller front of the same aspect ratio.  Returns (flops, entries,
    factor seconds, substitution seconds) of what was done."""
    rng = np.random.default_rng(seed)
    fl_done = ent_done = t_fac = t_sol = 0.0
    for p, b in shapes:
        p, b = int(p), int(b)
        fl = 8.0 * (p ** 3 / 3.0 + p * p * b + p * b * b)
        if fl > max_front_flops:
            s = (max_front_flops / fl) ** (1.0 / 3.0)
            p, b = max(int(p * s), 48), int(b * s)
            fl = 8.0 * (p ** 3 / 3.0 + p * p * b + p * b * b)
        dt, fac = _front_factor_time(p, b, rng)
        ds = _front_solve_time(p, b, fac, nrhs, rng)
        t_fac += dt
        t_sol += ds
        fl_done += fl
        ent_done += p * p + 2.0 * p * b
        if t_fac + t_sol > budget_s:
            break
    return fl_done, ent_done, t_fac, t_sol


class SerialSampler:
    """One worker process whose BLAS runs on a single thread (its
    environment is set before it starts), for the levels with at least as
    many fronts as host threads: a multifrontal solver runs those fronts
    concurrently, one per core (subtree parallelism), so a level's time is
    its work at the single-core rate divided by the thread count.  Started
    with the spawn method, so it is safe after CUDA has been initialised."""

    def __init__(self):
        import multiprocessing as mp
        keep = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")}
        for k in keep:
            os.environ[k] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(1)
        finally:
            for k, v in keep.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def run(self, *args):
        return self.pool.apply(sample_fronts, args)

    def close(self):
        self.pool.terminate()
        self.pool.join()


def sampled_rate(t, nrhs, passes, budget_s, seed=0, serial=None, nthreads=1):
    """Factor and substitution time of the whole tree estimated from a
    bounded sample, level by level (each level gets an equal share of
    budget_s).  Levels with at least nthreads fronts are sampled on one core
    by `serial` (a SerialSampler) and divided by nthreads; the others run
    their fronts one after another with threaded BLAS.  Each level's factor
    time is extrapolated by its sampled flop rate and its substitution time
    (passes forward + backward sweeps of nrhs right-hand sides) by its
    sampled factor-entry rate.  Returns (t_factor, t_solve, details)."""
    rng = np.random.default_rng(seed)
    p_all, b_all, lev = t["p"], t["b"], t["level"]
    levels = sorted(set(lev.tolist()))
    per_level = budget_s / len(levels)
    t_fac = t_sol = 0.0
    sampled = 0
    parallel_levels = 0
    for L in levels:
        ids = rng.permutation(np.where(lev == L)[0])
        pf, bf = p_all[ids].astype(np.float64), b_all[ids].astype(np.float64)
        lev_flops = float(np.sum(8.0 * (pf ** 3 / 3.0 + pf * pf * bf + pf * bf * bf)))
        lev_entries = float(np.sum(pf * pf + 2 * pf * bf))
        shapes = list(zip(p_all[ids].tolist(), b_all[ids].tolist()))
        if serial is not None and nthreads > 1 and len(ids) >= nthreads:
            fl, ent, tf, ts = serial.run(shapes, nrhs, per_level, per_level * 5e9, int(seed) + L)
            div = float(nthreads)
            parallel_levels += 1
        else:
            fl, ent, tf, ts = sample_fronts(shapes, nrhs, per_level, per_level * 1e11, int(seed) + L)
            div = 1.0
        sampled += 1 if fl else 0
        t_fac += lev_flops / (fl / max(tf, 1e-9)) / div
        t_sol += passes * lev_entries / (ent / max(ts, 1e-9)) / div
    return t_fac, t_sol, {"levels": len(levels), "levels_one_front_per_core": parallel_levels}
