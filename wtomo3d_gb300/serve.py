"""Request-serving loop over resident factorisations.

Requests (grid, model seed, frequency, 1..64 plane-wave or point sources)
arrive over time.  Factorisations stay resident on the device keyed by
(grid, model seed, frequency); a new one is admitted when the resident bytes
fit the budget, evicting the least recently used idle factorisations first.
Right-hand sides of all requests queued on the same factorisation are
solved together (continuous batching): requests that arrive while a batch
is on the GPU join the next batch of their key, and batches of different
keys, and factorisations of new keys, run at the same time on their own
handles and CUDA streams (one worker thread each; the library calls release
the interpreter lock).

The reference has no serving path: wtomo3d solves one frequency group per
MPI process in a batch run (elwave.f90:19-21,149).  Each solve here is the
same factor + FP64-refined solve as the batch path.

The scheduling logic is backend-agnostic; GpuBackend drives
libwtomo3d_gpu.so, and tests drive the same Server with a fake backend.
"""
import threading
import time
from collections import OrderedDict, deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    t_arrival: float                 # seconds after the start of the stream
    dims: tuple                      # (nx, ny, nz)
    seed: int                        # model seed (pool index)
    freq: float                      # Hz
    kind: str                        # "plane" or "point"
    params: list                     # plane: [(ain, baz)], point: [(x, y, z, comp)]
    # filled by the server
    t_start: float = None            # first batch containing it started
    t_done: float = None
    relres: np.ndarray = None
    result: object = None            # solution columns (n x nsrc) when kept
    batch_id: int = None

    @property
    def nsrc(self):
        return len(self.params)

    @property
    def key(self):
        return (tuple(self.dims), int(self.seed), float(self.freq))


@dataclass
class Entry:
    key: tuple
    bytes: float
    state: str = "factoring"         # "factoring" | "ready"
    busy: bool = False
    last_used: float = 0.0
    handle: object = None
    pending: deque = field(default_factory=deque)


def make_stream(n_requests, rate_hz, seed, grids=((48, 48, 48), (64, 64, 64), (96, 96, 64)),
                grid_weights=(0.5, 0.35, 0.15), freqs=(0.5, 1.0, 1.5, 2.0), n_models=8, max_src=64,
                plane_frac=0.75):
    """Seeded Poisson request stream: exponential inter-arrival times at mean
    rate `rate_hz`; grid, model seed (pool of n_models), frequency, source
    count (1..max_src) and source type drawn per request."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    gw = np.asarray(grid_weights, np.float64)
    gw = gw / gw.sum()
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate_hz)
        dims = tuple(grids[rng.choice(len(grids), p=gw)])
        ns = int(rng.integers(1, max_src + 1))
        if rng.random() < plane_frac:
            params = [(float(np.radians(rng.uniform(0.0, 30.0))), float(np.radians(rng.uniform(0.0, 360.0))))
                      for _ in range(ns)]
            kind = "plane"
        else:
            params = [(float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.3, 0.7)), float(rng.uniform(0.2, 0.6)),
                       int(rng.integers(0, 3))) for _ in range(ns)]
            kind = "point"
        out.append(Request(i, t, dims, int(rng.integers(0, n_models)), float(rng.choice(freqs)), kind, params))
    return out


class Server:
    """Continuous-batching scheduler over a factorisation cache."""

    def __init__(self, backend, budget_bytes=120e9, max_batch=64, workers=4):
        self.backend = backend
        self.budget = float(budget_bytes)
        self.max_batch = int(max_batch)
        self.pool = ThreadPoolExecutor(max_workers=workers)
        self.cv = threading.Condition()
        self.entries = OrderedDict()          # key -> Entry
        self.used = 0.0                       # resident bytes admitted
        self.waiting = deque()                # keys with requests but no entry, in arrival order
        self.unadmitted = {}                  # key -> deque of requests waiting for admission
        self.errors = []
        self.log = {"factorizations": 0, "evictions": 0, "batches": 0, "hits": 0, "misses": 0,
                    "peak_resident_bytes": 0.0, "max_concurrent_jobs": 0}
        self._jobs = 0
        self._t0 = None
        self._batch_seq = 0

    # -- time --------------------------------------------------------------
    def now(self):
        return time.perf_counter() - self._t0

    # -- scheduling (called with self.cv held) ------------------------------
    def _admit(self, key):
        need = self.backend.bytes_needed(key)
        if need > self.budget:
            raise RuntimeError("a factorisation of %s needs %.1f GB, over the budget" % (key, need / 1e9))
        # idle factorisations, least recently used first
        idle = sorted((e for e in self.entries.values() if e.state == "ready" and not e.busy and not e.pending),
                      key=lambda e: e.last_used)
        free, victims = self.budget - self.used, []
        while free < need and idle:
            victims.append(idle.pop(0))
            free += victims[-1].bytes
        if free < need:
            return False                      # wait for running work to finish
        # the device must also hold the transient memory of the new
        # factorisation (workspace, Krylov bases) next to everything resident
        can_open = getattr(self.backend, "can_open", None)
        if can_open is not None:
            freeing = sum(v.bytes for v in victims)
            while not can_open(key, freeing) and idle:
                victims.append(idle.pop(0))
                freeing += victims[-1].bytes
            if not can_open(key, freeing) and self._jobs > 0:
                return False
        for v in victims:
            del self.entries[v.key]
            self.used -= v.bytes
            self.log["evictions"] += 1
        e = Entry(key=key, bytes=need)
        self.entries[key] = e
        self.used += need
        self.log["peak_resident_bytes"] = max(self.log["peak_resident_bytes"], self.used)
        e.pending.extend(self.unadmitted.pop(key))
        self.log["factorizations"] += 1
        self._submit(self._factor_job, e, victims)
        return True

    def _schedule(self):
        # admissions in arrival order; a key that does not fit blocks the
        # ones behind it (no starvation of large grids)
        while self.waiting:
            if not self._admit(self.waiting[0]):
                break
            self.waiting.popleft()
        for e in list(self.entries.values()):
            if e.state == "ready" and not e.busy and e.pending:
                batch, cols = [], 0
                while e.pending and (not batch or cols + e.pending[0].nsrc <= self.max_batch):
                    r = e.pending.popleft()
                    batch.append(r)
                    cols += r.nsrc
                e.busy = True
                self._batch_seq += 1
                t = self.now()
                for r in batch:
                    r.t_start = t
                    r.batch_id = self._batch_seq
                self.log["batches"] += 1
                self._submit(self._solve_job, e, batch)

    def _submit(self, fn, *args):
        self._jobs += 1
        self.log["max_concurrent_jobs"] = max(self.log["max_concurrent_jobs"], self._jobs)
        self.pool.submit(self._run_job, fn, *args)

    def _run_job(self, fn, *args):
        try:
            fn(*args)
        except Exception as exc:   # surfaced by run()
            with self.cv:
                self.errors.append(exc)
        finally:
            with self.cv:
                self._jobs -= 1
                self._schedule()
                self.cv.notify_all()

    # -- jobs (worker threads) ---------------------------------------------
    def _factor_job(self, e, victims):
        # the evicted handles free their device memory before the new one allocates
        for v in victims:
            self.backend.close(v.handle)
            v.handle = None
        for attempt in range(6):
            try:
                h = self.backend.open(e.key)
                break
            except Exception as exc:
                is_oom = getattr(self.backend, "is_oom", lambda x: False)
                if attempt == 5 or not is_oom(exc):
                    raise
                # out of device memory: release every idle factorisation, then
                # wait for running work before retrying
                with self.cv:
                    idle = [x for x in self.entries.values()
                            if x is not e and x.state == "ready" and not x.busy and not x.pending]
                    for x in idle:
                        del self.entries[x.key]
                        self.used -= x.bytes
                        self.log["evictions"] += 1
                for x in idle:
                    self.backend.close(x.handle)
                    x.handle = None
                with self.cv:
                    if not idle:
                        self.cv.wait(timeout=1.0)
        with self.cv:
            e.handle = h
            actual = self.backend.resident_bytes(h)
            self.used += actual - e.bytes
            e.bytes = actual
            self.log["peak_resident_bytes"] = max(self.log["peak_resident_bytes"], self.used)
            e.state = "ready"
            e.last_used = self.now()

    def _solve_job(self, e, batch):
        results = self.backend.solve(e.handle, e.key, batch)
        with self.cv:
            t = self.now()
            for r, (x, rr) in zip(batch, results):
                r.result, r.relres, r.t_done = x, rr, t
            e.busy = False
            e.last_used = t

    # -- driver --------------------------------------------------------------
    def submit(self, r):
        with self.cv:
            e = self.entries.get(r.key)
            if e is not None:
                self.log["hits"] += 1
                e.pending.append(r)
            else:
                self.log["misses"] += 1
                if r.key not in self.unadmitted:
                    self.unadmitted[r.key] = deque()
                    self.waiting.append(r.key)
                self.unadmitted[r.key].append(r)
            self._schedule()

    def run(self, stream, timeout_s=None):
        """Feeds the requests at their arrival times (real time) and returns
        when all are done.  Returns the summary of the run."""
        self._t0 = time.perf_counter()
        pending = sorted(stream, key=lambda r: r.t_arrival)
        i = 0
        with self.cv:
            while True:
                if self.errors:
                    raise self.errors[0]
                t = self.now()
                while i < len(pending) and pending[i].t_arrival <= t:
                    self.cv.release()
                    try:
                        self.submit(pending[i])
                    finally:
                        self.cv.acquire()
                    i += 1
                if i == len(pending) and all(r.t_done is not None for r in pending):
                    break
                if timeout_s is not None and t > timeout_s:
                    raise TimeoutError("serving run exceeded %.0f s" % timeout_s)
                wait = pending[i].t_arrival - t if i < len(pending) else 0.5
                self.cv.wait(timeout=max(1e-4, min(wait, 0.5)))
        return self.summary(pending)

    def close(self):
        with self.cv:
            entries = list(self.entries.values())
            self.entries.clear()
            self.used = 0.0
        self.pool.shutdown(wait=True)
        for e in entries:
            if e.handle is not None:
                self.backend.close(e.handle)

    def summary(self, reqs):
        lat = np.array([(r.t_done - r.t_arrival) * 1e3 for r in reqs])
        t_end = max(r.t_done for r in reqs)
        nsolves = sum(r.nsrc for r in reqs)
        worst = max(float(np.max(r.relres)) for r in reqs if r.relres is not None)
        d = {"requests": len(reqs), "solves": nsolves, "wall_s": t_end,
             "solves_per_s": nsolves / t_end, "p50_ms": float(np.percentile(lat, 50)),
             "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
             "max_relres": worst, "budget_gb": self.budget / 1e9}
        d.update({k: (v / 1e9 if k.endswith("bytes") else v) for k, v in self.log.items()})
        d["peak_resident_gb"] = d.pop("peak_resident_bytes")
        return d


class GpuBackend:
    """Factorisations and batched solves on libwtomo3d_gpu.so.

    Models: layered-plus-random (four flat layers, 5% Gaussian-correlated
    perturbation of 200 m correlation length, Gardner density) with the
    request's seed; plane waves against the unperturbed layered background.
    Point sources sit at the fractional position (x, y, z) of the grid, unit
    force on component comp.  Solutions (scattered field for plane waves)
    are FP64-refined to `tol`."""

    def __init__(self, dx=20.0, pml_nodes=10, tol=1e-8, maxit=20, keep_results=False, precision=None, max_batch=64,
                 workspaces_per_grid=1):
        import wtomo3d_gb300 as wt
        self.wt = wt
        # factorisations of one grid run concurrently up to this many at once
        # (each concurrent one holds its own level update buffers)
        self.workspaces = int(workspaces_per_grid)
        wt._check(wt.lib().wt3d_set_workspaces_per_grid(self.workspaces))
        self.dx, self.pml_nodes, self.tol, self.maxit = dx, pml_nodes, tol, maxit
        self.keep = keep_results
        self.max_batch = max_batch
        self.precision = wt.PREC_MIXED if precision is None else precision
        self._models = {}
        self._open = {}
        self._lock = threading.Lock()

    def grid(self, dims):
        nx, ny, nz = dims
        return self.wt.Grid(nx, ny, nz, self.dx, pmld=self.pml_nodes * self.dx, fst=1, usemin=1)

    def model(self, dims, seed):
        from wtomo3d_gb300 import model
        with self._lock:
            k = (tuple(dims), seed)
            if k not in self._models:
                nx, ny, nz = dims
                self._models[k] = (model.layered_random(nx, ny, nz, self.dx, seed=seed),
                                   model.layered(nx, ny, nz), self.wt.Layered1D(*model.layered1d(nz, self.dx)))
            return self._models[k]

    def bytes_needed(self, key):
        g = self.grid(key[0])
        r, extra, _ = self.wt.solver_bytes(g, self.precision)
        return r + extra + 2.0 * g.n * self.max_batch * 16      # + the batch buffers

    def can_open(self, key, freeing):
        """Free device memory (plus what the evictions release) covers the new
        handle, a factorisation workspace of its grid unless every workspace
        the grid may have is held already, the Krylov bases of a slow solve and
        a margin."""
        g = self.grid(key[0])
        _, _, ws = self.wt.solver_bytes(g, self.precision)
        with self._lock:
            shared = self._open.get(tuple(key[0]), 0) >= self.workspaces
        transient = (0.0 if shared else 1.25 * ws) + 17.0 * g.n * 32 * 16 + 4e9
        free, _ = self.wt.mem_info()
        return free + freeing >= self.bytes_needed(key) + transient

    def open(self, key):
        dims, seed, freq = key
        mdl, bg, _ = self.model(dims, seed)
        s = self.wt.Solver(self.grid(dims), self.precision)
        try:
            s.set_model(*mdl)
            s.set_background(*bg)
            s.factor(2 * np.pi * freq)
            s.batch_buffers(self.max_batch)
        except Exception:
            s.close()
            raise
        with self._lock:
            self._open[tuple(dims)] = self._open.get(tuple(dims), 0) + 1
        return s

    def is_oom(self, exc):
        return getattr(exc, "code", None) == self.wt.WT3D_ERR_NOMEM

    def resident_bytes(self, s):
        st = s.stats()
        return float(st["device_bytes"])

    def close(self, s):
        dims = (s.grid.nx, s.grid.ny, s.grid.nz)
        s.close()
        with self._lock:
            self._open[dims] = self._open.get(dims, 1) - 1

    def solve(self, s, key, batch):
        from wtomo3d_gb300 import model
        dims, seed, freq = key
        nx, ny, nz = dims
        _, _, lay = self.model(dims, seed)
        n = s.grid.n
        cols = sum(r.nsrc for r in batch)
        dF, dX = s.batch_buffers(cols)
        col_bytes = n * 16
        c0 = 0
        for r in batch:
            if r.kind == "plane":
                s.rhs_planewave(lay, np.array([p[0] for p in r.params]), np.array([p[1] for p in r.params]),
                                d_F=dF + c0 * col_bytes)
            else:
                B = np.asfortranarray(np.stack(
                    [model.point_force(nx, ny, nz, self.dx, x * (nx - 1) * self.dx, y * (ny - 1) * self.dx,
                                       z * (nz - 1) * self.dx, comp=c) for (x, y, z, c) in r.params], axis=1))
                s.memcpy(dF + c0 * col_bytes, B.ctypes.data, B.nbytes)
            c0 += r.nsrc
        relres = s.solve_device(dF, dX, cols, tol=self.tol, maxit=self.maxit, allow_noconv=True)
        out, c0 = [], 0
        for r in batch:
            x = None
            if self.keep:
                x = np.empty((n, r.nsrc), np.complex128, order="F")
                s.memcpy(x.ctypes.data, dX + c0 * col_bytes, x.nbytes)
            out.append((x, relres[c0:c0 + r.nsrc].copy()))
            c0 += r.nsrc
        return out
