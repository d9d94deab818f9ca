"""Host logic of the serving loop (wtomo3d_gb300.serve) with a fake backend:
admission under the byte budget with LRU eviction, continuous batching of
requests that share a factorisation, overlap of work on different keys, and
per-request routing of results."""
import threading
import time

import numpy as np
import pytest

from wtomo3d_gb300 import serve


class FakeBackend:
    def __init__(self, factor_s=0.05, solve_s=0.02, size=lambda dims: float(np.prod(dims))):
        self.factor_s, self.solve_s, self.size = factor_s, solve_s, size
        self.lock = threading.Lock()
        self.open_handles = {}
        self.events = []          # (t0, t1, kind, key, ncols)
        self.opened = []
        self.closed = []
        self.active = 0
        self.max_active = 0

    def bytes_needed(self, key):
        return self.size(key[0])

    def _enter(self):
        with self.lock:
            self.active += 1
            self.max_active = max(self.max_active, self.active)

    def _leave(self):
        with self.lock:
            self.active -= 1

    def open(self, key):
        self._enter()
        t0 = time.perf_counter()
        time.sleep(self.factor_s)
        h = {"key": key, "busy": False}
        with self.lock:
            self.open_handles[id(h)] = h
            self.opened.append(key)
            self.events.append((t0, time.perf_counter(), "factor", key, 0))
        self._leave()
        return h

    def resident_bytes(self, h):
        return self.size(h["key"][0])

    def close(self, h):
        assert not h["busy"], "closed a handle with a batch in flight"
        with self.lock:
            del self.open_handles[id(h)]
            self.closed.append(h["key"])

    def solve(self, h, key, batch):
        assert h["key"] == key
        h["busy"] = True
        self._enter()
        t0 = time.perf_counter()
        cols = sum(r.nsrc for r in batch)
        time.sleep(self.solve_s + 1e-4 * cols)
        out = [(self.answer(key, r), np.full(r.nsrc, 1e-12)) for r in batch]
        with self.lock:
            self.events.append((t0, time.perf_counter(), "solve", key, cols))
        self._leave()
        h["busy"] = False
        return out

    @staticmethod
    def answer(key, r):
        dims, seed, freq = key
        return np.array([hash((dims, seed, freq, tuple(p))) % 1000003 for p in r.params], np.float64)


def _req(rid, t, dims, seed, freq, ns=2):
    return serve.Request(rid, t, dims, seed, freq, "plane", [(0.1 * (rid + 1), 0.2 * k) for k in range(ns)])


def test_stream_is_seeded_and_poisson():
    a = serve.make_stream(400, rate_hz=5.0, seed=3)
    b = serve.make_stream(400, rate_hz=5.0, seed=3)
    assert [(r.t_arrival, r.key, r.nsrc) for r in a] == [(r.t_arrival, r.key, r.nsrc) for r in b]
    gaps = np.diff([0.0] + [r.t_arrival for r in a])
    assert abs(gaps.mean() - 0.2) < 0.03
    assert all(1 <= r.nsrc <= 64 for r in a)
    assert {r.dims for r in a} == {(48, 48, 48), (64, 64, 64), (96, 96, 64)}
    assert {r.seed for r in a} <= set(range(8)) and {r.freq for r in a} == {0.5, 1.0, 1.5, 2.0}


def test_every_request_gets_its_own_result():
    be = FakeBackend()
    srv = serve.Server(be, budget_bytes=1e9, max_batch=64, workers=4)
    stream = serve.make_stream(60, rate_hz=400.0, seed=1, grids=((4, 4, 4), (5, 5, 5)), grid_weights=(1, 1),
                               n_models=2, freqs=(1.0, 2.0), max_src=8)
    summ = srv.run(stream, timeout_s=60)
    srv.close()
    for r in stream:
        assert r.t_done is not None and r.t_done >= r.t_arrival
        np.testing.assert_array_equal(r.result, FakeBackend.answer(r.key, r))
    assert summ["requests"] == 60 and summ["solves"] == sum(r.nsrc for r in stream)
    assert summ["p99_ms"] >= summ["p50_ms"] > 0
    assert summ["factorizations"] == len({r.key for r in stream})   # budget large: no eviction
    assert summ["evictions"] == 0
    assert not be.open_handles


def test_lru_eviction_under_budget():
    size = lambda dims: 10.0
    be = FakeBackend(factor_s=0.01, solve_s=0.005, size=size)
    srv = serve.Server(be, budget_bytes=25.0, max_batch=64, workers=2)   # two factorisations fit
    A, B, C = ((4, 4, 4), 0, 1.0), ((4, 4, 4), 1, 1.0), ((4, 4, 4), 2, 1.0)
    seq = [A, B, A, C, B, A]
    stream = [_req(i, 0.15 * i, *k) for i, k in enumerate(seq)]
    summ = srv.run(stream, timeout_s=30)
    srv.close()
    # A, B resident; A used again; C evicts B (the least recent); B evicts A; A evicts C
    assert be.opened == [A, B, C, B, A]
    assert be.closed[:3] == [B, A, C]
    assert summ["evictions"] == 3 and summ["hits"] == 1
    assert summ["peak_resident_gb"] * 1e9 <= 25.0


def test_no_admission_while_memory_is_busy():
    """A key that does not fit waits until a running batch releases its
    factorisation; the busy handle is never closed under it."""
    be = FakeBackend(factor_s=0.01, solve_s=0.2)
    srv = serve.Server(be, budget_bytes=100.0, max_batch=64, workers=4)
    A, B = ((4, 4, 4), 0, 1.0), ((4, 4, 4), 1, 1.0)
    stream = [_req(0, 0.0, *A), _req(1, 0.05, *B)]
    srv.run(stream, timeout_s=30)
    srv.close()
    t_solve_a = [e for e in be.events if e[2] == "solve" and e[3] == A][0]
    t_factor_b = [e for e in be.events if e[2] == "factor" and e[3] == B][0]
    assert t_factor_b[0] >= t_solve_a[1]


def test_continuous_batching_and_overlap():
    be = FakeBackend(factor_s=0.02, solve_s=0.15)
    srv = serve.Server(be, budget_bytes=1e6, max_batch=16, workers=4)
    A, B = ((4, 4, 4), 0, 1.0), ((5, 5, 5), 0, 1.0)
    stream = []
    for i in range(24):      # requests keep arriving while batches run
        stream.append(_req(len(stream), 0.02 * i, *A, ns=3))
        stream.append(_req(len(stream), 0.02 * i + 0.01, *B, ns=3))
    srv.run(stream, timeout_s=60)
    srv.close()
    solves = [e for e in be.events if e[2] == "solve"]
    assert max(e[4] for e in solves) > 3            # several requests in one batch
    assert all(e[4] <= 16 for e in solves)          # batch width bounded
    # batches on A and B overlapped in time
    sa = [e for e in solves if e[3] == A]
    sb = [e for e in solves if e[3] == B]
    assert any(a[0] < b[1] and b[0] < a[1] for a in sa for b in sb)
    assert len({r.batch_id for r in stream}) < len(stream)
    for r in stream:
        np.testing.assert_array_equal(r.result, FakeBackend.answer(r.key, r))


def test_request_larger_than_budget_is_an_error():
    be = FakeBackend()
    srv = serve.Server(be, budget_bytes=10.0)
    with pytest.raises(RuntimeError):
        srv.run([_req(0, 0.0, (4, 4, 4), 0, 1.0)], timeout_s=10)
    srv.close()
