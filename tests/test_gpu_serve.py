"""Serving loop on the GPU: a seeded Poisson stream over two grids, three
model seeds and two frequencies, with a budget that forces evictions.  Every
request's solution must match the same request solved alone on a fresh
handle: both are FP64-refined to relative residual 1e-10, and they must agree
to 1e-7 relative (max-norm) -- the batch a request lands in changes only the
number of refinement steps its columns get."""
import copy

import numpy as np
import pytest

from wtomo3d_gb300 import serve

pytestmark = pytest.mark.gpu
pytest.importorskip("torch")


def test_serving_same_alone_and_in_the_mix():
    grids = ((20, 20, 16), (24, 22, 18))
    # two factorisation workspaces per grid: factorisations of one grid overlap
    be = serve.GpuBackend(dx=20.0, pml_nodes=4, tol=1e-10, maxit=30, keep_results=True, workspaces_per_grid=2)
    sizes = [be.bytes_needed((g, 0, 1.0)) for g in grids]
    budget = sizes[0] + sizes[1] + 0.5 * sizes[0]            # two or three resident at most
    stream = serve.make_stream(18, rate_hz=40.0, seed=5, grids=grids, grid_weights=(1, 1), n_models=3,
                               freqs=(1.0, 2.0), max_src=6, plane_frac=0.6)
    srv = serve.Server(be, budget_bytes=budget, max_batch=16, workers=4)
    summ = srv.run(stream, timeout_s=900)
    srv.close()
    assert summ["evictions"] > 0
    assert summ["peak_resident_gb"] * 1e9 <= budget
    assert summ["max_relres"] <= 1e-10
    assert summ["batches"] < summ["requests"]                 # some requests shared a batch
    alone = serve.GpuBackend(dx=20.0, pml_nodes=4, tol=1e-10, maxit=30, keep_results=True, workspaces_per_grid=1)
    worst = 0.0
    for key in {r.key for r in stream}:
        h = alone.open(key)
        for r in [q for q in stream if q.key == key]:
            (x, rr), = alone.solve(h, key, [copy.copy(r)])
            assert np.all(rr <= 1e-10)
            d = np.abs(r.result - x).max() / np.abs(x).max()
            worst = max(worst, d)
            assert d <= 1e-7, (r.rid, d)
        alone.close(h)
    print("serving: %s; worst alone-vs-mix difference %.2e" % (summ, worst))
