"""The CPU baseline's multifrontal (oracle/cpu_multifrontal.py): its own
nested-dissection tree is the product's host analysis, front for front, and
its FP64 factor and solve agree with SuperLU."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import cpu_multifrontal as cmf
from test_symbolic import export
from wtomo3d_gb300 import Grid, model


@pytest.mark.parametrize("dims,leaf", [((6, 5, 7), 8), ((9, 9, 6), 27), ((40, 40, 40), 64), ((24, 20, 16), 64)])
def test_tree_equals_product_analysis(dims, leaf):
    t = cmf.nd_tree(*dims, leaf=leaf)
    e = export(*dims, leaf)
    for k in ("p", "b", "first", "parent", "level"):
        np.testing.assert_array_equal(t[k], e[k], err_msg=k)
    np.testing.assert_array_equal(t["perm"], e["perm"])
    np.testing.assert_array_equal(t["border"], e["border"])
    np.testing.assert_allclose(t["flops"], e["flops"], rtol=1e-12)


def test_factor_solve_matches_superlu(oracle):
    nx, ny, nz = 8, 7, 9
    g = Grid(nx, ny, nz, 20.0, pmld=2 * 20.0, fst=1)
    vp, vs, rho = model.layered_random(nx, ny, nz, g.dx, seed=5)
    ir, jc = oracle.pattern(nx, ny, nz)
    a, _ = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir)
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    rng = np.random.default_rng(0)
    B = rng.standard_normal((g.n, 3)) + 1j * rng.standard_normal((g.n, 3))
    t = cmf.nd_tree(nx, ny, nz, leaf=27)
    X, tf, ts = cmf.timed_full(A, t, B)
    Xr = spla.splu(A.tocsc()).solve(B)
    assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-9
    assert tf > 0 and ts > 0
