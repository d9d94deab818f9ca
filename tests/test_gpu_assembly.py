"""GPU parity of the pattern and the assembly against the CPU oracle.

Pattern: bit-exact.  Values: complex128, |a_gpu - a_oracle| <= 1e-12 max|a|
and per entry <= 1e-12 relative for every entry above 1e-9 max|a|."""
import numpy as np
import pytest
import scipy.sparse as sp

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

pytestmark = pytest.mark.gpu

TOL = 1e-12


def check_values(a_gpu, a_ref, irptr=None):
    """Normwise: max |a_gpu - a_ref| <= TOL max |a_ref|; per row: every entry
    within TOL of the largest entry of its row (entries that are small because
    of cancellation are judged against their row, not themselves)."""
    scale = np.abs(a_ref).max()
    err = np.abs(a_gpu - a_ref)
    assert err.max() <= TOL * scale, err.max() / scale
    if irptr is not None:
        rows = np.repeat(np.arange(len(irptr) - 1), np.diff(irptr))
        rowmax = np.zeros(len(irptr) - 1)
        np.maximum.at(rowmax, rows, np.abs(a_ref))
        rel = err / rowmax[rows]
        assert rel.max() <= TOL, rel.max()


@pytest.mark.parametrize("dims", [(2, 2, 2), (3, 4, 5), (7, 6, 9), (17, 11, 13)])
def test_pattern_bit_exact(oracle, dims):
    ir, jc = oracle.pattern(*dims)
    ir1, jc1 = wt.pattern(*dims, base=1)
    np.testing.assert_array_equal(ir1, ir)
    np.testing.assert_array_equal(jc1, jc)
    ir0, jc0 = wt.pattern(*dims, base=0)
    np.testing.assert_array_equal(ir0, ir - 1)
    np.testing.assert_array_equal(jc0, jc - 1)


CASES = [
    # (dims, dx, pml nodes, fst, usemin, f, tau, model)
    ((12, 11, 13), 25.0, 3, 0, 1, 1.0, None, "homog"),          # all-PML, Dirichlet top (config 1 style)
    ((12, 13, 11), 20.0, 3, 1, 1, 1.5, None, "layered"),        # free surface, Min cells
    ((11, 12, 10), 20.0, 3, 1, 0, 2.0, None, "layered"),        # traction-free top rows
    ((10, 10, 12), 20.0, 2, 1, 1, 0.5, 3.0, "layered"),         # anti-alias complex omega
    ((9, 10, 5), 20.0, 3, 1, 1, 1.0, None, "layered"),          # nz <= 2 ipml edge case
    ((6, 5, 7), 20.0, 1, 0, 1, 1.0, None, "homog"),             # one-node PML
]


@pytest.mark.parametrize("case", CASES)
def test_assembly_parity(oracle, case):
    dims, dx, pn, fst, usemin, f, tau, mdl = case
    g = Grid(*dims, dx, pmld=pn * dx, fst=fst, usemin=usemin)
    if mdl == "homog":
        vp, vs, rho = model.homogeneous(*dims)
    else:
        vp, vs, rho = model.layered_random(*dims, dx, seed=7)
    om = 2 * np.pi * f + (1j / tau if tau else 0)
    ir, jc = oracle.pattern(*dims)
    a_ref, ierr = oracle.assemble(g, vp, vs, rho, om, ir)
    assert ierr == 0
    a = wt.assemble(g, vp, vs, rho, om)
    check_values(a, a_ref, ir)


def test_assembly_config1_40cubed(oracle):
    """Config 1: 40^3, h = 25 m, homogeneous, 10-node PML on all faces, 1 Hz."""
    g = Grid(40, 40, 40, 25.0, pmld=10 * 25.0, fst=0)
    vp, vs, rho = model.homogeneous(40, 40, 40)
    ir, jc = oracle.pattern(40, 40, 40)
    a_ref, ierr = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir)
    assert ierr == 0
    a = wt.assemble(g, vp, vs, rho, 2 * np.pi * 1.0)
    check_values(a, a_ref, ir)


def test_assembly_golden(oracle):
    import make_golden
    for name in make_golden.CASES:
        g, vp, vs, rho, om, z = make_golden.load_case(name)
        check_values(wt.assemble(g, vp, vs, rho, om), z["a"], z["irptr"])


def test_attenuation_and_complex_frequency_match_oracle(oracle):
    """Q dispersion (dispersion.f:78-114) fused into the device Lame step, and
    the anti-alias complex frequency 2 pi f + i/tau (elwave.f90:164), against
    the oracle's restatement; a dispersed operator factors and solves."""
    g = Grid(14, 13, 12, 25.0, pmld=75.0, fst=1)
    vp, vs, rho = model.layered_random(14, 13, 12, 25.0, seed=5, corr_len=75.0)
    rng = np.random.default_rng(8)
    qp = rng.uniform(0.005, 0.03, vp.shape).astype(np.float32)
    qs = rng.uniform(0.01, 0.05, vp.shape).astype(np.float32)
    ir, jc = oracle.pattern(14, 13, 12)
    with wt.Solver(g) as s:
        s.set_model(vp, vs, rho)
        s.set_attenuation(qp, qs, freqbase=20.0)
        for om in (2 * np.pi * 1.5, 2 * np.pi * 4.0 + 1j / 2.0):
            s.factor(om)
            ref, ierr = oracle.assemble_q(g, vp, vs, rho, qp, qs, 20.0, om, ir)
            assert ierr == 0
            n = g.n
            # the device operator against the oracle's on random probe vectors
            P = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
            A = sp.csr_matrix((ref, jc - 1, ir - 1), shape=(n, n))
            Y = s.apply(P)
            assert np.abs(Y - A @ P).max() <= 1e-12 * (abs(A) @ abs(P)).max()
            b = model.point_force(14, 13, 12, 25.0, 150.0, 150.0, 150.0)
            x = s.solve(b, tol=1e-10, maxit=30)
            assert np.linalg.norm(A @ x - b) <= 1e-9 * np.linalg.norm(b)
        s.set_attenuation(None, None)
