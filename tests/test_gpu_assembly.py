"""GPU parity of the pattern and the assembly against the CPU oracle.

Pattern: bit-exact.  Values: complex128, |a_gpu - a_oracle| <= 1e-12 max|a|
and per entry <= 1e-12 relative for every entry above 1e-9 max|a|."""
import numpy as np
import pytest

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
