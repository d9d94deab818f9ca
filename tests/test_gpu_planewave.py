"""GPU plane-wave sources: the incident field u0 and the scattered-field source
f = (A_bg - A) u0 against the oracle (Haskell response, expansion and two
complex128 operators assembled on the CPU); f = 0 when the model equals the
background; u0 nearly satisfies the background operator away from the PML;
and the scattered-field solve reaches its residual."""
import numpy as np
import pytest
import scipy.sparse as sp

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

pytestmark = pytest.mark.gpu


def oracle_A(oracle, g, vp, vs, rho, om):
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a, ierr = oracle.assemble(g, vp, vs, rho, om, ir)
    assert ierr == 0
    return sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))


@pytest.fixture(scope="module")
def case():
    g = Grid(16, 14, 20, 20.0, pmld=3 * 20.0, fst=1)
    vp0, vs0, rho0 = model.layered(g.nx, g.ny, g.nz)
    vp, vs, rho = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=3)
    lay = model.layered1d(g.nz, g.dx)
    return g, (vp0, vs0, rho0), (vp, vs, rho), lay


def test_planewave_rhs_matches_oracle(oracle, case):
    g, bg, mdl, lay = case
    om = 2 * np.pi * 1.5
    ain = np.radians([5.0, 18.0, 29.0])
    baz = np.radians([0.0, 130.0, 275.0])
    sw = np.array([0, 0, 1])
    with wt.Solver(g) as s:
        s.set_model(*mdl)
        s.set_background(*bg)
        s.factor(om)
        F, U0 = s.rhs_planewave(wt.Layered1D(*lay), ain, baz, sw)
    A = oracle_A(oracle, g, *mdl, om)
    Abg = oracle_A(oracle, g, *bg, om)
    for j in range(3):
        u0 = oracle.planewave(g, lay, om, ain[j], baz[j], bool(sw[j]))
        assert np.abs(U0[:, j] - u0).max() <= 1e-12 * np.abs(u0).max()
        f = (Abg - A) @ u0
        assert np.abs(F[:, j] - f).max() <= 1e-11 * np.abs(f).max()


def test_homogeneous_background_gives_no_source(case):
    """hetfldsrc.f90:1010-1016: model == background => (A_bg - A) u0 = 0."""
    g, bg, mdl, lay = case
    with wt.Solver(g) as s:
        s.set_model(*bg)
        s.set_background(*bg)
        s.factor(2 * np.pi)
        F, U0 = s.rhs_planewave(wt.Layered1D(*lay), np.radians([20.0]), np.radians([45.0]))
    assert np.abs(F).max() == 0.0
    assert np.abs(U0).max() > 0.1


def test_incident_field_solves_background_interior(oracle):
    """In a homogeneous background the discrete plane P wave (x-z plane) nearly
    satisfies the interior rows of A_bg (O((kh)^2) residual)."""
    g = Grid(20, 8, 24, 20.0, pmld=2 * 20.0, fst=1)
    lay = (np.array([3000.0, 3000.0]), np.array([1732.0, 1732.0]), np.array([2400.0, 2400.0]),
           np.array([0.0, 100.0]))
    vp, vs, rho = model.homogeneous(g.nx, g.ny, g.nz, 3000.0, 1732.0, 2400.0)
    om = 2 * np.pi * 2.0
    A = oracle_A(oracle, g, vp, vs, rho, om)
    u0 = oracle.planewave(g, lay, om, np.radians(25.0), 0.0)
    r = A @ u0
    node = lambda iz, ix, iy: iz + g.nz * (ix + g.nx * iy)
    # interior nodes away from the PML and the free surface
    rows = [3 * node(iz, ix, 4) + c for iz in range(8, 16) for ix in range(6, 14) for c in (0, 2)]
    rel = np.abs(r[rows]).max() / (om * om * 2400.0 * np.abs(u0).max())
    assert rel < 2e-3, rel


def test_scattered_field_solve(case):
    g, bg, mdl, lay = case
    om = 2 * np.pi * 1.0
    with wt.Solver(g) as s:
        s.set_model(*mdl)
        s.set_background(*bg)
        s.factor(om)
        F, _ = s.rhs_planewave(wt.Layered1D(*lay), np.radians([10.0, 25.0]), np.radians([30.0, 200.0]))
        X = s.solve(F, tol=1e-10)
        assert s.last_relres.max() <= 1e-10
        Y = s.apply(X)
    assert np.abs(Y - F).max() <= 1e-9 * np.abs(F).max()
