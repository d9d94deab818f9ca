"""CPU checks of the FP64 oracle gradient: central differences of the
waveform misfit with complex128 SuperLU solves on small grids, for point
forces and for plane waves (total-field formulation)."""
import numpy as np
import pytest

import grad_cpu
from wtomo3d_gb300 import Grid, model


def _setup(g, seed, nsrc=2):
    vp, vs, rho = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=seed, std=0.05, corr_len=3 * g.dx)
    rng = np.random.default_rng(seed)
    n = 3 * g.nx * g.ny * g.nz
    B = np.zeros((n, nsrc), np.complex128)
    for j in range(nsrc):
        b = model.point_force(g.nx, g.ny, g.nz, g.dx, (g.nx // 2 + j) * g.dx, (g.ny // 2) * g.dx,
                              (g.nz // 2 + j % 2) * g.dx, comp=j % 3)
        B[:, j] = b
    iy, ix = np.meshgrid(np.arange(2, g.ny - 2, 2), np.arange(2, g.nx - 2, 2), indexing="ij")
    depth = 0 if g.fst else 1          # the top row is Dirichlet without a free surface
    rec = (depth + g.nz * ix + g.nz * g.nx * iy).reshape(-1)
    true = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=seed + 100, std=0.03, corr_len=3 * g.dx)
    true = tuple(np.asarray(t, np.float32) * np.asarray(m, np.float32) / np.asarray(m0, np.float32)
                 for t, m, m0 in zip(true, (vp, vs, rho), model.layered(g.nx, g.ny, g.nz)))
    return (vp, vs, rho), true, B, rec, rng


def _fd(oracle, g, mdl, omega, B, rec, dobs, cell, which, h=2e-3):
    """Central difference of the misfit, Richardson-extrapolated from steps
    h and h/2 (truncation O(h^4)); steps are the float32-representable ones."""
    d1 = _fd1(oracle, g, mdl, omega, B, rec, dobs, cell, which, h)
    d2 = _fd1(oracle, g, mdl, omega, B, rec, dobs, cell, which, h / 2)
    return (4 * d2 - d1) / 3


def _fd1(oracle, g, mdl, omega, B, rec, dobs, cell, which, h, U0fn=None):
    vals = []
    for sgn in (1, -1):
        m = [np.array(x, np.float32, copy=True) for x in mdl]
        m[which][cell] = np.float32(m[which][cell] * (1 + sgn * h))
        vals.append((m[which][cell], m))
    (vpl, mp), (vmi, mm) = vals
    chis = []
    for m in (mp, mm):
        A = grad_cpu.operator(oracle, g, m, omega)
        if U0fn is None:
            U, _ = grad_cpu.forward(A, B)
        else:
            U, _ = grad_cpu.forward(A, U0fn(m, A), None)
        chis.append(grad_cpu.misfit(U, rec, dobs))
    return (chis[0] - chis[1]) / (float(vpl) - float(vmi))


@pytest.mark.parametrize("fst,usemin", [(1, 1), (0, 1), (1, 0)])
def test_oracle_gradient_matches_misfit_fd(oracle, fst, usemin):
    g = Grid(9, 8, 7, 25.0, pmld=50.0, fst=fst, usemin=usemin)
    omega = 2 * np.pi * 6.0
    mdl, true, B, rec, rng = _setup(g, seed=5)
    Ut, _ = grad_cpu.forward(grad_cpu.operator(oracle, g, true, omega), B)
    dobs = grad_cpu.receivers_pred(Ut, rec)
    chi, grad, U, Lam = grad_cpu.misfit_gradient(oracle, g, mdl, omega, B, rec, dobs)
    assert chi > 0
    gmax = [np.abs(x).max() for x in grad]
    cells = [(int(rng.integers(0, g.nz - 1)), int(rng.integers(1, g.nx - 1)), int(rng.integers(1, g.ny - 1)))
             for _ in range(4)]
    cells.append((0, 2, 3))          # top row (free surface or Dirichlet)
    cells.append((1, 1, 1))          # next to the outer faces
    for cell in cells:
        for which in range(3):
            fd = _fd(oracle, g, mdl, omega, B, rec, dobs, cell, which)
            an = grad[which][cell]
            assert abs(fd - an) <= 1e-5 * abs(an) + 1e-6 * gmax[which], (cell, which, fd, an)


def test_oracle_gradient_planewave_total_field(oracle):
    """Plane-wave sources: A u = A_bg u0 for the total field, so the
    gradient uses the total field while the misfit FD re-solves the
    scattered-field system at each perturbed model."""
    g = Grid(9, 8, 8, 25.0, pmld=50.0, fst=1, usemin=1)
    omega = 2 * np.pi * 4.0
    mdl, true, _, rec, rng = _setup(g, seed=8)
    bg = model.layered(g.nx, g.ny, g.nz)
    l1d = model.layered1d(g.nz, g.dx)
    u0 = np.stack([oracle.planewave(g, l1d, omega, a, b) for a, b in ((0.2, 0.7), (0.4, 2.5))], axis=1)
    A_bg = grad_cpu.operator(oracle, g, bg, omega)

    def rhs(m, A):
        return (A_bg - A) @ u0

    A_true = grad_cpu.operator(oracle, g, true, omega)
    Ut, _ = grad_cpu.forward(A_true, rhs(true, A_true), u0)
    dobs = grad_cpu.receivers_pred(Ut, rec)
    A = grad_cpu.operator(oracle, g, mdl, omega)
    chi, grad, U, Lam = grad_cpu.misfit_gradient(oracle, g, mdl, omega, rhs(mdl, A), rec, dobs, U0=u0)
    gmax = [np.abs(x).max() for x in grad]
    for cell in [(2, 4, 4), (0, 3, 5), (5, 2, 6)]:
        for which in range(3):
            fds = []
            for h in (2e-3, 1e-3):
                vals = []
                for sgn in (1, -1):
                    m = [np.array(x, np.float32, copy=True) for x in mdl]
                    m[which][cell] = np.float32(m[which][cell] * (1 + sgn * h))
                    Am = grad_cpu.operator(oracle, g, m, omega)
                    Um, _ = grad_cpu.forward(Am, rhs(m, Am), u0)
                    vals.append((float(m[which][cell]), grad_cpu.misfit(Um, rec, dobs)))
                fds.append((vals[0][1] - vals[1][1]) / (vals[0][0] - vals[1][0]))
            fd = (4 * fds[1] - fds[0]) / 3
            an = grad[which][cell]
            assert abs(fd - an) <= 1e-5 * abs(an) + 1e-6 * gmax[which], (cell, which, fd, an)
