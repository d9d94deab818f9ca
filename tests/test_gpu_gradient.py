"""GPU adjoint-state gradient: the per-node contraction against the FP64
oracle gradient (central differences of the oracle's node blocks), the full
misfit/gradient pipeline against the FP64 CPU pipeline (oracle assembly +
SuperLU + oracle contraction), and central finite differences of the misfit
at 20 seeded cells on the 64x64x48 workload."""
import numpy as np
import pytest

import grad_cpu
import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    """(n, m) host complex array -> device buffer holding it column-major."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, np.complex128).T)).to("cuda")


@pytest.mark.parametrize("fst,usemin", [(1, 1), (0, 1), (1, 0)])
def test_contraction_matches_oracle(oracle, fst, usemin):
    g = Grid(12, 11, 10, 25.0, pmld=75.0, fst=fst, usemin=usemin)
    mdl = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=4, corr_len=75.0)
    omega = 2 * np.pi * 3.0
    rng = np.random.default_rng(11)
    U = rng.standard_normal((g.n, 3)) + 1j * rng.standard_normal((g.n, 3))
    Lam = rng.standard_normal((g.n, 3)) + 1j * rng.standard_normal((g.n, 3))
    ref = oracle.gradient(g, *mdl, omega, U, Lam)
    with wt.Solver(g) as s:
        s.set_model(*mdl)
        s.factor(omega)
        dU, dL = _dev(U), _dev(Lam)
        got = s.gradient_contract(dU.data_ptr(), dL.data_ptr(), 3)
        del dU, dL
    for k in range(3):
        scale = np.abs(ref[k]).max()
        assert scale > 0
        err = np.abs(got[k] - ref[k])
        assert err.max() <= 1e-8 * scale, (k, err.max() / scale)


def test_misfit_gradient_matches_cpu_pipeline(oracle):
    g = Grid(16, 15, 14, 25.0, pmld=100.0, fst=1, usemin=1)
    omega = 2 * np.pi * 2.0
    mdl = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=2, corr_len=100.0)
    bg = model.layered(g.nx, g.ny, g.nz)
    true = model.perturbed(mdl[0], mdl[1], g.dx, seed=9, std=0.03, corr_len=100.0)
    lay = model.layered1d(g.nz, g.dx)
    ain = np.radians([4.0, 17.0, 26.0, 11.0])
    baz = np.radians([10.0, 100.0, 220.0, 300.0])
    rec = model.surface_receivers(g.nx, g.ny, g.nz, g.pml()[2], 4, 3)
    u0 = np.stack([oracle.planewave(g, lay, omega, a, b) for a, b in zip(ain, baz)], axis=1)
    A_bg = grad_cpu.operator(oracle, g, bg, omega)
    A_true = grad_cpu.operator(oracle, g, true, omega)
    Ut, _ = grad_cpu.forward(A_true, (A_bg - A_true) @ u0, u0)
    dobs = grad_cpu.receivers_pred(Ut, rec)
    A = grad_cpu.operator(oracle, g, mdl, omega)
    chi_c, grad_c, _, _ = grad_cpu.misfit_gradient(oracle, g, mdl, omega, (A_bg - A) @ u0, rec, dobs, U0=u0)
    with wt.Solver(g) as s:
        s.set_model(*mdl)
        s.set_background(*bg)
        s.factor(omega)
        F = torch.zeros((len(ain), g.n), dtype=torch.complex128, device="cuda")
        U0 = torch.zeros_like(F)
        s.rhs_planewave(wt.Layered1D(*lay), ain, baz, d_F=F.data_ptr(), d_U0=U0.data_ptr())
        chi_g, grad_g, dpred = s.misfit_gradient(F.data_ptr(), U0.data_ptr(), len(ain), rec, dobs, tol=1e-12,
                                                 maxit=30, allow_noconv=True)
        del F, U0
    errs = [np.abs(grad_g[k] - grad_c[k]).max() / np.abs(grad_c[k]).max() for k in range(3)]
    print("chi rel err %.3e  grad rel err %s" % (abs(chi_g - chi_c) / chi_c, ["%.3e" % e for e in errs]))
    assert abs(chi_g - chi_c) <= 1e-7 * chi_c
    for k in range(3):
        assert errs[k] <= 1e-6, k


def test_gradient_fd_64x64x48():
    """Central differences (step 1e-4 relative, float32-representable steps)
    of the misfit at 20 seeded cells.  Each perturbed wavefield is u + du with
    A(m +- dm) du = -(A(m +- dm) - A(m)) u solved by refinement with the
    resident factors of A(m), so the misfit difference is formed from du
    without cancellation against the misfit itself."""
    nx, ny, nz, h = 64, 64, 48, 25.0
    g = Grid(nx, ny, nz, h, pmld=10 * h, fst=1, usemin=1)
    ipml = g.pml()[2]
    omega = 2 * np.pi * 1.0
    mdl = model.layered_random(nx, ny, nz, h, seed=1)
    bg = model.layered(nx, ny, nz)
    true = model.perturbed(mdl[0], mdl[1], h, seed=2, std=0.03)
    lay = wt.Layered1D(*model.layered1d(nz, h))
    rng = np.random.Generator(np.random.PCG64(41))
    nsrc = 16
    ain = np.radians(rng.uniform(0.0, 30.0, nsrc))
    baz = np.radians(rng.uniform(0.0, 360.0, nsrc))
    rec = model.surface_receivers(nx, ny, nz, ipml, 8, 5)
    n = g.n
    with wt.Solver(g) as s:
        s.set_background(*bg)
        F = torch.zeros((nsrc, n), dtype=torch.complex128, device="cuda")
        U0 = torch.zeros_like(F)
        zero = np.zeros(nsrc * len(rec) * 3, np.complex128)
        # observed data from the true model
        s.set_model(*true)
        s.factor(omega)
        s.rhs_planewave(lay, ain, baz, d_F=F.data_ptr(), d_U0=U0.data_ptr())
        _, _, dobs = s.misfit_gradient(F.data_ptr(), U0.data_ptr(), nsrc, rec, zero, tol=1e-11, maxit=30,
                                       allow_noconv=True)
        # misfit and gradient at the current model
        s.set_model(*mdl)
        s.factor(omega)
        s.rhs_planewave(lay, ain, baz, d_F=F.data_ptr(), d_U0=U0.data_ptr())
        chi, grad, dpred = s.misfit_gradient(F.data_ptr(), U0.data_ptr(), nsrc, rec, dobs, tol=1e-11, maxit=30,
                                             allow_noconv=True)
        assert chi > 0
        # total field u at the current model and A(m) u
        X = torch.zeros_like(F)
        s.solve_device(F.data_ptr(), X.data_ptr(), nsrc, tol=1e-11, maxit=30, allow_noconv=True)
        Ut = X + U0
        Y0 = torch.zeros_like(F)
        s.apply_device(Ut.data_ptr(), Y0.data_ptr(), nsrc)
        idx = torch.from_numpy((3 * rec[:, None] + np.arange(3)[None, :]).reshape(-1)).to("cuda")
        res = (Ut[:, idx].reshape(-1).cpu().numpy() - dobs)
        Y = torch.zeros_like(F)
        dU = torch.zeros_like(F)
        cells = np.stack([rng.integers(0, nz - ipml, 20), rng.integers(ipml, nx - ipml, 20),
                          rng.integers(ipml, ny - ipml, 20)], axis=1)
        worst = 0.0
        for (iz, ix, iy) in cells:
            for which in range(3):
                dR, vals = [], []
                for sgn in (1, -1):
                    m = [np.array(x, np.float32, copy=True) for x in mdl]
                    m[which][iz, ix, iy] = np.float32(m[which][iz, ix, iy] * (1 + sgn * 1e-4))
                    vals.append(float(m[which][iz, ix, iy]))
                    s.set_model(*m)
                    s.update_operator()
                    s.apply_device(Ut.data_ptr(), Y.data_ptr(), nsrc)
                    B = Y0 - Y
                    s.solve_device(B.data_ptr(), dU.data_ptr(), nsrc, tol=1e-10, maxit=30, allow_noconv=True)
                    dR.append(dU[:, idx].reshape(-1).cpu().numpy())
                dchi = np.vdot(res, dR[0] - dR[1]).real + 0.5 * (np.vdot(dR[0], dR[0]).real -
                                                                np.vdot(dR[1], dR[1]).real)
                fd = dchi / (vals[0] - vals[1])
                an = grad[which][iz, ix, iy]
                rel = abs(fd - an) / abs(an)
                worst = max(worst, rel)
                assert rel <= 1e-4, ((iz, ix, iy), which, fd, an)
        s.set_model(*mdl)
        s.update_operator()
        del F, U0, X, Ut, Y0, Y, dU, idx
    print("worst relative FD error", worst)
