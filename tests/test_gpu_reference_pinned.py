"""GPU parity against outputs of the reference's own Fortran statements
(tests/golden/ref_*.npz, made by tests/golden/make_reference_golden.py from
the reference's source text): the CUDA pattern bit for bit, the CUDA operator
values to 1e-12 relative in complex128 (plain and after Q dispersion), the
scattered-field plane-wave sources, and the device point sources."""
import numpy as np
import pytest
import scipy.sparse as sp

import make_reference_golden as mrg
import wtomo3d_gb300 as wt
from test_gpu_assembly import check_values
from wtomo3d_gb300 import Grid

pytestmark = pytest.mark.gpu


def load(name):
    return dict(np.load(mrg.path(name)))


def grid_of(z):
    nx, ny, nz = (int(v) for v in z["dims"])
    return Grid(nx, ny, nz, float(z["dx"]), pmld=float(z["pmld"]), fst=int(z["fst"]), usemin=int(z["usemin"]))


@pytest.mark.parametrize("name", sorted(mrg.ASM_CASES))
def test_cuda_assembly_matches_reference_statements(name):
    z = load("asm_" + name)
    g = grid_of(z)
    ir, jc = wt.pattern(g.nx, g.ny, g.nz, base=1)
    np.testing.assert_array_equal(ir, z["irptr"])
    np.testing.assert_array_equal(jc, z["jcptr"])
    a = wt.assemble(g, z["vp"], z["vs"], z["rho"], complex(z["omega"]))
    check_values(a, z["a"], z["irptr"])


def test_cuda_dispersed_operator_matches_reference_statements():
    """The device operator after the fused Q step, probed by products with
    random vectors against the reference's DISPERSION + ASMBLE operator."""
    z = load("asm_q")
    g = grid_of(z)
    n = g.n
    A = sp.csr_matrix((z["a"], z["jcptr"] - 1, z["irptr"] - 1), shape=(n, n))
    rng = np.random.default_rng(4)
    P = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    with wt.Solver(g) as s:
        s.set_model(z["vp"], z["vs"], z["rho"])
        s.set_attenuation(z["qp"], z["qs"], freqbase=float(z["freqbase"]))
        s.factor(complex(z["omega"]))
        Y = s.apply(P)
    assert np.abs(Y - A @ P).max() <= 1e-12 * (abs(A) @ abs(P)).max()


def test_cuda_planewave_sources_match_reference_hetfldsrc():
    z = load("hetfldsrc")
    g = grid_of(z)
    lay = wt.Layered1D(z["lay_vp"], z["lay_vs"], z["lay_rho"], z["lay_zt"])
    w = z["waves"]
    with wt.Solver(g) as s:
        s.set_model(z["vp"], z["vs"], z["rho"])
        s.set_background(z["vp0"], z["vs0"], z["rho0"])
        s.factor(complex(z["omega"]))
        F, U0 = s.rhs_planewave(lay, np.radians(w[:, 0]), np.radians(w[:, 1]), w[:, 2].astype(np.int32))
    for j in range(len(w)):
        assert np.abs(U0[:, j] - z["u0"][j]).max() <= 1e-12 * np.abs(z["u0"][j]).max()
        assert np.abs(F[:, j] - z["f"][j]).max() <= 1e-11 * np.abs(z["f"][j]).max()


def test_cuda_point_sources_match_reference_srcsetup():
    """Device right-hand sides of unit vertical forces against SRCSETUP's
    spread fields (1e-7 where the reference's polynomial I0 enters)."""
    import torch
    z = load("srcsetup")
    nx, ny, nz = (int(v) for v in z["dims"])
    dx = float(z["dx"])
    g = Grid(nx, ny, nz, dx, pmld=2 * dx, fst=1, usemin=1)
    rng = np.random.default_rng(0)
    vp = np.full((nz, nx, ny), 4000.0, np.float32)
    with wt.Solver(g) as s:
        s.set_model(vp, vp / 1.8, np.full_like(vp, 2500.0))
        s.factor(2 * np.pi)
        for k, (x, y, zz, ireg, sprd) in enumerate(z["cases"]):
            F = torch.zeros((1, g.n), dtype=torch.complex128, device="cuda")
            s.rhs_sources(np.array([[x, y, zz]]), np.array([2], np.int32), F.data_ptr(), ireg=int(ireg),
                          sprd=float(sprd))
            got = F.cpu().numpy()[0, 2::3]
            ref = z["swave"][k]
            tol = 1e-7 if (int(ireg) > 0 and sprd <= 0.5) else 1e-14
            assert np.abs(got - ref).max() <= tol * np.abs(ref).max(), (k, np.abs(got - ref).max())
            assert np.abs(F.cpu().numpy()[0, 0::3]).max() == 0
            del F
