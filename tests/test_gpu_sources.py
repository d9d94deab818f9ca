"""Device point-force right-hand sides and receiver sampling with
SRCSETUP/SRCREG weights, against host constructions from the same weights."""
import numpy as np
import pytest

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_rhs_sources_and_receivers():
    g = Grid(24, 22, 20, 20.0, pmld=80.0, fst=1)
    xyz = np.array([[207.3, 181.9, 163.1], [120.0, 200.0, 13.1], [300.5, 150.2, 90.0]])
    comp = np.array([2, 0, 1], np.int32)
    sterm = np.array([1.0, 0.5 - 2j, -1j])
    with wt.Solver(g) as s:
        s.set_model(*model.homogeneous(24, 22, 20))
        s.factor(2 * np.pi)
        for ireg, sprd in ((0, 0.5), (3, 0.5), (1, 1.25)):
            F = torch.zeros((3, g.n), dtype=torch.complex128, device="cuda")
            s.rhs_sources(xyz, comp, F.data_ptr(), sterm=sterm, ireg=ireg, sprd=sprd)
            got = F.cpu().numpy()
            for j in range(3):
                ref = np.zeros(g.n, np.complex128)
                node, w = wt.source_weights(g, *xyz[j], ireg, sprd)
                np.add.at(ref, 3 * node + comp[j], w * sterm[j])
                assert np.abs(got[j] - ref).max() <= 1e-14 * np.abs(ref).max()
            # receivers sample with the same weights
            rng = np.random.default_rng(3)
            U = rng.standard_normal((2, g.n)) + 1j * rng.standard_normal((2, g.n))
            dU = torch.from_numpy(U).cuda()
            smp = s.sample_receivers(dU.data_ptr(), 2, xyz, ireg, sprd)
            for j in range(2):
                for r in range(3):
                    node, w = wt.source_weights(g, *xyz[r], ireg, sprd)
                    for c in range(3):
                        assert abs(smp[j, r, c] - np.dot(w, U[j, 3 * node + c])) < 1e-12
            # receiver responses and inactive pairs (makeuh.f:92-103)
            resp = np.array([1.0, 0.5j, -2.0])
            act = np.array([[1, 0, 1], [1, 1, 0]])
            smr = s.sample_receivers(dU.data_ptr(), 2, xyz, ireg, sprd, response=resp, active=act)
            np.testing.assert_allclose(smr, np.where(act[:, :, None] != 0, smp * resp[None, :, None], 0),
                                       rtol=1e-12, atol=1e-14 * np.abs(smp).max())
            del F, dU


def test_pressure_matches_makeuh_restatement():
    """Hydrophone pressure (makeuh.f:113-167) against a numpy restatement on
    the same receiver weights and the model's Lame parameters."""
    g = Grid(24, 22, 20, 20.0, pmld=80.0, fst=1)
    vp, vs, rho = model.layered_random(24, 22, 20, 20.0, seed=4, corr_len=80.0)
    om = 2 * np.pi * 2.0
    xyz = np.array([[207.3, 181.9, 63.1], [120.0, 200.0, 13.1]])
    rng = np.random.default_rng(5)
    U = rng.standard_normal((2, g.n)) + 1j * rng.standard_normal((2, g.n))
    with wt.Solver(g) as s:
        s.set_model(vp, vs, rho)
        s.factor(om)
        dU = torch.from_numpy(U).cuda()
        for ireg in (0, 3):
            got = s.sample_pressure(dU.data_ptr(), 2, xyz, ireg, 0.5)
            act = np.array([[1, 0], [0, 1]])
            np.testing.assert_allclose(s.sample_pressure(dU.data_ptr(), 2, xyz, ireg, 0.5, active=act),
                                       np.where(act != 0, got, 0), rtol=1e-12, atol=1e-14 * np.abs(got).max())
            for j in range(2):
                for r in range(2):
                    x, y, z = xyz[r]
                    div = 0
                    for a in range(3):
                        pm = []
                        for sgn in (-1, 1):
                            q = [x, y, z]
                            q[a] += sgn * g.dx
                            node, w = wt.source_weights(g, *q, ireg, 0.5)
                            pm.append(np.dot(w, U[j, 3 * node + a]))
                        div += -(pm[1] - pm[0]) / (2 * g.dx * (-1j * om))
                    ix, iy, iz = [min(max(int(1.5 + c / g.dx), 1), m) for c, m in ((x, 24), (y, 22), (z, 20))]
                    P, S, R = [float(t[iz - 1, ix - 1, iy - 1]) for t in (vp, vs, rho)]
                    mu = S * S * R
                    lam = P * P * R - 2 * mu
                    assert abs(got[j, r] - (lam + 2 * mu / 3) * div) <= 1e-10 * abs((lam + 2 * mu / 3) * div)
        del dU
