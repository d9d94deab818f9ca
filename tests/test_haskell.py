"""CPU tests of the Thomson-Haskell response: the oracle against the
free-surface closed form of a half-space, and the library's host restatement
(wt3d_haskgrn, no GPU needed) against the oracle."""
import numpy as np
import pytest

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import model


def halfspace(vp=5000.0, vs=2887.0, rho=2700.0):
    # two identical layers: the reference needs nl >= 2 (haskgrn.f:427-434)
    return (np.array([vp, vp]), np.array([vs, vs]), np.array([rho, rho]), np.array([0.0, 500.0]))


@pytest.mark.parametrize("ain_deg", [5.0, 15.0, 25.0, 35.0])
def test_free_surface_p_ratio(oracle, ain_deg):
    """Incident P on a free surface: |u_r/u_z| = 2 p eta_b / (1/b^2 - 2 p^2)."""
    vp, vs, rho, zt = halfspace()
    ain = np.radians(ain_deg)
    U, W = oracle.haskgrn(vp, vs, rho, zt, 2 * np.pi * 1.0, ain, 4, 20.0)
    p = np.sin(ain) / vp[0]
    eb = np.sqrt(1 / vs[0] ** 2 - p * p)
    want = 2 * p * eb / (1 / vs[0] ** 2 - 2 * p * p)
    np.testing.assert_allclose(abs(U[0]) / abs(W[0]), want, rtol=1e-10)


def test_normal_incidence_doubling(oracle):
    """Near-vertical incidence: the free surface doubles the vertical amplitude."""
    vp, vs, rho, zt = halfspace()
    U, W = oracle.haskgrn(vp, vs, rho, zt, 2 * np.pi, np.radians(0.01), 2, 20.0)
    np.testing.assert_allclose(abs(W[0]), 2.0, rtol=1e-6)
    assert abs(U[0]) < 1e-3


@pytest.mark.parametrize("s_wave", [False, True])
@pytest.mark.parametrize("f", [0.5, 2.0])
def test_library_haskgrn_matches_oracle(oracle, s_wave, f):
    """The product's host restatement equals the oracle's (config-2 layering,
    64 nodes, both quirks exercised: layer refresh and half-space nodes)."""
    nz, dx = 64, 20.0
    vp, vs, rho, zt = model.layered1d(nz, dx)
    ain = np.radians(22.0)
    Uo, Wo = oracle.haskgrn(vp, vs, rho, zt, 2 * np.pi * f, ain, nz, dx, s_wave)
    L = wt.Layered1D(vp, vs, rho, zt)
    U, W = wt.haskgrn(L, 2 * np.pi * f, ain, nz, dx, s_wave)
    scale = max(np.abs(Uo).max(), np.abs(Wo).max())
    assert np.abs(U - Uo).max() <= 1e-12 * scale
    assert np.abs(W - Wo).max() <= 1e-12 * scale
    assert np.all(np.isfinite(U)) and np.all(np.isfinite(W))


def test_node_above_model_top_is_rejected(oracle):
    """The reference's dloc < 0 guard (haskgrn.f:435-440): a node depth above
    the top of the 1-D model is an error in the oracle and in the library;
    the same model starting at the surface is accepted."""
    import ctypes
    vp, vs, rho, zt = halfspace()
    zt_low = zt + 50.0                 # model top 50 m below the surface
    arr = [np.ascontiguousarray(a, np.float64) for a in (vp, vs, rho, zt_low)]
    U = np.zeros(4, np.complex128)
    W = np.zeros(4, np.complex128)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = oracle.L.ora_haskgrn(2, *[p(a) for a in arr], 2 * np.pi, np.radians(10.0), 0, 4, 20.0, 0.0, p(U), p(W))
    assert rc != 0
    with pytest.raises(wt.WT3DError):
        wt.haskgrn(wt.Layered1D(vp, vs, rho, zt_low), 2 * np.pi, np.radians(10.0), 4, 20.0)
    wt.haskgrn(wt.Layered1D(vp, vs, rho, zt), 2 * np.pi, np.radians(10.0), 4, 20.0)
