"""CPU tests of the oracle: pattern, the reference's own self-checks, physics
known answers, precision modes, and the committed golden fixtures."""
import os

import numpy as np
import pytest

from wtomo3d_gb300 import Grid, model

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def box_pattern(nx, ny, nz):
    """Independent construction of the 27-point 3-dof CSR (1-based)."""
    rows, cols = [], []
    for iy in range(ny):
        for ix in range(nx):
            for iz in range(nz):
                g = iz + nz * (ix + nx * iy)
                nb = []
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        for dz in (-1, 0, 1):
                            y, x, z = iy + dy, ix + dx, iz + dz
                            if 0 <= y < ny and 0 <= x < nx and 0 <= z < nz:
                                nb.append(z + nz * (x + nx * y))
                for r in range(3):
                    rows.append([3 * h + q + 1 for h in nb for q in range(3)])
    irptr = np.cumsum([1] + [len(r) for r in rows]).astype(np.int32)
    return irptr, np.concatenate(rows).astype(np.int32)


@pytest.mark.parametrize("dims", [(2, 2, 2), (3, 4, 5), (5, 3, 2), (7, 6, 4)])
def test_pattern_closed_form_and_definition(oracle, dims):
    nx, ny, nz = dims
    n, nedge = oracle.getsize(nx, ny, nz)
    assert n == 3 * nx * ny * nz
    # srgraphs.f:626-636 closed form: nzero = 2 nedge + numvert
    assert 2 * nedge + n == 9 * (3 * nx - 2) * (3 * ny - 2) * (3 * nz - 2)
    ir, jc = oracle.pattern(nx, ny, nz)
    ir2, jc2 = box_pattern(nx, ny, nz)
    np.testing.assert_array_equal(ir, ir2)
    np.testing.assert_array_equal(jc, jc2)
    # every row holds its diagonal, columns ascending
    for i in range(n):
        row = jc[ir[i] - 1:ir[i + 1] - 1]
        assert np.all(np.diff(row) > 0)
        assert (i + 1) in row


@pytest.mark.parametrize("fst,usemin", [(0, 1), (1, 1), (1, 0)])
def test_row_nnz_selfcheck(oracle, fst, usemin):
    # asmble.f90:556-564 / 619-626: every row fits its irptr slot
    g = Grid(9, 8, 10, 25.0, pmld=2 * 25.0, fst=fst, usemin=usemin)
    vp, vs, rho = model.homogeneous(g.nx, g.ny, g.nz)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a, ierr = oracle.assemble(g, vp, vs, rho, 2 * np.pi, ir)
    assert ierr == 0
    assert np.all(np.isfinite(a))


def test_rigid_translation_interior(oracle):
    """Homogeneous interior rows annihilate constants in the stiffness part and
    the lumped mass weights sum to one: A (1,0,0) = omega^2 rho (1,0,0)."""
    g = Grid(14, 13, 15, 25.0, pmld=3 * 25.0, fst=0)
    vp, vs, rho = model.homogeneous(g.nx, g.ny, g.nz)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    w = 2 * np.pi * 1.3
    a, ierr = oracle.assemble(g, vp, vs, rho, w, ir)
    import scipy.sparse as sp
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    _, _, ipml = g.pml()
    for comp in range(3):
        x = np.zeros(g.n)
        x[comp::3] = 1
        y = A @ x
        for (iz, ix, iy) in [(8, 7, 7), (ipml + 1, ipml + 1, ipml + 1), (g.nz - ipml, g.nx - ipml, g.ny - ipml)]:
            gi = (iz - 1) + g.nz * (ix - 1) + g.nz * g.nx * (iy - 1)
            np.testing.assert_allclose(y[3 * gi + comp], w * w * 2700.0, rtol=1e-12)
            for c2 in range(3):
                if c2 != comp:
                    assert abs(y[3 * gi + c2]) < 1e-9 * w * w * 2700.0


def _plane_wave_residual(oracle, f, d, pol, c):
    import scipy.sparse as sp
    g = Grid(24, 24, 24, 20.0, pmld=2 * 20.0, fst=0)
    vp, vs, rho = model.homogeneous(g.nx, g.ny, g.nz, 3000.0, 1732.0, 2400.0)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    w = 2 * np.pi * f
    a, _ = oracle.assemble(g, vp, vs, rho, w, ir)
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    iz, ix, iy = np.meshgrid(np.arange(g.nz), np.arange(g.nx), np.arange(g.ny), indexing="ij")
    xs = np.stack([ix, iy, iz], -1).reshape(-1, 3, order="F") * g.dx   # node order
    ph = np.exp(1j * (w / c) * xs @ d)
    u = np.zeros(g.n, complex)
    for q in range(3):
        u[q::3] = pol[q] * ph
    r = A @ u
    gi = 11 + 24 * 11 + 576 * 11
    return np.abs(r[3 * gi:3 * gi + 3]).max() / (w * w * 2400.0)


def test_plane_wave_dispersion_xz():
    """Discrete plane P and S waves travelling in the x-z plane nearly satisfy
    the homogeneous interior rows, with an O((kh)^2) residual."""
    from oracle_ctypes import Oracle
    o = Oracle()
    d = np.array([0.6, 0.0, 0.8])
    p_lo = _plane_wave_residual(o, 2.0, d, d, 3000.0)
    p_hi = _plane_wave_residual(o, 4.0, d, d, 3000.0)
    assert p_hi < 0.01 and p_lo < p_hi / 3.0, (p_lo, p_hi)
    s_pol = np.array([0.8, 0.0, -0.6])
    s_lo = _plane_wave_residual(o, 1.0, d, s_pol, 1732.0)
    s_hi = _plane_wave_residual(o, 2.0, d, s_pol, 1732.0)
    assert s_hi < 0.01 and s_lo < s_hi / 3.0, (s_lo, s_hi)
    # the wrong speed leaves an O(1) residual
    assert _plane_wave_residual(o, 2.0, d, d, 1500.0) > 0.3


def test_reference_stencil_v_anisotropy(oracle):
    """Pins a quirk of the reference interior stencil (pfdfd3d.f:216-226 a2n,
    pfdfd3d.f:343-355 a5m): the v (y) displacement couples to its x neighbours
    with lambda+2mu and to its y neighbours with mu, so K applied to
    v = y^2 yields 2 mu (not 2(lambda+2mu)) and v = x^2 yields 2(lambda+2mu).
    The GPU path reproduces this exactly; it is documented, not corrected."""
    import scipy.sparse as sp
    g = Grid(12, 12, 12, 1.0, pmld=2.0, fst=0)
    lam, mu = 2.0, 1.0
    vp, vs, rho = model.homogeneous(12, 12, 12, np.sqrt(lam + 2 * mu), np.sqrt(mu), 1.0)
    ir, jc = oracle.pattern(12, 12, 12)
    a, _ = oracle.assemble(g, vp, vs, rho, 0.0, ir)
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    iz, ix, iy = np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij")
    X, Y, Z = [t.reshape(-1, order="F").astype(float) for t in (ix, iy, iz)]
    gi = 6 + 12 * 6 + 144 * 6

    def f(ux, uy, uz):
        u = np.zeros(g.n)
        u[0::3], u[1::3], u[2::3] = ux, uy, uz
        return (A @ u)[3 * gi:3 * gi + 3].real

    np.testing.assert_allclose(f(X ** 2, 0 * X, 0 * X), [2 * (lam + 2 * mu), 0, 0], atol=1e-9)
    np.testing.assert_allclose(f(0 * X, 0 * X, Z ** 2), [0, 0, 2 * (lam + 2 * mu)], atol=1e-9)
    np.testing.assert_allclose(f(0 * X, Y ** 2, 0 * X), [0, 2 * mu, 0], atol=1e-9)
    np.testing.assert_allclose(f(0 * X, X ** 2, 0 * X), [0, 2 * (lam + 2 * mu), 0], atol=1e-9)


def test_c64_mode_tracks_c128(oracle):
    g = Grid(10, 9, 11, 20.0, pmld=3 * 20.0, fst=1)
    vp, vs, rho = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=3)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a128, e1 = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.5, ir, "c128")
    a64, e2 = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.5, ir, "c64")
    assert e1 == 0 and e2 == 0
    err = np.abs(a64 - a128).max() / np.abs(a128).max()
    assert err < 1e-6, err


def test_free_surface_paths_differ(oracle):
    """usemin (Min cells, PFDFD/PML rows) and TPFREE rows differ only on the top plane."""
    g1 = Grid(8, 8, 9, 25.0, pmld=2 * 25.0, fst=1, usemin=1)
    g2 = Grid(8, 8, 9, 25.0, pmld=2 * 25.0, fst=1, usemin=0)
    vp, vs, rho = model.homogeneous(8, 8, 9)
    ir, jc = oracle.pattern(8, 8, 9)
    a1, _ = oracle.assemble(g1, vp, vs, rho, 2 * np.pi, ir)
    a2, _ = oracle.assemble(g2, vp, vs, rho, 2 * np.pi, ir)
    rows = np.repeat(np.arange(g1.n), np.diff(ir))
    iz = (rows // 3) % g1.nz
    diff = np.abs(a1 - a2) > 0
    assert diff.any()
    assert np.all(iz[diff] == 0)


@pytest.mark.parametrize("name", ["asm_c1_small", "asm_fst_tpfree", "asm_layered"])
def test_golden_fixtures(oracle, name):
    """Regression pin of the oracle against fixtures made by tests/golden/make_golden.py."""
    import make_golden
    g, vp, vs, rho, om, z = make_golden.load_case(name)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    np.testing.assert_array_equal(ir, z["irptr"])
    np.testing.assert_array_equal(jc, z["jcptr"])
    a, ierr = oracle.assemble(g, vp, vs, rho, om, ir)
    assert ierr == 0
    np.testing.assert_allclose(a, z["a"], rtol=0, atol=1e-13 * np.abs(z["a"]).max())


def test_dispersion_oracle_limits(oracle):
    """DISPERSION (dispersion.f:78-114): 1/Q = 0 leaves the elastic operator;
    at Re(omega) = 2 pi freqbase only the imaginary velocity part appears, so
    the operator's real part is that of the elastic one up to O(1/Q^2)."""
    import numpy as np
    from wtomo3d_gb300 import Grid, model
    g = Grid(10, 9, 8, 25.0, pmld=50.0, fst=1)
    vp, vs, rho = model.layered_random(10, 9, 8, 25.0, seed=2, corr_len=50.0)
    ir, jc = oracle.pattern(10, 9, 8)
    zero = np.zeros_like(vp)
    om = 2 * np.pi * 3.0
    a0, _ = oracle.assemble(g, vp, vs, rho, om, ir)
    aq0, _ = oracle.assemble_q(g, vp, vs, rho, zero, zero, 20.0, om, ir)
    assert np.abs(aq0 - a0).max() <= 1e-12 * np.abs(a0).max()
    q = np.full_like(vp, 0.01)
    aq, _ = oracle.assemble_q(g, vp, vs, rho, q, q, 3.0, om, ir)
    assert np.abs(aq.imag).max() > 1e-4 * np.abs(a0).max()          # attenuation present
    assert np.abs(aq.real - a0.real).max() <= 1e-3 * np.abs(a0).max()  # (1 - i q/2)^2: real part 1 - q^2/4


def test_pml_without_damping_is_the_interior_stencil(oracle):
    """The reference's PML fidelity hooks (fdfd3d.f:56-57, pml3d.f:297-304):
    with zero damping (pmlr = 1, so pmlf = 3 ln(1/pmlr) / (2 pmld^3) = 0,
    hence r1 = 1 and r2 = 0) every row inside a 6-node PML equals the same row
    assembled as an interior row (a grid whose PML is only the boundary
    layer), bit for bit.  omega is real, so the REAL(omega^2) quirk of the
    interior mass terms (pfdfd3d.f:140-142) cannot differ."""
    import scipy.sparse as sp
    nx, ny, nz, dx = 14, 13, 12, 20.0
    vp, vs, rho = model.layered_random(nx, ny, nz, dx, seed=3)
    om = 2 * np.pi * 1.3
    ir, jc = oracle.pattern(nx, ny, nz)
    g_pml = Grid(nx, ny, nz, dx, pmld=5 * dx, pmlr=1.0, fst=0)
    g_int = Grid(nx, ny, nz, dx, pmld=0.5 * dx, pmlr=1.0, fst=0)
    assert g_pml.pml()[1] == 0.0 and g_pml.pml()[2] == 6 and g_int.pml()[2] == 1
    a_pml, e1 = oracle.assemble(g_pml, vp, vs, rho, om, ir)
    a_int, e2 = oracle.assemble(g_int, vp, vs, rho, om, ir)
    assert e1 == 0 and e2 == 0
    n = g_pml.n
    A = sp.csr_matrix((a_pml, jc - 1, ir - 1), shape=(n, n))
    B = sp.csr_matrix((a_int, jc - 1, ir - 1), shape=(n, n))
    rows = []
    for iy in range(2, ny):
        for ix in range(2, nx):
            for iz in range(2, nz):
                if min(ix, iy, iz) <= 6 or ix > nx - 6 or iy > ny - 6 or iz > nz - 6:
                    g = (iz - 1) + nz * (ix - 1) + nz * nx * (iy - 1)
                    rows += [3 * g, 3 * g + 1, 3 * g + 2]
    rows = np.array(rows)
    assert rows.size > 3000
    assert (A[rows] != B[rows]).nnz == 0
    # with damping the same rows do differ: the comparison has teeth
    a_damped, _ = oracle.assemble(Grid(nx, ny, nz, dx, pmld=5 * dx, fst=0), vp, vs, rho, om, ir)
    D = sp.csr_matrix((a_damped, jc - 1, ir - 1), shape=(n, n))
    assert (D[rows] != B[rows]).nnz > 0
