"""GPU tests of the general-pattern path: wt3d_solver_create_csr and the
job protocol with a CSR pattern that is not the grid graph (STRUMPACK takes
any pattern, strumpack_finter.c:42-48).  The same kernels factor and solve;
only the ordering, the scatter map and the FP64 residual kernel differ."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

pytestmark = pytest.mark.gpu


def elastic(oracle, g, seed, f=1.0, dtype="c128"):
    vp, vs, rho = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=seed)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a, ierr = oracle.assemble(g, vp, vs, rho, 2 * np.pi * f, ir, dtype)
    assert ierr == 0
    return sp.csr_matrix((a.astype(np.complex128), jc - 1, ir - 1), shape=(g.n, g.n)), (vp, vs, rho)


def rhs(n, k, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))


def point_loads(g, k, seed):
    """k physical loads for the elastic operator: three point forces each at
    seeded nodes away from the Dirichlet faces (a dense random vector is not
    a meaningful load: |A||x|/|b| reaches 1e10)."""
    r = np.random.default_rng(seed)
    B = np.zeros((g.n, k), complex)
    for j in range(k):
        for _ in range(3):
            iz, ix, iy = r.integers(0, g.nz - 1), r.integers(1, g.nx - 1), r.integers(1, g.ny - 1)
            node = iz + g.nz * (ix + g.nx * iy)
            B[3 * node + r.integers(0, 3), j] += r.standard_normal() + 1j * r.standard_normal()
    return B


@pytest.mark.parametrize("prec", [wt.PREC_MIXED, wt.PREC_FP64])
def test_node_permuted_operator_matches_grid_handle(oracle, prec):
    """The elastic operator under a random node permutation, through the
    general handle (complex128 values), gives the grid handle's wavefields,
    forward and adjoint."""
    g = Grid(14, 12, 13, 20.0, pmld=3 * 20.0, fst=1)
    A, (vp, vs, rho) = elastic(oracle, g, seed=11)
    q = np.random.default_rng(5).permutation(g.nnodes)
    perm = (3 * q[:, None] + np.arange(3)).reshape(-1)
    Ap = sp.csr_matrix(A[perm][:, perm])
    B = point_loads(g, 3, 1)
    with wt.Solver(g, prec) as s:
        s.set_model(vp, vs, rho)
        s.factor(2 * np.pi * 1.0)
        Xg = s.solve(B, tol=1e-10, maxit=30)
        Yg = s.solve_adjoint(B, tol=1e-10, maxit=30)
    with wt.Solver.from_csr(Ap.indptr, Ap.indices, prec) as s:
        s.set_values(Ap.data, np.complex128)
        Xp = s.solve(B[perm], tol=1e-10, maxit=30)
        assert s.last_relres.max() <= 1e-10
        Yp = s.solve_adjoint(B[perm], tol=1e-10, maxit=30)
        st = s.stats()
        assert st["nnz"] == Ap.nnz
        # A x through the general residual kernel
        Z = s.apply(Xp)
    # both orderings meet the residual target; the wavefields then agree to
    # the operator's conditioning (a dense 1e-10 residual moves this
    # solution by ~1e-3, a load-shaped one by 1e-10)
    for Xa, Xb in ((Xg, Xp), (Yg, Yp)):
        assert np.linalg.norm(Xa[perm] - Xb) / np.linalg.norm(Xa) <= 1e-6
    np.testing.assert_allclose(Z, Ap @ Xp, rtol=0, atol=1e-11 * np.abs(Ap @ Xp).max())
    res = np.linalg.norm(B[perm] - Ap @ Xp, axis=0) / np.linalg.norm(B, axis=0)
    assert res.max() <= 2e-10
    resa = np.linalg.norm(B[perm] - Ap.conj().T @ Yp, axis=0) / np.linalg.norm(B, axis=0)
    assert resa.max() <= 2e-10


def test_random_pattern_unsorted_rows_both_precisions():
    """A random structurally symmetric complex matrix (rows in random column
    order, some rows without a diagonal entry) against SuperLU."""
    rng = np.random.default_rng(2)
    n = 2500
    R = sp.random(n, n, density=3e-3, random_state=3, format="csr")
    P = sp.csr_matrix(((R + R.T) != 0).astype(float) + sp.eye(n))
    A = sp.csr_matrix(P, dtype=complex, copy=True)
    A.data = rng.standard_normal(A.nnz) + 1j * rng.standard_normal(A.nnz)
    A = sp.csr_matrix(A + sp.diags(4.0 + np.abs(A).sum(axis=1).A1 * (rng.random(n) < 0.5)))
    A.eliminate_zeros()
    ind, dat = A.indices.copy(), A.data.copy()
    for r in range(n):
        s0, s1 = A.indptr[r], A.indptr[r + 1]
        o = rng.permutation(s1 - s0)
        ind[s0:s1], dat[s0:s1] = ind[s0:s1][o], dat[s0:s1][o]
    B0 = rhs(n, 4, 3)
    Xr = spla.spsolve(A.tocsc(), B0)
    for prec in (wt.PREC_MIXED, wt.PREC_FP64):
        with wt.Solver.from_csr(A.indptr, ind, prec) as s:
            s.set_values(dat, np.complex128)
            X = s.solve(B0, tol=1e-10, maxit=30)
        assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) <= 1e-7     # condition number ~8.5e3


def test_disconnected_pattern_with_isolated_unknowns():
    """Separate meshes and isolated unknowns: fronts without a border below
    the root, and separators that touch nothing."""
    n1 = 40
    T = sp.diags([np.ones(n1 - 1), np.ones(n1), np.ones(n1 - 1)], [-1, 0, 1])
    P = sp.block_diag([sp.kron(sp.eye(n1), T) + sp.kron(T, sp.eye(n1)), sp.eye(50), sp.kron(T, T)]).tocsr()
    rng = np.random.default_rng(4)
    A = sp.csr_matrix(P, dtype=complex, copy=True)
    A.data = rng.standard_normal(A.nnz) + 1j * rng.standard_normal(A.nnz)
    A = sp.csr_matrix(A + sp.diags(1.0 + np.abs(A).sum(axis=1).A1))
    B0 = rhs(A.shape[0], 2, 5)
    with wt.Solver.from_csr(A.indptr, A.indices) as s:
        s.set_values(A.data)      # complex64, as the job protocol passes them
        X = s.solve(B0, tol=1e-10)
    A64 = A.astype(np.complex64).astype(np.complex128)
    res = np.linalg.norm(B0 - A64 @ X, axis=0) / np.linalg.norm(B0, axis=0)
    assert res.max() <= 2e-10


def test_grid_only_calls_refuse_a_general_handle():
    P = sp.csr_matrix(sp.eye(30) + sp.eye(30, k=1) + sp.eye(30, k=-1))
    with wt.Solver.from_csr(P.indptr, P.indices) as s:
        for call in (lambda: wt.lib().wt3d_factor(s._h, 1.0, 0.0),
                     lambda: wt.lib().wt3d_set_model(s._h, None, None, None),
                     lambda: wt.lib().wt3d_update_operator(s._h)):
            with pytest.raises(wt.WT3DError) as e:
                wt._check(call())
            assert e.value.code == wt.WT3D_ERR_STATE
    with pytest.raises(wt.WT3DError) as e:
        wt.Solver.from_csr([0, 2, 3], [0, 0, 1])     # duplicate entry
    assert e.value.code == wt.WT3D_ERR_PATTERN


def test_unsymmetric_pattern_handle_and_job_protocol():
    """An unsymmetric pattern (upwinded convection-diffusion) is stored as
    A + A^T with zeros in the added entries: the handle in both precisions
    and the job protocol (1-based, complex64) solve it like SuperLU."""
    from test_symbolic import convection_diffusion
    A = convection_diffusion(60, seed=3)
    n = A.shape[0]
    B0 = rhs(n, 2, 6)
    Xr = spla.spsolve(A.tocsc(), B0)
    for prec in (wt.PREC_MIXED, wt.PREC_FP64):
        with wt.Solver.from_csr(A.indptr, A.indices, prec) as s:
            s.set_values(A.data, np.complex128)
            X = s.solve(B0, tol=1e-10)
            Y = s.apply(X)
            assert s.stats()["nnz"] == ((A + A.T) != 0).sum()
        assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) <= 1e-8
        np.testing.assert_allclose(Y, A @ X, rtol=0, atol=1e-12 * np.abs(A @ X).max())
    ir = (A.indptr + 1).astype(np.int32)
    jc = (A.indices + 1).astype(np.int32)
    a = A.data.astype(np.complex64)
    dummy = np.zeros(n, np.complex64)
    assert wt.strumpack_serial_finter(1, n, A.nnz, ir, jc, a, dummy, dummy.copy()) == 0
    try:
        assert wt.strumpack_serial_finter(2, n, A.nnz, ir, jc, a, dummy, dummy.copy()) == 0
        b = B0[:, 0].astype(np.complex64)
        sol = np.zeros(n, np.complex64)
        assert wt.strumpack_serial_finter(3, n, A.nnz, ir, jc, a, b, sol) == 0
        A64 = A.astype(np.complex64).astype(np.complex128)
        xr = spla.spsolve(A64.tocsc(), b.astype(np.complex128))
        assert np.linalg.norm(sol - xr) / np.linalg.norm(xr) <= 1e-6
    finally:
        assert wt.strumpack_serial_finter(-1, n, A.nnz, ir, jc, a, dummy, dummy.copy()) == 0


def test_job_protocol_with_a_permuted_operator(oracle):
    """strumpack_serial_finter with the reference's complex64 operator under
    a random node permutation: job 1 does not recognise the grid graph and
    falls back to the general ordering; jobs 2 and 3 solve as before."""
    g = Grid(10, 9, 11, 20.0, pmld=3 * 20.0, fst=1)
    vp, vs, rho = model.layered_random(g.nx, g.ny, g.nz, g.dx, seed=2)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a64, ierr = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir, "c64")
    assert ierr == 0
    A = sp.csr_matrix((a64, jc - 1, ir - 1), shape=(g.n, g.n))
    q = np.random.default_rng(8).permutation(g.nnodes)
    perm = (3 * q[:, None] + np.arange(3)).reshape(-1)
    Ap = sp.csr_matrix(A[perm][:, perm])
    Ap.sort_indices()
    irp = (Ap.indptr + 1).astype(np.int32)
    jcp = (Ap.indices + 1).astype(np.int32)
    ap = Ap.data.astype(np.complex64)
    n, nnz = g.n, Ap.nnz
    dummy = np.zeros(n, np.complex64)
    assert wt.strumpack_serial_finter(1, n, nnz, irp, jcp, ap, dummy, dummy.copy()) == 0
    try:
        assert wt.strumpack_serial_finter(2, n, nnz, irp, jcp, ap, dummy, dummy.copy()) == 0
        b = point_loads(g, 1, 9)[perm, 0].astype(np.complex64)
        sol = np.zeros(n, np.complex64)
        assert wt.strumpack_serial_finter(3, n, nnz, irp, jcp, ap, b, sol) == 0
        xr = spla.spsolve(Ap.astype(np.complex128).tocsc(), b.astype(np.complex128))
        assert np.linalg.norm(sol - xr) / np.linalg.norm(xr) <= 1e-6
        assert wt.lib().wt3d_finter_last_relres() <= 1e-10
    finally:
        assert wt.strumpack_serial_finter(-1, n, nnz, irp, jcp, ap, dummy, dummy.copy()) == 0
