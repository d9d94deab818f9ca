"""FP64 CPU waveform-gradient pipeline used as the checker of the GPU
gradient: oracle assembly (complex128), scipy SuperLU forward and
conjugate-transpose solves, oracle gradient contraction.  Test
infrastructure only."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def operator(oracle, g, model, omega):
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a, ierr = oracle.assemble(g, *model, omega, ir)
    assert ierr == 0
    n = len(ir) - 1
    return sp.csr_matrix((a, jc - 1, ir - 1), shape=(n, n))


def receivers_pred(U, rec):
    """pred[(j*nrec + r)*3 + c] = U[3 rec_r + c, j]"""
    idx = (3 * np.asarray(rec)[:, None] + np.arange(3)[None, :]).reshape(-1)
    return U[idx, :].T.reshape(-1)


def misfit(U, rec, dobs):
    r = receivers_pred(U, rec) - dobs
    return 0.5 * float(np.vdot(r, r).real)


def forward(A, B, U0=None):
    lu = spla.splu(A.tocsc())
    X = lu.solve(np.asarray(B, np.complex128))
    if U0 is not None:
        X = X + U0
    return X, lu


def misfit_gradient(oracle, g, model, omega, B, rec, dobs, U0=None):
    """chi, (dchi/dVp, dchi/dVs, dchi/drho), total wavefields, adjoint fields."""
    A = operator(oracle, g, model, omega)
    U, lu = forward(A, B, U0)
    res = receivers_pred(U, rec) - dobs
    S = np.zeros_like(U)
    nrec = len(rec)
    for j in range(U.shape[1]):
        for r in range(nrec):
            for c in range(3):
                S[3 * rec[r] + c, j] += res[(j * nrec + r) * 3 + c]
    Lam = lu.solve(S, trans="H")
    grad = oracle.gradient(g, *model, omega, U, Lam)
    return 0.5 * float(np.vdot(res, res).real), grad, U, Lam
