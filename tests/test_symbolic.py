"""CPU tests of the host analysis (nested dissection + symbolic
factorisation) exported by libwtomo3d_gpu without a GPU: the ordering is a
permutation, fronts are in postorder, every operator entry falls inside its
front, and a dense numpy multifrontal LU run over the exported structure
solves A x = b like SuperLU does."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model


def export(nx, ny, nz, leaf=64):
    L = wt.lib()
    info = (ctypes.c_longlong * 8)()
    fl = ctypes.c_double()
    L.wt3d_analyse_info.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_void_p]
    assert L.wt3d_analyse_info(nx, ny, nz, leaf, info, ctypes.byref(fl)) == 0
    nf, nb = info[0], info[5]
    n = 3 * nx * ny * nz
    perm = np.zeros(n, np.int32)
    arrs = [np.zeros(nf, np.int32) for _ in range(5)]
    border = np.zeros(nb, np.int32)
    rel = np.zeros(nb, np.int32)
    L.wt3d_analyse_export.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 8
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    assert L.wt3d_analyse_export(nx, ny, nz, leaf, p(perm), *[p(a) for a in arrs], p(border), p(rel)) == 0
    fp, fb, ffirst, fpar, flev = arrs
    return dict(perm=perm, p=fp, b=fb, first=ffirst, parent=fpar, level=flev, border=border, rel=rel,
                info=list(info), flops=fl.value)


@pytest.mark.parametrize("dims,leaf", [((6, 5, 7), 8), ((9, 9, 6), 27), ((40, 40, 40), 64)])
def test_structure(dims, leaf):
    e = export(*dims, leaf)
    n = 3 * np.prod(dims)
    assert np.array_equal(np.sort(e["perm"]), np.arange(n))
    # pivots of the fronts tile 0..n-1 in postorder
    assert e["first"][0] == 0
    assert np.all(e["first"][1:] == e["first"][:-1] + e["p"][:-1])
    assert e["first"][-1] + e["p"][-1] == n
    assert e["parent"][-1] == -1 and e["b"][-1] == 0
    for f, par in enumerate(e["parent"][:-1]):
        assert par > f and e["level"][par] == e["level"][f] - 1
    off = np.concatenate([[0], np.cumsum(e["b"])])
    for f in range(len(e["p"])):
        bd = e["border"][off[f]:off[f + 1]]
        assert np.all(np.diff(bd) > 0)
        assert bd.size == 0 or bd[0] >= e["first"][f] + e["p"][f]
    # factor entries (fronts start at even offsets: 16-byte-aligned complex64
    # blocks) and flops agree with the per-front formula
    p, b = e["p"].astype(float), e["b"].astype(float)
    fac = 0
    for pf, bf in zip(e["p"].tolist(), e["b"].tolist()):
        fac += fac & 1
        fac += pf * (pf + bf) + bf * pf
    assert e["info"][1] == fac
    np.testing.assert_allclose(e["flops"], (8 * (p ** 3 / 3 + p * p * b + p * b * b)).sum(), rtol=1e-12)


def test_tma_addressable_substitution_blocks():
    """96x96x64: fronts start at even offsets, so a substitution block is
    16-byte aligned exactly when its stride is even (L21: p, U12: p + b).
    Among the blocks the tall-skinny tensor-core kernel takes (M >= 128,
    K >= 256), about half of the bytes qualify for TMA (49 %)."""
    e = export(96, 96, 64)
    p, b = e["p"].astype(np.int64), e["b"].astype(np.int64)
    fac, off = 0, []
    for pf, bf in zip(p.tolist(), b.tolist()):
        fac += fac & 1
        off.append(fac)
        fac += pf * (pf + bf) + bf * pf
    off = np.array(off)
    assert e["info"][1] == fac
    tot = ok = 0
    for f in range(len(p)):
        pf, bf = int(p[f]), int(b[f])
        if bf >= 128 and pf >= 256:   # forward border update: L21 (b x p, stride p)
            base = off[f] + pf * (pf + bf)
            tot += bf * pf
            ok += bf * pf if (base % 2 == 0 and pf % 2 == 0) else 0
        if pf >= 128 and bf >= 256:   # backward: U12 (p x b, stride p + b)
            base = off[f] + pf
            tot += bf * pf
            ok += bf * pf if (base % 2 == 0 and (pf + bf) % 2 == 0) else 0
    assert tot > 0 and 0.45 < ok / tot < 0.55, ok / tot


def test_top_separator_size():
    # 96x96x64: the first cut is the x = 48 plane, 96*64 nodes = 18432 dofs
    e = export(96, 96, 64)
    assert e["p"][-1] == 18432 and e["b"][-1] == 0


def numpy_multifrontal_solve(A, e, rhs):
    """Dense multifrontal LU (no pivoting across fronts) over the exported
    structure; returns x in the natural ordering."""
    perm = e["perm"]
    n = len(perm)
    iperm = np.empty(n, np.int64)
    iperm[perm] = np.arange(n)
    Ap = A[perm][:, perm].tocsr()
    off = np.concatenate([[0], np.cumsum(e["b"])])
    nfr = len(e["p"])
    upd = {}
    facs = []
    for f in range(nfr):
        p, b, first = e["p"][f], e["b"][f], e["first"][f]
        idx = np.concatenate([np.arange(first, first + p), e["border"][off[f]:off[f + 1]]])
        F = np.zeros((p + b, p + b), complex)
        # original entries whose smaller (new) index is a pivot of this front
        sub = Ap[first:first + p][:, idx].toarray()
        F[:p, :] = sub
        subT = Ap[idx[p:]][:, first:first + p].toarray()
        F[p:, :p] = subT
        for c in [c for c in range(f) if e["parent"][c] == f]:
            U, crel = upd.pop(c)
            F[np.ix_(crel, crel)] += U
        L11U11 = F[:p, :p].copy()
        import scipy.linalg as sla
        lu, piv = sla.lu_factor(L11U11)
        U12 = sla.lu_solve((lu, piv), F[:p, p:]) if b else np.zeros((p, 0))
        L21 = F[p:, :p]
        if b:
            upd[f] = (F[p:, p:] - L21 @ U12, e["rel"][off[f]:off[f + 1]])
        facs.append((lu, piv, U12, L21, idx))
    y = rhs[perm].astype(complex)
    # forward: block elimination with the Schur complements
    import scipy.linalg as sla
    for f in range(nfr):
        lu, piv, U12, L21, idx = facs[f]
        p = e["p"][f]
        z = sla.lu_solve((lu, piv), y[idx[:p]])
        if len(idx) > p:
            y[idx[p:]] -= L21 @ z
        y[idx[:p]] = z          # store A11^-1 (b - ...) for the backward sweep
    for f in reversed(range(nfr)):
        lu, piv, U12, L21, idx = facs[f]
        p = e["p"][f]
        if len(idx) > p:
            y[idx[:p]] -= U12 @ y[idx[p:]]
    x = np.empty(n, complex)
    x[perm] = y
    return x


@pytest.mark.parametrize("dims,leaf", [((6, 5, 7), 8), ((8, 7, 6), 27)])
def test_numpy_multifrontal_matches_superlu(oracle, dims, leaf):
    nx, ny, nz = dims
    g = Grid(nx, ny, nz, 20.0, pmld=2 * 20.0, fst=1)
    vp, vs, rho = model.layered_random(nx, ny, nz, g.dx, seed=5)
    ir, jc = oracle.pattern(nx, ny, nz)
    a, _ = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir)
    A = sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))
    rng = np.random.default_rng(0)
    b = rng.standard_normal(g.n) + 1j * rng.standard_normal(g.n)
    x_ref = spla.spsolve(A.tocsc(), b)
    e = export(nx, ny, nz, leaf)
    x = numpy_multifrontal_solve(A, e, b)
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9
