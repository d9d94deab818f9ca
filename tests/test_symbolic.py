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
        for c in [c for c in range(f) if e["parent"][c] == f and c in upd]:   # children with a border
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


# ---------------------------------------------------------------------------
# general structurally symmetric patterns (wt3d_analyse_csr_*)
# ---------------------------------------------------------------------------
def check_structure(e, n):
    assert np.array_equal(np.sort(e["perm"]), np.arange(n))
    assert e["first"][0] == 0
    assert np.all(e["first"][1:] == e["first"][:-1] + e["p"][:-1])
    assert e["first"][-1] + e["p"][-1] == n
    assert np.all(e["p"] > 0)
    roots = np.flatnonzero(e["parent"] == -1)
    assert list(roots) == [len(e["p"]) - 1] and e["b"][-1] == 0
    for f, par in enumerate(e["parent"][:-1]):
        assert par > f and e["level"][par] == e["level"][f] - 1
    off = np.concatenate([[0], np.cumsum(e["b"])])
    for f in range(len(e["p"])):
        bd = e["border"][off[f]:off[f + 1]]
        assert np.all(np.diff(bd) > 0)
        assert bd.size == 0 or bd[0] >= e["first"][f] + e["p"][f]


def general_case(A, leaf=0, seed=0):
    """Export the general analysis of A's pattern, check the structure and
    solve with the numpy multifrontal over it against SuperLU."""
    A = sp.csr_matrix(A)
    e = wt.analyse_csr_export(A.indptr, A.indices, 0, leaf)
    check_structure(e, A.shape[0])
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(A.shape[0]) + 1j * rng.standard_normal(A.shape[0])
    x = numpy_multifrontal_solve(A, e, b)
    xr = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9
    return e


def random_values(P, seed=0, dominant=True):
    """Complex values on pattern P (csr), diagonally dominant."""
    rng = np.random.default_rng(seed)
    A = sp.csr_matrix(P, dtype=complex, copy=True)
    A.data = rng.standard_normal(A.nnz) + 1j * rng.standard_normal(A.nnz)
    if dominant:
        A = A + sp.diags(np.abs(A).sum(axis=1).A1 + 1.0)
    return sp.csr_matrix(A)


def elastic_operator(oracle, nx, ny, nz):
    g = Grid(nx, ny, nz, 20.0, pmld=2 * 20.0, fst=1)
    vp, vs, rho = model.layered_random(nx, ny, nz, g.dx, seed=5)
    ir, jc = oracle.pattern(nx, ny, nz)
    a, _ = oracle.assemble(g, vp, vs, rho, 2 * np.pi * 1.0, ir)
    return sp.csr_matrix((a, jc - 1, ir - 1), shape=(g.n, g.n))


def test_general_grid_operator_fill_close_to_plane_separators(oracle):
    """The elastic operator's own pattern through the general analysis: the
    3 dofs of a node form one supervariable, the solve is exact, and the
    factorisation costs at most 1.25x the flops of the plane-separator
    ordering (1.05x measured)."""
    A = elastic_operator(oracle, 8, 7, 6)
    e = general_case(A, leaf=81)
    # supervariables of 3 dofs: every front holds whole nodes
    assert np.all(e["p"] % 3 == 0) and np.all(e["b"] % 3 == 0)
    eg = export(8, 7, 6, 27)
    assert e["flops"] <= 1.25 * eg["flops"], (e["flops"], eg["flops"])


def test_general_grid_fill_at_20_cubed(oracle):
    ir, jc = oracle.pattern(20, 20, 20)
    info, fl = wt.analyse_csr(ir, jc, base=1)
    eg = export(20, 20, 20, 64)
    assert fl <= 1.25 * eg["flops"], (fl, eg["flops"])     # 1.05x measured


def test_general_node_permuted_operator(oracle):
    """A symmetric node permutation hides the grid (job 1 no longer
    recognises it) but keeps the 3-dof supervariables."""
    A = elastic_operator(oracle, 6, 5, 7)
    nn = A.shape[0] // 3
    q = np.random.default_rng(3).permutation(nn)
    perm = (3 * q[:, None] + np.arange(3)).reshape(-1)
    general_case(A[perm][:, perm], leaf=30)


def test_general_dof_permuted_operator(oracle):
    """A random dof permutation breaks the supervariables as well."""
    A = elastic_operator(oracle, 5, 5, 5)
    perm = np.random.default_rng(4).permutation(A.shape[0])
    general_case(A[perm][:, perm], leaf=40)


def test_general_2d_five_point():
    n1 = 30
    T = sp.diags([np.ones(n1 - 1), np.ones(n1), np.ones(n1 - 1)], [-1, 0, 1])
    P = sp.kron(sp.eye(n1), T) + sp.kron(T, sp.eye(n1))
    e = general_case(random_values(P, 1), leaf=16)
    assert len(e["p"]) > 8


def test_general_disconnected_and_isolated():
    """Two separate meshes plus isolated unknowns (a diagonal block)."""
    n1 = 12
    T = sp.diags([np.ones(n1 - 1), np.ones(n1), np.ones(n1 - 1)], [-1, 0, 1])
    P2 = sp.kron(sp.eye(n1), T) + sp.kron(T, sp.eye(n1))
    P = sp.block_diag([P2, sp.eye(7), sp.kron(T, T)])
    general_case(random_values(P, 2), leaf=10)


def test_general_unsorted_rows_random_pattern():
    """A random symmetric pattern whose rows list their columns in random order."""
    rng = np.random.default_rng(7)
    n = 300
    R = sp.random(n, n, density=0.01, random_state=8, format="csr")
    P = ((R + R.T) != 0).astype(float) + sp.eye(n)
    A = random_values(P, 3)
    A = sp.csr_matrix(A)
    # shuffle the entries inside each row
    ind, dat = A.indices.copy(), A.data.copy()
    for r in range(n):
        s0, s1 = A.indptr[r], A.indptr[r + 1]
        o = rng.permutation(s1 - s0)
        ind[s0:s1], dat[s0:s1] = ind[s0:s1][o], dat[s0:s1][o]
    B = sp.csr_matrix((dat, ind, A.indptr.copy()), shape=A.shape)
    assert not B.has_sorted_indices
    e = wt.analyse_csr_export(B.indptr, B.indices, 0, 24)
    check_structure(e, n)
    b = rng.standard_normal(n) + 0j
    x = numpy_multifrontal_solve(B, e, b)
    xr = spla.spsolve(A.tocsc(), b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9


def test_general_dense_and_single():
    general_case(random_values(np.ones((40, 40)), 4), leaf=8)
    e = wt.analyse_csr_export(np.array([0, 1]), np.array([0]))
    assert list(e["p"]) == [1] and list(e["b"]) == [0]
    # one row without its diagonal entry is still a valid pattern
    e = wt.analyse_csr_export(np.array([0, 0]), np.array([], np.int32))
    assert list(e["p"]) == [1]


def test_general_long_path_is_balanced():
    """A tridiagonal pattern of 200k unknowns: the level structure of a path
    splits it in the middle each time, so the tree is ~log2(n / leaf) deep
    and every front is small."""
    n = 200_000
    T = sp.diags([np.ones(n - 1), np.ones(n), np.ones(n - 1)], [-1, 0, 1], format="csr")
    info, fl = wt.analyse_csr(T.indptr, T.indices, 0, 64)
    nfronts, levels, maxp, maxb = info[0], info[2], info[3], info[4]
    assert levels <= 20 and maxp <= 64 and maxb <= 2 * levels


def convection_diffusion(n1, seed=0):
    """Upwinded 2-D convection-diffusion: each unknown couples to its west
    and south neighbours and to its east neighbour only on even rows, so the
    pattern is not structurally symmetric."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for j in range(n1):
        for i in range(n1):
            r = i + n1 * j
            rows.append(r); cols.append(r); vals.append(4.0 + rng.random() + 1j * rng.random())
            if i > 0:
                rows.append(r); cols.append(r - 1); vals.append(-1.0 - 0.5 * rng.random())
            if j > 0:
                rows.append(r); cols.append(r - n1); vals.append(-1.0 - 0.5 * rng.random())
            if i < n1 - 1 and j % 2 == 0:
                rows.append(r); cols.append(r + 1); vals.append(-0.3 + 0.1j)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n1 * n1, n1 * n1))


def test_general_unsymmetric_pattern():
    """An unsymmetric pattern is ordered through A + A^T, as STRUMPACK does."""
    A = convection_diffusion(24)
    assert (A != 0).sum() != ((A + A.T) != 0).sum()
    general_case(A, leaf=20)


def test_general_bad_patterns_are_rejected():
    # duplicate column in a row
    with pytest.raises(wt.WT3DError) as e:
        wt.analyse_csr([0, 2, 3], [0, 0, 1])
    assert e.value.code == wt.WT3D_ERR_PATTERN
    # column out of range
    with pytest.raises(wt.WT3DError) as e:
        wt.analyse_csr([0, 1, 2], [0, 5])
    assert e.value.code == wt.WT3D_ERR_PATTERN
    # row pointers that do not start at the base
    with pytest.raises(wt.WT3DError) as e:
        wt.analyse_csr([1, 2, 3], [0, 1], base=0)
    assert e.value.code == wt.WT3D_ERR_PATTERN


def test_general_ordering_is_deterministic(oracle):
    """Subtrees of the general dissection run on several threads; the
    bisections draw their random streams from the position in the tree, so
    two analyses of the same pattern agree exactly (40^3: 64,000
    supervariables, large enough for the threaded levels), and the ordering
    stays within 1.15x of the plane separators' flops."""
    ir, jc = oracle.pattern(40, 40, 40)
    e1 = wt.analyse_csr_export(ir, jc, base=1)
    e2 = wt.analyse_csr_export(ir, jc, base=1)
    for k in ("perm", "p", "b", "parent", "border", "rel"):
        np.testing.assert_array_equal(e1[k], e2[k])
    assert e1["flops"] <= 1.15 * export(40, 40, 40, 64)["flops"]


def test_general_pathological_graphs():
    """A diagonal matrix (every unknown its own component), a star (one
    row coupled to all others) and a long cycle: balanced trees, the solve
    over the exported structure still exact."""
    n = 20000
    e = wt.analyse_csr_export(np.arange(n + 1), np.arange(n), 0, 64)
    check_structure(e, n)
    assert e["info"][2] <= 20 and max(e["b"]) == 0      # no coupling, no borders
    m = 400
    rows = [list(range(m))] + [[0, i] for i in range(1, m)]
    P = sp.csr_matrix((np.ones(sum(map(len, rows))), np.concatenate(rows),
                       np.cumsum([0] + [len(r) for r in rows])), shape=(m, m))
    general_case(random_values(P, 5), leaf=16)
    c = 3000
    C = sp.diags([np.ones(c - 1), np.ones(c), np.ones(c - 1)], [-1, 0, 1], format="lil")
    C[0, c - 1] = C[c - 1, 0] = 1
    general_case(random_values(sp.csr_matrix(C), 6), leaf=32)
