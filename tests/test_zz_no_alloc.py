"""The allocation-free GEMM entry point (wt3d_gemm_noalloc) against the
allocating tensor-core entry point, on two calls in a row.

wt3d_gemm_noalloc serves callers that cannot call cudaMalloc: their device
memory belongs to another allocator or a fixed budget, or they run on a path
that must not allocate.  It keeps its scratch in a fixed array inside the
library; this test only allocates the caller's own inputs and outputs.
"""
import ctypes

import numpy as np
import pytest

import wtomo3d_gb300 as wt

pytestmark = pytest.mark.gpu


def _lib():
    L = wt.lib()
    L.wt3d_gemm_noalloc.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                         ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.wt3d_gemm_noalloc_max_floats.restype = ctypes.c_longlong
    L.wt3d_debug_gemm.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    return L


def _allocating_reference(L, A, B, C):
    """The existing tensor-core entry point (allocates its own workspace)."""
    out = np.ascontiguousarray(C).copy()
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = L.wt3d_debug_gemm(1, A.shape[0], B.shape[1], A.shape[1], p(A), A.shape[1], p(B), B.shape[1], p(out),
                           out.shape[1])
    assert rc == 0, L.wt3d_last_error()
    return out


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    L = _lib()
    shapes = [(300, 260, 129), (512, 384, 700)]
    for call, (M, N, K) in enumerate(shapes):
        r = np.random.default_rng(100 + call)
        A = (r.standard_normal((M, K)) + 1j * r.standard_normal((M, K))).astype(np.complex64)
        B = (r.standard_normal((K, N)) + 1j * r.standard_normal((K, N))).astype(np.complex64)
        C = (r.standard_normal((M, N)) + 1j * r.standard_normal((M, N))).astype(np.complex64)
        ref = _allocating_reference(L, A, B, C)
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        dC = torch.from_numpy(C).cuda()
        torch.cuda.synchronize()
        rc = L.wt3d_gemm_noalloc(M, N, K, ctypes.c_void_p(dA.data_ptr()), K, ctypes.c_void_p(dB.data_ptr()), N,
                                 ctypes.c_void_p(dC.data_ptr()), N, None)
        assert rc == 0, L.wt3d_last_error()
        out = dC.cpu().numpy()
        scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C)
        # same tolerance as the tensor-core GEMM tests
        assert (np.abs(out - ref) / scale).max() < 1e-6 + 3e-7 * np.sqrt(K)
        exact = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
        assert (np.abs(out - exact) / scale).max() < 1e-6 + 3e-7 * np.sqrt(K)


def test_noalloc_strided_operands_on_a_caller_stream():
    """Leading dimensions wider than the operands (views into wider arrays)
    and a caller stream: the product matches, and the padding columns of C
    are left as they were."""
    import torch
    L = _lib()
    M, N, K = 200, 140, 96
    lda, ldb, ldc = K + 24, N + 12, N + 20
    r = np.random.default_rng(7)
    cplx = lambda *sh: (r.standard_normal(sh) + 1j * r.standard_normal(sh)).astype(np.complex64)
    Aw, Bw, Cw = cplx(M, lda), cplx(K, ldb), cplx(M, ldc)
    A, B, C = Aw[:, :K], Bw[:, :N], Cw[:, :N]
    ref = _allocating_reference(L, np.ascontiguousarray(A), np.ascontiguousarray(B), C)
    dA, dB, dC = (torch.from_numpy(x).cuda() for x in (Aw, Bw, Cw))
    st = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(2):
        dC.copy_(torch.from_numpy(Cw))
        torch.cuda.synchronize()
        rc = L.wt3d_gemm_noalloc(M, N, K, ctypes.c_void_p(dA.data_ptr()), lda, ctypes.c_void_p(dB.data_ptr()), ldb,
                                 ctypes.c_void_p(dC.data_ptr()), ldc, ctypes.c_void_p(st.cuda_stream))
        assert rc == 0, L.wt3d_last_error()
        out = dC.cpu().numpy()
        scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C)
        assert (np.abs(out[:, :N] - ref) / scale).max() < 1e-6 + 3e-7 * np.sqrt(K)
        assert np.array_equal(out[:, N:], Cw[:, N:]), "padding columns of C were written"


def test_noalloc_rejects_oversized_problem():
    L = _lib()
    lim = L.wt3d_gemm_noalloc_max_floats()
    assert lim > 0
    N = int(lim // 8) + 1024     # 4 N Kr alone exceeds the limit for K = 1
    rc = L.wt3d_gemm_noalloc(1, N, 1, ctypes.c_void_p(16), 1, ctypes.c_void_p(16), N, ctypes.c_void_p(16), N, None)
    assert rc == wt.WT3D_ERR_ARG
    assert b"limit" in L.wt3d_last_error()
