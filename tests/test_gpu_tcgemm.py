"""The tcgen05 complex64 GEMM (3xTF32 split, real expansion of B) against a
complex128 numpy product, next to the SIMT kernel, on ragged shapes."""
import ctypes

import numpy as np
import pytest

import wtomo3d_gb300 as wt

pytestmark = pytest.mark.gpu


def gemm(path, A, B, C):
    L = wt.lib()
    L.wt3d_debug_gemm.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    M, K = A.shape
    N = B.shape[1]
    A = np.ascontiguousarray(A, np.complex64)
    B = np.ascontiguousarray(B, np.complex64)
    C = np.ascontiguousarray(C, np.complex64).copy()
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = L.wt3d_debug_gemm(path, M, N, K, p(A), A.shape[1], p(B), B.shape[1], p(C), C.shape[1])
    assert rc == 0, L.wt3d_last_error()
    return C


@pytest.mark.parametrize("shape", [(128, 128, 16), (130, 70, 37), (64, 200, 64), (300, 260, 129), (512, 640, 1000)])
@pytest.mark.parametrize("path", [1, 0])
def test_gemm_accuracy(shape, path):
    M, N, K = shape
    r = np.random.default_rng(M * 7 + N * 3 + K)
    A = (r.standard_normal((M, K)) + 1j * r.standard_normal((M, K))).astype(np.complex64)
    B = (r.standard_normal((K, N)) + 1j * r.standard_normal((K, N))).astype(np.complex64)
    C = (r.standard_normal((M, N)) + 1j * r.standard_normal((M, N))).astype(np.complex64)
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    out = gemm(path, A, B, C)
    # FP32-class product: error relative to sum |a||b| per entry
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C)
    err = (np.abs(out - ref) / scale).max()
    assert err < 1e-6 + 3e-7 * np.sqrt(K), err   # FP32 accumulation grows with K


def test_gemm_strided_views():
    """Sub-blocks of larger arrays (the front layout): lda/ldb/ldc > widths."""
    r = np.random.default_rng(1)
    F = (r.standard_normal((400, 900)) + 1j * r.standard_normal((400, 900))).astype(np.complex64)
    L = wt.lib()
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    A = F[100:300, 0:64]
    B = F[0:64, 300:800]
    C = F[100:300, 300:800]
    ref = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    out = gemm(1, A, B, C)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64) + np.abs(C)
    assert (np.abs(out - ref) / scale).max() < 2e-6


def gemm_ld(path, A, lda, B, C):
    """C -= A B (path 5: C -= A^H B) with A passed as the first A.shape[1]
    columns of rows lda apart."""
    L = wt.lib()
    L.wt3d_debug_gemm.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                       ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    rows, cols = A.shape
    M, K = (cols, rows) if path == 5 else (rows, cols)
    N = B.shape[1]
    Abuf = np.zeros((rows, lda), np.complex64)
    Abuf[:, :cols] = A
    Abuf[:, cols:] = np.nan     # never read
    B = np.ascontiguousarray(B, np.complex64)
    C = np.ascontiguousarray(C, np.complex64).copy()
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = L.wt3d_debug_gemm(path, M, N, K, p(Abuf), lda, p(B), B.shape[1], p(C), C.shape[1])
    assert rc == 0, L.wt3d_last_error()
    return C


@pytest.mark.parametrize("shape", [(128, 32, 256), (130, 32, 300), (1000, 17, 777), (300, 1, 4099),
                                   (2048, 32, 5000)])
@pytest.mark.parametrize("path", [3, 4])
@pytest.mark.parametrize("stride", ["odd", "even"])
def test_tall_skinny_tensor_core_gemm(shape, path, stride):
    """The substitution passes' tensor-core kernel (A split on the fly, ragged
    M and K, fewer than 32 columns, K split across CTAs); path 4 gathers B rows
    K-1-k and scatters C rows M-1-r.  An odd leading dimension puts rows off
    16-byte boundaries (A copied by the loader warps); an even one lets TMA
    stream A."""
    M, N, K = shape
    r = np.random.default_rng(M + 5 * N + 11 * K + path)
    A = (r.standard_normal((M, K)) + 1j * r.standard_normal((M, K))).astype(np.complex64)
    B = (r.standard_normal((K, N)) + 1j * r.standard_normal((K, N))).astype(np.complex64)
    C = (r.standard_normal((M, N)) + 1j * r.standard_normal((M, N))).astype(np.complex64)
    Bq = B[::-1] if path == 4 else B
    prod = A.astype(np.complex128) @ Bq.astype(np.complex128)
    scale = np.abs(A).astype(np.float64) @ np.abs(Bq).astype(np.float64)
    if path == 4:
        prod, scale = prod[::-1], scale[::-1]
    ref = C.astype(np.complex128) - prod
    if stride == "odd":
        lda = K + 3 if K % 2 == 0 else K
    else:
        lda = K if K % 2 == 0 else K + 1
    out = gemm_ld(path, A, lda, B, C)
    err = (np.abs(out - ref) / (scale + np.abs(C))).max()
    assert err < 1e-6 + 3e-7 * np.sqrt(K), err


@pytest.mark.parametrize("shape", [(128, 32, 256), (130, 32, 300), (1000, 17, 777), (300, 1, 4099),
                                   (2048, 32, 5000)])
def test_tall_skinny_tensor_core_gemm_conjugate(shape):
    """Path 5: C -= A^H B with A stored as the K x M block (the adjoint
    substitution passes read factor blocks this way), odd row stride."""
    M, N, K = shape
    r = np.random.default_rng(3 * M + N + 7 * K)
    At = (r.standard_normal((K, M)) + 1j * r.standard_normal((K, M))).astype(np.complex64)
    B = (r.standard_normal((K, N)) + 1j * r.standard_normal((K, N))).astype(np.complex64)
    C = (r.standard_normal((M, N)) + 1j * r.standard_normal((M, N))).astype(np.complex64)
    AH = At.astype(np.complex128).conj().T
    ref = C.astype(np.complex128) - AH @ B.astype(np.complex128)
    scale = np.abs(AH) @ np.abs(B).astype(np.float64)
    lda = M + 3 if M % 2 == 0 else M
    out = gemm_ld(5, At, lda, B, C)
    err = (np.abs(out - ref) / (scale + np.abs(C))).max()
    assert err < 1e-6 + 3e-7 * np.sqrt(K), err
