"""CPU tests of the C ABI: the library loads, exports every symbol the
public header declares, and fails loudly (no CPU fallback) without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import wtomo3d_gb300 as wt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "wtomo3d_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+([A-Za-z_][A-Za-z0-9_]*)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "return")))


def test_header_symbols_exported():
    names = header_functions()
    assert "strumpack_serial_finter" in names and "wt3d_solve" in names
    L = wt.lib()
    for n in names:
        assert hasattr(L, n), "missing export: " + n


def test_pattern_nnz_closed_form():
    for dims in [(2, 2, 2), (40, 40, 40), (96, 96, 64), (128, 128, 96)]:
        nx, ny, nz = dims
        assert wt.lib().wt3d_pattern_nnz(nx, ny, nz) == 9 * (3 * nx - 2) * (3 * ny - 2) * (3 * nz - 2)
    assert wt.lib().wt3d_pattern_nnz(40, 40, 40) == 14787288
    assert wt.lib().wt3d_pattern_nnz(96, 96, 64) == 139871160
    assert wt.lib().wt3d_pattern_nnz(128, 128, 96) == 375608376


def _has_gpu():
    import torch
    return torch.cuda.is_available()


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU error path")
def test_no_gpu_fails_loudly():
    g = wt.Grid(4, 4, 4, 10.0)
    with pytest.raises(wt.WT3DError) as e:
        wt.Solver(g)
    assert e.value.code == wt.WT3D_ERR_NOGPU
    with pytest.raises(wt.WT3DError):
        wt.pattern(4, 4, 4)


def test_job_protocol_order_errors():
    """Out-of-order jobs report ierr = 1 like strumpack_finter.c:71-76,95-99."""
    n, nnz = 24, 24 * 24
    ir = np.zeros(n + 1, np.int32)
    jc = np.zeros(nnz, np.int32)
    a = np.zeros(nnz, np.complex64)
    b = np.zeros(n, np.complex64)
    x = np.zeros(n, np.complex64)
    assert wt.strumpack_serial_finter(2, n, nnz, ir, jc, a, b, x) == 1
    assert wt.strumpack_serial_finter(3, n, nnz, ir, jc, a, b, x) == 1
    assert wt.strumpack_serial_finter(-1, n, nnz, ir, jc, a, b, x) == 0


def test_job1_rejects_malformed_pattern():
    """Job 1 takes the grid graph or any well-formed pattern; a row that lists
    a column twice is refused on the host, before any device work."""
    n = 24
    rows = [[j for j in (i, i + 1) if j < n] + [i] for i in range(n)]
    ir = np.cumsum([1] + [len(r) for r in rows]).astype(np.int32)
    jc = (np.concatenate(rows) + 1).astype(np.int32)
    a = np.ones(len(jc), np.complex64)
    b = np.zeros(n, np.complex64)
    assert wt.strumpack_serial_finter(1, n, len(jc), ir, jc, a, b, b.copy()) == 1
    assert "duplicate" in wt.lib().wt3d_last_error().decode()


def test_too_large_grid_is_rejected_before_any_device_work():
    """nnz must fit int32 CSR indices (the reference's INTEGER pattern)."""
    import ctypes
    import pytest
    import wtomo3d_gb300 as wt
    g = wt.Grid(400, 400, 400, 10.0)
    with pytest.raises(wt.WT3DError) as e:
        wt.solver_bytes(g)
    assert e.value.code == wt.WT3D_ERR_ARG
    with pytest.raises(wt.WT3DError) as e:
        wt.Solver(wt.Grid(1, 5, 5, 10.0))
    assert e.value.code == wt.WT3D_ERR_ARG


def test_finter_refinement_setter_rejects_bad_arguments():
    """The drop-in's refinement setter checks its arguments on the host."""
    L = wt.lib()
    L.wt3d_finter_set_refinement.argtypes = [ctypes.c_double, ctypes.c_int]
    assert L.wt3d_finter_set_refinement(0.0, 5) == wt.WT3D_ERR_ARG
    assert L.wt3d_finter_set_refinement(1e-8, -1) == wt.WT3D_ERR_ARG
    assert L.wt3d_finter_set_refinement(1e-10, 20) == 0


def test_general_constructor_checks_pattern_before_device_work():
    """wt3d_solver_create_csr refuses malformed patterns on the host, with or
    without a GPU: no entries, duplicates, columns out of range, bad base."""
    cases = [
        ([0, 0, 0], [], 0),            # no entries
        ([0, 2, 3], [0, 0, 1], 0),     # duplicate in row 0
        ([0, 1, 2], [0, 7], 0),        # column out of range
        ([1, 2, 3], [1, 2], 2),        # index base 2
    ]
    for ir, jc, base in cases:
        with pytest.raises(wt.WT3DError) as e:
            wt.Solver.from_csr(np.array(ir), np.array(jc, np.int32), base=base)
        assert e.value.code in (wt.WT3D_ERR_PATTERN, wt.WT3D_ERR_ARG), (ir, jc, base, e.value.code)
