"""wtomo3d-gb300: GB300-native frequency-domain elastic forward modelling.

Python mirror of the C ABI in include/wtomo3d_gpu.h.  The compute runs in
libwtomo3d_gpu.so (hand-written CUDA for sm_103a); this module only marshals
host arrays through ctypes.  There is no CPU fallback: if the library or a
GPU is missing, every call raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwtomo3d_gpu.so")

WT3D_OK = 0
WT3D_ERR_ARG = 1
WT3D_ERR_CUDA = 2
WT3D_ERR_NOMEM = 3
WT3D_ERR_STATE = 4
WT3D_ERR_PATTERN = 5
WT3D_ERR_NOCONV = 6
WT3D_ERR_NOGPU = 7

PREC_MIXED = 0
PREC_FP64 = 1


class WT3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("wtomo3d error %d: %s" % (code, msg))
        self.code = code


class Grid(ctypes.Structure):
    """wt3d_grid: grid and boundary description (dx = dy = dz)."""
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("pmld", ctypes.c_double), ("pmlr", ctypes.c_double),
                ("fst", ctypes.c_int), ("usemin", ctypes.c_int)]

    def __init__(self, nx, ny, nz, dx, pmld=0.0, pmlr=0.0, fst=True, usemin=True):
        super().__init__(nx, ny, nz, float(dx), float(pmld), float(pmlr), int(bool(fst)), int(bool(usemin)))

    @property
    def nnodes(self):
        return self.nx * self.ny * self.nz

    @property
    def n(self):
        return 3 * self.nnodes

    @property
    def nnz(self):
        return 9 * (3 * self.nx - 2) * (3 * self.ny - 2) * (3 * self.nz - 2)

    def pml(self):
        """(pmld, pmlf, ipml) as readini.f90:81-84 computes them (in double)."""
        pmld = self.pmld if self.pmld > 0 else 10.0 * self.dx
        pmlr = self.pmlr if self.pmlr > 0 else 1e-3
        ipml = int(pmld / self.dx) + 1
        pmlf = 3.0 * np.log(1.0 / pmlr) / (2.0 * pmld ** 3)
        return pmld, pmlf, ipml


class Layered1D(ctypes.Structure):
    """wt3d_layered1d: nl layers (the last is the half-space), ztop[0] = 0."""
    _fields_ = [("nl", ctypes.c_int), ("vp", ctypes.c_void_p), ("vs", ctypes.c_void_p),
                ("rho", ctypes.c_void_p), ("ztop", ctypes.c_void_p)]

    def __init__(self, vp, vs, rho, ztop):
        self._keep = [np.ascontiguousarray(a, np.float64) for a in (vp, vs, rho, ztop)]
        super().__init__(len(self._keep[0]), *[ctypes.c_void_p(a.ctypes.data) for a in self._keep])


def haskgrn(layers, omega, ain, nz, dz, s_wave=False, zorig=0.0):
    """Thomson-Haskell response (U, W) at nz node depths (host, FP64)."""
    U = np.zeros(nz, np.complex128)
    W = np.zeros(nz, np.complex128)
    _check(lib().wt3d_haskgrn(ctypes.byref(layers), float(omega), float(ain), int(bool(s_wave)), int(nz),
                              float(dz), float(zorig), _ptr(U), _ptr(W)))
    return U, W


class Stats(ctypes.Structure):
    _fields_ = [("n", ctypes.c_longlong), ("nnz", ctypes.c_longlong), ("nfronts", ctypes.c_longlong),
                ("factor_entries", ctypes.c_longlong), ("factor_flops", ctypes.c_double),
                ("factor_bytes", ctypes.c_double), ("device_bytes", ctypes.c_double),
                ("t_analyse_ms", ctypes.c_double), ("t_assemble_ms", ctypes.c_double),
                ("t_factor_ms", ctypes.c_double), ("t_solve_ms", ctypes.c_double),
                ("perturbed_pivots", ctypes.c_int), ("levels", ctypes.c_int),
                ("kernels_factor", ctypes.c_int), ("kernels_solve", ctypes.c_int),
                ("t_gradient_ms", ctypes.c_double), ("workspace_bytes", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """Load libwtomo3d_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libwtomo3d_gpu.so is not built: run `python -c \"import __graft_entry__ as g; "
                               "g.build()\"` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        vp = ctypes.c_void_p
        L.wt3d_last_error.restype = ctypes.c_char_p
        L.wt3d_pattern_nnz.restype = ctypes.c_longlong
        L.wt3d_pattern_nnz.argtypes = [ctypes.c_int] * 3
        L.wt3d_pattern.argtypes = [ctypes.c_int] * 4 + [vp, vp]
        L.wt3d_assemble.argtypes = [ctypes.POINTER(Grid), vp, vp, vp, ctypes.c_double, ctypes.c_double, vp]
        L.wt3d_solver_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(Grid), ctypes.c_int]
        L.wt3d_solver_destroy.argtypes = [vp]
        L.wt3d_set_model.argtypes = [vp, vp, vp, vp]
        L.wt3d_factor.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.wt3d_set_values_c64.argtypes = [vp, vp]
        L.wt3d_set_values_c128.argtypes = [vp, vp]
        L.wt3d_solver_create_csr.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_longlong, vp, vp,
                                             ctypes.c_int, ctypes.c_int]
        L.wt3d_analyse_csr_info.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, ctypes.c_int, ctypes.c_int,
                                            vp, vp]
        L.wt3d_analyse_csr_export.argtypes = [ctypes.c_int, ctypes.c_longlong, vp, vp, ctypes.c_int, ctypes.c_int]\
            + [vp] * 8
        L.wt3d_factor_values.argtypes = [vp]
        for f in (L.wt3d_solve, L.wt3d_solve_adjoint):
            f.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.c_int, vp, vp]
        L.wt3d_solve_device.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_double, ctypes.c_int, vp, vp,
                                        ctypes.c_int]
        L.wt3d_apply.argtypes = [vp, ctypes.c_int, vp, vp]
        L.wt3d_apply_device.argtypes = [vp, ctypes.c_int, vp, vp]
        L.wt3d_solver_bytes.argtypes = [ctypes.POINTER(Grid), ctypes.c_int, vp]
        L.wt3d_set_sm_reserve.argtypes = [ctypes.c_int]
        L.wt3d_batch_buffers.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        L.wt3d_memcpy.argtypes = [vp, vp, vp, ctypes.c_longlong]
        L.wt3d_mem_info.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.wt3d_source_weights.argtypes = [ctypes.POINTER(Grid)] + [ctypes.c_double] * 3 + [ctypes.c_int,
                                          ctypes.c_double, ctypes.c_int, vp, vp, ctypes.POINTER(ctypes.c_int)]
        L.wt3d_rhs_sources.argtypes = [vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, ctypes.c_double, vp]
        L.wt3d_sample_receivers.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp]
        L.wt3d_sample_pressure.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int, vp, ctypes.c_int, ctypes.c_double, vp]
        L.wt3d_update_operator.argtypes = [vp]
        L.wt3d_gradient_contract.argtypes = [vp, ctypes.c_int, vp, vp, vp]
        L.wt3d_misfit_gradient.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp, ctypes.c_double,
                                           ctypes.c_int, vp, vp, vp]
        L.wt3d_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
        L.wt3d_get_stream.restype = vp
        L.wt3d_get_stream.argtypes = [vp]
        L.wt3d_profile_factor.argtypes = [vp, vp]
        L.wt3d_profile_solve.argtypes = [vp, ctypes.c_int, vp]
        L.wt3d_set_device.argtypes = [ctypes.c_int]
        L.wt3d_haskgrn.argtypes = [ctypes.POINTER(Layered1D), ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, vp]
        L.wt3d_set_background.argtypes = [vp, vp, vp, vp]
        L.wt3d_set_attenuation.argtypes = [vp, vp, vp, ctypes.c_double]
        L.wt3d_rhs_planewave.argtypes = [vp, ctypes.POINTER(Layered1D), ctypes.c_int, vp, vp, vp, vp, vp]
        ip = ctypes.POINTER(ctypes.c_int)
        L.strumpack_serial_finter.argtypes = [ip, ip, ip, vp, vp, vp, vp, vp, ip]
        L.strumpack_serial_finter.restype = None
        L.wt3d_finter_set_refinement.argtypes = [ctypes.c_double, ctypes.c_int]
        L.wt3d_set_workspaces_per_grid.argtypes = [ctypes.c_int]
        L.wt3d_finter_last_relres.restype = ctypes.c_double
        L.wt3d_finter_last_relres.argtypes = []
        _lib = L
    return _lib


def _check(rc, allow=()):
    if rc != WT3D_OK and rc not in allow:
        raise WT3DError(rc, lib().wt3d_last_error().decode())
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _f32(a, n):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, order="F"))
    if a.size != n:
        raise ValueError("model array has %d entries, expected %d" % (a.size, n))
    return a


def set_sm_reserve(n):
    """SMs the factorisations' persistent tensor-core GEMM leaves to other work."""
    _check(lib().wt3d_set_sm_reserve(int(n)))


def set_device(dev):
    """Select the CUDA device of the calling thread for this library."""
    _check(lib().wt3d_set_device(int(dev)))


def pattern(nx, ny, nz, base=1):
    """CSR pattern of the 27-point 3-dof grid graph (srel3d + SPARSE_ADJ2CRS)."""
    n = 3 * nx * ny * nz
    nnz = lib().wt3d_pattern_nnz(nx, ny, nz)
    irptr = np.empty(n + 1, np.int32)
    jcptr = np.empty(nnz, np.int32)
    _check(lib().wt3d_pattern(nx, ny, nz, base, _ptr(irptr), _ptr(jcptr)))
    return irptr, jcptr


def assemble(grid, vp, vs, rho, omega):
    """Complex128 CSR values of A(omega) in the order of pattern() (ASMBLE)."""
    n = grid.nnodes
    vp, vs, rho = _f32(vp, n), _f32(vs, n), _f32(rho, n)
    a = np.empty(grid.nnz, np.complex128)
    om = complex(omega)
    _check(lib().wt3d_assemble(ctypes.byref(grid), _ptr(vp), _ptr(vs), _ptr(rho), om.real, om.imag, _ptr(a)))
    return a


def source_weights(grid, x, y, z, ireg=0, sprd=0.5):
    """(0-based nodes, weights) with which a point at (x, y, z) metres spreads
    onto the grid (SRCSETUP/SRCREG)."""
    cnt = ctypes.c_int(0)
    _check(lib().wt3d_source_weights(ctypes.byref(grid), x, y, z, int(ireg), float(sprd), 0, None, None,
                                     ctypes.byref(cnt)))
    node = np.zeros(cnt.value, np.int64)
    w = np.zeros(cnt.value)
    _check(lib().wt3d_source_weights(ctypes.byref(grid), x, y, z, int(ireg), float(sprd), cnt.value, _ptr(node),
                                     _ptr(w), ctypes.byref(cnt)))
    return node, w


def mem_info():
    """(free, total) device bytes of the current device."""
    f, t = ctypes.c_double(), ctypes.c_double()
    _check(lib().wt3d_mem_info(ctypes.byref(f), ctypes.byref(t)))
    return f.value, t.value


def solver_bytes(grid, precision=PREC_MIXED):
    """(resident, plane-wave extra, shared workspace) device bytes of a
    handle for `grid`, from the host analysis (cached per grid)."""
    out = np.zeros(3)
    _check(lib().wt3d_solver_bytes(ctypes.byref(grid), int(precision), _ptr(out)))
    return float(out[0]), float(out[1]), float(out[2])


def _csr_arrays(indptr, indices):
    ir = np.ascontiguousarray(indptr, np.int32)
    jc = np.ascontiguousarray(indices, np.int32)
    return ir, jc, len(ir) - 1, len(jc)


def analyse_csr(indptr, indices, base=0, leaf_dofs=0):
    """Host analysis of a general structurally symmetric CSR pattern (no GPU):
    returns (info[8], flops) as wt3d_analyse_csr_info does."""
    ir, jc, n, nnz = _csr_arrays(indptr, indices)
    info = np.zeros(8, np.int64)
    fl = ctypes.c_double()
    _check(lib().wt3d_analyse_csr_info(n, nnz, _ptr(ir), _ptr(jc), int(base), int(leaf_dofs), _ptr(info),
                                       ctypes.byref(fl)))
    return info, fl.value


def analyse_csr_export(indptr, indices, base=0, leaf_dofs=0):
    """Elimination structure of a general pattern: dict of perm, per-front p,
    b, first, parent, level, and the border dofs with their parent positions."""
    ir, jc, n, nnz = _csr_arrays(indptr, indices)
    info, flops = analyse_csr(ir, jc, base, leaf_dofs)
    nf, nb = int(info[0]), int(info[5])
    perm = np.zeros(n, np.int32)
    arrs = [np.zeros(nf, np.int32) for _ in range(5)]
    border = np.zeros(nb, np.int32)
    rel = np.zeros(nb, np.int32)
    _check(lib().wt3d_analyse_csr_export(n, nnz, _ptr(ir), _ptr(jc), int(base), int(leaf_dofs), _ptr(perm),
                                         *[_ptr(a) for a in arrs], _ptr(border), _ptr(rel)))
    fp, fb, ffirst, fpar, flev = arrs
    return dict(perm=perm, p=fp, b=fb, first=ffirst, parent=fpar, level=flev, border=border, rel=rel,
                info=[int(v) for v in info], flops=flops)


class Solver:
    """Handle-based multifrontal solver on one GPU (wt3d_solver_*)."""

    def __init__(self, grid, precision=PREC_MIXED):
        self.grid = grid
        self.n = grid.n
        self.precision = precision
        self._h = ctypes.c_void_p()
        _check(lib().wt3d_solver_create(ctypes.byref(self._h), ctypes.byref(grid), precision))

    @classmethod
    def from_csr(cls, indptr, indices, precision=PREC_MIXED, base=0):
        """Handle for any structurally symmetric CSR pattern
        (wt3d_solver_create_csr); values come from set_values in the same CSR
        order.  The grid-only calls (model, sources, gradient) raise."""
        ir, jc, n, nnz = _csr_arrays(indptr, indices)
        self = cls.__new__(cls)
        self.grid = None
        self.n = n
        self.precision = precision
        self._h = ctypes.c_void_p()
        _check(lib().wt3d_solver_create_csr(ctypes.byref(self._h), n, nnz, _ptr(ir), _ptr(jc), int(base),
                                            precision))
        return self

    def close(self):
        if self._h:
            lib().wt3d_solver_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_model(self, vp, vs, rho):
        n = self.grid.nnodes
        self._model = (_f32(vp, n), _f32(vs, n), _f32(rho, n))
        _check(lib().wt3d_set_model(self._h, *[_ptr(a) for a in self._model]))

    def factor(self, omega):
        om = complex(omega)
        _check(lib().wt3d_factor(self._h, om.real, om.imag))

    def set_values(self, a, dtype=np.complex64):
        """Set operator values in CSR order (complex64 as the job protocol
        takes them, or complex128) and factor."""
        if np.dtype(dtype) == np.complex128:
            a = np.ascontiguousarray(a, dtype=np.complex128)
            _check(lib().wt3d_set_values_c128(self._h, _ptr(a)))
        else:
            a = np.ascontiguousarray(a, dtype=np.complex64)
            _check(lib().wt3d_set_values_c64(self._h, _ptr(a)))
        _check(lib().wt3d_factor_values(self._h))

    def _solve(self, fn, B, tol, maxit, allow_noconv):
        B = np.asarray(B, dtype=np.complex128)
        one = B.ndim == 1
        Bf = np.asfortranarray(B.reshape(self.n, -1))
        nrhs = Bf.shape[1]
        X = np.empty_like(Bf, order="F")
        relres = np.zeros(nrhs)
        iters = ctypes.c_int(0)
        rc = fn(self._h, nrhs, _ptr(Bf), _ptr(X), tol, maxit, _ptr(relres), ctypes.byref(iters))
        _check(rc, allow=(WT3D_ERR_NOCONV,) if allow_noconv else ())
        self.last_relres, self.last_iters = relres, iters.value
        return X[:, 0] if one else X

    def solve(self, B, tol=1e-8, maxit=20, allow_noconv=False):
        """X = A^-1 B with FP64 refinement to ||b - A x|| / ||b|| <= tol."""
        return self._solve(lib().wt3d_solve, B, tol, maxit, allow_noconv)

    def solve_adjoint(self, B, tol=1e-8, maxit=20, allow_noconv=False):
        """X = A^-H B reusing the resident factors."""
        return self._solve(lib().wt3d_solve_adjoint, B, tol, maxit, allow_noconv)

    def apply(self, X):
        X = np.asarray(X, dtype=np.complex128)
        one = X.ndim == 1
        Xf = np.asfortranarray(X.reshape(self.n, -1))
        Y = np.empty_like(Xf, order="F")
        _check(lib().wt3d_apply(self._h, Xf.shape[1], _ptr(Xf), _ptr(Y)))
        return Y[:, 0] if one else Y

    def batch_buffers(self, ncols):
        """Device pointers (F, X) of handle-owned n x ncols complex128 buffers."""
        f, x = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().wt3d_batch_buffers(self._h, int(ncols), ctypes.byref(f), ctypes.byref(x)))
        return f.value, x.value

    def memcpy(self, dst, src, nbytes):
        """Copy between host and device addresses (ints) on the handle's stream."""
        _check(lib().wt3d_memcpy(self._h, ctypes.c_void_p(dst), ctypes.c_void_p(src), int(nbytes)))

    def rhs_sources(self, xyz, comp, d_F, sterm=None, ireg=0, sprd=0.5):
        """Point-force RHS columns on the device (d_F: n x nsrc, column-major)."""
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        comp = np.ascontiguousarray(comp, np.int32).reshape(-1)
        st = None if sterm is None else np.ascontiguousarray(sterm, np.complex128).reshape(-1)
        _check(lib().wt3d_rhs_sources(self._h, len(comp), _ptr(xyz), _ptr(comp), None if st is None else _ptr(st),
                                      int(ireg), float(sprd), ctypes.c_void_p(d_F)))

    def sample_receivers(self, d_U, nrhs, xyz, ireg=0, sprd=0.5, response=None, active=None):
        """Three-component receiver samples, shape (nrhs, nrec, 3); optionally
        times the receiver responses at this frequency (nrec,) and zero for
        inactive source-receiver pairs active[nrhs, nrec] == 0 (makeuh.f:76-104;
        see wtomo3d_gb300.receivers)."""
        from . import receivers
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros((nrhs, len(xyz), 3), np.complex128)
        _check(lib().wt3d_sample_receivers(self._h, int(nrhs), ctypes.c_void_p(d_U), len(xyz), _ptr(xyz), int(ireg),
                                           float(sprd), _ptr(out)))
        if response is None and active is None:
            return out
        return receivers.apply_geophone_response(out, response, active)

    def sample_pressure(self, d_U, nrhs, xyz, ireg=0, sprd=0.5, active=None):
        """Hydrophone pressure (makeuh.f), shape (nrhs, nrec); zero for
        inactive source-hydrophone pairs active[nrhs, nrec] == 0."""
        from . import receivers
        xyz = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros((nrhs, len(xyz)), np.complex128)
        _check(lib().wt3d_sample_pressure(self._h, int(nrhs), ctypes.c_void_p(d_U), len(xyz), _ptr(xyz), int(ireg),
                                          float(sprd), _ptr(out)))
        return out if active is None else receivers.apply_hydrophone_mask(out, active)

    def apply_device(self, d_X, d_Y, nrhs):
        """Y = A X on device arrays (column-major n x nrhs complex128)."""
        _check(lib().wt3d_apply_device(self._h, int(nrhs), ctypes.c_void_p(d_X), ctypes.c_void_p(d_Y)))

    def update_operator(self):
        """Re-assemble A from the current model at the factored omega; the
        factors stay and precondition later solves."""
        _check(lib().wt3d_update_operator(self._h))

    def _split_grad(self, g):
        nn, G = self.grid.nnodes, self.grid
        return [g[k * nn:(k + 1) * nn].reshape((G.nz, G.nx, G.ny), order="F") for k in range(3)]

    def gradient_contract(self, d_U, d_Lam, nrhs, d_grad=None):
        """-Re sum_j Lam_j^H dA/dm U_j for m = (Vp, Vs, rho) at every node.
        With d_grad (device double[3*nn]) writes there; otherwise returns
        three host arrays of shape (nz, nx, ny)."""
        if d_grad is not None:
            _check(lib().wt3d_gradient_contract(self._h, int(nrhs), ctypes.c_void_p(d_U), ctypes.c_void_p(d_Lam),
                                                ctypes.c_void_p(d_grad)))
            return None
        import torch
        g = torch.empty(3 * self.grid.nnodes, dtype=torch.float64, device="cuda")
        _check(lib().wt3d_gradient_contract(self._h, int(nrhs), ctypes.c_void_p(d_U), ctypes.c_void_p(d_Lam),
                                            ctypes.c_void_p(g.data_ptr())))
        return self._split_grad(g.cpu().numpy())

    def misfit_gradient(self, d_F, d_U0, nsrc, rec_node, dobs, tol=1e-8, maxit=20, allow_noconv=False):
        """Waveform misfit 1/2 sum |u(rec) - dobs|^2 and its gradient.
        d_F: device scattered-field (or point) RHS, d_U0: device background
        field or None; rec_node: 0-based node indices; dobs: complex
        [(j*nrec + r)*3 + c].  Returns (chi, [dVp, dVs, drho], dpred)."""
        rec = np.ascontiguousarray(rec_node, np.int64)
        dobs = np.ascontiguousarray(dobs, np.complex128).reshape(-1)
        if dobs.size != nsrc * len(rec) * 3:
            raise ValueError("dobs must hold nsrc * nrec * 3 values")
        chi = ctypes.c_double(0)
        grad = np.zeros(3 * self.grid.nnodes)
        dpred = np.zeros_like(dobs)
        rc = lib().wt3d_misfit_gradient(self._h, int(nsrc), ctypes.c_void_p(d_F), ctypes.c_void_p(d_U0 or 0),
                                        len(rec), _ptr(rec), _ptr(dobs), tol, maxit, ctypes.byref(chi),
                                        _ptr(grad), _ptr(dpred))
        _check(rc, allow=(WT3D_ERR_NOCONV,) if allow_noconv else ())
        return chi.value, self._split_grad(grad), dpred

    @property
    def stream(self):
        """cudaStream_t (as an int) of the handle's factorisation and operator calls."""
        return lib().wt3d_get_stream(self._h) or 0

    def solve_device(self, d_B, d_X, nrhs, tol=1e-8, maxit=20, adjoint=False, allow_noconv=False):
        """Solve with device pointers (column-major n x nrhs complex128)."""
        relres = np.zeros(nrhs)
        iters = ctypes.c_int(0)
        rc = lib().wt3d_solve_device(self._h, nrhs, ctypes.c_void_p(d_B), ctypes.c_void_p(d_X), tol, maxit,
                                     _ptr(relres), ctypes.byref(iters), int(adjoint))
        _check(rc, allow=(WT3D_ERR_NOCONV,) if allow_noconv else ())
        self.last_relres, self.last_iters = relres, iters.value
        return relres

    def profile_factor(self):
        """Per-kernel-kind milliseconds of one factorisation (no graph)."""
        kinds = ["memset", "scatter", "extend_add", "panel", "trsm", "gemm_simt", "sub_step", "tc_split",
                 "gemm_tc"]
        out = np.zeros(len(kinds) + 2)
        _check(lib().wt3d_profile_factor(self._h, _ptr(out)))
        d = {k + "_ms": float(out[i]) for i, k in enumerate(kinds)}
        d["gemm_flops"] = float(out[len(kinds)])
        d["gemm_launches"] = int(out[len(kinds) + 1])
        return d

    def set_attenuation(self, qp_inv, qs_inv, freqbase=20.0):
        """1/Qp, 1/Qs per node (None, None: elastic); dispersion at every factor()."""
        n = self.grid.nnodes
        if qp_inv is None:
            _check(lib().wt3d_set_attenuation(self._h, None, None, 0.0))
            self._q = None
            return
        self._q = (_f32(qp_inv, n), _f32(qs_inv, n))
        _check(lib().wt3d_set_attenuation(self._h, _ptr(self._q[0]), _ptr(self._q[1]), float(freqbase)))

    def set_background(self, vp, vs, rho):
        n = self.grid.nnodes
        self._bg = (_f32(vp, n), _f32(vs, n), _f32(rho, n))
        _check(lib().wt3d_set_background(self._h, *[_ptr(a) for a in self._bg]))

    def rhs_planewave(self, layers, ain, baz, s_wave=None, d_F=None, d_U0=None):
        """Scattered-field plane-wave sources at the factored omega.  With device
        pointers d_F (and d_U0) writes there; otherwise returns host arrays
        (F, U0) of shape (n, nsrc)."""
        ain = np.ascontiguousarray(ain, np.float64)
        baz = np.ascontiguousarray(baz, np.float64)
        ns = len(ain)
        sw = np.ascontiguousarray(s_wave if s_wave is not None else np.zeros(ns), np.int32)
        if d_F is not None:
            _check(lib().wt3d_rhs_planewave(self._h, ctypes.byref(layers), ns, _ptr(ain), _ptr(baz), _ptr(sw),
                                            ctypes.c_void_p(d_F), ctypes.c_void_p(d_U0 or 0)))
            return None
        import torch
        F = torch.zeros((ns, self.grid.n), dtype=torch.complex128, device="cuda")
        U0 = torch.zeros_like(F)
        _check(lib().wt3d_rhs_planewave(self._h, ctypes.byref(layers), ns, _ptr(ain), _ptr(baz), _ptr(sw),
                                        ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(U0.data_ptr())))
        return F.cpu().numpy().T.copy(), U0.cpu().numpy().T.copy()

    def profile_solve(self, m):
        """Per-kernel-kind milliseconds of one substitution pass over m columns
        and of one FP64 residual."""
        kinds = ["memset", "scatter", "extend_add", "panel", "trsm", "gemm_simt", "sub_step", "tc_split",
                 "gemm_tc"]
        out = np.zeros(12)
        _check(lib().wt3d_profile_solve(self._h, int(m), _ptr(out)))
        d = {k + "_ms": float(out[i]) for i, k in enumerate(kinds) if out[i] > 0}
        d["gemm_flops"] = float(out[9])
        d["residual_ms"] = float(out[11])
        return d

    def stats(self):
        s = Stats()
        _check(lib().wt3d_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()


def strumpack_serial_finter(job, nrows, nnz, irptr, jcptr, a, rhs, sol):
    """Call the drop-in job-protocol entry point exactly as the Fortran driver
    does (by reference, 1-based CSR, complex64).  Returns ierr."""
    c = ctypes.c_int
    ierr = c(0)
    lib().strumpack_serial_finter(ctypes.byref(c(job)), ctypes.byref(c(nrows)), ctypes.byref(c(nnz)),
                                  _ptr(irptr), _ptr(jcptr), _ptr(a), _ptr(rhs), _ptr(sol), ctypes.byref(ierr))
    return ierr.value
