"""ctypes binding of the CPU oracle (oracle/wt3d_oracle.c).

Test infrastructure only: the checker the CUDA path is compared against.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class OGrid(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("dx", ctypes.c_double),
                ("pmld", ctypes.c_double), ("pmlr", ctypes.c_double), ("fst", ctypes.c_int),
                ("usemin", ctypes.c_int)]


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


class Oracle:
    def __init__(self):
        from wtomo3d_gb300 import build
        path = build.build_oracle()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ora_srel3d_getsize.argtypes = [ctypes.c_int] * 3 + [ctypes.POINTER(ctypes.c_longlong)] * 2
        L.ora_pattern.argtypes = [ctypes.c_int] * 3 + [vp, vp]
        for f in (L.ora_assemble_c128, L.ora_assemble_c64):
            f.argtypes = [ctypes.POINTER(OGrid), vp, vp, vp, ctypes.c_double, ctypes.c_double, vp, vp]
        L.ora_assemble_q_c128.argtypes = [ctypes.POINTER(OGrid), vp, vp, vp, vp, vp, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, vp, vp]
        L.ora_node_blocks_c128.argtypes = [ctypes.POINTER(OGrid), vp, vp, vp, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
        L.ora_spmv_c128.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp]
        L.ora_source_weights.argtypes = [ctypes.POINTER(OGrid)] + [ctypes.c_double] * 3 + [ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, vp]
        L.ora_gradient_c128.argtypes = [ctypes.POINTER(OGrid), vp, vp, vp, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, vp, vp, vp]
        L.ora_haskgrn.argtypes = [ctypes.c_int, vp, vp, vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double, ctypes.c_double, vp, vp]
        self.L = L

    @staticmethod
    def grid(g):
        pmld = g.pmld if g.pmld > 0 else 10.0 * g.dx
        pmlr = g.pmlr if g.pmlr > 0 else 1e-3
        return OGrid(g.nx, g.ny, g.nz, g.dx, pmld, pmlr, g.fst, g.usemin)

    def getsize(self, nx, ny, nz):
        nv, ne = ctypes.c_longlong(), ctypes.c_longlong()
        self.L.ora_srel3d_getsize(nx, ny, nz, ctypes.byref(nv), ctypes.byref(ne))
        return nv.value, ne.value

    def pattern(self, nx, ny, nz):
        n, ne = self.getsize(nx, ny, nz)
        ir = np.zeros(n + 1, np.int32)
        jc = np.zeros(2 * ne + n, np.int32)
        rc = self.L.ora_pattern(nx, ny, nz, _p(ir), _p(jc))
        assert rc == 0
        return ir, jc

    def assemble(self, g, vp, vs, rho, omega, irptr, precision="c128"):
        og = self.grid(g)
        vp, vs, rho = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, order="F")) for x in (vp, vs, rho)]
        dt = np.complex128 if precision == "c128" else np.complex64
        a = np.zeros(irptr[-1] - 1, dt)
        f = self.L.ora_assemble_c128 if precision == "c128" else self.L.ora_assemble_c64
        om = complex(omega)
        ierr = f(ctypes.byref(og), _p(vp), _p(vs), _p(rho), om.real, om.imag, _p(irptr), _p(a))
        return a, ierr

    def assemble_q(self, g, vp, vs, rho, qp, qs, freqbase, omega, irptr):
        """complex128 ASMBLE after DISPERSION (qp, qs = 1/Q per node)."""
        og = self.grid(g)
        arrs = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, order="F")) for x in (vp, vs, rho, qp, qs)]
        a = np.zeros(irptr[-1] - 1, np.complex128)
        om = complex(omega)
        ierr = self.L.ora_assemble_q_c128(ctypes.byref(og), *[_p(x) for x in arrs], float(freqbase), om.real,
                                          om.imag, _p(irptr), _p(a))
        return a, ierr

    def node_blocks(self, g, vp, vs, rho, omega, iz, ix, iy):
        og = self.grid(g)
        vp, vs, rho = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, order="F")) for x in (vp, vs, rho)]
        blk = np.zeros(27 * 9, np.complex128)
        act = np.zeros(27, np.int32)
        om = complex(omega)
        ierr = self.L.ora_node_blocks_c128(ctypes.byref(og), _p(vp), _p(vs), _p(rho), om.real, om.imag,
                                           iz, ix, iy, _p(blk), _p(act))
        return blk.reshape(27, 3, 3), act, ierr

    def source_field(self, g, x, y, z, ireg, sprd, sterm=1.0):
        """Node field (model order, complex) of a spread source (ireg > 0)."""
        og = self.grid(g)
        f = np.zeros(g.nx * g.ny * g.nz, np.complex128)
        st = complex(sterm)
        rc = self.L.ora_source_weights(ctypes.byref(og), x, y, z, int(ireg), float(sprd), st.real, st.imag, _p(f))
        assert rc == 0, rc
        return f

    def gradient(self, g, vp, vs, rho, omega, U, Lam):
        """FP64 gradient (dchi/dVp, dchi/dVs, dchi/drho), each (nz, nx, ny),
        of dchi/dm = -Re sum_j Lam_j^H dA/dm U_j; U, Lam are (3nn, nrhs)."""
        og = self.grid(g)
        vp, vs, rho = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1, order="F")) for x in (vp, vs, rho)]
        U = np.asfortranarray(np.asarray(U, np.complex128).reshape(len(vp) * 3, -1))
        Lam = np.asfortranarray(np.asarray(Lam, np.complex128).reshape(len(vp) * 3, -1))
        assert U.shape == Lam.shape
        grad = np.zeros(3 * len(vp), np.float64)
        om = complex(omega)
        rc = self.L.ora_gradient_c128(ctypes.byref(og), _p(vp), _p(vs), _p(rho), om.real, om.imag, U.shape[1],
                                      _p(U), _p(Lam), _p(grad))
        assert rc == 0
        return [grad[k * len(vp):(k + 1) * len(vp)].reshape((g.nz, g.nx, g.ny), order="F") for k in range(3)]

    def haskgrn(self, vp, vs, rho, ztop, omega, ain, nz, dz, s_wave=False, zorig=0.0):
        arr = [np.ascontiguousarray(a, np.float64) for a in (vp, vs, rho, ztop)]
        U = np.zeros(nz, np.complex128)
        W = np.zeros(nz, np.complex128)
        rc = self.L.ora_haskgrn(len(arr[0]), *[_p(a) for a in arr], float(omega), float(ain), int(bool(s_wave)),
                                int(nz), float(dz), float(zorig), _p(U), _p(W))
        assert rc == 0, rc
        return U, W

    def planewave(self, g, layers1d, omega, ain, baz, s_wave=False):
        """Incident field u0 on the grid (the definition documented with the
        GPU kernel): [U* rx, U* ry, W*] exp(i omega p (x rx + y ry)), with the
        Haskell response conjugated to the operator's time sign."""
        vp, vs, rho, zt = layers1d
        U, W = self.haskgrn(vp, vs, rho, zt, omega, ain, g.nz, g.dx, s_wave)
        U, W = U.conj(), W.conj()
        vh = vs[-1] if s_wave else vp[-1]
        p = np.sin(ain) / vh
        rx, ry = -np.cos(baz), -np.sin(baz)
        iz, ix, iy = np.meshgrid(np.arange(g.nz), np.arange(g.nx), np.arange(g.ny), indexing="ij")
        iz, ix, iy = [t.reshape(-1, order="F") for t in (iz, ix, iy)]
        ph = np.exp(1j * omega * p * (ix * g.dx * rx + iy * g.dx * ry))
        u0 = np.zeros(3 * len(iz), np.complex128)
        u0[0::3] = U[iz] * rx * ph
        u0[1::3] = U[iz] * ry * ph
        u0[2::3] = W[iz] * ph
        return u0
