"""Golden fixtures computed by the reference's own Fortran statements.

Recipe: runs the reference source tree through oracle/fortran_eval.py (an
evaluator of the Fortran text, complex128) and stores inputs and outputs as
tests/golden/ref_*.npz.  The GPU machine has no copy of the reference, so the
fixtures travel instead; tests/test_reference_pinned.py re-runs a subset here
when the reference tree is present and checks that the stored fixtures are
exactly what the reference's statements produce.

    python tests/golden/make_reference_golden.py [reference-tree]

Cases
  assembly (ASMBLE, asmble.f90:1-636 with SETCOEFS3D, CALCWTS, FDFD3D,
  PFDFD3D, PML3D, FIXED3D, TPFREE, ZEROAS; pattern from srel3d +
  SPARSE_ADJ2CRS; lambda/mu from modelio.f90:78-92; ipml/pmlf from
  readini.f90:83-84) on random heterogeneous models covering every FDFD3D
  region (fdfd3d.f:53-115); one case after DISPERSION (dispersion.f);
  HASKGRN (haskgrn.f) for P and S plane waves on the configuration-2 layering;
  HETFLDSRC (hetfldsrc.f90) for a plane-wave incident field on a perturbed
  model (ny == nz, where the reference's output index at hetfldsrc.f90:1020
  is the true node index);
  SRCSETUP/SRCREG (srcsetup.f, srcreg.f) point sources: nearest node,
  Kaiser-windowed sinc and discrete Dirac spreading, mirrored at the free
  surface.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DEFAULT_REFERENCE = "/root/reference"


def _paths():
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def random_model(nx, ny, nz, seed):
    """Independent random Vp, Vs, rho per node (float32, [iz, ix, iy]): every
    3x3x3 neighbourhood is different."""
    rng = np.random.default_rng(seed)
    vp = (3000.0 + 3000.0 * rng.random((nz, nx, ny))).astype(np.float32)
    vs = (vp / (1.55 + 0.5 * rng.random((nz, nx, ny)))).astype(np.float32)
    rho = (1800.0 + 1000.0 * rng.random((nz, nx, ny))).astype(np.float32)
    return vp, vs, rho


# name: (nx, ny, nz, dx, pml nodes, fst, usemin, omega, seed)
ASM_CASES = {
    "pml6_cw": (7, 6, 8, 20.0, 2, 0, 1, 2 * np.pi * 1.3 + 0.2j, 11),      # PML on all faces, complex omega
    "fs_min": (6, 7, 8, 20.0, 2, 1, 1, 2 * np.pi * 1.0, 12),              # free surface, Min cells
    "fs_tpfree": (6, 6, 7, 25.0, 2, 1, 0, 2 * np.pi * 0.7, 13),           # free surface, traction-free rows
    "overlap": (6, 7, 6, 20.0, 3, 0, 1, 2 * np.pi * 2.0, 14),             # ipml = 4: the PMLs overlap
}
Q_CASE = (6, 6, 7, 20.0, 2, 1, 1, 2 * np.pi * 1.5, 15)                    # DISPERSION, then ASMBLE
HASK_NZ, HASK_DX = 40, 20.0
HASK_CASES = [(s, f, a) for s in (0, 1) for f in (0.5, 2.0) for a in (4.0, 22.0)]
HET_CASE = (8, 7, 7, 20.0, 2, 1, 1, 2 * np.pi * 1.5)
HET_WAVES = [(18.0, 130.0, 0), (27.0, 300.0, 1)]
SRC_GRID = (8, 7, 7, 20.0)
SRC_CASES = [(61.0, 47.0, 33.0, 0, 0.0), (61.0, 47.0, 33.0, 4, 0.4), (70.0, 50.0, 12.0, 4, 0.3),
             (55.0, 65.0, 21.0, 3, 0.8), (40.0, 60.0, 5.0, 2, 0.7), (33.3, 81.7, 2.5, 3, 0.5)]


def assembly_case(name, ref):
    import fortran_eval as fe
    nx, ny, nz, dx, pn, fst, usemin, om, seed = ASM_CASES[name]
    vp, vs, rho = random_model(nx, ny, nz, seed)
    ir, jc, a, ierr, info = fe.reference_assemble(ref, nx, ny, nz, dx, vp, vs, rho, om, pn * dx, fst, usemin)
    return dict(dims=np.array([nx, ny, nz]), dx=dx, pmld=pn * dx, fst=fst, usemin=usemin, omega=complex(om),
                vp=vp, vs=vs, rho=rho, irptr=np.array(ir, np.int32), jcptr=np.array(jc, np.int32),
                a=np.array(a, np.complex128), ierr=ierr, ipml=info["ipml"], pmlf=info["pmlf"])


def q_case(ref):
    import fortran_eval as fe
    nx, ny, nz, dx, pn, fst, usemin, om, seed = Q_CASE
    vp, vs, rho = random_model(nx, ny, nz, seed)
    rng = np.random.default_rng(seed + 100)
    qp = rng.uniform(0.005, 0.03, vp.shape).astype(np.float32)
    qs = rng.uniform(0.01, 0.05, vp.shape).astype(np.float32)
    ir, jc, a, ierr = fe.reference_dispersed_assemble(ref, nx, ny, nz, dx, vp, vs, rho, qp, qs, 20.0, om, pn * dx,
                                                      fst, usemin)
    return dict(dims=np.array([nx, ny, nz]), dx=dx, pmld=pn * dx, fst=fst, usemin=usemin, omega=complex(om),
                vp=vp, vs=vs, rho=rho, qp=qp, qs=qs, freqbase=20.0, irptr=np.array(ir, np.int32),
                jcptr=np.array(jc, np.int32), a=np.array(a, np.complex128), ierr=ierr)


def hask_case(ref):
    import fortran_eval as fe
    from wtomo3d_gb300 import model
    vp, vs, rho, zt = model.layered1d(HASK_NZ, HASK_DX)
    U, W, err = [], [], []
    for s_wave, f, ain in HASK_CASES:
        u, w, ierr = fe.reference_haskgrn(ref, vp, vs, rho, zt, 2 * np.pi * f, np.radians(ain), HASK_NZ, HASK_DX,
                                          bool(s_wave))
        U.append(u)
        W.append(w)
        err.append(ierr)
    return dict(vp=vp, vs=vs, rho=rho, zt=zt, nz=HASK_NZ, dz=HASK_DX, cases=np.array(HASK_CASES, np.float64),
                U=np.array(U, np.complex128), W=np.array(W, np.complex128), ierr=np.array(err))


def het_case(ref):
    import fortran_eval as fe
    import oracle_ctypes
    from wtomo3d_gb300 import Grid, model
    nx, ny, nz, dx, pn, fst, usemin, om = HET_CASE
    g = Grid(nx, ny, nz, dx, pmld=pn * dx, fst=fst, usemin=usemin)
    bg = model.layered(nx, ny, nz)
    mdl = model.layered_random(nx, ny, nz, dx, seed=3)
    lay = model.layered1d(nz, dx)
    o = oracle_ctypes.Oracle()
    U0, F = [], []
    for ain, baz, sw in HET_WAVES:
        # the incident field by the documented plane-wave expansion (the
        # reference's planewvexp.f90 is missing from its tree)
        u0 = o.planewave(g, lay, om, np.radians(ain), np.radians(baz), bool(sw))
        f, ierr = fe.reference_hetfldsrc(ref, nx, ny, nz, dx, mdl, bg, om, pn * dx, fst, usemin, u0)
        assert ierr == 0
        U0.append(u0)
        F.append(f)
    return dict(dims=np.array([nx, ny, nz]), dx=dx, pmld=pn * dx, fst=fst, usemin=usemin, omega=complex(om),
                vp=mdl[0], vs=mdl[1], rho=mdl[2], vp0=bg[0], vs0=bg[1], rho0=bg[2],
                lay_vp=lay[0], lay_vs=lay[1], lay_rho=lay[2], lay_zt=lay[3], waves=np.array(HET_WAVES, np.float64),
                u0=np.array(U0), f=np.array(F, np.complex128))


def src_case(ref):
    import fortran_eval as fe
    nx, ny, nz, dx = SRC_GRID
    S = []
    for x, y, z, ireg, sprd in SRC_CASES:
        sw, ierr = fe.reference_point_source(ref, nx, ny, nz, dx, True, x, y, z, sprd, ireg)
        assert ierr == 0
        S.append(sw)
    return dict(dims=np.array([nx, ny, nz]), dx=dx, cases=np.array(SRC_CASES, np.float64),
                swave=np.array(S, np.complex128))


def path(name):
    return os.path.join(HERE, "ref_%s.npz" % name)


def main(ref=DEFAULT_REFERENCE):
    _paths()
    for name in ASM_CASES:
        np.savez_compressed(path("asm_" + name), **assembly_case(name, ref))
        print("wrote", path("asm_" + name))
    np.savez_compressed(path("asm_q"), **q_case(ref))
    np.savez_compressed(path("haskgrn"), **hask_case(ref))
    np.savez_compressed(path("hetfldsrc"), **het_case(ref))
    np.savez_compressed(path("srcsetup"), **src_case(ref))
    print("done")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REFERENCE)
