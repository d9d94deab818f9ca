"""The oracle pinned to the reference's own Fortran statements.

tests/golden/ref_*.npz hold outputs of the reference's code (ASMBLE and the
routines it calls, DISPERSION, HASKGRN, HETFLDSRC, SRCSETUP/SRCREG) run from
its source text by oracle/fortran_eval.py (tests/golden/make_reference_golden.py
is the recipe).  Here the C oracle, and the library's host code where it has
some, are compared with them; when the reference tree is present the
fixtures are recomputed from it and must match exactly.
"""
import os
import platform

import numpy as np
import pytest
import scipy.sparse as sp

import make_reference_golden as mrg
import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model

# x86-64 builds of the oracle evaluate every formula in the reference's
# operation order without fused multiply-adds: bit for bit.  Elsewhere the C
# compiler may contract a*b + c into one rounding.
EXACT = platform.machine() in ("x86_64", "AMD64")
TOL_ASM = 0.0 if EXACT else 1e-14


def load(name):
    return dict(np.load(mrg.path(name)))


def grid_of(z):
    nx, ny, nz = (int(v) for v in z["dims"])
    return Grid(nx, ny, nz, float(z["dx"]), pmld=float(z["pmld"]), fst=int(z["fst"]), usemin=int(z["usemin"]))


@pytest.mark.parametrize("name", sorted(mrg.ASM_CASES))
def test_oracle_assembly_equals_reference_statements(oracle, name):
    z = load("asm_" + name)
    g = grid_of(z)
    assert int(z["ierr"]) == 0
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    np.testing.assert_array_equal(ir, z["irptr"])
    np.testing.assert_array_equal(jc, z["jcptr"])
    a, ierr = oracle.assemble(g, z["vp"], z["vs"], z["rho"], complex(z["omega"]), ir)
    assert ierr == 0
    ref = z["a"]
    assert len(np.unique(ref)) > 0.1 * len(ref)             # a real operator: many distinct values
    err = np.abs(a - ref).max()
    assert err <= TOL_ASM * np.abs(ref).max(), err
    # the closed-form nnz of the reference's own self-check (srgraphs.f:626-636)
    assert len(ref) == g.nnz


def test_oracle_dispersed_assembly_equals_reference_statements(oracle):
    z = load("asm_q")
    g = grid_of(z)
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    a, ierr = oracle.assemble_q(g, z["vp"], z["vs"], z["rho"], z["qp"], z["qs"], float(z["freqbase"]),
                                complex(z["omega"]), ir)
    assert ierr == 0 and int(z["ierr"]) == 0
    assert np.abs(a - z["a"]).max() <= TOL_ASM * np.abs(z["a"]).max()


def test_haskgrn_equals_reference_statements(oracle):
    """The oracle's and the library's host Thomson-Haskell response against
    HASKGRN run from its text (P and S, two frequencies, two angles)."""
    z = load("haskgrn")
    lay = (z["vp"], z["vs"], z["rho"], z["zt"])
    L = wt.Layered1D(*lay)
    for k, (s_wave, f, ain) in enumerate(z["cases"]):
        assert int(z["ierr"][k]) == 0
        om, a = 2 * np.pi * f, np.radians(ain)
        Uo, Wo = oracle.haskgrn(*lay, om, a, int(z["nz"]), float(z["dz"]), bool(s_wave))
        U, W = wt.haskgrn(L, om, a, int(z["nz"]), float(z["dz"]), bool(s_wave))
        scale = max(np.abs(z["U"][k]).max(), np.abs(z["W"][k]).max())
        for got in ((Uo, Wo), (U, W)):
            assert np.abs(got[0] - z["U"][k]).max() <= 1e-13 * scale
            assert np.abs(got[1] - z["W"][k]).max() <= 1e-13 * scale


def test_scattered_field_source_equals_reference_statements(oracle):
    """(A_bg - A) u0 from two oracle operators against HETFLDSRC's per-node
    accumulation (summation order differs: 1e-12 of the largest entry)."""
    z = load("hetfldsrc")
    g = grid_of(z)
    om = complex(z["omega"])
    ir, jc = oracle.pattern(g.nx, g.ny, g.nz)
    A = sp.csr_matrix((oracle.assemble(g, z["vp"], z["vs"], z["rho"], om, ir)[0], jc - 1, ir - 1), shape=(g.n, g.n))
    Ab = sp.csr_matrix((oracle.assemble(g, z["vp0"], z["vs0"], z["rho0"], om, ir)[0], jc - 1, ir - 1),
                       shape=(g.n, g.n))
    for j in range(len(z["waves"])):
        f = (Ab - A) @ z["u0"][j]
        assert np.abs(f - z["f"][j]).max() <= 1e-12 * np.abs(z["f"][j]).max()
        assert np.abs(z["f"][j]).max() > 0


def test_point_sources_equal_reference_statements(oracle):
    """Nearest-node, sinc-spread and Dirac-spread point sources with
    free-surface mirroring.  The reference evaluates I0 by a polynomial fit
    (srcreg.f:309-331) accurate to about 1e-7; the oracle and the library use
    the series: agreement to 1e-7 of the largest weight, exact for the
    nearest-node and Dirac cases, which do not use I0."""
    z = load("srcsetup")
    nx, ny, nz = (int(v) for v in z["dims"])
    g = Grid(nx, ny, nz, float(z["dx"]), pmld=2 * float(z["dx"]), fst=1, usemin=1)
    for k, (x, y, zz, ireg, sprd) in enumerate(z["cases"]):
        ref = z["swave"][k]
        ireg = int(ireg)
        lib = np.zeros(g.nnodes, np.complex128)
        node, w = wt.source_weights(g, x, y, zz, ireg, sprd)
        np.add.at(lib, node, w)
        tol = 1e-7 if (ireg > 0 and sprd <= 0.5) else 1e-14
        assert np.abs(lib - ref).max() <= tol * np.abs(ref).max(), (k, np.abs(lib - ref).max())
        if ireg > 0:
            ora = oracle.source_field(g, x, y, zz, ireg, sprd)
            assert np.abs(ora - ref).max() <= tol * np.abs(ref).max()
        assert np.count_nonzero(ref) == np.count_nonzero(lib)


REF = os.environ.get("WT3D_REFERENCE_TREE", mrg.DEFAULT_REFERENCE)
needs_ref = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "asmble.f90")),
                               reason="reference source tree not present")


@needs_ref
def test_fixtures_are_what_the_reference_statements_give():
    """Recomputes two assembly fixtures, the Haskell fixture and the source
    fixture from the reference tree: identical to the stored ones."""
    mrg._paths()
    for name in ("fs_min", "overlap"):
        z = load("asm_" + name)
        new = mrg.assembly_case(name, REF)
        np.testing.assert_array_equal(new["a"], z["a"])
        np.testing.assert_array_equal(new["jcptr"], z["jcptr"])
    np.testing.assert_array_equal(mrg.hask_case(REF)["U"], load("haskgrn")["U"])
    np.testing.assert_array_equal(mrg.src_case(REF)["swave"], load("srcsetup")["swave"])


@needs_ref
def test_planted_stencil_change_is_detected(oracle):
    """The comparison is sensitive: the same evaluation with one coefficient of
    the reference's mass-lumping fit perturbed in the evaluator's copy of the
    program (not in any file) no longer matches the oracle."""
    import fortran_eval as fe
    mrg._paths()
    nx, ny, nz, dx, pn, fst, usemin, om, seed = mrg.ASM_CASES["fs_min"]
    vp, vs, rho = mrg.random_model(nx, ny, nz, seed)
    P = fe.load_assembly(REF)
    u = P.units["calcwts"]
    u.stmts = [(ln, lab, t.replace("0.6367377d+00", "0.6367378d+00")) for ln, lab, t in u.stmts]
    ir, jc, a, ierr, _ = fe.reference_assemble(REF, nx, ny, nz, dx, vp, vs, rho, om, pn * dx, fst, usemin,
                                               program=P)
    g = Grid(nx, ny, nz, dx, pmld=pn * dx, fst=fst, usemin=usemin)
    ora, _ = oracle.assemble(g, vp, vs, rho, om, np.array(ir, np.int32))
    assert np.abs(np.array(a) - ora).max() > 1e-12 * np.abs(ora).max()
