"""Generate the golden fixtures of tests/golden/*.npz from the CPU oracle.

The reference ships no golden vectors; these fixtures pin the oracle's own
output (pattern bit-exact, complex128 values) so that later changes to the
restatement are caught.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

CASES = {
    # 10-node-style PML on all faces, scaled down: 2-node PML, fst off, 1 Hz
    "asm_c1_small": dict(dims=(7, 6, 8), dx=25.0, pml_nodes=2, fst=0, usemin=1, f=1.0, tau=None, model="homog"),
    # free surface with traction-free rows (usemin off), anti-alias complex omega
    "asm_fst_tpfree": dict(dims=(6, 7, 6), dx=20.0, pml_nodes=2, fst=1, usemin=0, f=1.5, tau=2.0, model="homog"),
    # free surface Min cells, layered + random model
    "asm_layered": dict(dims=(6, 6, 7), dx=20.0, pml_nodes=3, fst=1, usemin=1, f=2.0, tau=None, model="layered"),
}


def load_case(name):
    """Grid, model arrays and omega of a committed fixture (model stored in the file)."""
    from wtomo3d_gb300 import Grid
    c = CASES[name]
    z = np.load(os.path.join(HERE, name + ".npz"))
    nx, ny, nz = c["dims"]
    g = Grid(nx, ny, nz, c["dx"], pmld=c["pml_nodes"] * c["dx"], fst=c["fst"], usemin=c["usemin"])
    return g, z["vp"], z["vs"], z["rho"], complex(z["omega"]), z


def build_case(c):
    from wtomo3d_gb300 import Grid, model
    nx, ny, nz = c["dims"]
    g = Grid(nx, ny, nz, c["dx"], pmld=c["pml_nodes"] * c["dx"], fst=c["fst"], usemin=c["usemin"])
    if c["model"] == "homog":
        vp, vs, rho = model.homogeneous(nx, ny, nz)
    else:
        vp, vs, rho = model.layered_random(nx, ny, nz, c["dx"], seed=11)
    om = 2 * np.pi * c["f"] + (1j / c["tau"] if c["tau"] else 0)
    return g, vp, vs, rho, om


def main():
    import oracle_ctypes
    o = oracle_ctypes.Oracle()
    for name, c in CASES.items():
        g, vp, vs, rho, om = build_case(c)
        ir, jc = o.pattern(g.nx, g.ny, g.nz)
        a, ierr = o.assemble(g, vp, vs, rho, om, ir)
        assert ierr == 0
        np.savez_compressed(os.path.join(HERE, name + ".npz"), irptr=ir, jcptr=jc, a=a, vp=vp, vs=vs, rho=rho,
                            omega=np.complex128(om))
        print(name, g.nx, g.ny, g.nz, len(a))


if __name__ == "__main__":
    main()
