"""Sources and receivers between nodes (SRCSETUP/SRCREG): the library's
weights against the oracle's restatement, and the properties the reference's
construction implies."""
import numpy as np
import pytest

import wtomo3d_gb300 as wt
from wtomo3d_gb300 import Grid, model


def _field(g, x, y, z, ireg, sprd):
    node, w = wt.source_weights(g, x, y, z, ireg, sprd)
    f = np.zeros(g.nx * g.ny * g.nz)
    np.add.at(f, node, w)
    return f


CASES = [
    # (x, y, z) in metres on a 20 m grid, ireg, sprd, fst
    ((200.0, 180.0, 160.0), 3, 0.5, 1),      # on a node
    ((207.3, 181.9, 163.1), 1, 0.5, 1),
    ((207.3, 181.9, 163.1), 2, 0.5, 1),
    ((207.3, 181.9, 163.1), 4, 0.5, 0),
    ((207.3, 181.9, 13.1), 3, 0.5, 1),       # region crosses the free surface: mirrored
    ((207.3, 181.9, 13.1), 3, 0.5, 0),       # ... or the absorbing top: dropped
    ((7.3, 181.9, 83.1), 2, 0.5, 1),         # crosses the x = 0 face
    ((207.3, 181.9, 163.1), 1, 0.75, 1),     # discrete Dirac
    ((207.3, 181.9, 163.1), 1, 1.0, 1),
    ((207.3, 181.9, 23.1), 1, 1.5, 1),
    ((207.3, 181.9, 23.1), 1, 1.5, 0),
]


@pytest.mark.parametrize("case", CASES)
def test_weights_match_oracle(oracle, case):
    (x, y, z), ireg, sprd, fst = case
    g = Grid(24, 22, 20, 20.0, pmld=80.0, fst=fst)
    ref = oracle.source_field(g, x, y, z, ireg, sprd).real
    got = _field(g, x, y, z, ireg, sprd)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_on_node_sinc_is_a_single_node():
    g = Grid(24, 22, 20, 20.0)
    for ireg in (1, 2, 5):
        node, w = wt.source_weights(g, 200.0, 180.0, 160.0, ireg, 0.5)
        keep = np.abs(w) > 1e-15
        assert keep.sum() == 1 and abs(w[keep][0] - 1.0) < 1e-15
        assert node[keep][0] == 8 + 20 * (10 + 24 * 9)


def test_dirac_weights_sum_to_one_and_mirror_with_sign():
    g = Grid(24, 22, 20, 20.0, fst=1)
    _, w = wt.source_weights(g, 207.3, 181.9, 163.1, 1, 1.25)
    assert abs(w.sum() - 1.0) < 1e-13
    # near the free top the mirrored terms enter with the opposite sign
    node, w = wt.source_weights(g, 207.3, 181.9, 3.1, 1, 1.25)
    assert (w < 0).any()
    g0 = Grid(24, 22, 20, 20.0, fst=0)
    _, w0 = wt.source_weights(g0, 207.3, 181.9, 3.1, 1, 1.25)
    assert (w0 > 0).all() and w0.sum() < 1.0


def test_sinc_weights_interpolate_smooth_fields():
    """A Kaiser-windowed sinc samples a band-limited field at the source point:
    a wave at 8 nodes per wavelength is reproduced to a small error."""
    g = Grid(40, 40, 40, 10.0)
    k = 2 * np.pi / 80.0
    iz, ix, iy = np.meshgrid(np.arange(40), np.arange(40), np.arange(40), indexing="ij")
    fld = np.cos(k * (ix * 10.0) + 0.3) * np.cos(k * 0.7 * (iy * 10.0)) * np.cos(k * 0.4 * (iz * 10.0))
    fld = fld.reshape(-1, order="F")
    x, y, z = 203.7, 188.2, 191.9
    exact = np.cos(k * x + 0.3) * np.cos(k * 0.7 * y) * np.cos(k * 0.4 * z)
    node, w = wt.source_weights(g, x, y, z, 4, 0.5)
    assert abs(np.dot(w, fld[node]) - exact) < 2e-3


def test_ireg0_is_the_nearest_node():
    g = Grid(24, 22, 20, 20.0)
    node, w = wt.source_weights(g, 207.3, 189.9, 163.1, 0)
    b = model.point_force(24, 22, 20, 20.0, 207.3, 189.9, 163.1, comp=0)
    assert len(node) == 1 and w[0] == 1.0 and np.nonzero(b)[0][0] == 3 * node[0]
