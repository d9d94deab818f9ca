"""Model IO index map (modelio.f90:98-130) on raw little-endian files."""
import numpy as np

from wtomo3d_gb300 import modelio


def test_index_map_and_round_trip(tmp_path):
    nx, ny, nz = 5, 4, 3
    flat = np.arange(nx * ny * nz, dtype=np.float32)
    w = modelio.h5_to_wt(flat, nx, ny, nz)
    for iz in range(1, nz + 1):
        for iy in range(1, ny + 1):
            for ix in range(1, nx + 1):
                indx = (iz - 1) * nx * ny + (iy - 1) * nx + ix   # modelio.f90:106
                assert w[iz - 1, ix - 1, iy - 1] == flat[indx - 1]
    p = tmp_path / "vp.bin"
    modelio.write_model(p, w)
    assert np.array_equal(np.fromfile(p, "<f4"), flat)
    assert np.array_equal(modelio.read_model(p, nx, ny, nz), w)
