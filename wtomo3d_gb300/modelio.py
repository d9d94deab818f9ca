"""Model input and output as raw little-endian float32 files.

The reference keeps models in HDF5 with x fastest, then y, then z (file
index (iz-1) nx ny + (iy-1) nx + ix) and converts them to its (nz, nx, ny)
working order (modelio.f90:98-130, MODELIO_H52WT_MODEL / MODELIO_WT2H5_MODEL).
HDF5 is not available here; the same index map is applied to raw binaries.
Arrays in this package are (nz, nx, ny) numpy arrays indexed [iz, ix, iy].
"""
import numpy as np


def h5_to_wt(flat, nx, ny, nz):
    """File order (x fastest, y, z) -> (nz, nx, ny) (MODELIO_H52WT_MODEL)."""
    a = np.asarray(flat, np.float32).reshape(nz, ny, nx)      # [iz, iy, ix]
    return np.ascontiguousarray(a.transpose(0, 2, 1))         # [iz, ix, iy]


def wt_to_h5(wmod):
    """(nz, nx, ny) -> file order (x fastest, y, z) (MODELIO_WT2H5_MODEL)."""
    return np.ascontiguousarray(np.asarray(wmod, np.float32).transpose(0, 2, 1)).reshape(-1)


def read_model(path, nx, ny, nz):
    """One model array from a raw little-endian float32 file in the
    reference's HDF5 element order."""
    flat = np.fromfile(path, dtype="<f4")
    if flat.size != nx * ny * nz:
        raise ValueError("%s holds %d values, expected %d" % (path, flat.size, nx * ny * nz))
    return h5_to_wt(flat, nx, ny, nz)


def write_model(path, wmod):
    """Write a (nz, nx, ny) array as raw little-endian float32 in the
    reference's HDF5 element order."""
    wt_to_h5(wmod).astype("<f4").tofile(path)
