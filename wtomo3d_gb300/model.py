"""Synthetic earth models for the benchmark configurations.

Arrays are returned with shape (nz, nx, ny) and are indexed [iz, ix, iy] like
the reference's MODEL_MODULE arrays (modules.F90:10-21); flattening with
order="F" gives the node order g = iz + nz*ix + nz*nx*iy.
"""
import numpy as np


def homogeneous(nx, ny, nz, vp=5000.0, vs=2887.0, rho=2700.0):
    shape = (nz, nx, ny)
    return (np.full(shape, vp, np.float32), np.full(shape, vs, np.float32), np.full(shape, rho, np.float32))


def gardner(vp):
    """rho = 310 * vp^0.25 (kg/m^3, vp in m/s)."""
    return (310.0 * np.power(vp, 0.25)).astype(np.float32)


def correlated_field(nx, ny, nz, dx, corr_len, seed):
    """Zero-mean, unit-std Gaussian random field with a Gaussian correlation
    of length corr_len, made by FFT filtering of seeded white noise (PCG64)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    w = rng.standard_normal((nz, nx, ny))
    kz = np.fft.fftfreq(nz, d=dx) * 2 * np.pi
    kx = np.fft.fftfreq(nx, d=dx) * 2 * np.pi
    ky = np.fft.rfftfreq(ny, d=dx) * 2 * np.pi
    K2 = kz[:, None, None] ** 2 + kx[None, :, None] ** 2 + ky[None, None, :] ** 2
    f = np.fft.irfftn(np.fft.rfftn(w) * np.exp(-K2 * corr_len ** 2 / 8.0), s=w.shape, axes=(0, 1, 2))
    f -= f.mean()
    s = f.std()
    return f / s if s > 0 else f


def layered(nx, ny, nz, layer_vp=(3000.0, 4000.0, 5000.0, 6000.0), vpvs=1.73):
    """Equal-thickness flat layers along depth (z), Vs = Vp/vpvs, Gardner rho."""
    nl = len(layer_vp)
    iz = np.arange(nz)
    lay = np.minimum(iz * nl // nz, nl - 1)
    vp1 = np.asarray(layer_vp, np.float64)[lay]
    vp = np.broadcast_to(vp1[:, None, None], (nz, nx, ny)).astype(np.float64)
    vs = vp / vpvs
    return vp.astype(np.float32), vs.astype(np.float32), gardner(vp)


def layered_random(nx, ny, nz, dx, seed, std=0.05, corr_len=200.0,
                   layer_vp=(3000.0, 4000.0, 5000.0, 6000.0), vpvs=1.73):
    """Four flat layers plus a multiplicative seeded Gaussian-correlated
    perturbation of Vp and Vs (std `std`, correlation length corr_len m);
    rho recomputed from the perturbed Vp by Gardner's relation."""
    vp0, vs0, _ = layered(nx, ny, nz, layer_vp, vpvs)
    d = correlated_field(nx, ny, nz, dx, corr_len, seed)
    vp = vp0.astype(np.float64) * (1.0 + std * d)
    vs = vs0.astype(np.float64) * (1.0 + std * d)
    return vp.astype(np.float32), vs.astype(np.float32), gardner(vp)


def point_force(nx, ny, nz, dx, xloc, yloc, zloc, comp=2, sterm=1.0 + 0.0j):
    """Nearest-node point force (srcsetup.f:50-73 with ireg = 0) as a dof
    vector of length 3*nx*ny*nz; comp 0/1/2 = u/v/w (w = vertical)."""
    ixs = int(np.float32(0.5) + np.float32(xloc / dx)) + 1
    iys = int(np.float32(0.5) + np.float32(yloc / dx)) + 1
    izs = int(np.float32(0.5) + np.float32(zloc / dx)) + 1
    b = np.zeros(3 * nx * ny * nz, np.complex128)
    g = (izs - 1) + nz * (ixs - 1) + nz * nx * (iys - 1)
    b[3 * g + comp] = sterm
    return b


def layered1d(nz, dx, layer_vp=(3000.0, 4000.0, 5000.0, 6000.0), vpvs=1.73):
    """1-D description of layered(): (vp, vs, rho, ztop) float64 arrays for the
    Thomson-Haskell response, ztop[i] the depth of the first node of layer i
    (layer index iz*nl//nz), the last layer being the half-space."""
    nl = len(layer_vp)
    vp = np.asarray(layer_vp, np.float64)
    first = np.array([-(-i * nz // nl) for i in range(nl)], np.float64)   # ceil(i nz / nl)
    ztop = first * dx
    vs = (vp / vpvs).astype(np.float32).astype(np.float64)
    rho = (310.0 * np.power(vp, 0.25)).astype(np.float32).astype(np.float64)
    return vp, vs, rho, ztop


def perturbed(vp, vs, dx, seed, std=0.03, corr_len=200.0):
    """Multiplicative seeded Gaussian-correlated perturbation (std `std`) of
    Vp and Vs; rho recomputed from the perturbed Vp by Gardner's relation."""
    nz, nx, ny = np.shape(vp)
    d = correlated_field(nx, ny, nz, dx, corr_len, seed)
    vp2 = np.asarray(vp, np.float64) * (1.0 + std * d)
    vs2 = np.asarray(vs, np.float64) * (1.0 + std * d)
    return vp2.astype(np.float32), vs2.astype(np.float32), gardner(vp2)


def surface_receivers(nx, ny, nz, ipml, nrx=8, nry=5, depth=0):
    """0-based node indices of nrx x nry receivers on a regular grid at node
    depth `depth`, spread over the area inside the lateral absorbing layers."""
    ix = np.rint(np.linspace(ipml, nx - 1 - ipml, nrx)).astype(np.int64)
    iy = np.rint(np.linspace(ipml, ny - 1 - ipml, nry)).astype(np.int64)
    IY, IX = np.meshgrid(iy, ix, indexing="ij")
    return (depth + nz * IX + nz * nx * IY).reshape(-1)
