// 27-point elastic FDFD operator assembly with PML on sm_103a.
//
// GB300 design (one thread per grid node, z fastest so a warp covers 32
// consecutive nodes of a z-line and its neighbour loads coalesce):
//   * The reference computes the PML stretch factors inside PML3D on every one
//     of the up to 27 calls per node (pml3d.f:185-342).  Here they are built
//     once per node.
//   * The interior stencil PFDFD3D (pfdfd3d.f:137-576) equals the PML3D stencil
//     (pml3d.f:344-800) with r1 = 1 and r2 = 0 on every axis (the scalings
//     d1dxsq, d2dxsq, d4dxsq are exactly r1?qodq/4, r1?qo2dq and r1?r1?o4dq/4
//     at r1 = 1, and the r2 terms vanish).  So interior and PML nodes run one
//     branch-free formula set with per-axis factors that are identity outside
//     the absorbing layer: warps straddling the PML edge do not diverge.
//   * FIXED3D (fixed3d.f:42-343) and TPFREE (tpfree.f:57-427) keep their own
//     short paths.
// Region selection reproduces FDFD3D (fdfd3d.f:50-115) exactly, including the
// free-surface case that evaluates PML3D at iz = ipml+1 (z stretch off).
//
// Output: the 3 rows of node g are contiguous in the CSR (row u at
// irptr[3g]); active 3x3 blocks are written in slot order
// s = 9(dy+1)+3(dx+1)+(dz+1), the column order of srel3d (srgraphs.f:681-714).
#include "common.cuh"
#include "wtomo3d_gpu.h"
#include "internal.h"
#include <cub/cub.cuh>

namespace wt3d {

// ---------------------------------------------------------------------------
// model -> Lame parameters (modelio.f90:78-92), complex with zero imaginary part
// ---------------------------------------------------------------------------
__global__ void k_lame(long long n, const float *__restrict__ vp, const float *__restrict__ vs,
                       const float *__restrict__ rho, cx<double> *__restrict__ da,
                       cx<double> *__restrict__ mu, double *__restrict__ ro)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r = rho[i], s = vs[i], p = vp[i];
    double m = s * s * r;
    mu[i] = cx<double>(m, 0.0);
    da[i] = cx<double>(p * p * r - 2.0 * m, 0.0);
    ro[i] = r;
}

// ---------------------------------------------------------------------------
// per-node coefficient set
// ---------------------------------------------------------------------------
template <class R>
struct NodeCoefs {
    cx<R> u[9], da[9], lmu[9], lpu[9], lp2u[9];  // cells 1..8
    R ro[27];                                    // ro[(i-1) + 3(j-1) + 9(k-1)], i=x j=y k=z
    R wm1, wm2, wm3, wm4;
    R vpreal;
};

// Octant-cell averages (setcoefs3d.f:108-174) from a clamped 3x3x3 gather.
template <class R>
__device__ __forceinline__ void gather_coefs(const cx<R> *__restrict__ da, const cx<R> *__restrict__ mu,
                                             const R *__restrict__ ro, int nx, int ny, int nz,
                                             int iz, int ix, int iy, bool fst, NodeCoefs<R> &c)
{
    cx<R> ml[27], dl[27];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        int zg = min(max(iz + k - 1, 0), nz - 1);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            int yg = min(max(iy + j - 1, 0), ny - 1);
#pragma unroll
            for (int i = 0; i < 3; i++) {
                int xg = min(max(ix + i - 1, 0), nx - 1);
                long long off = zg + (long long)nz * (xg + (long long)nx * yg);
                int q = i + 3 * j + 9 * k;
                ml[q] = mu[off];
                dl[q] = da[off];
                c.ro[q] = ro[off];
            }
        }
    }
#define IDX(i, j, k) (((i)-1) + 3 * ((j)-1) + 9 * ((k)-1))
    // plane averages of the 4 quadrants (x-,y-), (x-,y+), (x+,y-), (x+,y+)
    cx<R> pm[3][4], pd[3][4];
#pragma unroll
    for (int k = 1; k <= 3; k++) {
        pm[k - 1][0] = (ml[IDX(1, 1, k)] + ml[IDX(2, 1, k)] + ml[IDX(1, 2, k)] + ml[IDX(2, 2, k)]) / R(4);
        pm[k - 1][1] = (ml[IDX(1, 3, k)] + ml[IDX(2, 3, k)] + ml[IDX(1, 2, k)] + ml[IDX(2, 2, k)]) / R(4);
        pm[k - 1][2] = (ml[IDX(3, 1, k)] + ml[IDX(2, 1, k)] + ml[IDX(3, 2, k)] + ml[IDX(2, 2, k)]) / R(4);
        pm[k - 1][3] = (ml[IDX(3, 3, k)] + ml[IDX(2, 3, k)] + ml[IDX(3, 2, k)] + ml[IDX(2, 2, k)]) / R(4);
        pd[k - 1][0] = (dl[IDX(1, 1, k)] + dl[IDX(2, 1, k)] + dl[IDX(1, 2, k)] + dl[IDX(2, 2, k)]) / R(4);
        pd[k - 1][1] = (dl[IDX(1, 3, k)] + dl[IDX(2, 3, k)] + dl[IDX(1, 2, k)] + dl[IDX(2, 2, k)]) / R(4);
        pd[k - 1][2] = (dl[IDX(3, 1, k)] + dl[IDX(2, 1, k)] + dl[IDX(3, 2, k)] + dl[IDX(2, 2, k)]) / R(4);
        pd[k - 1][3] = (dl[IDX(3, 3, k)] + dl[IDX(2, 3, k)] + dl[IDX(3, 2, k)] + dl[IDX(2, 2, k)]) / R(4);
    }
    const bool top = fst && iz == 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        c.u[q + 1] = top ? cx<R>(0) : (pm[0][q] + pm[1][q]) / R(2);
        c.da[q + 1] = top ? cx<R>(0) : (pd[0][q] + pd[1][q]) / R(2);
        c.u[q + 5] = (pm[2][q] + pm[1][q]) / R(2);
        c.da[q + 5] = (pd[2][q] + pd[1][q]) / R(2);
    }
    if (top) {
#pragma unroll
        for (int q = 0; q < 9; q++) c.ro[q] = R(0);   // upper density plane (k = 1)
    }
#pragma unroll
    for (int q = 1; q <= 8; q++) {
        c.lmu[q] = c.da[q] - c.u[q];
        c.lpu[q] = c.da[q] + c.u[q];
        c.lp2u[q] = c.lpu[q] + c.u[q];
    }
    // centre velocities and mass-lumping weights (setcoefs3d.f:224-226, calcwts.f)
    const R r0 = c.ro[IDX(2, 2, 2)];
    cx<R> d0 = dl[IDX(2, 2, 2)], m0 = ml[IDX(2, 2, 2)];
    cx<R> vp2 = (d0 + R(2) * m0) / r0;
    R vp = csqrt_(vp2).re;
    R vs = csqrt_(m0 / r0).re;
    c.vpreal = vp;
    double x = (double)vp / (double)vs;
    double w1 = 0.2909366 + x * (-0.1792402e-01 + x * (0.7329184e-02 + x * -0.1055034e-02));
    double w2 = 0, w3 = 0;
    if (w1 > 1.0) w1 = 1.0;
    else w2 = 0.6367377 + x * (-0.7982022e-02 + x * (0.3385164e-02 + x * -0.5065399e-03));
    if (w1 + w2 > 1.0) w2 = 0.0;
    else w3 = 0.07244875 + x * (0.2569959e-01 + x * (-0.1060011e-01 + x * 0.1540534e-02));
    if (w1 + w2 + w3 > 1.0) w3 = 1.0 - (w1 + w2);
    c.wm1 = (R)w1; c.wm2 = (R)w2; c.wm3 = (R)w3; c.wm4 = (R)(1.0 - (w1 + w2 + w3));
#undef IDX
}

// Per-node stretch factors for the unified stencil.  ax_idx is the 1-based
// index used by PML3D for that axis (0 = axis switched off).
template <class R>
struct Stretch {
    cx<R> X2, Y2, Z2, XY, XZ, YZ, rx, ry, rz;
};

template <class R>
__device__ __forceinline__ void axis_factor(int idx, int n, int ipml, R dx, R pmld, R pmlf, R vpreal,
                                            cx<R> eyeom, cx<R> &r1, cx<R> &r2)
{
    R dp = 0; int isn = 0;
    if (idx > 0) {
        if (idx <= ipml) { dp = pmld - R(idx - 1) * dx; isn = 1; }
        else if (n - idx + 1 <= ipml) { dp = pmld - R(n - idx) * dx; isn = -1; }
    }
    if (isn == 0) { r1 = cx<R>(1); r2 = cx<R>(0); return; }
    // kmax = 1, fdom = 0 (pml3d.f:170,174): kappa = 1, alpha = 0
    cx<R> dn(dp * dp * vpreal * pmlf, R(0));
    r1 = eyeom / (eyeom + dn);
    cx<R> r1sq = r1 * r1;
    cx<R> t = eyeom / (eyeom * eyeom);
    r2 = (R(isn) * R(2)) * (r1sq * r1) * dp * ((vpreal * pmlf) * t);
}

template <class R>
__device__ __forceinline__ void build_stretch(int ixi, int iyi, int izi, int nx, int ny, int nz, int ipml,
                                              R dx, R pmld, R pmlf, R vpreal, cx<R> omega, Stretch<R> &f)
{
    cx<R> eyeom = cx<R>(R(0), R(-1)) * omega;
    cx<R> r1x, r2x, r1y, r2y, r1z, r2z;
    axis_factor<R>(ixi, nx, ipml, dx, pmld, pmlf, vpreal, eyeom, r1x, r2x);
    axis_factor<R>(iyi, ny, ipml, dx, pmld, pmlf, vpreal, eyeom, r1y, r2y);
    axis_factor<R>(izi, nz, ipml, dx, pmld, pmlf, vpreal, eyeom, r1z, r2z);
    const R dxx = dx * dx, dxx4 = R(4) * dxx, dx2 = R(2) * dx;
    f.rx = (r2x / dx2) / R(4);
    f.ry = (r2y / dx2) / R(4);
    f.rz = (r2z / dx2) / R(4);
    f.X2 = (((r1x * r1x) / dxx) / R(4)) / R(2);
    f.Y2 = (((r1y * r1y) / dxx) / R(4)) / R(2);
    f.Z2 = (((r1z * r1z) / dxx) / R(4)) / R(2);
    f.XY = ((r1x * r1y) / dxx4) / R(4);
    f.XZ = ((r1x * r1z) / dxx4) / R(4);
    f.YZ = ((r1y * r1z) / dxx4) / R(4);
}

// 3x3 block of slot S in the unified PML form: b[0..8] = UU UV UW VU VV VW WU WV WW.
template <int S, class R>
__device__ __forceinline__ void stencil_block(const NodeCoefs<R> &c, const Stretch<R> &f, R m2, R m3, R m4,
                                              cx<R> m1, cx<R> *b)
{
    const cx<R> *u = c.u, *L = c.lp2u, *P = c.lpu, *M = c.lmu;
    const cx<R> X2 = f.X2, Y2 = f.Y2, Z2 = f.Z2, XY = f.XY, XZ = f.XZ, YZ = f.YZ;
    const cx<R> rx = f.rx, ry = f.ry, rz = f.rz;
    const cx<R> XpY = X2 + Y2, XpZ = X2 + Z2, YpZ = Y2 + Z2;
#define RO(i, j, k) c.ro[((i)-1) + 3 * ((j)-1) + 9 * ((k)-1)]
#define PUT(uu, uv, uw, vu, vv, vw, wu, wv, ww) \
    { b[0] = uu; b[1] = uv; b[2] = uw; b[3] = vu; b[4] = vv; b[5] = vw; b[6] = wu; b[7] = wv; b[8] = ww; }
    // corner blocks: one cell q, mass weight wm4/8
    if constexpr (S == 0) {      // a1m: cell 1
        cx<R> ms(m4 * RO(1, 1, 1));
        cx<R> uu = X2 * L[1] + YpZ * u[1] - rx * L[1] - (ry + rz) * u[1] + ms;
        cx<R> vv = Y2 * L[1] + XpZ * u[1] - ry * L[1] - (rx + rz) * u[1] + ms;
        cx<R> ww = Z2 * L[1] + XpY * u[1] - rz * L[1] - (rx + ry) * u[1] + ms;
        cx<R> uv = XY * P[1], uw = XZ * P[1], vw = YZ * P[1];
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 18) {  // a1p: cell 2
        cx<R> ms(m4 * RO(1, 3, 1));
        cx<R> uu = X2 * L[2] + YpZ * u[2] - rx * L[2] + (ry - rz) * u[2] + ms;
        cx<R> vv = Y2 * L[2] + XpZ * u[2] + ry * L[2] - (rx + rz) * u[2] + ms;
        cx<R> ww = Z2 * L[2] + XpY * u[2] - rz * L[2] - (rx - ry) * u[2] + ms;
        cx<R> uv = -(XY * P[2]), uw = XZ * P[2], vw = -(YZ * P[2]);
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 2) {   // a3m: cell 5
        cx<R> ms(m4 * RO(1, 1, 3));
        cx<R> uu = X2 * L[5] + YpZ * u[5] - rx * L[5] - (ry - rz) * u[5] + ms;
        cx<R> vv = Y2 * L[5] + XpZ * u[5] - ry * L[5] - (rx - rz) * u[5] + ms;
        cx<R> ww = Z2 * L[5] + XpY * u[5] + rz * L[5] - (rx - ry) * u[5] + ms;
        cx<R> uv = XY * P[5], uw = -(XZ * P[5]), vw = -(YZ * P[5]);
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 20) {  // a3p: cell 6
        cx<R> ms(m4 * RO(1, 3, 3));
        cx<R> uu = X2 * L[6] + YpZ * u[6] - rx * L[6] + (ry + rz) * u[6] + ms;
        cx<R> vv = Y2 * L[6] + XpZ * u[6] + ry * L[6] - (rx - rz) * u[6] + ms;
        cx<R> ww = Z2 * L[6] + XpY * u[6] + rz * L[6] - (rx + ry) * u[6] + ms;
        cx<R> uv = -(XY * P[6]), uw = -(XZ * P[6]), vw = YZ * P[6];
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 6) {   // a7m: cell 3
        cx<R> ms(m4 * RO(3, 1, 1));
        cx<R> uu = X2 * L[3] + YpZ * u[3] + rx * L[3] - (ry + rz) * u[3] + ms;
        cx<R> vv = Y2 * L[3] + XpZ * u[3] - ry * L[3] + (rx - rz) * u[3] + ms;
        cx<R> ww = Z2 * L[3] + XpY * u[3] - rz * L[3] + (rx + ry) * u[3] + ms;
        cx<R> uv = -(XY * P[3]), uw = -(XZ * P[3]), vw = YZ * P[3];
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 24) {  // a7p: cell 4
        cx<R> ms(m4 * RO(3, 3, 1));
        cx<R> uu = X2 * L[4] + YpZ * u[4] + rx * L[4] + (ry - rz) * u[4] + ms;
        cx<R> vv = Y2 * L[4] + XpZ * u[4] + ry * L[4] + (rx - rz) * u[4] + ms;
        cx<R> ww = Z2 * L[4] + XpY * u[4] - rz * L[4] + (rx - ry) * u[4] + ms;
        cx<R> uv = XY * P[4], uw = -(XZ * P[4]), vw = -(YZ * P[4]);
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 8) {   // a9m: cell 7
        cx<R> ms(m4 * RO(3, 1, 3));
        cx<R> uu = X2 * L[7] + YpZ * u[7] + rx * L[7] - (ry - rz) * u[7] + ms;
        cx<R> vv = Y2 * L[7] + XpZ * u[7] - ry * L[7] + (rx + rz) * u[7] + ms;
        cx<R> ww = Z2 * L[7] + XpY * u[7] + rz * L[7] + (rx - ry) * u[7] + ms;
        cx<R> uv = -(XY * P[7]), uw = XZ * P[7], vw = -(YZ * P[7]);
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    } else if constexpr (S == 26) {  // a9p: cell 8
        cx<R> ms(m4 * RO(3, 3, 3));
        cx<R> uu = X2 * L[8] + YpZ * u[8] + rx * L[8] + (ry + rz) * u[8] + ms;
        cx<R> vv = Y2 * L[8] + XpZ * u[8] + ry * L[8] + (rx + rz) * u[8] + ms;
        cx<R> ww = Z2 * L[8] + XpY * u[8] + rz * L[8] + (rx + ry) * u[8] + ms;
        cx<R> uv = XY * P[8], uw = XZ * P[8], vw = YZ * P[8];
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    }
    // edge blocks along y (dy = 0, dx, dz = +-1): two cells, mass wm3/12
    else if constexpr (S == 9) {     // a1n: cells 1,2
        cx<R> ms(m3 * RO(1, 2, 1));
        cx<R> d = -(Y2 * (u[1] + u[2])) + ms;
        cx<R> uv = XY * (M[2] - M[1]), uw = XZ * (P[1] + P[2]), vw = YZ * (M[1] - M[2]);
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    } else if constexpr (S == 11) {  // a3n: cells 5,6
        cx<R> ms(m3 * RO(1, 2, 3));
        cx<R> d = -(Y2 * (u[5] + u[6])) + ms;
        cx<R> uv = -(XY * (M[5] - M[6])), uw = -(XZ * (P[5] + P[6])), vw = -(YZ * (M[5] - M[6]));
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    } else if constexpr (S == 15) {  // a7n: cells 3,4
        cx<R> ms(m3 * RO(3, 2, 1));
        cx<R> d = -(Y2 * (u[4] + u[3])) + ms;
        cx<R> uv = -(XY * (M[4] - M[3])), uw = -(XZ * (P[4] + P[3])), vw = -(YZ * (M[4] - M[3]));
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    } else if constexpr (S == 17) {  // a9n: cells 7,8
        cx<R> ms(m3 * RO(3, 2, 3));
        cx<R> d = -(Y2 * (u[8] + u[7])) + ms;
        cx<R> uv = XY * (M[7] - M[8]), uw = XZ * (P[8] + P[7]), vw = YZ * (M[8] - M[7]);
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    }
    // edge blocks along z (dz = 0, dx, dy = +-1)
    else if constexpr (S == 1) {     // a2m: cells 1,5
        cx<R> ms(m3 * RO(1, 1, 2));
        cx<R> d = -(Z2 * (u[1] + u[5])) + ms, w = -(Z2 * (L[1] + L[5])) + ms;
        cx<R> uv = XY * (P[1] + P[5]), uw = -(XZ * (M[1] - M[5])), vw = -(YZ * (M[1] - M[5]));
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    } else if constexpr (S == 19) {  // a2p: cells 2,6
        cx<R> ms(m3 * RO(1, 3, 2));
        cx<R> d = -(Z2 * (u[2] + u[6])) + ms, w = -(Z2 * (L[2] + L[6])) + ms;
        cx<R> uv = -(XY * (P[2] + P[6])), uw = -(XZ * (M[2] - M[6])), vw = -(YZ * (M[6] - M[2]));
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    } else if constexpr (S == 7) {   // a8m: cells 3,7
        cx<R> ms(m3 * RO(3, 1, 2));
        cx<R> d = -(Z2 * (u[7] + u[3])) + ms, w = -(Z2 * (L[7] + L[3])) + ms;
        cx<R> uv = -(XY * (P[7] + P[3])), uw = -(XZ * (M[7] - M[3])), vw = -(YZ * (M[3] - M[7]));
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    } else if constexpr (S == 25) {  // a8p: cells 4,8
        cx<R> ms(m3 * RO(3, 3, 2));
        cx<R> d = -(Z2 * (u[8] + u[4])) + ms, w = -(Z2 * (L[8] + L[4])) + ms;
        cx<R> uv = XY * (P[8] + P[4]), uw = -(XZ * (M[8] - M[4])), vw = -(YZ * (M[8] - M[4]));
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    }
    // edge blocks along x (dx = 0, dy, dz = +-1)
    else if constexpr (S == 3) {     // a4m: cells 1,3
        cx<R> ms(m3 * RO(2, 1, 1));
        cx<R> d = -(X2 * (L[1] + L[3])) + ms, w = -(X2 * (u[1] + u[3])) + ms;
        cx<R> uv = XY * (M[1] - M[3]), uw = XZ * (M[1] - M[3]), vw = YZ * (P[1] + P[3]);
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    } else if constexpr (S == 21) {  // a4p: cells 2,4
        cx<R> ms(m3 * RO(2, 3, 1));
        cx<R> d = -(X2 * (L[2] + L[4])) + ms, w = -(X2 * (u[2] + u[4])) + ms;
        cx<R> uv = XY * (M[4] - M[2]), uw = XZ * (M[2] - M[4]), vw = -(YZ * (P[2] + P[4]));
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    } else if constexpr (S == 5) {   // a6m: cells 5,7
        cx<R> ms(m3 * RO(2, 1, 3));
        cx<R> d = -(X2 * (L[7] + L[5])) + ms, w = -(X2 * (u[7] + u[5])) + ms;
        cx<R> uv = XY * (M[5] - M[7]), uw = XZ * (M[7] - M[5]), vw = -(YZ * (P[7] + P[5]));
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    } else if constexpr (S == 23) {  // a6p: cells 6,8
        cx<R> ms(m3 * RO(2, 3, 3));
        cx<R> d = -(X2 * (L[8] + L[6])) + ms, w = -(X2 * (u[8] + u[6])) + ms;
        cx<R> uv = XY * (M[8] - M[6]), uw = XZ * (M[8] - M[6]), vw = YZ * (P[8] + P[6]);
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    }
    // face blocks (one nonzero offset): four cells, mass wm2/6
    else if constexpr (S == 10) {    // a2n (dx = -1): cells 1,2,5,6
        cx<R> ms(m2 * RO(1, 2, 2));
        cx<R> d = X2 * (L[1] + L[6] + L[2] + L[5]) + ms, w = X2 * (u[1] + u[6] + u[2] + u[5]) + ms;
        cx<R> uv = XY * (M[2] - M[5] + M[6] - M[1]);
        cx<R> uw = -(XZ * (M[2] - M[5] + M[1] - M[6]));
        cx<R> vw = YZ * (P[2] + P[5] - P[1] - P[6]);
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    } else if constexpr (S == 16) {  // a8n (dx = +1): cells 3,4,7,8
        cx<R> ms(m2 * RO(3, 2, 2));
        cx<R> d = X2 * (L[8] + L[3] + L[7] + L[4]) + ms, w = X2 * (u[8] + u[3] + u[7] + u[4]) + ms;
        cx<R> uv = XY * (M[7] - M[4] + M[3] - M[8]);
        cx<R> uw = -(XZ * (M[7] - M[4] + M[8] - M[3]));
        cx<R> vw = YZ * (P[7] + P[4] - P[8] - P[3]);
        PUT(d, uv, uw, -uv, d, vw, -uw, vw, w);
    } else if constexpr (S == 12) {  // a4n (dz = -1): cells 1..4
        cx<R> ms(m2 * RO(2, 2, 1));
        cx<R> d = Z2 * (u[1] + u[4] + u[2] + u[3]) + ms, w = Z2 * (L[1] + L[4] + L[2] + L[3]) + ms;
        cx<R> uv = -(XY * (P[1] + P[4] - P[2] - P[3]));
        cx<R> uw = XZ * (M[1] - M[4] + M[2] - M[3]);
        cx<R> vw = YZ * (M[1] - M[4] + M[3] - M[2]);
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    } else if constexpr (S == 14) {  // a6n (dz = +1): cells 5..8
        cx<R> ms(m2 * RO(2, 2, 3));
        cx<R> d = Z2 * (u[8] + u[5] + u[7] + u[6]) + ms, w = Z2 * (L[8] + L[5] + L[7] + L[6]) + ms;
        cx<R> uv = -(XY * (P[8] + P[5] - P[7] - P[6]));
        cx<R> uw = XZ * (M[8] - M[5] + M[7] - M[6]);
        cx<R> vw = YZ * (M[8] - M[5] + M[6] - M[7]);
        PUT(d, uv, uw, uv, d, vw, -uw, -vw, w);
    } else if constexpr (S == 4) {   // a5m (dy = -1): cells 1,3,5,7
        cx<R> ms(m2 * RO(2, 1, 2));
        cx<R> d = Y2 * (u[1] + u[7] + u[5] + u[3]) + ms;
        cx<R> uv = XY * (M[1] - M[7] + M[5] - M[3]);
        cx<R> uw = -(XZ * (P[1] + P[7] - P[5] - P[3]));
        cx<R> vw = -(YZ * (M[1] - M[7] - M[5] + M[3]));
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    } else if constexpr (S == 22) {  // a5p (dy = +1): cells 2,4,6,8
        cx<R> ms(m2 * RO(2, 3, 2));
        cx<R> d = Y2 * (u[8] + u[2] + u[4] + u[6]) + ms;
        cx<R> uv = XY * (M[8] - M[2] + M[4] - M[6]);
        cx<R> uw = -(XZ * (P[8] + P[2] - P[4] - P[6]));
        cx<R> vw = -(YZ * (M[8] - M[2] - M[4] + M[6]));
        PUT(d, uv, uw, -uv, d, vw, uw, -vw, d);
    }
    // centre block: all eight cells, mass wm1 * omega^2 * rho
    else if constexpr (S == 13) {
        cx<R> ms = m1;
        cx<R> ls = L[1] + L[2] + L[3] + L[4] + L[5] + L[6] + L[7] + L[8];
        cx<R> us = u[1] + u[2] + u[3] + u[4] + u[5] + u[6] + u[7] + u[8];
        cx<R> uu = -(X2 * ls) - YpZ * us + rx * (L[1] - L[8] + L[2] - L[7] + L[5] - L[4] + L[6] - L[3])
                 + (ry + rz) * (u[1] - u[8] + u[3] - u[6]) + (ry - rz) * (u[7] - u[2] + u[5] - u[4]) + ms;
        cx<R> vv = -(Y2 * ls) - XpZ * us + ry * (L[1] - L[2] + L[5] - L[6] + L[7] - L[8] + L[3] - L[4])
                 + (rx + rz) * (u[1] - u[8] + u[2] - u[7]) + (rx - rz) * (u[6] - u[3] + u[5] - u[4]) + ms;
        cx<R> ww = -(Z2 * ls) - XpY * us + rz * (L[1] - L[8] + L[2] - L[7] + L[4] - L[5] + L[3] - L[6])
                 + (rx + ry) * (u[1] - u[8] + u[5] - u[4]) + (rx - ry) * (u[2] - u[7] + u[6] - u[3]) + ms;
        cx<R> uv = XY * (P[2] - P[1] + P[7] - P[8] + P[3] - P[4] + P[6] - P[5]);
        cx<R> uw = XZ * (P[4] - P[1] + P[5] - P[8] + P[3] - P[2] + P[6] - P[7]);
        cx<R> vw = YZ * (P[2] - P[1] + P[7] - P[8] + P[4] - P[3] + P[5] - P[6]);
        PUT(uu, uv, uw, uv, vv, vw, uw, vw, ww);
    }
#undef RO
#undef PUT
}

// Traction-free top rows (TPFREE, tpfree.f:57-427): only 5 slots are nonzero.
template <int S, class R>
__device__ __forceinline__ void tpfree_block(const NodeCoefs<R> &c, cx<R> r1x, cx<R> r1y, R dxo8, cx<R> *b)
{
#pragma unroll
    for (int q = 0; q < 9; q++) b[q] = cx<R>(0);
    const cx<R> *u = c.u, *D = c.da, *L = c.lp2u;
    const cx<R> one(1);
    if constexpr (S == 2) {
        b[0] = dxo8 * u[5]; b[2] = -(r1x * dxo8 * u[5]); b[4] = dxo8 * u[5]; b[5] = -(r1y * dxo8 * u[5]);
        b[6] = -(r1x * dxo8 * D[5]); b[7] = -(r1y * dxo8 * D[5]); b[8] = dxo8 * L[5];
    } else if constexpr (S == 20) {
        b[0] = dxo8 * u[6]; b[2] = -(r1x * dxo8 * u[6]); b[4] = dxo8 * u[6]; b[5] = r1y * dxo8 * u[6];
        b[6] = -(r1x * dxo8 * D[6]); b[7] = r1y * dxo8 * D[6]; b[8] = dxo8 * L[6];
    } else if constexpr (S == 8) {
        b[0] = dxo8 * u[7]; b[2] = r1x * dxo8 * u[7]; b[4] = dxo8 * u[7]; b[5] = -(r1y * dxo8 * u[7]);
        b[6] = r1x * dxo8 * D[7]; b[7] = -(r1y * dxo8 * D[7]); b[8] = dxo8 * L[7];
    } else if constexpr (S == 26) {
        b[0] = dxo8 * u[8]; b[2] = r1x * dxo8 * u[8]; b[4] = dxo8 * u[8]; b[5] = r1y * dxo8 * u[8];
        b[6] = r1x * dxo8 * D[8]; b[7] = r1y * dxo8 * D[8]; b[8] = dxo8 * L[8];
    } else if constexpr (S == 13) {
        cx<R> su = u[8] + u[7] + u[6] + u[5];
        b[0] = -(one * dxo8 * su); b[4] = b[0];
        b[2] = r1x * dxo8 * (u[5] - u[8] + u[6] - u[7]);
        b[5] = r1y * dxo8 * (D[5] - D[8] - D[6] + D[7]);
        b[6] = r1x * dxo8 * (D[5] - D[8] + D[6] - D[7]);
        b[7] = r1y * dxo8 * (D[5] - D[8] - D[6] + D[7]);
        b[8] = -(one * dxo8 * (L[8] + L[7] + L[6] + L[5]));
    }
}

enum Region { REG_FIXED = 0, REG_STENCIL = 1, REG_TPFREE = 2 };

struct AsmParams {
    int nx, ny, nz, ipml, fst, usemin;
    double dx, pmld, pmlf;
    double om_re, om_im;
};

template <int S, class R, class OutT>
__device__ __forceinline__ void emit_slot(int region, const NodeCoefs<R> &c, const Stretch<R> &f, R m2, R m3,
                                          R m4, cx<R> m1, cx<R> r1x, cx<R> r1y, R dxo8, unsigned mask,
                                          OutT *__restrict__ ru, OutT *__restrict__ rv, OutT *__restrict__ rw)
{
    if (!((mask >> S) & 1u)) return;
    cx<R> b[9];
    if (region == REG_STENCIL) stencil_block<S, R>(c, f, m2, m3, m4, m1, b);
    else if (region == REG_TPFREE) tpfree_block<S, R>(c, r1x, r1y, dxo8, b);
    else {
#pragma unroll
        for (int q = 0; q < 9; q++) b[q] = cx<R>(0);
        if (S == 13) { b[0] = cx<R>(1); b[4] = cx<R>(1); b[8] = cx<R>(1); }
    }
    const int off = 3 * __popc(mask & ((1u << S) - 1u));
#pragma unroll
    for (int q = 0; q < 3; q++) {
        ru[off + q] = OutT{(decltype(OutT::x))b[q].re, (decltype(OutT::x))b[q].im};
        rv[off + q] = OutT{(decltype(OutT::x))b[3 + q].re, (decltype(OutT::x))b[3 + q].im};
        rw[off + q] = OutT{(decltype(OutT::x))b[6 + q].re, (decltype(OutT::x))b[6 + q].im};
    }
}

template <class R, class OutT, int... Ss>
__device__ __forceinline__ void emit_all(std::integer_sequence<int, Ss...>, int region, const NodeCoefs<R> &c,
                                         const Stretch<R> &f, R m2, R m3, R m4, cx<R> m1, cx<R> r1x, cx<R> r1y,
                                         R dxo8, unsigned mask, OutT *ru, OutT *rv, OutT *rw)
{
    (emit_slot<Ss, R, OutT>(region, c, f, m2, m3, m4, m1, r1x, r1y, dxo8, mask, ru, rv, rw), ...);
}

// One thread per grid node.  OutT = double2 (complex128 CSR values).
template <class R, class OutT>
__global__ void __launch_bounds__(128) k_assemble(AsmParams p, const cx<R> *__restrict__ da,
                                                  const cx<R> *__restrict__ mu, const R *__restrict__ ro,
                                                  const int *__restrict__ irptr, OutT *__restrict__ a)
{
    const long long nn = (long long)p.nx * p.ny * p.nz;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nn) return;
    const int iz = (int)(g % p.nz);
    const int ix = (int)((g / p.nz) % p.nx);
    const int iy = (int)(g / ((long long)p.nz * p.nx));
    // 1-based indices as the reference uses them
    const int jz = iz + 1, jx = ix + 1, jy = iy + 1;

    unsigned mask = 0;
#pragma unroll
    for (int s = 0; s < 27; s++) {
        int dy = s / 9 - 1, dxo = (s / 3) % 3 - 1, dz = s % 3 - 1;
        bool ok = (iy + dy >= 0) && (iy + dy < p.ny) && (ix + dxo >= 0) && (ix + dxo < p.nx) &&
                  (iz + dz >= 0) && (iz + dz < p.nz);
        mask |= (ok ? 1u : 0u) << s;
    }

    // region dispatch of FDFD3D (fdfd3d.f:53-115)
    const bool xyin = (jx > p.ipml) && (jx <= p.nx - p.ipml) && (jy > p.ipml) && (jy <= p.ny - p.ipml);
    int region = REG_STENCIL;
    int zidx = jz;  // z index fed to the stretch factor (0 = z stretch off)
    // Interior nodes (all axes inside) can never sit on the outer faces, so the
    // Dirichlet test may come first.  Above the bottom of the top PML layer a
    // free surface switches the z stretch off: PFDFD3D when x and y are
    // interior, PML3D evaluated at iz = ipml+1 otherwise.
    if (jz == p.nz || jx == 1 || jx == p.nx || jy == 1 || jy == p.ny) region = REG_FIXED;
    else if (jz <= p.ipml) {
        if (jz == 1 && !p.fst) region = REG_FIXED;
        else if (jz == 1 && !p.usemin) region = REG_TPFREE;
        else if (p.fst) zidx = xyin ? 0 : p.ipml + 1;
    }

    NodeCoefs<R> c;
    Stretch<R> f;
    R m2 = 0, m3 = 0, m4 = 0, dxo8 = 0;
    cx<R> m1(0), r1x(1), r1y(1);
    if (region != REG_FIXED) {
        gather_coefs<R>(da, mu, ro, p.nx, p.ny, p.nz, iz, ix, iy, p.fst != 0, c);
        const cx<R> om((R)p.om_re, (R)p.om_im);
        const cx<R> om2 = om * om;
        m2 = (om2 * c.wm2 / R(6)).re;     // REAL(omegasq*wm2/6): imaginary part dropped (pfdfd3d.f:140-142)
        m3 = (om2 * c.wm3 / R(12)).re;
        m4 = (om2 * c.wm4 / R(8)).re;
        m1 = c.wm1 * om2 * c.ro[13];
        if (region == REG_STENCIL) {
            build_stretch<R>(jx, jy, zidx, p.nx, p.ny, p.nz, p.ipml, (R)p.dx, (R)p.pmld, (R)p.pmlf, c.vpreal, om, f);
        } else {
            cx<R> eyeom = cx<R>(R(0), R(-1)) * om, r2;
            axis_factor<R>(jx, p.nx, p.ipml, (R)p.dx, (R)p.pmld, (R)p.pmlf, c.vpreal, eyeom, r1x, r2);
            axis_factor<R>(jy, p.ny, p.ipml, (R)p.dx, (R)p.pmld, (R)p.pmlf, c.vpreal, eyeom, r1y, r2);
            dxo8 = R(1) / ((R)p.dx * R(8));
        }
    }
    const int len = 3 * __popc(mask);
    OutT *ru = a + irptr[3 * g];
    OutT *rv = ru + len;
    OutT *rw = rv + len;
    emit_all<R, OutT>(std::make_integer_sequence<int, 27>{}, region, c, f, m2, m3, m4, m1, r1x, r1y, dxo8, mask,
                      ru, rv, rw);
}

// ---------------------------------------------------------------------------
// CSR pattern of the 27-point, 3-dof grid graph (srel3d + SPARSE_ADJ2CRS)
// ---------------------------------------------------------------------------
__global__ void k_node_nnz(int nx, int ny, int nz, long long nn, long long *cnt)
{
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nn) return;
    int iz = (int)(g % nz), ix = (int)((g / nz) % nx), iy = (int)(g / ((long long)nz * nx));
    int cz = 1 + (iz > 0) + (iz < nz - 1), cxn = 1 + (ix > 0) + (ix < nx - 1), cy = 1 + (iy > 0) + (iy < ny - 1);
    cnt[g] = 9LL * cz * cxn * cy;
}

__global__ void k_pattern(int nx, int ny, int nz, long long nn, const long long *__restrict__ start, int base,
                          int *__restrict__ irptr, int *__restrict__ jcptr)
{
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nn) return;
    int iz = (int)(g % nz), ix = (int)((g / nz) % nx), iy = (int)(g / ((long long)nz * nx));
    long long s0 = start[g];
    int cz = 1 + (iz > 0) + (iz < nz - 1), cxn = 1 + (ix > 0) + (ix < nx - 1), cy = 1 + (iy > 0) + (iy < ny - 1);
    int len = 3 * cz * cxn * cy;
    for (int r = 0; r < 3; r++) {
        long long rs = s0 + (long long)r * len;
        irptr[3 * g + r] = (int)(rs + base);
        int k = 0;
        for (int dy = -1; dy <= 1; dy++) {
            int y = iy + dy; if (y < 0 || y >= ny) continue;
            for (int dx = -1; dx <= 1; dx++) {
                int x = ix + dx; if (x < 0 || x >= nx) continue;
                for (int dz = -1; dz <= 1; dz++) {
                    int z = iz + dz; if (z < 0 || z >= nz) continue;
                    long long nb = z + (long long)nz * (x + (long long)nx * y);
                    for (int q = 0; q < 3; q++) jcptr[rs + k++] = (int)(3 * nb + q + base);
                }
            }
        }
    }
    if (g == nn - 1) irptr[3 * nn] = (int)(s0 + 3LL * len + base);
}

// ---------------------------------------------------------------------------
// host entry points
// ---------------------------------------------------------------------------
void grid_pml(const wt3d_grid &g, double &pmld, double &pmlf, int &ipml)
{
    pmld = g.pmld > 0 ? g.pmld : 10.0 * g.dx;           // readini.f90:82
    double pmlr = g.pmlr > 0 ? g.pmlr : 1e-3;           // readini.f90:81
    ipml = (int)(pmld / g.dx) + 1;                      // readini.f90:83
    pmlf = 3.0 * std::log(1.0 / pmlr) / (2.0 * pmld * pmld * pmld);   // readini.f90:84
}

int device_pattern(int nx, int ny, int nz, int base, int *d_irptr, int *d_jcptr, cudaStream_t st)
{
    long long nn = (long long)nx * ny * nz;
    long long *cnt = nullptr, *start = nullptr;
    void *tmp = nullptr;
    size_t tmpb = 0;
    WT_CUDA(cudaMallocAsync(&cnt, sizeof(long long) * nn, st));
    WT_CUDA(cudaMallocAsync(&start, sizeof(long long) * nn, st));
    int th = 256;
    k_node_nnz<<<ceil_div(nn, th), th, 0, st>>>(nx, ny, nz, nn, cnt);
    cub::DeviceScan::ExclusiveSum(nullptr, tmpb, cnt, start, nn, st);
    WT_CUDA(cudaMallocAsync(&tmp, tmpb, st));
    cub::DeviceScan::ExclusiveSum(tmp, tmpb, cnt, start, nn, st);
    k_pattern<<<ceil_div(nn, th), th, 0, st>>>(nx, ny, nz, nn, start, base, d_irptr, d_jcptr);
    WT_CUDA(cudaGetLastError());
    WT_CUDA(cudaFreeAsync(tmp, st));
    WT_CUDA(cudaFreeAsync(cnt, st));
    WT_CUDA(cudaFreeAsync(start, st));
    return WT3D_OK;
}

int device_lame(long long nn, const float *d_vp, const float *d_vs, const float *d_rho, void *d_da, void *d_mu,
                double *d_ro, cudaStream_t st)
{
    int th = 256;
    k_lame<<<ceil_div(nn, th), th, 0, st>>>(nn, d_vp, d_vs, d_rho, (cx<double> *)d_da, (cx<double> *)d_mu, d_ro);
    WT_CUDA(cudaGetLastError());
    return WT3D_OK;
}

int device_assemble(const wt3d_grid &g, const void *d_da, const void *d_mu, const double *d_ro, double om_re,
                    double om_im, const int *d_irptr, void *d_a, cudaStream_t st)
{
    AsmParams p;
    p.nx = g.nx; p.ny = g.ny; p.nz = g.nz; p.fst = g.fst; p.usemin = g.usemin; p.dx = g.dx;
    grid_pml(g, p.pmld, p.pmlf, p.ipml);
    p.om_re = om_re; p.om_im = om_im;
    long long nn = (long long)g.nx * g.ny * g.nz;
    int th = 128;
    k_assemble<double, double2><<<ceil_div(nn, th), th, 0, st>>>(p, (const cx<double> *)d_da,
                                                                  (const cx<double> *)d_mu, d_ro, d_irptr,
                                                                  (double2 *)d_a);
    WT_CUDA(cudaGetLastError());
    return WT3D_OK;
}

}  // namespace wt3d
