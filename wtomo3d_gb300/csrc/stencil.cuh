// Device-side stencil of the 27-point elastic operator, shared by the
// assembly kernel and the adjoint-gradient kernel.  See assemble.cu for the
// mapping to the reference routines.
#pragma once
#include "common.cuh"
#include <utility>

namespace wt3d {

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

// Region dispatch of FDFD3D (fdfd3d.f:53-115) for the 0-based node (iz,ix,iy).
// zidx is the z index fed to the stretch factor (0 = z stretch off); mask has
// bit s set for every slot whose neighbour lies inside the grid.
__device__ __forceinline__ void node_region(const AsmParams &p, int iz, int ix, int iy, int &region, int &zidx,
                                            unsigned &mask)
{
    mask = 0;
#pragma unroll
    for (int s = 0; s < 27; s++) {
        int dy = s / 9 - 1, dxo = (s / 3) % 3 - 1, dz = s % 3 - 1;
        bool ok = (iy + dy >= 0) && (iy + dy < p.ny) && (ix + dxo >= 0) && (ix + dxo < p.nx) &&
                  (iz + dz >= 0) && (iz + dz < p.nz);
        mask |= (ok ? 1u : 0u) << s;
    }
    // 1-based indices as the reference uses them
    const int jz = iz + 1, jx = ix + 1, jy = iy + 1;
    const bool xyin = (jx > p.ipml) && (jx <= p.nx - p.ipml) && (jy > p.ipml) && (jy <= p.ny - p.ipml);
    region = REG_STENCIL;
    zidx = jz;
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
}

}  // namespace wt3d
