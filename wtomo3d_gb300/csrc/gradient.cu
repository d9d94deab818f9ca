// Adjoint-state waveform-tomography gradient on sm_103a.
//
// For an operator A(m) with A u_j = b_j (b independent of the model: point
// forces, or A_bg u0 for the total field of a plane wave) and a misfit
// chi = 1/2 sum |R u_j - d_j|^2, the gradient with respect to a real model
// parameter m is
//     dchi/dm = -Re sum_j lam_j^H (dA/dm) u_j,    A^H lam_j = R^T (R u_j - d_j).
// The reference has no gradient code on this path; the operator it
// differentiates is the one ASMBLE builds (asmble.f90:96-601 over
// setcoefs3d.f:79-233, calcwts.f:1-75, pfdfd3d.f:137-576, pml3d.f:167-800,
// tpfree.f:57-427), from the Lame arrays of modelio.f90:78-92.
//
// Two kernels, no atomics (the result does not depend on scheduling):
//
//  k_grad_rows, one thread per operator row node n.  Row n depends on the
//  model only through its coefficient set: the eight octant-cell means of mu
//  and lambda, the 27 densities, the mass-lumping weights wm(vp/vs) of the
//  centre node and, inside the PML, the centre node's vp (vpreal).  The row's
//  contribution c_n = sum_s <B_s, G_s>, G_s = sum_j conj(lam_j,n) (x) u_j,n+s,
//  is linear in the cell means and densities at fixed weights and stretch,
//  so its derivative with respect to cell mean q is the row evaluated with a
//  unit coefficient set (only the slots whose neighbour lies in cell q are
//  evaluated).  The weight and vpreal derivatives follow from calcwts' cubic
//  polynomials and from r1 = e/(e+d), r2 = 2 isn r1^3 dp vpreal pmlf / e.
//  Only real parts are kept: every later factor is real.
//
//  k_grad_nodes, one thread per node g: gathers from the 27 rows whose
//  coefficient sets contain g (1/8 per cell mean that contains g, its density
//  position, and the centre terms of its own row) and applies the chain rule
//  mu = Vs^2 rho, lambda = Vp^2 rho - 2 mu.
#include "common.cuh"
#include "wtomo3d_gpu.h"
#include "internal.h"
#include "stencil.cuh"

namespace wt3d {

// per-row derivative record, stored as D[k * nn + n]
constexpr int GD_U = 0;     // 8: d c_n / d (cell mean of mu, cells 1..8)
constexpr int GD_DA = 8;    // 8: d c_n / d (cell mean of lambda)
constexpr int GD_RO = 16;   // 27: d c_n / d (density at the neighbour of slot s)
constexpr int GD_X = 43;    // d c_n / d (vp/vs of the centre node), through calcwts
constexpr int GD_VP = 44;   // d c_n / d (vpreal of the centre node), through the PML stretch
constexpr int GD_N = 45;

// Octant cells (bit q, q = 1..8) that contain the neighbour at slot s.  Cells
// 1..4 are the upper (z-) octants, 5..8 the lower; within each, the x-/y-
// quadrants are ordered (x-,y-), (x-,y+), (x+,y-), (x+,y+) (setcoefs3d.f:108-174).
__host__ __device__ constexpr unsigned slot_cells(int s)
{
    const int dy = s / 9 - 1, dx = (s / 3) % 3 - 1, dz = s % 3 - 1;
    unsigned m = 0;
    for (int q = 1; q <= 8; q++) {
        const int quad = (q - 1) & 3;
        const bool xin = quad < 2 ? dx <= 0 : dx >= 0;
        const bool yin = (quad & 1) == 0 ? dy <= 0 : dy >= 0;
        const bool zin = q > 4 ? dz >= 0 : dz <= 0;
        if (xin && yin && zin) m |= 1u << q;
    }
    return m;
}

// Index of the density of slot s's neighbour in NodeCoefs::ro.
__host__ __device__ constexpr int slot_ro(int s)
{
    return ((s / 3) % 3) + 3 * (s / 9) + 9 * (s % 3);
}

// Unit coefficient set: mu (kind 0) or lambda (kind 1) mean of cell q equal to
// one, everything else zero.  lmu/lpu/lp2u follow setcoefs3d.f:196-221.
__device__ __forceinline__ void unit_coefs(int q, int kind, NodeCoefs<double> &c)
{
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const bool on = k == q;
        c.u[k] = cx<double>(on && kind == 0 ? 1.0 : 0.0);
        c.da[k] = cx<double>(on && kind == 1 ? 1.0 : 0.0);
        c.lmu[k] = cx<double>(on ? (kind == 0 ? -1.0 : 1.0) : 0.0);
        c.lpu[k] = cx<double>(on ? 1.0 : 0.0);
        c.lp2u[k] = cx<double>(on ? (kind == 0 ? 2.0 : 1.0) : 0.0);
    }
#pragma unroll
    for (int k = 0; k < 27; k++) c.ro[k] = 0.0;
    c.wm1 = c.wm2 = c.wm3 = c.wm4 = 0.0;
    c.vpreal = 0.0;
}

__device__ __forceinline__ double re_dot9(const cx<double> *b, const cx<double> *G)
{
    double s = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) s += b[k].re * G[k].re - b[k].im * G[k].im;
    return s;
}

// G[3a+b] = sum_j conj(lam_j[3n+a]) u_j[3 nb + b]
__device__ __forceinline__ void outer_sum(const double2 *__restrict__ U, const double2 *__restrict__ L, long long ld,
                                          int m, long long n, long long nb, cx<double> *G)
{
#pragma unroll
    for (int k = 0; k < 9; k++) G[k] = cx<double>(0);
    for (int j = 0; j < m; j++) {
        const double2 *lj = L + (long long)j * ld + 3 * n;
        const double2 *uj = U + (long long)j * ld + 3 * nb;
        cx<double> l[3], u[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double2 x = __ldg(lj + a), y = __ldg(uj + a);
            l[a] = cx<double>(x.x, -x.y);
            u[a] = cx<double>(y.x, y.y);
        }
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) G[3 * a + b] = G[3 * a + b] + l[a] * u[b];
    }
}

// d(wm1..wm4)/dx of CALCWTS (calcwts.f:31-71), following the clamping branch taken.
__device__ __forceinline__ void calcwts_dx(double x, double *dw)
{
    double w1 = 0.2909366 + x * (-0.1792402e-01 + x * (0.7329184e-02 + x * -0.1055034e-02));
    double d1 = -0.1792402e-01 + x * (2 * 0.7329184e-02 + x * 3 * -0.1055034e-02);
    double w2 = 0, w3 = 0, d2 = 0, d3 = 0;
    if (w1 > 1.0) { w1 = 1.0; d1 = 0; }
    else {
        w2 = 0.6367377 + x * (-0.7982022e-02 + x * (0.3385164e-02 + x * -0.5065399e-03));
        d2 = -0.7982022e-02 + x * (2 * 0.3385164e-02 + x * 3 * -0.5065399e-03);
    }
    if (w1 + w2 > 1.0) { w2 = 0.0; d2 = 0; }
    else {
        w3 = 0.07244875 + x * (0.2569959e-01 + x * (-0.1060011e-01 + x * 0.1540534e-02));
        d3 = 0.2569959e-01 + x * (2 * -0.1060011e-01 + x * 3 * 0.1540534e-02);
    }
    if (w1 + w2 + w3 > 1.0) d3 = -(d1 + d2);
    dw[0] = d1; dw[1] = d2; dw[2] = d3; dw[3] = -(d1 + d2 + d3);
}

// d r1 / d vpreal and d r2 / d vpreal of one axis (pml3d.f:273-295 differentiated).
__device__ __forceinline__ void axis_factor_d(int idx, int n, int ipml, double dx, double pmld, double pmlf,
                                              double vpreal, cx<double> eyeom, cx<double> &r1, cx<double> &dr1,
                                              cx<double> &dr2)
{
    double dp = 0; int isn = 0;
    if (idx > 0) {
        if (idx <= ipml) { dp = pmld - double(idx - 1) * dx; isn = 1; }
        else if (n - idx + 1 <= ipml) { dp = pmld - double(n - idx) * dx; isn = -1; }
    }
    if (isn == 0) { r1 = cx<double>(1); dr1 = cx<double>(0); dr2 = cx<double>(0); return; }
    const cx<double> dn(dp * dp * vpreal * pmlf, 0.0);
    r1 = eyeom / (eyeom + dn);
    const cx<double> t = eyeom / (eyeom * eyeom);
    dr1 = -((r1 * r1) * t) * (dp * dp * pmlf);
    const cx<double> r1sq = r1 * r1;
    dr2 = (double(isn) * 2.0 * dp * pmlf) * t * (3.0 * vpreal * (r1sq * dr1) + r1sq * r1);
}

// ---------------------------------------------------------------------------
// pass 0: cell-mean, density and weight derivatives of each row
// ---------------------------------------------------------------------------
template <int S>
__device__ __forceinline__ void rows_slot(int region, unsigned mask, const Stretch<double> &f, cx<double> r1x,
                                          cx<double> r1y, double dxo8, const NodeCoefs<double> &c, cx<double> om2,
                                          double m2, double m3, double m4, const double2 *U, const double2 *L,
                                          long long ld, int m, long long n, int nz, int nx, double *du, double *dd,
                                          double *dwm, double *D, long long nn)
{
    if (!((mask >> S) & 1u)) {
        D[(long long)(GD_RO + S) * nn + n] = 0.0;
        return;
    }
    constexpr int dy = S / 9 - 1, dxo = (S / 3) % 3 - 1, dz = S % 3 - 1;
    const long long nb = n + dz + (long long)nz * (dxo + (long long)nx * dy);
    cx<double> G[9];
    outer_sum(U, L, ld, m, n, nb, G);
    constexpr unsigned cm = slot_cells(S);
#pragma unroll
    for (int q = 1; q <= 8; q++) {
        if (!((cm >> q) & 1u)) continue;
#pragma unroll
        for (int kind = 0; kind < 2; kind++) {
            NodeCoefs<double> cu;
            unit_coefs(q, kind, cu);
            cx<double> b[9];
            if (region == REG_STENCIL) stencil_block<S, double>(cu, f, 0.0, 0.0, 0.0, cx<double>(0), b);
            else tpfree_block<S, double>(cu, r1x, r1y, dxo8, b);
            const double v = re_dot9(b, G);
            if (kind == 0) du[q - 1] += v;
            else dd[q - 1] += v;
        }
    }
    double dro = 0.0;
    if (region == REG_STENCIL) {
        const cx<double> tr = G[0] + G[4] + G[8];
        constexpr int nzo = (dy != 0) + (dxo != 0) + (dz != 0);
        if constexpr (nzo == 0) {
            // centre mass wm1 * omega^2 * rho (pfdfd3d.f:362)
            dro = (c.wm1 * om2 * tr).re;
            dwm[0] += (om2 * c.ro[13] * tr).re;
        } else {
            // REAL(omega^2 wm/k) * rho on the diagonal (pfdfd3d.f:140-142)
            constexpr double k = nzo == 1 ? 6.0 : (nzo == 2 ? 12.0 : 8.0);
            const double mcoef = nzo == 1 ? m2 : (nzo == 2 ? m3 : m4);
            dro = mcoef * tr.re;
            dwm[nzo] += (om2.re / k) * c.ro[slot_ro(S)] * tr.re;
        }
    }
    D[(long long)(GD_RO + S) * nn + n] = dro;
}

template <int... Ss>
__device__ __forceinline__ void rows_all(std::integer_sequence<int, Ss...>, int region, unsigned mask,
                                         const Stretch<double> &f, cx<double> r1x, cx<double> r1y, double dxo8,
                                         const NodeCoefs<double> &c, cx<double> om2, double m2, double m3, double m4,
                                         const double2 *U, const double2 *L, long long ld, int m, long long n, int nz,
                                         int nx, double *du, double *dd, double *dwm, double *D, long long nn)
{
    (rows_slot<Ss>(region, mask, f, r1x, r1y, dxo8, c, om2, m2, m3, m4, U, L, ld, m, n, nz, nx, du, dd, dwm, D, nn),
     ...);
}

__global__ void __launch_bounds__(128) k_grad_rows(AsmParams p, const cx<double> *__restrict__ da,
                                                   const cx<double> *__restrict__ mu, const double *__restrict__ ro,
                                                   int m, long long ld, const double2 *__restrict__ U,
                                                   const double2 *__restrict__ L, double *__restrict__ D)
{
    const long long nn = (long long)p.nx * p.ny * p.nz;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int iz = (int)(n % p.nz);
    const int ix = (int)((n / p.nz) % p.nx);
    const int iy = (int)(n / ((long long)p.nz * p.nx));
    unsigned mask;
    int region, zidx;
    node_region(p, iz, ix, iy, region, zidx, mask);
    if (region == REG_FIXED) {
        for (int k = 0; k < GD_VP; k++) D[(long long)k * nn + n] = 0.0;
        return;
    }
    NodeCoefs<double> c;
    gather_coefs<double>(da, mu, ro, p.nx, p.ny, p.nz, iz, ix, iy, p.fst != 0, c);
    const cx<double> om(p.om_re, p.om_im);
    const cx<double> om2 = om * om;
    const double m2 = (om2 * c.wm2 / 6.0).re, m3 = (om2 * c.wm3 / 12.0).re, m4 = (om2 * c.wm4 / 8.0).re;
    Stretch<double> f;
    cx<double> r1x(1), r1y(1);
    double dxo8 = 0;
    if (region == REG_STENCIL) {
        build_stretch<double>(ix + 1, iy + 1, zidx, p.nx, p.ny, p.nz, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, om, f);
    } else {
        const cx<double> eyeom = cx<double>(0.0, -1.0) * om;
        cx<double> r2;
        axis_factor<double>(ix + 1, p.nx, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, eyeom, r1x, r2);
        axis_factor<double>(iy + 1, p.ny, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, eyeom, r1y, r2);
        dxo8 = 1.0 / (p.dx * 8.0);
    }
    double du[8], dd[8], dwm[4];
#pragma unroll
    for (int k = 0; k < 8; k++) du[k] = dd[k] = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++) dwm[k] = 0.0;
    // dwm index: 0 = wm1 (centre), 1 = wm2 (faces), 2 = wm3 (edges), 3 = wm4 (corners)
    rows_all(std::make_integer_sequence<int, 27>{}, region, mask, f, r1x, r1y, dxo8, c, om2, m2, m3, m4, U, L, ld,
             m, n, p.nz, p.nx, du, dd, dwm, D, nn);
    // a free surface on top zeroes the upper cell means (setcoefs3d.f:177-192):
    // they no longer depend on the model
    if (p.fst && iz == 0) {
#pragma unroll
        for (int k = 0; k < 4; k++) du[k] = dd[k] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
        D[(long long)(GD_U + k) * nn + n] = du[k];
        D[(long long)(GD_DA + k) * nn + n] = dd[k];
    }
    double dxr = 0.0;
    if (region == REG_STENCIL) {
        const double vs = csqrt_(mu[n] / ro[n]).re;
        double dw[4];
        calcwts_dx((double)c.vpreal / vs, dw);
        dxr = dwm[0] * dw[0] + dwm[1] * dw[1] + dwm[2] * dw[2] + dwm[3] * dw[3];
    }
    D[(long long)GD_X * nn + n] = dxr;
}

// ---------------------------------------------------------------------------
// pass 1: vpreal derivative of the PML rows
// ---------------------------------------------------------------------------
template <int S>
__device__ __forceinline__ void vp_slot(int region, unsigned mask, const NodeCoefs<double> &c,
                                        const Stretch<double> &fd, cx<double> dr1x, cx<double> dr1y, double dxo8,
                                        const double2 *U, const double2 *L, long long ld, int m, long long n, int nz,
                                        int nx, double &acc)
{
    if (!((mask >> S) & 1u)) return;
    constexpr int dy = S / 9 - 1, dxo = (S / 3) % 3 - 1, dz = S % 3 - 1;
    const long long nb = n + dz + (long long)nz * (dxo + (long long)nx * dy);
    cx<double> G[9], b[9];
    if (region == REG_STENCIL) {
        outer_sum(U, L, ld, m, n, nb, G);
        stencil_block<S, double>(c, fd, 0.0, 0.0, 0.0, cx<double>(0), b);   // linear in the stretch
        acc += re_dot9(b, G);
    } else {
        if constexpr (S != 2 && S != 20 && S != 8 && S != 26 && S != 13) return;   // zero TPFREE blocks
        outer_sum(U, L, ld, m, n, nb, G);
        // TPFREE blocks are affine in (r1x, r1y)
        cx<double> b0[9], bx[9], by[9];
        tpfree_block<S, double>(c, cx<double>(0), cx<double>(0), dxo8, b0);
        tpfree_block<S, double>(c, cx<double>(1), cx<double>(0), dxo8, bx);
        tpfree_block<S, double>(c, cx<double>(0), cx<double>(1), dxo8, by);
#pragma unroll
        for (int k = 0; k < 9; k++) b[k] = dr1x * (bx[k] - b0[k]) + dr1y * (by[k] - b0[k]);
        acc += re_dot9(b, G);
    }
}

template <int... Ss>
__device__ __forceinline__ void vp_all(std::integer_sequence<int, Ss...>, int region, unsigned mask,
                                       const NodeCoefs<double> &c, const Stretch<double> &fd, cx<double> dr1x,
                                       cx<double> dr1y, double dxo8, const double2 *U, const double2 *L, long long ld,
                                       int m, long long n, int nz, int nx, double &acc)
{
    (vp_slot<Ss>(region, mask, c, fd, dr1x, dr1y, dxo8, U, L, ld, m, n, nz, nx, acc), ...);
}

__global__ void __launch_bounds__(128) k_grad_vpreal(AsmParams p, const cx<double> *__restrict__ da,
                                                     const cx<double> *__restrict__ mu,
                                                     const double *__restrict__ ro, int m, long long ld,
                                                     const double2 *__restrict__ U, const double2 *__restrict__ L,
                                                     double *__restrict__ D)
{
    const long long nn = (long long)p.nx * p.ny * p.nz;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nn) return;
    const int iz = (int)(n % p.nz);
    const int ix = (int)((n / p.nz) % p.nx);
    const int iy = (int)(n / ((long long)p.nz * p.nx));
    unsigned mask;
    int region, zidx;
    node_region(p, iz, ix, iy, region, zidx, mask);
    double acc = 0.0;
    const int jx = ix + 1, jy = iy + 1;
    const bool in_pml = jx <= p.ipml || p.nx - jx + 1 <= p.ipml || jy <= p.ipml || p.ny - jy + 1 <= p.ipml ||
                        (zidx > 0 && (zidx <= p.ipml || p.nz - zidx + 1 <= p.ipml));
    if (region != REG_FIXED && in_pml) {
        NodeCoefs<double> c;
        gather_coefs<double>(da, mu, ro, p.nx, p.ny, p.nz, iz, ix, iy, p.fst != 0, c);
        const cx<double> om(p.om_re, p.om_im);
        const cx<double> eyeom = cx<double>(0.0, -1.0) * om;
        cx<double> r1x, r1y, r1z, d1x, d1y, d1z, d2x, d2y, d2z;
        axis_factor_d(jx, p.nx, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, eyeom, r1x, d1x, d2x);
        axis_factor_d(jy, p.ny, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, eyeom, r1y, d1y, d2y);
        Stretch<double> fd;
        double dxo8 = 0;
        if (region == REG_STENCIL) {
            axis_factor_d(zidx, p.nz, p.ipml, p.dx, p.pmld, p.pmlf, c.vpreal, eyeom, r1z, d1z, d2z);
            // derivative of build_stretch's scaled combinations
            const double dxx = p.dx * p.dx;
            fd.X2 = (2.0 * r1x * d1x) / (8.0 * dxx);
            fd.Y2 = (2.0 * r1y * d1y) / (8.0 * dxx);
            fd.Z2 = (2.0 * r1z * d1z) / (8.0 * dxx);
            fd.XY = (d1x * r1y + r1x * d1y) / (16.0 * dxx);
            fd.XZ = (d1x * r1z + r1x * d1z) / (16.0 * dxx);
            fd.YZ = (d1y * r1z + r1y * d1z) / (16.0 * dxx);
            fd.rx = d2x / (8.0 * p.dx);
            fd.ry = d2y / (8.0 * p.dx);
            fd.rz = d2z / (8.0 * p.dx);
        } else {
            dxo8 = 1.0 / (p.dx * 8.0);
        }
        vp_all(std::make_integer_sequence<int, 27>{}, region, mask, c, fd, d1x, d1y, dxo8, U, L, ld, m, n, p.nz,
               p.nx, acc);
    }
    D[(long long)GD_VP * nn + n] = acc;
}

// ---------------------------------------------------------------------------
// pass 2: gather per node and chain rule to (Vp, Vs, rho)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_grad_nodes(int nx, int ny, int nz, const cx<double> *__restrict__ da,
                                                    const cx<double> *__restrict__ mu,
                                                    const double *__restrict__ ro, const float *__restrict__ vp,
                                                    const float *__restrict__ vs, const float *__restrict__ rho,
                                                    const double *__restrict__ D, double *__restrict__ grad)
{
    const long long nn = (long long)nx * ny * nz;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nn) return;
    const int iz = (int)(g % nz);
    const int ix = (int)((g / nz) % nx);
    const int iy = (int)(g / ((long long)nz * nx));
    double gl = 0, gm = 0, gr = 0;
    for (int s = 0; s < 27; s++) {
        // g sits at offset s of row node r = g - offset
        const int dy = s / 9 - 1, dx = (s / 3) % 3 - 1, dz = s % 3 - 1;
        const int ry = iy - dy, rx = ix - dx, rz = iz - dz;
        if (ry < 0 || ry >= ny || rx < 0 || rx >= nx || rz < 0 || rz >= nz) continue;
        const long long r = rz + (long long)nz * (rx + (long long)nx * ry);
        const unsigned cm = slot_cells(s);
        double su = 0, sd = 0;
        for (int q = 1; q <= 8; q++) {
            if (!((cm >> q) & 1u)) continue;
            su += D[(long long)(GD_U + q - 1) * nn + r];
            sd += D[(long long)(GD_DA + q - 1) * nn + r];
        }
        gm += su * 0.125;
        gl += sd * 0.125;
        gr += D[(long long)(GD_RO + s) * nn + r];
    }
    // centre terms of row g: weights wm(vp/vs) and vpreal (setcoefs3d.f:224-226, pml3d.f:201-204)
    const double Dx = D[(long long)GD_X * nn + g], Dv = D[(long long)GD_VP * nn + g];
    if (Dx != 0.0 || Dv != 0.0) {
        const double r0 = ro[g];
        const cx<double> sp = csqrt_((da[g] + 2.0 * mu[g]) / r0);
        const cx<double> ss = csqrt_(mu[g] / r0);
        const double pv = sp.re, sv = ss.re;
        const double dvp_dl = (cx<double>(1.0) / (2.0 * r0 * sp)).re;
        const double dvp_dm = (cx<double>(1.0) / (r0 * sp)).re;
        const double dvp_dr = (-(sp / (2.0 * r0))).re;
        const double dvs_dm = (cx<double>(1.0) / (2.0 * r0 * ss)).re;
        const double dvs_dr = (-(ss / (2.0 * r0))).re;
        const double dx_dl = dvp_dl / sv;
        const double dx_dm = dvp_dm / sv - pv * dvs_dm / (sv * sv);
        const double dx_dr = dvp_dr / sv - pv * dvs_dr / (sv * sv);
        gl += Dx * dx_dl + Dv * dvp_dl;
        gm += Dx * dx_dm + Dv * dvp_dm;
        gr += Dx * dx_dr + Dv * dvp_dr;
    }
    // dchi/dm = -Re sum lam^H dA/dm u
    gl = -gl; gm = -gm; gr = -gr;
    const double P = vp[g], Sv = vs[g], Rh = rho[g];
    grad[g] = 2.0 * P * Rh * gl;
    grad[nn + g] = 2.0 * Sv * Rh * gm - 4.0 * Sv * Rh * gl;
    grad[2 * nn + g] = (P * P - 2.0 * Sv * Sv) * gl + Sv * Sv * gm + gr;
}

// ---------------------------------------------------------------------------
// receivers: predicted data, residual and adjoint source
// ---------------------------------------------------------------------------
__global__ void k_add_cm(long long total, const double2 *__restrict__ a, double2 *__restrict__ y)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    double2 v = y[i], w = a[i];
    y[i] = make_double2(v.x + w.x, v.y + w.y);
}

// res[(j*nrec + r)*3 + c] = U_j[3 rec_r + c] - dobs[...]; S_j[3 rec_r + c] += res
__global__ void k_receivers(int m, int nrec, long long ld, const long long *__restrict__ rec,
                            const double2 *__restrict__ U, const double2 *__restrict__ dobs,
                            double2 *__restrict__ pred, double2 *__restrict__ res, double2 *__restrict__ S)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)m * nrec * 3) return;
    const int c = (int)(i % 3);
    const int r = (int)((i / 3) % nrec);
    const int j = (int)(i / (3LL * nrec));
    const long long idx = (long long)j * ld + 3 * rec[r] + c;
    const double2 u = U[idx], d = dobs[i];
    const double2 e = make_double2(u.x - d.x, u.y - d.y);
    pred[i] = u;
    res[i] = e;
    atomicAdd(&S[idx].x, e.x);
    atomicAdd(&S[idx].y, e.y);
}

int device_gradient(const wt3d_grid &g, const void *d_da, const void *d_mu, const double *d_ro, const float *d_vp,
                    const float *d_vs, const float *d_rho, double om_re, double om_im, int m, long long ld,
                    const void *d_U, const void *d_L, double *d_D, double *d_grad, cudaStream_t st)
{
    AsmParams p;
    p.nx = g.nx; p.ny = g.ny; p.nz = g.nz; p.fst = g.fst; p.usemin = g.usemin; p.dx = g.dx;
    grid_pml(g, p.pmld, p.pmlf, p.ipml);
    p.om_re = om_re; p.om_im = om_im;
    const long long nn = (long long)g.nx * g.ny * g.nz;
    const auto *da = (const cx<double> *)d_da;
    const auto *mu = (const cx<double> *)d_mu;
    const auto *U = (const double2 *)d_U;
    const auto *L = (const double2 *)d_L;
    k_grad_rows<<<ceil_div(nn, 128), 128, 0, st>>>(p, da, mu, d_ro, m, ld, U, L, d_D);
    k_grad_vpreal<<<ceil_div(nn, 128), 128, 0, st>>>(p, da, mu, d_ro, m, ld, U, L, d_D);
    k_grad_nodes<<<ceil_div(nn, 256), 256, 0, st>>>(g.nx, g.ny, g.nz, da, mu, d_ro, d_vp, d_vs, d_rho, d_D, d_grad);
    WT_CUDA(cudaGetLastError());
    return WT3D_OK;
}

long long gradient_scratch_doubles(long long nn) { return (long long)GD_N * nn; }

int device_receivers(int m, int nrec, long long ld, const long long *d_rec, const void *d_U, const void *d_dobs,
                     void *d_pred, void *d_res, void *d_S, cudaStream_t st)
{
    const long long tot = (long long)m * nrec * 3;
    if (tot == 0) return WT3D_OK;
    k_receivers<<<ceil_div(tot, 256), 256, 0, st>>>(m, nrec, ld, d_rec, (const double2 *)d_U,
                                                    (const double2 *)d_dobs, (double2 *)d_pred, (double2 *)d_res,
                                                    (double2 *)d_S);
    WT_CUDA(cudaGetLastError());
    return WT3D_OK;
}

int device_add(long long total, const void *d_a, void *d_y, cudaStream_t st)
{
    k_add_cm<<<ceil_div(total, 256), 256, 0, st>>>(total, (const double2 *)d_a, (double2 *)d_y);
    WT_CUDA(cudaGetLastError());
    return WT3D_OK;
}

}  // namespace wt3d
