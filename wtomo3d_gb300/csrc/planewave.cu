// Haskell plane-wave right-hand sides.
//
//   * haskgrn (host, FP64): Thomson-Haskell response U(z), W(z) of a layered
//     1-D medium to a unit incident P or S plane wave (haskgrn.f:31-672).
//   * k_pw_expand (device): the incident field on the 3-D grid,
//         u0 = [U*(z) rx, U*(z) ry, W*(z)] exp(i omega p (x rx + y ry)),
//     with (rx, ry) = -(cos baz, sin baz) the horizontal propagation
//     direction of a wave arriving from back-azimuth baz and p = 1/cv the
//     horizontal slowness used by haskgrn.  The operator uses plane waves
//     exp(i(kx - omega t)) while Haskell's response is for the reverse sign,
//     so the background is conjugated (dispersion.f:17-22).  The reference's
//     own expansion (planewvexp.f90) is not in the tree; this is the
//     definition used here.
//   * k_hetfld (device): the scattered-field source f = (A_bg - A) u0 of
//     hetfldsrc.f90:55-1028 as a row-wise product with the two assembled
//     operators, times the source spectrum (1 for srcin = 3, srcsub.f:249-257).
//     Rows are indexed by the true node number g = iz + nz(ix-1) + nx nz(iy-1);
//     the reference's hetfldsrc.f90:1020 strides iy by nx*ny instead of nx*nz.
#include "devvec.cuh"
#include "wtomo3d_gpu.h"
#include <cmath>
#include <complex>
#include <vector>

namespace wt3d {

namespace {

struct HLayer {
    double r1, r2, gam, gam1, mu_c2, gam2, gam12;   // r_alpha, r_beta, gamma, gamma-1, rho cv^2, gamma^2, (gamma-1)^2
    double e1, e2, ca, sa, cb, sb;                    // cos/sin (or cosh/sinh) of P_m, Q_m and their type
};

// cos/sin of P_m = k h r_alpha (real r) or cosh/sinh (imaginary r), H53.
void phase_terms(double hc, double r1, double r2, bool p_real, bool s_real, HLayer &L)
{
    const double za = hc * r1, zb = hc * r2;
    if (p_real) { L.e1 = 1; L.ca = std::cos(za); L.sa = std::sin(za); }
    else { const double x = std::exp(za); L.e1 = -1; L.ca = 0.5 * (x + 1. / x); L.sa = 0.5 * (x - 1. / x); }
    if (s_real) { L.e2 = 1; L.cb = std::cos(zb); L.sb = std::sin(zb); }
    else { const double x = std::exp(zb); L.e2 = -1; L.cb = 0.5 * (x + 1. / x); L.sb = 0.5 * (x - 1. / x); }
}

// First two columns of the layer-matrix product a_top ... a_1 (surface to the
// bottom of layer `top`), real/imaginary alternation of H53 p.23.
void layer_product(const std::vector<HLayer> &Ls, const double *vs, int top, double B[4][2])
{
    double b[4][2] = {{1, 0}, {0, 1}, {0, 0}, {0, 0}};
    for (int m = 0; m < top; m++) {
        const HLayer &L = Ls[m];
        const double pd = L.sa / L.r1, qd = L.sb / L.r2, pm = L.e1 * L.sa * L.r1, qm = L.e2 * L.sb * L.r2;
        const double cp = L.ca, cq = L.cb, tm = L.mu_c2, g = L.gam, g1 = L.gam1;
        double a[4][4] = {};
        if (vs[m] != 0.0) {
            a[0][0] = g * cp - g1 * cq;  a[0][1] = g1 * pd + g * qm;  a[0][2] = (cq - cp) / tm;  a[0][3] = (pd + qm) / tm;
            a[1][0] = -g * pm - g1 * qd; a[1][1] = g * cq - g1 * cp;  a[1][2] = (pm + qd) / tm;  a[1][3] = a[0][2];
            a[2][0] = tm * g * g1 * (cp - cq); a[2][1] = tm * (L.gam12 * pd + L.gam2 * qm); a[2][2] = a[1][1];
            a[2][3] = a[0][1];
            a[3][0] = tm * (L.gam2 * pm + L.gam12 * qd); a[3][1] = a[2][0]; a[3][2] = a[1][0]; a[3][3] = a[0][0];
        } else {   // fluid layer, H53 eq. 6.3
            a[0][1] = -pd; a[0][2] = -cp / tm; a[1][1] = cp; a[1][2] = pm / tm; a[2][1] = tm * pd; a[2][2] = cp;
        }
        // entries alternate real/imaginary (R I R I / I R I R), so products of
        // two imaginary parts change sign: even rows flip the odd terms of
        // column 0, odd rows flip the even terms of column 1
        const double flip_odd[4] = {1, -1, 1, -1}, none[4] = {1, 1, 1, 1}, flip_even[4] = {-1, 1, -1, 1};
        double d[4][2];
        for (int i = 0; i < 4; i++) {
            const bool even = (i % 2) == 0;
            const double *sg0 = even ? flip_odd : none, *sg1 = even ? none : flip_even;
            double c0 = 0, c1 = 0;
            for (int j = 0; j < 4; j++) {
                c0 += sg0[j] * a[i][j] * b[j][0];
                c1 += sg1[j] * a[i][j] * b[j][1];
            }
            d[i][0] = c0;
            d[i][1] = c1;
        }
        for (int i = 0; i < 4; i++) { b[i][0] = d[i][0]; b[i][1] = d[i][1]; }
    }
    for (int i = 0; i < 4; i++) { B[i][0] = b[i][0]; B[i][1] = b[i][1]; }
}

}  // namespace

int haskgrn_host(const wt3d_layered1d &M, double omega, double ain, int s_wave, int nz, double dz, double zorig,
                 std::complex<double> *U, std::complex<double> *W)
{
    const int nl = M.nl;
    if (nl < 2 || !M.vp || !M.vs || !M.rho || !M.ztop || !(std::sin(ain) > 0)) {
        set_error("haskgrn: need nl >= 2 layers and 0 < incidence");
        return WT3D_ERR_ARG;
    }
    const double *vp = M.vp, *vs = M.vs, *rh = M.rho, *zt = M.ztop;
    const double cv = (s_wave ? vs[nl - 1] : vp[nl - 1]) / std::sin(ain);   // apparent horizontal speed
    const double k = omega / cv;                                               // horizontal wavenumber
    std::vector<HLayer> Ls(nl);
    std::vector<double> h(nl, 0.0);
    for (int i = 0; i + 1 < nl; i++) h[i] = zt[i + 1] - zt[i];
    for (int m = 0; m < nl; m++) {
        HLayer &L = Ls[m];
        const double ca = cv / vp[m], cb = vs[m] != 0.0 ? cv / vs[m] : 1.0;
        double x = ca * ca - 1.;
        L.r1 = std::copysign(std::sqrt(std::fabs(x)), x);
        x = cb * cb - 1.;
        L.r2 = std::copysign(std::sqrt(std::fabs(x)), x);
        L.gam = 2. / (cb * cb);
        L.gam1 = L.gam - 1.;
        if (m + 1 < nl) {
            L.mu_c2 = rh[m] * cv * cv;
            L.gam2 = L.gam * L.gam;
            L.gam12 = L.gam1 * L.gam1;
            phase_terms(k * h[m], L.r1, L.r2, cv > vp[m], cv > vs[m], L);
        }
    }
    // half-space inverse E (rows scaled by -alpha^2 and -2 beta^2, H53 eq. 2.16)
    const HLayer &H = Ls[nl - 1];
    double x = -H.gam1 * cv * cv;
    const double e11 = 2. * vs[nl - 1] * vs[nl - 1], e13 = -1. / rh[nl - 1];
    const double e22 = x / H.r1, e24 = e13 / H.r1, e31 = x / H.r2, e33 = -e13 / H.r2, e42 = -e11, e44 = e13;
    double b[4][2];
    layer_product(Ls, vs, nl - 1, b);
    const double s1 = -1. / (vp[nl - 1] * vp[nl - 1]), s2 = -1. / (2.0 * vs[nl - 1] * vs[nl - 1]);
    const double c11 = s1 * (e11 * b[0][0] + e13 * b[2][0]), c12 = s1 * (e11 * b[0][1] + e13 * b[2][1]);
    const double c21 = s1 * (e22 * b[1][0] + e24 * b[3][0]), c22 = s1 * (e22 * b[1][1] + e24 * b[3][1]);
    const double c31 = s2 * (e31 * b[0][0] + e33 * b[2][0]), c32 = s2 * (e31 * b[0][1] + e33 * b[2][1]);
    const double c41 = s2 * (e42 * b[1][0] + e44 * b[3][0]), c42 = s2 * (e42 * b[1][1] + e44 * b[3][1]);
    // D of H62 eq. 7 and the free-surface displacements (eqs. 5-6)
    const double dr = -c11 * c42 + c21 * c32 + c31 * c22 - c41 * c12;
    const double di = c11 * c32 + c21 * c42 - c31 * c12 - c41 * c22;
    const double dd = dr * dr + di * di;
    double ur, ui, wr, wi;
    if (!s_wave) {
        const double t = 2. * cv / (vp[nl - 1] * dd);
        wr = t * (c31 * dr - c41 * di); wi = t * (-c31 * di - c41 * dr);
        ur = t * (c42 * dr - c32 * di); ui = t * (-c42 * di - c32 * dr);
    } else {
        const double t = cv / (vs[nl - 1] * dd);
        wr = t * (-c11 * dr + c21 * di); wi = t * (c11 * di + c21 * dr);
        ur = t * (-c22 * dr + c12 * di); ui = t * (c22 * di + c12 * dr);
    }
    const double su_r = ur, su_i = ui, sw_r = wr, sw_i = wi;
    U[0] = {su_r, su_i};
    W[0] = {sw_r, sw_i};
    // downward propagation to every node depth
    int last_layer = 1, done = 0;
    int stale = nl;   // layer index the reference's refresh test reads (haskgrn.f:454,466)
    for (int iz = 2; iz <= nz; iz++) {
        const double dep = dz * (iz - 1) + zorig;
        int i = 2;
        while (i <= nl && !(dep < zt[i - 1])) i++;
        if (i > nl) i = nl;     // below the last interface: stays in layer nl-1
        const int lay = i - 1;
        const double dl = dep - zt[i - 2];
        if (dl < 0.) { set_error("haskgrn: node above the model top"); return WT3D_ERR_ARG; }
        if (lay != last_layer) {
            last_layer = lay;
            if (lay > 1) {
                done++;
                HLayer &L = Ls[done - 1];
                phase_terms(k * h[done - 1], L.r1, L.r2, cv > vp[stale - 1], cv > vs[stale - 1], L);
            }
        }
        HLayer &C = Ls[lay - 1];
        phase_terms(k * dl, C.r1, C.r2, cv > vp[lay - 1], cv > vs[lay - 1], C);
        layer_product(Ls, vs, lay, b);
        stale = lay + 1;
        U[iz - 1] = {b[0][0] * su_r - b[0][1] * sw_i, b[0][0] * su_i + b[0][1] * sw_r};
        W[iz - 1] = {-b[1][0] * su_i + b[1][1] * sw_r, b[1][0] * su_r + b[1][1] * sw_i};
    }
    return WT3D_OK;
}

// u0 on the grid for m sources; U0 row-major n x ld (complex128).
__global__ void k_pw_expand(int nx, int ny, int nz, double dx, int m, const double2 *__restrict__ Uz,
                            const double2 *__restrict__ Wz, const double *__restrict__ kx,
                            const double *__restrict__ ky, const double *__restrict__ rx,
                            const double *__restrict__ ry, double2 *__restrict__ U0, int ld)
{
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nn = (long long)nx * ny * nz;
    if (q >= nn * m) return;
    const long long g = q / m;
    const int j = (int)(q % m);
    const int iz = (int)(g % nz), ix = (int)((g / nz) % nx), iy = (int)(g / ((long long)nz * nx));
    const double ph = kx[j] * (ix * dx) + ky[j] * (iy * dx);
    double s, c;
    sincos(ph, &s, &c);
    double2 u = Uz[(long long)j * nz + iz], w = Wz[(long long)j * nz + iz];
    u.y = -u.y;   // conjugate: Haskell's time sign is the reverse of the operator's
    w.y = -w.y;
    const double2 ue = make_double2(u.x * c - u.y * s, u.x * s + u.y * c);
    const double2 we = make_double2(w.x * c - w.y * s, w.x * s + w.y * c);
    double2 *o = U0 + (3 * g) * ld + j;
    o[0] = make_double2(ue.x * rx[j], ue.y * rx[j]);
    o[ld] = make_double2(ue.x * ry[j], ue.y * ry[j]);
    o[2 * ld] = we;
}

// F[:, j] = (A_bg - A) U0[:, j] (column-major output, leading dimension n).
__global__ void __launch_bounds__(256) k_hetfld(long long n, int m, const int *__restrict__ irptr,
                                                const int *__restrict__ jcptr, const double2 *__restrict__ a,
                                                const double2 *__restrict__ abg, const double2 *__restrict__ U0,
                                                int ld, double2 *__restrict__ F)
{
    const int lane = threadIdx.x & 31;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = w0; i < n; i += nw) {
        for (int j = lane; j < m; j += 32) {
            double2 acc = make_double2(0, 0);
            for (int k = irptr[i]; k < irptr[i + 1]; k++) {
                const double2 d = make_double2(abg[k].x - a[k].x, abg[k].y - a[k].y);
                const double2 x = U0[(long long)jcptr[k] * ld + j];
                acc.x += d.x * x.x - d.y * x.y;
                acc.y += d.x * x.y + d.y * x.x;
            }
            F[(long long)j * n + i] = acc;
        }
    }
}

}  // namespace wt3d
