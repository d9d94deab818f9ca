// Point sources and receivers between grid nodes.
//
// SRCSETUP (srcsetup.f:50-211) spreads a source at (x, y, z) onto the grid
// with weights from SRCREG (srcreg.f:77-304), and with lsetup = .false.
// samples a wavefield with the same weights:
//   ireg = 0     nearest node, weight 1 (srcsetup.f:50-73);
//   ireg > 0     region of half-width ireg nodes around the top-left node,
//                sprd <= 0.5: separable Kaiser-windowed sinc
//                  w(d) = sin(pi d)/(pi d) * I0(a sqrt(1 - (d/ireg)^2)) / I0(a)
//                  (zero for d >= ireg), a from the table of srcreg.f:206-226
//                  (optimal up to half the Nyquist wavenumber);
//                sprd > 0.5: separable discrete Dirac of half-width sprd nodes
//                  (srcreg.f:269-304), region half-width INT(2 sprd), weights
//                  normalised to sum 1 (srcreg.f:134-141).
// Region nodes beyond a free surface are mirrored into the grid with a sign
// change; nodes beyond an absorbing face are dropped (srcsetup.f:131-210).
// Only the top face can be a free surface here (wt3d_grid::fst).
//
// Arithmetic is FP64 with I0 from std::cyl_bessel_i; the reference works in
// REAL with a rational approximation of I0 (srcreg.f:309-331), so the weights
// agree to ~1e-7 relative.
#include "internal.h"
#include "wtomo3d_gpu.h"
#include <cmath>
#include <vector>

namespace wt3d {

namespace {

double kaiser_a(int ireg)
{
    static const double a[10] = {0.0, 1.24, 2.94, 4.53, 6.31, 7.91, 9.42, 10.95, 12.53, 14.09};
    return ireg >= 1 && ireg <= 9 ? a[ireg] : 14.18;
}

// windowed sinc at distance d (nodes), half-width ireg (srcreg.f:167-265)
double wsinc(int ireg, double d)
{
    const double s = d <= 1e-10 ? 1.0 : std::sin(M_PI * d) / (M_PI * d);
    const double lx = d / (double)ireg;
    if (!(lx < 1.0)) return 0.0;
    const double a = kaiser_a(ireg);
    return s * std::cyl_bessel_i(0.0, a * std::sqrt(1.0 - lx * lx)) / std::cyl_bessel_i(0.0, a);
}

// discrete Dirac of half-width h at distance d (srcreg.f:269-304)
double ddirac(double h, double d)
{
    if (d < h) return (1.0 - d * d / (2.0 * h * h)) / (2.0 * h);
    if (d < 2.0 * h) return (1.0 + (d * d - 4.0 * d * h) / (4.0 * h * h)) / h;
    return 0.0;
}

}  // namespace

int source_weights(const wt3d_grid &g, double x, double y, double z, int ireg, double sprd,
                   std::vector<long long> &node, std::vector<double> &w)
{
    node.clear();
    w.clear();
    const double dx = g.dx;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    if (ireg < 0) { set_error("source_weights: ireg < 0"); return WT3D_ERR_ARG; }
    if (ireg == 0) {
        const int ix = (int)(0.5 + x / dx) + 1, iy = (int)(0.5 + y / dx) + 1, iz = (int)(0.5 + z / dx) + 1;
        if (ix < 1 || ix > nx || iy < 1 || iy > ny || iz < 1 || iz > nz) {
            set_error("source_weights: position outside the grid");
            return WT3D_ERR_ARG;
        }
        node.push_back((long long)(iz - 1) + (long long)nz * ((ix - 1) + (long long)nx * (iy - 1)));
        w.push_back(1.0);
        return WT3D_OK;
    }
    const bool dist = sprd > 0.5;
    if (dist && !(sprd > 1e-10)) { set_error("source_weights: spread too small"); return WT3D_ERR_ARG; }
    // top-left node and offsets (srcsetup.f:83-88)
    const int ixs = (int)(x / dx) + 1, iys = (int)(y / dx) + 1, izs = (int)(z / dx) + 1;
    const double xo = x - (ixs - 1) * dx, yo = y - (iys - 1) * dx, zo = z - (izs - 1) * dx;
    const int half = dist ? (int)(2.0 * sprd) : ireg;
    const int len = 2 * half + 1;   // ireg: 2 ireg + 1 (srcreg.f:82); spread: INT(4 sprd) + 1 (srcreg.f:109)
    const int lenw = dist ? (int)(4.0 * sprd) + 1 : len;
    // separable factors fs(i) along each axis, i = 1..lenw, centred at half + 1 + offset
    std::vector<double> fx(lenw), fy(lenw), fz(lenw);
    const double cx = half + 1 + xo / dx, cy = half + 1 + yo / dx, cz = half + 1 + zo / dx;
    for (int i = 1; i <= lenw; i++) {
        const double ddx = std::fabs(i - cx), ddy = std::fabs(i - cy), ddz = std::fabs(i - cz);
        fx[i - 1] = dist ? ddirac(sprd, ddx) : wsinc(ireg, ddx);
        fy[i - 1] = dist ? ddirac(sprd, ddy) : wsinc(ireg, ddy);
        fz[i - 1] = dist ? ddirac(sprd, ddz) : wsinc(ireg, ddz);
    }
    double amp = 1.0;
    if (dist) {
        amp = 0.0;
        for (int a = 0; a < lenw; a++)
            for (int b = 0; b < lenw; b++)
                for (int c = 0; c < lenw; c++) amp += fz[c] * fx[b] * fy[a];
        if (!(amp > 0)) { set_error("source_weights: zero spread weights"); return WT3D_ERR_ARG; }
    }
    // region [i - half, i + half], clipped at absorbing faces, mirrored at the free surface
    int zlo = izs - half, zhi = izs + half, xlo = ixs - half, xhi = ixs + half, ylo = iys - half, yhi = iys + half;
    if (zlo < 1 && !g.fst) zlo = 1;
    if (zhi > nz) zhi = nz;
    if (xlo < 1) xlo = 1;
    if (xhi > nx) xhi = nx;
    if (ylo < 1) ylo = 1;
    if (yhi > ny) yhi = ny;
    for (int iz = zlo; iz <= zhi; iz++) {
        const int kz = iz - (izs - half);
        const int izf = iz < 1 ? 2 - iz : iz;
        if (izf < 1 || izf > nz || kz >= lenw) continue;
        for (int ix = xlo; ix <= xhi; ix++) {
            const int kx = ix - (ixs - half);
            if (kx >= lenw) continue;
            for (int iy = ylo; iy <= yhi; iy++) {
                const int ky = iy - (iys - half);
                if (ky >= lenw) continue;
                const double v = fz[kz] * fx[kx] * fy[ky] / amp;
                if (v == 0.0) continue;
                node.push_back((long long)(izf - 1) + (long long)nz * ((ix - 1) + (long long)nx * (iy - 1)));
                w.push_back(izf == iz ? v : -v);
            }
        }
    }
    return WT3D_OK;
}

}  // namespace wt3d

using namespace wt3d;

extern "C" int wt3d_source_weights(const wt3d_grid *g, double x, double y, double z, int ireg, double sprd, int cap,
                                   long long *node, double *weight, int *count)
{
    if (!g || !count || (cap > 0 && (!node || !weight))) { set_error("wt3d_source_weights: bad arguments"); return WT3D_ERR_ARG; }
    std::vector<long long> nd;
    std::vector<double> w;
    int rc = source_weights(*g, x, y, z, ireg, sprd, nd, w);
    if (rc) return rc;
    *count = (int)nd.size();
    for (int i = 0; i < (int)nd.size() && i < cap; i++) {
        node[i] = nd[i];
        weight[i] = w[i];
    }
    return WT3D_OK;
}
