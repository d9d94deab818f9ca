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
#include "stencil.cuh"
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

// DISPERSION (dispersion.f:78-114) in FP64: qp, qs hold 1/Q.  At
// omega1 = Re(omega) and omegabase = 2 pi freqbase,
//   c = c1 * max(1 + (1/Q)/pi * ln(omega1/omegabase), 0.1),  vc = (c, -c (1/Q)/2),
//   mu = vcs^2 rho,  lambda = vcp^2 rho - 2 mu.
__global__ void k_lame_q(long long n, const float *__restrict__ vp, const float *__restrict__ vs,
                         const float *__restrict__ rho, const float *__restrict__ qp, const float *__restrict__ qs,
                         double fac1, cx<double> *__restrict__ da, cx<double> *__restrict__ mu,
                         double *__restrict__ ro)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double pi = 3.141592653589793;
    const double r = rho[i];
    double fs = 1.0 + ((double)qs[i] / pi) * fac1, fp = 1.0 + ((double)qp[i] / pi) * fac1;
    fs = fs < 0.1 ? 0.1 : fs;
    fp = fp < 0.1 ? 0.1 : fp;
    const double cs = vs[i] * fs, cp = vp[i] * fp;
    const cx<double> vcs(cs, -cs * (double)qs[i] / 2.0), vcp(cp, -cp * (double)qp[i] / 2.0);
    const cx<double> m = vcs * vcs * r;
    mu[i] = m;
    da[i] = vcp * vcp * r - 2.0 * m;
    ro[i] = r;
}

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
    const int jx = ix + 1, jy = iy + 1;
    unsigned mask;
    int region, zidx;
    node_region(p, iz, ix, iy, region, zidx, mask);

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

int device_lame_q(long long nn, const float *d_vp, const float *d_vs, const float *d_rho, const float *d_qp,
                  const float *d_qs, double omega_re, double freqbase, void *d_da, void *d_mu, double *d_ro,
                  cudaStream_t st)
{
    const double omegabase = freqbase * 2.0 * 3.141592653589793;
    const double eps = 10.0 * 1.1920929e-07;   // 10 EPSILON(1.0) (dispersion.f:49)
    if (!(omega_re > eps && omegabase > 0.0))  // no dispersion (dispersion.f:78-80)
        return device_lame(nn, d_vp, d_vs, d_rho, d_da, d_mu, d_ro, st);
    k_lame_q<<<ceil_div(nn, 256), 256, 0, st>>>(nn, d_vp, d_vs, d_rho, d_qp, d_qs, std::log(omega_re / omegabase),
                                                (cx<double> *)d_da, (cx<double> *)d_mu, d_ro);
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
