// Internal interfaces between the translation units of libwtomo3d_gpu.
#pragma once
#include <cuda_runtime.h>
#include <vector>
#include <string>
#include <cstdint>
#include "wtomo3d_gpu.h"

namespace wt3d {

void set_error(const std::string &msg);

// ---- assembly (assemble.cu) ----------------------------------------------
void grid_pml(const wt3d_grid &g, double &pmld, double &pmlf, int &ipml);
int device_pattern(int nx, int ny, int nz, int base, int *d_irptr, int *d_jcptr, cudaStream_t st);
int device_lame(long long nn, const float *d_vp, const float *d_vs, const float *d_rho, void *d_da, void *d_mu,
                double *d_ro, cudaStream_t st);
int device_lame_q(long long nn, const float *d_vp, const float *d_vs, const float *d_rho, const float *d_qp,
                  const float *d_qs, double omega_re, double freqbase, void *d_da, void *d_mu, double *d_ro,
                  cudaStream_t st);
int device_assemble(const wt3d_grid &g, const void *d_da, const void *d_mu, const double *d_ro, double om_re,
                    double om_im, const int *d_irptr, void *d_a, cudaStream_t st);

// ---- sources and receivers between nodes (sources.cpp) --------------------
int source_weights(const wt3d_grid &g, double x, double y, double z, int ireg, double sprd,
                   std::vector<long long> &node, std::vector<double> &w);

// ---- adjoint gradient (gradient.cu) --------------------------------------
long long gradient_scratch_doubles(long long nn);
int device_gradient(const wt3d_grid &g, const void *d_da, const void *d_mu, const double *d_ro, const float *d_vp,
                    const float *d_vs, const float *d_rho, double om_re, double om_im, int m, long long ld,
                    const void *d_U, const void *d_L, double *d_D, double *d_grad, cudaStream_t st);
int device_receivers(int m, int nrec, long long ld, const long long *d_rec, const void *d_U, const void *d_dobs,
                     void *d_pred, void *d_res, void *d_S, cudaStream_t st);
int device_add(long long total, const void *d_a, void *d_y, cudaStream_t st);

// ---- symbolic analysis (symbolic.cpp) -------------------------------------
// Nested dissection of the nx*ny*nz grid with one-node-thick plane
// separators (or of a general pattern's graph), and the multifrontal
// symbolic factorisation in that ordering.  Fronts are listed in postorder.
struct Front {
    int p = 0, b = 0;        // pivot dofs, border (update) dofs
    int first = 0;           // new index of the first pivot dof
    int parent = -1;
    int child[2] = {-1, -1};
    int nchild = 0;
    int level = 0;           // depth from the root
    long long fac_off = 0;   // complex offset of the P block (p x nf) in the factor pool; Lo (b x p) follows
    long long upd_off = 0;   // complex offset of F22 (b x b) in the level-parity update buffer
    long long border_off = 0;// offset into Symbolic::border (b entries)
    long long rel_off = 0;   // offset into Symbolic::rel (b entries): positions in the parent front
    int nf() const { return p + b; }
};

struct Symbolic {
    int nx = 0, ny = 0, nz = 0;
    long long nnodes = 0, n = 0;
    std::vector<int> perm;    // new dof -> old dof
    std::vector<int> iperm;   // old dof -> new dof
    std::vector<Front> fronts;
    std::vector<int> border;  // border dof new indices, per front
    std::vector<int> rel;     // per front: parent-front position of each border dof
    std::vector<std::vector<int>> levels;  // front ids per depth
    long long fac_total = 0;              // complex entries of all factors
    long long upd_size[2] = {0, 0};       // complex entries of the two update buffers
    double flops = 0;
    int max_p = 0, max_b = 0;
};

int symbolic_grid(int nx, int ny, int nz, int leaf_nodes, Symbolic &S);

// Any structurally symmetric pattern (rows irptr/jcptr with index base 0 or
// 1): automatic nested dissection on the supervariable graph, then the same
// symbolic factorisation; leaf fronts hold at most leaf_dofs dofs.
int symbolic_graph(long long n, const int *irptr, const int *jcptr, int base, long long leaf_dofs, Symbolic &S);

// 0-based pattern of A + A^T (STRUMPACK orders unsymmetric patterns the same
// way) from a checked CSR pattern: if A's pattern is already symmetric, sir/sjc
// are A's own rows in the caller's order and vmap is empty; otherwise rows are
// sorted and vmap[k] is the position of A's entry k in sjc.
int symmetrize(long long n, const int *irptr, const int *jcptr, int base, std::vector<int> &sir,
               std::vector<int> &sjc, std::vector<int> &vmap);

// Whether the build linked the CUDA toolkit's METIS (its vertex separator is
// then a candidate at every split of the general ordering).
bool metis_linked();

// Check a CSR pattern: pointers start at the base and grow, columns in range,
// no duplicates in a row and, if need_symmetric, structural symmetry.
int check_csr(long long n, long long nnz, const int *irptr, const int *jcptr, int base, bool need_symmetric);

// Position of the transposed entry (c, r) of every entry (r, c) of a
// structurally symmetric 0-based pattern; columns may be in any order.
std::vector<long long> transpose_positions(long long n, const int *irptr, const int *jcptr);

// Destination of every CSR entry (0-based CSR, natural ordering) in the factor
// pool: entry (r,c) belongs to the front holding min(new r, new c).
int scatter_map(const Symbolic &S, const std::vector<int> &irptr, const std::vector<int> &jcptr,
                std::vector<long long> &map);

// Recover (nx, ny, nz) from a 1-based CSR pattern produced by srel3d +
// SPARSE_ADJ2CRS and check it entry by entry.  Returns 0 on success.
int detect_grid(int n, long long nnz, const int *irptr, const int *jcptr, int &nx, int &ny, int &nz);

}  // namespace wt3d
