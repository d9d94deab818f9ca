// Host analysis: geometric nested dissection of the grid and the multifrontal
// symbolic factorisation.
//
// The reference hands the CSR pattern to STRUMPACK, which orders it with METIS
// nested dissection (strumpack_finter.c:42) and builds its own frontal tree.
// For the 27-point grid graph a one-node-thick coordinate plane is a vertex
// separator (no stencil edge crosses it), so bisecting the longest box axis
// gives a balanced nested dissection directly from (nx, ny, nz), with no
// graph partitioner.  Supernodes are whole separators (or leaf boxes); the
// border of a supernode is computed by the multifrontal rule
//     struct(S) = (adj(S) U struct(children)) restricted to later nodes,
// on grid nodes, then expanded to the 3 dofs per node.
#include "internal.h"
#include <algorithm>
#include <array>
#include <cstring>
#include <functional>

namespace wt3d {

namespace {

struct Box {
    int lo[3], hi[3];   // half-open, axes 0=x 1=y 2=z
    long long vol() const { return (long long)(hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]); }
};

struct Builder {
    int nx, ny, nz;
    int leaf;
    Symbolic &S;
    std::vector<int> newnode;        // natural node -> new node index
    std::vector<int> node_of_new;    // new node -> natural node
    std::vector<std::vector<int>> snodes;  // per front: natural nodes of the supernode
    int next = 0;

    Builder(int x, int y, int z, int lf, Symbolic &s) : nx(x), ny(y), nz(z), leaf(lf), S(s) {}

    long long nid(int ix, int iy, int iz) const { return iz + (long long)nz * (ix + (long long)nx * iy); }

    void number_box(const Box &b, std::vector<int> &out)
    {
        for (int iy = b.lo[1]; iy < b.hi[1]; iy++)
            for (int ix = b.lo[0]; ix < b.hi[0]; ix++)
                for (int iz = b.lo[2]; iz < b.hi[2]; iz++) {
                    long long g = nid(ix, iy, iz);
                    newnode[g] = next;
                    node_of_new[next] = (int)g;
                    next++;
                    out.push_back((int)g);
                }
    }

    int build(const Box &b, int depth)
    {
        int len[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
        int ax = 0;
        for (int a = 1; a < 3; a++)
            if (len[a] > len[ax]) ax = a;
        Front f;
        f.level = depth;
        std::vector<int> nodes;
        if (b.vol() <= leaf || len[ax] < 3) {
            number_box(b, nodes);
        } else {
            int m = (b.lo[ax] + b.hi[ax]) / 2;
            Box b1 = b, b2 = b, sep = b;
            b1.hi[ax] = m;
            b2.lo[ax] = m + 1;
            sep.lo[ax] = m;
            sep.hi[ax] = m + 1;
            int c1 = build(b1, depth + 1);
            int c2 = build(b2, depth + 1);
            f.child[0] = c1;
            f.child[1] = c2;
            f.nchild = 2;
            number_box(sep, nodes);
        }
        int id = (int)S.fronts.size();
        for (int c = 0; c < f.nchild; c++) S.fronts[f.child[c]].parent = id;
        f.p = 3 * (int)nodes.size();
        f.first = 3 * newnode[nodes[0]];
        S.fronts.push_back(f);
        snodes.push_back(std::move(nodes));
        return id;
    }
};

}  // namespace

int symbolic_grid(int nx, int ny, int nz, int leaf_nodes, Symbolic &S)
{
    if (nx < 2 || ny < 2 || nz < 2) {
        set_error("symbolic_grid: grid must be at least 2 nodes on every axis");
        return WT3D_ERR_ARG;
    }
    S = Symbolic();
    S.nx = nx; S.ny = ny; S.nz = nz;
    S.nnodes = (long long)nx * ny * nz;
    S.n = 3 * S.nnodes;
    if (S.n >= (1LL << 31)) {
        set_error("symbolic_grid: more than 2^31 unknowns");
        return WT3D_ERR_ARG;
    }
    Builder B(nx, ny, nz, leaf_nodes, S);
    B.newnode.assign(S.nnodes, -1);
    B.node_of_new.assign(S.nnodes, -1);
    Box root{{0, 0, 0}, {nx, ny, nz}};
    B.build(root, 0);

    const int nf = (int)S.fronts.size();
    // ---- borders: struct(S) on nodes, children before parents (postorder) ----
    std::vector<std::vector<int>> sn_struct(nf);   // new node indices, sorted
    std::vector<int> mark(S.nnodes, -1);
    for (int f = 0; f < nf; f++) {
        Front &F = S.fronts[f];
        int last_new = F.first / 3 + F.p / 3 - 1;
        std::vector<int> st;
        auto add = [&](int newn) {
            if (newn > last_new && mark[newn] != f) {
                mark[newn] = f;
                st.push_back(newn);
            }
        };
        for (int g : B.snodes[f]) {
            int iz = g % nz, ix = (g / nz) % nx, iy = g / (nz * nx);
            for (int dy = -1; dy <= 1; dy++) {
                int y = iy + dy; if (y < 0 || y >= ny) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    int x = ix + dx; if (x < 0 || x >= nx) continue;
                    for (int dz = -1; dz <= 1; dz++) {
                        int z = iz + dz; if (z < 0 || z >= nz) continue;
                        add(B.newnode[B.nid(x, y, z)]);
                    }
                }
            }
        }
        for (int c = 0; c < F.nchild; c++) {
            for (int w : sn_struct[F.child[c]]) add(w);
            std::vector<int>().swap(sn_struct[F.child[c]]);   // children no longer needed
        }
        std::sort(st.begin(), st.end());
        F.b = 3 * (int)st.size();
        F.border_off = (long long)S.border.size();
        for (int w : st)
            for (int q = 0; q < 3; q++) S.border.push_back(3 * w + q);
        sn_struct[f] = std::move(st);
    }

    // ---- permutation (dof level) ----
    S.perm.resize(S.n);
    S.iperm.resize(S.n);
    for (long long nn = 0; nn < S.nnodes; nn++) {
        int g = B.node_of_new[nn];
        for (int q = 0; q < 3; q++) {
            S.perm[3 * nn + q] = 3 * g + q;
            S.iperm[3 * g + q] = (int)(3 * nn + q);
        }
    }

    // ---- levels, storage offsets, flop count ----
    int maxlev = 0;
    for (auto &F : S.fronts) maxlev = std::max(maxlev, F.level);
    S.levels.assign(maxlev + 1, {});
    for (int f = 0; f < nf; f++) S.levels[S.fronts[f].level].push_back(f);
    long long fac = 0;
    for (int f = 0; f < nf; f++) {
        Front &F = S.fronts[f];
        fac += fac & 1;   // even offsets: 16-byte-aligned complex64 fronts (TMA-addressable blocks)
        F.fac_off = fac;
        fac += (long long)F.p * F.nf() + (long long)F.b * F.p;
        double p = F.p, b = F.b;
        S.flops += 8.0 * (p * p * p / 3.0 + p * p * b + p * b * b);
        S.max_p = std::max(S.max_p, F.p);
        S.max_b = std::max(S.max_b, F.b);
    }
    S.fac_total = fac;
    for (int l = 0; l <= maxlev; l++) {
        long long u = 0;
        for (int f : S.levels[l]) {
            S.fronts[f].upd_off = u;
            u += (long long)S.fronts[f].b * S.fronts[f].b;
        }
        S.upd_size[l & 1] = std::max(S.upd_size[l & 1], u);
    }

    // ---- relative positions of each border dof in the parent front ----
    std::vector<int> pos(S.n, -1);
    S.rel.assign(S.border.size(), -1);
    for (int f = 0; f < nf; f++) {
        const Front &P = S.fronts[f];
        if (P.nchild == 0) continue;
        for (int i = 0; i < P.p; i++) pos[P.first + i] = i;
        for (int j = 0; j < P.b; j++) pos[S.border[P.border_off + j]] = P.p + j;
        for (int c = 0; c < P.nchild; c++) {
            Front &C = S.fronts[P.child[c]];
            C.rel_off = C.border_off;
            for (int j = 0; j < C.b; j++) {
                int d = S.border[C.border_off + j];
                int r = pos[d];
                if (r < 0) {
                    set_error("symbolic_grid: child border entry missing from parent front");
                    return WT3D_ERR_PATTERN;
                }
                S.rel[C.rel_off + j] = r;
            }
        }
        for (int i = 0; i < P.p; i++) pos[P.first + i] = -1;
        for (int j = 0; j < P.b; j++) pos[S.border[P.border_off + j]] = -1;
    }
    return WT3D_OK;
}

int scatter_map(const Symbolic &S, const std::vector<int> &irptr, const std::vector<int> &jcptr,
                std::vector<long long> &map)
{
    const long long n = S.n;
    const long long nnz = irptr[n];
    map.assign(nnz, -1);
    // transposed position of every entry (structurally symmetric pattern)
    std::vector<long long> tpos(nnz);
    {
        std::vector<long long> cur(n);
        for (long long r = 0; r < n; r++) cur[r] = irptr[r];
        for (long long r = 0; r < n; r++)
            for (long long k = irptr[r]; k < irptr[r + 1]; k++) tpos[k] = cur[jcptr[k]]++;
    }
    std::vector<int> pos(n, -1);
    for (size_t f = 0; f < S.fronts.size(); f++) {
        const Front &F = S.fronts[f];
        const int nfr = F.nf();
        for (int i = 0; i < F.p; i++) pos[F.first + i] = i;
        for (int j = 0; j < F.b; j++) pos[S.border[F.border_off + j]] = F.p + j;
        const int last = F.first + F.p - 1;
        for (int i = 0; i < F.p; i++) {
            int R = F.first + i;
            int r = S.perm[R];
            for (long long k = irptr[r]; k < irptr[r + 1]; k++) {
                int C = S.iperm[jcptr[k]];
                if (C < F.first) continue;
                int lc = pos[C];
                if (lc < 0) { set_error("scatter_map: column outside front"); return WT3D_ERR_PATTERN; }
                map[k] = F.fac_off + (long long)i * nfr + lc;
                if (C > last) map[tpos[k]] = F.fac_off + (long long)F.p * nfr + (long long)(lc - F.p) * F.p + i;
            }
        }
        for (int i = 0; i < F.p; i++) pos[F.first + i] = -1;
        for (int j = 0; j < F.b; j++) pos[S.border[F.border_off + j]] = -1;
    }
    for (long long k = 0; k < nnz; k++)
        if (map[k] < 0) { set_error("scatter_map: unmapped entry"); return WT3D_ERR_PATTERN; }
    return WT3D_OK;
}

int detect_grid(int n, long long nnz, const int *irptr, const int *jcptr, int &nx, int &ny, int &nz)
{
    // Row 1 is node (1,1,1): its box holds nodes 1,2 (z), 1+nz, 2+nz (x) and
    // the same shifted by nx*nz (y); with 3 dofs the 7th column is 3nz+1 and
    // the 13th is 3nx*nz+1 (srgraphs.f:681-714).
    if (n % 3 != 0 || irptr[0] != 1) return WT3D_ERR_PATTERN;
    long long len0 = irptr[1] - irptr[0];
    if (len0 != 24) return WT3D_ERR_PATTERN;   // grid must be >= 2 on every axis
    int c7 = jcptr[6], c13 = jcptr[12];
    if ((c7 - 1) % 3 != 0 || (c13 - 1) % 3 != 0) return WT3D_ERR_PATTERN;
    nz = (c7 - 1) / 3;
    long long nxz = (c13 - 1) / 3;
    if (nz < 2 || nxz % nz != 0) return WT3D_ERR_PATTERN;
    nx = (int)(nxz / nz);
    long long nn = n / 3;
    if (nx < 2 || nn % nxz != 0) return WT3D_ERR_PATTERN;
    ny = (int)(nn / nxz);
    if (ny < 2) return WT3D_ERR_PATTERN;
    long long want = 9LL * (3LL * nx - 2) * (3LL * ny - 2) * (3LL * nz - 2);
    if (want != nnz) return WT3D_ERR_PATTERN;
    // full entry-by-entry check
    long long k = 0;
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                long long g = iz + (long long)nz * (ix + (long long)nx * iy);
                for (int r = 0; r < 3; r++) {
                    if (irptr[3 * g + r] != k + 1) return WT3D_ERR_PATTERN;
                    for (int dy = -1; dy <= 1; dy++) {
                        int y = iy + dy; if (y < 0 || y >= ny) continue;
                        for (int dx = -1; dx <= 1; dx++) {
                            int x = ix + dx; if (x < 0 || x >= nx) continue;
                            for (int dz = -1; dz <= 1; dz++) {
                                int z = iz + dz; if (z < 0 || z >= nz) continue;
                                long long nb = z + (long long)nz * (x + (long long)nx * y);
                                for (int q = 0; q < 3; q++)
                                    if (jcptr[k++] != 3 * nb + q + 1) return WT3D_ERR_PATTERN;
                            }
                        }
                    }
                }
            }
    if (irptr[n] != k + 1) return WT3D_ERR_PATTERN;
    return WT3D_OK;
}

}  // namespace wt3d
