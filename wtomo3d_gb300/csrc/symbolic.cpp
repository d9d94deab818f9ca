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
#include <atomic>
#include <cstdint>
#include <exception>
#include <new>
#include <system_error>
#include <limits>
#include <memory>
#include <mutex>
#include <thread>
#include <queue>

#ifdef WT3D_HAVE_METIS
// METIS as it ships with the CUDA toolkit (libmetis_static.a, no header): the
// two entry points of its public API used here, with its 64-bit index type
// (checked by the build's probe program).
extern "C" int METIS_SetDefaultOptions(int64_t *options);
extern "C" int METIS_ComputeVertexSeparator(int64_t *nvtxs, int64_t *xadj, int64_t *adjncy, int64_t *vwgt,
                                            int64_t *options, int64_t *sepsize, int64_t *part);
#endif

namespace wt3d {

bool metis_linked()
{
#ifdef WT3D_HAVE_METIS
    return true;
#else
    return false;
#endif
}

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

// Depth levels, storage offsets, flop count and the parent-front position of
// every border dof, for fronts already listed in postorder with their pivots,
// borders and permutation.
static int finalize(Symbolic &S, const char *who)
{
    const int nf = (int)S.fronts.size();
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
                    set_error(std::string(who) + ": child border entry missing from parent front");
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

    return finalize(S, "symbolic_grid");
}

// ---------------------------------------------------------------------------
// General structurally symmetric patterns
// ---------------------------------------------------------------------------
// STRUMPACK accepts any CSR pattern (strumpack_finter.c:42-48 hands it to a
// nested-dissection reordering).  A pattern that is not the grid graph is
// ordered here by automatic nested dissection (George and Liu, Computer
// Solution of Large Sparse Positive Definite Systems, 1981, ch. 8): the
// separator of a connected subgraph is the smaller of two candidates: one
// level of a breadth-first level structure rooted at a pseudo-peripheral
// vertex (the smallest level that leaves at least a fifth of the weight on
// either side, thinned to the vertices that touch both sides), and the vertex
// cover of a multilevel edge bisection (below).  A disconnected subgraph is split between
// its components, and one vertex of the second group becomes the (trivial)
// separator.  The graph is first compressed to supervariables, runs of
// consecutive rows with the same column set (the 3 dofs of an elastic node),
// so fronts never split a node.
namespace {

// ---- multilevel bisection (the METIS family of methods) -------------------
// A connected subgraph is also bisected by the multilevel scheme of Karypis
// and Kumar (SIAM J. Sci. Comput. 20(1), 1998): coarsen by heavy-edge
// matching, grow a bisection of the coarsest graph greedily from several
// seeds, refine the edge cut by Fiduccia-Mattheyses passes while projecting
// back, and turn the cut into a vertex separator by a minimum vertex cover of
// the cut edges (Konig's theorem on a maximum matching).  split() keeps the
// smaller of this separator and the level-structure one.
struct LGraph {
    int n = 0;
    std::vector<long long> xadj;
    std::vector<int> adj, ew;   // neighbours and edge weights
    std::vector<long long> vw;  // vertex weights
};

struct Rng {
    unsigned long long s;
    explicit Rng(unsigned long long seed) : s(seed * 0x9E3779B97F4A7C15ULL + 1) {}
    unsigned next()
    {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return (unsigned)(s >> 11);
    }
};

// Heavy-edge matching; returns the coarse graph and cmap (fine -> coarse).
LGraph coarsen(const LGraph &g, std::vector<int> &cmap, Rng &rng)
{
    std::vector<int> order(g.n), match(g.n, -1);
    for (int v = 0; v < g.n; v++) order[v] = v;
    for (int i = g.n - 1; i > 0; i--) std::swap(order[i], order[rng.next() % (unsigned)(i + 1)]);
    for (int v : order) {
        if (match[v] >= 0) continue;
        int best = -1, bw = -1;
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++) {
            const int u = g.adj[k];
            if (match[u] < 0 && u != v && g.ew[k] > bw) { bw = g.ew[k]; best = u; }
        }
        if (best >= 0) { match[v] = best; match[best] = v; }
        else match[v] = v;
    }
    cmap.assign(g.n, -1);
    int nc = 0;
    for (int v = 0; v < g.n; v++)
        if (cmap[v] < 0) { cmap[v] = nc; cmap[match[v]] = nc; nc++; }
    LGraph c;
    c.n = nc;
    c.vw.assign(nc, 0);
    c.xadj.assign(nc + 1, 0);
    std::vector<int> first(nc, -1);
    for (int v = 0; v < g.n; v++) {
        c.vw[cmap[v]] += g.vw[v];
        if (first[cmap[v]] < 0) first[cmap[v]] = v;
    }
    std::vector<int> mark(nc, -1);
    std::vector<long long> pos(nc, 0);
    for (int cv = 0; cv < nc; cv++) {
        const int a = first[cv], b = match[a];
        const int mem[2] = {a, b};
        for (int t = 0; t < (b == a ? 1 : 2); t++) {
            const int m = mem[t];
            for (long long k = g.xadj[m]; k < g.xadj[m + 1]; k++) {
                const int cu = cmap[g.adj[k]];
                if (cu == cv) continue;
                if (mark[cu] == cv) { c.ew[pos[cu]] += g.ew[k]; continue; }
                mark[cu] = cv;
                pos[cu] = (long long)c.adj.size();
                c.adj.push_back(cu);
                c.ew.push_back(g.ew[k]);
            }
        }
        c.xadj[cv + 1] = (long long)c.adj.size();
    }
    return c;
}

long long edge_cut(const LGraph &g, const std::vector<char> &side)
{
    long long cut = 0;
    for (int v = 0; v < g.n; v++)
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++)
            if (side[g.adj[k]] != side[v]) cut += g.ew[k];
    return cut / 2;
}

// Fiduccia-Mattheyses passes on a two-way edge cut; sides stay within maxw
// (a move out of an overweight side is always allowed).  External degrees
// are kept up to date across moves, so a pass only touches the boundary.
void fm_refine(const LGraph &g, std::vector<char> &side, long long maxw, int passes)
{
    long long pw[2] = {0, 0};
    for (int v = 0; v < g.n; v++) pw[(int)side[v]] += g.vw[v];
    std::vector<long long> ext(g.n, 0), tot(g.n, 0);
    std::vector<int> bnd, locked(g.n, -1);
    std::vector<char> inb(g.n, 0);
    for (int v = 0; v < g.n; v++) {
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++) {
            tot[v] += g.ew[k];
            if (side[g.adj[k]] != side[v]) ext[v] += g.ew[k];
        }
        if (ext[v] > 0) { bnd.push_back(v); inb[v] = 1; }
    }
    auto flip = [&](int v) {   // move v to the other side, keeping ext[] exact
        const int to = 1 - side[v];
        side[v] = (char)to;
        pw[1 - to] -= g.vw[v];
        pw[to] += g.vw[v];
        ext[v] = tot[v] - ext[v];
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++) {
            const int u = g.adj[k];
            ext[u] += side[u] == to ? -g.ew[k] : g.ew[k];
            if (ext[u] > 0 && !inb[u]) { inb[u] = 1; bnd.push_back(u); }
        }
        if (ext[v] > 0 && !inb[v]) { inb[v] = 1; bnd.push_back(v); }
    };
    for (int pass = 0; pass < passes; pass++) {
        // drop vertices that left the boundary
        size_t w = 0;
        for (int v : bnd) {
            if (ext[v] > 0) bnd[w++] = v;
            else inb[v] = 0;
        }
        bnd.resize(w);
        std::priority_queue<std::pair<long long, int>> pq;
        for (int v : bnd) pq.push({2 * ext[v] - tot[v], v});
        std::vector<int> moves;
        long long cut = 0, best = 0;
        size_t best_n = 0;
        long long best_over = std::max(pw[0], pw[1]);
        while (!pq.empty()) {
            auto [gv, v] = pq.top();
            pq.pop();
            if (locked[v] == pass || gv != 2 * ext[v] - tot[v]) continue;
            const int from = side[v], to = 1 - from;
            if (pw[to] + g.vw[v] > maxw && pw[from] <= maxw) continue;
            locked[v] = pass;
            flip(v);
            cut -= gv;
            moves.push_back(v);
            for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++) {
                const int u = g.adj[k];
                if (locked[u] != pass) pq.push({2 * ext[u] - tot[u], u});
            }
            const long long over = std::max(pw[0], pw[1]);
            const bool balanced = over <= maxw, best_bal = best_over <= maxw;
            if ((balanced && !best_bal) || (balanced == best_bal && (cut < best || (cut == best && over < best_over)))) {
                best = cut;
                best_n = moves.size();
                best_over = over;
            }
            if (moves.size() - best_n > 256) break;
        }
        for (size_t i = moves.size(); i > best_n; i--) flip(moves[i - 1]);
        if (best_n == 0) break;
    }
}

// Greedy graph growing from a seed until half the weight is on side 0: the
// frontier vertex with the largest cut reduction next (breadth-first order
// on a coarsest graph too large for the quadratic scan).
void grow(const LGraph &g, int seed, std::vector<char> &side, long long half)
{
    side.assign(g.n, 1);
    if (g.n > 2000) {
        std::vector<int> q{seed};
        std::vector<char> in(g.n, 0);
        in[seed] = 1;
        long long w0 = 0;
        for (size_t qi = 0; w0 < half; qi++) {
            if (qi == q.size()) {   // next component
                int u = 0;
                while (u < g.n && in[u]) u++;
                if (u == g.n) break;
                in[u] = 1;
                q.push_back(u);
            }
            const int v = q[qi];
            side[v] = 0;
            w0 += g.vw[v];
            for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++)
                if (!in[g.adj[k]]) { in[g.adj[k]] = 1; q.push_back(g.adj[k]); }
        }
        return;
    }
    std::vector<long long> gain(g.n, 0);
    std::vector<char> front(g.n, 0);
    long long w0 = 0;
    int v = seed;
    for (;;) {
        side[v] = 0;
        w0 += g.vw[v];
        if (w0 >= half) break;
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++) {
            const int u = g.adj[k];
            if (side[u] == 0) continue;
            front[u] = 1;
            gain[u] += 2LL * g.ew[k];
        }
        int best = -1;
        for (int u = 0; u < g.n; u++)
            if (side[u] == 1 && front[u] && (best < 0 || gain[u] > gain[best])) best = u;
        if (best < 0)
            for (int u = 0; u < g.n && best < 0; u++)
                if (side[u] == 1) best = u;
        if (best < 0) break;
        v = best;
    }
}

// Minimum vertex cover of the bipartite cut graph (side-0 and side-1
// endpoints of cut edges): maximum matching by Hopcroft and Karp (SIAM J.
// Comput. 2(4), 1973), then Konig's construction.
std::vector<int> cut_cover(const LGraph &g, const std::vector<char> &side)
{
    std::vector<int> L, R, id(g.n, -1);
    for (int v = 0; v < g.n; v++) {
        bool cut = false;
        for (long long k = g.xadj[v]; k < g.xadj[v + 1] && !cut; k++) cut = side[g.adj[k]] != side[v];
        if (!cut) continue;
        if (side[v] == 0) { id[v] = (int)L.size(); L.push_back(v); }
        else { id[v] = (int)R.size(); R.push_back(v); }
    }
    const int nl = (int)L.size(), nr = (int)R.size();
    std::vector<long long> bx(nl + 1, 0);   // cut edges from each L vertex to R
    std::vector<int> bj;
    for (int l = 0; l < nl; l++) {
        const int v = L[l];
        for (long long k = g.xadj[v]; k < g.xadj[v + 1]; k++)
            if (side[g.adj[k]] == 1) bj.push_back(id[g.adj[k]]);
        bx[l + 1] = (long long)bj.size();
    }
    std::vector<int> mL(nl, -1), mR(nr, -1), dist(nl);
    std::vector<long long> it(nl);
    const int INF = std::numeric_limits<int>::max();
    for (;;) {
        // breadth-first layers from the free L vertices
        std::vector<int> q;
        for (int l = 0; l < nl; l++) {
            dist[l] = mL[l] < 0 ? 0 : INF;
            if (mL[l] < 0) q.push_back(l);
        }
        bool found = false;
        for (size_t qi = 0; qi < q.size(); qi++) {
            const int l = q[qi];
            for (long long k = bx[l]; k < bx[l + 1]; k++) {
                const int l2 = mR[bj[k]];
                if (l2 < 0) found = true;
                else if (dist[l2] == INF) { dist[l2] = dist[l] + 1; q.push_back(l2); }
            }
        }
        if (!found) break;
        // vertex-disjoint shortest augmenting paths along the layers
        for (int l = 0; l < nl; l++) it[l] = bx[l];
        std::vector<int> stk, path;
        for (int l0 = 0; l0 < nl; l0++) {
            if (mL[l0] >= 0 || dist[l0] != 0) continue;
            stk.assign(1, l0);
            path.clear();
            while (!stk.empty()) {
                const int l = stk.back();
                if (it[l] == bx[l + 1]) {
                    dist[l] = INF;
                    stk.pop_back();
                    if (!path.empty()) path.pop_back();
                    continue;
                }
                const int r = bj[it[l]++];
                const int l2 = mR[r];
                if (l2 < 0) {
                    path.push_back(r);
                    for (size_t t = 0; t < stk.size(); t++) { mL[stk[t]] = path[t]; mR[path[t]] = stk[t]; }
                    break;
                }
                if (dist[l2] != INF && dist[l2] == dist[l] + 1) {
                    path.push_back(r);
                    stk.push_back(l2);
                }
            }
        }
    }
    // Z: reachable from free L vertices by alternating paths
    std::vector<char> zl(nl, 0), zr(nr, 0);
    std::vector<int> q;
    for (int l = 0; l < nl; l++)
        if (mL[l] < 0) { zl[l] = 1; q.push_back(l); }
    for (size_t qi = 0; qi < q.size(); qi++) {
        const int l = q[qi];
        for (long long k = bx[l]; k < bx[l + 1]; k++) {
            const int r = bj[k];
            if (zr[r]) continue;
            zr[r] = 1;
            const int l2 = mR[r];
            if (l2 >= 0 && !zl[l2]) { zl[l2] = 1; q.push_back(l2); }
        }
    }
    std::vector<int> cover;
    for (int l = 0; l < nl; l++)
        if (!zl[l]) cover.push_back(L[l]);
    for (int r = 0; r < nr; r++)
        if (zr[r]) cover.push_back(R[r]);
    return cover;
}

// Two-way multilevel bisection of g: side[v] in {0, 1}.
void ml_bisect(const LGraph &g0, std::vector<char> &side, unsigned long long seed)
{
    Rng rng(seed);
    std::vector<LGraph> gs;
    std::vector<std::vector<int>> cmaps;
    const LGraph *cur = &g0;
    while (cur->n > 160 && gs.size() < 40) {
        std::vector<int> cm;
        LGraph c = coarsen(*cur, cm, rng);
        if (c.n > (int)(0.92 * cur->n)) break;
        cmaps.push_back(std::move(cm));
        gs.push_back(std::move(c));
        cur = &gs.back();
    }
    long long W = 0;
    for (long long w : cur->vw) W += w;
    const long long maxw = (long long)(0.55 * (double)W) + 1;
    std::vector<char> best;
    long long best_cut = -1;
    const int trials = cur->n > 1000 ? 3 : 8;
    for (int t = 0; t < trials; t++) {
        std::vector<char> s;
        grow(*cur, (int)(rng.next() % (unsigned)cur->n), s, W / 2);
        fm_refine(*cur, s, maxw, 4);
        const long long c = edge_cut(*cur, s);
        if (best_cut < 0 || c < best_cut) { best_cut = c; best = s; }
    }
    side = best;
    for (int lv = (int)gs.size() - 1; lv >= 0; lv--) {
        const LGraph &fine = lv > 0 ? gs[lv - 1] : g0;
        std::vector<char> fs(fine.n);
        for (int v = 0; v < fine.n; v++) fs[v] = side[cmaps[lv][v]];
        long long Wf = 0;
        for (long long w : fine.vw) Wf += w;
        fm_refine(fine, fs, (long long)(0.55 * (double)Wf) + 1, 10);
        side.swap(fs);
    }
}

struct GraphND {
    int nv = 0;                      // supervariables
    std::vector<long long> xadj;     // quotient graph, no self loops
    std::vector<int> adj;
    std::vector<int> wt;             // dofs per supervariable
    std::vector<int> first_dof;      // first (old) dof of each supervariable
    long long leaf = 0;              // leaf fronts hold at most this many dofs
    Symbolic &S;
    // Subset id of each vertex (-1 once it is in a front).  Disjoint subsets
    // are dissected by concurrent threads: each writes only its own vertices,
    // but reads the ids of neighbours in other subsets, hence atomics.
    std::unique_ptr<std::atomic<int>[]> part;
    std::vector<int> lev;            // breadth-first level of each vertex
    std::vector<long long> seen;     // stamp of the last search that reached each vertex
    std::atomic<long long> stamp{0};
    std::atomic<int> next_part{1};
    std::vector<std::vector<int>> snodes;   // per front: supervariables, in numbering order
    std::vector<int> lid;            // local index of each vertex inside the subset being split
    static constexpr int MAXDEPTH = 256;
    int par_depth = 3;               // subtrees above this depth run on their own threads

    struct Node {                    // dissection tree, numbered in postorder afterwards
        std::vector<int> nodes;      // separator (or leaf) supervariables
        std::unique_ptr<Node> child[2];
        int depth = 0;
    };

    explicit GraphND(Symbolic &s) : S(s) {}

    int pid_of(int v) const { return part[v].load(std::memory_order_relaxed); }
    void set_pid(int v, int id) { part[v].store(id, std::memory_order_relaxed); }

    int degree(int v, int pid) const
    {
        int d = 0;
        for (long long k = xadj[v]; k < xadj[v + 1]; k++) d += pid_of(adj[k]) == pid;
        return d;
    }

    // Level structure of the component of `root` inside subset pid: fills
    // `levels` (vertex lists); returns the number of levels.
    int bfs(int root, int pid, std::vector<std::vector<int>> &levels, long long *used = nullptr)
    {
        const long long st = ++stamp;   // unique, and larger than any earlier search's
        if (used) *used = st;
        levels.assign(1, std::vector<int>{root});
        seen[root] = st;
        lev[root] = 0;
        for (int l = 0;; l++) {
            std::vector<int> nxt;
            for (int v : levels[l])
                for (long long k = xadj[v]; k < xadj[v + 1]; k++) {
                    int u = adj[k];
                    if (pid_of(u) != pid || seen[u] == st) continue;
                    seen[u] = st;
                    lev[u] = l + 1;
                    nxt.push_back(u);
                }
            if (nxt.empty()) break;
            levels.push_back(std::move(nxt));
        }
        return (int)levels.size();
    }

    long long weight(const std::vector<int> &vs) const
    {
        long long w = 0;
        for (int v : vs) w += wt[v];
        return w;
    }

    int min_degree_vertex(const std::vector<int> &vs, int pid) const
    {
        int best = vs[0], bd = degree(vs[0], pid);
        for (int v : vs) {
            int d = degree(v, pid);
            if (d < bd) { bd = d; best = v; }
        }
        return best;
    }

    // Split subset pid (vertices vs, weight W) into sep, s1, s2 with no edge
    // between s1 and s2; false if no useful split exists.
    bool split(const std::vector<int> &vs, int pid, long long W, unsigned long long seed, std::vector<int> &sep,
               std::vector<int> &s1, std::vector<int> &s2)
    {
        std::vector<std::vector<int>> L;
        int root = min_degree_vertex(vs, pid);
        long long s0 = 0;   // stamps only grow: seen[v] >= s0 marks this split's searches
        int nl = bfs(root, pid, L, &s0);
        long long reached = 0;
        for (auto &l : L) reached += weight(l);
        if (reached < W) {
            // disconnected: components, heaviest first, to the lighter group
            std::vector<std::vector<int>> comps(1);
            for (auto &l : L) comps[0].insert(comps[0].end(), l.begin(), l.end());
            for (int v : vs) {
                if (seen[v] >= s0) continue;
                std::vector<std::vector<int>> Lc;
                bfs(v, pid, Lc);
                std::vector<int> c;
                for (auto &l : Lc) c.insert(c.end(), l.begin(), l.end());
                comps.push_back(std::move(c));
            }
            std::sort(comps.begin(), comps.end(),
                      [&](const std::vector<int> &a, const std::vector<int> &b) { return weight(a) > weight(b); });
            std::vector<int> A, B;
            long long wa = 0, wb = 0;
            for (auto &c : comps) {
                long long w = weight(c);
                if (wa <= wb) { A.insert(A.end(), c.begin(), c.end()); wa += w; }
                else { B.insert(B.end(), c.begin(), c.end()); wb += w; }
            }
            if (B.size() < 2) std::swap(A, B);
            if (B.size() < 2) return false;   // two single supervariables heavier than a leaf
            int v = min_degree_vertex(B, pid);
            sep.assign(1, v);
            s1 = std::move(A);
            for (int u : B)
                if (u != v) s2.push_back(u);
            return true;
        }
        // pseudo-peripheral root: restart from a minimum-degree vertex of the
        // last level while the level structure gets deeper
        for (int it = 0; it < 3; it++) {
            int u = min_degree_vertex(L.back(), pid);
            std::vector<std::vector<int>> L2;
            int nl2 = bfs(u, pid, L2);
            if (nl2 <= nl) { bfs(root, pid, L); break; }
            root = u;
            nl = nl2;
            L.swap(L2);
        }
        if (nl < 3) return false;   // diameter < 2: nothing to separate
        std::vector<long long> lw(nl), cw(nl + 1, 0);
        for (int l = 0; l < nl; l++) { lw[l] = weight(L[l]); cw[l + 1] = cw[l] + lw[l]; }
        int s = -1;
        long long best_side = -1;
        for (int l = 1; l < nl - 1; l++) {
            long long side = std::min(cw[l], W - cw[l + 1]);
            if (5 * side < W) continue;
            if (s < 0 || lw[l] < lw[s] || (lw[l] == lw[s] && side > best_side)) { s = l; best_side = side; }
        }
        if (s < 0)
            for (int l = 1; l < nl - 1; l++) {
                long long side = std::min(cw[l], W - cw[l + 1]);
                if (side > best_side) { s = l; best_side = side; }
            }
        // thin the level: drop the vertices that touch only one side
        auto touches = [&](int v, bool later) {
            for (long long k = xadj[v]; k < xadj[v + 1]; k++) {
                int u = adj[k];
                if (pid_of(u) == pid && (later ? lev[u] > s : lev[u] < s)) return true;
            }
            return false;
        };
        std::vector<int> keepA, movA, keepB, movB;
        for (int v : L[s]) {
            (touches(v, true) ? keepA : movA).push_back(v);
            (touches(v, false) ? keepB : movB).push_back(v);
        }
        const bool useA = weight(keepA) <= weight(keepB);
        sep = useA ? keepA : keepB;
        for (int l = 0; l < s; l++) s1.insert(s1.end(), L[l].begin(), L[l].end());
        for (int l = s + 1; l < nl; l++) s2.insert(s2.end(), L[l].begin(), L[l].end());
        if (useA) s1.insert(s1.end(), movA.begin(), movA.end());
        else s2.insert(s2.end(), movB.begin(), movB.end());
        // the multilevel separator, if it is smaller
        std::vector<int> mSep, m1, m2;
        if (vs.size() >= 32 && multilevel(vs, pid, seed, mSep, m1, m2) &&
            split_score(mSep, m1, m2, W) < split_score(sep, s1, s2, W)) {
            sep.swap(mSep);
            s1.swap(m1);
            s2.swap(m2);
        }
#ifdef WT3D_HAVE_METIS
        // and METIS's vertex separator (the reference's ordering), if smaller still
        std::vector<int> tSep, t1, t2;
        if (vs.size() >= 32 && metis_separator(vs, pid, tSep, t1, t2) &&
            split_score(tSep, t1, t2, W) < split_score(sep, s1, s2, W)) {
            sep.swap(tSep);
            s1.swap(t1);
            s2.swap(t2);
        }
#endif
        return !sep.empty() && !s1.empty() && !s2.empty();
    }

#ifdef WT3D_HAVE_METIS
    // METIS_ComputeVertexSeparator on subset pid (calls serialised: the
    // library's thread safety is not documented).
    bool metis_separator(const std::vector<int> &vs, int pid, std::vector<int> &sep, std::vector<int> &s1,
                         std::vector<int> &s2)
    {
        int64_t n = (int64_t)vs.size();
        for (int64_t i = 0; i < n; i++) lid[vs[i]] = (int)i;
        std::vector<int64_t> xa(n + 1, 0), ad, vw(n), part(n, -1);
        for (int64_t i = 0; i < n; i++) {
            const int v = vs[i];
            vw[i] = wt[v];
            for (long long k = xadj[v]; k < xadj[v + 1]; k++)
                if (pid_of(adj[k]) == pid) ad.push_back(lid[adj[k]]);
            xa[i + 1] = (int64_t)ad.size();
        }
        if (ad.empty()) return false;
        int64_t opt[64] = {0}, sepsize = 0;
        int rc;
        {
            static std::mutex metis_mu;
            std::lock_guard<std::mutex> lk(metis_mu);
            if (METIS_SetDefaultOptions(opt) != 1) return false;
            rc = METIS_ComputeVertexSeparator(&n, xa.data(), ad.data(), vw.data(), opt, &sepsize, part.data());
        }
        if (rc != 1) return false;
        for (int64_t i = 0; i < n; i++) {
            if (part[i] < 0 || part[i] > 2) return false;
            (part[i] == 2 ? sep : part[i] == 0 ? s1 : s2).push_back(vs[i]);
        }
        // a vertex separator: no edge between the two sides
        for (int64_t i = 0; i < n; i++)
            if (part[i] < 2)
                for (int64_t k = xa[i]; k < xa[i + 1]; k++)
                    if (part[ad[k]] == 1 - part[i]) return false;
        return !sep.empty() && !s1.empty() && !s2.empty();
    }
#endif

    // Separator weight, or a penalty above any separator when a side holds
    // less than a fifth of the weight.
    long long split_score(const std::vector<int> &sep, const std::vector<int> &s1, const std::vector<int> &s2,
                          long long W) const
    {
        if (sep.empty() || s1.empty() || s2.empty()) return std::numeric_limits<long long>::max();
        const long long small = std::min(weight(s1), weight(s2));
        return 5 * small >= W ? weight(sep) : W + (W - small);
    }

    // Multilevel bisection of subset pid turned into a vertex separator.
    bool multilevel(const std::vector<int> &vs, int pid, unsigned long long seed, std::vector<int> &sep,
                    std::vector<int> &s1, std::vector<int> &s2)
    {
        LGraph g;
        g.n = (int)vs.size();
        for (int i = 0; i < g.n; i++) lid[vs[i]] = i;
        g.xadj.assign(g.n + 1, 0);
        g.vw.resize(g.n);
        for (int i = 0; i < g.n; i++) {
            const int v = vs[i];
            g.vw[i] = wt[v];
            for (long long k = xadj[v]; k < xadj[v + 1]; k++)
                if (pid_of(adj[k]) == pid) { g.adj.push_back(lid[adj[k]]); g.ew.push_back(1); }
            g.xadj[i + 1] = (long long)g.adj.size();
        }
        // large subsets (whose separators dominate the flops) try three
        // seeds, on threads of their own; the first lightest cover wins, so
        // the result does not depend on the threads
        const int tries = g.n >= 20000 ? 3 : 1;
        std::vector<std::vector<char>> sides(tries);
        std::vector<std::vector<int>> covers(tries);
        auto attempt = [&](int t) {
            ml_bisect(g, sides[t], seed * 7919ULL + (unsigned long long)t);
            covers[t] = cut_cover(g, sides[t]);
        };
        std::vector<std::thread> pool;
        std::exception_ptr err;
        std::mutex err_mu;
        for (int t = 1; t < tries; t++) {
            try {
                pool.emplace_back([&, t] {
                    try { attempt(t); }
                    catch (...) { std::lock_guard<std::mutex> lk(err_mu); err = std::current_exception(); }
                });
            } catch (const std::system_error &) {
                break;   // no thread: the remaining tries run below
            }
        }
        try {
            attempt(0);
            for (int t = (int)pool.size() + 1; t < tries; t++) attempt(t);
        } catch (...) {
            std::lock_guard<std::mutex> lk(err_mu);
            err = std::current_exception();
        }
        for (auto &th : pool) th.join();
        if (err) std::rethrow_exception(err);
        int bt = 0;
        long long best_w = -1;
        for (int t = 0; t < tries; t++) {
            long long w = 0;
            for (int i : covers[t]) w += g.vw[i];
            if (best_w < 0 || w < best_w) { best_w = w; bt = t; }
        }
        std::vector<char> side;
        std::vector<int> cover;
        side.swap(sides[bt]);
        cover.swap(covers[bt]);
        std::vector<char> inc(g.n, 0);
        for (int i : cover) inc[i] = 1;
        for (int i = 0; i < g.n; i++) (inc[i] ? sep : side[i] == 0 ? s1 : s2).push_back(vs[i]);
        return !sep.empty() && !s1.empty() && !s2.empty();
    }

    // seed: the random streams of this subtree's bisections, fixed by the
    // position in the tree so that the ordering does not depend on threads
    std::unique_ptr<Node> dissect(std::vector<int> vs, int pid, int depth, unsigned long long seed)
    {
        std::unique_ptr<Node> nd(new Node());
        nd->depth = depth;
        const long long W = weight(vs);
        std::vector<int> s1, s2;
        if (W > leaf && depth < MAXDEPTH && split(vs, pid, W, seed, nd->nodes, s1, s2)) {
            const int p1 = next_part++, p2 = next_part++;
            for (int v : s1) set_pid(v, p1);
            for (int v : s2) set_pid(v, p2);
            for (int v : nd->nodes) set_pid(v, -1);
            std::vector<int>().swap(vs);
            if (depth < par_depth && s1.size() + s2.size() >= 20000) {
                // the first subtree on a thread of its own (sequentially if no
                // thread can be made); errors of either side reach the caller
                std::exception_ptr e1, e2;
                std::thread t;
                try {
                    t = std::thread([&] {
                        try { nd->child[0] = dissect(std::move(s1), p1, depth + 1, 2 * seed + 1); }
                        catch (...) { e1 = std::current_exception(); }
                    });
                } catch (const std::system_error &) {
                }
                try {
                    if (!t.joinable()) nd->child[0] = dissect(std::move(s1), p1, depth + 1, 2 * seed + 1);
                    nd->child[1] = dissect(std::move(s2), p2, depth + 1, 2 * seed + 2);
                } catch (...) {
                    e2 = std::current_exception();
                }
                if (t.joinable()) t.join();
                if (e1) std::rethrow_exception(e1);
                if (e2) std::rethrow_exception(e2);
            } else {
                nd->child[0] = dissect(std::move(s1), p1, depth + 1, 2 * seed + 1);
                nd->child[1] = dissect(std::move(s2), p2, depth + 1, 2 * seed + 2);
            }
        } else {
            nd->nodes = std::move(vs);
            for (int v : nd->nodes) set_pid(v, -1);
        }
        return nd;
    }

    // Fronts in postorder: children first, then the separator.
    int number(Node &nd)
    {
        Front f;
        f.level = nd.depth;
        for (int c = 0; c < 2; c++)
            if (nd.child[c]) f.child[f.nchild++] = number(*nd.child[c]);
        const int id = (int)S.fronts.size();
        for (int c = 0; c < f.nchild; c++) S.fronts[f.child[c]].parent = id;
        S.fronts.push_back(f);
        snodes.push_back(std::move(nd.nodes));
        return id;
    }
};

}  // namespace

int check_csr(long long n, long long nnz, const int *irptr, const int *jcptr, int base, bool need_symmetric)
{
    if (n < 1 || n >= (1LL << 31) || nnz < 0 || nnz >= (1LL << 31) || !irptr || (nnz > 0 && !jcptr) ||
        (base != 0 && base != 1)) {
        set_error("CSR: bad sizes, pointers or index base");
        return WT3D_ERR_ARG;
    }
    if (irptr[0] != base || (long long)irptr[n] - base != nnz) {
        set_error("CSR: row pointers do not start at the index base or do not end at nnz");
        return WT3D_ERR_PATTERN;
    }
    std::vector<int> mark(n, -1), cnt(n, 0);
    for (long long r = 0; r < n; r++) {
        if (irptr[r + 1] < irptr[r]) { set_error("CSR: row pointers decrease"); return WT3D_ERR_PATTERN; }
        for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) {
            long long c = (long long)jcptr[k] - base;
            if (c < 0 || c >= n) { set_error("CSR: column index out of range"); return WT3D_ERR_PATTERN; }
            if (mark[c] == r) { set_error("CSR: duplicate entry in a row"); return WT3D_ERR_PATTERN; }
            mark[c] = (int)r;
            cnt[c]++;
        }
    }
    if (!need_symmetric) return WT3D_OK;
    // structural symmetry: column c holds as many entries as row c, and every
    // (r, c) has its (c, r)
    for (long long r = 0; r < n; r++)
        if (cnt[r] != irptr[r + 1] - irptr[r]) { set_error("CSR: pattern is not structurally symmetric"); return WT3D_ERR_PATTERN; }
    std::vector<long long> tptr(n + 1, 0);
    for (long long r = 0; r < n; r++) tptr[r + 1] = tptr[r] + cnt[r];
    std::vector<int> trow(nnz);
    {
        std::vector<long long> cur(tptr.begin(), tptr.end() - 1);
        for (long long r = 0; r < n; r++)
            for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) trow[cur[jcptr[k] - base]++] = (int)r;
    }
    std::fill(mark.begin(), mark.end(), -1);
    for (long long r = 0; r < n; r++) {
        for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) mark[jcptr[k] - base] = (int)r;
        for (long long k = tptr[r]; k < tptr[r + 1]; k++)
            if (mark[trow[k]] != r) { set_error("CSR: pattern is not structurally symmetric"); return WT3D_ERR_PATTERN; }
    }
    return WT3D_OK;
}

int symmetrize(long long n, const int *irptr, const int *jcptr, int base, std::vector<int> &sir,
               std::vector<int> &sjc, std::vector<int> &vmap)
{
    const long long nnz = (long long)irptr[n] - base;
    // transpose lists: the rows holding each column
    std::vector<long long> tptr(n + 1, 0);
    for (long long k = 0; k < nnz; k++) tptr[jcptr[k] - base + 1]++;
    for (long long r = 0; r < n; r++) tptr[r + 1] += tptr[r];
    std::vector<int> trow(nnz);
    {
        std::vector<long long> cur(tptr.begin(), tptr.end() - 1);
        for (long long r = 0; r < n; r++)
            for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) trow[cur[jcptr[k] - base]++] = (int)r;
    }
    // row r of A + A^T: row r of A, then the transposed entries it lacks
    std::vector<int> mark(n, -1);
    sir.assign(n + 1, 0);
    sjc.clear();
    sjc.reserve(nnz);
    bool symmetric = true;
    for (long long r = 0; r < n; r++) {
        for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) {
            mark[jcptr[k] - base] = (int)r;
            sjc.push_back(jcptr[k] - base);
        }
        for (long long k = tptr[r]; k < tptr[r + 1]; k++)
            if (mark[trow[k]] != (int)r) {
                mark[trow[k]] = (int)r;
                sjc.push_back(trow[k]);
                symmetric = false;
            }
        if ((long long)sjc.size() >= (1LL << 31)) {
            set_error("CSR: the symmetrised pattern has 2^31 entries or more");
            return WT3D_ERR_ARG;
        }
        sir[r + 1] = (int)sjc.size();
    }
    vmap.clear();
    if (symmetric) return WT3D_OK;   // the caller's own order, no value map
    // rows of the union in column order
    for (long long r = 0; r < n; r++) std::sort(sjc.begin() + sir[r], sjc.begin() + sir[r + 1]);
    vmap.resize(nnz);
    for (long long r = 0; r < n; r++) {
        const auto b = sjc.begin() + sir[r], e = sjc.begin() + sir[r + 1];
        for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++)
            vmap[k] = (int)(std::lower_bound(b, e, jcptr[k] - base) - sjc.begin());
    }
    return WT3D_OK;
}

static int symbolic_graph_impl(long long n, const int *irptr, const int *jcptr, int base, long long leaf_dofs,
                               Symbolic &S);

int symbolic_graph(long long n, const int *irptr, const int *jcptr, int base, long long leaf_dofs, Symbolic &S)
{
    try {
        return symbolic_graph_impl(n, irptr, jcptr, base, leaf_dofs, S);
    } catch (const std::bad_alloc &) {
        set_error("symbolic_graph: out of host memory");
        return WT3D_ERR_NOMEM;
    }
}

static int symbolic_graph_impl(long long n, const int *irptr, const int *jcptr, int base, long long leaf_dofs,
                               Symbolic &S)
{
    if (n < 1 || !irptr) { set_error("symbolic_graph: empty matrix or null row pointers"); return WT3D_ERR_ARG; }
    int rc = check_csr(n, (long long)irptr[n] - base, irptr, jcptr, base, true);
    if (rc) return rc;
    S = Symbolic();
    S.n = n;
    S.nnodes = 0;
    GraphND G(S);
    G.leaf = std::max(1LL, leaf_dofs);
    // ---- supervariables: runs of consecutive rows with equal column sets ----
    std::vector<int> sv_of(n), mark(n, -1);
    for (long long r = 0; r < n; r++) {
        bool same = false;
        if (r > 0) {
            const long long len = irptr[r + 1] - irptr[r], plen = irptr[r] - irptr[r - 1];
            if (len == plen) {
                for (long long k = irptr[r - 1] - base; k < irptr[r] - base; k++) mark[jcptr[k] - base] = (int)r;
                same = true;
                for (long long k = irptr[r] - base; k < irptr[r + 1] - base && same; k++)
                    same = mark[jcptr[k] - base] == (int)r;
            }
        }
        if (same) {
            sv_of[r] = G.nv - 1;
            G.wt[G.nv - 1]++;
        } else {
            sv_of[r] = G.nv++;
            G.wt.push_back(1);
            G.first_dof.push_back((int)r);
        }
    }
    // ---- quotient graph ----
    G.xadj.assign(G.nv + 1, 0);
    std::vector<int> smark(G.nv, -1);
    for (int v = 0; v < G.nv; v++) {
        const long long r = G.first_dof[v];
        smark[v] = v;
        for (long long k = irptr[r] - base; k < irptr[r + 1] - base; k++) {
            const int u = sv_of[jcptr[k] - base];
            if (smark[u] == v) continue;
            smark[u] = v;
            G.adj.push_back(u);
        }
        G.xadj[v + 1] = (long long)G.adj.size();
    }
    S.nnodes = G.nv;
    // ---- nested dissection ----
    G.part.reset(new std::atomic<int>[G.nv]);
    for (int v = 0; v < G.nv; v++) G.set_pid(v, 0);
    G.lev.assign(G.nv, 0);
    G.seen.assign(G.nv, 0);
    G.lid.assign(G.nv, -1);
    {
        // about one thread per hardware thread at the deepest threaded level
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        int d = 0;
        while ((1u << (d + 1)) <= hw && d < 6) d++;
        G.par_depth = std::max(1, d);
    }
    std::vector<int> all(G.nv);
    for (int v = 0; v < G.nv; v++) all[v] = v;
    std::unique_ptr<GraphND::Node> root = G.dissect(std::move(all), 0, 0, 1);
    G.number(*root);
    root.reset();
    const int nf = (int)S.fronts.size();
    // ---- numbering: fronts in postorder, supervariables in list order ----
    std::vector<int> newsv(G.nv), dof0(G.nv);
    {
        int q = 0;
        long long d = 0;
        for (int f = 0; f < nf; f++) {
            Front &F = S.fronts[f];
            F.first = (int)d;
            for (int v : G.snodes[f]) { newsv[v] = q++; dof0[v] = (int)d; d += G.wt[v]; }
            F.p = (int)(d - F.first);
        }
    }
    std::vector<int> sv_new(G.nv);   // new supervariable index -> supervariable
    for (int v = 0; v < G.nv; v++) sv_new[newsv[v]] = v;
    // ---- borders: struct on supervariables, children before parents ----
    std::vector<std::vector<int>> sn_struct(nf);
    std::fill(smark.begin(), smark.end(), -1);
    for (int f = 0; f < nf; f++) {
        Front &F = S.fronts[f];
        const int last_new = newsv[G.snodes[f].back()];
        std::vector<int> st;
        auto add = [&](int nw) {
            if (nw > last_new && smark[nw] != f) { smark[nw] = f; st.push_back(nw); }
        };
        for (int v : G.snodes[f])
            for (long long k = G.xadj[v]; k < G.xadj[v + 1]; k++) add(newsv[G.adj[k]]);
        for (int c = 0; c < F.nchild; c++) {
            for (int w : sn_struct[F.child[c]]) add(w);
            std::vector<int>().swap(sn_struct[F.child[c]]);
        }
        std::sort(st.begin(), st.end());
        F.border_off = (long long)S.border.size();
        for (int w : st) {
            const int v = sv_new[w];
            for (int q = 0; q < G.wt[v]; q++) S.border.push_back(dof0[v] + q);
        }
        F.b = (int)((long long)S.border.size() - F.border_off);
        sn_struct[f] = std::move(st);
    }
    // ---- permutation ----
    S.perm.resize(n);
    S.iperm.resize(n);
    for (int v = 0; v < G.nv; v++)
        for (int q = 0; q < G.wt[v]; q++) {
            S.perm[dof0[v] + q] = G.first_dof[v] + q;
            S.iperm[G.first_dof[v] + q] = dof0[v] + q;
        }
    return finalize(S, "symbolic_graph");
}

std::vector<long long> transpose_positions(long long n, const int *irptr, const int *jcptr)
{
    // Rows are walked in increasing order, so the t-th entry to reach column c
    // comes from the t-th smallest row holding c, whose transpose (c, r) is
    // the t-th entry of row c in column order.
    const long long nnz = irptr[n];
    std::vector<int> srt(nnz);   // per row: entry offsets in column order
    for (long long r = 0; r < n; r++) {
        const long long k0 = irptr[r], k1 = irptr[r + 1];
        bool sorted = true;
        for (long long k = k0; k < k1; k++) {
            srt[k] = (int)(k - k0);
            if (k > k0 && jcptr[k] < jcptr[k - 1]) sorted = false;
        }
        if (!sorted)
            std::sort(srt.begin() + k0, srt.begin() + k1,
                      [&](int x, int y) { return jcptr[k0 + x] < jcptr[k0 + y]; });
    }
    std::vector<long long> cur(irptr, irptr + n), tp(nnz);
    for (long long r = 0; r < n; r++)
        for (long long k = irptr[r]; k < irptr[r + 1]; k++) {
            const int c = jcptr[k];
            tp[k] = irptr[c] + srt[cur[c]++];
        }
    return tp;
}

int scatter_map(const Symbolic &S, const std::vector<int> &irptr, const std::vector<int> &jcptr,
                std::vector<long long> &map)
{
    const long long n = S.n;
    const long long nnz = irptr[n];
    map.assign(nnz, -1);
    // transposed position of every entry (structurally symmetric pattern)
    const std::vector<long long> tpos = transpose_positions(n, irptr.data(), jcptr.data());
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
