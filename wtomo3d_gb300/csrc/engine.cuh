// Multifrontal engine: device storage of the fronts, the static launch
// schedule of the factorisation and of the solves, and their execution.
#pragma once
#include "internal.h"
#include "mf_kernels.cuh"
#include "devvec.cuh"
#include "tc_gemm.h"
#include <type_traits>
#include <cstdlib>
#include <functional>
#include <map>
#include <memory>
#include <mutex>

namespace wt3d {

using Launch = std::function<void(cudaStream_t)>;

// Launch kinds, for the per-kernel profile.
enum LaunchKind { LK_MEMSET = 0, LK_SCATTER, LK_EXTEND_ADD, LK_PANEL, LK_TRSM, LK_GEMM, LK_SUBSTEP, LK_SPLIT,
                  LK_TCGEMM, LK_NKINDS };

struct LaunchRec {
    Launch fn;
    int kind;
    double flops;        // real-flop count of a GEMM launch (sum of 8 M N K)
    double bytes = 0;    // operand bytes of a GEMM launch (A, B read; C read and written)
};

// A list of launches plus the task arrays they read.
template <class T>
struct Schedule {
    std::vector<LaunchRec> launches;
    int kernels() const
    {
        int c = 0;
        for (auto &l : launches) c += l.kind != LK_MEMSET;
        return c;
    }
    DevVec<PanelTask> panel;
    DevVec<RowTask> row;
    DevVec<ColTask> col;
    DevVec<GemmTask<T>> gemm;
    DevVec<EATask> ea;
    DevVec<StepTask> step;                                    // fused substitution steps
    DevVec<cx<T>> zs;                                         // their per-front scratch slots
    std::vector<std::vector<GemmTask<float>>> tc_pending;   // tensor-core task lists, built after allocation
    std::vector<std::unique_ptr<TcLaunch>> tc;
    std::vector<std::vector<GemmTask<float>>> ts_pending;   // tall-skinny tensor-core task lists (solves)
    std::vector<char> ts_tma;                                 // ... whose A is streamed by TMA
    std::vector<std::unique_ptr<TsLaunch>> ts;
    DevVec<float> tsws;                                       // their expanded right-hand sides
    cudaGraphExec_t graph = nullptr;
    ~Schedule()
    {
        if (graph) cudaGraphExecDestroy(graph);
    }
};

// Buffers a factorisation needs only while it runs: the two level-parity
// update buffers and the tensor-core split-operand workspace.  Handles of the
// same grid and precision share one; `mu` serialises their factorisations.
template <class T>
struct FactorWorkspace {
    DevVec<cx<T>> upd0, upd1;
    DevVec<float> tcws;
    std::mutex mu;
    size_t bytes() const { return (upd0.n + upd1.n) * sizeof(cx<T>) + tcws.n * sizeof(float); }
};

template <class T>
class Engine {
public:
    const Symbolic *S = nullptr;
    DevVec<cx<T>> fac, X, dinv;   // dinv: per KB panel L_D^{-1}, U_D^{-1} (KB x KB each)
    std::shared_ptr<FactorWorkspace<T>> ws;
    DevVec<int> ipiv, border;
    DevVec<int> pord;   // per KB panel: the stored row at each position after its interchanges
    DevVec<int> rel;
    DevVec<FrontDev> fr;
    DevVec<long long> map;
    DevVec<int> npert;
    DevVec<unsigned long long> maxabs;
    std::unique_ptr<Schedule<T>> fsched;
    std::map<int, std::unique_ptr<Schedule<T>>> ssched[2];   // [adjoint][m]
    // outer block width of the two-level LU (WT3D_WB: a multiple of KB, 512 by default)
    const int WB = [] {
        const char *e = getenv("WT3D_WB");
        const int v = e ? atoi(e) : 512;
        return (v >= KB && v % KB == 0) ? v : 512;
    }();
    static constexpr int WS = 512;   // outer block width of the blocked substitutions
    // pivots below pivot_rel times the largest entry are perturbed: only
    // (near-)zero ones, since Dirichlet rows carry unit pivots next to O(1e8)
    // stiffness entries
    double pivot_rel = 1e-20;
    // tcgen05 path for complex64 front updates (WT3D_TC=0 selects the SIMT kernel)
    bool use_tc = std::is_same<T, float>::value && !(getenv("WT3D_TC") && getenv("WT3D_TC")[0] == '0');
    // tcgen05 path for the large blocks of complex64 substitution passes (WT3D_TS=0: SIMT)
    bool use_ts = std::is_same<T, float>::value && !(getenv("WT3D_TS") && getenv("WT3D_TS")[0] == '0');
    bool building_solve = false;   // set while a solve schedule is built: only those route to the TS kernel
    DevVec<float> own_tcws;   // private split workspace, only if the shared one is too small
    DevVec<int> tc_err;                                 // barrier-timeout flag of the tensor-core kernel
    std::vector<Schedule<T> *> built_tc;   // schedules whose tensor maps point into the split workspace
    // launch schedules as captured CUDA graphs (WT3D_GRAPHS=0: direct launches, for profilers)
    bool use_graphs = !(getenv("WT3D_GRAPHS") && getenv("WT3D_GRAPHS")[0] == '0');

    // device bytes this engine holds on its own (the shared workspace excluded)
    size_t device_bytes() const
    {
        size_t sw = 0;   // the solve schedules' tall-skinny workspaces
        for (const auto &m : ssched)
            for (const auto &kv : m) sw += kv.second->tsws.n * sizeof(float);
        return (fac.n + X.n + dinv.n) * sizeof(cx<T>) + (ipiv.n + border.n + rel.n + pord.n) * 4 + fr.n * sizeof(FrontDev) +
               map.n * 8 + scale.n * 8 + own_tcws.n * sizeof(float) + sw;
    }

    // Reads (and clears) the barrier-timeout flag of the tensor-core kernels;
    // call after the stream that ran them is synchronised.
    int check_tc_err()
    {
        int e = 0;
        WT_CUDA(cudaMemcpy(&e, tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (!e) return WT3D_OK;
        WT_CUDA(cudaMemset(tc_err.p, 0, sizeof(int)));
        set_error("tensor-core kernel: mbarrier wait expired (code " + std::to_string(e) + ")");
        return WT3D_ERR_CUDA;
    }
    size_t workspace_bytes() const { return ws ? ws->bytes() : 0; }
    // split workspace of the tensor-core launches: private if allocated, else the shared one
    float *tcws_base() const { return own_tcws.p ? own_tcws.p : ws->tcws.p; }
    size_t tcws_size() const { return own_tcws.p ? own_tcws.n : ws->tcws.n; }

    const int *d_irptr = nullptr, *d_jcptr = nullptr;   // natural 0-based CSR of the operator
    DevVec<double> scale;                              // Jacobi scaling 1/sqrt|a_ii|, natural ordering

    int init(const Symbolic &sym, const std::vector<long long> &hmap, const int *irp, const int *jcp,
             std::shared_ptr<FactorWorkspace<T>> w)
    {
        S = &sym;
        d_irptr = irp;
        d_jcptr = jcp;
        ws = w ? w : std::make_shared<FactorWorkspace<T>>();
        int rc;
        if ((rc = fac.alloc(sym.fac_total))) return rc;
        {
            std::lock_guard<std::mutex> lk(ws->mu);
            const size_t n0 = std::max<long long>(sym.upd_size[0], 1), n1 = std::max<long long>(sym.upd_size[1], 1);
            if (ws->upd0.n < n0 && (rc = ws->upd0.alloc(n0))) return rc;
            if (ws->upd1.n < n1 && (rc = ws->upd1.alloc(n1))) return rc;
        }
        if ((rc = X.alloc((size_t)sym.n * MAXRHS))) return rc;
        if ((rc = ipiv.alloc(sym.n))) return rc;
        if ((rc = border.upload(sym.border))) return rc;
        if ((rc = rel.upload(sym.rel))) return rc;
        if ((rc = map.upload(hmap))) return rc;
        if ((rc = npert.alloc(1))) return rc;
        if ((rc = maxabs.alloc(1))) return rc;
        if ((rc = scale.alloc(sym.n))) return rc;
        if ((rc = tc_err.alloc(1))) return rc;
        WT_CUDA(cudaMemset(tc_err.p, 0, sizeof(int)));
        if (use_tc && (rc = tc_init())) return rc;
        if (use_ts && (rc = ts_init())) return rc;
        std::vector<FrontDev> h(sym.fronts.size());
        long long npan = 0;
        for (size_t f = 0; f < h.size(); f++) {
            h[f].pan = (int)npan;
            npan += (sym.fronts[f].p + KB - 1) / KB;
            const Front &F = sym.fronts[f];
            h[f].fac = F.fac_off;
            h[f].upd = F.upd_off;
            h[f].border = F.border_off;
            h[f].p = F.p;
            h[f].b = F.b;
            h[f].first = F.first;
            h[f].parity = F.level & 1;
        }
        if ((rc = fr.upload(h))) return rc;
        if ((rc = dinv.alloc((size_t)npan * 2 * KB * KB))) return rc;
        if ((rc = pord.alloc((size_t)npan * KB))) return rc;
        // kernel attributes are per device: once for each device this process uses
        static std::once_flag attr_once[64];
        int dev = 0;
        cudaGetDevice(&dev);
        std::call_once(attr_once[dev & 63], [] {
            size_t sp = sizeof(cx<T>) * (KB * (KB + 1) + 2 * KB * (KB + 1));
            cudaFuncSetAttribute(k_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp);
            cudaFuncSetAttribute(k_tile_inverse<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sp);
            cudaFuncSetAttribute(k_trsm_row<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(cx<T>) * (KB * (KB + 1) + KB * (TRW + 1))));
            cudaFuncSetAttribute(k_trsm_col<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(cx<T>) * (KB * (KB + 1) + TCR * (KB + 1))));
            if constexpr (std::is_same<T, float>::value) {
                cudaFuncSetAttribute(k_trsm_row_h<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)band_row_smem());
                cudaFuncSetAttribute(k_trsm_col_h<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)band_col_smem());
            }
            cudaFuncSetAttribute(k_sub_step<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(cx<T>) * sub_step_smem_elems()));
        });
        return build_factor_schedule();
    }

    // ---------------------------------------------------------------------
    static void add_gemm(std::vector<GemmTask<T>> &v, long long &tiles, const cx<T> *A, int lda, const cx<T> *B,
                         int ldb, cx<T> *C, int ldc, int M, int N, int K, const int *brow = nullptr,
                         const int *crow = nullptr, int conjA = 0)
    {
        if (M <= 0 || N <= 0 || K <= 0) return;
        GemmTask<T> g{};
        g.A = A; g.B = B; g.C = C; g.brow = brow; g.crow = crow;
        g.lda = lda; g.ldb = ldb; g.ldc = ldc; g.M = M; g.N = N; g.K = K;
        g.tiles_n = (N + GBN - 1) / GBN;
        g.tile0 = tiles;
        g.conjA = conjA;
        tiles += (long long)((M + GBM - 1) / GBM) * g.tiles_n;
        v.push_back(g);
    }

    static double gemm_bytes(const GemmTask<T> &g)
    {
        return ((double)g.M * g.K + (double)g.K * g.N + 2.0 * g.M * g.N) * sizeof(cx<T>);
    }

    // Appends the launches for GEMM tasks [b, end) of `all`: tasks the
    // tensor-core kernel takes (complex64 path) go to a tcgen05 launch, the
    // rest to the SIMT kernel with tile numbering rebased to the launch.
    void push_gemm_launch(Schedule<T> &sc, std::vector<GemmTask<T>> &all, size_t b, long long /*tiles*/)
    {
        if (all.size() == b) return;
        std::vector<GemmTask<T>> simt;
        if constexpr (std::is_same<T, float>::value) {
            std::vector<GemmTask<float>> tcv;
            for (size_t i = b; i < all.size(); i++) {
                if (use_tc && tc_eligible(all[i])) tcv.push_back(all[i]);
                else simt.push_back(all[i]);
            }
            if (!tcv.empty()) {
                double fl = 0, by = 0;
                for (auto &g : tcv) { fl += 8.0 * g.M * (double)g.N * g.K; by += gemm_bytes(g); }
                const int idx = (int)sc.tc_pending.size();
                sc.tc_pending.push_back(std::move(tcv));
                Schedule<T> *psc = &sc;
                sc.launches.push_back({[psc, idx](cudaStream_t st) { tc_split(*psc->tc[idx], st); }, LK_SPLIT, 0});
                sc.launches.push_back({[psc, idx, this](cudaStream_t st) { tc_mma(*psc->tc[idx], tc_err.p, st); },
                                       LK_TCGEMM, fl, by});
            }
            if (use_ts && building_solve) {
                // blocks TMA can address (16-byte aligned, even stride) and the rest:
                // one tall-skinny launch each
                std::vector<GemmTask<float>> tsv[2], rest;
                for (auto &g : simt) {
                    if (!ts_eligible(g)) rest.push_back(g);
                    else tsv[ts_tma_ok(g) ? 1 : 0].push_back(g);
                }
                for (int tma = 0; tma < 2; tma++) {
                    if (tsv[tma].empty()) continue;
                    double fl = 0, by = 0;
                    for (auto &g : tsv[tma]) { fl += 8.0 * g.M * (double)g.N * g.K; by += gemm_bytes(g); }
                    const int idx = (int)sc.ts_pending.size();
                    sc.ts_pending.push_back(std::move(tsv[tma]));
                    sc.ts_tma.push_back((char)tma);
                    Schedule<T> *psc = &sc;
                    sc.launches.push_back({[psc, idx](cudaStream_t st) { ts_expand(*psc->ts[idx], st); }, LK_SPLIT, 0});
                    sc.launches.push_back({[psc, idx, this](cudaStream_t st) { ts_mma(*psc->ts[idx], tc_err.p, st); },
                                           LK_TCGEMM, fl, by});
                }
                simt.swap(rest);
            }
        } else {
            simt.assign(all.begin() + b, all.end());
        }
        all.resize(b);
        if (simt.empty()) return;
        // tasks with at most 32 columns go to the tall-skinny kernel
        std::vector<GemmTask<T>> narrow, wide;
        for (auto &g : simt) (g.N <= TSBN ? narrow : wide).push_back(g);
        Schedule<T> *psc = &sc;
        if (!narrow.empty()) {
            // split-K: tasks whose K exceeds a chunk sized for ~8 CTAs per SM
            // over the whole launch are cut into K-chunks that subtract their
            // partial products atomically
            double work = 0;
            for (auto &g : narrow) work += (double)((g.M + TSBM - 1) / TSBM) * g.K;
            const int kchunk = std::max(256, (int)((work / (8.0 * 152) + TSBK - 1) / TSBK) * TSBK);
            std::vector<GemmTask<T>> split;
            for (auto &g : narrow) {
                if (g.K <= kchunk + kchunk / 2) { split.push_back(g); continue; }
                for (int k0 = 0; k0 < g.K; k0 += kchunk) {
                    GemmTask<T> c = g;
                    c.K = std::min(kchunk, g.K - k0);
                    c.A = g.conjA ? g.A + (long long)k0 * g.lda : g.A + k0;
                    if (g.brow) c.brow = g.brow + k0;
                    else c.B = g.B + (long long)k0 * g.ldb;
                    c.atom = 1;
                    split.push_back(c);
                }
            }
            narrow.swap(split);
            const size_t b0 = all.size();
            long long tiles = 0;
            double fl = 0, by = 0;
            for (auto &g : narrow) {
                g.tile0 = tiles;
                tiles += (g.M + TSBM - 1) / TSBM;
                fl += 8.0 * g.M * (double)g.N * g.K;
                by += gemm_bytes(g);
                all.push_back(g);
            }
            const int nt = (int)narrow.size();
            sc.launches.push_back({[psc, b0, nt, tiles](cudaStream_t st) {
                k_gemm_ts<T><<<(unsigned)tiles, 256, 0, st>>>(psc->gemm.p + b0, nt);
            }, LK_GEMM, fl, by});
        }
        if (!wide.empty()) {
            const size_t b0 = all.size();
            long long tiles = 0;
            double fl = 0, by = 0;
            for (auto &g : wide) {
                g.tile0 = tiles;
                tiles += (long long)((g.M + GBM - 1) / GBM) * g.tiles_n;
                fl += 8.0 * g.M * (double)g.N * g.K;
                by += gemm_bytes(g);
                all.push_back(g);
            }
            const int nt = (int)wide.size();
            sc.launches.push_back({[psc, b0, nt, tiles](cudaStream_t st) {
                k_gemm<T><<<(unsigned)tiles, 256, 0, st>>>(psc->gemm.p + b0, nt);
            }, LK_GEMM, fl, by});
        }
    }

    // Allocates a solve schedule's own B~ workspace (sized for its largest
    // tall-skinny launch; launches run one after another) and builds the
    // tensor maps of its tall-skinny tensor-core launches.
    int finish_ts(Schedule<T> &sc)
    {
        if constexpr (std::is_same<T, float>::value) {
            long long need = 0;
            for (auto &v : sc.ts_pending) need = std::max(need, ts_workspace_floats(v.data(), (int)v.size()));
            if (need == 0) return WT3D_OK;
            int rc;
            if ((rc = sc.tsws.alloc(need))) return rc;
            sc.ts.clear();
            for (size_t i = 0; i < sc.ts_pending.size(); i++) {
                auto &v = sc.ts_pending[i];
                sc.ts.emplace_back(new TsLaunch());
                if ((rc = ts_build_launch(*sc.ts.back(), v.data(), (int)v.size(), sc.tsws.p, sc.ts_tma[i] != 0)))
                    return rc;
            }
        }
        return WT3D_OK;
    }

    // Allocates the shared tensor-core workspace and builds the tensor maps of
    // every pending tensor-core launch of a schedule.
    int finish_tc(Schedule<T> &sc)
    {
        if constexpr (std::is_same<T, float>::value) {
            long long need = 0;
            for (auto &v : sc.tc_pending) need = std::max(need, tc_workspace_floats(v.data(), (int)v.size()));
            if (need > 0 && tcws_base() == nullptr) {
                // first user of the shared workspace sizes it
                std::lock_guard<std::mutex> lk(ws->mu);
                if (ws->tcws.n == 0) {
                    int rc = ws->tcws.alloc(need);
                    if (rc) return rc;
                }
            }
            if (need > (long long)tcws_size()) {
                int rc = own_tcws.alloc(need);
                if (rc) return rc;
                // schedules built earlier point into the old workspace: rebuild their maps
                for (auto *o : built_tc) {
                    for (size_t i = 0; i < o->tc_pending.size(); i++) {
                        o->tc[i].reset(new TcLaunch());
                        if ((rc = tc_build_launch(*o->tc[i], o->tc_pending[i].data(), (int)o->tc_pending[i].size(),
                                                  tcws_base())))
                            return rc;
                    }
                    if (o->graph) { cudaGraphExecDestroy(o->graph); o->graph = nullptr; }
                }
            }
            sc.tc.clear();
            for (auto &v : sc.tc_pending) {
                sc.tc.emplace_back(new TcLaunch());
                int rc = tc_build_launch(*sc.tc.back(), v.data(), (int)v.size(), tcws_base());
                if (rc) return rc;
            }
            built_tc.push_back(&sc);
        }
        return WT3D_OK;
    }

    int build_factor_schedule()
    {
        auto sc = std::make_unique<Schedule<T>>();
        std::vector<PanelTask> hp;
        std::vector<RowTask> hr;
        std::vector<ColTask> hc;
        std::vector<GemmTask<T>> hg;
        std::vector<EATask> he;
        Schedule<T> *psc = sc.get();
        const Symbolic &sym = *S;
        cx<T> *F = fac.p;
        cx<T> *U[2] = {ws->upd0.p, ws->upd1.p};
        // zero the factor pool, scale and scatter the operator
        {
            cx<T> *fp = F; size_t bytes = fac.n * sizeof(cx<T>);
            long long *mp = map.p;
            Engine<T> *self = this;
            const long long n = sym.n;
            sc->launches.push_back({[fp, bytes](cudaStream_t st) { cudaMemsetAsync(fp, 0, bytes, st); }, LK_MEMSET, 0});
            sc->launches.push_back({[self, n](cudaStream_t st) {
                k_jacobi_scale<<<ceil_div(n, 256), 256, 0, st>>>(n, self->d_irptr, self->d_jcptr, self->a_dev,
                                                                 self->scale.p);
            }, LK_SCATTER, 0});
            sc->launches.push_back({[self, mp, n, fp](cudaStream_t st) {
                k_scatter<T><<<ceil_div(n, 256), 256, 0, st>>>(n, self->d_irptr, self->d_jcptr, mp, self->a_dev,
                                                               self->scale.p, fp);
            }, LK_SCATTER, 0});
        }
        const int nlev = (int)sym.levels.size();
        for (int L = nlev - 1; L >= 0; L--) {
            const std::vector<int> &fl = sym.levels[L];
            // zero this level's update region
            long long usz = 0;
            for (int f : fl) usz += (long long)sym.fronts[f].b * sym.fronts[f].b;
            if (usz > 0) {
                cx<T> *up = U[L & 1];
                size_t bytes = usz * sizeof(cx<T>);
                sc->launches.push_back({[up, bytes](cudaStream_t st) { cudaMemsetAsync(up, 0, bytes, st); }, LK_MEMSET, 0});
            }
            // extend-add, one child slot at a time (siblings overlap in the parent)
            for (int slot = 0; slot < 2; slot++) {
                size_t b0 = he.size();
                long long rows = 0;
                for (int f : fl) {
                    const Front &P = sym.fronts[f];
                    if (P.nchild <= slot) continue;
                    int c = P.child[slot];
                    if (sym.fronts[c].b == 0) continue;
                    he.push_back(EATask{c, f, rows});
                    rows += sym.fronts[c].b;
                }
                if (he.size() > b0) {
                    int nt = (int)(he.size() - b0);
                    sc->launches.push_back({[psc, this, b0, nt, rows](cudaStream_t st) {
                        k_extend_add<T><<<ceil_div(rows * 32, 256), 256, 0, st>>>(
                            psc->ea.p + b0, nt, rows, fr.p, rel.p, fac.p, ws->upd0.p, ws->upd1.p);
                    }, LK_EXTEND_ADD, 0});
                }
            }
            // Two-level blocked partial LU, level-synchronous over fronts.
            // Inner KB-wide panels: panel LU, row band (all columns right of
            // the panel), column band (all rows below), and rank-KB updates
            // confined to the rows or the columns of the current WB-wide outer
            // block.  Once an outer block is done, the rows and columns below
            // and right of it receive one rank-WB update, so most of the
            // elimination runs as K = WB GEMMs on the tensor cores.
            int maxp = 0;
            for (int f : fl) maxp = std::max(maxp, sym.fronts[f].p);
            for (int c0 = 0; c0 < maxp; c0 += WB) {
                for (int k = c0; k < std::min(c0 + WB, maxp); k += KB) {
                    size_t p0 = hp.size(), r0 = hr.size(), cc0 = hc.size(), g0 = hg.size();
                    long long tiles = 0;
                    for (int f : fl) {
                        const Front &Fr = sym.fronts[f];
                        if (Fr.p <= k) continue;
                        const int nf = Fr.nf(), kb = std::min(KB, Fr.p - k), k2 = k + kb;
                        const int cend = std::min(c0 + WB, Fr.p);
                        hp.push_back(PanelTask{f, k});
                        for (int c = k2; c < nf; c += TRW) hr.push_back(RowTask{f, k, c});
                        for (int r = k2; r < Fr.p; r += TCR) hc.push_back(ColTask{f, k, r, 0});
                        for (int r = 0; r < Fr.b; r += TCR) hc.push_back(ColTask{f, k, r, 1});
                        cx<T> *Pb = F + Fr.fac_off;
                        cx<T> *Lo = Pb + (long long)Fr.p * nf;
                        // rows inside the outer block, every column right of the panel
                        add_gemm(hg, tiles, Pb + (long long)k2 * nf + k, nf, Pb + (long long)k * nf + k2, nf,
                                 Pb + (long long)k2 * nf + k2, nf, cend - k2, nf - k2, kb);
                        // rows below the outer block, columns inside it
                        add_gemm(hg, tiles, Pb + (long long)cend * nf + k, nf, Pb + (long long)k * nf + k2, nf,
                                 Pb + (long long)cend * nf + k2, nf, Fr.p - cend, cend - k2, kb);
                        add_gemm(hg, tiles, Lo + k, Fr.p, Pb + (long long)k * nf + k2, nf, Lo + k2, Fr.p, Fr.b,
                                 cend - k2, kb);
                    }
                    int np = (int)(hp.size() - p0), nr = (int)(hr.size() - r0), ncl = (int)(hc.size() - cc0);
                    size_t smp = sizeof(cx<T>) * (KB * (KB + 1) + 2 * KB * (KB + 1));
                    size_t smr = sizeof(cx<T>) * (KB * (KB + 1) + KB * (TRW + 1));
                    size_t smc = sizeof(cx<T>) * (KB * (KB + 1) + TCR * (KB + 1));
                    sc->launches.push_back({[psc, this, p0, np, smp](cudaStream_t st) {
                        k_panel<T><<<np, 256, smp, st>>>(psc->panel.p + p0, fr.p, fac.p, ipiv.p, maxabs.p, pivot_rel,
                                                         npert.p, pord.p);
                    }, LK_PANEL, 0});
                    if (nr)
                        sc->launches.push_back({[psc, this, r0, nr, smr](cudaStream_t st) {
                            if constexpr (std::is_same<T, float>::value)
                                k_trsm_row_h<0><<<nr, TRW, band_row_smem(), st>>>(psc->row.p + r0, fr.p, fac.p, pord.p);
                            else
                                k_trsm_row<T><<<nr, TRW, smr, st>>>(psc->row.p + r0, fr.p, fac.p, pord.p);
                        }, LK_TRSM, 0});
                    if (ncl)
                        sc->launches.push_back({[psc, this, cc0, ncl, smc](cudaStream_t st) {
                            if constexpr (std::is_same<T, float>::value)
                                k_trsm_col_h<0><<<ncl, TCR, band_col_smem(), st>>>(psc->col.p + cc0, fr.p, fac.p);
                            else
                                k_trsm_col<T><<<ncl, TCR, smc, st>>>(psc->col.p + cc0, fr.p, fac.p);
                        }, LK_TRSM, 0});
                    push_gemm_launch(*sc, hg, g0, tiles);
                }
                // rank-WB update of everything below and right of the outer block
                size_t g0 = hg.size();
                long long tiles = 0;
                for (int f : fl) {
                    const Front &Fr = sym.fronts[f];
                    if (Fr.p <= c0) continue;
                    const int nf = Fr.nf(), cend = std::min(c0 + WB, Fr.p), w = cend - c0;
                    cx<T> *Pb = F + Fr.fac_off;
                    cx<T> *Lo = Pb + (long long)Fr.p * nf;
                    add_gemm(hg, tiles, Pb + (long long)cend * nf + c0, nf, Pb + (long long)c0 * nf + cend, nf,
                             Pb + (long long)cend * nf + cend, nf, Fr.p - cend, nf - cend, w);
                    add_gemm(hg, tiles, Lo + c0, Fr.p, Pb + (long long)c0 * nf + cend, nf, Lo + cend, Fr.p, Fr.b,
                             Fr.p - cend, w);
                }
                push_gemm_launch(*sc, hg, g0, tiles);
            }
            // Schur complement F22 -= L21 U12 (K = p)
            {
                size_t g0 = hg.size();
                long long tiles = 0;
                for (int f : fl) {
                    const Front &Fr = sym.fronts[f];
                    if (Fr.b == 0) continue;
                    const int nf = Fr.nf();
                    cx<T> *Pb = F + Fr.fac_off;
                    cx<T> *Lo = Pb + (long long)Fr.p * nf;
                    add_gemm(hg, tiles, Lo, Fr.p, Pb + Fr.p, nf, U[L & 1] + Fr.upd_off, Fr.b, Fr.b, Fr.b, Fr.p);
                }
                push_gemm_launch(*sc, hg, g0, tiles);
            }
        }
        // the tile inverses the solves use, for every panel at once
        {
            const int npall = (int)hp.size();
            const size_t smi = sizeof(cx<T>) * (KB * (KB + 1) + 2 * KB * (KB + 1));
            if (npall)
                sc->launches.push_back({[psc, this, npall, smi](cudaStream_t st) {
                    k_tile_inverse<T><<<npall, 2 * KB, smi, st>>>(psc->panel.p, fr.p, fac.p, dinv.p);
                }, LK_PANEL, 0});
        }
        int rc;
        if ((rc = sc->panel.upload(hp))) return rc;
        if ((rc = sc->row.upload(hr))) return rc;
        if ((rc = sc->col.upload(hc))) return rc;
        if ((rc = sc->gemm.upload(hg))) return rc;
        if ((rc = sc->ea.upload(he))) return rc;
        if ((rc = finish_tc(*sc))) return rc;
        fsched = std::move(sc);
        return WT3D_OK;
    }

    // Solve schedule for m right-hand sides in X (new ordering, row-major n x MAXRHS).
    Schedule<T> *solve_schedule(int m, bool adjoint)
    {
        auto it = ssched[adjoint].find(m);
        if (it != ssched[adjoint].end()) return it->second.get();
        auto sc = std::make_unique<Schedule<T>>();
        Schedule<T> *psc = sc.get();
        std::vector<PanelTask> hp;
        std::vector<GemmTask<T>> hg;
        const Symbolic &sym = *S;
        cx<T> *F = fac.p;
        cx<T> *Xp = X.p;
        struct Flag {
            bool &f;
            Flag(bool &x) : f(x) { f = true; }
            ~Flag() { f = false; }
        } building(building_solve);
        const int ldx = MAXRHS;
        const int nlev = (int)sym.levels.size();
        // Two-level blocking of the in-front substitutions, like the
        // factorisation's: inside each WS-wide outer block the KB panels are
        // solved one by one, each step one fused launch (k_sub_step: the
        // diagonal-tile product and the update of the block's other rows);
        // the rows outside the block then receive one K = WS update, which
        // the tall-skinny tensor-core kernel takes.
        std::vector<StepTask> hs;
        size_t smd_step = sizeof(cx<T>) * sub_step_smem_elems();
        int maxslots = 0;
        // one fused launch over the step tasks [s0, end)
        auto step_launch = [&](size_t s0, int mode) {
            const int ns = (int)(hs.size() - s0);
            if (!ns) return;
            sc->launches.push_back({[psc, this, s0, ns, smd_step, m, mode, Xp, ldx](cudaStream_t st) {
                // programmatic dependent launch: see k_sub_step
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3((unsigned)ns);
                cfg.blockDim = dim3(SUB_THREADS);
                cfg.dynamicSmemBytes = smd_step;
                cfg.stream = st;
                cudaLaunchAttribute at[1];
                at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
                at[0].val.programmaticStreamSerializationAllowed = 1;
                cfg.attrs = at;
                cfg.numAttrs = 1;
                cudaLaunchKernelEx(&cfg, k_sub_step<T>, (const StepTask *)(psc->step.p + s0), (const FrontDev *)fr.p,
                                   (const cx<T> *)fac.p, (const cx<T> *)dinv.p, (const int *)pord.p, Xp, ldx, m, mode,
                                   psc->zs.p);
            }, LK_SUBSTEP, 0, (double)ns * (KB * KB + 2.0 * KB * m) * sizeof(cx<T>)});
        };
        // the tasks of one panel step of front f (slot = its position in the level)
        auto add_step = [&](int f, int slot, int k, int kprev, int u0, int u1) {
            const int nup = u1 > u0 ? (u1 - u0 + SUB_RB - 1) / SUB_RB : 0;
            hs.push_back(StepTask{f, k, 0, 0, nup ? 0 : 3, kprev, slot});
            for (int r = u0; r < u1; r += SUB_RB) hs.push_back(StepTask{f, k, r, std::min(r + SUB_RB, u1), 1, -1, slot});
        };
        // ---- forward sweep: leaves to root ----
        for (int L = nlev - 1; L >= 0; L--) {
            const std::vector<int> &fl = sym.levels[L];
            maxslots = std::max(maxslots, (int)fl.size());
            int maxp = 0;
            for (int f : fl) maxp = std::max(maxp, sym.fronts[f].p);
            for (int c0 = 0; c0 < maxp; c0 += WS) {
                for (int k = c0; k < std::min(c0 + WS, maxp); k += KB) {
                    const size_t s0 = hs.size();
                    for (int si = 0; si < (int)fl.size(); si++) {
                        const Front &Fr = sym.fronts[fl[si]];
                        if (Fr.p <= k) continue;
                        const int k2 = k + std::min(KB, Fr.p - k), cend = std::min(c0 + WS, Fr.p);
                        add_step(fl[si], si, k, k > c0 ? k - KB : -1, k2, cend);
                    }
                    step_launch(s0, adjoint ? 2 : 0);
                }
                // rows below the outer block
                size_t g0 = hg.size();
                long long tiles = 0;
                for (int f : fl) {
                    const Front &Fr = sym.fronts[f];
                    if (Fr.p <= c0) continue;
                    const int nf = Fr.nf(), cend = std::min(c0 + WS, Fr.p);
                    cx<T> *Pb = F + Fr.fac_off;
                    cx<T> *Y = Xp + (long long)Fr.first * ldx;
                    if (!adjoint)   // Y[cend:p] -= L[cend:p, c0:cend] Y[c0:cend]
                        add_gemm(hg, tiles, Pb + (long long)cend * nf + c0, nf, Y + (long long)c0 * ldx, ldx,
                                 Y + (long long)cend * ldx, ldx, Fr.p - cend, m, cend - c0);
                    else            // Y[cend:p] -= U[c0:cend, cend:p]^H Y[c0:cend]
                        add_gemm(hg, tiles, Pb + (long long)c0 * nf + cend, nf, Y + (long long)c0 * ldx, ldx,
                                 Y + (long long)cend * ldx, ldx, Fr.p - cend, m, cend - c0, nullptr, nullptr, 1);
                }
                push_gemm_launch(*sc, hg, g0, tiles);
            }
            // border update  X[border] -= L21 Y   (adjoint: U12^H Y)
            size_t g0 = hg.size();
            long long tiles = 0;
            for (int f : fl) {
                const Front &Fr = sym.fronts[f];
                if (Fr.b == 0) continue;
                const int nf = Fr.nf();
                cx<T> *Pb = F + Fr.fac_off;
                cx<T> *Lo = Pb + (long long)Fr.p * nf;
                cx<T> *Y = Xp + (long long)Fr.first * ldx;
                const int *crow = border.p + Fr.border_off;
                if (!adjoint) add_gemm(hg, tiles, Lo, Fr.p, Y, ldx, Xp, ldx, Fr.b, m, Fr.p, nullptr, crow, 0);
                else add_gemm(hg, tiles, Pb + Fr.p, nf, Y, ldx, Xp, ldx, Fr.b, m, Fr.p, nullptr, crow, 1);
            }
            push_gemm_launch(*sc, hg, g0, tiles);
        }
        // ---- backward sweep: root to leaves ----
        for (int L = 0; L < nlev; L++) {
            const std::vector<int> &fl = sym.levels[L];
            size_t g0 = hg.size();
            long long tiles = 0;
            int maxp = 0;
            for (int f : fl) {
                const Front &Fr = sym.fronts[f];
                maxp = std::max(maxp, Fr.p);
                if (Fr.b == 0) continue;
                const int nf = Fr.nf();
                cx<T> *Pb = F + Fr.fac_off;
                cx<T> *Lo = Pb + (long long)Fr.p * nf;
                cx<T> *Y = Xp + (long long)Fr.first * ldx;
                const int *brow = border.p + Fr.border_off;
                if (!adjoint)   // Y -= U12 X[border]
                    add_gemm(hg, tiles, Pb + Fr.p, nf, Xp, ldx, Y, ldx, Fr.p, m, Fr.b, brow, nullptr, 0);
                else            // Y -= L21^H X[border]
                    add_gemm(hg, tiles, Lo, Fr.p, Xp, ldx, Y, ldx, Fr.p, m, Fr.b, brow, nullptr, 1);
            }
            push_gemm_launch(*sc, hg, g0, tiles);
            for (int c0 = (maxp - 1) / WS * WS; c0 >= 0; c0 -= WS) {
                const int nsteps = (std::min(c0 + WS, maxp) - c0 + KB - 1) / KB;
                for (int s = nsteps - 1; s >= 0; s--) {
                    const int k = c0 + s * KB;
                    const size_t s0 = hs.size();
                    for (int si = 0; si < (int)fl.size(); si++) {
                        const Front &Fr = sym.fronts[fl[si]];
                        if (Fr.p <= k) continue;
                        const int cend = std::min(c0 + WS, Fr.p);
                        // the rows above the panel inside the block (right-looking for both modes)
                        add_step(fl[si], si, k, k + KB < cend ? k + KB : -1, c0, k);
                    }
                    step_launch(s0, adjoint ? 3 : 1);
                }
                if (c0 > 0) {
                    // rows above the block:  Y[0:c0] -= U[0:c0, c0:cend] Y[c0:cend]
                    //                 (adjoint: Y[0:c0] -= L[c0:cend, 0:c0]^H Y[c0:cend])
                    size_t g1 = hg.size();
                    long long t1 = 0;
                    for (int f : fl) {
                        const Front &Fr = sym.fronts[f];
                        if (Fr.p <= c0) continue;
                        const int nf = Fr.nf(), cend = std::min(c0 + WS, Fr.p);
                        cx<T> *Pb = F + Fr.fac_off;
                        cx<T> *Y = Xp + (long long)Fr.first * ldx;
                        if (!adjoint)
                            add_gemm(hg, t1, Pb + c0, nf, Y + (long long)c0 * ldx, ldx, Y, ldx, c0, m, cend - c0);
                        else
                            add_gemm(hg, t1, Pb + (long long)c0 * nf, nf, Y + (long long)c0 * ldx, ldx, Y, ldx, c0, m,
                                     cend - c0, nullptr, nullptr, 1);
                    }
                    push_gemm_launch(*sc, hg, g1, t1);
                }
            }
        }
        if (sc->step.upload(hs) || sc->zs.alloc((size_t)std::max(maxslots, 1) * KB * MAXRHS)) return nullptr;
        if (sc->panel.upload(hp) || sc->gemm.upload(hg) || finish_tc(*sc) || finish_ts(*sc)) return nullptr;
        Schedule<T> *ret = sc.get();
        ssched[adjoint][m] = std::move(sc);
        return ret;
    }

    const double2 *a_dev = nullptr;   // complex128 operator values (set before factor)

    int run(Schedule<T> &sc, cudaStream_t st)
    {
        if (use_graphs) {
            if (!sc.graph) {
                cudaGraph_t g;
                WT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                for (auto &l : sc.launches) l.fn(st);
                WT_CUDA(cudaStreamEndCapture(st, &g));
                cudaError_t e = cudaGraphInstantiate(&sc.graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
                    sc.graph = nullptr;
                    return WT3D_ERR_CUDA;
                }
            }
            WT_CUDA(cudaGraphLaunch(sc.graph, st));
        } else {
            for (auto &l : sc.launches) l.fn(st);
        }
        WT_CUDA(cudaGetLastError());
        return WT3D_OK;
    }

    // Factorisation with one event pair around every launch (no graph):
    // out[k] = milliseconds spent in launches of kind k, out[LK_NKINDS] =
    // GEMM real flops, out[LK_NKINDS+1] = GEMM launches.
    // Runs a schedule once with an event pair around every launch; ms[i] per launch.
    int profile_each(Schedule<T> &sc, cudaStream_t st, std::vector<float> &ms)
    {
        const size_t nl = sc.launches.size();
        std::vector<cudaEvent_t> ev(2 * nl);
        for (auto &e : ev) WT_CUDA(cudaEventCreate(&e));
        for (size_t i = 0; i < nl; i++) {
            WT_CUDA(cudaEventRecord(ev[2 * i], st));
            sc.launches[i].fn(st);
            WT_CUDA(cudaEventRecord(ev[2 * i + 1], st));
        }
        WT_CUDA(cudaStreamSynchronize(st));
        ms.assign(nl, 0.f);
        for (size_t i = 0; i < nl; i++) cudaEventElapsedTime(&ms[i], ev[2 * i], ev[2 * i + 1]);
        for (auto &e : ev) cudaEventDestroy(e);
        WT_CUDA(cudaGetLastError());
        return WT3D_OK;
    }

    // The factor schedule under profile_each (the factorisation is complete afterwards).
    int profile_factor_each(const double2 *d_a, long long nnz, cudaStream_t st, std::vector<float> &ms)
    {
        a_dev = d_a;
        WT_CUDA(cudaMemsetAsync(maxabs.p, 0, sizeof(unsigned long long), st));
        k_maxabs<<<1216, 256, 0, st>>>(nnz, d_a, maxabs.p);
        return profile_each(*fsched, st, ms);
    }

    int profile_factor(const double2 *d_a, long long nnz, cudaStream_t st, double *out)
    {
        a_dev = d_a;
        WT_CUDA(cudaMemsetAsync(maxabs.p, 0, sizeof(unsigned long long), st));
        k_maxabs<<<1216, 256, 0, st>>>(nnz, d_a, maxabs.p);
        const size_t nl = fsched->launches.size();
        std::vector<cudaEvent_t> ev(2 * nl);
        for (auto &e : ev) WT_CUDA(cudaEventCreate(&e));
        for (size_t i = 0; i < nl; i++) {
            WT_CUDA(cudaEventRecord(ev[2 * i], st));
            fsched->launches[i].fn(st);
            WT_CUDA(cudaEventRecord(ev[2 * i + 1], st));
        }
        WT_CUDA(cudaStreamSynchronize(st));
        for (int k = 0; k < LK_NKINDS + 2; k++) out[k] = 0;
        for (size_t i = 0; i < nl; i++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
            out[fsched->launches[i].kind] += ms;
            if (fsched->launches[i].kind == LK_GEMM || fsched->launches[i].kind == LK_TCGEMM) {
                out[LK_NKINDS] += fsched->launches[i].flops;
                out[LK_NKINDS + 1] += 1;
            }
        }
        for (auto &e : ev) cudaEventDestroy(e);
        WT_CUDA(cudaGetLastError());
        return WT3D_OK;
    }

    // One pass of a solve schedule with an event pair per launch: out[k] = ms of kind k.
    int profile_schedule(Schedule<T> &sc, cudaStream_t st, double *out)
    {
        const size_t nl = sc.launches.size();
        std::vector<cudaEvent_t> ev(2 * nl);
        for (auto &e : ev) WT_CUDA(cudaEventCreate(&e));
        for (size_t i = 0; i < nl; i++) {
            WT_CUDA(cudaEventRecord(ev[2 * i], st));
            sc.launches[i].fn(st);
            WT_CUDA(cudaEventRecord(ev[2 * i + 1], st));
        }
        WT_CUDA(cudaStreamSynchronize(st));
        for (int k = 0; k < LK_NKINDS + 2; k++) out[k] = 0;
        for (size_t i = 0; i < nl; i++) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
            out[sc.launches[i].kind] += ms;
            if (sc.launches[i].kind == LK_GEMM || sc.launches[i].kind == LK_TCGEMM) {
                out[LK_NKINDS] += sc.launches[i].flops;
                out[LK_NKINDS + 1] += 1;
            }
        }
        for (auto &e : ev) cudaEventDestroy(e);
        return WT3D_OK;
    }

    int factor(const double2 *d_a, long long nnz, cudaStream_t st, int *h_npert)
    {
        if (d_a != a_dev && fsched->graph) { cudaGraphExecDestroy(fsched->graph); fsched->graph = nullptr; }
        a_dev = d_a;
        WT_CUDA(cudaMemsetAsync(maxabs.p, 0, sizeof(unsigned long long), st));
        k_maxabs<<<1216, 256, 0, st>>>(nnz, d_a, maxabs.p);
        WT_CUDA(cudaMemsetAsync(npert.p, 0, sizeof(int), st));
        int rc = run(*fsched, st);
        if (rc) return rc;
        if (h_npert) {
            WT_CUDA(cudaMemcpyAsync(h_npert, npert.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        }
        return WT3D_OK;
    }

};

}  // namespace wt3d
