// Tensor-core (tcgen05, 3xTF32) complex64 GEMM: host interface.
#pragma once
#include "mf_kernels.cuh"
#include "devvec.cuh"

namespace wt3d {

// One GEMM of a tensor-core launch (complex dims; Kr = real K padded to 32).
struct TcTask {
    const cx<float> *A;
    const cx<float> *B;
    cx<float> *C;
    float *ahi, *alo, *bhi, *blo;   // split operands in the launch workspace (FP16 pairs in the f16 mode)
    // f16 mode: per row of A and per complex column of B, the inverse of the
    // power-of-two scale
    float *sa, *sb;
    int lda, ldb, ldc, M, N, K, Kr;
    int tiles_n;
    int map0;                       // first of this task's 4 tensor maps
    long long tile0, a_work0, b_work0, a_row0, b_col0;   // b_col0: first 32-column group of B (f16 split)
};

struct TcLaunch {
    DevVec<TcTask> tasks;
    DevVec<unsigned char> maps;    // CUtensorMap array (4 per task)
    int ntasks = 0;
    long long tiles = 0, a_work = 0, b_tiles = 0, a_rows = 0, b_cols = 0;
    bool f16 = false;              // 2 x FP16 split with power-of-two row/column scales (else 3 x TF32)
};

// One GEMM of a tall-skinny tensor-core launch (substitution passes: N <= 32).
struct TsTask {
    const cx<float> *A;
    const cx<float> *B;
    cx<float> *C;
    const int *brow, *crow;         // optional row gather of B, row scatter of C
    float *bhi, *blo;               // expanded, split B~ (64 x Kr) in the launch workspace
    int lda, ldb, ldc, M, N, K, Kr;
    int kchunk, nkc, atom;          // K-chunk per work unit, chunks, atomic epilogue
    int conjA;                      // A^H of the stored K x M block (lda its row stride)
    int map0;                       // first of this task's 3 tensor maps (B~ hi, B~ lo, raw A)
    long long unit0, b_work0;
};

struct TsLaunch {
    DevVec<TsTask> tasks;
    DevVec<unsigned char> maps;    // CUtensorMap array (3 per task)
    int ntasks = 0;
    long long units = 0, b_tiles = 0;
    bool tma = false;              // A streamed by TMA (every task 16-byte aligned with an even stride)
};

int tc_init();
int ts_init();
bool ts_eligible(const GemmTask<float> &g);
bool ts_tma_ok(const GemmTask<float> &g);
long long ts_workspace_floats(const GemmTask<float> *g, int n);
int ts_build_launch(TsLaunch &L, const GemmTask<float> *g, int n, float *ws, bool tma);
void ts_expand(const TsLaunch &L, cudaStream_t st);
void ts_mma(const TsLaunch &L, int *err, cudaStream_t st);
bool tc_eligible(const GemmTask<float> &g);
long long tc_workspace_floats(const GemmTask<float> *g, int n);
int tc_build_launch(TcLaunch &L, const GemmTask<float> *g, int n, float *ws);
void tc_split(const TcLaunch &L, cudaStream_t st);
void tc_mma(const TcLaunch &L, int *err, cudaStream_t st);

}  // namespace wt3d
