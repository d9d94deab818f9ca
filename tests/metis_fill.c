/* Fill of a symmetric elimination ordering, and METIS_NodeND for comparison.
 *
 * Test and measurement tool only (no part of the library).  Usage:
 *   metis_fill GRAPH metis      order by METIS_NodeND (default options)
 *   metis_fill GRAPH perm PERM  use the ordering in PERM
 * GRAPH: int64 n, int64 xadj[n+1], int64 adj[xadj[n]] (0-based, symmetric,
 * no self loops); PERM: int64 perm[n], new position -> vertex.  Prints
 * "nnzL <sum of column counts incl. diagonal> flops <sum of squared
 * off-diagonal column counts> maxcol <largest column count>".
 *
 * METIS ships in the CUDA toolkit as libmetis_static.a without a header; its
 * index type is 64 bits wide (checked by calling it on a 3 x 3 grid).  The
 * column structures follow the elimination-tree rule
 *   struct(j) = (adj(j) U struct(children of j)) minus {<= j},
 *   parent(j) = min struct(j),
 * with each structure dropped once its parent has absorbed it. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t idx_t;
int METIS_SetDefaultOptions(idx_t *options);
int METIS_NodeND(idx_t *nvtxs, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *options, idx_t *perm, idx_t *iperm);

static void *xmalloc(size_t n)
{
    void *p = malloc(n ? n : 1);
    if (!p) { fprintf(stderr, "out of memory\n"); exit(2); }
    return p;
}

static idx_t *read_all(const char *path, size_t *count)
{
    FILE *f = fopen(path, "rb");
    if (!f) { perror(path); exit(2); }
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    idx_t *b = xmalloc((size_t)sz);
    if (fread(b, 1, (size_t)sz, f) != (size_t)sz) { fprintf(stderr, "short read\n"); exit(2); }
    fclose(f);
    *count = (size_t)sz / sizeof(idx_t);
    return b;
}

int main(int argc, char **argv)
{
    if (argc < 3) { fprintf(stderr, "usage: metis_fill GRAPH metis|perm [PERM]\n"); return 1; }
    size_t cnt;
    idx_t *g = read_all(argv[1], &cnt);
    idx_t n = g[0], *xadj = g + 1, *adj = g + 2 + n;
    idx_t *perm = xmalloc(sizeof(idx_t) * n), *iperm = xmalloc(sizeof(idx_t) * n);
    if (!strcmp(argv[2], "metis")) {
        idx_t opt[64];
        memset(opt, 0, sizeof(opt));
        METIS_SetDefaultOptions(opt);
        /* row i of the permuted matrix is row perm[i] of the original */
        if (METIS_NodeND(&n, xadj, adj, NULL, opt, perm, iperm) != 1) { fprintf(stderr, "METIS failed\n"); return 3; }
    } else {
        size_t pc;
        idx_t *p = read_all(argv[3], &pc);
        if ((idx_t)pc != n) { fprintf(stderr, "perm size\n"); return 1; }
        memcpy(perm, p, sizeof(idx_t) * n);
        free(p);
    }
    idx_t *pos = xmalloc(sizeof(idx_t) * n);   /* vertex -> new position */
    for (idx_t i = 0; i < n; i++) pos[i] = -1;
    for (idx_t i = 0; i < n; i++) {
        if (perm[i] < 0 || perm[i] >= n || pos[perm[i]] >= 0) { fprintf(stderr, "not a permutation\n"); return 1; }
        pos[perm[i]] = i;
    }
    /* children lists (linked through next[]), pending structures */
    idx_t *head = xmalloc(sizeof(idx_t) * n), *next = xmalloc(sizeof(idx_t) * n), *mark = xmalloc(sizeof(idx_t) * n);
    idx_t **st = xmalloc(sizeof(idx_t *) * n), *len = xmalloc(sizeof(idx_t) * n);
    for (idx_t i = 0; i < n; i++) { head[i] = -1; mark[i] = -1; st[i] = NULL; }
    idx_t cap = 1024, *buf = xmalloc(sizeof(idx_t) * cap);
    double nnzL = 0, flops = 0;
    idx_t maxcol = 0;
    for (idx_t j = 0; j < n; j++) {
        idx_t m = 0;
        const idx_t v = perm[j];
        mark[j] = j;
#define ADD(x) do { idx_t y_ = (x); if (y_ > j && mark[y_] != j) { mark[y_] = j; \
        if (m == cap) { cap *= 2; buf = realloc(buf, sizeof(idx_t) * cap); if (!buf) exit(2); } buf[m++] = y_; } } while (0)
        for (idx_t k = xadj[v]; k < xadj[v + 1]; k++) ADD(pos[adj[k]]);
        for (idx_t c = head[j]; c >= 0; c = next[c]) {
            for (idx_t t = 0; t < len[c]; t++) ADD(st[c][t]);
            free(st[c]);
            st[c] = NULL;
        }
#undef ADD
        nnzL += (double)(m + 1);
        flops += (double)m * (double)m;
        if (m + 1 > maxcol) maxcol = m + 1;
        if (m > 0) {
            idx_t par = buf[0];
            for (idx_t t = 1; t < m; t++) if (buf[t] < par) par = buf[t];
            st[j] = xmalloc(sizeof(idx_t) * m);
            memcpy(st[j], buf, sizeof(idx_t) * m);
            len[j] = m;
            next[j] = head[par];
            head[par] = j;
        }
    }
    printf("nnzL %.6e flops %.6e maxcol %lld\n", nnzL, flops, (long long)maxcol);
    return 0;
}
