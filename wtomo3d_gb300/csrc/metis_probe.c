/* Build-time probe of the METIS library that ships with the CUDA toolkit
 * (libmetis_static.a, no header): the build runs this program once and links
 * METIS into libwtomo3d_gpu.so only if METIS_ComputeVertexSeparator, called
 * with 64-bit indices on a 4 x 4 grid graph, returns a valid vertex
 * separator.  Prints "metis idx64 ok" on success. */
#include <stdint.h>
#include <stdio.h>

typedef int64_t idx_t;
int METIS_SetDefaultOptions(idx_t *options);
int METIS_ComputeVertexSeparator(idx_t *nvtxs, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *options,
                                 idx_t *sepsize, idx_t *part);

int main(void)
{
    idx_t n = 16, xadj[17], adj[64], part[16], opt[64], sepsize = -1;
    int k = 0;
    for (int v = 0; v < 16; v++) {
        const int i = v % 4, j = v / 4;
        xadj[v] = k;
        if (i > 0) adj[k++] = v - 1;
        if (i < 3) adj[k++] = v + 1;
        if (j > 0) adj[k++] = v - 4;
        if (j < 3) adj[k++] = v + 4;
    }
    xadj[16] = k;
    for (int i = 0; i < 64; i++) opt[i] = 0;
    if (METIS_SetDefaultOptions(opt) != 1) return 2;
    if (METIS_ComputeVertexSeparator(&n, xadj, adj, NULL, opt, &sepsize, part) != 1) return 3;
    idx_t cnt[3] = {0, 0, 0};
    for (int v = 0; v < 16; v++) {
        if (part[v] < 0 || part[v] > 2) return 4;
        cnt[part[v]]++;
        for (int t = (int)xadj[v]; t < xadj[v + 1]; t++)
            if (part[v] + part[adj[t]] == 1) return 5;   /* an edge between the two sides */
    }
    if (cnt[0] == 0 || cnt[1] == 0 || cnt[2] != sepsize) return 6;
    printf("metis idx64 ok\n");
    return 0;
}
