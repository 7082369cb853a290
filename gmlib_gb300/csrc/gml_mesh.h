/*
 * gml_mesh.h -- device entry points of the native mesh kernels
 * (gml_mesh_kernels.cu), called by gml_native.c.
 */
#ifndef GML_MESH_H
#define GML_MESH_H

#include "gmlib3_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

struct GmdCtx;

int gmd_mesh_vt_csr(struct GmdCtx *ctx, const void *tet, int nt, int nv,
                    int *ptr, int *vt, int *tmp, int *err);
int gmd_mesh_boundary(struct GmdCtx *ctx, const void *tet, int nt, const int *ptr,
                      const int *vt, int *fixed);
/* fixed[v] = (ref[v] != 0), ref being the device copy of the vertex references */
int gmd_mesh_fixed_from_ref(struct GmdCtx *ctx, const int *ref, int nv, int *fixed);
/* ball of points as SELL-C-sigma: rows are vertices sorted by ball size in
   windows of `window` rows (32, 64, 128 or GML_SIGMA = 256; rowv packs
   (size << 26) | vertex), slices of 32 rows, rows padded to a multiple of 256 */
#define GML_SIGMA 256
int gmd_mesh_point_count(struct GmdCtx *ctx, const void *tet, int nv, const int *ptr,
                         const int *vt, const int *fixed, int *pdeg, unsigned *rowv,
                         long long *width, long long *soff, int *err, int window);
int gmd_mesh_point_fill(struct GmdCtx *ctx, const void *tet, int nrow, const int *ptr,
                        const int *vt, const unsigned *rowv, const long long *soff, int *col);
/* bps: resident blocks per SM for the persistent grid (0: the kernel's
   maximum); a smaller grid leaves room for a concurrent kernel */
int gmd_mesh_laplace(struct GmdCtx *ctx, int nrow, const unsigned *rowv, const long long *soff,
                     const int *col, const void *in, void *out, float omega, int *err, int bps);
int gmd_mesh_stats_init(struct GmdCtx *ctx, GmlxQualStats *st, int n);
int gmd_mesh_quality(struct GmdCtx *ctx, int nt, const void *tet, const void *crd, float thr,
                     float *qout, unsigned *flags, GmlxQualStats *st, int *err, int bps);

/* batched meshes (gml_batch.c): a (mesh, range) tile queue drained by one
   persistent launch */
typedef struct { int phase, mesh, beg, end; } GmdBatchTile;     /* phase < nsweep: slices */
typedef struct { int t0, nt, f0, s0, s1; float thr; } GmdBatchMesh;
typedef struct
{
   int                  ntile, nsweep, nmesh, nphase;
   const GmdBatchTile   *tiles;
   const GmdBatchMesh   *mesh;
   const int            *need;       /* tiles per (mesh, phase) */
   int                  *done;       /* finished tiles per (mesh, phase) */
   int                  *head, *abort, *err;
   const unsigned       *rowv;
   const long long      *soff;
   const int            *col;
   void                 *buf0, *buf1;
   const void           *tet;
   unsigned             *flags;
   GmlxQualStats        *stats;
   float                omega;
   int                  spin;        /* tries (about 256 ns each) before a waiting tile gives up */
}GmdBatchArgs;

int gmd_batch_queue(struct GmdCtx *ctx, const GmdBatchArgs *a, int grid);       /* block tiles */
int gmd_batch_queue_warp(struct GmdCtx *ctx, const GmdBatchArgs *a, int grid);  /* warp tiles */
int gmd_batch_grid(struct GmdCtx *ctx);
int gmd_mesh_laplace_slices(struct GmdCtx *ctx, int s0, int s1, const unsigned *rowv,
                            const long long *soff, const int *col, const void *in, void *out,
                            float omega);

/* CUDA graphs on the instance stream */
int  gmd_graph_begin(struct GmdCtx *ctx);
int  gmd_graph_end(struct GmdCtx *ctx, void **exec);
int  gmd_graph_launch(struct GmdCtx *ctx, void *exec);
void gmd_graph_free(void *exec);

#ifdef __cplusplus
}
#endif

#endif
