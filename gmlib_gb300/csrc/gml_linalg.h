/*
 * gml_linalg.h -- SELL-32 block sparse matrices and block-vector kernels
 * shared by the host layer (gml_linalg.c, gml_solver.c) and the CUDA
 * kernels (gml_linalg_kernels.cu).
 */
#ifndef GML_LINALG_H
#define GML_LINALG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* SELL-32 image of a block CSR matrix on the device: entry k of row r
   (slice s = r/32, lane = r%32) has its column at
   Col[(SlcOff[s] + k) * 32 + lane] and block value c (row-major b x b) at
   Val[((SlcOff[s] + k) * b*b + c) * 32 + lane]; Deg[r] is the row's block
   count and padding entries hold column 0 and zero values. */
typedef struct
{
   int      NmbLin, BlkSiz, FltSiz, NmbSlc;
   size_t   bytes;
   size_t   NmbCol;          /* sum of slice widths */
   int64_t  *SlcOff;
   int      *Deg, *Col;
   void     *Val;
}GmlSellDev;

struct GmdCtx;

/* y = A x ; x and y lines have xs / ys scalars (>= block size) */
int gmd_sell_spmv(struct GmdCtx *ctx, const GmlSellDev *A, const void *x, int xs,
                  void *y, int ys, double alpha, double beta, double *dotout, int flags);
int gmd_vec_add3(struct GmdCtx *ctx, const void *u, const void *v, const void *w, void *y,
                 size_t n, int fltsiz);
int gmd_vec_scale(struct GmdCtx *ctx, void *u, size_t n, int fltsiz, double s);
int gmd_vec_rownorm(struct GmdCtx *ctx, const void *u, int us, int nlanes, int fltsiz,
                    int nlin, float *out);
/* device SELL-32 repack: row degrees and slice widths, then the fill;
   err bit 1: decreasing row pointers, bit 2: column out of range */
int gmd_sell_widths(struct GmdCtx *ctx, int nrow, const int *lin, int *deg, long long *width,
                    int *err);
int gmd_sell_fill(struct GmdCtx *ctx, int nrow, int bb, int fltsiz, const int *lin,
                  const int *col, const void *val, const long long *soff, int *Col, void *Val,
                  int *err);
int gmd_vec_diag(struct GmdCtx *ctx, const void *d, int ds, const void *u, void *v, int vs,
                 int b, int fltsiz, int nlin);

#ifdef __cplusplus
}
#endif

#ifdef GML_INTERNAL_H
void gml_sell_dev_free(GmlSct *gml, GmlSellDev *d);
void gml_release_matrices(GmlSct *gml);
void gml_release_solvers(GmlSct *gml);
#endif

#endif
