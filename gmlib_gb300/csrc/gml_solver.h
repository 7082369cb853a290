/*
 * gml_solver.h -- device side of the conjugate-gradient solvers
 * (gml_solver_kernels.cu), called by gml_solver.c.
 *
 * All scalars of an iteration (residual norms, step lengths, stop test) live
 * in device memory in one GmdSvScal, so iterations run back to back on the
 * stream (and inside CUDA graphs) without host round trips; the host reads
 * the structure only to decide whether to replay more iterations.  Dot
 * products are accumulated per thread in the vectors' precision (FP32 as an
 * error-free TwoSum pair) and combined in FP64 or float pairs; the
 * reductions are deterministic (per-block partials folded in a fixed order,
 * by the last block or by every block of the next kernel).
 */
#ifndef GML_SOLVER_H
#define GML_SOLVER_H

#include <stddef.h>
#include "gml_linalg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
   double   rr;        /* recursive residual norm^2 of the running CG */
   double   pq;        /* p . A p */
   double   alpha, beta;
   double   stop;      /* rr threshold of the running CG */
   double   bb;        /* |b|^2 */
   double   rt;        /* true residual norm^2 (FP64) */
   double   pad;
   unsigned long long ticket;
   int      done;      /* 1 converged or iteration cap, 2 breakdown (p.Ap <= 0) */
   int      it, maxit, spare;
}GmdSvScal;

#define GMD_SV_MAXBLK 16384

struct GmdCtx;

/* lanes of a vector line for block size B (GmlNewVector's padding) */
int  gmd_sv_lanes(int B);

/* x = 0, r = p = b (n scalars of padded lines), b64 = b (may be NULL),
   bb = rr = rt = |b|^2, stop = tol2 bb */
int  gmd_sv_init(struct GmdCtx *ctx, size_t n, int B, const double *bsrc, double *b64,
                 void *x, void *r, void *p, int fltsiz, double *part, GmdSvScal *sc, double tol2,
                 int maxit);

/* q = A p.  FP32 matrix: the per-block partials of p.q in spart
   (gmd_sv_spmv_blocks float pairs); FP64: p.q in sc->pq (spart is the
   scratch of that fold).  With r and pn given, p is the previous direction
   and the product uses the new one, r + beta p formed line by line and
   written to pn (pn != p). */
int  gmd_sv_spmv(struct GmdCtx *ctx, const GmlSellDev *A, const void *r, const void *p,
                 void *pn, void *q, void *spart, GmdSvScal *sc);
int  gmd_sv_spmv_blocks(int nrow);

/* pq = fold of the nsp SpMV partials (sc->pq when nsp = 0), alpha = rr / pq, x += alpha p,
   r -= alpha q, rr' = |r|^2, beta = rr' / rr, stop test (breakdown flag
   when pq <= 0) */
int  gmd_sv_update(struct GmdCtx *ctx, int fltsiz, size_t n, void *x, void *r, const void *p,
                   const void *q, const void *spart, int nsp, double *part, GmdSvScal *sc);

/* p = r + beta p */
int  gmd_sv_dir(struct GmdCtx *ctx, int fltsiz, size_t n, void *p, const void *r,
                GmdSvScal *sc);

/* r = b - A x in FP64, rt = |r|^2 */
int  gmd_sv_residual(struct GmdCtx *ctx, const GmlSellDev *A, const double *b, const double *x,
                     double *r, double *part, GmdSvScal *sc);

/* inner FP32 system of a refinement step: r32 = p32 = r64 / sqrt(rt),
   d32 = 0, rr = |r32|^2, stop = tin2 rr, it = 0 */
int  gmd_sv_ir_begin(struct GmdCtx *ctx, size_t n, const double *r64, float *r32, float *p32,
                     float *d32, double *part, GmdSvScal *sc, double tin2, int maxit);

/* x64 += sqrt(rt) d32 */
int  gmd_sv_ir_end(struct GmdCtx *ctx, size_t n, double *x64, const float *d32, GmdSvScal *sc);

/* FP32 copy of FP64 matrix values */
int  gmd_sv_to_f32(struct GmdCtx *ctx, const double *src, float *dst, size_t n);

#ifdef __cplusplus
}
#endif

#endif
