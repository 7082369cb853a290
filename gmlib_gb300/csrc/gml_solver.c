/*
 * gml_solver.c -- conjugate-gradient solvers on GmlNewMatrix block matrices
 * (no counterpart in the reference, whose LinearSolver example runs a
 * fixed-point loop, examples/LinearSolver/LinearSolver.c:300-338).
 *
 * GmlxSolveCG(mode = GmlxCgFp64)   plain CG in FP64;
 * GmlxSolveCG(mode = GmlxCgMixed)  FP32 CG inside FP64 iterative refinement:
 *   x = 0, r = b
 *   repeat
 *      solve A d = r / |r| with FP32 CG (FP32 copy of A, FP32 vectors, FP64
 *      dots) until its residual falls by the inner factor (1e-5: two
 *      refinement steps reach 1e-10 on the cube systems, measured fastest)
 *      x += |r| d                                   (FP64)
 *      r = b - A x with the FP64 matrix, |r|        (FP64)
 *   until |r| <= tol |b|
 *
 * An FP64 iteration is three kernels: q = A p and p.q (folded by its last
 * block); the update (alpha, x, r and |r|^2, beta and the stop flag);
 * p = r + beta p.  An FP32 iteration is two: the SpMV forms p = r + beta
 * p_old line by line from r and the previous direction (double-buffered by
 * iteration parity), writes it and leaves per-block partials of p.q, which
 * every block of the update folds itself.  On this part the FP64 pipe makes
 * the fused form slower in FP64.
 *
 * Both stop on the relative residual.  Iterations run as CUDA graphs of
 * GML_CG_CHUNK iterations replayed on the instance's stream; the scalars stay
 * on the device, and the host reads them once per replay while the next
 * replay is already queued (replays past convergence do nothing).  The
 * reported residual is always recomputed as b - A x in FP64 at the end.
 *
 * Work vectors have the padded lines of GmlNewVector (4 lanes for b <= 4, 8
 * for b <= 8, zero padding), so a line is gathered with 16-byte loads; they
 * are allocated on the first solve with a matrix, the FP32 copy of the
 * matrix values on the first mixed solve, and both are kept until GmlStop.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_internal.h"
#include "gml_device.h"
#include "gml_mesh.h"
#include "gml_solver.h"

#define GML_CG_CHUNK  8          /* iterations per graph replay (even: parity of p) */
#define GML_CG_MAXOUT 20         /* refinement steps */

typedef struct
{
   GmlMatSct   *mat;             /* the FP64 matrix solved with */
   int         nrow, B, vs;
   size_t      n;                /* scalars of a vector: rows x lanes */
   GmlSellDev  A32;              /* FP32 values, structure shared with the FP64 matrix */
   int         have32;
   double      *b64, *x64, *r64, *p64, *q64, *part, *spart;
   float       *d32, *r32, *p32[2], *q32;     /* p32[0], p32[1]: directions by parity */
   GmdSvScal   *sc, *hsc;        /* device scalars, pinned host copies (2 slots) */
   void        *g64, *g32;       /* graphs of `chunk` iterations */
   void        *ev[2], *t0, *t1;
   void        *tr[4];           /* phase and kernel timing of GML_CG_TRACE */
   int         chunk;            /* iterations per replay of g64 / g32 */
}GmlSolver;

/* the inner FP32 solve of the refinement loop stops when its residual has
   fallen by this factor (10^-6 needed more iterations in total) */
static double inner_factor(void)
{
   return 1e-5;
}

/* iterations per graph replay, even so that every replay starts on
   direction buffer 0 */
static int cg_chunk(void)
{
   return (GML_CG_CHUNK + 1) & ~1;
}

static void solver_free(GmlSct *gml, GmlSolver *s)
{
   if(!s)
      return;
   gmd_free(gml->dev, s->b64); gmd_free(gml->dev, s->x64); gmd_free(gml->dev, s->r64);
   gmd_free(gml->dev, s->p64); gmd_free(gml->dev, s->q64); gmd_free(gml->dev, s->part);
   gmd_free(gml->dev, s->d32); gmd_free(gml->dev, s->r32); gmd_free(gml->dev, s->p32[0]);
   gmd_free(gml->dev, s->p32[1]); gmd_free(gml->dev, s->q32); gmd_free(gml->dev, s->sc);
   if(s->have32)
      gmd_free(gml->dev, s->A32.Val);
   gmd_host_free(s->hsc);
   gmd_graph_free(s->g64);
   gmd_graph_free(s->g32);
   for(int i=0;i<2;i++)
      gmd_event_free(s->ev[i]);
   gmd_event_free(s->t0);
   gmd_event_free(s->t1);
   for(int i=0;i<4;i++)
      gmd_event_free(s->tr[i]);
   free(s);
}

void gml_release_solvers(GmlSct *gml)
{
   for(int i=1;i<=GmlMaxMat;i++)
      if(gml->mat[i].Sol)
      {
         solver_free(gml, (GmlSolver *)gml->mat[i].Sol);
         gml->mat[i].Sol = NULL;
      }
}

static GmlSolver *solver_get(GmlSct *gml, GmlMatSct *mat, int mixed)
{
   GmlSolver *s = (GmlSolver *)mat->Sol;
   GmlSellDev *A = (GmlSellDev *)mat->Val;

   if(!s)
   {
      size_t n = (size_t)A->NmbLin * gmd_sv_lanes(A->BlkSiz);
      s = calloc(1, sizeof(GmlSolver));
      if(!s)
         return NULL;
      s->mat = mat;
      s->nrow = A->NmbLin;
      s->B = A->BlkSiz;
      s->vs = gmd_sv_lanes(A->BlkSiz);
      s->n = n;
      s->b64 = gmd_alloc(gml->dev, n * 8);
      s->x64 = gmd_alloc(gml->dev, n * 8);
      s->r64 = gmd_alloc(gml->dev, n * 8);
      s->part = gmd_alloc(gml->dev, 2 * GMD_SV_MAXBLK * 8);
      s->spart = s->part + GMD_SV_MAXBLK;     /* SpMV partials, read by the update */
      s->sc = gmd_alloc(gml->dev, sizeof(GmdSvScal));
      s->hsc = gmd_host_alloc(2 * sizeof(GmdSvScal));
      s->ev[0] = gmd_event_new_sync();
      s->ev[1] = gmd_event_new_sync();
      s->t0 = gmd_event_new();
      s->t1 = gmd_event_new();
      for(int i=0;i<4;i++)
         s->tr[i] = gmd_event_new();
      s->chunk = cg_chunk();
      mat->Sol = s;
      if(!s->b64 || !s->x64 || !s->r64 || !s->part || !s->sc || !s->hsc
      || !s->ev[0] || !s->ev[1] || !s->t0 || !s->t1 || !s->tr[0] || !s->tr[1] || !s->tr[2] || !s->tr[3])
         return NULL;
   }
   if(!mixed && !s->p64)
   {
      s->p64 = gmd_alloc(gml->dev, s->n * 8);
      s->q64 = gmd_alloc(gml->dev, s->n * 8);
      if(!s->p64 || !s->q64)
         return NULL;
   }
   if(mixed && !s->have32)
   {
      size_t nv = A->NmbCol * 32 * (size_t)A->BlkSiz * A->BlkSiz;
      s->A32 = *A;
      s->A32.FltSiz = 4;
      s->A32.Val = gmd_alloc(gml->dev, nv * 4);
      s->d32 = gmd_alloc(gml->dev, s->n * 4);
      s->r32 = gmd_alloc(gml->dev, s->n * 4);
      s->p32[0] = gmd_alloc(gml->dev, s->n * 4);
      s->p32[1] = gmd_alloc(gml->dev, s->n * 4);
      s->q32 = gmd_alloc(gml->dev, s->n * 4);
      if(!s->A32.Val || !s->d32 || !s->r32 || !s->p32[0] || !s->p32[1] || !s->q32)
         return NULL;
      if(!gmd_sv_to_f32(gml->dev, (const double *)A->Val, (float *)s->A32.Val, nv))
         return NULL;
      s->A32.bytes = A->bytes - nv * 4;
      s->have32 = 1;
   }
   return s;
}

/* the kernels of CG iteration i: FP64 on (x64, r64, p64, q64), three
   kernels; FP32 on (d32, r32, p32[i & 1] -> p32[~i & 1], q32), two.  Kernel k
   of the iteration is launched between the calls mark(k) and mark(k + 1)
   when mark is given (per-kernel timing). */
static int cg_iteration(GmlSct *gml, GmlSolver *s, int fs, int i,
                        int (*mark)(GmlSct *, GmlSolver *, int))
{
   const int nsp = gmd_sv_spmv_blocks(s->nrow);
   GmlSellDev *A64 = (GmlSellDev *)s->mat->Val;
   if(fs == 8)
      return (!mark || mark(gml, s, 0))
          && gmd_sv_spmv(gml->dev, A64, NULL, s->p64, NULL, s->q64, s->spart, s->sc)
          && (!mark || mark(gml, s, 1))
          && gmd_sv_update(gml->dev, 8, s->n, s->x64, s->r64, s->p64, s->q64, s->spart, 0,
                           s->part, s->sc)
          && (!mark || mark(gml, s, 2))
          && gmd_sv_dir(gml->dev, 8, s->n, s->p64, s->r64, s->sc)
          && (!mark || mark(gml, s, 3));
   {
      float *po = s->p32[i & 1], *pn = s->p32[(i & 1) ^ 1];
      return (!mark || mark(gml, s, 0))
          && gmd_sv_spmv(gml->dev, &s->A32, s->r32, po, pn, s->q32, s->spart, s->sc)
          && (!mark || mark(gml, s, 1))
          && gmd_sv_update(gml->dev, 4, s->n, s->d32, s->r32, pn, s->q32, s->spart, nsp,
                           s->part, s->sc)
          && (!mark || mark(gml, s, 2));
   }
}

static int capture(GmlSct *gml, GmlSolver *s, int fs, void **graph)
{
   int ok = 1;
   if(*graph)
      return 1;
   if(!gmd_graph_begin(gml->dev))
      return 0;
   for(int i=0;i<s->chunk && ok;i++)
      ok = cg_iteration(gml, s, fs, i, NULL);
   if(!gmd_graph_end(gml->dev, graph))
      return 0;
   return ok;
}

static int read_scalars(GmlSct *gml, GmlSolver *s, GmdSvScal *out);

/* replay the iteration graph until the device stop flag is set; two replays
   are kept in flight, each followed by a copy of the scalars to its own
   pinned slot.  Returns the iterations done, or -1. */
static int run_cg(GmlSct *gml, GmlSolver *s, void *graph, int maxit)
{
   int launched = 0, checked = 0, cap = maxit / s->chunk + 2;
   for(;;)
   {
      while(launched < cap && launched - checked < 2)
      {
         int slot = launched & 1;
         if(!gmd_graph_launch(gml->dev, graph)
         || !gmd_d2h_async(gml->dev, &s->hsc[slot], s->sc, sizeof(GmdSvScal))
         || !gmd_event_record(gml->dev, s->ev[slot]))
            return -1;
         launched++;
      }
      if(checked == launched)
         return -1;
      {
         int slot = checked & 1;
         if(!gmd_event_wait(s->ev[slot]))
            return -1;
         checked++;
         if(s->hsc[slot].done)
         {
            /* drain the replay still queued (it does nothing) */
            for(;checked<launched;checked++)
               if(!gmd_event_wait(s->ev[checked & 1]))
                  return -1;
            return s->hsc[slot].done == 2 ? -2 : s->hsc[slot].it;
         }
      }
      if(launched == cap && checked == launched)
         return -1;
   }
}

/* GML_CG_TRACE=1 prints the wall and device time of each phase of a solve
   (stderr); GML_CG_TRACE=2 also runs the iterations one kernel at a time
   without graphs and prints each kernel's mean device time */
static int trace_on(void)
{
   static int on = -1;
   if(on < 0)
   {
      const char *e = getenv("GML_CG_TRACE");
      on = e && (*e == '1' || *e == '2') ? *e - '0' : 0;
   }
   return on;
}

static int mark_event(GmlSct *gml, GmlSolver *s, int k)
{
   return gmd_event_record(gml->dev, s->tr[k]);
}

/* the iterations of run_cg, launched one by one with an event between the
   kernels; synchronises after each iteration */
static int run_cg_timed(GmlSct *gml, GmlSolver *s, int fs, int maxit)
{
   const int nk = fs == 8 ? 3 : 2;
   double t[3] = {0., 0., 0.};
   int n = 0;
   GmdSvScal h;
   for(;;)
   {
      if(!cg_iteration(gml, s, fs, n, mark_event) || !read_scalars(gml, s, &h))
         return -1;
      for(int k=0;k<nk;k++)
         t[k] += gmd_event_elapsed_s(s->tr[k], s->tr[k+1]);
      n++;
      if(h.done || n > maxit)
         break;
   }
   if(fs == 8)
      fprintf(stderr, "cg kernels fp64: spmv %.1f us  update %.1f us  dir %.1f us  (%d launches each)\n",
              1e6 * t[0] / n, 1e6 * t[1] / n, 1e6 * t[2] / n, n);
   else
      fprintf(stderr, "cg kernels fp32: spmv+dir %.1f us  update %.1f us  (%d launches each)\n",
              1e6 * t[0] / n, 1e6 * t[1] / n, n);
   return h.done == 1 ? h.it : h.done == 2 ? -2 : -1;
}

/* wall and device time of the phase that ends here; the device time runs
   from the previous trace point (events on the instance's stream) */
static void trace(GmlSct *gml, GmlSolver *s, const char *what, double *t, int it)
{
   double now, dev;
   if(!trace_on())
      return;
   gmd_event_record(gml->dev, s->tr[1]);
   dev = gmd_event_elapsed_s(s->tr[0], s->tr[1]);
   now = GmlGetWallClock();
   fprintf(stderr, "cg %-10s %8.3f ms wall %8.3f ms device  it %d  chunk %d\n", what,
           1e3 * (now - *t), 1e3 * dev, it, s->chunk);
   *t = now;
   gmd_event_record(gml->dev, s->tr[0]);
}

static int read_scalars(GmlSct *gml, GmlSolver *s, GmdSvScal *out)
{
   if(!gmd_d2h_async(gml->dev, &s->hsc[0], s->sc, sizeof(GmdSvScal)) || !gmd_sync(gml->dev))
      return 0;
   *out = s->hsc[0];
   return 1;
}

int GmlxSolveCG(size_t GmlIdx, int MatIdx, int RhsIdx, int SolIdx, int mode, double tol,
                int MaxIte, GmlxSolveInfo *info)
{
   GETGMLPTR(gml, GmlIdx);
   GmlMatSct *mat;
   GmlVecSct *rv, *sv;
   GmlSellDev *A;
   GmlSolver *s;
   GmdSvScal h;
   int it = 0, out = 0, r;
   double tin, tt = GmlGetWallClock();

   if(info)
      memset(info, 0, sizeof(GmlxSolveInfo));
   if(gml->Offline)
      return 0;
   if(MatIdx < 1 || MatIdx > GmlMaxMat || !gml->mat[MatIdx].use)
   {
      printf("Invalid matrix index: %d\n", MatIdx);
      return -1;
   }
   mat = &gml->mat[MatIdx];
   A = (GmlSellDev *)mat->Val;
   if(RhsIdx < 1 || RhsIdx > GmlMaxVec || !gml->vec[RhsIdx].use
   || SolIdx < 1 || SolIdx > GmlMaxVec || !gml->vec[SolIdx].use)
   {
      printf("Invalid vector index: %d or %d\n", RhsIdx, SolIdx);
      return -2;
   }
   rv = &gml->vec[RhsIdx];
   sv = &gml->vec[SolIdx];
   if(mat->FltTyp != GmlDbl || rv->FltTyp != GmlDbl || sv->FltTyp != GmlDbl
   || rv->BlkSiz != mat->BlkSiz || sv->BlkSiz != mat->BlkSiz
   || rv->NmbLin != mat->NmbLin || sv->NmbLin != mat->NmbLin)
   {
      printf("GmlxSolveCG needs an FP64 matrix and FP64 vectors of its size and block size\n");
      return -3;
   }
   if((mode != GmlxCgFp64 && mode != GmlxCgMixed) || !(tol > 0.) || MaxIte < 1)
      return -4;
   if(!(s = solver_get(gml, mat, mode == GmlxCgMixed)))
   {
      printf("Cannot allocate the solver's work vectors\n");
      return -5;
   }
   if(rv->NmbValTyp * rv->VecValSiz != s->vs || sv->NmbValTyp * sv->VecValSiz != s->vs)
      return -3;
   gmd_event_record(gml->dev, s->t0);
   if(trace_on())
      gmd_event_record(gml->dev, s->tr[0]);

   if(mode == GmlxCgFp64)
   {
      if(!gmd_sv_init(gml->dev, s->n, s->B, gml->dat[rv->idx].GpuMem, s->b64, s->x64, s->r64, s->p64,
                      8, s->part, s->sc, tol * tol, MaxIte)
      || !capture(gml, s, 8, &s->g64))
         return -6;
      r = trace_on() == 2 ? run_cg_timed(gml, s, 8, MaxIte) : run_cg(gml, s, s->g64, MaxIte);
      trace(gml, s, "fp64 cg", &tt, r);
      if(r < 0)
      {
         printf("CG failed (%s)\n", r == -2 ? "p.Ap <= 0: matrix not positive definite" : "device");
         return -7;
      }
      it = r;
      out = 1;
      if(!gmd_sv_residual(gml->dev, A, s->b64, s->x64, s->r64, s->part, s->sc))
         return -6;
   }
   else
   {
      tin = inner_factor();
      if(!gmd_sv_init(gml->dev, s->n, s->B, gml->dat[rv->idx].GpuMem, s->b64, s->x64, s->r64, s->r64,
                      8, s->part, s->sc, tol * tol, MaxIte)
      || !capture(gml, s, 4, &s->g32))
         return -6;
      if(!read_scalars(gml, s, &h))
         return -6;
      trace(gml, s, "init", &tt, 0);
      while(h.rt > tol * tol * h.bb && out < GML_CG_MAXOUT && it < MaxIte)
      {
         if(!gmd_sv_ir_begin(gml->dev, s->n, s->r64, s->r32, s->p32[0], s->d32, s->part, s->sc,
                             tin * tin, MaxIte - it))
            return -6;
         r = trace_on() == 2 ? run_cg_timed(gml, s, 4, MaxIte - it)
                             : run_cg(gml, s, s->g32, MaxIte - it);
         trace(gml, s, "fp32 cg", &tt, r);
         if(r < 0)
         {
            printf("CG failed (%s)\n", r == -2 ? "p.Ap <= 0: matrix not positive definite" : "device");
            return -7;
         }
         it += r;
         out++;
         if(!gmd_sv_ir_end(gml->dev, s->n, s->x64, s->d32, s->sc)
         || !gmd_sv_residual(gml->dev, A, s->b64, s->x64, s->r64, s->part, s->sc)
         || !read_scalars(gml, s, &h))
            return -6;
         trace(gml, s, "residual", &tt, 0);
      }
   }

   if(!gmd_d2d_async(gml->dev, gml->dat[sv->idx].GpuMem, s->x64, s->n * 8))
      return -6;
   gmd_event_record(gml->dev, s->t1);
   if(!read_scalars(gml, s, &h))
      return -6;
   if(info)
   {
      info->NmbIte = it;
      info->NmbOut = out;
      info->RelRes = h.bb > 0. ? sqrt(h.rt / h.bb) : 0.;
      info->Seconds = gmd_event_elapsed_s(s->t0, s->t1);
   }
   return h.rt <= tol * tol * h.bb ? 1 : 0;
}
