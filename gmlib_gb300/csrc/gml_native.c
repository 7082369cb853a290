/*
 * gml_native.c -- host side of the native mesh kernels (no counterpart in the
 * reference API): topology setup, Laplacian smoothing over the ball of
 * points, mean-ratio quality statistics, and the smoothing workload captured
 * as a CUDA graph.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"
#include "gml_mesh.h"

#include "gml_native.h"

/* measured on the 128^3 smoothing step: the quality pass on 2 blocks per
   SM beside the sweep on 3 overlaps best (1.31 ms against 1.42 ms with
   both on their full grids) */
#ifndef GML_SPLIT_Q
#define GML_SPLIT_Q 2
#endif
#ifndef GML_SPLIT_L
#define GML_SPLIT_L 3
#endif

static int ready(GmlSct *gml, NatSct **n, GmlDatSct **ver, GmlDatSct **tet);
static int sweeps(GmlSct *gml, NatSct *n, GmlDatSct *ver, int ns, float omega);

NatSct *gmlx_nat(GmlSct *gml)
{
   if(!gml->ext)
      gml->ext = calloc(1, sizeof(NatSct));
   return (NatSct *)gml->ext;
}

static void free_state(GmlSct *gml, NatSct *n)
{
   gmd_sync(gml->dev);
   gmd_free(gml->dev, n->ptr);   gmd_free(gml->dev, n->vt);
   gmd_free(gml->dev, n->tmp);   gmd_free(gml->dev, n->err);
   gmd_free(gml->dev, n->fixed); gmd_free(gml->dev, n->pdeg);
   gmd_free(gml->dev, n->pcol);  gmd_free(gml->dev, n->rowv);
   gmd_free(gml->dev, n->width); gmd_free(gml->dev, n->soff);
   gmd_free(gml->dev, n->crd2);
   gmd_free(gml->dev, n->flags); gmd_free(gml->dev, n->stats);
   gmd_graph_free(n->graph);
   for(int e=0;e<=GML_MAXSTATS;e++)
   {
      gmd_event_free(n->evL[e]);
      gmd_event_free(n->evQ[e]);
   }
   memset(n, 0, sizeof(NatSct));
}

void gmlx_native_release(GmlSct *gml)
{
   if(gml->ext)
   {
      free_state(gml, (NatSct *)gml->ext);
      free(gml->ext);
      gml->ext = NULL;
   }
}

static int mesh_dat(GmlSct *gml, GmlDatSct **ver, GmlDatSct **tet)
{
   if(!gml->TypIdx[ GmlVertices ] || !gml->TypIdx[ GmlTetrahedra ])
   {
      puts("The native mesh kernels need vertices and tetrahedra.");
      return 0;
   }
   *ver = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   *tet = &gml->dat[ gml->TypIdx[ GmlTetrahedra ] ];
   return 1;
}

int GmlxMeshSetup(size_t GmlIdx, int fix)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *ver, *tet;
   NatSct *n;
   int nv, nt, err = 0, *pdeg_h, nslice;
   long long tot;

   if(gml->Offline || !mesh_dat(gml, &ver, &tet))
      return 0;

   n = gmlx_nat(gml);
   {
      const int wreq = n->wreq;
      free_state(gml, n);
      n->wreq = wreq;
   }
   nv = ver->NmbLin;
   nt = tet->NmbLin;
   if(nv >= (1 << 26))
   {
      puts("GmlxMeshSetup: more than 2^26 vertices");
      return 0;
   }
   n->nv = nv;
   n->nrow = ((nv + GML_SIGMA - 1) / GML_SIGMA) * GML_SIGMA;
   n->window = n->wreq ? n->wreq : gmlx_tune_get("w", 0, nv, gmd_num_sms(gml->dev));
   if(n->window != 32 && n->window != 64 && n->window != 128 && n->window != GML_SIGMA)
      n->window = GML_SIGMA;
   nslice = n->nrow / 32;
   n->nt = nt;
   n->fix = fix;

   n->ptr   = gmd_alloc(gml->dev, (size_t)(nv + 1) * sizeof(int));
   n->vt    = gmd_alloc(gml->dev, (size_t)nt * 4 * sizeof(int));
   n->tmp   = gmd_alloc(gml->dev, (size_t)nv * sizeof(int));
   n->err   = gmd_alloc(gml->dev, sizeof(int));
   n->pdeg  = gmd_alloc(gml->dev, (size_t)nv * sizeof(int));
   n->rowv  = gmd_alloc(gml->dev, (size_t)n->nrow * sizeof(unsigned));
   n->width = gmd_alloc(gml->dev, (size_t)(nslice + 1) * sizeof(long long));
   n->soff  = gmd_alloc(gml->dev, (size_t)(nslice + 1) * sizeof(long long));
   n->crd2  = gmd_alloc(gml->dev, (size_t)nv * 16);
   n->flags = gmd_alloc(gml->dev, (size_t)((nt + 31) / 32) * sizeof(unsigned));
   n->stats = gmd_alloc(gml->dev, GML_MAXSTATS * sizeof(GmlxQualStats));
   n->nstats = GML_MAXSTATS;
   if(!n->ptr || !n->vt || !n->tmp || !n->err || !n->pdeg || !n->rowv || !n->width
   || !n->soff || !n->crd2 || !n->flags || !n->stats)
   {
      free_state(gml, n);
      return 0;
   }

   if(!gmd_mesh_vt_csr(gml->dev, tet->GpuMem, nt, nv, n->ptr, n->vt, n->tmp, n->err))
   {
      free_state(gml, n);
      return 0;
   }

   if(fix == 1)
   {
      /* vertices with a non-zero reference are fixed, read from the device
         copy of the references (zero until set, as the host mirror), in
         stream order after any upload of them */
      const GmlDatSct *rd = gml->RefIdx[ GmlVertices ] ? &gml->dat[ gml->RefIdx[ GmlVertices ] ] : NULL;
      n->fixed = gmd_alloc(gml->dev, (size_t)nv * sizeof(int));
      if(!n->fixed || (rd && rd->GpuMem && rd->NmbLin >= nv
                       && !gmd_mesh_fixed_from_ref(gml->dev, (const int *)rd->GpuMem, nv, n->fixed)))
      {
         free_state(gml, n);
         return 0;
      }
   }
   else if(fix == 2)
   {
      n->fixed = gmd_alloc(gml->dev, (size_t)nv * sizeof(int));
      gmd_mesh_boundary(gml->dev, tet->GpuMem, nt, n->ptr, n->vt, n->fixed);
   }

   if(!gmd_mesh_point_count(gml->dev, tet->GpuMem, nv, n->ptr, n->vt, n->fixed, n->pdeg,
                            n->rowv, n->width, n->soff, n->err, n->window))
   {
      free_state(gml, n);
      return 0;
   }

   pdeg_h = malloc((size_t)nv * sizeof(int));
   if(!pdeg_h)
   {
      free_state(gml, n);
      return 0;
   }
   gmd_d2h(gml->dev, &err, n->err, sizeof(int));
   gmd_d2h(gml->dev, &tot, n->soff + nslice, sizeof(long long));
   gmd_d2h(gml->dev, pdeg_h, n->pdeg, (size_t)nv * sizeof(int));

   if(err)
   {
      printf("GmlxMeshSetup: %s\n", (err & 2) ? "vertex index out of range in the tetrahedra"
                                               : "a ball of points exceeds 63 vertices");
      free(pdeg_h);
      free_state(gml, n);
      return 0;
   }

   n->stored = tot * 32;
   n->used = 0;
   n->maxdeg = 0;
   for(int i=0;i<nv;i++)
   {
      n->used += pdeg_h[i];
      if(pdeg_h[i] > n->maxdeg) n->maxdeg = pdeg_h[i];
   }
   free(pdeg_h);

   n->pcol = gmd_alloc(gml->dev, (size_t)(tot > 0 ? tot : 1) * 32 * sizeof(int));
   if(!n->pcol)
   {
      free_state(gml, n);
      return 0;
   }
   gmd_mesh_point_fill(gml->dev, tet->GpuMem, n->nrow, n->ptr, n->vt, n->rowv, n->soff, n->pcol);
   gmd_sync(gml->dev);
   n->ready = 1;
   return 1;
}

int GmlxSetBallWindow(size_t GmlIdx, int window)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n;
   if(window && window != 32 && window != 64 && window != 128 && window != GML_SIGMA)
      return 0;
   if(!(n = gmlx_nat(gml)))
      return 0;
   n->wreq = window;
   return 1;
}

int GmlxBallWindow(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n = gml->ext;
   return n && n->ready ? n->window : 0;
}

/* Time nsweeps sweeps with each sorting window on the current mesh (rebuilt
   by GmlxMeshSetup with the fixing rule in force), keep the fastest, record
   it in the tuning table for meshes of this size, and leave the mesh built
   with it; the coordinates are restored. */
int GmlxMeshTune(size_t GmlIdx, int nsweeps, float omega)
{
   static const int cand[] = { 64, 128, GML_SIGMA };
   GETGMLPTR(gml, GmlIdx);
   NatSct *n;
   GmlDatSct *ver, *tet;
   void *save, *e0, *e1;
   double best_t = 1e30;
   int best = GML_SIGMA, fix;

   if(!ready(gml, &n, &ver, &tet) || nsweeps < 1)
      return 0;
   fix = n->fix;
   if(!(save = gmd_alloc(gml->dev, (size_t)n->nv * 16)))
      return 0;
   e0 = gmd_event_new();
   e1 = gmd_event_new();
   gmd_d2d_async(gml->dev, save, ver->GpuMem, (size_t)n->nv * 16);
   for(int c=0;c<(int)(sizeof(cand) / sizeof(cand[0]));c++)
   {
      double t;
      n->wreq = cand[c];
      if(!GmlxMeshSetup(GmlIdx, fix) || !sweeps(gml, n, ver, 1, omega))
         break;
      gmd_event_record(gml->dev, e0);
      if(!sweeps(gml, n, ver, nsweeps, omega))
         break;
      gmd_event_record(gml->dev, e1);
      t = gmd_event_elapsed_s(e0, e1);
      gmd_d2d_async(gml->dev, ver->GpuMem, save, (size_t)n->nv * 16);
      if(t > 0. && t < best_t)
      {
         best_t = t;
         best = cand[c];
      }
   }
   gmd_d2d_async(gml->dev, ver->GpuMem, save, (size_t)n->nv * 16);
   gmd_sync(gml->dev);
   gmd_free(gml->dev, save);
   gmd_event_free(e0);
   gmd_event_free(e1);
   gmlx_tune_set("w", 0, n->nv, gmd_num_sms(gml->dev), best);
   n->wreq = best;
   if(!GmlxMeshSetup(GmlIdx, fix))
      return 0;
   return best;
}

int GmlxMeshBallInfo(size_t GmlIdx, long long *stored, long long *used, int *maxdeg)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n = gml->ext;
   if(!n || !n->ready)
      return 0;
   if(stored) *stored = n->stored;
   if(used) *used = n->used;
   if(maxdeg) *maxdeg = n->maxdeg;
   return 1;
}

static int ready(GmlSct *gml, NatSct **n, GmlDatSct **ver, GmlDatSct **tet)
{
   *n = gml->ext;
   if(!*n || !(*n)->ready)
   {
      puts("GmlxMeshSetup must be called first.");
      return 0;
   }
   if(!mesh_dat(gml, ver, tet))
      return 0;
   if((*ver)->NmbLin != (*n)->nv || (*tet)->NmbLin != (*n)->nt)
   {
      puts("The mesh changed since GmlxMeshSetup.");
      return 0;
   }
   return 1;
}

/* sweeps alternate between the vertex buffer and a second buffer; an odd
   count ends with a copy back */
static int sweeps(GmlSct *gml, NatSct *n, GmlDatSct *ver, int ns, float omega)
{
   void *a = ver->GpuMem, *b = n->crd2;
   for(int s=0;s<ns;s++)
   {
      if(!gmd_mesh_laplace(gml->dev, n->nrow, n->rowv, n->soff, n->pcol, a, b, omega, n->err, 0))
         return 0;
      void *t = a; a = b; b = t;
   }
   if(a != ver->GpuMem)
      gmd_d2d_async(gml->dev, ver->GpuMem, a, (size_t)n->nv * 16);
   return 1;
}

int GmlxSmooth(size_t GmlIdx, int nsweeps, float omega)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n;
   GmlDatSct *ver, *tet;
   if(!ready(gml, &n, &ver, &tet) || nsweeps < 0)
      return 0;
   if(!n->NmbSweepKrn)
      n->NmbSweepKrn = gml_new_kernel_slot(gml, GmlKrnGenerated + 100, "laplace_sell");
   gml_lib_timer_begin(gml, &gml->krn[ n->NmbSweepKrn ]);
   if(!sweeps(gml, n, ver, nsweeps, omega))
      return 0;
   gml_lib_timer_end(gml, &gml->krn[ n->NmbSweepKrn ]);
   return 1;
}

void gmlx_decode_stats(const GmlxQualStats *s, GmlxQuality *r)
{
   unsigned kmin = (unsigned)(s->MinKey >> 32), kmax = ~(unsigned)(s->MaxKey >> 32);
   unsigned umin = (kmin & 0x80000000u) ? (kmin & 0x7fffffffu) : ~kmin;
   unsigned umax = (kmax & 0x80000000u) ? (kmax & 0x7fffffffu) : ~kmax;
   memcpy(&r->MinQal, &umin, 4);
   memcpy(&r->MaxQal, &umax, 4);
   r->MinIdx = (int)(s->MinKey & 0xffffffffu);
   r->MaxIdx = (int)(s->MaxKey & 0xffffffffu);
   r->SumQal = s->Sum;
   r->NmbInv = s->NmbInv;
   r->NmbF64 = s->NmbF64;
   memcpy(r->Hist, s->Hist, sizeof(r->Hist));
}

/* device error bits set by the kernels: 1 ball too large, 2 bad vertex
   index, 4 a shared-memory staging copy did not arrive in time */
static int device_errors(GmlSct *gml, NatSct *n)
{
   int err = 0;
   gmd_d2h(gml->dev, &err, n->err, sizeof(int));
   if(err & 4)
      puts("GMlib: a quality-kernel staging copy timed out; statistics are incomplete.");
   return err;
}

float gmlx_det_threshold(double h)
{
   return (float)(1e-6 * h * h * h);
}

int GmlxQualityStats(size_t GmlIdx, double h, int QalIdx, GmlxQuality *res)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n;
   GmlDatSct *ver, *tet, *q = NULL;
   GmlxQualStats st;

   if(!ready(gml, &n, &ver, &tet))
      return 0;
   if(QalIdx)
   {
      if(QalIdx < 1 || QalIdx > GmlMaxDat || !gml->dat[QalIdx].use)
         return 0;
      q = &gml->dat[ QalIdx ];
      if(q->ItmTyp != GmlFlt || q->NmbItm != 1 || q->NmbLin != n->nt)
         return 0;
   }
   if(!n->NmbQalKrn)
      n->NmbQalKrn = gml_new_kernel_slot(gml, GmlKrnGenerated + 100, "tet_quality");
   gml_lib_timer_begin(gml, &gml->krn[ n->NmbQalKrn ]);
   gmd_mesh_stats_init(gml->dev, n->stats, 1);
   if(!gmd_mesh_quality(gml->dev, n->nt, tet->GpuMem, ver->GpuMem, gmlx_det_threshold(h),
                        q ? (float *)q->GpuMem : NULL, n->flags, n->stats, n->err, 0))
      return 0;
   gml_lib_timer_end(gml, &gml->krn[ n->NmbQalKrn ]);
   if(res)
   {
      if(!gmd_d2h(gml->dev, &st, n->stats, sizeof(st)) || (device_errors(gml, n) & 4))
         return 0;
      gmlx_decode_stats(&st, res);
   }
   return 1;
}

int GmlxInvertedFlags(size_t GmlIdx, unsigned *flags, size_t nwords)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n = gml->ext;
   size_t need;
   if(!n || !n->ready)
      return 0;
   need = (size_t)(n->nt + 31) / 32;
   if(nwords < need)
      return 0;
   return gmd_d2h(gml->dev, flags, n->flags, need * sizeof(unsigned));
}

/* resident blocks per SM of the quality pass and of the sweep when they run
   side by side in the graph (0: each kernel's maximum) */
static void graph_split(int *qb, int *lb)
{
   *qb = GML_SPLIT_Q;
   *lb = GML_SPLIT_L;
}

int GmlxSmoothQualityLoop(size_t GmlIdx, int nsweeps, float omega, double h, GmlxQuality *res)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n;
   GmlDatSct *ver, *tet;
   GmlxQualStats *st;
   int qb = 0, lb = 0;

   if(!ready(gml, &n, &ver, &tet) || nsweeps < 1 || nsweeps > n->nstats)
      return 0;

   if(!n->graph || n->gsweeps != nsweeps || n->gomega != omega || n->gh != h
   || n->gver != ver->GpuMem || n->gtet != tet->GpuMem)
   {
      void *a = ver->GpuMem, *b = n->crd2;
      gmd_graph_free(n->graph);
      n->graph = NULL;
      /* Sweep s+1 and the quality of sweep s read the same coordinates and
         are independent: the graph runs them on two streams.  Sweep s+2
         overwrites the buffer that quality s reads (ping-pong), so it waits
         for it.  x_s lives in a when s is even, in b when s is odd. */
      if(!n->evL[0])
         for(int e=0;e<=GML_MAXSTATS;e++)
         {
            n->evL[e] = gmd_event_new_sync();
            n->evQ[e] = gmd_event_new_sync();
         }
      graph_split(&qb, &lb);
      if(!gmd_graph_begin(gml->dev))
         return 0;
      gmd_mesh_stats_init(gml->dev, n->stats, nsweeps);
      gmd_event_record(gml->dev, n->evL[0]);
      gmd_mesh_laplace(gml->dev, n->nrow, n->rowv, n->soff, n->pcol, a, b, omega, n->err, 0);
      gmd_event_record(gml->dev, n->evL[1]);
      for(int s=1;s<=nsweeps;s++)
      {
         void *xs = (s & 1) ? b : a, *xn = (s & 1) ? a : b;
         gmd_use_side(gml->dev, 1);
         gmd_stream_wait(gml->dev, n->evL[s]);
         gmd_mesh_quality(gml->dev, n->nt, tet->GpuMem, xs, gmlx_det_threshold(h), NULL, n->flags,
                          n->stats + s - 1, n->err, qb);
         gmd_event_record(gml->dev, n->evQ[s]);
         gmd_use_side(gml->dev, 0);
         if(s < nsweeps)
         {
            if(s >= 2)
               gmd_stream_wait(gml->dev, n->evQ[s-1]);
            gmd_mesh_laplace(gml->dev, n->nrow, n->rowv, n->soff, n->pcol, xs, xn, omega, n->err, lb);
            gmd_event_record(gml->dev, n->evL[s+1]);
         }
      }
      gmd_stream_wait(gml->dev, n->evQ[nsweeps]);
      if(nsweeps & 1)
         gmd_d2d_async(gml->dev, ver->GpuMem, b, (size_t)n->nv * 16);
      if(!gmd_graph_end(gml->dev, &n->graph))
         return 0;
      n->gsweeps = nsweeps;
      n->gomega = omega;
      n->gh = h;
      n->gver = ver->GpuMem;
      n->gtet = tet->GpuMem;
   }

   if(!n->NmbLoopKrn)
      n->NmbLoopKrn = gml_new_kernel_slot(gml, GmlKrnGenerated + 100, "smooth_quality_graph");
   gml_lib_timer_begin(gml, &gml->krn[ n->NmbLoopKrn ]);
   if(!gmd_graph_launch(gml->dev, n->graph))
      return 0;
   gml_lib_timer_end(gml, &gml->krn[ n->NmbLoopKrn ]);

   if(res)
   {
      st = malloc((size_t)nsweeps * sizeof(GmlxQualStats));
      if(!st || !gmd_d2h(gml->dev, st, n->stats, (size_t)nsweeps * sizeof(GmlxQualStats))
      || (device_errors(gml, n) & 4))
      {
         free(st);
         return 0;
      }
      for(int s=0;s<nsweeps;s++)
         gmlx_decode_stats(&st[s], &res[s]);
      free(st);
   }
   return 1;
}

int GmlxMeshBytes(size_t GmlIdx, double *sweep_bytes, double *quality_bytes)
{
   GETGMLPTR(gml, GmlIdx);
   NatSct *n = gml->ext;
   if(!n || !n->ready)
      return 0;
   /* sweep: degree + used ball columns + own coordinates read + write;
      quality: connectivity + coordinates once + flag words */
   if(sweep_bytes)
      *sweep_bytes = 4.0 * n->nv + 4.0 * (double)n->used + 32.0 * n->nv;
   if(quality_bytes)
      *quality_bytes = 16.0 * n->nt + 16.0 * n->nv + 4.0 * ((n->nt + 31) / 32);
   return 1;
}
