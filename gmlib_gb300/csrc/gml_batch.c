/*
 * gml_batch.c -- many tetrahedral meshes of uneven size smoothed and
 * measured together (no counterpart in the reference, which handles one mesh
 * per instance and one launch per kernel call, sources/gmlib3.c:3064-3222).
 *
 * Layout.  The meshes are packed into the instance's vertex and tetrahedron
 * datatypes: mesh m owns vertices [VerOff[m], VerOff[m] + NmbVer[m]) and
 * tets [TetOff[m], TetOff[m] + NmbTet[m]), its tets holding packed vertex
 * indices.  Every VerOff is a multiple of 256 (padding vertices are fixed
 * and belong to no tet), so the ball-of-points windows and slices built by
 * GmlxMeshSetup on the packed mesh never mix two meshes.  Inverted-element
 * flags are per mesh, from word FlgOff[m].
 *
 * Work.  GmlxBatchRun applies nsweeps Jacobi sweeps then the quality pass to
 * every mesh, in one of two ways:
 *   GmlxBatchQueue  one persistent launch drains a (mesh, range) tile queue:
 *                   phase-major tiles, a tile waits only for the previous
 *                   phase of its own mesh (device counters), so small and
 *                   large meshes overlap; the launch and its counter resets
 *                   are captured once as a CUDA graph and replayed;
 *   GmlxBatchLoop   the plain per-mesh launch loop (nsweeps sweep launches
 *                   and one quality launch per mesh), for comparison.
 * Both give the same per-mesh results as running the mesh alone: the sweep
 * arithmetic per vertex and the quality per tet are the same; only the FP64
 * sum of the qualities depends on the accumulation order.
 *
 * Tuning.  GmlxBatchTune times the queue on the packed meshes (restoring
 * the coordinates afterwards) with tiles claimed per block or per warp,
 * several tile sizes and two grid sizes, and keeps the fastest.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_native.h"
#include "gml_device.h"

#define BAT_ALIGN 256

typedef struct
{
   int            nmesh, nv, nt, ready, fix;
   int            *VerOff, *TetOff, *FlgOff, *NmbVer, *NmbTet;
   double         *h;
   GmdBatchMesh   *mh, *md;
   GmdBatchTile   *td;
   int            *need, *done, *ctl;      /* ctl: head, abort, err */
   int            ntile, nphase, tsweeps;
   int            tile_slices, tile_tets, grid, maxgrid;
   int            warp;                   /* 1: tiles claimed per warp */
   unsigned       *flags;
   GmlxQualStats  *stats, *hstats;
   void           *graph;
   int            gsweeps;
   float          gomega;
   int            *hneed;                 /* host copy of need */
   int            spin, hold;             /* wait limit; tiles held back (GmlxBatchSetWaitLimit) */
}BatSct;

#define BAT_SPIN (1 << 22)                 /* default wait limit: about 1 s */

static void bat_free_tiles(GmlSct *gml, BatSct *b)
{
   free(b->hneed);              b->hneed = NULL;
   gmd_free(gml->dev, b->td);   b->td = NULL;
   gmd_free(gml->dev, b->need); b->need = NULL;
   gmd_free(gml->dev, b->done); b->done = NULL;
   gmd_graph_free(b->graph);    b->graph = NULL;
   b->ntile = 0;
   b->tsweeps = -1;
}

void gmlx_batch_release(GmlSct *gml)
{
   BatSct *b = (BatSct *)gml->bat;
   if(!b)
      return;
   gmd_sync(gml->dev);
   bat_free_tiles(gml, b);
   gmd_free(gml->dev, b->md);
   gmd_free(gml->dev, b->ctl);
   gmd_free(gml->dev, b->flags);
   gmd_free(gml->dev, b->stats);
   gmd_host_free(b->hstats);
   free(b->VerOff); free(b->TetOff); free(b->FlgOff); free(b->NmbVer); free(b->NmbTet);
   free(b->h); free(b->mh);
   free(b);
   gml->bat = NULL;
}

static BatSct *bat(GmlSct *gml)
{
   BatSct *b = (BatSct *)gml->bat;
   if(!b)
      puts("GmlxBatchCreate must be called first.");
   return b;
}

int GmlxBatchCreate(size_t GmlIdx, int NmbMsh, const int *NmbVer, const int *NmbTet,
                    const double *h)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b;
   long long nv = 0, nt = 0, nf = 0;
   int m, vi, ti;

   if(gml->Offline || NmbMsh < 1 || !NmbVer || !NmbTet || !h)
      return 0;
   if(gml->bat || gml->TypIdx[ GmlVertices ] || gml->TypIdx[ GmlTetrahedra ])
   {
      puts("GmlxBatchCreate needs an instance without vertices and tetrahedra.");
      return 0;
   }
   for(m=0;m<NmbMsh;m++)
   {
      if(NmbVer[m] < 1 || NmbTet[m] < 1)
         return 0;
      nv += ((long long)NmbVer[m] + BAT_ALIGN - 1) / BAT_ALIGN * BAT_ALIGN;
      nt += NmbTet[m];
      nf += (NmbTet[m] + 31) / 32;
   }
   if(nv >= (1LL << 26) || nt > 2147483647LL)
   {
      puts("GmlxBatchCreate: more than 2^26 packed vertices or 2^31 tets");
      return 0;
   }

   b = calloc(1, sizeof(BatSct));
   if(!b)
      return 0;
   gml->bat = b;
   b->nmesh = NmbMsh;
   b->nv = (int)nv;
   b->nt = (int)nt;
   b->tsweeps = -1;
   b->tile_slices = 32;
   b->tile_tets = 4096;
   b->VerOff = malloc((size_t)(NmbMsh + 1) * sizeof(int));
   b->TetOff = malloc((size_t)(NmbMsh + 1) * sizeof(int));
   b->FlgOff = malloc((size_t)(NmbMsh + 1) * sizeof(int));
   b->NmbVer = malloc((size_t)NmbMsh * sizeof(int));
   b->NmbTet = malloc((size_t)NmbMsh * sizeof(int));
   b->h = malloc((size_t)NmbMsh * sizeof(double));
   b->mh = calloc((size_t)NmbMsh, sizeof(GmdBatchMesh));
   if(!b->VerOff || !b->TetOff || !b->FlgOff || !b->NmbVer || !b->NmbTet || !b->h || !b->mh)
      goto fail;
   b->VerOff[0] = b->TetOff[0] = b->FlgOff[0] = 0;
   for(m=0;m<NmbMsh;m++)
   {
      b->NmbVer[m] = NmbVer[m];
      b->NmbTet[m] = NmbTet[m];
      b->h[m] = h[m];
      b->VerOff[m+1] = b->VerOff[m] + (NmbVer[m] + BAT_ALIGN - 1) / BAT_ALIGN * BAT_ALIGN;
      b->TetOff[m+1] = b->TetOff[m] + NmbTet[m];
      b->FlgOff[m+1] = b->FlgOff[m] + (NmbTet[m] + 31) / 32;
   }

   b->md = gmd_alloc(gml->dev, (size_t)NmbMsh * sizeof(GmdBatchMesh));
   b->ctl = gmd_alloc(gml->dev, 4 * sizeof(int));
   b->flags = gmd_alloc(gml->dev, (size_t)(nf > 0 ? nf : 1) * sizeof(unsigned));
   b->stats = gmd_alloc(gml->dev, (size_t)NmbMsh * sizeof(GmlxQualStats));
   b->hstats = gmd_host_alloc((size_t)NmbMsh * sizeof(GmlxQualStats));
   if(!b->md || !b->ctl || !b->flags || !b->stats || !b->hstats)
      goto fail;

   if(!(vi = GmlNewMeshData(GmlIdx, GmlVertices, b->nv))
   || !(ti = GmlNewMeshData(GmlIdx, GmlTetrahedra, b->nt)))
      goto fail;
   /* padding vertices: at the origin and fixed */
   {
      int *ref = (int *)gml->dat[ gml->RefIdx[ GmlVertices ] ].CpuMem;
      for(m=0;m<NmbMsh;m++)
         for(int v=b->VerOff[m]+NmbVer[m];v<b->VerOff[m+1];v++)
            ref[v] = 1;
   }
   return 1;

fail:
   gmlx_batch_release(gml);
   return 0;
}

int GmlxBatchSetMesh(size_t GmlIdx, int MshIdx, const float *crd, const int *ref, const int *tet)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   GmlDatSct *vd, *rd, *td;
   int m = MshIdx, i, nv;
   float *vc;
   int *vr, *tc;

   if(!b || m < 0 || m >= b->nmesh || !crd || !tet)
      return 0;
   vd = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   rd = &gml->dat[ gml->RefIdx[ GmlVertices ] ];
   td = &gml->dat[ gml->TypIdx[ GmlTetrahedra ] ];
   nv = b->NmbVer[m];
   for(i=0;i<4*b->NmbTet[m];i++)
      if(tet[i] < 0 || tet[i] >= nv)
      {
         printf("GmlxBatchSetMesh: mesh %d, tet %d has vertex %d out of range\n", m, i / 4, tet[i]);
         return 0;
      }
   gml_wait_upload(gml, vd);
   gml_wait_upload(gml, rd);
   gml_wait_upload(gml, td);
   vc = (float *)vd->CpuMem + 4 * (size_t)b->VerOff[m];
   vr = (int *)rd->CpuMem + b->VerOff[m];
   tc = (int *)td->CpuMem + 4 * (size_t)b->TetOff[m];
   memcpy(vc, crd, (size_t)nv * 4 * sizeof(float));
   for(i=0;i<nv;i++)
      vr[i] = ref ? ref[i] : 0;
   for(i=0;i<4*b->NmbTet[m];i++)
      tc[i] = tet[i] + b->VerOff[m];
   b->ready = 0;
   return 1;
}

int GmlxBatchGetMesh(size_t GmlIdx, int MshIdx, float *crd)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   GmlDatSct *vd;
   if(!b || MshIdx < 0 || MshIdx >= b->nmesh || !crd)
      return 0;
   vd = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   return gmd_d2h(gml->dev, crd, (const char *)vd->GpuMem + (size_t)b->VerOff[MshIdx] * 16,
                  (size_t)b->NmbVer[MshIdx] * 16);
}

/* tile table for nsweeps sweeps with the current tile sizes */
static int bat_tiles(GmlSct *gml, BatSct *b, int nsweeps)
{
   int nphase = nsweeps + 1, m, p, cnt = 0, k;
   size_t cap = 0;
   GmdBatchTile *t;
   int *need;

   if(b->td && b->tsweeps == nsweeps)
      return 1;
   bat_free_tiles(gml, b);
   for(m=0;m<b->nmesh;m++)
   {
      int ns = (b->VerOff[m+1] - b->VerOff[m]) / 32;
      cap += (size_t)nsweeps * ((ns + b->tile_slices - 1) / b->tile_slices);
      cap += (size_t)((b->NmbTet[m] + b->tile_tets - 1) / b->tile_tets);
   }
   if(cap > 2147483647u)
      return 0;
   t = malloc(cap * sizeof(GmdBatchTile));
   need = calloc((size_t)b->nmesh * nphase, sizeof(int));
   if(!t || !need)
   {
      free(t); free(need);
      return 0;
   }
   for(p=0;p<nsweeps;p++)
      for(m=0;m<b->nmesh;m++)
      {
         int s0 = b->VerOff[m] / 32, s1 = b->VerOff[m+1] / 32;
         for(k=s0;k<s1;k+=b->tile_slices)
         {
            GmdBatchTile x = { p, m, k, k + b->tile_slices < s1 ? k + b->tile_slices : s1 };
            t[cnt++] = x;
            need[ m * nphase + p ]++;
         }
      }
   for(m=0;m<b->nmesh;m++)
      for(k=0;k<b->NmbTet[m];k+=b->tile_tets)
      {
         GmdBatchTile x = { nsweeps, m, k, k + b->tile_tets < b->NmbTet[m] ? k + b->tile_tets
                                                                         : b->NmbTet[m] };
         t[cnt++] = x;
         need[ m * nphase + nsweeps ]++;
      }

   b->td = gmd_alloc(gml->dev, (size_t)cnt * sizeof(GmdBatchTile));
   b->need = gmd_alloc(gml->dev, (size_t)b->nmesh * nphase * sizeof(int));
   b->done = gmd_alloc(gml->dev, (size_t)b->nmesh * nphase * sizeof(int));
   if(!b->td || !b->need || !b->done)
   {
      free(t); free(need);
      bat_free_tiles(gml, b);
      return 0;
   }
   b->hneed = malloc((size_t)b->nmesh * nphase * sizeof(int));
   if(!b->hneed)
   {
      free(t); free(need);
      bat_free_tiles(gml, b);
      return 0;
   }
   memcpy(b->hneed, need, (size_t)b->nmesh * nphase * sizeof(int));
   need[0] += b->hold;
   gmd_h2d_async(gml->dev, b->td, t, (size_t)cnt * sizeof(GmdBatchTile));
   gmd_h2d_async(gml->dev, b->need, need, (size_t)b->nmesh * nphase * sizeof(int));
   gmd_sync(gml->dev);
   free(t);
   free(need);
   b->ntile = cnt;
   b->nphase = nphase;
   b->tsweeps = nsweeps;
   return 1;
}

int GmlxBatchSetup(size_t GmlIdx, int fix)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   int m;

   if(!b)
      return 0;
   if(!gml_upload(gml, gml->TypIdx[ GmlVertices ]) || !gml_upload(gml, gml->RefIdx[ GmlVertices ])
   || !gml_upload(gml, gml->TypIdx[ GmlTetrahedra ]))
      return 0;
   if(!GmlxMeshSetup(GmlIdx, fix))
      return 0;
   for(m=0;m<b->nmesh;m++)
   {
      GmdBatchMesh x;
      x.t0 = b->TetOff[m];
      x.nt = b->NmbTet[m];
      x.f0 = b->FlgOff[m];
      x.s0 = b->VerOff[m] / 32;
      x.s1 = b->VerOff[m+1] / 32;
      x.thr = gmlx_det_threshold(b->h[m]);
      b->mh[m] = x;
   }
   gmd_h2d_async(gml->dev, b->md, b->mh, (size_t)b->nmesh * sizeof(GmdBatchMesh));
   if(!gmd_sync(gml->dev))
      return 0;
   b->maxgrid = gmd_batch_grid(gml->dev);
   if(!b->grid || b->grid > b->maxgrid)
      b->grid = b->maxgrid;
   bat_free_tiles(gml, b);
   b->fix = fix;
   b->ready = 1;
   return 1;
}

static int bat_ready(GmlSct *gml, BatSct **b, NatSct **n)
{
   *b = bat(gml);
   *n = (NatSct *)gml->ext;
   if(!*b || !(*b)->ready || !*n || !(*n)->ready || (*n)->nv != (*b)->nv)
   {
      puts("GmlxBatchSetup must be called after the meshes are set.");
      return 0;
   }
   return 1;
}

/* the queue run: counter resets, statistics init, the persistent launch and
   the copy back of an odd sweep count */
static int bat_queue_work(GmlSct *gml, BatSct *b, NatSct *n, int nsweeps, float omega)
{
   GmlDatSct *vd = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   GmlDatSct *td = &gml->dat[ gml->TypIdx[ GmlTetrahedra ] ];
   GmdBatchArgs a;

   memset(&a, 0, sizeof(a));
   a.ntile = b->ntile;
   a.nsweep = nsweeps;
   a.nmesh = b->nmesh;
   a.nphase = b->nphase;
   a.tiles = b->td;
   a.mesh = b->md;
   a.need = b->need;
   a.done = b->done;
   a.head = b->ctl;
   a.abort = b->ctl + 1;
   a.err = n->err;
   a.rowv = n->rowv;
   a.soff = n->soff;
   a.col = n->pcol;
   a.buf0 = vd->GpuMem;
   a.buf1 = n->crd2;
   a.tet = td->GpuMem;
   a.flags = b->flags;
   a.stats = b->stats;
   a.omega = omega;
   a.spin = b->spin > 0 ? b->spin : BAT_SPIN;
   return gmd_memset_async(gml->dev, b->ctl, 0, 2 * sizeof(int))
       && gmd_memset_async(gml->dev, b->done, 0, (size_t)b->nmesh * b->nphase * sizeof(int))
       && gmd_mesh_stats_init(gml->dev, b->stats, b->nmesh)
       && (b->warp ? gmd_batch_queue_warp(gml->dev, &a, b->grid)
                   : gmd_batch_queue(gml->dev, &a, b->grid))
       && (!(nsweeps & 1) || gmd_d2d_async(gml->dev, vd->GpuMem, n->crd2, (size_t)b->nv * 16));
}

static int bat_loop_work(GmlSct *gml, BatSct *b, NatSct *n, int nsweeps, float omega)
{
   GmlDatSct *vd = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   GmlDatSct *td = &gml->dat[ gml->TypIdx[ GmlTetrahedra ] ];
   void *fin = (nsweeps & 1) ? n->crd2 : vd->GpuMem;

   if(!gmd_mesh_stats_init(gml->dev, b->stats, b->nmesh))
      return 0;
   for(int m=0;m<b->nmesh;m++)
   {
      const GmdBatchMesh *x = &b->mh[m];
      void *in = vd->GpuMem, *out = n->crd2;
      for(int s=0;s<nsweeps;s++)
      {
         void *t;
         if(!gmd_mesh_laplace_slices(gml->dev, x->s0, x->s1, n->rowv, n->soff, n->pcol, in, out,
                                     omega))
            return 0;
         t = in; in = out; out = t;
      }
      if(!gmd_mesh_quality(gml->dev, x->nt, (const int *)td->GpuMem + 4 * (size_t)x->t0, fin,
                           x->thr, NULL, b->flags + x->f0, b->stats + m, n->err, 0))
         return 0;
   }
   return !(nsweeps & 1) || gmd_d2d_async(gml->dev, vd->GpuMem, n->crd2, (size_t)b->nv * 16);
}

/* the device error bits of the last run, cleared once read so that the
   instance runs on */
static int bat_errors(GmlSct *gml, NatSct *n)
{
   int err = 0;
   if(!gmd_d2h(gml->dev, &err, n->err, sizeof(int)))
      return -1;
   if(err && !gmd_memset_async(gml->dev, n->err, 0, sizeof(int)))
      return -1;
   if(err & 16)
      puts("GMlib: a batched tile waited too long for its dependencies; results are incomplete.");
   if(err & 4)
      puts("GMlib: a quality-kernel staging copy timed out; statistics are incomplete.");
   fflush(stdout);
   return err & (16 | 4);
}

int GmlxBatchRun(size_t GmlIdx, int nsweeps, float omega, int mode, GmlxQuality *res)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b;
   NatSct *n;

   if(!bat_ready(gml, &b, &n) || nsweeps < 0 || nsweeps > 1000)
      return 0;
   if(mode == GmlxBatchQueue)
   {
      if(!bat_tiles(gml, b, nsweeps))
         return 0;
      if(b->graph && (b->gsweeps != nsweeps || b->gomega != omega))
      {
         gmd_graph_free(b->graph);
         b->graph = NULL;
      }
      if(!b->graph)
      {
         int ok;
         if(!gmd_graph_begin(gml->dev))
            return 0;
         ok = bat_queue_work(gml, b, n, nsweeps, omega);
         if(!gmd_graph_end(gml->dev, &b->graph) || !ok)
         {
            gmd_graph_free(b->graph);
            b->graph = NULL;
            return 0;
         }
         b->gsweeps = nsweeps;
         b->gomega = omega;
      }
      if(!gmd_graph_launch(gml->dev, b->graph))
         return 0;
   }
   else if(mode == GmlxBatchLoop)
   {
      if(!bat_loop_work(gml, b, n, nsweeps, omega))
         return 0;
   }
   else
      return 0;

   if(res)
   {
      if(!gmd_d2h(gml->dev, b->hstats, b->stats, (size_t)b->nmesh * sizeof(GmlxQualStats))
      || bat_errors(gml, n))
         return 0;
      for(int m=0;m<b->nmesh;m++)
         gmlx_decode_stats(&b->hstats[m], &res[m]);
   }
   return 1;
}

int GmlxBatchSetWaitLimit(size_t GmlIdx, int spin, int hold)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = (BatSct *)gml->bat;

   if(!b || spin < 0 || hold < 0)
      return 0;
   b->spin = spin;
   b->hold = hold;
   /* the queue launch is captured with its arguments: capture it again */
   gmd_graph_free(b->graph);
   b->graph = NULL;
   if(b->td)
   {
      const int first = b->hneed[0] + hold;
      if(!gmd_h2d_async(gml->dev, b->need, &first, sizeof(int)) || !gmd_sync(gml->dev))
         return 0;
   }
   return 1;
}

int GmlxBatchFlags(size_t GmlIdx, int MshIdx, unsigned *flags, size_t nwords)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   size_t need;
   if(!b || MshIdx < 0 || MshIdx >= b->nmesh || !flags)
      return 0;
   need = (size_t)(b->FlgOff[MshIdx + 1] - b->FlgOff[MshIdx]);
   if(nwords < need)
      return 0;
   return gmd_d2h(gml->dev, flags, b->flags + b->FlgOff[MshIdx], need * sizeof(unsigned));
}

int GmlxBatchTune(size_t GmlIdx, int nsweeps, float omega)
{
   GETGMLPTR(gml, GmlIdx);
   /* (tiles per warp or per block, slices per sweep tile, tets per quality
      tile, grid as a fraction of the resident maximum: 2 full, 1 half) */
   static const int cand[][4] = {
      { 0, 8, 2048, 2 }, { 0, 32, 4096, 2 }, { 0, 128, 16384, 2 }, { 0, 32, 4096, 1 },
      { 1, 2, 512, 2 },  { 1, 4, 1024, 2 },  { 1, 16, 4096, 2 },   { 1, 4, 1024, 1 } };
   const int ncand = (int)(sizeof(cand) / sizeof(cand[0]));
   BatSct *b;
   NatSct *n;
   GmlDatSct *vd;
   void *save, *e0, *e1;
   double best = 1e30;
   int bs = 0, bt = 0, bg = 0, bw = 0, c;

   if(!bat_ready(gml, &b, &n) || nsweeps < 0)
      return 0;
   vd = &gml->dat[ gml->TypIdx[ GmlVertices ] ];
   save = gmd_alloc(gml->dev, (size_t)b->nv * 16);
   e0 = gmd_event_new();
   e1 = gmd_event_new();
   if(!save || !e0 || !e1)
   {
      gmd_free(gml->dev, save);
      gmd_event_free(e0);
      gmd_event_free(e1);
      return 0;
   }
   gmd_d2d_async(gml->dev, save, vd->GpuMem, (size_t)b->nv * 16);
   bs = b->tile_slices; bt = b->tile_tets; bg = b->grid; bw = b->warp;
   for(c=0;c<ncand;c++)
   {
      double t;
      b->warp = cand[c][0];
      b->tile_slices = cand[c][1];
      b->tile_tets = cand[c][2];
      b->grid = cand[c][3] == 2 ? b->maxgrid : (b->maxgrid + 1) / 2;
      bat_free_tiles(gml, b);
      if(!GmlxBatchRun(GmlIdx, nsweeps, omega, GmlxBatchQueue, NULL))
         continue;
      gmd_event_record(gml->dev, e0);
      GmlxBatchRun(GmlIdx, nsweeps, omega, GmlxBatchQueue, NULL);
      gmd_event_record(gml->dev, e1);
      t = gmd_event_elapsed_s(e0, e1);
      if(t < best)
      {
         best = t;
         bs = b->tile_slices; bt = b->tile_tets; bg = b->grid; bw = b->warp;
      }
   }
   b->tile_slices = bs;
   b->tile_tets = bt;
   b->grid = bg;
   b->warp = bw;
   bat_free_tiles(gml, b);
   gmd_d2d_async(gml->dev, vd->GpuMem, save, (size_t)b->nv * 16);
   gmd_sync(gml->dev);
   gmd_free(gml->dev, save);
   gmd_event_free(e0);
   gmd_event_free(e1);
   return 1;
}

int GmlxBatchSetTiles(size_t GmlIdx, int WarpTiles, int TileSlices, int TileTets, int grid)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   if(!b || TileSlices < 1 || TileTets < 32 || (TileTets & 31) || grid < 0)
      return 0;
   b->warp = WarpTiles ? 1 : 0;
   b->tile_slices = TileSlices;
   b->tile_tets = TileTets;
   if(grid > 0)
      b->grid = grid;
   bat_free_tiles(gml, b);
   return 1;
}

int GmlxBatchInfo(size_t GmlIdx, int *TileSlices, int *TileTets, int *grid, int *ntile,
                  int *WarpTiles)
{
   GETGMLPTR(gml, GmlIdx);
   BatSct *b = bat(gml);
   if(!b)
      return 0;
   if(TileSlices) *TileSlices = b->tile_slices;
   if(TileTets) *TileTets = b->tile_tets;
   if(grid) *grid = b->grid;
   if(ntile) *ntile = b->ntile;
   if(WarpTiles) *WarpTiles = b->warp;
   return 1;
}
