/*
 * gml_serve.c -- a request loop serving quality, smoothing and solve
 * requests on many meshes and systems from one GPU (no counterpart in the
 * reference, whose callers drive one mesh per instance themselves).
 *
 * Targets.  A mesh (vertices, refs, tets, edge length h) or a block system
 * (CSR matrix and right-hand side) is registered once; its host arrays stay
 * owned by the caller and must outlive the server.  A resident target lives
 * in its own GMlib instance on the device (own CUDA stream): mesh data plus
 * the native topology, or the FP64 matrix and its vectors.
 *
 * Continuous batching (GmlxServeBatching).  Requests arrive at their given
 * times (open loop).  The dispatcher admits a waiting request as soon as
 *   - one of NmbSlot worker slots is free,
 *   - its target is idle (requests on one target run one after the other),
 *   - its target is resident, or its estimated device bytes fit in the
 *     budget once idle resident targets are evicted, least recently used
 *     first;
 * requests behind a blocked one are still considered (no head-of-line
 * blocking).  Each slot is a host thread running the request on its target's
 * stream, so the work of up to NmbSlot requests overlaps on the device; a
 * slot takes the next admitted request the moment it finishes.
 *
 * Serial plain launches (GmlxServeSerial).  One request at a time in arrival
 * order, each on a fresh instance: create, upload, set up, run, stop.
 *
 * Requests leave their target as they found it (a smoothing request puts
 * the registered coordinates back afterwards), so every result is the same
 * whatever ran before or beside it.  Latency = finish - arrival.
 */
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"

#define SRV_SWEEPS   10
#define SRV_OMEGA    1.0f
#define SRV_TOL      1e-10
#define SRV_MAXIT    20000
#define SRV_MAXSLOT  64

typedef struct
{
   int            kind;                   /* 0 mesh, 1 system */
   int            nv, nt;
   const float    *crd;
   const int      *ref, *tet;
   double         h;
   int            nrow, nblk;
   const int      *lin, *col;
   const double   *val, *rhs;
   size_t         g;                      /* instance while resident, else 0 */
   int            vidx, mat, vb, vx;
   double         bytes;                  /* estimated device bytes */
   int            busy, reserved;
   double         last;
}SrvTarget;

typedef struct
{
   int            dev, slots;
   double         budget;
   SrvTarget      *tg;
   int            ntg, captg;
   /* run state */
   pthread_mutex_t mu;
   pthread_cond_t cv_work, cv_done, cv_reap;
   GmlxRequest    *req;
   int            nreq, *queue, qhead, qtail, inflight, completed, stop;
   size_t         *reap;                  /* instances of evicted targets, to stop */
   int            nreap, capreap;
   double         resident, peak, t0;
   int            loads, evictions;
}SrvSct;

static double now_s(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* device bytes of a resident target: datatypes and native topology of a
   mesh (48 B per tet, 120 B per vertex); FP64 and FP32 matrix copies and
   the solver vectors of a system (stored blocks padded to 1/0.9) */
static double estimate(const SrvTarget *t)
{
   if(t->kind == 0)
      return 48.0 * t->nt + 120.0 * t->nv + 4e6;
   return (4.0 + 72.0 + 36.0) * t->nblk / 0.9 + 300.0 * t->nrow + 4e6;
}

static int load(SrvSct *s, SrvTarget *t);
static void unload(SrvSct *s, SrvTarget *t);
static int run_request(SrvTarget *t, GmlxRequest *r);

/* One small mesh and one small system through every request kind, so that
   the device context and the library's lazily loaded kernels are ready
   before the first request: without it the requests of the first 0.2 s of a
   run waited about 0.3 s, which was the whole p99 of a 2000-request trace. */
static void warm_up(SrvSct *s)
{
   int nv = 0, nt = 0, nl = 0, nb = 0;
   SrvTarget m, y;
   GmlxRequest r;
   float *crd;
   int *tet, *ref, *lin = NULL, *col = NULL;
   double *val = NULL, *rhs = NULL;

   memset(&m, 0, sizeof(m));
   memset(&y, 0, sizeof(y));
   GmlxCubeSizes(4, &nv, &nt);
   crd = malloc((size_t)nv * 16);
   tet = malloc((size_t)nt * 16);
   ref = calloc((size_t)nv, sizeof(int));
   if(crd && tet && ref && GmlxCubeMesh(4, 1, 0.2, 1, crd, tet, ref))
   {
      m.kind = 0; m.nv = nv; m.nt = nt; m.crd = crd; m.tet = tet; m.ref = ref; m.h = 0.25;
      if(load(s, &m))
      {
         memset(&r, 0, sizeof(r));
         r.kind = GmlxReqQuality;
         run_request(&m, &r);
         r.kind = GmlxReqSmooth;
         run_request(&m, &r);
      }
      unload(s, &m);
   }
   if(GmlxCubeSpdSizes(4, 0, &nl, &nb))
   {
      lin = malloc((size_t)(nl + 1) * sizeof(int));
      col = malloc((size_t)nb * sizeof(int));
      val = malloc((size_t)nb * 9 * sizeof(double));
      rhs = malloc((size_t)nl * 3 * sizeof(double));
      if(lin && col && val && rhs && GmlxCubeSpdMatrix(4, 0, 1, lin, col, val, rhs))
      {
         y.kind = 1; y.nrow = nl; y.nblk = nb; y.lin = lin; y.col = col; y.val = val; y.rhs = rhs;
         if(load(s, &y))
         {
            memset(&r, 0, sizeof(r));
            r.kind = GmlxReqSolve;
            run_request(&y, &r);
         }
         unload(s, &y);
      }
   }
   free(crd); free(tet); free(ref);
   free(lin); free(col); free(val); free(rhs);
}

size_t GmlxServeNew(int dev, double BudgetBytes, int NmbSlot)
{
   SrvSct *s;
   if(NmbSlot < 1 || NmbSlot > SRV_MAXSLOT || !(BudgetBytes > 0.))
      return 0;
   s = calloc(1, sizeof(SrvSct));
   if(!s)
      return 0;
   s->dev = dev;
   s->slots = NmbSlot;
   s->budget = BudgetBytes;
   warm_up(s);
   return (size_t)s;
}

static int add_target(SrvSct *s, const SrvTarget *t)
{
   if(s->ntg == s->captg)
   {
      int cap = s->captg ? 2 * s->captg : 64;
      SrvTarget *n = realloc(s->tg, (size_t)cap * sizeof(SrvTarget));
      if(!n)
         return -1;
      s->tg = n;
      s->captg = cap;
   }
   s->tg[ s->ntg ] = *t;
   s->tg[ s->ntg ].bytes = estimate(t);
   return s->ntg++;
}

int GmlxServeAddMesh(size_t srv, int NmbVer, const float *crd, const int *ref, int NmbTet,
                     const int *tet, double h)
{
   SrvSct *s = (SrvSct *)srv;
   SrvTarget t;
   if(!s || NmbVer < 2 || NmbTet < 1 || !crd || !tet || !(h > 0.))
      return -1;
   memset(&t, 0, sizeof(t));
   t.kind = 0;
   t.nv = NmbVer; t.nt = NmbTet;
   t.crd = crd; t.ref = ref; t.tet = tet; t.h = h;
   return add_target(s, &t);
}

int GmlxServeAddSystem(size_t srv, int NmbLin, int NmbBlk, const int *lin, const int *col,
                       const double *val, const double *rhs)
{
   SrvSct *s = (SrvSct *)srv;
   SrvTarget t;
   if(!s || NmbLin < 1 || NmbBlk < 1 || !lin || !col || !val || !rhs)
      return -1;
   memset(&t, 0, sizeof(t));
   t.kind = 1;
   t.nrow = NmbLin; t.nblk = NmbBlk;
   t.lin = lin; t.col = col; t.val = val; t.rhs = rhs;
   return add_target(s, &t);
}

/* ------------------------------------------------------------------------- */

static void unload(SrvSct *s, SrvTarget *t)
{
   (void)s;
   if(t->g)
      GmlStop(t->g);
   t->g = 0;
}

static int load(SrvSct *s, SrvTarget *t)
{
   size_t g = GmlInit(s->dev);
   if(!g)
      return 0;
   GmlxSetTiming(g, 0);
   /* no informational messages from served instances; their whole-datatype
      sets go to the device only and their host mirrors stay pageable and
      untouched: nothing reads them, and page-locked mirrors cost the
      pinning at every load and, at every eviction, a cudaFreeHost that
      waits for all work on the device */
   ((GmlSct *)g)->Quiet = 1;
   ((GmlSct *)g)->MirOff = 1;
   t->g = g;
   if(t->kind == 0)
   {
      GmlSct *gml = (GmlSct *)g;
      int vi = GmlNewMeshData(g, GmlVertices, t->nv), ti = GmlNewMeshData(g, GmlTetrahedra, t->nt);
      if(!vi || !ti)
         goto fail;
      t->vidx = vi;
      if(!GmlxSetData(g, vi, t->crd, (size_t)t->nv * 16)
      || !GmlxSetData(g, ti, t->tet, (size_t)t->nt * 16))
         goto fail;
      if(t->ref)
      {
         int ri = gml->RefIdx[ GmlVertices ];
         if(!GmlxSetData(g, ri, t->ref, (size_t)t->nv * 4))
            goto fail;
      }
      if(!GmlxMeshSetup(g, 1))
         goto fail;
   }
   else
   {
      t->mat = GmlNewMatrix(g, t->nrow, t->nblk, 3, (void *)t->val, (int *)t->col, (int *)t->lin,
                            GmlDbl);
      t->vb = GmlNewVector(g, t->nrow, 3, (void *)t->rhs, GmlDbl);
      t->vx = GmlNewVector(g, t->nrow, 3, NULL, GmlDbl);
      if(t->mat <= 0 || t->vb <= 0 || t->vx <= 0)
         goto fail;
   }
   return 1;
fail:
   unload(s, t);
   return 0;
}

static int run_request(SrvTarget *t, GmlxRequest *r)
{
   if(r->kind == GmlxReqQuality)
      return t->kind == 0 && GmlxQualityStats(t->g, t->h, 0, &r->qal) == 1;
   if(r->kind == GmlxReqSmooth)
   {
      GmlxQuality res[SRV_SWEEPS];
      if(t->kind != 0 || GmlxSmoothQualityLoop(t->g, SRV_SWEEPS, SRV_OMEGA, t->h, res) != 1)
         return 0;
      r->qal = res[ SRV_SWEEPS - 1 ];
      /* put the registered coordinates back */
      return GmlxSetData(t->g, t->vidx, t->crd, (size_t)t->nv * 16) == 1
          && GmlxSynchronize(t->g) == 1;
   }
   if(r->kind == GmlxReqSolve)
   {
      GmlxSolveInfo info;
      int rc;
      if(t->kind != 1)
         return 0;
      rc = GmlxSolveCG(t->g, t->mat, t->vb, t->vx, GmlxCgMixed, SRV_TOL, SRV_MAXIT, &info);
      r->NmbIte = info.NmbIte;
      r->RelRes = info.RelRes;
      return rc == 1;
   }
   return 0;
}

/* make room for `need` bytes by evicting idle resident targets, least
   recently used first; called with the lock held.  An evicted instance is
   handed to the reaper thread: stopping it frees pinned host memory, which
   waits for all work on the device, and must not hold up the dispatcher or
   the slots (they need the lock to take and finish requests). */
static int reserve(SrvSct *s, double need)
{
   while(s->resident + need > s->budget)
   {
      SrvTarget *v = NULL;
      for(int i=0;i<s->ntg;i++)
      {
         SrvTarget *t = &s->tg[i];
         if((t->g || t->reserved) && !t->busy && (!v || t->last < v->last))
            v = t;
      }
      if(!v)
         return 0;
      if(v->g && s->reap && s->nreap < s->capreap)
      {
         s->reap[ s->nreap++ ] = v->g;
         v->g = 0;
         pthread_cond_signal(&s->cv_reap);
      }
      else
         unload(s, v);
      v->reserved = 0;
      s->resident -= v->bytes;
      s->evictions++;
   }
   s->resident += need;
   if(s->resident > s->peak)
      s->peak = s->resident;
   return 1;
}

static void *worker(void *arg)
{
   SrvSct *s = (SrvSct *)arg;
   pthread_mutex_lock(&s->mu);
   for(;;)
   {
      GmlxRequest *r;
      SrvTarget *t;
      int ok = 1, k;
      while(s->qhead == s->qtail && !s->stop)
         pthread_cond_wait(&s->cv_work, &s->mu);
      if(s->qhead == s->qtail)
         break;
      k = s->queue[ s->qhead++ ];
      r = &s->req[k];
      t = &s->tg[ r->target ];
      pthread_mutex_unlock(&s->mu);

      r->start = now_s() - s->t0;
      if(!t->g)
      {
         ok = load(s, t);
         __atomic_add_fetch(&s->loads, 1, __ATOMIC_RELAXED);
      }
      ok = ok && run_request(t, r);
      r->finish = now_s() - s->t0;
      r->status = ok ? 1 : 0;

      pthread_mutex_lock(&s->mu);
      if(!t->g && t->reserved)
      {
         /* the load failed: release the reservation */
         t->reserved = 0;
         s->resident -= t->bytes;
      }
      t->busy = 0;
      t->last = now_s();
      s->inflight--;
      s->completed++;
      pthread_cond_signal(&s->cv_done);
   }
   pthread_mutex_unlock(&s->mu);
   return NULL;
}

/* stops the instances of evicted targets, outside the lock */
static void *reaper(void *arg)
{
   SrvSct *s = (SrvSct *)arg;
   pthread_mutex_lock(&s->mu);
   for(;;)
   {
      while(!s->nreap && !s->stop)
         pthread_cond_wait(&s->cv_reap, &s->mu);
      if(!s->nreap)
         break;
      {
         size_t g = s->reap[ --s->nreap ];
         pthread_mutex_unlock(&s->mu);
         GmlStop(g);
         pthread_mutex_lock(&s->mu);
      }
   }
   pthread_mutex_unlock(&s->mu);
   return NULL;
}

static int cmp_double(const void *a, const void *b)
{
   double x = *(const double *)a, y = *(const double *)b;
   return x < y ? -1 : x > y;
}

static void summarize(SrvSct *s, GmlxRequest *req, int n, double wall, GmlxServeStats *st)
{
   double *lat = malloc((size_t)(n > 0 ? n : 1) * sizeof(double)), sum = 0.;
   int ok = 0;
   memset(st, 0, sizeof(*st));
   for(int i=0;i<n;i++)
      if(req[i].status == 1)
      {
         lat[ok++] = req[i].finish - req[i].arrival;
         sum += req[i].finish - req[i].arrival;
      }
   if(lat && ok)
   {
      qsort(lat, (size_t)ok, sizeof(double), cmp_double);
      st->p50 = lat[ (int)(0.50 * (ok - 1) + 0.5) ];
      st->p99 = lat[ (int)(0.99 * (ok - 1) + 0.5) ];
      st->max = lat[ ok - 1 ];
      st->mean = sum / ok;
   }
   free(lat);
   st->completed = ok;
   st->failed = n - ok;
   st->seconds = wall;
   st->throughput = wall > 0. ? ok / wall : 0.;
   st->loads = s->loads;
   st->evictions = s->evictions;
   st->peak_bytes = s->peak;
}

static int run_serial(SrvSct *s, GmlxRequest *req, int n)
{
   for(int i=0;i<n;i++)
   {
      GmlxRequest *r = &req[i];
      SrvTarget *t;
      double wait;
      if(r->target < 0 || r->target >= s->ntg)
      {
         r->status = 0;
         continue;
      }
      /* a private copy: targets kept resident by an earlier run stay as they are */
      t = &s->tg[ r->target ];
      {
         SrvTarget tmp = *t;
         tmp.g = 0;
         wait = r->arrival - (now_s() - s->t0);
         if(wait > 0.)
         {
            struct timespec ts = { (time_t)wait, (long)((wait - floor(wait)) * 1e9) };
            nanosleep(&ts, NULL);
         }
         r->start = now_s() - s->t0;
         r->status = load(s, &tmp) && run_request(&tmp, r);
         s->loads++;
         unload(s, &tmp);
         r->finish = now_s() - s->t0;
      }
   }
   return 1;
}

static int run_batching(SrvSct *s, GmlxRequest *req, int n)
{
   pthread_t th[SRV_MAXSLOT];
   int *pend = malloc((size_t)n * sizeof(int)), npend = 0, next = 0, i, nth = 0;

   pthread_t rp;
   int have_rp;

   s->queue = malloc((size_t)n * sizeof(int));
   s->capreap = s->ntg;
   s->reap = malloc((size_t)(s->capreap ? s->capreap : 1) * sizeof(size_t));
   s->nreap = 0;
   if(!pend || !s->queue || !s->reap)
   {
      free(pend);
      free(s->queue);
      free(s->reap);
      s->queue = NULL;
      s->reap = NULL;
      return 0;
   }
   s->qhead = s->qtail = s->inflight = s->completed = s->stop = 0;
   pthread_mutex_init(&s->mu, NULL);
   pthread_cond_init(&s->cv_work, NULL);
   pthread_cond_init(&s->cv_done, NULL);
   pthread_cond_init(&s->cv_reap, NULL);
   for(i=0;i<s->slots;i++)
      if(pthread_create(&th[nth], NULL, worker, s) == 0)
         nth++;
   have_rp = pthread_create(&rp, NULL, reaper, s) == 0;
   if(!have_rp)
      s->capreap = 0;                     /* evictions stop instances in place */

   pthread_mutex_lock(&s->mu);
   while(s->completed < n)
   {
      double tnow = now_s() - s->t0;
      int j = 0;
      while(next < n && req[next].arrival <= tnow)
         pend[npend++] = next++;
      for(i=0;i<npend;i++)
      {
         int k = pend[i];
         GmlxRequest *r = &req[k];
         SrvTarget *t;
         int admit = 0;
         if(r->target < 0 || r->target >= s->ntg || s->tg[r->target].bytes > s->budget)
         {
            r->status = 0;
            r->start = r->finish = tnow;
            s->completed++;
            continue;
         }
         t = &s->tg[ r->target ];
         if(s->inflight < s->slots && !t->busy)
         {
            if(t->g || t->reserved)
               admit = 1;
            else if(reserve(s, t->bytes))
            {
               t->reserved = 1;
               admit = 1;
            }
         }
         if(admit)
         {
            t->busy = 1;
            s->inflight++;
            s->queue[ s->qtail++ ] = k;
            pthread_cond_signal(&s->cv_work);
         }
         else
            pend[j++] = k;
      }
      npend = j;
      if(s->completed >= n)
         break;
      {
         struct timespec ts;
         double until = next < n ? req[next].arrival : tnow + 0.05;
         if(npend)
            until = fmin(until, tnow + 0.001);
         until += s->t0;
         ts.tv_sec = (time_t)until;
         ts.tv_nsec = (long)((until - floor(until)) * 1e9);
         pthread_cond_timedwait(&s->cv_done, &s->mu, &ts);
      }
   }
   s->stop = 1;
   pthread_cond_broadcast(&s->cv_work);
   pthread_cond_broadcast(&s->cv_reap);
   pthread_mutex_unlock(&s->mu);
   for(i=0;i<nth;i++)
      pthread_join(th[i], NULL);
   if(have_rp)
      pthread_join(rp, NULL);             /* it stops what is left to reap first */
   pthread_cond_destroy(&s->cv_work);
   pthread_cond_destroy(&s->cv_done);
   pthread_cond_destroy(&s->cv_reap);
   pthread_mutex_destroy(&s->mu);
   free(pend);
   free(s->queue);
   free(s->reap);
   s->queue = NULL;
   s->reap = NULL;
   s->nreap = s->capreap = 0;
   return nth > 0;
}

int GmlxServeRun(size_t srv, GmlxRequest *req, int NmbReq, int mode, GmlxServeStats *st)
{
   SrvSct *s = (SrvSct *)srv;
   struct timespec ts;
   int ok;
   if(!s || !req || NmbReq < 1)
      return 0;
   for(int i=1;i<NmbReq;i++)
      if(req[i].arrival < req[i-1].arrival)
         return 0;
   for(int i=0;i<NmbReq;i++)
   {
      req[i].status = -1;
      req[i].start = req[i].finish = 0.;
   }
   /* the CUDA context exists before the clock starts */
   clock_gettime(CLOCK_MONOTONIC, &ts);
   s->loads = s->evictions = 0;
   s->peak = mode == GmlxServeSerial ? 0. : s->resident;
   s->req = req;
   s->nreq = NmbReq;
   s->t0 = now_s();
   if(mode == GmlxServeSerial)
      ok = run_serial(s, req, NmbReq);
   else if(mode == GmlxServeBatching)
      ok = run_batching(s, req, NmbReq);
   else
      return 0;
   if(st)
      summarize(s, req, NmbReq, now_s() - s->t0, st);
   return ok;
}

double GmlxServeTargetBytes(size_t srv, int target)
{
   SrvSct *s = (SrvSct *)srv;
   if(!s || target < 0 || target >= s->ntg)
      return -1.;
   return s->tg[target].bytes;
}

int GmlxServeResident(size_t srv, double *bytes)
{
   SrvSct *s = (SrvSct *)srv;
   int n = 0;
   if(!s)
      return -1;
   for(int i=0;i<s->ntg;i++)
      n += s->tg[i].g != 0;
   if(bytes)
      *bytes = s->resident;
   return n;
}

void GmlxServeFree(size_t srv)
{
   SrvSct *s = (SrvSct *)srv;
   if(!s)
      return;
   for(int i=0;i<s->ntg;i++)
      unload(s, &s->tg[i]);
   free(s->tg);
   free(s);
}
