/*
 * oracle_mesh.c -- CPU restatement of the native mesh kernels (Laplacian
 * smoothing over the ball of points, mean-ratio quality statistics,
 * inverted-element flags, boundary detection).  TEST INFRASTRUCTURE ONLY.
 *
 * Definitions (the workload of the smoothing configuration; the reference
 * has no such kernels, its NodeSmoothing example relaxes toward per-tet
 * optimal points instead, examples/NodeSmoothing/gather.cl):
 *   ball of points  the distinct vertices sharing a tet with v, ascending
 *   sweep           x_v' = x_v + w (mean over the ball - x_v), Jacobi order,
 *                   fixed vertices unchanged
 *   quality         q = 12 (3|V|)^(2/3) / sum of the 6 squared edge lengths,
 *                   V = det/6, negated when det <= 0 (FP64 determinant of the
 *                   FP32 coordinates); histogram bin clamp(floor(64 q), 0, 63)
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

static int cmp_int(const void *a, const void *b)
{
   int x = *(const int *)a, y = *(const int *)b;
   return (x > y) - (x < y);
}

/* ball of points as CSR (ptr has nv+1 entries); fixed vertices (fixed[v] != 0)
   get an empty ball.  Returns the number of entries, -1 on overflow. */
long long orc_point_ball(int nv, int nt, const int *tet, const int *fixed,
                         long long *ptr, int *col, long long cap)
{
   int *cnt = calloc(nv + 1, sizeof(int)), *vt, *fill;
   long long *vp = malloc((size_t)(nv + 1) * sizeof(long long)), tot = 0;
   int i, j, v;

   for(i=0;i<4*nt;i++)
      cnt[ tet[i] ]++;
   vp[0] = 0;
   for(v=0;v<nv;v++)
      vp[v+1] = vp[v] + cnt[v];
   vt = malloc((size_t)(vp[nv] > 0 ? vp[nv] : 1) * sizeof(int));
   fill = calloc(nv, sizeof(int));
   for(i=0;i<nt;i++)
      for(j=0;j<4;j++)
      {
         v = tet[4*i+j];
         vt[ vp[v] + fill[v]++ ] = i;
      }

   {
      int buf[4096];
      for(v=0;v<nv;v++)
      {
         int n = 0, k, u;
         if(ptr) ptr[v] = tot;
         if(fixed && fixed[v])
            continue;
         for(k=vp[v];k<vp[v+1];k++)
            for(j=0;j<4;j++)
            {
               u = tet[ 4 * vt[k] + j ];
               if(u != v && n < 4096)
                  buf[n++] = u;
            }
         qsort(buf, n, sizeof(int), cmp_int);
         for(k=0;k<n;k++)
            if(k == 0 || buf[k] != buf[k-1])
            {
               if(col && tot < cap)
                  col[tot] = buf[k];
               tot++;
            }
      }
      if(ptr) ptr[nv] = tot;
   }

   free(cnt); free(vp); free(vt); free(fill);
   return tot;
}

/* vertices of faces owned by a single tetrahedron */
typedef struct { int a, b, c; } Tri3;

static int cmp_tri(const void *p, const void *q)
{
   const Tri3 *x = p, *y = q;
   if(x->a != y->a) return (x->a > y->a) - (x->a < y->a);
   if(x->b != y->b) return (x->b > y->b) - (x->b < y->b);
   return (x->c > y->c) - (x->c < y->c);
}

void orc_boundary_vertices(int nv, int nt, const int *tet, int *fixed)
{
   Tri3 *f = malloc((size_t)nt * 4 * sizeof(Tri3));
   long long i, n = 4LL * nt;
   memset(fixed, 0, (size_t)nv * sizeof(int));
   for(i=0;i<nt;i++)
      for(int j=0;j<4;j++)
      {
         int v[3] = { tet[4*i+((j+1)&3)], tet[4*i+((j+2)&3)], tet[4*i+((j+3)&3)] }, t;
         if(v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
         if(v[1] > v[2]) { t = v[1]; v[1] = v[2]; v[2] = t; }
         if(v[0] > v[1]) { t = v[0]; v[0] = v[1]; v[1] = t; }
         f[4*i+j].a = v[0]; f[4*i+j].b = v[1]; f[4*i+j].c = v[2];
      }
   qsort(f, n, sizeof(Tri3), cmp_tri);
   for(i=0;i<n;)
   {
      long long k = i + 1;
      while(k < n && !cmp_tri(&f[i], &f[k])) k++;
      if(k - i == 1)
         fixed[ f[i].a ] = fixed[ f[i].b ] = fixed[ f[i].c ] = 1;
      i = k;
   }
   free(f);
}

/* Jacobi sweeps in FP64; crd holds 4 doubles per vertex, updated in place */
void orc_laplace(int nv, double *crd, const long long *ptr, const int *col, double w, int nsweeps)
{
   double *nx = malloc((size_t)nv * 4 * sizeof(double));
   for(int s=0;s<nsweeps;s++)
   {
      #pragma omp parallel for schedule(static)
      for(int v=0;v<nv;v++)
      {
         long long d = ptr[v+1] - ptr[v];
         double sx = 0, sy = 0, sz = 0;
         if(!d)
         {
            memcpy(&nx[4*(size_t)v], &crd[4*(size_t)v], 4 * sizeof(double));
            continue;
         }
         for(long long k=ptr[v];k<ptr[v+1];k++)
         {
            const double *p = &crd[ 4 * (size_t)col[k] ];
            sx += p[0]; sy += p[1]; sz += p[2];
         }
         nx[4*(size_t)v]   = crd[4*(size_t)v]   + w * (sx / d - crd[4*(size_t)v]);
         nx[4*(size_t)v+1] = crd[4*(size_t)v+1] + w * (sy / d - crd[4*(size_t)v+1]);
         nx[4*(size_t)v+2] = crd[4*(size_t)v+2] + w * (sz / d - crd[4*(size_t)v+2]);
         nx[4*(size_t)v+3] = 0.;
      }
      memcpy(crd, nx, (size_t)nv * 4 * sizeof(double));
   }
   free(nx);
}

/* mean-ratio statistics on FP32 coordinates; flags: bit t%32 of word t/32 */
void orc_quality_stats(int nt, const float *crd, const int *tet, double *q, unsigned *hist,
                       unsigned *flags, unsigned *ninv)
{
   unsigned inv = 0;
   if(hist) memset(hist, 0, 64 * sizeof(unsigned));
   if(flags) memset(flags, 0, (size_t)((nt + 31) / 32) * sizeof(unsigned));
   for(int t=0;t<nt;t++)
   {
      double x = orc_mean_ratio1(crd, &tet[4*t]);
      double det = orc_det1(crd, &tet[4*t]);
      int bin;
      /* the sign comes from the FP64 determinant */
      if(det <= 0) { x = -fabs(x); inv++; if(flags) flags[t >> 5] |= 1u << (t & 31); }
      else x = fabs(x);
      q[t] = x;
      bin = (int)floor(x * 64.0);
      bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
      if(hist) hist[bin]++;
   }
   if(ninv) *ninv = inv;
}
