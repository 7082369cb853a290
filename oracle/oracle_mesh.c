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

/* ------------------------------------------------------------------------- */
/* P2 tetrahedron quality (reference examples/P2Quality/quality.cl:1-255,      */
/* computed in FP64).  Nodes: the 4 vertices and the 6 mid-edge nodes of the   */
/* local edges (0,1) (1,2) (2,0) (3,0) (3,1) (3,2) (quality.cl:7-17 and the    */
/* tetrahedron row of the edge table, sources/gmlib3.c:337).                   */
/*   L    = max over the edges of |a - m| + |m - b|              (:6-17)      */
/*   S    = sum of |cross| (twice the area) of the 16 triangles  (:19-35)      */
/*          splitting each face at its mid-edge nodes                          */
/*   V1   = 6 x the volume of the straight tetrahedron           (:38)         */
/*   V2   = 6 x the volume enclosed by those 16 triangles        (:40-47)      */
/*   Jmin, Jmax = extreme Bernstein coefficients of the Jacobian determinant   */
/*          of the quadratic map, on the control net c_e = 2 m_e - (a + b)/2   */
/*          (:49-245)                                                          */
/*   q    = (Jmin / Jmax) (2 sqrt(6) V2 / (L S)) (min(V1,V2) / max(V1,V2))     */
/*          (:247-250)                                                         */
/* ------------------------------------------------------------------------- */

static const int P2_EDGE[6][2] = { {0,1}, {1,2}, {2,0}, {3,0}, {3,1}, {3,2} };

static void p2_sub(const double *a, const double *b, double *r)
{ r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2]; }

static double p2_det(const double *a, const double *b, const double *c)
{
   return a[0] * (b[1] * c[2] - b[2] * c[1])
        - a[1] * (b[0] * c[2] - b[2] * c[0])
        + a[2] * (b[0] * c[1] - b[1] * c[0]);
}

static double p2_cross_len(const double *a, const double *b, const double *c)
{
   double u[3], v[3], x, y, z;
   p2_sub(b, a, u);
   p2_sub(c, a, v);
   x = u[1] * v[2] - u[2] * v[1];
   y = u[2] * v[0] - u[0] * v[2];
   z = u[0] * v[1] - u[1] * v[0];
   return sqrt(x * x + y * y + z * z);
}

static double p2_dist(const double *a, const double *b)
{
   double d[3];
   p2_sub(a, b, d);
   return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

/* index of the edge joining local vertices i != j */
static int p2_edge_of(int i, int j)
{
   for(int e=0;e<6;e++)
      if((P2_EDGE[e][0] == i && P2_EDGE[e][1] == j) || (P2_EDGE[e][0] == j && P2_EDGE[e][1] == i))
         return e;
   return -1;
}

double orc_p2_quality1(const double ver[4][3], const double mid[6][3])
{
   /* faces oriented outward for a positive tetrahedron: opposite vertex 0..3 */
   static const int FAC[4][3] = { {1,2,3}, {0,3,2}, {0,1,3}, {0,2,1} };
   double L = 0., S = 0., V1, V2 = 0., jmin = 0., jmax = 0., ctl[4][4][3], d[3][4][3];
   int f, k, a, b, c, e, first = 1;

   for(e=0;e<6;e++)
   {
      double l = p2_dist(ver[ P2_EDGE[e][0] ], mid[e]) + p2_dist(mid[e], ver[ P2_EDGE[e][1] ]);
      L = e ? fmax(L, l) : l;
   }

   /* the 16 boundary triangles: per face (a,b,c) with mids mab, mbc, mca:
      (a,mab,mca) (mab,b,mbc) (mca,mbc,c) (mab,mbc,mca), same orientation */
   for(f=0;f<4;f++)
   {
      const double *A = ver[ FAC[f][0] ], *B = ver[ FAC[f][1] ], *C = ver[ FAC[f][2] ];
      const double *mab = mid[ p2_edge_of(FAC[f][0], FAC[f][1]) ];
      const double *mbc = mid[ p2_edge_of(FAC[f][1], FAC[f][2]) ];
      const double *mca = mid[ p2_edge_of(FAC[f][2], FAC[f][0]) ];
      const double *tri[4][3] = { {A, mab, mca}, {mab, B, mbc}, {mca, mbc, C}, {mab, mbc, mca} };
      for(k=0;k<4;k++)
      {
         double p[3], q[3], r[3];
         S += p2_cross_len(tri[k][0], tri[k][1], tri[k][2]);
         /* enclosed volume x 6 = sum of det(p - v0, q - v0, r - v0) */
         p2_sub(tri[k][0], ver[0], p);
         p2_sub(tri[k][1], ver[0], q);
         p2_sub(tri[k][2], ver[0], r);
         V2 += p2_det(p, q, r);
      }
   }
   {
      double u[3], v[3], w[3];
      p2_sub(ver[1], ver[0], u);
      p2_sub(ver[2], ver[0], v);
      p2_sub(ver[3], ver[0], w);
      V1 = p2_det(u, v, w);
   }

   /* control net P[i][j] (i <= j): vertices on the diagonal, edge control
      points off it */
   for(a=0;a<4;a++)
      for(k=0;k<3;k++)
         ctl[a][a][k] = ver[a][k];
   for(e=0;e<6;e++)
   {
      int i = P2_EDGE[e][0], j = P2_EDGE[e][1];
      for(k=0;k<3;k++)
      {
         double cp = 2. * mid[e][k] - .5 * (ver[i][k] + ver[j][k]);
         ctl[i][j][k] = cp;
         ctl[j][i][k] = cp;
      }
   }
   /* derivative control vectors d[t][g] = P[g][t+1] - P[g][0], g = 0..3:
      the Jacobian's column t is 2 sum_g d[t][g] lambda_g */
   for(k=0;k<3;k++)
      for(int g=0;g<4;g++)
         for(int x=0;x<3;x++)
            d[k][g][x] = ctl[g][k+1][x] - ctl[g][0][x];

   /* det J = 8 sum_{a,b,c} det(d0[a], d1[b], d2[c]) l_a l_b l_c; the cubic
      Bernstein coefficient of the multi-index {a,b,c} is 8 (gamma! / 3!) x the
      sum over its orderings */
   {
      double bin[4][4][4];
      memset(bin, 0, sizeof(bin));
      for(a=0;a<4;a++)
         for(b=0;b<4;b++)
            for(c=0;c<4;c++)
            {
               int s[3] = {a, b, c}, t;
               if(s[0] > s[1]) { t = s[0]; s[0] = s[1]; s[1] = t; }
               if(s[1] > s[2]) { t = s[1]; s[1] = s[2]; s[2] = t; }
               if(s[0] > s[1]) { t = s[0]; s[0] = s[1]; s[1] = t; }
               bin[s[0]][s[1]][s[2]] += p2_det(d[0][a], d[1][b], d[2][c]);
            }
      for(a=0;a<4;a++)
         for(b=a;b<4;b++)
            for(c=b;c<4;c++)
            {
               double w = (a == b && b == c) ? 8. : (a == b || b == c) ? 8. / 3. : 4. / 3.;
               double nj = w * bin[a][b][c];
               if(first) { jmin = jmax = nj; first = 0; }
               else { jmin = fmin(jmin, nj); jmax = fmax(jmax, nj); }
            }
   }
   return (jmin / jmax) * ((2. * sqrt(6.) * V2) / (L * S)) * (fmin(V1, V2) / fmax(V1, V2));
}

/* P2 quality of nt tetrahedra: tet (4 vertex indices), tedg (6 edge indices,
   local edge order above), crd / mid float4 lines */
void orc_p2_quality(int nt, const int *tet, const int *tedg, const float *crd,
                    const float *mid, double *q)
{
   #pragma omp parallel for schedule(static)
   for(int i=0;i<nt;i++)
   {
      double ver[4][3], md[6][3];
      for(int k=0;k<4;k++)
         for(int x=0;x<3;x++)
            ver[k][x] = crd[ 4 * (size_t)tet[ 4 * (size_t)i + k ] + x ];
      for(int e=0;e<6;e++)
         for(int x=0;x<3;x++)
            md[e][x] = mid[ 4 * (size_t)tedg[ 6 * (size_t)i + e ] + x ];
      q[i] = orc_p2_quality1(ver, md);
   }
}
