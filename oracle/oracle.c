/*
 * oracle.c -- CPU restatement of the GMlib mesh-kernel path.  TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU baseline leg of the
 * benchmark call it as the checker; the library never does.
 *
 * Each function follows a reference file:line.  Integer outputs (ball and
 * degree tables, edge lists, argmin, flags, histograms) reproduce the
 * reference algorithm itself: the ball builder below keeps the reference's
 * chained hash table with head insertion (sources/gmlib3.c:1645-1721) rather
 * than the counting scheme of the library, so the two are independent.
 * Floating-point outputs are evaluated in FP64 on the FP32 inputs.
 *
 * Parity pinning: the reference ships no tests or golden values; its kernel
 * bodies (toolkit.cl, compute_quality.cl, scatter.cl, gather.cl) are compiled
 * as C++ by oracle/refcl.py where the reference sources are present and
 * compared with this file in the tests; the fixtures of tests/golden were
 * produced that way.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

/* ------------------------------------------------------------------------- */
/* chained hash of the reference (sources/gmlib3.c:297-358, 1627-1721)        */
/* ------------------------------------------------------------------------- */

typedef struct { int EleIdx, ItmIdx, NxtDat, nod[4]; } Buc;
typedef struct { int DatLen, TabSiz, NmbDat, NxtDat, *HshTab; Buc *DatTab; } Hsh;

static int hsh_init(Hsh *h, int DatLen, int TabSiz)
{
   h->DatLen = DatLen;
   h->TabSiz = TabSiz > 0 ? TabSiz : 1;
   h->NmbDat = h->TabSiz;
   h->NxtDat = 1;
   h->HshTab = calloc(h->TabSiz, sizeof(int));
   h->DatTab = malloc((size_t)(h->NmbDat + 1) * sizeof(Buc));
   return h->HshTab && h->DatTab;
}

static void hsh_free(Hsh *h) { free(h->HshTab); free(h->DatTab); }

/* CalHshKey (:1627-1638), in 64-bit to avoid the reference's int overflow */
static int hsh_key(const Hsh *h, const int *t)
{
   static const long long wei[4] = { 3, 5, 7, 11 };
   long long k = 0;
   if(h->DatLen == 1)
      return t[0];
   for(int i=0;i<h->DatLen;i++)
      k += wei[i] * t[i];
   return (int)(k % h->TabSiz);
}

/* AddHsh (:1645-1674): insertion at the head of the chain */
static void hsh_add(Hsh *h, int key, int EleIdx, int ItmIdx, const int *t)
{
   Buc *b;
   if(h->NxtDat >= h->NmbDat)
   {
      h->NmbDat *= 2;
      h->DatTab = realloc(h->DatTab, (size_t)(h->NmbDat + 1) * sizeof(Buc));
   }
   b = &h->DatTab[ h->NxtDat ];
   b->EleIdx = EleIdx;
   b->ItmIdx = ItmIdx;
   b->NxtDat = h->HshTab[key];
   for(int i=0;i<h->DatLen;i++)
      b->nod[i] = t[i];
   h->HshTab[key] = h->NxtDat++;
}

/* GetHsh (:1681-1721): walk the chain, collect matching entries */
static int hsh_get(const Hsh *h, int key, const int *t, int *UsrTab, int cap)
{
   int deg = 0, p = h->HshTab[key];
   while(p)
   {
      const Buc *b = &h->DatTab[p];
      int ok = 1;
      for(int i=0;i<h->DatLen;i++)
         if(b->nod[i] != t[i]) { ok = 0; break; }
      if(ok)
      {
         if(UsrTab && deg < cap)
            UsrTab[deg] = (b->EleIdx << 4) | b->ItmIdx;
         deg++;
      }
      p = b->NxtDat;
   }
   return deg;
}

/* ------------------------------------------------------------------------- */
/* vertex -> tetrahedron ball (NewBallData uplink, :743-1168)                 */
/* ------------------------------------------------------------------------- */

int orc_ver_tet_ball(int nv, int nt, const int *tet, int BalSiz, int MaxSiz,
                     int *deg, int *MaxPosOut, int *HghSizOut, int *base, int *high)
{
   Hsh h;
   int i, j, MaxDeg = 0, MaxPos = -1, HghSiz = 0;

   if(!hsh_init(&h, 1, nv))
      return 0;

   for(i=0;i<nt;i++)
      for(j=0;j<4;j++)
         hsh_add(&h, tet[4*i+j], i, j, &tet[4*i+j]);

   for(i=0;i<nv;i++)
   {
      deg[i] = hsh_get(&h, i, &i, NULL, 0);
      if(deg[i] > MaxDeg) MaxDeg = deg[i];
      if(MaxPos < 0 && deg[i] > BalSiz) MaxPos = i;
   }

   if(BalSiz == MaxSiz || MaxDeg <= BalSiz)
   {
      MaxPos = nv;
      HghSiz = 0;
   }
   else
   {
      int p2 = 1;
      while(p2 < MaxDeg) p2 <<= 1;
      if(MaxDeg > MaxSiz) { hsh_free(&h); return 0; }
      HghSiz = p2 < MaxSiz ? p2 : MaxSiz;
   }

   *MaxPosOut = MaxPos;
   *HghSizOut = HghSiz;

   if(base || high)
   {
      int *tmp = malloc((size_t)(MaxDeg > 0 ? MaxDeg : 1) * sizeof(int));
      for(i=0;i<nv;i++)
      {
         int d = hsh_get(&h, i, &i, tmp, MaxDeg);
         if(i < MaxPos || !HghSiz)
         {
            if(base)
               for(j=0;j<d && j<BalSiz;j++)
                  base[ (size_t)i * BalSiz + j ] = tmp[j];
         }
         else
         {
            /* line MaxPos: its first BalSiz entries in the base row and its
               whole ball in high row 0 (the reference leaves that row empty) */
            if(i == MaxPos && base)
               for(j=0;j<d && j<BalSiz;j++)
                  base[ (size_t)i * BalSiz + j ] = tmp[j];
            if(high)
               for(j=0;j<d && j<HghSiz;j++)
                  high[ (size_t)(i - MaxPos) * HghSiz + j ] = tmp[j];
         }
      }
      free(tmp);
   }

   hsh_free(&h);
   return 1;
}

/* ------------------------------------------------------------------------- */
/* unique edges (GmlExtractEdges, :3719-3873), tetrahedra only                */
/* ------------------------------------------------------------------------- */

static const int TetEdg[6][2] = { {0,1}, {1,2}, {2,0}, {3,0}, {3,1}, {3,2} };

int orc_tet_edges(int nt, const int *tet, int *edges)
{
   Hsh h;
   int i, j, n = 0, t[2];

   if(!hsh_init(&h, 2, 6 * nt))
      return -1;

   for(i=0;i<nt;i++)
      for(j=0;j<6;j++)
      {
         int a = tet[ 4*i + TetEdg[j][0] ], b = tet[ 4*i + TetEdg[j][1] ], key;
         t[0] = a < b ? a : b;
         t[1] = a < b ? b : a;
         key = hsh_key(&h, t);
         if(hsh_get(&h, key, t, NULL, 0))
            continue;
         hsh_add(&h, key, i, j, t);
         if(edges)
         {
            edges[2*n] = t[0];
            edges[2*n+1] = t[1];
         }
         n++;
      }

   hsh_free(&h);
   return n;
}

/* ------------------------------------------------------------------------- */
/* geometry in FP64 on float4 coordinates (w taken into account like the      */
/* OpenCL built-ins, but w = 0 for vertices)                                   */
/* ------------------------------------------------------------------------- */

typedef struct { double x, y, z, w; } D4;

static D4 ld4(const float *c, int v) { D4 r = { c[4*v], c[4*v+1], c[4*v+2], c[4*v+3] }; return r; }
static D4 sub(D4 a, D4 b) { D4 r = { a.x-b.x, a.y-b.y, a.z-b.z, a.w-b.w }; return r; }
static double dot4(D4 a, D4 b) { return a.x*b.x + a.y*b.y + a.z*b.z + a.w*b.w; }
static D4 cross4(D4 a, D4 b)
{
   D4 r = { a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x, 0. };
   return r;
}

/* single-precision constants of the reference kernels, as compiled */
#define C_TRISRF  ((double)0.5f)
#define C_TETVOL  ((double)0.166666f)
#define C_QAL     ((double)7.348469f)

/* examples/MeshQuality/compute_quality.cl:1-17 with toolkit.cl CalTriSrf
   (:124-127) and CalTetVol (:130-133).  The stray semicolons of lines 11-12
   make srf the area of faces (0,1,2) and (0,1,3) only. */
double orc_quality_ref1(const float *crd, const int *t)
{
   D4 a = ld4(crd, t[0]), b = ld4(crd, t[1]), c = ld4(crd, t[2]), d = ld4(crd, t[3]);
   double len, srf, vol, l;
   D4 e;

   e = sub(a, b); len = dot4(e, e);
   e = sub(a, c); l = dot4(e, e); if(l > len) len = l;
   e = sub(a, d); l = dot4(e, e); if(l > len) len = l;
   e = sub(b, c); l = dot4(e, e); if(l > len) len = l;
   e = sub(b, d); l = dot4(e, e); if(l > len) len = l;
   e = sub(c, d); l = dot4(e, e); if(l > len) len = l;

   { D4 n = cross4(sub(c, a), sub(b, a)); srf  = C_TRISRF * sqrt(dot4(n, n)); }
   { D4 n = cross4(sub(d, a), sub(b, a)); srf += C_TRISRF * sqrt(dot4(n, n)); }

   vol = C_TETVOL * dot4(cross4(sub(b, a), sub(c, a)), sub(d, a));
   return C_QAL * vol / (srf * sqrt(len));
}

void orc_quality_ref(int nt, const float *crd, const int *tet, double *q)
{
   for(int i=0;i<nt;i++)
      q[i] = orc_quality_ref1(crd, &tet[4*i]);
}

/* Mean-ratio quality of a tetrahedron: 12 (3|V|)^(2/3) / sum of squared edge
   lengths, 1 for the regular tet, signed by the orientation (negative for an
   inverted element).  V = det(b-a, c-a, d-a) / 6. */
double orc_mean_ratio1(const float *crd, const int *t)
{
   D4 a = ld4(crd, t[0]), b = ld4(crd, t[1]), c = ld4(crd, t[2]), d = ld4(crd, t[3]);
   D4 ab = sub(b, a), ac = sub(c, a), ad = sub(d, a), bc = sub(c, b), bd = sub(d, b), cd = sub(d, c);
   double det = dot4(cross4(ab, ac), ad);
   double l2 = dot4(ab, ab) + dot4(ac, ac) + dot4(ad, ad) + dot4(bc, bc) + dot4(bd, bd) + dot4(cd, cd);
   double v = fabs(det) / 6.0;
   double q = 12.0 * cbrt(9.0 * v * v) / l2;
   return det < 0 ? -q : q;
}

void orc_mean_ratio(int nt, const float *crd, const int *tet, double *q)
{
   for(int i=0;i<nt;i++)
      q[i] = orc_mean_ratio1(crd, &tet[4*i]);
}

/* signed FP64 determinant det(b-a, c-a, d-a) of the FP32 coordinates */
double orc_det1(const float *crd, const int *t)
{
   D4 a = ld4(crd, t[0]), b = ld4(crd, t[1]), c = ld4(crd, t[2]), d = ld4(crd, t[3]);
   return dot4(cross4(sub(b, a), sub(c, a)), sub(d, a));
}

/* ------------------------------------------------------------------------- */
/* reductions (reduce.cl:6-137 and the CPU finish of :3297-3327), exact       */
/* summation order independent: long double accumulation                      */
/* ------------------------------------------------------------------------- */

double orc_reduce(int op, int n, const float *x)
{
   long double s = 0.L;
   double m;
   int i;

   switch(op)
   {
      case 0: m = 3.402823466e38; for(i=0;i<n;i++) if(x[i] < m) m = x[i]; return m;
      case 1: m = -3.402823466e38; for(i=0;i<n;i++) if(x[i] > m) m = x[i]; return m;
      case 2: for(i=0;i<n;i++) s += x[i]; return (double)s;
      case 3: for(i=0;i<n;i++) s += (x[i] != 0.f); return (double)s;
      case 4: for(i=0;i<n;i++) s += fabsl((long double)x[i]); return (double)s;
      case 5: for(i=0;i<n;i++) s += (long double)x[i] * x[i]; return (double)s;
      case 6: m = 0; for(i=0;i<n;i++) if(fabs(x[i]) > m) m = fabs(x[i]); return m;
   }
   return 0.;
}

/* min / argmin / max / argmax, smallest index wins ties */
void orc_minmax_arg(int n, const double *x, double *vmin, int *imin, double *vmax, int *imax)
{
   int i, a = 0, b = 0;
   for(i=1;i<n;i++)
   {
      if(x[i] < x[a]) a = i;
      if(x[i] > x[b]) b = i;
   }
   *vmin = x[a]; *imin = a; *vmax = x[b]; *imax = b;
}

/* ------------------------------------------------------------------------- */
/* NodeSmoothing scatter / gather (examples/NodeSmoothing/scatter.cl:1-46,    */
/* gather.cl:1-17) in FP64                                                     */
/* ------------------------------------------------------------------------- */

static D4 d4add(D4 a, D4 b) { D4 r = { a.x+b.x, a.y+b.y, a.z+b.z, a.w+b.w }; return r; }
static D4 d4mul(D4 a, double s) { D4 r = { a.x*s, a.y*s, a.z*s, a.w*s }; return r; }

void orc_scatter(int nt, const float *crd, const int *tet, double *opt)
{
   static const int face[4][3] = { {1,2,3}, {0,2,3}, {1,0,3}, {1,2,0} };
   static const int ed[4][3] = { {3,4,5}, {1,2,5}, {0,2,4}, {0,1,3} };
   static const int nrm[4][2] = { {4,5}, {5,2}, {2,4}, {3,1} };
   const double k = (double)0.816496f, third = (double)(1.f/3.f);

   for(int i=0;i<nt;i++)
   {
      D4 v[4], e[6];
      double len[6];
      int j;
      for(j=0;j<4;j++)
         v[j] = ld4(crd, tet[4*i+j]);
      e[0] = sub(v[0], v[1]); e[1] = sub(v[0], v[2]); e[2] = sub(v[0], v[3]);
      e[3] = sub(v[1], v[2]); e[4] = sub(v[1], v[3]); e[5] = sub(v[2], v[3]);
      for(j=0;j<6;j++)
         len[j] = dot4(e[j], e[j]);
      for(j=0;j<4;j++)
      {
         double m = len[ ed[j][0] ];
         D4 ctr, n;
         double nn;
         if(len[ ed[j][1] ] > m) m = len[ ed[j][1] ];
         if(len[ ed[j][2] ] > m) m = len[ ed[j][2] ];
         m = k * sqrt(m);
         ctr = d4mul(d4add(d4add(v[ face[j][0] ], v[ face[j][1] ]), v[ face[j][2] ]), third);
         n = cross4(e[ nrm[j][0] ], e[ nrm[j][1] ]);
         nn = sqrt(dot4(n, n));
         n = d4mul(n, nn > 0 ? m / nn : 0.);
         n = d4add(ctr, n);
         opt[ 16*(size_t)i + 4*j ]     = n.x;
         opt[ 16*(size_t)i + 4*j + 1 ] = n.y;
         opt[ 16*(size_t)i + 4*j + 2 ] = n.z;
         opt[ 16*(size_t)i + 4*j + 3 ] = n.w;
      }
   }
}

/* gather over the vertex ball (codes (tet << 4) | local index), relaxation
   0.2 toward the mean of the optimal points, residual |old - new|^2 */
void orc_gather(int nv, const float *crd, const int *deg, const int *ball, int width,
                const double *opt, double *newcrd, double *res)
{
   const double w = (double)0.2f;
   for(int v=0;v<nv;v++)
   {
      D4 s = { 0, 0, 0, 0 }, o = ld4(crd, v), c;
      for(int k=0;k<deg[v];k++)
      {
         int code = ball[ (size_t)v * width + k ], t = code >> 4, j = code & 7;
         D4 p = { opt[16*(size_t)t+4*j], opt[16*(size_t)t+4*j+1], opt[16*(size_t)t+4*j+2], opt[16*(size_t)t+4*j+3] };
         s = d4add(s, p);
      }
      s = d4mul(s, deg[v] ? 1.0 / deg[v] : 0.);
      c = d4add(o, d4mul(sub(s, o), w));
      newcrd[4*(size_t)v] = c.x; newcrd[4*(size_t)v+1] = c.y;
      newcrd[4*(size_t)v+2] = c.z; newcrd[4*(size_t)v+3] = c.w;
      { D4 d = sub(o, c); res[v] = dot4(d, d); }
   }
}
