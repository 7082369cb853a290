/*
 * gml_problem.c -- synthetic symmetric positive definite block systems on
 * the vertex graph of a tetrahedral cube (host utility, no counterpart in the
 * reference library).
 *
 * The reference's LinearSolver example assembles a block matrix on the edge
 * graph of a tet mesh: unique edges from GmlExtractEdges give the
 * off-diagonal blocks of both triangles and the diagonal goes into its own
 * vector (examples/LinearSolver/LinearSolver.c:157-258).  The system built
 * here has the same sparsity, with the diagonal block stored in the matrix:
 *
 *   mesh      GmlxCubeMesh(n, split) without jitter, Hilbert renumbered, so
 *             the rows follow the vertex order the mesh kernels use;
 *   pattern   row v holds v itself and every vertex sharing a tet with v,
 *             columns ascending (2E + V blocks for E edges);
 *   values    each edge {i < j} gets a 3x3 block B with entries uniform in
 *             [-1, 0], drawn from a counter-based generator keyed by
 *             (seed, i, j) so the values do not depend on the traversal
 *             order; A_ij = B and A_ji = B^T.  The diagonal block of row v is
 *             diag(1 + sum over the off-diagonal entries of each scalar row of
 *             their absolute values): symmetric and strictly diagonally
 *             dominant with a positive diagonal, hence positive definite;
 *   rhs       uniform in [-1, 1] per scalar, from the seed.
 *
 * A 6-tet split with one diagonal per face and one per hex has
 * E = 3n(n+1)^2 + 3n^2(n+1) + n^3 edges whatever the diagonals' directions,
 * so both splits of GmlxCubeMesh give the same sizes.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "gmlib3_gb300.h"

#define SPD_MAXNGB 128

static uint64_t spd_mix(uint64_t z)
{
   z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
   z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
   return z ^ (z >> 31);
}

/* uniform in [0, 1) from a 64-bit word */
static double spd_unit(uint64_t z)
{
   return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

int GmlxCubeSpdSizes(int n, int split, int *NmbLin, int *NmbBlk)
{
   long long m = (long long)n + 1, e, v;
   (void)split;
   if(n < 1)
      return 0;
   v = m * m * m;
   e = 3LL * n * m * m + 3LL * n * n * m + (long long)n * n * n;
   if(2 * e + v > 2147483647LL)
      return 0;
   if(NmbLin) *NmbLin = (int)v;
   if(NmbBlk) *NmbBlk = (int)(2 * e + v);
   return 1;
}

/* off-diagonal block of the edge {lo, hi}, row-major, as seen from row lo */
static void spd_block(uint64_t seed, int lo, int hi, double b[9])
{
   uint64_t key = spd_mix(seed ^ (0x9e3779b97f4a7c15ULL * ((uint64_t)(uint32_t)lo + 1)))
                ^ spd_mix((uint64_t)(uint32_t)hi * 0xd1b54a32d192ed03ULL + 0x2545f4914f6cdd1dULL);
   for(int c=0;c<9;c++)
      b[c] = -spd_unit(spd_mix(key + 0x632be59bd9b4e019ULL * (uint64_t)(c + 1)));
}

int GmlxCubeSpdMatrix(int n, int split, uint64_t seed, int *lin, int *col, double *val,
                      double *rhs)
{
   int nv, nt, NmbLin, NmbBlk, v, t, k, ok = 0;
   float *crd = NULL;
   int *tet = NULL, *ref = NULL, *vtp = NULL, *vtl = NULL, *fill = NULL;

   if(!GmlxCubeSpdSizes(n, split, &NmbLin, &NmbBlk) || !lin || !col || !val)
      return 0;
   GmlxCubeSizes(n, &nv, &nt);
   crd = malloc((size_t)nv * 4 * sizeof(float));
   tet = malloc((size_t)nt * 4 * sizeof(int));
   ref = malloc((size_t)nv * sizeof(int));
   vtp = calloc((size_t)nv + 1, sizeof(int));
   vtl = malloc((size_t)nt * 4 * sizeof(int));
   fill = calloc((size_t)nv, sizeof(int));
   if(!crd || !tet || !ref || !vtp || !vtl || !fill)
      goto done;
   if(!GmlxCubeMesh(n, split, 0.0, seed, crd, tet, ref)
   || !GmlxHilbertRenumber(nv, crd, ref, nt, tet, NULL))
      goto done;

   /* vertex -> tet lists */
   for(t=0;t<4*nt;t++)
      vtp[ tet[t] + 1 ]++;
   for(v=0;v<nv;v++)
      vtp[v+1] += vtp[v];
   for(t=0;t<nt;t++)
      for(k=0;k<4;k++)
      {
         int w = tet[4*t+k];
         vtl[ vtp[w] + fill[w]++ ] = t;
      }

   /* rows: v and its neighbours, ascending */
   lin[0] = 0;
   for(v=0;v<nv;v++)
   {
      int ngb[SPD_MAXNGB], cnt = 0, i, j, pos, dia = -1;
      double sum[3] = { 0., 0., 0. };
      ngb[cnt++] = v;
      for(i=vtp[v];i<vtp[v+1];i++)
         for(k=0;k<4;k++)
         {
            int w = tet[ 4 * vtl[i] + k ], seen = 0;
            for(j=0;j<cnt;j++)
               if(ngb[j] == w) { seen = 1; break; }
            if(seen)
               continue;
            if(cnt == SPD_MAXNGB)
               goto done;
            ngb[cnt++] = w;
         }
      /* insertion sort (rows are short) */
      for(i=1;i<cnt;i++)
      {
         int x = ngb[i];
         for(j=i-1;j>=0 && ngb[j] > x;j--)
            ngb[j+1] = ngb[j];
         ngb[j+1] = x;
      }
      pos = lin[v];
      if(pos + cnt > NmbBlk)
         goto done;
      for(i=0;i<cnt;i++)
      {
         int w = ngb[i];
         double *b = val + 9 * (size_t)(pos + i);
         col[pos + i] = w;
         if(w == v)
         {
            dia = pos + i;
            continue;
         }
         if(v < w)
            spd_block(seed, v, w, b);
         else
         {
            double bt[9];
            spd_block(seed, w, v, bt);
            for(int r=0;r<3;r++)
               for(int c=0;c<3;c++)
                  b[3*r+c] = bt[3*c+r];
         }
         for(int r=0;r<3;r++)
            sum[r] += -(b[3*r] + b[3*r+1] + b[3*r+2]);     /* entries are <= 0 */
      }
      {
         double *d = val + 9 * (size_t)dia;
         memset(d, 0, 9 * sizeof(double));
         for(int r=0;r<3;r++)
            d[4*r] = 1.0 + sum[r];
      }
      lin[v+1] = pos + cnt;
   }
   if(lin[nv] != NmbBlk)
      goto done;

   if(rhs)
      for(v=0;v<3*nv;v++)
         rhs[v] = 2.0 * spd_unit(spd_mix(seed ^ (0xa0761d6478bd642fULL * (uint64_t)(v + 1)))) - 1.0;
   ok = 1;

done:
   free(crd); free(tet); free(ref); free(vtp); free(vtl); free(fill);
   return ok;
}
