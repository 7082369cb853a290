/*
 * baseline.c -- multithreaded CPU port of the smoothing workload, timed as
 * the CPU baseline of the benchmark.  TEST INFRASTRUCTURE ONLY (the checker
 * side; the library never calls it).
 *
 * Same work as one GPU step: nsweeps times (Jacobi Laplacian sweep over the
 * ball of points in CSR form, then mean-ratio quality with a 64-bin
 * histogram, min/argmin and the inverted count), FP32 arithmetic, OpenMP
 * over vertices and tetrahedra on all host cores.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

int orc_threads(void)
{
   return omp_get_max_threads();
}

void orc_bench_step(int nv, int nt, float *crd, float *tmp, const int *tet,
                    const long long *ptr, const int *col, float omega, int nsweeps,
                    unsigned *hist, float *qmin, int *imin, unsigned *ninv)
{
   for(int s=0;s<nsweeps;s++)
   {
      float *in = (s & 1) ? tmp : crd, *out = (s & 1) ? crd : tmp;
      unsigned h[64] = {0}, inv = 0;
      float bm = 3.4e38f;
      int bi = 0;

      #pragma omp parallel for schedule(static)
      for(int v=0;v<nv;v++)
      {
         long long d = ptr[v+1] - ptr[v];
         const float *p = &in[4*(size_t)v];
         float sx = 0.f, sy = 0.f, sz = 0.f;
         if(!d)
         {
            memcpy(&out[4*(size_t)v], p, 16);
            continue;
         }
         for(long long k=ptr[v];k<ptr[v+1];k++)
         {
            const float *q = &in[ 4 * (size_t)col[k] ];
            sx += q[0]; sy += q[1]; sz += q[2];
         }
         float inv_d = 1.f / (float)d;
         out[4*(size_t)v]   = p[0] + omega * (sx * inv_d - p[0]);
         out[4*(size_t)v+1] = p[1] + omega * (sy * inv_d - p[1]);
         out[4*(size_t)v+2] = p[2] + omega * (sz * inv_d - p[2]);
         out[4*(size_t)v+3] = 0.f;
      }

      #pragma omp parallel
      {
         unsigned lh[64] = {0}, linv = 0;
         float lm = 3.4e38f;
         int li = 0;
         #pragma omp for schedule(static) nowait
         for(int t=0;t<nt;t++)
         {
            const float *a = &out[4*(size_t)tet[4*t]], *b = &out[4*(size_t)tet[4*t+1]];
            const float *c = &out[4*(size_t)tet[4*t+2]], *d = &out[4*(size_t)tet[4*t+3]];
            float ab[3], ac[3], ad[3], bc[3], bd[3], cd[3], det, l2, q;
            for(int k=0;k<3;k++)
            {
               ab[k] = b[k] - a[k]; ac[k] = c[k] - a[k]; ad[k] = d[k] - a[k];
               bc[k] = c[k] - b[k]; bd[k] = d[k] - b[k]; cd[k] = d[k] - c[k];
            }
            det = ab[0] * (ac[1]*ad[2] - ac[2]*ad[1]) + ab[1] * (ac[2]*ad[0] - ac[0]*ad[2])
                + ab[2] * (ac[0]*ad[1] - ac[1]*ad[0]);
            l2 = 0.f;
            for(int k=0;k<3;k++)
               l2 += ab[k]*ab[k] + ac[k]*ac[k] + ad[k]*ad[k] + bc[k]*bc[k] + bd[k]*bd[k] + cd[k]*cd[k];
            q = 12.f * powf(3.f * fabsf(det) / 6.f, 2.f / 3.f) / l2;
            if(!(det > 0.f)) { q = -q; linv++; }
            int bin = (int)(q * 64.f);
            bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
            lh[bin]++;
            if(q < lm) { lm = q; li = t; }
         }
         #pragma omp critical
         {
            for(int k=0;k<64;k++) h[k] += lh[k];
            inv += linv;
            if(lm < bm || (lm == bm && li < bi)) { bm = lm; bi = li; }
         }
      }
      if(hist) memcpy(hist + 64 * s, h, sizeof(h));
      if(qmin) qmin[s] = bm;
      if(imin) imin[s] = bi;
      if(ninv) ninv[s] = inv;
   }
   if(nsweeps & 1)
      memcpy(crd, tmp, (size_t)nv * 16);
}
