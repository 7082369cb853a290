/*
 * oracle_linalg.c -- FP64 serial oracle of the block sparse algebra
 * (TEST INFRASTRUCTURE: the checker, never part of the library).
 *
 *   orc_bsr_spmv   y = A x for a block CSR matrix (b x b row-major blocks),
 *                  the product the reference's MulMatVec kernels compute
 *                  block by block (sources/multmatvec.cl:30-68) from the CSR
 *                  arrays given to GmlNewMatrix (sources/gmlib3.c:1175-1427);
 *   orc_cg         textbook conjugate gradients (Hestenes and Stiefel, 1952)
 *                  in FP64 with long-double dot products, x0 = 0, stopping
 *                  on |r| <= tol |b| of the recursive residual;
 *   orc_rel_residual  |b - A x| / |b| with long-double accumulation.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

void orc_bsr_spmv(int nrow, int b, const int *lin, const int *col, const double *val,
                  const double *x, double *y)
{
   for(int r=0;r<nrow;r++)
   {
      long double acc[8] = { 0 };
      for(int k=lin[r];k<lin[r+1];k++)
      {
         const double *blk = val + (size_t)k * b * b;
         const double *xv = x + (size_t)col[k] * b;
         for(int i=0;i<b;i++)
            for(int j=0;j<b;j++)
               acc[i] += (long double)blk[i * b + j] * xv[j];
      }
      for(int i=0;i<b;i++)
         y[(size_t)r * b + i] = (double)acc[i];
   }
}

static double orc_dot(size_t n, const double *u, const double *v)
{
   long double s = 0;
   for(size_t i=0;i<n;i++)
      s += (long double)u[i] * v[i];
   return (double)s;
}

double orc_rel_residual(int nrow, int b, const int *lin, const int *col, const double *val,
                        const double *rhs, const double *x)
{
   size_t n = (size_t)nrow * b;
   double *ax = malloc(n * sizeof(double));
   long double rr = 0, bb = 0;
   if(!ax)
      return -1.;
   orc_bsr_spmv(nrow, b, lin, col, val, x, ax);
   for(size_t i=0;i<n;i++)
   {
      long double d = (long double)rhs[i] - ax[i];
      rr += d * d;
      bb += (long double)rhs[i] * rhs[i];
   }
   free(ax);
   return bb > 0 ? (double)sqrtl(rr / bb) : 0.;
}

int orc_cg(int nrow, int b, const int *lin, const int *col, const double *val,
           const double *rhs, double *x, double tol, int maxit)
{
   size_t n = (size_t)nrow * b;
   double *r = malloc(n * sizeof(double)), *p = malloc(n * sizeof(double));
   double *q = malloc(n * sizeof(double));
   double rr, bb, stop;
   int it = 0;
   if(!r || !p || !q)
   {
      free(r); free(p); free(q);
      return -1;
   }
   memset(x, 0, n * sizeof(double));
   memcpy(r, rhs, n * sizeof(double));
   memcpy(p, rhs, n * sizeof(double));
   bb = rr = orc_dot(n, r, r);
   stop = tol * tol * bb;
   while(rr > stop && it < maxit)
   {
      double pq, a, rn, beta;
      orc_bsr_spmv(nrow, b, lin, col, val, p, q);
      pq = orc_dot(n, p, q);
      if(!(pq > 0.))
         break;
      a = rr / pq;
      for(size_t i=0;i<n;i++)
      {
         x[i] += a * p[i];
         r[i] -= a * q[i];
      }
      rn = orc_dot(n, r, r);
      beta = rn / rr;
      rr = rn;
      for(size_t i=0;i<n;i++)
         p[i] = r[i] + beta * p[i];
      it++;
   }
   free(r); free(p); free(q);
   return it;
}
