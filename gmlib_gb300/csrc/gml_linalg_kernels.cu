/*
 * gml_linalg_kernels.cu -- block sparse mat-vec and block-vector kernels.
 *
 * Replaces sources/multmatvec.cl (MulMatVecSlc16..256, block sizes 4 and 5;
 * block size 7 has no kernel there), multdiagmatvec.cl, addvec.cl,
 * scalevec.cl and normvec.cl.  All are HBM-bound streaming kernels:
 *
 *   SpMV     one thread per block row over the SELL-32 layout of
 *            gml_linalg.c: column indices and block values of entry k are
 *            128-byte runs per warp, x lines are gathered with 16-byte
 *            vector loads (x fits in L2), y is written once.
 *            Bytes per row: 4 (degree) + deg * (4 + 4*b*b or 8*b*b) + the
 *            output line; the x gathers are served by L2.
 *   vectors  grid-stride loops over 16-byte chunks.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include "gml_device.h"

/* block-sparse SpMV tuning: the k-loop unroll and the load used for the
   matrix streams (column indices and values, read once per product).
   Measured on the 96^3 cube system (FP32): no unrolling and evict-first
   streaming loads (ld.global.cs) take the reference-API SpMV from 97.8 to
   92.2 us and the CG's fused SpMV from 120.1 to 108.1 us; the streamed
   matrix no longer pushes the just-written vectors out of L2, so the CG
   update also drops from 27.0 to 22.7 us. */
#ifndef SPMV_UNROLL
#define SPMV_UNROLL 1
#endif
constexpr int kSpmvUnroll = SPMV_UNROLL;   /* pragma arguments are not macro-expanded */
#ifndef SPMV_STREAM
#define SPMV_STREAM 1
#endif
#if SPMV_STREAM
#define SPMV_LDM(p) __ldcs(p)
#else
#define SPMV_LDM(p) __ldg(p)
#endif
#include "gml_linalg.h"

#define LA_THREADS 256

/* load one vector line of XS scalars with 16-byte loads */
template<class T, int XS> __device__ __forceinline__ void load_line(const T *__restrict__ p, T *out)
{
   constexpr int NCH = (XS * (int)sizeof(T) + 15) / 16;
   if((XS * sizeof(T)) % 16 == 0)
   {
#pragma unroll
      for(int c=0;c<NCH;c++)
      {
         float4 v = __ldg(reinterpret_cast<const float4 *>(p) + c);
         const T *t = reinterpret_cast<const T *>(&v);
#pragma unroll
         for(int i=0;i<(int)(16/sizeof(T));i++)
            out[ c * (16 / sizeof(T)) + i ] = t[i];
      }
   }
   else
   {
#pragma unroll
      for(int i=0;i<XS;i++)
         out[i] = __ldg(p + i);
   }
}

template<int B, class T, int XS>
__global__ void __launch_bounds__(LA_THREADS)
sell_spmv_kernel(int n, const int64_t *__restrict__ soff, const int *__restrict__ deg,
                 const int *__restrict__ col, const T *__restrict__ val,
                 const T *__restrict__ x, T *__restrict__ y, int ys)
{
   int r = blockIdx.x * blockDim.x + threadIdx.x;
   if(r >= n)
      return;

   const int lane = r & 31;
   const int64_t base = __ldg(&soff[ r >> 5 ]);
   const int d = __ldg(&deg[r]);
   const int *cp = col + base * 32 + lane;
   const T *vp = val + base * (B * B * 32) + lane;
   T acc[B];

#pragma unroll
   for(int i=0;i<B;i++)
      acc[i] = (T)0;

#pragma unroll kSpmvUnroll
   for(int k=0;k<d;k++)
   {
      const int c = SPMV_LDM(cp + (size_t)k * 32);
      T xv[XS];
      load_line<T, XS>(x + (size_t)c * XS, xv);
      const T *blk = vp + (size_t)k * (B * B * 32);
#pragma unroll
      for(int i=0;i<B;i++)
#pragma unroll
         for(int j=0;j<B;j++)
            acc[i] += SPMV_LDM(blk + (i * B + j) * 32) * xv[j];
   }

   T *yl = y + (size_t)r * ys;
#pragma unroll
   for(int i=0;i<B;i++)
      yl[i] = acc[i];
   for(int i=B;i<ys;i++)
      yl[i] = (T)0;
}

template<int B, class T>
static int launch_spmv(const GmlSellDev *A, const void *x, int xs, void *y, int ys, cudaStream_t st)
{
   int nb = (A->NmbLin + LA_THREADS - 1) / LA_THREADS;
   if(xs == 4)
      sell_spmv_kernel<B, T, 4><<<nb, LA_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg, A->Col,
         (const T *)A->Val, (const T *)x, (T *)y, ys);
   else if(xs == 8)
      sell_spmv_kernel<B, T, 8><<<nb, LA_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg, A->Col,
         (const T *)A->Val, (const T *)x, (T *)y, ys);
   else
      return 0;
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_sell_spmv(GmdCtx *ctx, const GmlSellDev *A, const void *x, int xs,
                             void *y, int ys, double alpha, double beta, double *dotout, int flags)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   (void)alpha; (void)beta; (void)dotout; (void)flags;
   if(!ctx)
      return 0;
   if(A->FltSiz == 4)
   {
      switch(A->BlkSiz)
      {
         case 3: return launch_spmv<3, float>(A, x, xs, y, ys, st);
         case 4: return launch_spmv<4, float>(A, x, xs, y, ys, st);
         case 5: return launch_spmv<5, float>(A, x, xs, y, ys, st);
         case 7: return launch_spmv<7, float>(A, x, xs, y, ys, st);
      }
   }
   else
   {
      switch(A->BlkSiz)
      {
         case 3: return launch_spmv<3, double>(A, x, xs, y, ys, st);
         case 4: return launch_spmv<4, double>(A, x, xs, y, ys, st);
         case 5: return launch_spmv<5, double>(A, x, xs, y, ys, st);
         case 7: return launch_spmv<7, double>(A, x, xs, y, ys, st);
      }
   }
   return 0;
}

/* ------------------------------------------------------------------------- */
/* vectors                                                                    */
/* ------------------------------------------------------------------------- */

template<class T>
__global__ void __launch_bounds__(LA_THREADS)
add3_kernel(const T *__restrict__ u, const T *__restrict__ v, const T *__restrict__ w,
            T *__restrict__ y, size_t n)
{
   size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
   for(;i<n;i+=nth)
      y[i] = __ldg(&u[i]) + __ldg(&v[i]) + __ldg(&w[i]);
}

__global__ void __launch_bounds__(LA_THREADS)
add3_f4_kernel(const float4 *__restrict__ u, const float4 *__restrict__ v,
               const float4 *__restrict__ w, float4 *__restrict__ y, size_t n4)
{
   size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
   for(;i<n4;i+=nth)
   {
      float4 a = __ldg(&u[i]), b = __ldg(&v[i]), c = __ldg(&w[i]);
      y[i] = make_float4(a.x + b.x + c.x, a.y + b.y + c.y, a.z + b.z + c.z, a.w + b.w + c.w);
   }
}

static unsigned grid_for(GmdCtx *ctx, size_t n)
{
   size_t g = (n + LA_THREADS - 1) / LA_THREADS, cap = (size_t)gmd_num_sms(ctx) * 8;
   if(g > cap) g = cap;
   return (unsigned)(g ? g : 1);
}

extern "C" int gmd_vec_add3(GmdCtx *ctx, const void *u, const void *v, const void *w, void *y,
                            size_t n, int fltsiz)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if(!ctx)
      return 0;
   if(fltsiz == 4 && n % 4 == 0)
      add3_f4_kernel<<<grid_for(ctx, n / 4), LA_THREADS, 0, st>>>((const float4 *)u, (const float4 *)v,
         (const float4 *)w, (float4 *)y, n / 4);
   else if(fltsiz == 4)
      add3_kernel<float><<<grid_for(ctx, n), LA_THREADS, 0, st>>>((const float *)u, (const float *)v,
         (const float *)w, (float *)y, n);
   else
      add3_kernel<double><<<grid_for(ctx, n), LA_THREADS, 0, st>>>((const double *)u, (const double *)v,
         (const double *)w, (double *)y, n);
   return cudaGetLastError() == cudaSuccess;
}

__device__ __forceinline__ float4 scale16(float4 a, float s)
{
   return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}

__device__ __forceinline__ double2 scale16(double2 a, double s)
{
   return make_double2(a.x * s, a.y * s);
}

template<class T>
__global__ void __launch_bounds__(LA_THREADS) scale_kernel(T *__restrict__ u, size_t n, T s)
{
   size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (size_t)gridDim.x * blockDim.x;
   for(;i<n;i+=nth)
      u[i] *= s;
}

/* in place, 16 bytes per access and two accesses in flight per thread */
template<class V, class T>
__global__ void __launch_bounds__(LA_THREADS) scale16_kernel(V *__restrict__ u, size_t n16, T s)
{
   const size_t nth = (size_t)gridDim.x * blockDim.x;
   size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
   for(;i + nth < n16;i+=2*nth)
   {
      V a = u[i], b = u[i + nth];
      u[i] = scale16(a, s);
      u[i + nth] = scale16(b, s);
   }
   if(i < n16)
      u[i] = scale16(u[i], s);
}

extern "C" int gmd_vec_scale(GmdCtx *ctx, void *u, size_t n, int fltsiz, double s)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if(!ctx)
      return 0;
   if(fltsiz == 4 && n % 4 == 0 && ((uintptr_t)u & 15) == 0)
      scale16_kernel<float4, float><<<grid_for(ctx, n / 4), LA_THREADS, 0, st>>>((float4 *)u, n / 4,
                                                                                 (float)s);
   else if(fltsiz == 8 && n % 2 == 0 && ((uintptr_t)u & 15) == 0)
      scale16_kernel<double2, double><<<grid_for(ctx, n / 2), LA_THREADS, 0, st>>>((double2 *)u,
                                                                                   n / 2, s);
   else if(fltsiz == 4)
      scale_kernel<float><<<grid_for(ctx, n), LA_THREADS, 0, st>>>((float *)u, n, (float)s);
   else
      scale_kernel<double><<<grid_for(ctx, n), LA_THREADS, 0, st>>>((double *)u, n, s);
   return cudaGetLastError() == cudaSuccess;
}

template<class T>
__global__ void __launch_bounds__(LA_THREADS)
rownorm_kernel(const T *__restrict__ u, int us, int nl, int nlin, float *__restrict__ out)
{
   int l = blockIdx.x * blockDim.x + threadIdx.x;
   if(l >= nlin)
      return;
   T s = (T)0;
   for(int c=0;c<nl;c++)
   {
      T x = __ldg(&u[ (size_t)l * us + c ]);
      s += x * x;
   }
   out[l] = (float)sqrt(s);
}

extern "C" int gmd_vec_rownorm(GmdCtx *ctx, const void *u, int us, int nlanes, int fltsiz,
                               int nlin, float *out)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   int nb = (nlin + LA_THREADS - 1) / LA_THREADS;
   if(!ctx)
      return 0;
   if(fltsiz == 4)
      rownorm_kernel<float><<<nb, LA_THREADS, 0, st>>>((const float *)u, us, nlanes, nlin, out);
   else
      rownorm_kernel<double><<<nb, LA_THREADS, 0, st>>>((const double *)u, us, nlanes, nlin, out);
   return cudaGetLastError() == cudaSuccess;
}

template<class T>
__global__ void __launch_bounds__(LA_THREADS)
diag_kernel(const T *__restrict__ d, int ds, const T *__restrict__ u, T *__restrict__ v,
            int vs, int b, int nlin)
{
   int l = blockIdx.x * blockDim.x + threadIdx.x;
   if(l >= nlin)
      return;
   const T *dl = d + (size_t)l * ds;
   const T *ul = u + (size_t)l * vs;
   T *vl = v + (size_t)l * vs;
   T x[8];
   for(int j=0;j<b && j<8;j++)
      x[j] = __ldg(&ul[j]);
   for(int i=0;i<b;i++)
   {
      T s = (T)0;
      for(int j=0;j<b && j<8;j++)
         s += __ldg(&dl[ i * b + j ]) * x[j];
      vl[i] = s;
   }
   for(int i=b;i<vs;i++)
      vl[i] = (T)0;
}

/* 3x3 blocks, the common case: the block line (9 of 16 stored values) and
   the vector lines (3 of 4) move as 16-byte pieces.  The products are summed
   in the generic kernel's order, so the results are the same. */
__global__ void __launch_bounds__(LA_THREADS)
diag3_f32_kernel(const float4 *__restrict__ d, int ds4, const float4 *__restrict__ u,
                 float4 *__restrict__ v, int nlin)
{
   const int l = blockIdx.x * blockDim.x + threadIdx.x;
   if(l >= nlin)
      return;
   const float4 *dl = d + (size_t)l * ds4;
   const float4 a = __ldg(dl), b = __ldg(dl + 1), c = __ldg(dl + 2), x = __ldg(u + l);
   v[l] = make_float4(a.x * x.x + a.y * x.y + a.z * x.z,
                      a.w * x.x + b.x * x.y + b.y * x.z,
                      b.z * x.x + b.w * x.y + c.x * x.z, 0.f);
}

__global__ void __launch_bounds__(LA_THREADS)
diag3_f64_kernel(const double2 *__restrict__ d, int ds2, const double2 *__restrict__ u,
                 double2 *__restrict__ v, int nlin)
{
   const int l = blockIdx.x * blockDim.x + threadIdx.x;
   if(l >= nlin)
      return;
   const double2 *dl = d + (size_t)l * ds2;
   const double2 m0 = __ldg(dl), m1 = __ldg(dl + 1), m2 = __ldg(dl + 2), m3 = __ldg(dl + 3);
   const double2 m4 = __ldg(dl + 4), x0 = __ldg(u + 2 * (size_t)l), x1 = __ldg(u + 2 * (size_t)l + 1);
   /* block values m00 m01 | m02 m10 | m11 m12 | m20 m21 | m22 -, vector x y | z - */
   v[2 * (size_t)l]     = make_double2(m0.x * x0.x + m0.y * x0.y + m1.x * x1.x,
                                       m1.y * x0.x + m2.x * x0.y + m2.y * x1.x);
   v[2 * (size_t)l + 1] = make_double2(m3.x * x0.x + m3.y * x0.y + m4.x * x1.x, 0.);
}

extern "C" int gmd_vec_diag(GmdCtx *ctx, const void *d, int ds, const void *u, void *v, int vs,
                            int b, int fltsiz, int nlin)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   int nb = (nlin + LA_THREADS - 1) / LA_THREADS;
   if(!ctx || b > 8)
      return 0;
   const int aligned = !(((uintptr_t)d | (uintptr_t)u | (uintptr_t)v) & 15);
   if(b == 3 && vs == 4 && aligned && fltsiz == 4 && ds % 4 == 0 && ds >= 12)
   {
      diag3_f32_kernel<<<nb, LA_THREADS, 0, st>>>((const float4 *)d, ds / 4, (const float4 *)u,
                                                  (float4 *)v, nlin);
      return cudaGetLastError() == cudaSuccess;
   }
   if(b == 3 && vs == 4 && aligned && fltsiz == 8 && ds % 2 == 0 && ds >= 10)
   {
      diag3_f64_kernel<<<nb, LA_THREADS, 0, st>>>((const double2 *)d, ds / 2, (const double2 *)u,
                                                  (double2 *)v, nlin);
      return cudaGetLastError() == cudaSuccess;
   }
   if(fltsiz == 4)
      diag_kernel<float><<<nb, LA_THREADS, 0, st>>>((const float *)d, ds, (const float *)u,
                                                    (float *)v, vs, b, nlin);
   else
      diag_kernel<double><<<nb, LA_THREADS, 0, st>>>((const double *)d, ds, (const double *)u,
                                                     (double *)v, vs, b, nlin);
   return cudaGetLastError() == cudaSuccess;
}

/* ------------------------------------------------------------------------- */
/* SELL-32 repack of a block CSR matrix on the device                         */
/* ------------------------------------------------------------------------- */

/* one warp per slice: row degrees and the slice width (longest row) */
__global__ void __launch_bounds__(LA_THREADS)
sell_width_kernel(int nrow, const int *__restrict__ lin, int *__restrict__ deg,
                  long long *__restrict__ width, int *err)
{
   const int sl = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
   const int lane = threadIdx.x & 31, nsl = (nrow + 31) / 32;
   if(sl >= nsl)
      return;
   const int r = sl * 32 + lane;
   int d = 0;
   if(r < nrow)
   {
      d = lin[r + 1] - lin[r];
      if(d < 0)
      {
         atomicOr(err, 1);
         d = 0;
      }
      deg[r] = d;
   }
   const int w = __reduce_max_sync(0xffffffffu, d);
   if(lane == 0)
      width[sl] = w;
}

/* one thread per row: entry k of row r goes to run (soff[slice] + k) of its
   slice; out-of-range columns are reported and stored as column 0 with zero
   values */
template<class T>
__global__ void __launch_bounds__(LA_THREADS)
sell_fill_kernel(int nrow, int bb, const int *__restrict__ lin, const int *__restrict__ col,
                 const T *__restrict__ val, const long long *__restrict__ soff,
                 int *__restrict__ Col, T *__restrict__ Val, int *err)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   if(r >= nrow)
      return;
   const int lane = r & 31, b0 = lin[r], d = lin[r + 1] - b0;
   const long long base = soff[r >> 5];
   for(int k=0;k<d;k++)
   {
      const long long e = base + k;
      const int c = col[b0 + k];
      const bool ok = c >= 0 && c < nrow;
      if(!ok)
         atomicOr(err, 2);
      Col[e * 32 + lane] = ok ? c : 0;
      for(int v=0;v<bb;v++)
         Val[(e * bb + v) * 32 + lane] = ok ? val[(size_t)(b0 + k) * bb + v] : (T)0;
   }
}

extern "C" int gmd_sell_widths(GmdCtx *ctx, int nrow, const int *lin, int *deg, long long *width,
                               int *err)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const int nsl = (nrow + 31) / 32;
   const unsigned g = (unsigned)(((long long)nsl * 32 + LA_THREADS - 1) / LA_THREADS);
   sell_width_kernel<<<g, LA_THREADS, 0, st>>>(nrow, lin, deg, width, err);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_sell_fill(GmdCtx *ctx, int nrow, int bb, int fltsiz, const int *lin,
                             const int *col, const void *val, const long long *soff, int *Col,
                             void *Val, int *err)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const unsigned g = (unsigned)((nrow + LA_THREADS - 1) / LA_THREADS);
   if(fltsiz == 4)
      sell_fill_kernel<float><<<g, LA_THREADS, 0, st>>>(nrow, bb, lin, col, (const float *)val,
                                                        soff, Col, (float *)Val, err);
   else
      sell_fill_kernel<double><<<g, LA_THREADS, 0, st>>>(nrow, bb, lin, col, (const double *)val,
                                                         soff, Col, (double *)Val, err);
   return cudaGetLastError() == cudaSuccess;
}
