/*
 * gml_solver_kernels.cu -- kernels of the conjugate-gradient solvers.
 *
 * The reference has no Krylov solver: its LinearSolver example iterates a
 * fixed-point (Jacobi-like) update with GmlMultMatVec, GmlMultDiagMatVec and
 * GmlAddVec3 (examples/LinearSolver/LinearSolver.c:300-338).  These kernels
 * run CG on the same SELL-32 block matrices (gml_linalg.c) in two forms:
 *
 *   FP64       matrix, vectors and dots in FP64;
 *   refinement FP32 matrix copy and FP32 vectors inside the CG iterations,
 *              dots accumulated in FP64, and an FP64 outer loop that keeps x,
 *              recomputes the true residual b - A x with the FP64 matrix and
 *              restarts the FP32 CG on it.
 *
 * Three kernels make an iteration:
 *
 *   spmv_dot   q = A p and p.q, one thread per block row, the SELL-32 entry
 *              runs read as 128-byte lines, p lines gathered through L2 with
 *              16-byte loads; the last block to finish sets alpha = rr / p.q;
 *   update     x += alpha p, r -= alpha q and |r|^2; the last block sets
 *              beta, rr and the stop flag;
 *   dir        p = r + beta p.
 *
 * Every kernel returns at once when the stop flag is set, so a CUDA graph of
 * a fixed number of iterations can be replayed past convergence.  The dots
 * are deterministic: per-block partials are folded in a fixed order.
 *
 * Vectors keep GmlNewVector's padded lines (4 lanes for b <= 4, 8 for
 * b <= 8).  HBM bytes per iteration (n = lanes * rows scalars, s = scalar
 * size): spmv_dot = matrix (4 + s b^2 per stored block, 4 per row) + 2 n s,
 * update = 6 n s, dir = 3 n s.
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
#include "gml_solver.h"

#define SV_THREADS 256

__device__ __forceinline__ double sv_warp_sum(double v)
{
   for(int o=16;o>0;o>>=1)
      v += __shfl_xor_sync(0xffffffffu, v, o);
   return v;
}

/* block sum of v into thread 0 */
__device__ __forceinline__ double sv_block_sum(double v)
{
   __shared__ double sh[SV_THREADS / 32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   v = sv_warp_sum(v);
   __syncthreads();
   if(lane == 0)
      sh[wid] = v;
   __syncthreads();
   v = 0.;
   if(wid == 0)
   {
      v = lane < SV_THREADS / 32 ? sh[lane] : 0.;
      v = sv_warp_sum(v);
   }
   return v;
}

/* grid sum: every block contributes v; returns 1 in thread 0 of the last
   block to arrive, with *tot the sum of the per-block partials in block
   order */
__device__ __forceinline__ int sv_grid_sum(double v, double *part, GmdSvScal *sc, double *tot)
{
   __shared__ int last;
   v = sv_block_sum(v);
   if(threadIdx.x == 0)
   {
      part[ blockIdx.x ] = v;
      __threadfence();
      last = (atomicAdd(&sc->ticket, 1ULL) == (unsigned long long)(gridDim.x - 1));
   }
   __syncthreads();
   if(!last)
      return 0;
   __threadfence();
   v = 0.;
   for(int i=threadIdx.x;i<(int)gridDim.x;i+=blockDim.x)
      v += ((volatile double *)part)[i];
   v = sv_block_sum(v);
   if(threadIdx.x != 0)
      return 0;
   sc->ticket = 0ULL;
   *tot = v;
   return 1;
}

__device__ __forceinline__ int sv_stopped(const GmdSvScal *sc)
{
   return *(volatile const int *)&sc->done;
}

/* ------------------------------------------------------------------------- */
/* vectors are padded lines of VS scalars (VS = 4 for b <= 4, 8 for b <= 8),   */
/* the layout of GmlNewVector, so that a line is one or two 16-byte loads and */
/* the flat vector kernels run on 16-byte chunks; padding lanes stay zero     */
/* ------------------------------------------------------------------------- */

template<class T> struct Vec16;
template<> struct Vec16<float>  { typedef float4  type; static constexpr int n = 4; };
template<> struct Vec16<double> { typedef double2 type; static constexpr int n = 2; };

template<class T> __device__ __forceinline__ T lane(const typename Vec16<T>::type &v, int i)
{
   return reinterpret_cast<const T *>(&v)[i];
}

/* dot of two 16-byte chunks in their own precision */
template<class T> __device__ __forceinline__ T dot16(const typename Vec16<T>::type &a,
                                                     const typename Vec16<T>::type &b)
{
   T s = (T)0;
#pragma unroll
   for(int i=0;i<Vec16<T>::n;i++)
      s = fma(lane<T>(a, i), lane<T>(b, i), s);
   return s;
}

/* per-thread dot accumulator.  FP64 vectors add in FP64.  FP32 vectors add
   into an error-free TwoSum pair in FP32 and convert once at the end: a
   conversion and an FP64 add per element would put the FP64 pipe, a small
   fraction of the FP32 rate on this part, on the per-element path (it made
   the FP32 SpMV and update kernels 25-50 % slower than their memory time). */
template<class T> struct SvAcc;
template<> struct SvAcc<double>
{
   double s = 0.;
   __device__ __forceinline__ void add(double v) { s += v; }
   __device__ __forceinline__ double get() const { return s; }
};
template<> struct SvAcc<float>
{
   float s = 0.f, c = 0.f;
   __device__ __forceinline__ void add(float v)
   {
      const float t = s + v, bp = t - s;
      c += (s - (t - bp)) + (v - bp);
      s = t;
   }
   __device__ __forceinline__ double get() const { return (double)s + (double)c; }
};

template<class VT>
__global__ void __launch_bounds__(SV_THREADS)
sv_init_kernel(size_t n, int B, int VS, const double *__restrict__ bsrc,
               double *__restrict__ b64, VT *__restrict__ x, VT *__restrict__ r,
               VT *__restrict__ p, double *part, GmdSvScal *sc, double tol2, int maxit)
{
   double acc = 0., tot;
   for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<n;i+=(size_t)gridDim.x*blockDim.x)
   {
      const double v = (int)(i % (size_t)VS) < B ? bsrc[i] : 0.;   /* padding lanes are zero */
      if(b64) b64[i] = v;
      x[i] = (VT)0;
      r[i] = (VT)v;
      p[i] = (VT)v;
      acc += v * v;
   }
   if(sv_grid_sum(acc, part, sc, &tot))
   {
      sc->bb = tot;
      sc->rr = tot;
      sc->rt = tot;
      sc->beta = 0.;
      sc->stop = tol2 * tot;
      sc->it = 0;
      sc->maxit = maxit;
      sc->done = tot > 0. ? 0 : 1;
   }
}

/* line c of a vector, VS scalars gathered with 16-byte loads */
template<int VS, class T>
__device__ __forceinline__ void sv_load_line(const T *__restrict__ v, size_t c, T out[VS])
{
   typedef typename Vec16<T>::type V;
   const V *vp = reinterpret_cast<const V *>(v + c * VS);
#pragma unroll
   for(int u=0;u<VS/Vec16<T>::n;u++)
   {
      const V t = __ldg(vp + u);
#pragma unroll
      for(int i=0;i<Vec16<T>::n;i++)
         out[ u * Vec16<T>::n + i ] = lane<T>(t, i);
   }
}

/* the x lines of a product: a plain vector, or the CG direction formed on the
   fly, p = r + beta p_old, one FMA per scalar (the same expression wherever a
   line is formed, so every thread sees the same p) */
template<int VS, class T> struct SvPlain
{
   const T *__restrict__ x;
   __device__ __forceinline__ void operator()(size_t c, T out[VS]) const
   {
      sv_load_line<VS, T>(x, c, out);
   }
};

template<int VS, class T> struct SvDirection
{
   const T *__restrict__ r;
   const T *__restrict__ p;
   T beta;
   __device__ __forceinline__ void operator()(size_t c, T out[VS]) const
   {
      T rl[VS], pl[VS];
      sv_load_line<VS, T>(r, c, rl);
      sv_load_line<VS, T>(p, c, pl);
#pragma unroll
      for(int i=0;i<VS;i++)
         out[i] = fma(beta, pl[i], rl[i]);
   }
};

/* y = A x for the block row r (one thread per row); F fetches x lines */
template<int B, int VS, class T, class F>
__device__ __forceinline__ void sv_row_product(int r, const int64_t *__restrict__ soff,
                                               const int *__restrict__ deg,
                                               const int *__restrict__ col,
                                               const T *__restrict__ val,
                                               const F &fetch, T y[VS])
{
   const int lane_ = r & 31;
   const int64_t base = __ldg(&soff[ r >> 5 ]);
   const int d = __ldg(&deg[r]);
   const int *cp = col + base * 32 + lane_;
   const T *vp = val + base * (B * B * 32) + lane_;
#pragma unroll
   for(int i=0;i<VS;i++)
      y[i] = (T)0;
#pragma unroll kSpmvUnroll
   for(int k=0;k<d;k++)
   {
      const int c = SPMV_LDM(cp + (size_t)k * 32);
      T xv[VS];
      fetch((size_t)c, xv);
      const T *blk = vp + (size_t)k * (B * B * 32);
#pragma unroll
      for(int i=0;i<B;i++)
#pragma unroll
         for(int j=0;j<B;j++)
            y[i] += SPMV_LDM(blk + (i * B + j) * 32) * xv[j];
   }
}

/* ------------------------------------------------------------------------- */
/* per-block dot partials handed from the SpMV to the update kernel: a       */
/* TwoSum pair for FP32, a double for FP64.  The update kernel folds them in  */
/* every block (same order, same result everywhere), so the SpMV needs no     */
/* grid-wide ticket: its blocks end without a fence or an atomic.             */
/* ------------------------------------------------------------------------- */

template<class T> struct SvPart;
template<> struct SvPart<float>  { typedef float2 type; };
template<> struct SvPart<double> { typedef double type; };

/* sum of two unevaluated float pairs, renormalised (TwoSum of the leading
   parts, trailing parts added to the error) */
__device__ __forceinline__ float2 sv_pair_add(float2 a, float2 b)
{
   const float s = a.x + b.x, bp = s - a.x;
   const float e = ((a.x - (s - bp)) + (b.x - bp)) + (a.y + b.y);
   const float h = s + e;
   return make_float2(h, e - (h - s));
}

__device__ __forceinline__ float2 sv_part_zero(float2) { return make_float2(0.f, 0.f); }
__device__ __forceinline__ double sv_part_zero(double) { return 0.; }
__device__ __forceinline__ float2 sv_part_add(float2 a, float2 b) { return sv_pair_add(a, b); }
__device__ __forceinline__ double sv_part_add(double a, double b) { return a + b; }
__device__ __forceinline__ float2 sv_part_of(const SvAcc<float> &a) { return make_float2(a.s, a.c); }
__device__ __forceinline__ double sv_part_of(const SvAcc<double> &a) { return a.s; }
__device__ __forceinline__ double sv_part_value(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ double sv_part_value(double a) { return a; }
__device__ __forceinline__ float2 sv_shfl_down(float2 v, int o)
{
   return make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ double sv_shfl_down(double v, int o)
{
   return __shfl_down_sync(0xffffffffu, v, o);
}

/* block fold of one partial per thread, fixed tree; result in thread 0 */
template<class P> __device__ __forceinline__ P sv_block_part(P v)
{
   __shared__ P sh[SV_THREADS / 32];
   const int lane_ = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
   for(int o=16;o>0;o>>=1)
      v = sv_part_add(v, sv_shfl_down(v, o));
   __syncthreads();
   if(lane_ == 0)
      sh[wid] = v;
   __syncthreads();
   if(wid == 0)
   {
      v = lane_ < SV_THREADS / 32 ? sh[lane_] : sv_part_zero(v);
#pragma unroll
      for(int o=16;o>0;o>>=1)
         v = sv_part_add(v, sv_shfl_down(v, o));
   }
   return v;
}

/* the value of np partials, folded in a fixed order, in every thread */
template<class P> __device__ __forceinline__ double sv_fold_parts(const P *__restrict__ part, int np)
{
   __shared__ double val;
   P a = sv_part_zero(P()), b = sv_part_zero(P());
   int i = threadIdx.x;
   for(;i+SV_THREADS<np;i+=2*SV_THREADS)
   {
      a = sv_part_add(a, __ldg(part + i));
      b = sv_part_add(b, __ldg(part + i + SV_THREADS));
   }
   if(i < np)
      a = sv_part_add(a, __ldg(part + i));
   a = sv_block_part(sv_part_add(a, b));
   if(threadIdx.x == 0)
      val = sv_part_value(a);
   __syncthreads();
   return val;
}

/* q = A p for every row.  FP32: the block partials of p.q in spart; FP64:
   p.q folded by the last block into sc->pq.  FUSE:
   p = r + beta p_old is formed on the fly from r and p_old and written to
   pn (the CG direction update needs no pass of its own). */
template<int B, int VS, class T, bool FUSE>
__global__ void __launch_bounds__(SV_THREADS)
sv_spmv_kernel(int nrow, const int64_t *__restrict__ soff, const int *__restrict__ deg,
               const int *__restrict__ col, const T *__restrict__ val,
               const T *__restrict__ r, const T *__restrict__ p, T *__restrict__ pn,
               T *__restrict__ q, typename SvPart<T>::type *spart, GmdSvScal *sc)
{
   typedef typename Vec16<T>::type V;
   constexpr int NV = VS / Vec16<T>::n;
   SvAcc<T> acc;
   if(sv_stopped(sc))
      return;
   const T beta = FUSE ? (T)sc->beta : (T)0;
   for(int row=blockIdx.x*blockDim.x+threadIdx.x;row<nrow;row+=gridDim.x*blockDim.x)
   {
      T y[VS], pr[VS];
      if(FUSE)
      {
         const SvDirection<VS, T> f = {r, p, beta};
         sv_row_product<B, VS, T>(row, soff, deg, col, val, f, y);
         f((size_t)row, pr);
      }
      else
      {
         const SvPlain<VS, T> f = {p};
         sv_row_product<B, VS, T>(row, soff, deg, col, val, f, y);
         f((size_t)row, pr);
      }
      V *qp = reinterpret_cast<V *>(q + (size_t)row * VS);
      V *pp = reinterpret_cast<V *>(pn + (size_t)row * VS);
#pragma unroll
      for(int u=0;u<NV;u++)
      {
         V t, w;
#pragma unroll
         for(int i=0;i<Vec16<T>::n;i++)
         {
            reinterpret_cast<T *>(&t)[i] = y[ u * Vec16<T>::n + i ];
            reinterpret_cast<T *>(&w)[i] = pr[ u * Vec16<T>::n + i ];
         }
         qp[u] = t;
         if(FUSE)
            pp[u] = w;
         acc.add(dot16<T>(w, t));
      }
   }
   if constexpr(sizeof(T) == 8)
   {
      /* FP64: this kernel is bound by the FP64 pipe, which hides a grid-wide
         fold at its end, while a fold of every partial in each block of the
         update kernel would cost that kernel ~25 %; pq goes to the scalars */
      double tot;
      if(sv_grid_sum(acc.get(), spart, sc, &tot))
         sc->pq = tot;
   }
   else
   {
      const typename SvPart<T>::type v = sv_block_part(sv_part_of(acc));
      if(threadIdx.x == 0)
         spart[ blockIdx.x ] = v;
   }
}

/* pq = the folded SpMV partials, alpha = rr / pq, x += alpha p, r -= alpha
   q and |r|^2; the last block sets beta, rr and the stop flag (or the
   breakdown flag when pq <= 0, with x and r left unchanged) */
template<class T>
__global__ void __launch_bounds__(SV_THREADS)
sv_update_kernel(size_t n, T *__restrict__ x, T *__restrict__ r, const T *__restrict__ p,
                 const T *__restrict__ q, const typename SvPart<T>::type *__restrict__ spart,
                 int nsp, double *part, GmdSvScal *sc)
{
   typedef typename Vec16<T>::type V;
   const size_t nv = n / Vec16<T>::n;
   SvAcc<T> acc;
   double tot;
   if(sv_stopped(sc))
      return;
   const double pq = nsp ? sv_fold_parts(spart, nsp) : sc->pq;
   const double al = pq > 0. ? sc->rr / pq : 0.;
   const T a = (T)al;
   V *xv = reinterpret_cast<V *>(x), *rv = reinterpret_cast<V *>(r);
   const V *pv = reinterpret_cast<const V *>(p), *qv = reinterpret_cast<const V *>(q);
   if(pq > 0.)
      for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<nv;i+=(size_t)gridDim.x*blockDim.x)
      {
         V xx = xv[i], rr = rv[i];
         const V pp = pv[i], qq = qv[i];
#pragma unroll
         for(int k=0;k<Vec16<T>::n;k++)
         {
            reinterpret_cast<T *>(&xx)[k] += a * lane<T>(pp, k);
            reinterpret_cast<T *>(&rr)[k] -= a * lane<T>(qq, k);
         }
         xv[i] = xx;
         rv[i] = rr;
         acc.add(dot16<T>(rr, rr));
      }
   if(sv_grid_sum(acc.get(), part, sc, &tot))
   {
      sc->pq = pq;
      sc->alpha = al;
      if(!(pq > 0.))
      {
         sc->done = 2;
         return;
      }
      sc->beta = tot / sc->rr;
      sc->rr = tot;
      sc->it += 1;
      if(tot <= sc->stop || sc->it >= sc->maxit)
         sc->done = 1;
   }
}

template<class T>
__global__ void __launch_bounds__(SV_THREADS)
sv_dir_kernel(size_t n, T *__restrict__ p, const T *__restrict__ r, const GmdSvScal *sc)
{
   typedef typename Vec16<T>::type V;
   const size_t nv = n / Vec16<T>::n;
   if(sv_stopped(sc))
      return;
   const T b = (T)sc->beta;
   V *pv = reinterpret_cast<V *>(p);
   const V *rv = reinterpret_cast<const V *>(r);
   for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<nv;i+=(size_t)gridDim.x*blockDim.x)
   {
      V pp = pv[i];
      const V rr = rv[i];
#pragma unroll
      for(int k=0;k<Vec16<T>::n;k++)
         reinterpret_cast<T *>(&pp)[k] = lane<T>(rr, k) + b * lane<T>(pp, k);
      pv[i] = pp;
   }
}

template<int B, int VS>
__global__ void __launch_bounds__(SV_THREADS)
sv_residual_kernel(int nrow, const int64_t *__restrict__ soff, const int *__restrict__ deg,
                   const int *__restrict__ col, const double *__restrict__ val,
                   const double *__restrict__ b, const double *__restrict__ x,
                   double *__restrict__ res, double *part, GmdSvScal *sc)
{
   double acc = 0., tot;
   for(int r=blockIdx.x*blockDim.x+threadIdx.x;r<nrow;r+=gridDim.x*blockDim.x)
   {
      double y[VS];
      const SvPlain<VS, double> f = {x};
      sv_row_product<B, VS, double>(r, soff, deg, col, val, f, y);
#pragma unroll
      for(int i=0;i<VS;i++)
      {
         const double v = i < B ? __ldg(&b[ (size_t)r * VS + i ]) - y[i] : 0.;
         res[ (size_t)r * VS + i ] = v;
         acc += v * v;
      }
   }
   if(sv_grid_sum(acc, part, sc, &tot))
      sc->rt = tot;
}

__global__ void __launch_bounds__(SV_THREADS)
sv_ir_begin_kernel(size_t n, const double *__restrict__ r64, float *__restrict__ r32,
                   float *__restrict__ p32, float *__restrict__ d32, double *part,
                   GmdSvScal *sc, double tin2, int maxit)
{
   SvAcc<float> acc;
   double tot;
   const double rt = sc->rt;
   const double s = rt > 0. ? 1.0 / sqrt(rt) : 0.;
   for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<n;i+=(size_t)gridDim.x*blockDim.x)
   {
      const float v = (float)(r64[i] * s);
      r32[i] = v;
      p32[i] = v;
      d32[i] = 0.f;
      acc.add(v * v);
   }
   if(sv_grid_sum(acc.get(), part, sc, &tot))
   {
      sc->rr = tot;
      sc->beta = 0.;
      sc->stop = tin2 * tot;
      sc->it = 0;
      sc->maxit = maxit;
      sc->done = tot > 0. ? 0 : 1;
   }
}

__global__ void __launch_bounds__(SV_THREADS)
sv_ir_end_kernel(size_t n, double *__restrict__ x64, const float *__restrict__ d32,
                 const GmdSvScal *sc)
{
   const double s = sqrt(sc->rt);
   for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<n;i+=(size_t)gridDim.x*blockDim.x)
      x64[i] += s * (double)d32[i];
}

__global__ void __launch_bounds__(SV_THREADS)
sv_to_f32_kernel(const double *__restrict__ src, float *__restrict__ dst, size_t n)
{
   for(size_t i=(size_t)blockIdx.x*blockDim.x+threadIdx.x;i<n;i+=(size_t)gridDim.x*blockDim.x)
      dst[i] = (float)src[i];
}

/* ------------------------------------------------------------------------- */
/* host wrappers                                                              */
/* ------------------------------------------------------------------------- */

static int sv_ok(void)
{
   return cudaGetLastError() == cudaSuccess;
}

/* resident blocks per SM of a kernel at SV_THREADS threads (8 if the query
   fails) */
static int sv_occupancy(const void *fn)
{
   int per = 0;
   if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, SV_THREADS, 0) != cudaSuccess
   || per < 1)
   {
      cudaGetLastError();
      per = 8;
   }
   return per;
}

/* flat kernels: grid-stride over one wave of resident blocks (per = blocks
   per SM), so that no second partial wave leaves SMs idle */
static unsigned sv_flat_grid(GmdCtx *ctx, size_t n, int per = 8)
{
   size_t g = (n + SV_THREADS - 1) / SV_THREADS, cap = (size_t)per * gmd_num_sms(ctx);
   if(g > cap) g = cap;
   if(g > GMD_SV_MAXBLK) g = GMD_SV_MAXBLK;
   return (unsigned)(g ? g : 1);
}

/* the occupancy of each iteration kernel, queried once (thread-safe statics) */
template<class T> static int sv_update_occ(void)
{
   static const int per = sv_occupancy((const void *)sv_update_kernel<T>);
   return per;
}

template<class T> static int sv_dir_occ(void)
{
   static const int per = sv_occupancy((const void *)sv_dir_kernel<T>);
   return per;
}

/* row kernels: one thread per block row */
static unsigned sv_row_grid(int nrow)
{
   long long g = ((long long)nrow + SV_THREADS - 1) / SV_THREADS;
   if(g > GMD_SV_MAXBLK) g = GMD_SV_MAXBLK;
   return (unsigned)(g < 1 ? 1 : g);
}

extern "C" int gmd_sv_lanes(int B)
{
   return B <= 4 ? 4 : 8;
}

extern "C" int gmd_sv_init(GmdCtx *ctx, size_t n, int B, const double *bsrc, double *b64,
                           void *x, void *r, void *p, int fltsiz, double *part, GmdSvScal *sc,
                           double tol2, int maxit)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const unsigned g = sv_flat_grid(ctx, n);
   const int vs = gmd_sv_lanes(B);
   if(fltsiz == 8)
      sv_init_kernel<double><<<g, SV_THREADS, 0, st>>>(n, B, vs, bsrc, b64, (double *)x,
         (double *)r, (double *)p, part, sc, tol2, maxit);
   else
      sv_init_kernel<float><<<g, SV_THREADS, 0, st>>>(n, B, vs, bsrc, b64, (float *)x,
         (float *)r, (float *)p, part, sc, tol2, maxit);
   return sv_ok();
}

template<int B, int VS, class T>
static void sv_spmv_launch(cudaStream_t st, const GmlSellDev *A, const void *r, const void *p,
                           void *pn, void *q, void *spart, GmdSvScal *sc)
{
   typedef typename SvPart<T>::type P;
   const unsigned g = sv_row_grid(A->NmbLin);
   if(r)
      sv_spmv_kernel<B, VS, T, true><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
         A->Col, (const T *)A->Val, (const T *)r, (const T *)p, (T *)pn, (T *)q, (P *)spart, sc);
   else
      sv_spmv_kernel<B, VS, T, false><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
         A->Col, (const T *)A->Val, NULL, (const T *)p, NULL, (T *)q, (P *)spart, sc);
}

template<class T>
static int sv_spmv_t(cudaStream_t st, const GmlSellDev *A, const void *r, const void *p,
                     void *pn, void *q, void *spart, GmdSvScal *sc)
{
   switch(A->BlkSiz)
   {
      case 3: sv_spmv_launch<3, 4, T>(st, A, r, p, pn, q, spart, sc); break;
      case 4: sv_spmv_launch<4, 4, T>(st, A, r, p, pn, q, spart, sc); break;
      case 5: sv_spmv_launch<5, 8, T>(st, A, r, p, pn, q, spart, sc); break;
      case 7: sv_spmv_launch<7, 8, T>(st, A, r, p, pn, q, spart, sc); break;
      default: return 0;
   }
   return sv_ok();
}

extern "C" int gmd_sv_spmv_blocks(int nrow)
{
   return (int)sv_row_grid(nrow);
}

extern "C" int gmd_sv_spmv(GmdCtx *ctx, const GmlSellDev *A, const void *r, const void *p,
                           void *pn, void *q, void *spart, GmdSvScal *sc)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if((r == NULL) != (pn == NULL))
      return 0;
   return A->FltSiz == 8 ? sv_spmv_t<double>(st, A, r, p, pn, q, spart, sc)
                         : sv_spmv_t<float>(st, A, r, p, pn, q, spart, sc);
}

extern "C" int gmd_sv_update(GmdCtx *ctx, int fltsiz, size_t n, void *x, void *r,
                             const void *p, const void *q, const void *spart, int nsp,
                             double *part, GmdSvScal *sc)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if(nsp < 0 || nsp > GMD_SV_MAXBLK)
      return 0;
   if(fltsiz == 8)
      sv_update_kernel<double><<<sv_flat_grid(ctx, n / 2, sv_update_occ<double>()), SV_THREADS,
         0, st>>>(n, (double *)x, (double *)r, (const double *)p, (const double *)q,
                  (const double *)spart, nsp, part, sc);
   else
      sv_update_kernel<float><<<sv_flat_grid(ctx, n / 4, sv_update_occ<float>()), SV_THREADS,
         0, st>>>(n, (float *)x, (float *)r, (const float *)p, (const float *)q,
                  (const float2 *)spart, nsp, part, sc);
   return sv_ok();
}

extern "C" int gmd_sv_dir(GmdCtx *ctx, int fltsiz, size_t n, void *p, const void *r,
                          GmdSvScal *sc)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if(fltsiz == 8)
      sv_dir_kernel<double><<<sv_flat_grid(ctx, n / 2, sv_dir_occ<double>()), SV_THREADS, 0, st>>>(n, (double *)p,
         (const double *)r, sc);
   else
      sv_dir_kernel<float><<<sv_flat_grid(ctx, n / 4, sv_dir_occ<float>()), SV_THREADS, 0, st>>>(n, (float *)p,
         (const float *)r, sc);
   return sv_ok();
}

extern "C" int gmd_sv_residual(GmdCtx *ctx, const GmlSellDev *A, const double *b,
                               const double *x, double *r, double *part, GmdSvScal *sc)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const double *val = (const double *)A->Val;
   const unsigned g = sv_row_grid(A->NmbLin);
   if(A->FltSiz != 8)
      return 0;
   switch(A->BlkSiz)
   {
      case 3: sv_residual_kernel<3, 4><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
                 A->Col, val, b, x, r, part, sc); break;
      case 4: sv_residual_kernel<4, 4><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
                 A->Col, val, b, x, r, part, sc); break;
      case 5: sv_residual_kernel<5, 8><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
                 A->Col, val, b, x, r, part, sc); break;
      case 7: sv_residual_kernel<7, 8><<<g, SV_THREADS, 0, st>>>(A->NmbLin, A->SlcOff, A->Deg,
                 A->Col, val, b, x, r, part, sc); break;
      default: return 0;
   }
   return sv_ok();
}

extern "C" int gmd_sv_ir_begin(GmdCtx *ctx, size_t n, const double *r64, float *r32, float *p32,
                               float *d32, double *part, GmdSvScal *sc, double tin2, int maxit)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   sv_ir_begin_kernel<<<sv_flat_grid(ctx, n), SV_THREADS, 0, st>>>(n, r64, r32, p32, d32, part,
      sc, tin2, maxit);
   return sv_ok();
}

extern "C" int gmd_sv_ir_end(GmdCtx *ctx, size_t n, double *x64, const float *d32, GmdSvScal *sc)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   sv_ir_end_kernel<<<sv_flat_grid(ctx, n), SV_THREADS, 0, st>>>(n, x64, d32, sc);
   return sv_ok();
}

extern "C" int gmd_sv_to_f32(GmdCtx *ctx, const double *src, float *dst, size_t n)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   sv_to_f32_kernel<<<sv_flat_grid(ctx, n), SV_THREADS, 0, st>>>(src, dst, n);
   return sv_ok();
}
