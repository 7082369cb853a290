/*
 * gml_reduce.cu -- single-pass reductions of a float field.
 *
 * Replaces the reference's reduce.cl kernels (sources/reduce.cl:6-137) and the
 * serial CPU finish of GmlReduceVector (sources/gmlib3.c:3297-3327).  The
 * reference reduces each work-group in __local memory, downloads one partial
 * per group and finishes on the host in float, dropping the last partial
 * group when the line count is not a multiple of the group size (:3299).
 * Here one launch does everything:
 *
 *   - each thread streams float4 chunks (grid-stride, 16-byte loads) and
 *     accumulates sums with an error-free TwoSum pair in FP32, so the FP64
 *     units (a small fraction of FP32 throughput on this part) are not on the
 *     per-element path;
 *   - the warp folds with __shfl_xor_sync, the block through shared memory,
 *     and the block result is stored in FP64;
 *   - the last block to finish (ticket counter) folds the block results in
 *     FP64 and writes the final value, then re-arms the counter.
 *
 * Operations (enum reduction_opp of gmlib3.h): Min, Max, Sum, L0 (number of
 * non-zero values), L1 (sum of |x|), L2 (sum of x^2, no square root, as the
 * reference), Linf (max |x|).
 *
 * Scratch layout of gml_reduce_f32_kernel (device, bytes): [0,8) ticket
 * counter, [8,16) result, [16, 16 + 8*nblk) per-block partials (one double
 * each).  gml_minmax_arg_kernel has its own layout (see there).
 *
 * Line indices are 64-bit inside the kernels: with up to 2^31 - 1 lines, a
 * grid-stride index can pass INT_MAX on its last step.
 */
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <mutex>
#include "gml_device.h"
#include "gmlib3_gb300.h"

#define RED_THREADS 512
#define RED_MAXBLK  1024

struct GmdCtx;   /* opaque here; stream obtained through gmd_stream */

__device__ __forceinline__ void two_sum(float &s, float &c, float x)
{
   float t = s + x;
   float bp = t - s;
   c += (s - (t - bp)) + (x - bp);
   s = t;
}

template<int OP> __device__ __forceinline__ void red_elem(float x, float &s, float &c)
{
   if(OP == 0)      s = fminf(s, x);
   else if(OP == 1) s = fmaxf(s, x);
   else if(OP == 2) two_sum(s, c, x);
   else if(OP == 3) s += (x != 0.0f) ? 1.0f : 0.0f;      /* counts stay exact below 2^24 per thread */
   else if(OP == 4) two_sum(s, c, fabsf(x));
   else if(OP == 5) two_sum(s, c, x * x);
   else             s = fmaxf(s, fabsf(x));
}

template<int OP> __device__ __forceinline__ double red_join(double a, double b)
{
   if(OP == 0) return fmin(a, b);
   if(OP == 1 || OP == 6) return fmax(a, b);
   return a + b;
}

template<int OP> __device__ __forceinline__ float red_init()
{
   if(OP == 0) return FLT_MAX;
   if(OP == 1) return -FLT_MAX;
   return 0.0f;
}

template<int OP>
__global__ void __launch_bounds__(RED_THREADS)
gml_reduce_f32_kernel(const float *__restrict__ in, int n, unsigned long long *scratch)
{
   unsigned long long *ticket = scratch;
   double *result  = (double *)(scratch + 1);
   double *partial = (double *)(scratch + 2);
   __shared__ double sh[ RED_THREADS / 32 ];
   __shared__ int last;

   float s = red_init<OP>(), c = 0.0f;
   const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
   const long long nth = (long long)gridDim.x * blockDim.x;
   const long long n4 = ((((uintptr_t)in) & 15) == 0) ? (long long)(n >> 2) : 0;
   const float4 *in4 = (const float4 *)in;

   for(long long i=tid;i<n4;i+=nth)
   {
      float4 v = __ldg(&in4[i]);
      red_elem<OP>(v.x, s, c); red_elem<OP>(v.y, s, c);
      red_elem<OP>(v.z, s, c); red_elem<OP>(v.w, s, c);
   }
   for(long long i=4*n4+tid;i<n;i+=nth)
      red_elem<OP>(__ldg(&in[i]), s, c);

   double d = (double)s + (double)c;
   for(int o=16;o>0;o>>=1)
      d = red_join<OP>(d, __shfl_xor_sync(0xffffffffu, d, o));
   if((threadIdx.x & 31) == 0)
      sh[ threadIdx.x >> 5 ] = d;
   __syncthreads();
   if(threadIdx.x < 32)
   {
      d = threadIdx.x < (blockDim.x >> 5) ? sh[ threadIdx.x ] : (double)red_init<OP>();
      for(int o=16;o>0;o>>=1)
         d = red_join<OP>(d, __shfl_xor_sync(0xffffffffu, d, o));
      if(threadIdx.x == 0)
      {
         partial[ blockIdx.x ] = d;
         __threadfence();
         last = (atomicAdd(ticket, 1ULL) == (unsigned long long)(gridDim.x - 1));
      }
   }
   __syncthreads();
   if(!last)
      return;

   /* last block: fold the per-block partials in FP64 */
   __threadfence();
   d = (double)red_init<OP>();
   for(int i=threadIdx.x;i<(int)gridDim.x;i+=blockDim.x)
      d = red_join<OP>(d, ((volatile double *)partial)[i]);
   for(int o=16;o>0;o>>=1)
      d = red_join<OP>(d, __shfl_xor_sync(0xffffffffu, d, o));
   if((threadIdx.x & 31) == 0)
      sh[ threadIdx.x >> 5 ] = d;
   __syncthreads();
   if(threadIdx.x == 0)
   {
      for(int w=1;w<(int)(blockDim.x >> 5);w++)
         d = red_join<OP>(d, sh[w]);
      *result = d;
      *ticket = 0ULL;
   }
}

/* ------------------------------------------------------------------------- */
/* min / argmin / max / argmax with smallest-index ties                       */
/* ------------------------------------------------------------------------- */

/* order-preserving map of a float to an unsigned key; -0 and +0 get the
   same key, so that a tie between them goes to the smallest index.  A NaN
   keeps its bit pattern's place: above +inf with the sign bit clear, below
   -inf with it set. */
__device__ __forceinline__ unsigned fkey(float f)
{
   unsigned u = __float_as_uint(f == 0.0f ? 0.0f : f);
   return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float funkey(unsigned k)
{
   return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void __launch_bounds__(RED_THREADS)
gml_minmax_arg_kernel(const float *__restrict__ in, int n, unsigned long long *scratch)
{
   /* scratch: [0] ticket, [1] min key, [2] max key (inverted), [3..] partials */
   unsigned long long *ticket = scratch;
   unsigned long long *part = scratch + 3;
   __shared__ unsigned long long shmin[ RED_THREADS / 32 ], shmax[ RED_THREADS / 32 ];
   __shared__ int last;
   unsigned long long kmin = ~0ULL, kmax = ~0ULL;
   const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
   const long long nth = (long long)gridDim.x * blockDim.x;

   for(long long i=tid;i<n;i+=nth)
   {
      unsigned k = fkey(__ldg(&in[i]));
      unsigned long long a = ((unsigned long long)k << 32) | (unsigned)i;
      unsigned long long b = ((unsigned long long)(~k) << 32) | (unsigned)i;
      kmin = a < kmin ? a : kmin;
      kmax = b < kmax ? b : kmax;
   }
   for(int o=16;o>0;o>>=1)
   {
      unsigned long long x = __shfl_xor_sync(0xffffffffu, kmin, o);
      unsigned long long y = __shfl_xor_sync(0xffffffffu, kmax, o);
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
   }
   if((threadIdx.x & 31) == 0)
   {
      shmin[ threadIdx.x >> 5 ] = kmin;
      shmax[ threadIdx.x >> 5 ] = kmax;
   }
   __syncthreads();
   if(threadIdx.x == 0)
   {
      for(int w=1;w<(int)(blockDim.x >> 5);w++)
      {
         kmin = shmin[w] < kmin ? shmin[w] : kmin;
         kmax = shmax[w] < kmax ? shmax[w] : kmax;
      }
      part[ 2 * blockIdx.x ] = kmin;
      part[ 2 * blockIdx.x + 1 ] = kmax;
      __threadfence();
      last = (atomicAdd(ticket, 1ULL) == (unsigned long long)(gridDim.x - 1));
   }
   __syncthreads();
   if(!last)
      return;
   __threadfence();
   kmin = ~0ULL; kmax = ~0ULL;
   for(int i=threadIdx.x;i<(int)gridDim.x;i+=blockDim.x)
   {
      unsigned long long x = ((volatile unsigned long long *)part)[ 2*i ];
      unsigned long long y = ((volatile unsigned long long *)part)[ 2*i+1 ];
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
   }
   for(int o=16;o>0;o>>=1)
   {
      unsigned long long x = __shfl_xor_sync(0xffffffffu, kmin, o);
      unsigned long long y = __shfl_xor_sync(0xffffffffu, kmax, o);
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
   }
   if((threadIdx.x & 31) == 0)
   {
      shmin[ threadIdx.x >> 5 ] = kmin;
      shmax[ threadIdx.x >> 5 ] = kmax;
   }
   __syncthreads();
   if(threadIdx.x == 0)
   {
      for(int w=1;w<(int)(blockDim.x >> 5);w++)
      {
         kmin = shmin[w] < kmin ? shmin[w] : kmin;
         kmax = shmax[w] < kmax ? shmax[w] : kmax;
      }
      scratch[1] = kmin;
      scratch[2] = kmax;
      *ticket = 0ULL;
   }
}

static int red_blocks(GmdCtx *ctx, int n)
{
   int nb = (n + 4 * RED_THREADS - 1) / (4 * RED_THREADS);
   int cap = 2 * gmd_num_sms(ctx);
   if(nb > cap) nb = cap;
   if(nb > RED_MAXBLK) nb = RED_MAXBLK;
   if(nb < 1) nb = 1;
   return nb;
}

extern "C" size_t gmd_reduce_scratch_bytes(int n)
{
   (void)n;
   return (size_t)(3 + 2 * RED_MAXBLK) * sizeof(unsigned long long);
}

extern "C" int gmd_reduce_f32(GmdCtx *ctx, int op, const float *in, int n, double *res,
                              void *scratch)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   unsigned long long *scr = (unsigned long long *)scratch;
   int nb = red_blocks(ctx, n);

   if(n <= 0)
   {
      *res = (op == 0) ? (double)FLT_MAX : (op == 1) ? -(double)FLT_MAX : 0.0;
      return 1;
   }

   switch(op)
   {
      case 0: gml_reduce_f32_kernel<0><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 1: gml_reduce_f32_kernel<1><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 2: gml_reduce_f32_kernel<2><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 3: gml_reduce_f32_kernel<3><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 4: gml_reduce_f32_kernel<4><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 5: gml_reduce_f32_kernel<5><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      case 6: gml_reduce_f32_kernel<6><<<nb, RED_THREADS, 0, st>>>(in, n, scr); break;
      default: return 0;
   }
   if(cudaGetLastError() != cudaSuccess)
      return 0;
   if(cudaMemcpyAsync(res, scr + 1, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return 0;
   return cudaStreamSynchronize(st) == cudaSuccess;
}

extern "C" int gmd_minmax_arg_f32(GmdCtx *ctx, const float *in, int n,
                                  float *vmin, int *imin, float *vmax, int *imax,
                                  void *scratch)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   unsigned long long *scr = (unsigned long long *)scratch, host[2];
   int nb = red_blocks(ctx, n);

   if(n <= 0)
      return 0;
   gml_minmax_arg_kernel<<<nb, RED_THREADS, 0, st>>>(in, n, scr);
   if(cudaGetLastError() != cudaSuccess)
      return 0;
   if(cudaMemcpyAsync(host, scr + 1, 2 * sizeof(unsigned long long),
                      cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return 0;
   if(cudaStreamSynchronize(st) != cudaSuccess)
      return 0;
   {
      unsigned kmin = (unsigned)(host[0] >> 32), kmax = ~(unsigned)(host[1] >> 32);
      unsigned umin = (kmin & 0x80000000u) ? (kmin & 0x7fffffffu) : ~kmin;
      unsigned umax = (kmax & 0x80000000u) ? (kmax & 0x7fffffffu) : ~kmax;
      float fmn, fmx;
      memcpy(&fmn, &umin, 4);
      memcpy(&fmx, &umax, 4);
      if(vmin) *vmin = fmn;
      if(imin) *imin = (int)(host[0] & 0xffffffffu);
      if(vmax) *vmax = fmx;
      if(imax) *imax = (int)(host[1] & 0xffffffffu);
   }
   return 1;
}

/* ------------------------------------------------------------------------- */
/* GmlxReduceNoAlloc: the reduction above with its scratch in static device   */
/* memory, for callers that cannot allocate                                   */
/* ------------------------------------------------------------------------- */

/* [0] ticket, [1] result, [2, 2 + RED_MAXBLK) per-block partials.  Static
   device storage is zero when the module loads, so the ticket starts at
   zero; every completed launch re-arms it to zero in its last block.  The
   array exists once per device: calls in flight at the same time on one
   device (two streams, or two host threads) share it and race. */
static __device__ __align__(256) unsigned long long gml_noalloc_scratch[2 + RED_MAXBLK];

#define NOALLOC_MAXDEV 64
static std::mutex noalloc_lock;
static unsigned long long *noalloc_addr[NOALLOC_MAXDEV];
static int noalloc_nsm[NOALLOC_MAXDEV];

static int noalloc_fail(const char *fmt, ...)
{
   va_list ap;
   va_start(ap, fmt);
   fprintf(stderr, "GmlxReduceNoAlloc: ");
   vfprintf(stderr, fmt, ap);
   fprintf(stderr, "\n");
   va_end(ap);
   return 0;
}

extern "C" int GmlxReduceNoAlloc(const float *DevVec, size_t NmbLin, int RedOpp,
                                 double *res, void *stream)
{
   cudaStream_t st = (cudaStream_t)stream;
   unsigned long long *scr;
   int dev = -1, nsm, nb;
   cudaError_t e;

   if(!res)
      return noalloc_fail("res is NULL");
   if(RedOpp < GmlMin || RedOpp > GmlLinf)
      return noalloc_fail("unknown reduction operation %d", RedOpp);
   if(NmbLin > (size_t)GMLX_NOALLOC_MAX_LINES)
      return noalloc_fail("%lld lines exceed the maximum of %lld",
                          (long long)NmbLin, (long long)GMLX_NOALLOC_MAX_LINES);
   if(NmbLin == 0)
   {
      *res = (RedOpp == GmlMin) ? (double)FLT_MAX : (RedOpp == GmlMax) ? -(double)FLT_MAX : 0.0;
      return 1;
   }
   if(!DevVec)
      return noalloc_fail("DevVec is NULL with %lld lines", (long long)NmbLin);

   if((e = cudaGetDevice(&dev)) != cudaSuccess)
      return noalloc_fail("cudaGetDevice failed (error %d)", (int)e);
   if(dev < 0 || dev >= NOALLOC_MAXDEV)
      return noalloc_fail("device %d is beyond the %d devices supported", dev, NOALLOC_MAXDEV);

   /* first call on this device: resolve the scratch address (with the device
      current) and the SM count; later calls read the cached values */
   {
      std::lock_guard<std::mutex> g(noalloc_lock);
      if(!noalloc_addr[dev])
      {
         void *p = NULL;
         if((e = cudaGetSymbolAddress(&p, gml_noalloc_scratch)) != cudaSuccess || !p)
            return noalloc_fail("cudaGetSymbolAddress failed on device %d (error %d)", dev, (int)e);
         if((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            return noalloc_fail("cudaDeviceGetAttribute failed on device %d (error %d)", dev, (int)e);
         noalloc_nsm[dev] = nsm;
         noalloc_addr[dev] = (unsigned long long *)p;
      }
      scr = noalloc_addr[dev];
      nsm = noalloc_nsm[dev];
   }

   {
      long long want = ((long long)NmbLin + 4 * RED_THREADS - 1) / (4 * RED_THREADS);
      long long cap = 2LL * nsm < RED_MAXBLK ? 2LL * nsm : RED_MAXBLK;
      nb = (int)(want < cap ? want : cap);
      if(nb < 1) nb = 1;
   }

   {
      const int n = (int)NmbLin;
      switch(RedOpp)
      {
         case 0: gml_reduce_f32_kernel<0><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         case 1: gml_reduce_f32_kernel<1><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         case 2: gml_reduce_f32_kernel<2><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         case 3: gml_reduce_f32_kernel<3><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         case 4: gml_reduce_f32_kernel<4><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         case 5: gml_reduce_f32_kernel<5><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
         default: gml_reduce_f32_kernel<6><<<nb, RED_THREADS, 0, st>>>(DevVec, n, scr); break;
      }
   }
   if((e = cudaGetLastError()) != cudaSuccess)
      return noalloc_fail("launch failed (error %d)", (int)e);
   if((e = cudaMemcpyAsync(res, scr + 1, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return noalloc_fail("reading the result failed (error %d)", (int)e);
   if((e = cudaStreamSynchronize(st)) != cudaSuccess)
      return noalloc_fail("stream synchronisation failed (error %d)", (int)e);
   return 1;
}
