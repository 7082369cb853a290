/*
 * gml_scan.cu -- exclusive prefix sums of int and long long arrays on the
 * device, used by the setup paths (vertex -> tet offsets, slice offsets of
 * the SELL layouts).
 *
 * Three launches, each reading and writing the array once:
 *   1. every block of 1024 threads sums a tile of SC_ITEMS x 1024 entries;
 *   2. one block scans the tile sums (loops when there are more than 1024);
 *   3. every block rescans its tile from its offset and writes the result.
 * out has n + 1 entries; out[n] is the total.  in and out may not alias.
 */
#include <cuda_runtime.h>
#include "gml_device.h"

#define SC_THREADS 1024
#define SC_ITEMS   8
#define SC_TILE    (SC_THREADS * SC_ITEMS)

template<class T> __device__ __forceinline__ T sc_warp_incl(T v)
{
   const int lane = threadIdx.x & 31;
   for(int o=1;o<32;o<<=1)
   {
      T y = __shfl_up_sync(0xffffffffu, v, o);
      if(lane >= o) v += y;
   }
   return v;
}

/* exclusive scan of one value per thread over the block; *total = sum */
template<class T> __device__ __forceinline__ T sc_block_excl(T v, T *total)
{
   __shared__ T wsum[32];
   const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
   T s = sc_warp_incl(v);
   __syncthreads();
   if(lane == 31) wsum[w] = s;
   __syncthreads();
   if(w == 0)
   {
      T x = lane < (int)(blockDim.x >> 5) ? wsum[lane] : (T)0;
      T t = sc_warp_incl(x);
      wsum[lane] = t - x;
      if(lane == 31)
         *total = t;                     /* lane 31 holds the block total */
   }
   __syncthreads();
   return wsum[w] + s - v;
}

template<class T>
__global__ void __launch_bounds__(SC_THREADS) sc_tile_sum(const T *__restrict__ in, int n, T *bsum)
{
   __shared__ T tot;
   const long long base = (long long)blockIdx.x * SC_TILE;
   T s = 0;
#pragma unroll
   for(int k=0;k<SC_ITEMS;k++)
   {
      const long long i = base + (long long)k * SC_THREADS + threadIdx.x;
      if(i < n) s += in[i];
   }
   sc_block_excl(s, &tot);
   __syncthreads();
   if(threadIdx.x == 0)
      bsum[blockIdx.x] = tot;
}

template<class T>
__global__ void __launch_bounds__(SC_THREADS) sc_scan_sums(T *bsum, int nb, T *out_total)
{
   __shared__ T tot, carry;
   if(threadIdx.x == 0)
      carry = 0;
   __syncthreads();
   for(int b0=0;b0<nb;b0+=SC_THREADS)
   {
      const int i = b0 + threadIdx.x;
      const T v = i < nb ? bsum[i] : (T)0;
      const T e = sc_block_excl(v, &tot);
      __syncthreads();
      if(i < nb) bsum[i] = carry + e;
      __syncthreads();
      if(threadIdx.x == 0) carry += tot;
      __syncthreads();
   }
   if(threadIdx.x == 0)
      *out_total = carry;
}

/* rescan: thread t owns entries base + t*SC_ITEMS .. + SC_ITEMS - 1 */
template<class T>
__global__ void __launch_bounds__(SC_THREADS) sc_tile_scan(const T *__restrict__ in, T *out, int n,
                                                           const T *bsum)
{
   __shared__ T tot;
   const long long base = (long long)blockIdx.x * SC_TILE + (long long)threadIdx.x * SC_ITEMS;
   T v[SC_ITEMS], s = 0;
#pragma unroll
   for(int k=0;k<SC_ITEMS;k++)
   {
      v[k] = base + k < n ? in[base + k] : (T)0;
      s += v[k];
   }
   T e = sc_block_excl(s, &tot) + bsum[blockIdx.x];
#pragma unroll
   for(int k=0;k<SC_ITEMS;k++)
   {
      if(base + k < n) out[base + k] = e;
      e += v[k];
   }
}

template<class T>
static int sc_run(GmdCtx *ctx, const T *in, T *out, int n, T *scratch)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const int nb = (n + SC_TILE - 1) / SC_TILE;
   if(n <= 0)
      return cudaMemsetAsync(out, 0, sizeof(T), st) == cudaSuccess;
   sc_tile_sum<T><<<nb, SC_THREADS, 0, st>>>(in, n, scratch);
   sc_scan_sums<T><<<1, SC_THREADS, 0, st>>>(scratch, nb, out + n);
   sc_tile_scan<T><<<nb, SC_THREADS, 0, st>>>(in, out, n, scratch);
   return cudaGetLastError() == cudaSuccess;
}

/* the tile sums live in stream-ordered scratch (no device-wide sync) */
template<class T>
static int sc_alloc_run(GmdCtx *ctx, const T *in, T *out, int n)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const size_t bytes = (size_t)((n + SC_TILE - 1) / SC_TILE + 1) * sizeof(T);
   void *scr = NULL;
   int ok;
   if(cudaMallocAsync(&scr, bytes, st) != cudaSuccess)
      return 0;
   ok = sc_run<T>(ctx, in, out, n, (T *)scr);
   return (cudaFreeAsync(scr, st) == cudaSuccess) && ok;
}

extern "C" int gmd_scan_excl_i32(GmdCtx *ctx, const int *in, int *out, int n)
{
   return sc_alloc_run<int>(ctx, in, out, n);
}

extern "C" int gmd_scan_excl_i64(GmdCtx *ctx, const long long *in, long long *out, int n)
{
   return sc_alloc_run<long long>(ctx, in, out, n);
}
