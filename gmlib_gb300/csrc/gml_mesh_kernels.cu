/*
 * gml_mesh_kernels.cu -- native mesh kernels (no counterpart in the
 * reference API; they serve the ball-of-points smoothing and quality
 * workloads directly instead of through generated scatter/gather pairs).
 *
 * Topology (built on the GPU, deterministic):
 *   vertex -> tetrahedron CSR   count (atomics), single-block exclusive scan,
 *                               fill (atomic slots; order within a ball is
 *                               not used by the kernels below)
 *   ball of points              per vertex, the distinct vertices of its
 *                               tetrahedra, sorted ascending, stored in
 *                               SELL-32 (slices of 32 vertices, column-major,
 *                               slice width = longest ball in the slice);
 *                               fixed vertices get an empty ball
 *   boundary vertices           vertices of faces owned by a single tet
 *
 * Hot kernels (HBM-bound):
 *   laplace_sell   one Jacobi sweep x' = x + w (mean(ball) - x); per vertex
 *                  4 (degree) + 4 deg (columns, 128-byte runs per warp)
 *                  + 16 (own) + 16 (write) bytes; the neighbour gathers hit
 *                  L2 (coordinates are 16 V bytes).
 *   tet_quality    mean-ratio quality 12 (3|V|)^(2/3) / sum l^2 signed by
 *                  orientation, 64-bin histogram, min/argmin, max/argmax,
 *                  sum, inverted-element count and bit flags; 16 bytes of
 *                  connectivity per tet streamed, coordinates from L2.  The
 *                  determinant is recomputed in FP64 whenever the FP32 value
 *                  is below max(1e-6 h^3, 16 eps32 * permanent), a bound on
 *                  the FP32 error, so the orientation flags are exact.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include "gml_device.h"
#include "gml_mesh.h"

#define MK_THREADS 256

/* ========================================================================= */
/* scans (single block, chunked; used for setup-sized arrays)                 */
/* ========================================================================= */

template<class T>
__global__ void __launch_bounds__(1024) scan_excl_kernel(const T *in, T *out, int n)
{
   __shared__ T wsum[32];
   __shared__ T carry;
   int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
   if(tid == 0)
      carry = 0;
   __syncthreads();
   for(int base=0;base<n;base+=1024)
   {
      int i = base + tid;
      T x = i < n ? in[i] : (T)0, s = x;
      for(int o=1;o<32;o<<=1)
      {
         T y = __shfl_up_sync(0xffffffffu, s, o);
         if(lane >= o) s += y;
      }
      if(lane == 31) wsum[w] = s;
      __syncthreads();
      if(w == 0)
      {
         T ws = wsum[lane], t = ws;
         for(int o=1;o<32;o<<=1)
         {
            T y = __shfl_up_sync(0xffffffffu, t, o);
            if(lane >= o) t += y;
         }
         wsum[lane] = t - ws;
      }
      __syncthreads();
      T excl = carry + wsum[w] + s - x;
      if(i < n) out[i] = excl;
      __syncthreads();
      if(tid == 1023) carry = excl + x;
      __syncthreads();
   }
   if(tid == 0)
      out[n] = carry;
}

/* ========================================================================= */
/* vertex -> tet CSR                                                          */
/* ========================================================================= */

__global__ void count_vt_kernel(const int4 *__restrict__ tet, int nt, int nv, int *deg, int *err)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if(t >= nt) return;
   int4 e = tet[t];
   int v[4] = { e.x, e.y, e.z, e.w };
   for(int j=0;j<4;j++)
   {
      if(v[j] < 0 || v[j] >= nv) { atomicOr(err, 2); continue; }
      atomicAdd(&deg[ v[j] ], 1);
   }
}

__global__ void fill_vt_kernel(const int4 *__restrict__ tet, int nt, int nv, const int *ptr,
                               int *fill, int *vt)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if(t >= nt) return;
   int4 e = tet[t];
   int v[4] = { e.x, e.y, e.z, e.w };
   for(int j=0;j<4;j++)
   {
      if(v[j] < 0 || v[j] >= nv) continue;
      int p = atomicAdd(&fill[ v[j] ], 1);
      vt[ ptr[ v[j] ] + p ] = t;
   }
}

/* ========================================================================= */
/* boundary vertices: faces owned by a single tetrahedron                     */
/* ========================================================================= */

__device__ __forceinline__ int tet_has(int4 e, int v)
{
   return e.x == v || e.y == v || e.z == v || e.w == v;
}

__global__ void boundary_kernel(const int4 *__restrict__ tet, int nt, const int *__restrict__ ptr,
                                const int *__restrict__ vt, int *fixed)
{
   int t = blockIdx.x * blockDim.x + threadIdx.x;
   if(t >= nt) return;
   int4 e = tet[t];
   int v[4] = { e.x, e.y, e.z, e.w };
   for(int f=0;f<4;f++)
   {
      int a = v[(f+1)&3], b = v[(f+2)&3], c = v[(f+3)&3], shared = 0;
      /* walk the ball of the lowest-degree face vertex */
      int da = ptr[a+1] - ptr[a], db = ptr[b+1] - ptr[b], dc = ptr[c+1] - ptr[c];
      int s = a;
      if(db < da && db <= dc) s = b;
      else if(dc < da && dc < db) s = c;
      for(int k=ptr[s];k<ptr[s+1];k++)
      {
         int u = vt[k];
         if(u == t) continue;
         int4 g = tet[u];
         if(tet_has(g, a) && tet_has(g, b) && tet_has(g, c)) { shared = 1; break; }
      }
      if(!shared)
      {
         fixed[a] = 1; fixed[b] = 1; fixed[c] = 1;
      }
   }
}

/* ========================================================================= */
/* ball of points                                                             */
/* ========================================================================= */

#define PB_MAX 64

/* distinct vertices of the tets around v, ascending; returns the count or
   -1 when the ball exceeds PB_MAX */
__device__ int point_ball(int v, const int4 *__restrict__ tet, const int *__restrict__ ptr,
                          const int *__restrict__ vt, int *lst)
{
   int n = 0;
   for(int k=ptr[v];k<ptr[v+1];k++)
   {
      int4 e = tet[ vt[k] ];
      int u4[4] = { e.x, e.y, e.z, e.w };
      for(int j=0;j<4;j++)
      {
         int u = u4[j], found = 0;
         if(u == v) continue;
         for(int i=0;i<n;i++)
            if(lst[i] == u) { found = 1; break; }
         if(found) continue;
         if(n == PB_MAX) return -1;
         lst[n++] = u;
      }
   }
   for(int i=1;i<n;i++)
   {
      int x = lst[i], j = i - 1;
      while(j >= 0 && lst[j] > x) { lst[j+1] = lst[j]; j--; }
      lst[j+1] = x;
   }
   return n;
}

__global__ void point_count_kernel(int nv, const int4 *__restrict__ tet, const int *__restrict__ ptr,
                                   const int *__restrict__ vt, const int *__restrict__ fixed,
                                   int *pdeg, int *err)
{
   int v = blockIdx.x * blockDim.x + threadIdx.x;
   int lst[PB_MAX];
   if(v >= nv) return;
   if(fixed && fixed[v]) { pdeg[v] = 0; return; }
   int n = point_ball(v, tet, ptr, vt, lst);
   if(n < 0) { atomicOr(err, 1); n = 0; }
   pdeg[v] = n;
}

__global__ void slice_width_kernel(int nv, const int *__restrict__ pdeg, long long *w)
{
   int s = blockIdx.x * blockDim.x + threadIdx.x, ns = (nv + 31) / 32;
   if(s >= ns) return;
   int m = 0;
   for(int r=s*32;r<s*32+32 && r<nv;r++)
      m = max(m, pdeg[r]);
   w[s] = m;
}

__global__ void point_fill_kernel(int nv, const int4 *__restrict__ tet, const int *__restrict__ ptr,
                                  const int *__restrict__ vt, const int *__restrict__ pdeg,
                                  const long long *__restrict__ soff, int *pcol)
{
   int v = blockIdx.x * blockDim.x + threadIdx.x;
   int lst[PB_MAX];
   if(v >= nv || pdeg[v] == 0) return;
   int n = point_ball(v, tet, ptr, vt, lst);
   long long base = soff[v >> 5];
   for(int k=0;k<n && k<pdeg[v];k++)
      pcol[ (base + k) * 32 + (v & 31) ] = lst[k];
}

/* ========================================================================= */
/* Laplacian sweep over the ball of points                                    */
/* ========================================================================= */

__global__ void __launch_bounds__(MK_THREADS)
laplace_sell_kernel(int nv, const long long *__restrict__ soff, const int *__restrict__ pdeg,
                    const int *__restrict__ pcol, const float4 *__restrict__ in,
                    float4 *__restrict__ out, float omega)
{
   int v = blockIdx.x * blockDim.x + threadIdx.x;
   if(v >= nv) return;
   const int d = __ldg(&pdeg[v]);
   const float4 p = __ldg(&in[v]);
   if(d == 0)
   {
      out[v] = p;
      return;
   }
   const int *cp = pcol + __ldg(&soff[v >> 5]) * 32 + (v & 31);
   float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll 4
   for(int k=0;k<d;k++)
   {
      const int c = __ldg(cp + (size_t)k * 32);
      const float4 q = __ldg(&in[c]);
      sx += q.x; sy += q.y; sz += q.z;
   }
   const float inv = 1.0f / (float)d;
   out[v] = make_float4(p.x + omega * (sx * inv - p.x), p.y + omega * (sy * inv - p.y),
                        p.z + omega * (sz * inv - p.z), 0.f);
}

/* ========================================================================= */
/* mean-ratio quality, histogram, extrema, inverted flags                     */
/* ========================================================================= */

__device__ __forceinline__ unsigned mk_fkey(float f)
{
   unsigned u = __float_as_uint(f);
   return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void stats_init_kernel(GmlxQualStats *st, int n)
{
   int i = blockIdx.x * blockDim.x + threadIdx.x;
   if(i >= n) return;
   GmlxQualStats *s = st + i;
   s->MinKey = ~0ULL;
   s->MaxKey = ~0ULL;
   s->Sum = 0.;
   s->NmbInv = 0;
   s->NmbF64 = 0;
   for(int b=0;b<64;b++)
      s->Hist[b] = 0;
}

__global__ void __launch_bounds__(MK_THREADS)
tet_quality_kernel(int nt, const int4 *__restrict__ tet, const float4 *__restrict__ crd,
                   float thr, float *__restrict__ qout, unsigned *__restrict__ flags,
                   GmlxQualStats *st)
{
   __shared__ unsigned hist[64];
   __shared__ unsigned long long smin[MK_THREADS / 32], smax[MK_THREADS / 32];
   __shared__ double ssum[MK_THREADS / 32];
   __shared__ unsigned sinv[MK_THREADS / 32], sf64[MK_THREADS / 32];

   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   unsigned long long kmin = ~0ULL, kmax = ~0ULL;
   float s = 0.f, c = 0.f;
   unsigned ninv = 0, nf64 = 0;

   if(threadIdx.x < 64)
      hist[threadIdx.x] = 0;
   __syncthreads();

   const int stride = gridDim.x * blockDim.x;
   /* every warp handles 32 consecutive tets per iteration (ballot words) */
   for(int base=blockIdx.x*blockDim.x + wid*32; base<nt; base+=stride)
   {
      const int t = base + lane;
      int inv = 0;
      if(t < nt)
      {
         const int4 e = __ldg(&tet[t]);
         const float4 a = __ldg(&crd[e.x]), b = __ldg(&crd[e.y]);
         const float4 cc = __ldg(&crd[e.z]), d = __ldg(&crd[e.w]);
         const float abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
         const float acx = cc.x - a.x, acy = cc.y - a.y, acz = cc.z - a.z;
         const float adx = d.x - a.x, ady = d.y - a.y, adz = d.z - a.z;
         const float bcx = cc.x - b.x, bcy = cc.y - b.y, bcz = cc.z - b.z;
         const float bdx = d.x - b.x, bdy = d.y - b.y, bdz = d.z - b.z;
         const float cdx = d.x - cc.x, cdy = d.y - cc.y, cdz = d.z - cc.z;
         const float m1 = acy * adz - acz * ady, m2 = acz * adx - acx * adz, m3 = acx * ady - acy * adx;
         float det = abx * m1 + aby * m2 + abz * m3;
         int pos = det > 0.f;
         const float perm = fabsf(abx) * (fabsf(acy * adz) + fabsf(acz * ady))
                          + fabsf(aby) * (fabsf(acz * adx) + fabsf(acx * adz))
                          + fabsf(abz) * (fabsf(acx * ady) + fabsf(acy * adx));
         if(fabsf(det) < fmaxf(thr, 9.5367431640625e-07f * perm))
         {
            /* FP64 determinant of the FP32 coordinates decides the sign */
            const double Ax = a.x, Ay = a.y, Az = a.z;
            const double bx = b.x - Ax, by = b.y - Ay, bz = b.z - Az;
            const double cx = cc.x - Ax, cy = cc.y - Ay, cz = cc.z - Az;
            const double dx = d.x - Ax, dy = d.y - Ay, dz = d.z - Az;
            const double dd = bx * (cy * dz - cz * dy) + by * (cz * dx - cx * dz) + bz * (cx * dy - cy * dx);
            det = (float)dd;
            pos = dd > 0.;
            nf64++;
         }
         const float l2 = abx*abx + aby*aby + abz*abz + acx*acx + acy*acy + acz*acz
                        + adx*adx + ady*ady + adz*adz + bcx*bcx + bcy*bcy + bcz*bcz
                        + bdx*bdx + bdy*bdy + bdz*bdz + cdx*cdx + cdy*cdy + cdz*cdz;
         const float vol = fabsf(det) * (1.0f / 6.0f);
         const float cb = cbrtf(3.0f * vol);
         float q = 12.0f * cb * cb / l2;
         inv = !pos;
         if(inv) q = -q;
         if(qout) qout[t] = q;
         int bin = (int)(q * 64.0f);
         bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
         atomicAdd(&hist[bin], 1u);
         const unsigned k = mk_fkey(q);
         const unsigned long long a64 = ((unsigned long long)k << 32) | (unsigned)t;
         const unsigned long long b64 = ((unsigned long long)(~k) << 32) | (unsigned)t;
         kmin = a64 < kmin ? a64 : kmin;
         kmax = b64 < kmax ? b64 : kmax;
         /* TwoSum accumulation */
         const float tt = s + q, bp = tt - s;
         c += (s - (tt - bp)) + (q - bp);
         s = tt;
      }
      const unsigned word = __ballot_sync(0xffffffffu, inv);
      if(lane == 0)
      {
         ninv += __popc(word);
         if(flags)
            flags[ base >> 5 ] = word;
      }
   }

   /* block reduction */
   double dsum = (double)s + (double)c;
   for(int o=16;o>0;o>>=1)
   {
      unsigned long long x = __shfl_xor_sync(0xffffffffu, kmin, o);
      unsigned long long y = __shfl_xor_sync(0xffffffffu, kmax, o);
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
      dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
      nf64 += __shfl_xor_sync(0xffffffffu, nf64, o);
   }
   if(lane == 0)
   {
      smin[wid] = kmin; smax[wid] = kmax; ssum[wid] = dsum; sinv[wid] = ninv; sf64[wid] = nf64;
   }
   __syncthreads();
   if(threadIdx.x == 0)
   {
      for(int w=1;w<MK_THREADS/32;w++)
      {
         kmin = smin[w] < kmin ? smin[w] : kmin;
         kmax = smax[w] < kmax ? smax[w] : kmax;
         dsum += ssum[w];
         ninv += sinv[w];
         nf64 += sf64[w];
      }
      atomicMin(&st->MinKey, kmin);
      atomicMin(&st->MaxKey, kmax);
      atomicAdd(&st->Sum, dsum);
      atomicAdd(&st->NmbInv, ninv);
      atomicAdd(&st->NmbF64, nf64);
   }
   if(threadIdx.x < 64 && hist[threadIdx.x])
      atomicAdd(&st->Hist[threadIdx.x], hist[threadIdx.x]);
}

/* ========================================================================= */
/* host wrappers                                                              */
/* ========================================================================= */

static unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

extern "C" int gmd_mesh_vt_csr(GmdCtx *ctx, const void *tet, int nt, int nv,
                               int *ptr, int *vt, int *tmp, int *err)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   cudaMemsetAsync(tmp, 0, (size_t)nv * sizeof(int), st);
   count_vt_kernel<<<nblk(nt, MK_THREADS), MK_THREADS, 0, st>>>((const int4 *)tet, nt, nv, tmp, err);
   scan_excl_kernel<int><<<1, 1024, 0, st>>>(tmp, ptr, nv);
   cudaMemsetAsync(tmp, 0, (size_t)nv * sizeof(int), st);
   fill_vt_kernel<<<nblk(nt, MK_THREADS), MK_THREADS, 0, st>>>((const int4 *)tet, nt, nv, ptr, tmp, vt);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_boundary(GmdCtx *ctx, const void *tet, int nt, const int *ptr,
                                 const int *vt, int *fixed)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   boundary_kernel<<<nblk(nt, MK_THREADS), MK_THREADS, 0, st>>>((const int4 *)tet, nt, ptr, vt, fixed);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_point_count(GmdCtx *ctx, const void *tet, int nv, const int *ptr,
                                    const int *vt, const int *fixed, int *pdeg,
                                    long long *width, long long *soff, int *err)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   int ns = (nv + 31) / 32;
   point_count_kernel<<<nblk(nv, 128), 128, 0, st>>>(nv, (const int4 *)tet, ptr, vt, fixed, pdeg, err);
   slice_width_kernel<<<nblk(ns, MK_THREADS), MK_THREADS, 0, st>>>(nv, pdeg, width);
   scan_excl_kernel<long long><<<1, 1024, 0, st>>>(width, soff, ns);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_point_fill(GmdCtx *ctx, const void *tet, int nv, const int *ptr,
                                   const int *vt, const int *pdeg, const long long *soff, int *pcol)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   point_fill_kernel<<<nblk(nv, 128), 128, 0, st>>>(nv, (const int4 *)tet, ptr, vt, pdeg, soff, pcol);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_laplace(GmdCtx *ctx, int nv, const long long *soff, const int *pdeg,
                                const int *pcol, const void *in, void *out, float omega)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   laplace_sell_kernel<<<nblk(nv, MK_THREADS), MK_THREADS, 0, st>>>(nv, soff, pdeg, pcol,
      (const float4 *)in, (float4 *)out, omega);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_stats_init(GmdCtx *ctx, GmlxQualStats *st, int n)
{
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   stats_init_kernel<<<nblk(n, 64), 64, 0, s>>>(st, n);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_quality(GmdCtx *ctx, int nt, const void *tet, const void *crd, float thr,
                                float *qout, unsigned *flags, GmlxQualStats *st)
{
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   long long need = nblk(nt, MK_THREADS);
   long long cap = (long long)gmd_num_sms(ctx) * 8;
   unsigned g = (unsigned)(need < cap ? need : cap);
   if(g < 1) g = 1;
   tet_quality_kernel<<<g, MK_THREADS, 0, s>>>(nt, (const int4 *)tet, (const float4 *)crd, thr,
                                               qout, flags, st);
   return cudaGetLastError() == cudaSuccess;
}
