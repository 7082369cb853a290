/*
 * gml_mesh_kernels.cu -- native mesh kernels (no counterpart in the
 * reference API; they serve the ball-of-points smoothing and quality
 * workloads directly instead of through generated scatter/gather pairs).
 *
 * Topology (built on the GPU, deterministic):
 *   vertex -> tetrahedron CSR   count (atomics), exclusive scan (gml_scan.cu),
 *                               fill (atomic slots; order within a ball is
 *                               not used by the kernels below)
 *   ball of points              per vertex, the distinct vertices of its
 *                               tetrahedra, sorted ascending, stored as
 *                               SELL-C-sigma (C = 32, sigma = 256: sorted by
 *                               size inside windows of 256 vertices); fixed
 *                               vertices get an empty ball
 *   boundary vertices           vertices of faces owned by a single tet
 *
 * Hot kernels (HBM-bound):
 *   laplace_pf_kernel
 *                  one Jacobi sweep x' = x + w (mean(ball) - x), one thread
 *                  per row; per vertex 4 (packed row word) + 4 deg (entries,
 *                  128-byte runs per warp) + 16 (own) + 16 (write) bytes;
 *                  neighbour gathers hit L2 (the coordinates are 16 V bytes).
 *   tet_quality_tma_kernel
 *                  mean-ratio quality 12 (3|V|)^(2/3) / sum l^2 signed by
 *                  orientation, 64-bin histogram, min/argmin, max/argmax,
 *                  sum, inverted-element count and bit flags; the 16 bytes
 *                  per tet of connectivity are staged through shared memory
 *                  by TMA bulk copies, coordinates come from L2.  The
 *                  determinant is recomputed in FP64 whenever the FP32 value
 *                  is below max(1e-6 h^3, 16 eps32 * permanent), a bound on
 *                  the FP32 error, so the orientation flags are exact.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include "gml_device.h"
#include "gml_mesh.h"

#define MK_THREADS 256

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

#define PB_MAX 63

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

/* SELL-C-sigma layout of the balls of points.  Vertices are sorted by
   decreasing ball size inside windows of sigma consecutive vertices (32 to
   SIGMA = 256, a tuning choice; the Hilbert locality of the numbering is
   kept), rows are grouped by 32 into
   slices as wide as their first row, and entry k of the 32 rows of a slice
   is stored contiguously.  rowv[r] packs the vertex of row r and its ball
   size: (d << 26) | v.  One thread per row then streams column indices in
   128-byte runs with almost no padding. */
#define SIGMA      256
#define ROW_SHIFT  26
#define ROW_MASK   ((1u << ROW_SHIFT) - 1u)
#define ROW_NONE   0xffffffffu

/* ------------------------------------------------------------------------- */
/* TMA bulk copies and mbarriers (inline PTX)                                 */
/* ------------------------------------------------------------------------- */

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
   return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_bulk_g2s(void *dst, const void *src, unsigned bytes,
                                             unsigned long long *bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

/* the same copy with an L2 evict-first hint: for data read once per pass
   (connectivity), so that it does not push the reused coordinates out */
__device__ __forceinline__ void tma_bulk_g2s_stream(void *dst, const void *src, unsigned bytes,
                                                    unsigned long long *bar)
{
   unsigned long long pol;
   asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
                " [%0], [%1], %2, [%3], %4;"
                :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(pol) : "memory");
}

/* wait for the phase with the given parity; the thread is suspended in
   hardware (no issue slots used) for at most about 20 us per call */
__device__ __forceinline__ int mbar_try_wait(unsigned long long *bar, unsigned parity)
{
   unsigned ok;
   asm volatile("{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
   return (int)ok;
}

/* bounded wait: gives up after QK_SPIN suspended tries (well under a
   second in total), so a lost transfer ends the kernel with an error flag
   instead of hanging it */
#define QK_SPIN (1 << 14)

__device__ __forceinline__ int mbar_wait_bounded(unsigned long long *bar, unsigned parity)
{
   for(int i=0;i<QK_SPIN;i++)
      if(mbar_try_wait(bar, parity))
         return 1;
   return 0;
}

/* one block per window of blockDim.x (<= SIGMA) rows: each row's rank in
   decreasing ball size, ties in vertex order */
__global__ void __launch_bounds__(SIGMA)
window_sort_kernel(int nv, const int *__restrict__ pdeg, unsigned *rowv)
{
   __shared__ int dd[SIGMA];
   const int w = blockDim.x, t = threadIdx.x, v = blockIdx.x * w + t;
   const int d = v < nv ? pdeg[v] : -1;
   dd[t] = d;
   __syncthreads();
   int rank = 0;
   for(int u=0;u<w;u++)
   {
      const int du = dd[u];
      rank += (du > d) || (du == d && u < t);
   }
   rowv[ blockIdx.x * w + rank ] = v < nv ? (((unsigned)d << ROW_SHIFT) | (unsigned)v) : ROW_NONE;
}

__global__ void slice_width_kernel(int nslice, const unsigned *__restrict__ rowv, long long *w)
{
   const int s = blockIdx.x * blockDim.x + threadIdx.x;
   if(s >= nslice) return;
   const unsigned r = rowv[ 32 * s ];
   w[s] = r == ROW_NONE ? 0 : (long long)(r >> ROW_SHIFT);
}

__global__ void point_fill_kernel(int nrow, const int4 *__restrict__ tet, const int *__restrict__ ptr,
                                  const int *__restrict__ vt, const unsigned *__restrict__ rowv,
                                  const long long *__restrict__ soff, int *col)
{
   const int r = blockIdx.x * blockDim.x + threadIdx.x;
   int lst[PB_MAX];
   if(r >= nrow) return;
   const unsigned pk = rowv[r];
   if(pk == ROW_NONE || !(pk >> ROW_SHIFT)) return;
   const int v = (int)(pk & ROW_MASK), d = (int)(pk >> ROW_SHIFT);
   const int n = point_ball(v, tet, ptr, vt, lst);
   const long long base = soff[ r >> 5 ];
   for(int k=0;k<n && k<d;k++)
      col[ (base + k) * 32 + (r & 31) ] = lst[k];
}

/* ========================================================================= */
/* Laplacian sweep over the ball of points, one thread per SELL row           */
/* ========================================================================= */

/* The sweep as a persistent kernel: warp w handles slices w, w + W, ...
   and, before working on a slice, asks the TMA unit to prefetch the column
   block of its next slice into L2 (cp.async.bulk.prefetch.L2), so the
   column loads of the next slice hit L2 instead of HBM.  Inside a row the
   column loads of entries k+4..k+7 are issued before the coordinate
   gathers of entries k..k+3, keeping about eight loads in flight per
   thread. */
__device__ __forceinline__ void prefetch_l2(const void *p, unsigned bytes)
{
   asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

#ifndef LP_BLOCKS
#define LP_BLOCKS 6                        /* resident blocks per SM */
#endif
#ifndef LP_PFDIST
#define LP_PFDIST 1                        /* L2 prefetch distance, in slices per warp */
#endif
#ifndef LP_STREAM
#define LP_STREAM 1                        /* evict-first loads of the column runs */
#endif
#if LP_STREAM
#define LP_LDC(p) __ldcs(p)
#else
#define LP_LDC(p) __ldg(p)
#endif

template<int U>
__global__ void __launch_bounds__(MK_THREADS, LP_BLOCKS)
laplace_pf_kernel(int nslice, const unsigned *__restrict__ rowv, const long long *__restrict__ soff,
                  const int *__restrict__ col, const float4 *__restrict__ in,
                  float4 *__restrict__ out, float omega)
{
   const int lane = threadIdx.x & 31;
   const int w0 = (blockIdx.x * MK_THREADS + threadIdx.x) >> 5;
   const int nw = (gridDim.x * MK_THREADS) >> 5;

   /* the column runs of the first LP_PFDIST slices, then one slice
      LP_PFDIST iterations ahead of the current one */
   if(lane == 0)
      for(int k=0;k<LP_PFDIST;k++)
      {
         const int s0 = w0 + k * nw;
         if(s0 < nslice)
         {
            const long long c0 = __ldg(&soff[s0]), c1 = __ldg(&soff[s0 + 1]);
            if(c1 > c0)
               prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
         }
      }

   for(int sl=w0; sl<nslice; sl+=nw)
   {
      const int nx = sl + LP_PFDIST * nw;
      if(lane == 0 && nx < nslice)
      {
         const long long c0 = __ldg(&soff[nx]), c1 = __ldg(&soff[nx + 1]);
         if(c1 > c0)
            prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
      }
      const unsigned pk = __ldg(&rowv[ sl * 32 + lane ]);
      if(pk == ROW_NONE)
         continue;
      const int v = (int)(pk & ROW_MASK), d = (int)(pk >> ROW_SHIFT);
      const float4 p = __ldg(&in[v]);
      if(d == 0)
      {
         out[v] = p;
         continue;
      }
      const int *cp = col + __ldg(&soff[sl]) * 32 + lane;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      int c[U];
#pragma unroll
      for(int u=0;u<U;u++)
         c[u] = u < d ? LP_LDC(cp + u * 32) : 0;
      for(int k=0;k<d;k+=U)
      {
         int nc[U];
#pragma unroll
         for(int u=0;u<U;u++)
            nc[u] = k + U + u < d ? LP_LDC(cp + (size_t)(k + U + u) * 32) : 0;
#pragma unroll
         for(int u=0;u<U;u++)
            if(k + u < d)
            {
               const float4 q = __ldg(&in[ c[u] ]);
               sx += q.x; sy += q.y; sz += q.z;
            }
#pragma unroll
         for(int u=0;u<U;u++)
            c[u] = nc[u];
      }
      const float inv = 1.0f / (float)d;
      out[v] = make_float4(p.x + omega * (sx * inv - p.x), p.y + omega * (sy * inv - p.y),
                           p.z + omega * (sz * inv - p.z), 0.f);
   }
}

/* ========================================================================= */
/* mean-ratio quality, histogram, extrema, inverted flags                     */
/* ========================================================================= */

/* order-preserving key of a float, -0 folded onto +0 (ties between them go
   to the smallest index) */
__device__ __forceinline__ unsigned mk_fkey(float f)
{
   unsigned u = __float_as_uint(f == 0.0f ? 0.0f : f);
   return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

/* log2(x) and 1/sqrt(x) on the special-function unit */
__device__ __forceinline__ float log2f_fast(float x)
{
   float y;
   asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
   return y;
}

__device__ __forceinline__ float rsqrtf_fast(float x)
{
   float y;
   asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
   return y;
}

/* 2^x on the special-function unit (ex2.approx.ftz.f32) */
__device__ __forceinline__ float exp2f_fast(float x)
{
   float y;
   asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
   return y;
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

/* signed mean-ratio quality of one tet; *inv = det <= 0 (FP64 sign when the
   FP32 determinant is below the threshold or below a bound of its own
   rounding error), *f64 = 1 when the FP64 determinant was used.
   q = 12 (|det|/2)^(2/3) / l2 is evaluated with the special-function unit
   (log2/exp2, about 2^-22 relative error) and a fast reciprocal. */
/* FP64 determinant of the FP32 coordinates (rare path, kept out of line so
   that it costs nothing to the common path); returns det > 0 */
__device__ __noinline__ int det64_positive(const float4 a, const float4 b, const float4 c,
                                           const float4 d, float *det)
{
   const double Ax = a.x, Ay = a.y, Az = a.z;
   const double bx = b.x - Ax, by = b.y - Ay, bz = b.z - Az;
   const double cx = c.x - Ax, cy = c.y - Ay, cz = c.z - Az;
   const double dx = d.x - Ax, dy = d.y - Ay, dz = d.z - Az;
   const double dd = bx * (cy * dz - cz * dy) + by * (cz * dx - cx * dz) + bz * (cx * dy - cy * dx);
   *det = (float)dd;
   return dd > 0.;
}

/* coordinate loads: through L1 (read-only path) within one kernel, or at L2
   (.cg) when other blocks of the same launch wrote them */
template<bool CG> __device__ __forceinline__ float4 ld_crd(const float4 *p)
{
   return CG ? __ldcg(p) : __ldg(p);
}

template<bool CG = false>
__device__ __forceinline__ float tet_mean_ratio(const int4 e, const float4 *__restrict__ crd,
                                                float thr, int *inv, int *f64)
{
   const float4 a = ld_crd<CG>(&crd[e.x]), b = ld_crd<CG>(&crd[e.y]);
   const float4 c = ld_crd<CG>(&crd[e.z]), d = ld_crd<CG>(&crd[e.w]);
   const float abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
   const float acx = c.x - a.x, acy = c.y - a.y, acz = c.z - a.z;
   const float adx = d.x - a.x, ady = d.y - a.y, adz = d.z - a.z;
#if QK_L2ID
   /* sum over the 6 edges of |xi - xj|^2 = 4 sum |xi|^2 - |sum xi|^2 with a
      as the origin (4 points) */
   const float sx = abx + acx + adx, sy = aby + acy + ady, sz = abz + acz + adz;
   const float n2 = abx*abx + aby*aby + abz*abz + acx*acx + acy*acy + acz*acz
                  + adx*adx + ady*ady + adz*adz;
   const float l2 = 4.0f * n2 - (sx*sx + sy*sy + sz*sz);
#else
   const float bcx = acx - abx, bcy = acy - aby, bcz = acz - abz;
   const float bdx = adx - abx, bdy = ady - aby, bdz = adz - abz;
   const float cdx = adx - acx, cdy = ady - acy, cdz = adz - acz;
   const float l2 = abx*abx + aby*aby + abz*abz + acx*acx + acy*acy + acz*acz
                  + adx*adx + ady*ady + adz*adz + bcx*bcx + bcy*bcy + bcz*bcz
                  + bdx*bdx + bdy*bdy + bdz*bdz + cdx*cdx + cdy*cdy + cdz*cdz;
#endif
   float det = abx * (acy * adz - acz * ady) + aby * (acz * adx - acx * adz)
             + abz * (acx * ady - acy * adx);
   int pos = det > 0.f;
   /* The FP32 determinant is off by at most about 7 eps32 times the sum of
      the absolute values of its six products, a sum bounded by
      (|ab|_1 |ac|_1 |ad|_1) <= l2^(3/2); below 16 eps32 l2^(3/2) (1% margin
      for rsqrt) the sign is taken from the FP64 determinant. */
   const bool need = fabsf(det) < fmaxf(thr, 9.7e-07f * l2 * l2 * rsqrtf_fast(l2));
   *f64 = need;
#if QK_UNIFORM
   /* the rare FP64 path behind a warp-uniform test */
   if(__any_sync(__activemask(), need))
#endif
   if(need)
      pos = det64_positive(a, b, c, d, &det);
   const float v23 = exp2f_fast(0.6666666865f * log2f_fast(0.5f * fabsf(det)));
   const float q = __fdividef(12.0f * v23, l2);
   *inv = !pos;
   return pos ? q : -q;
}

/* per-thread accumulators of the statistics (a thread sees its tets in
   increasing index order, so strict comparisons keep the smallest index) */
struct QAcc
{
   float mn, mx, s, c;
   int mi, xi;
   unsigned ninv, nf64;
};

__device__ __forceinline__ void qacc_add(QAcc &a, float q, int t, int f64)
{
   if(q < a.mn) { a.mn = q; a.mi = t; }
   if(q > a.mx) { a.mx = q; a.xi = t; }
   const float tt = a.s + q, bp = tt - a.s;
   a.c += (a.s - (tt - bp)) + (q - bp);
   a.s = tt;
   a.nf64 += f64;
}

#ifndef QK_HIST
#define QK_HIST 1
#endif
#ifndef QK_L2ID
#define QK_L2ID 1
#endif
#ifndef QK_EVICT
#define QK_EVICT 1           /* connectivity copies with an L2 evict-first hint
                                (75.6 -> 69.9 us per pass on the 128^3 cube: the
                                once-read tets no longer evict the coordinates) */
#endif
#if QK_EVICT
#define QK_TMA tma_bulk_g2s_stream
#else
#define QK_TMA tma_bulk_g2s
#endif
#ifndef BT_STREAM
#define BT_STREAM 1          /* the batch kernels read tets and column runs
                                evict-first (8.29 -> 8.15 ms for the 512 meshes) */
#endif
#if BT_STREAM
#define BT_LDT(p) __ldcs(p)
#define BT_LDC(p) __ldcs(p)
#else
#define BT_LDT(p) __ldg(p)
#define BT_LDC(p) __ldg(p)
#endif
#ifndef QK_UNIFORM
#define QK_UNIFORM 0
#endif

/* histogram update of a warp.  QK_HIST 0: lanes with the same bin add once
   (match_any leaders); 1: one shared atomic per tet */
__device__ __forceinline__ void hist_add_warp(unsigned *hist, float q, int valid, int lane)
{
   int bin = (int)(q * 64.0f);
   bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
#if QK_HIST == 1
   (void)lane;
   if(valid)
      atomicAdd(&hist[bin], 1u);
#else
   if(!valid) bin = 64 + lane;
   const unsigned peers = __match_any_sync(0xffffffffu, bin);
   if(valid && lane == __ffs(peers) - 1)
      atomicAdd(&hist[bin], (unsigned)__popc(peers));
#endif
}

/* block reduction of the accumulators into the global statistics */
__device__ __forceinline__ void qacc_flush(QAcc &a, unsigned *hist, GmlxQualStats *st)
{
   __shared__ unsigned long long smin[MK_THREADS / 32], smax[MK_THREADS / 32];
   __shared__ double ssum[MK_THREADS / 32];
   __shared__ unsigned sinv[MK_THREADS / 32], sf64[MK_THREADS / 32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   double dsum = (double)a.s + (double)a.c;
   unsigned long long kmin = ~0ULL, kmax = ~0ULL;
   unsigned ninv = a.ninv, nf64 = a.nf64;

   if(a.mi >= 0)
   {
      const unsigned k = mk_fkey(a.mn), kx = mk_fkey(a.mx);
      kmin = ((unsigned long long)k << 32) | (unsigned)a.mi;
      kmax = ((unsigned long long)(~kx) << 32) | (unsigned)a.xi;
   }
   for(int o=16;o>0;o>>=1)
   {
      unsigned long long x = __shfl_xor_sync(0xffffffffu, kmin, o);
      unsigned long long y = __shfl_xor_sync(0xffffffffu, kmax, o);
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
      dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
      nf64 += __shfl_xor_sync(0xffffffffu, nf64, o);
      ninv += __shfl_xor_sync(0xffffffffu, ninv, o);
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

#ifndef QK_CHUNK
#define QK_CHUNK  1024                     /* tets per stage: 16 KB */
#endif
#ifndef QK_STAGES
#define QK_STAGES 2
#endif
#ifndef QK_BLOCKS
#define QK_BLOCKS 4                        /* resident blocks per SM */
#endif
#define QK_SMEM   (QK_STAGES * QK_CHUNK * 16)

/* The tetrahedron stream (16 bytes per tet, read once) is staged through
   shared memory by TMA bulk copies, QK_STAGES chunks ahead; the coordinate
   gathers (16 V bytes, L2 resident) are issued from registers, two tets per
   thread at a time.  Each warp handles 32 consecutive tets per pass, so its
   ballot is one word of the inverted-element bit flags. */
/* one pass over 512 tets of a staged chunk: a thread takes tets j and
   j + 256; FULL (every tet valid) removes all validity tests, WQ writes the
   per-tet quality */
template<bool FULL, bool WQ>
__device__ __forceinline__ void quality_pass(const int4 *chunk, int n, int start, int pass,
                                             const float4 *__restrict__ crd, float thr,
                                             float *__restrict__ qout, unsigned *__restrict__ flags,
                                             QAcc &a, unsigned *hist, int lane, int wid)
{
   const int j0 = pass * 2 * MK_THREADS + wid * 32 + lane, j1 = j0 + MK_THREADS;
   const bool v0 = FULL || j0 < n, v1 = FULL || j1 < n;
   int inv0 = 0, inv1 = 0, f0 = 0, f1 = 0;
   float q0 = 0.f, q1 = 0.f;
   if(v0) q0 = tet_mean_ratio(chunk[j0], crd, thr, &inv0, &f0);
   if(v1) q1 = tet_mean_ratio(chunk[j1], crd, thr, &inv1, &f1);
   if(v0 && q0 < a.mn) { a.mn = q0; a.mi = start + j0; }
   if(v0 && q0 > a.mx) { a.mx = q0; a.xi = start + j0; }
   if(v1 && q1 < a.mn) { a.mn = q1; a.mi = start + j1; }
   if(v1 && q1 > a.mx) { a.mx = q1; a.xi = start + j1; }
   if(WQ)
   {
      if(v0) qout[start + j0] = q0;
      if(v1) qout[start + j1] = q1;
   }
   {
      /* one TwoSum per pair (invalid tets contribute 0) */
      const float pq = q0 + q1, tt = a.s + pq, bp = tt - a.s;
      a.c += (a.s - (tt - bp)) + (pq - bp);
      a.s = tt;
      a.nf64 += f0 + f1;
   }
   hist_add_warp(hist, q0, v0, lane);
   hist_add_warp(hist, q1, v1, lane);
   const unsigned w0 = __ballot_sync(0xffffffffu, inv0);
   const unsigned w1 = __ballot_sync(0xffffffffu, inv1);
   if(lane == 0)
   {
      const int b0 = pass * 2 * MK_THREADS + wid * 32, b1 = b0 + MK_THREADS;
      a.ninv += __popc(w0) + __popc(w1);
      if(FULL || b0 < n) flags[ (start + b0) >> 5 ] = w0;
      if(FULL || b1 < n) flags[ (start + b1) >> 5 ] = w1;
   }
}


template<bool WQ>
__global__ void __launch_bounds__(MK_THREADS, QK_BLOCKS)
tet_quality_tma_kernel(int nt, const int4 *__restrict__ tet, const float4 *__restrict__ crd,
                       float thr, float *__restrict__ qout, unsigned *__restrict__ flags,
                       GmlxQualStats *st, int *err)
{
   extern __shared__ __align__(128) unsigned char qk_smem[];
   __shared__ __align__(8) unsigned long long bar[QK_STAGES];
   __shared__ unsigned hist[64];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   const int nchunk = (nt + QK_CHUNK - 1) / QK_CHUNK;
   const int mine = blockIdx.x < nchunk ? (nchunk - 1 - blockIdx.x) / gridDim.x + 1 : 0;
   int4 *stage = (int4 *)qk_smem;
   QAcc a = { 3.402823466e38f, -3.402823466e38f, 0.f, 0.f, -1, -1, 0u, 0u };

   if(threadIdx.x < 64)
      hist[threadIdx.x] = 0;
   if(threadIdx.x == 0)
   {
      for(int s=0;s<QK_STAGES;s++)
         mbar_init(&bar[s], 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      for(int s=0;s<QK_STAGES && s<mine;s++)
      {
         const int start = (blockIdx.x + s * gridDim.x) * QK_CHUNK;
         const unsigned bytes = (unsigned)(min(QK_CHUNK, nt - start) * 16);
         mbar_expect_tx(&bar[s], bytes);
         QK_TMA(stage + s * QK_CHUNK, tet + start, bytes, &bar[s]);
      }
   }
   __syncthreads();

   for(int i=0;i<mine;i++)
   {
      const int s = i % QK_STAGES;
      const unsigned parity = (unsigned)((i / QK_STAGES) & 1);
      const int ok = mbar_wait_bounded(&bar[s], parity);
      if(__syncthreads_or(!ok))
      {
         /* lost transfer: report, let the issued copies land, stop */
         if(threadIdx.x == 0)
         {
            atomicOr(err, 4);
            for(int j=i;j<mine && j<i+QK_STAGES;j++)
               mbar_wait_bounded(&bar[j % QK_STAGES], (unsigned)((j / QK_STAGES) & 1));
         }
         __syncthreads();
         return;
      }

      const int start = (blockIdx.x + i * gridDim.x) * QK_CHUNK;
      const int n = min(QK_CHUNK, nt - start);
      const int4 *chunk = stage + s * QK_CHUNK;

      /* passes of 512 tets; only the last chunk can be partial */
      if(n == QK_CHUNK)
      {
#pragma unroll
         for(int pass=0;pass<QK_CHUNK/(2*MK_THREADS);pass++)
            quality_pass<true, WQ>(chunk, n, start, pass, crd, thr, qout, flags, a, hist, lane, wid);
      }
      else
      {
#pragma unroll 1
         for(int pass=0;pass<QK_CHUNK/(2*MK_THREADS);pass++)
            quality_pass<false, WQ>(chunk, n, start, pass, crd, thr, qout, flags, a, hist, lane, wid);
      }

      /* every thread is done with stage s: refill it */
      __syncthreads();
      if(threadIdx.x == 0 && i + QK_STAGES < mine)
      {
         const int nstart = (blockIdx.x + (i + QK_STAGES) * gridDim.x) * QK_CHUNK;
         const unsigned bytes = (unsigned)(min(QK_CHUNK, nt - nstart) * 16);
         mbar_expect_tx(&bar[s], bytes);
         QK_TMA(stage + s * QK_CHUNK, tet + nstart, bytes, &bar[s]);
      }
   }

   qacc_flush(a, hist, st);
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
   if(!gmd_scan_excl_i32(ctx, tmp, ptr, nv))
      return 0;
   cudaMemsetAsync(tmp, 0, (size_t)nv * sizeof(int), st);
   fill_vt_kernel<<<nblk(nt, MK_THREADS), MK_THREADS, 0, st>>>((const int4 *)tet, nt, nv, ptr, tmp, vt);
   return cudaGetLastError() == cudaSuccess;
}

/* fixed[v] = ref[v] != 0 */
__global__ void fixed_from_ref_kernel(const int *__restrict__ ref, int nv, int *fixed)
{
   const int v = blockIdx.x * blockDim.x + threadIdx.x;
   if(v < nv)
      fixed[v] = ref[v] != 0;
}

extern "C" int gmd_mesh_fixed_from_ref(GmdCtx *ctx, const int *ref, int nv, int *fixed)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   if(nv <= 0)
      return 1;
   fixed_from_ref_kernel<<<nblk(nv, MK_THREADS), MK_THREADS, 0, st>>>(ref, nv, fixed);
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
                                    const int *vt, const int *fixed, int *pdeg, unsigned *rowv,
                                    long long *width, long long *soff, int *err, int window)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const int nrow = (nv + SIGMA - 1) / SIGMA * SIGMA, nslice = nrow / 32;
   if(window < 32 || window > SIGMA || SIGMA % window)
      return 0;
   point_count_kernel<<<nblk(nv, 128), 128, 0, st>>>(nv, (const int4 *)tet, ptr, vt, fixed, pdeg, err);
   window_sort_kernel<<<nrow / window, window, 0, st>>>(nv, pdeg, rowv);
   slice_width_kernel<<<nblk(nslice, MK_THREADS), MK_THREADS, 0, st>>>(nslice, rowv, width);
   if(!gmd_scan_excl_i64(ctx, width, soff, nslice))
      return 0;
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_point_fill(GmdCtx *ctx, const void *tet, int nrow, const int *ptr,
                                   const int *vt, const unsigned *rowv, const long long *soff,
                                   int *col)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   point_fill_kernel<<<nblk(nrow, 128), 128, 0, st>>>(nrow, (const int4 *)tet, ptr, vt, rowv, soff, col);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_laplace(GmdCtx *ctx, int nrow, const unsigned *rowv, const long long *soff,
                                const int *col, const void *in, void *out, float omega, int *err,
                                int bps)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const int nslice = nrow / 32;
   const long long need = nblk(nslice, MK_THREADS / 32);
   const long long cap = (long long)gmd_num_sms(ctx) * (bps > 0 && bps < LP_BLOCKS ? bps : LP_BLOCKS);
   (void)err;
   if(nslice <= 0)
      return 1;
   laplace_pf_kernel<8><<<(unsigned)(need < cap ? need : cap), MK_THREADS, 0, st>>>(
      nslice, rowv, soff, col, (const float4 *)in, (float4 *)out, omega);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_stats_init(GmdCtx *ctx, GmlxQualStats *st, int n)
{
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   stats_init_kernel<<<nblk(n, 64), 64, 0, s>>>(st, n);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_quality(GmdCtx *ctx, int nt, const void *tet, const void *crd, float thr,
                                float *qout, unsigned *flags, GmlxQualStats *st, int *err, int bps)
{
   static int attr_set = 0;
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   long long need = nblk(nt, QK_CHUNK);
   long long cap = (long long)gmd_num_sms(ctx) * (bps > 0 && bps < QK_BLOCKS ? bps : QK_BLOCKS);
   unsigned g = (unsigned)(need < cap ? need : cap);
   if(nt <= 0)
      return 1;
   if(!attr_set)
   {
      if(cudaFuncSetAttribute(tet_quality_tma_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              QK_SMEM) != cudaSuccess
      || cudaFuncSetAttribute(tet_quality_tma_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              QK_SMEM) != cudaSuccess)
         return 0;
      attr_set = 1;
   }
   if(!flags)
      return 0;
   if(qout)
      tet_quality_tma_kernel<true><<<g, MK_THREADS, QK_SMEM, s>>>(nt, (const int4 *)tet,
         (const float4 *)crd, thr, qout, flags, st, err);
   else
      tet_quality_tma_kernel<false><<<g, MK_THREADS, QK_SMEM, s>>>(nt, (const int4 *)tet,
         (const float4 *)crd, thr, qout, flags, st, err);
   return cudaGetLastError() == cudaSuccess;
}

/* ========================================================================= */
/* batched meshes: one persistent launch over a (mesh, range) tile queue      */
/* ========================================================================= */

/* Tiles are claimed in queue order with one atomic per tile.  The queue is
   phase-major (every sweep-0 tile of every mesh, then sweep 1, ..., then the
   quality tiles), and a tile of phase p of mesh m starts only when all tiles
   of phase p - 1 of mesh m are done (per-(mesh, phase) counters).  A waiting
   tile only depends on tiles claimed before it, by blocks that are running,
   so the queue always drains; the wait is nevertheless bounded (a.spin
   tries of about 256 ns, 2^22 by default) and a timeout aborts the launch
   with error bit 16.

   Coordinates written by other blocks of the same launch are read at L2
   (ld.global.cg), never through L1.  Sweep tiles are whole slices of the
   SELL ball of points (a mesh's vertex range starts on a window boundary, so
   slices never mix meshes); quality tiles are tet ranges of one mesh starting
   at a multiple of 32, so each warp's ballot is one flag word of that mesh. */


__device__ __forceinline__ void batch_sweep_slices(int s0, int s1, const unsigned *__restrict__ rowv,
                                                   const long long *__restrict__ soff,
                                                   const int *__restrict__ col,
                                                   const float4 *in, float4 *out, float omega)
{
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   if(lane == 0 && s0 + wid < s1)
   {
      const long long c0 = __ldg(&soff[s0 + wid]), c1 = __ldg(&soff[s0 + wid + 1]);
      if(c1 > c0)
         prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
   }
   for(int sl=s0+wid; sl<s1; sl+=MK_THREADS/32)
   {
      /* the next slice of this warp: its column run into L2 */
      const int nx = sl + MK_THREADS / 32;
      if(lane == 0 && nx < s1)
      {
         const long long c0 = __ldg(&soff[nx]), c1 = __ldg(&soff[nx + 1]);
         if(c1 > c0)
            prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
      }
      const unsigned pk = __ldg(&rowv[ sl * 32 + lane ]);
      if(pk == ROW_NONE)
         continue;
      const int v = (int)(pk & ROW_MASK), d = (int)(pk >> ROW_SHIFT);
      const float4 p = __ldcg(&in[v]);
      if(d == 0)
      {
         out[v] = p;
         continue;
      }
      const int *cp = col + __ldg(&soff[sl]) * 32 + lane;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      int c[8];
#pragma unroll
      for(int u=0;u<8;u++)
         c[u] = u < d ? BT_LDC(cp + u * 32) : 0;
      for(int k=0;k<d;k+=8)
      {
         int nc[8];
#pragma unroll
         for(int u=0;u<8;u++)
            nc[u] = k + 8 + u < d ? BT_LDC(cp + (size_t)(k + 8 + u) * 32) : 0;
#pragma unroll
         for(int u=0;u<8;u++)
            if(k + u < d)
            {
               const float4 q = __ldcg(&in[ c[u] ]);
               sx += q.x; sy += q.y; sz += q.z;
            }
#pragma unroll
         for(int u=0;u<8;u++)
            c[u] = nc[u];
      }
      const float inv = 1.0f / (float)d;
      out[v] = make_float4(p.x + omega * (sx * inv - p.x), p.y + omega * (sy * inv - p.y),
                           p.z + omega * (sz * inv - p.z), 0.f);
   }
}

/* quality of local tets [beg, end) of one mesh; accumulators in a and hist */
__device__ __forceinline__ void batch_quality_range(int beg, int end, const int4 *__restrict__ tet,
                                                    const float4 *crd, float thr,
                                                    unsigned *__restrict__ flags, QAcc &a,
                                                    unsigned *hist)
{
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   for(int base=beg+wid*32; base<end; base+=MK_THREADS)
   {
      const int j = base + lane;
      const bool v = j < end;
      int inv = 0, f = 0;
      float q = 0.f;
      if(v)
      {
         q = tet_mean_ratio<true>(BT_LDT(&tet[j]), crd, thr, &inv, &f);
         if(q < a.mn) { a.mn = q; a.mi = j; }
         if(q > a.mx) { a.mx = q; a.xi = j; }
         const float tt = a.s + q, bp = tt - a.s;
         a.c += (a.s - (tt - bp)) + (q - bp);
         a.s = tt;
         a.nf64 += f;
         int bin = (int)(q * 64.0f);
         bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
         atomicAdd(&hist[bin], 1u);
      }
      const unsigned w = __ballot_sync(0xffffffffu, inv);
      if(lane == 0)
      {
         a.ninv += __popc(w);
         flags[ base >> 5 ] = w;
      }
   }
}

__global__ void __launch_bounds__(MK_THREADS, 5)
batch_queue_kernel(GmdBatchArgs a)
{
   __shared__ int s_tile;
   __shared__ unsigned hist[64];
   QAcc acc = { 3.402823466e38f, -3.402823466e38f, 0.f, 0.f, -1, -1, 0u, 0u };

   if(threadIdx.x < 64)
      hist[threadIdx.x] = 0;
   for(;;)
   {
      __syncthreads();
      if(threadIdx.x == 0)
      {
         int t = -1;
         if(!*(volatile int *)a.abort)
            t = atomicAdd(a.head, 1);
         if(t >= a.ntile)
            t = -1;
         if(t >= 0)
         {
            const GmdBatchTile tl = a.tiles[t];
            if(tl.phase > 0)
            {
               const int k = tl.mesh * a.nphase + tl.phase - 1, need = a.need[k];
               volatile int *dp = a.done + k;
               int it = 0;
               while(*dp < need)
               {
                  if(++it > a.spin || *(volatile int *)a.abort)
                  {
                     atomicOr(a.err, 16);
                     *(volatile int *)a.abort = 1;
                     t = -1;
                     break;
                  }
                  __nanosleep(256);
               }
               __threadfence();
            }
         }
         s_tile = t;
      }
      __syncthreads();
      const int t = s_tile;
      if(t < 0)
         break;
      const GmdBatchTile tl = a.tiles[t];
      const GmdBatchMesh m = a.mesh[tl.mesh];
      float4 *b0 = (float4 *)a.buf0, *b1 = (float4 *)a.buf1;
      if(tl.phase < a.nsweep)
      {
         const float4 *in = (tl.phase & 1) ? b1 : b0;
         float4 *out = (tl.phase & 1) ? b0 : b1;
         batch_sweep_slices(tl.beg, tl.end, a.rowv, a.soff, a.col, in, out, a.omega);
      }
      else
      {
         const float4 *crd = (a.nsweep & 1) ? b1 : b0;
         batch_quality_range(tl.beg, tl.end, (const int4 *)a.tet + m.t0, crd, m.thr, a.flags + m.f0,
                             acc, hist);
         qacc_flush(acc, hist, a.stats + tl.mesh);
         __syncthreads();
         if(threadIdx.x < 64)
            hist[threadIdx.x] = 0;
         acc = QAcc{ 3.402823466e38f, -3.402823466e38f, 0.f, 0.f, -1, -1, 0u, 0u };
      }
      /* every thread's writes are visible at GPU scope before the tile counts */
      __threadfence();
      __syncthreads();
      if(threadIdx.x == 0)
         atomicAdd(a.done + tl.mesh * a.nphase + tl.phase, 1);
   }
}

/* The same queue drained by warps instead of blocks: each warp claims its
   own tiles, waits for its own dependencies and counts its tiles done, so
   no block barrier sits in the tile loop.  Quality statistics are folded
   per warp (registers and a per-warp histogram) and flushed per tile. */
__device__ __forceinline__ void warp_sweep_slices(int s0, int s1, const unsigned *__restrict__ rowv,
                                                  const long long *__restrict__ soff,
                                                  const int *__restrict__ col,
                                                  const float4 *in, float4 *out, float omega)
{
   const int lane = threadIdx.x & 31;
   if(lane == 0)
   {
      const long long c0 = __ldg(&soff[s0]), c1 = __ldg(&soff[s0 + 1]);
      if(c1 > c0)
         prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
   }
   for(int sl=s0; sl<s1; sl++)
   {
      if(lane == 0 && sl + 1 < s1)
      {
         const long long c0 = __ldg(&soff[sl + 1]), c1 = __ldg(&soff[sl + 2]);
         if(c1 > c0)
            prefetch_l2(col + c0 * 32, (unsigned)((c1 - c0) * 128));
      }
      const unsigned pk = __ldg(&rowv[ sl * 32 + lane ]);
      if(pk == ROW_NONE)
         continue;
      const int v = (int)(pk & ROW_MASK), d = (int)(pk >> ROW_SHIFT);
      const float4 p = __ldcg(&in[v]);
      if(d == 0)
      {
         out[v] = p;
         continue;
      }
      const int *cp = col + __ldg(&soff[sl]) * 32 + lane;
      float sx = 0.f, sy = 0.f, sz = 0.f;
      int c[8];
#pragma unroll
      for(int u=0;u<8;u++)
         c[u] = u < d ? BT_LDC(cp + u * 32) : 0;
      for(int k=0;k<d;k+=8)
      {
         int nc[8];
#pragma unroll
         for(int u=0;u<8;u++)
            nc[u] = k + 8 + u < d ? BT_LDC(cp + (size_t)(k + 8 + u) * 32) : 0;
#pragma unroll
         for(int u=0;u<8;u++)
            if(k + u < d)
            {
               const float4 q = __ldcg(&in[ c[u] ]);
               sx += q.x; sy += q.y; sz += q.z;
            }
#pragma unroll
         for(int u=0;u<8;u++)
            c[u] = nc[u];
      }
      const float inv = 1.0f / (float)d;
      out[v] = make_float4(p.x + omega * (sx * inv - p.x), p.y + omega * (sy * inv - p.y),
                           p.z + omega * (sz * inv - p.z), 0.f);
   }
}

__device__ __forceinline__ void warp_quality_range(int beg, int end, const int4 *__restrict__ tet,
                                                   const float4 *crd, float thr,
                                                   unsigned *__restrict__ flags, QAcc &a,
                                                   unsigned *hist)
{
   const int lane = threadIdx.x & 31;
   for(int base=beg; base<end; base+=32)
   {
      const int j = base + lane;
      const bool v = j < end;
      int inv = 0, f = 0;
      float q = 0.f;
      if(v)
      {
         q = tet_mean_ratio<true>(BT_LDT(&tet[j]), crd, thr, &inv, &f);
         if(q < a.mn) { a.mn = q; a.mi = j; }
         if(q > a.mx) { a.mx = q; a.xi = j; }
         const float tt = a.s + q, bp = tt - a.s;
         a.c += (a.s - (tt - bp)) + (q - bp);
         a.s = tt;
         a.nf64 += f;
         int bin = (int)(q * 64.0f);
         bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
         atomicAdd(&hist[bin], 1u);
      }
      const unsigned w = __ballot_sync(0xffffffffu, inv);
      if(lane == 0)
      {
         a.ninv += __popc(w);
         flags[ base >> 5 ] = w;
      }
   }
}

/* warp reduction of the accumulators into a mesh's statistics; resets them */
__device__ __forceinline__ void warp_flush(QAcc &a, unsigned *hist, GmlxQualStats *st)
{
   const int lane = threadIdx.x & 31;
   double dsum = (double)a.s + (double)a.c;
   unsigned long long kmin = ~0ULL, kmax = ~0ULL;
   unsigned ninv = a.ninv, nf64 = a.nf64;
   if(a.mi >= 0)
   {
      const unsigned k = mk_fkey(a.mn), kx = mk_fkey(a.mx);
      kmin = ((unsigned long long)k << 32) | (unsigned)a.mi;
      kmax = ((unsigned long long)(~kx) << 32) | (unsigned)a.xi;
   }
   for(int o=16;o>0;o>>=1)
   {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, kmin, o);
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, kmax, o);
      kmin = x < kmin ? x : kmin;
      kmax = y < kmax ? y : kmax;
      dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
      nf64 += __shfl_xor_sync(0xffffffffu, nf64, o);
      ninv += __shfl_xor_sync(0xffffffffu, ninv, o);
   }
   if(lane == 0)
   {
      atomicMin(&st->MinKey, kmin);
      atomicMin(&st->MaxKey, kmax);
      atomicAdd(&st->Sum, dsum);
      atomicAdd(&st->NmbInv, ninv);
      atomicAdd(&st->NmbF64, nf64);
   }
   __syncwarp();
   for(int b=lane;b<64;b+=32)
   {
      if(hist[b])
         atomicAdd(&st->Hist[b], hist[b]);
      hist[b] = 0;
   }
   __syncwarp();
   a = QAcc{ 3.402823466e38f, -3.402823466e38f, 0.f, 0.f, -1, -1, 0u, 0u };
}

__global__ void __launch_bounds__(MK_THREADS, 5)
batch_warp_kernel(GmdBatchArgs a)
{
   __shared__ unsigned hist_all[MK_THREADS / 32][64];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   unsigned *hist = hist_all[wid];
   QAcc acc = { 3.402823466e38f, -3.402823466e38f, 0.f, 0.f, -1, -1, 0u, 0u };
   float4 *b0 = (float4 *)a.buf0, *b1 = (float4 *)a.buf1;

   for(int b=lane;b<64;b+=32)
      hist[b] = 0;
   __syncwarp();
   for(;;)
   {
      int t = -1;
      if(lane == 0)
      {
         if(!*(volatile int *)a.abort)
            t = atomicAdd(a.head, 1);
         if(t >= a.ntile)
            t = -1;
         if(t >= 0)
         {
            const GmdBatchTile tl = a.tiles[t];
            if(tl.phase > 0)
            {
               const int k = tl.mesh * a.nphase + tl.phase - 1, need = a.need[k];
               volatile int *dp = a.done + k;
               int it = 0;
               while(*dp < need)
               {
                  if(++it > a.spin || *(volatile int *)a.abort)
                  {
                     atomicOr(a.err, 16);
                     *(volatile int *)a.abort = 1;
                     t = -1;
                     break;
                  }
                  __nanosleep(256);
               }
               __threadfence();
            }
         }
      }
      t = __shfl_sync(0xffffffffu, t, 0);
      if(t < 0)
         break;
      const GmdBatchTile tl = a.tiles[t];
      const GmdBatchMesh m = a.mesh[tl.mesh];
      if(tl.phase < a.nsweep)
      {
         const float4 *in = (tl.phase & 1) ? b1 : b0;
         float4 *out = (tl.phase & 1) ? b0 : b1;
         warp_sweep_slices(tl.beg, tl.end, a.rowv, a.soff, a.col, in, out, a.omega);
      }
      else
      {
         const float4 *crd = (a.nsweep & 1) ? b1 : b0;
         warp_quality_range(tl.beg, tl.end, (const int4 *)a.tet + m.t0, crd, m.thr, a.flags + m.f0,
                            acc, hist);
         warp_flush(acc, hist, a.stats + tl.mesh);
      }
      /* the warp's writes are visible at GPU scope before the tile counts */
      __threadfence();
      __syncwarp();
      if(lane == 0)
         atomicAdd(a.done + tl.mesh * a.nphase + tl.phase, 1);
   }
}

extern "C" int gmd_batch_queue_warp(GmdCtx *ctx, const GmdBatchArgs *a, int grid)
{
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   batch_warp_kernel<<<grid, MK_THREADS, 0, s>>>(*a);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_batch_queue(GmdCtx *ctx, const GmdBatchArgs *a, int grid)
{
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   batch_queue_kernel<<<grid, MK_THREADS, 0, s>>>(*a);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_batch_grid(GmdCtx *ctx)
{
   int per = 0;
   if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_queue_kernel, MK_THREADS, 0)
      != cudaSuccess || per < 1)
      per = 1;
   return per * gmd_num_sms(ctx);
}

/* per-mesh launch loop pieces: the sweep of a slice range, the quality of one mesh */
extern "C" int gmd_mesh_laplace_slices(GmdCtx *ctx, int s0, int s1, const unsigned *rowv,
                                       const long long *soff, const int *col, const void *in,
                                       void *out, float omega)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   const int ns = s1 - s0;
   unsigned g = (unsigned)((ns + MK_THREADS / 32 - 1) / (MK_THREADS / 32));
   if(ns <= 0)
      return 1;
   laplace_pf_kernel<8><<<g, MK_THREADS, 0, st>>>(ns, rowv + (size_t)s0 * 32, soff + s0, col,
      (const float4 *)in, (float4 *)out, omega);
   return cudaGetLastError() == cudaSuccess;
}
