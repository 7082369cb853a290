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
 *                               tetrahedra, sorted ascending, in CSR form;
 *                               each entry carries the row of its vertex
 *                               inside the vertex's group of 32; fixed
 *                               vertices get an empty ball
 *   boundary vertices           vertices of faces owned by a single tet
 *
 * Hot kernels (HBM-bound):
 *   laplace_warp   one Jacobi sweep x' = x + w (mean(ball) - x), one warp
 *                  per 32 consecutive vertices; per vertex 4 (row pointer)
 *                  + 4 deg (entries, streamed in 128-byte runs) + 16 (own)
 *                  + 16 (write) bytes; neighbour gathers hit L2 (the
 *                  coordinates are 16 V bytes).
 *   tet_quality    mean-ratio quality 12 (3|V|)^(2/3) / sum l^2 signed by
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
/* ball of points (CSR, entries tagged with the row inside its warp group)    */
/* ========================================================================= */

#define PB_MAX 64
#define PB_ROW_SHIFT 27
#define PB_COL_MASK ((1u << PB_ROW_SHIFT) - 1u)
#define PB_NONE     0xffffffffu           /* no entry (a column never reaches 2^27 - 1) */

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

/* entry = (v & 31) << 27 | neighbour: the row of v inside its group of 32
   vertices travels with the column so that a warp can reduce a group's
   contiguous entries without a search */
__global__ void point_fill_kernel(int nv, const int4 *__restrict__ tet, const int *__restrict__ ptr,
                                  const int *__restrict__ vt, const int *__restrict__ pptr,
                                  int *pcol)
{
   int v = blockIdx.x * blockDim.x + threadIdx.x;
   int lst[PB_MAX];
   if(v >= nv) return;
   int d = pptr[v+1] - pptr[v];
   if(!d) return;
   int n = point_ball(v, tet, ptr, vt, lst);
   for(int k=0;k<n && k<d;k++)
      pcol[ pptr[v] + k ] = (int)(((unsigned)(v & 31) << PB_ROW_SHIFT) | (unsigned)lst[k]);
}

/* ========================================================================= */
/* Laplacian sweep: one warp per group of 32 consecutive vertices             */
/* ========================================================================= */

/* The group's entries are contiguous in the CSR arrays; the warp streams
   them 32 at a time (coalesced 128-byte column loads, 32 independent
   coordinate gathers), sums each row's run with a shuffle segmented scan
   whose tail lane adds into shared memory (one writer per row and chunk,
   chunks in order: the summation order is fixed, results are
   reproducible), then lane r updates vertex 32g + r. */
__global__ void __launch_bounds__(MK_THREADS)
laplace_warp_kernel(int nv, const int *__restrict__ pptr, const int *__restrict__ pcol,
                    const float4 *__restrict__ in, float4 *__restrict__ out, float omega)
{
   __shared__ float acc[MK_THREADS / 32][3][32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   const int v0 = (blockIdx.x * MK_THREADS + threadIdx.x) & ~31;
   if(v0 >= nv)
      return;
   const int v = v0 + lane;
   const int vl = v < nv ? v : nv;
   const int e0 = __ldg(&pptr[v0]);
   const int p0 = __ldg(&pptr[vl]), p1 = __ldg(&pptr[v < nv ? v + 1 : nv]);
   const int e1 = __shfl_sync(0xffffffffu, p1, 31);
   float *ax = acc[wid][0], *ay = acc[wid][1], *az = acc[wid][2];

   ax[lane] = 0.f; ay[lane] = 0.f; az[lane] = 0.f;
   __syncwarp();

   for(int base=e0; base<e1; base+=64)
   {
      /* two chunks of 32 entries in flight */
      const int ea = base + lane, eb = base + 32 + lane;
      const unsigned ka = ea < e1 ? (unsigned)__ldg(&pcol[ea]) : PB_NONE;
      const unsigned kb = eb < e1 ? (unsigned)__ldg(&pcol[eb]) : PB_NONE;
      float4 qa = make_float4(0.f, 0.f, 0.f, 0.f), qb = qa;
      if(ka != PB_NONE) qa = __ldg(&in[ ka & PB_COL_MASK ]);
      if(kb != PB_NONE) qb = __ldg(&in[ kb & PB_COL_MASK ]);
#pragma unroll
      for(int h=0;h<2;h++)
      {
         const unsigned key = h ? kb : ka;
         const int r = key != PB_NONE ? (int)(key >> PB_ROW_SHIFT) : 32;
         float x = h ? qb.x : qa.x, y = h ? qb.y : qa.y, z = h ? qb.z : qa.z;
#pragma unroll
         for(int o=1;o<32;o<<=1)
         {
            const float xo = __shfl_up_sync(0xffffffffu, x, o);
            const float yo = __shfl_up_sync(0xffffffffu, y, o);
            const float zo = __shfl_up_sync(0xffffffffu, z, o);
            const int ro = __shfl_up_sync(0xffffffffu, r, o);
            if(lane >= o && ro == r)
            {
               x += xo; y += yo; z += zo;
            }
         }
         const int rn = __shfl_down_sync(0xffffffffu, r, 1);
         if(r < 32 && (lane == 31 || rn != r))
         {
            ax[r] += x; ay[r] += y; az[r] += z;
         }
         __syncwarp();
      }
   }

   if(v < nv)
   {
      const float4 p = __ldg(&in[v]);
      const int d = p1 - p0;
      if(d == 0)
         out[v] = p;
      else
      {
         const float inv = 1.0f / (float)d;
         out[v] = make_float4(p.x + omega * (ax[lane] * inv - p.x),
                              p.y + omega * (ay[lane] * inv - p.y),
                              p.z + omega * (az[lane] * inv - p.z), 0.f);
      }
   }
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

/* signed mean-ratio quality of one tet; *inv = det <= 0 (FP64 sign when the
   FP32 determinant is below the threshold or its error bound), *f64 = 1
   when the FP64 determinant was used */
__device__ __forceinline__ float tet_mean_ratio(const int4 e, const float4 *__restrict__ crd,
                                                float thr, int *inv, int *f64)
{
   const float4 a = __ldg(&crd[e.x]), b = __ldg(&crd[e.y]);
   const float4 c = __ldg(&crd[e.z]), d = __ldg(&crd[e.w]);
   const float abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
   const float acx = c.x - a.x, acy = c.y - a.y, acz = c.z - a.z;
   const float adx = d.x - a.x, ady = d.y - a.y, adz = d.z - a.z;
   const float m1 = acy * adz - acz * ady, m2 = acz * adx - acx * adz, m3 = acx * ady - acy * adx;
   float det = abx * m1 + aby * m2 + abz * m3;
   int pos = det > 0.f;
   const float perm = fabsf(abx) * (fabsf(acy * adz) + fabsf(acz * ady))
                    + fabsf(aby) * (fabsf(acz * adx) + fabsf(acx * adz))
                    + fabsf(abz) * (fabsf(acx * ady) + fabsf(acy * adx));
   *f64 = 0;
   if(fabsf(det) < fmaxf(thr, 9.5367431640625e-07f * perm))
   {
      const double Ax = a.x, Ay = a.y, Az = a.z;
      const double bx = b.x - Ax, by = b.y - Ay, bz = b.z - Az;
      const double cx = c.x - Ax, cy = c.y - Ay, cz = c.z - Az;
      const double dx = d.x - Ax, dy = d.y - Ay, dz = d.z - Az;
      const double dd = bx * (cy * dz - cz * dy) + by * (cz * dx - cx * dz) + bz * (cx * dy - cy * dx);
      det = (float)dd;
      pos = dd > 0.;
      *f64 = 1;
   }
   const float bcx = c.x - b.x, bcy = c.y - b.y, bcz = c.z - b.z;
   const float bdx = d.x - b.x, bdy = d.y - b.y, bdz = d.z - b.z;
   const float cdx = d.x - c.x, cdy = d.y - c.y, cdz = d.z - c.z;
   const float l2 = abx*abx + aby*aby + abz*abz + acx*acx + acy*acy + acz*acz
                  + adx*adx + ady*ady + adz*adz + bcx*bcx + bcy*bcy + bcz*bcz
                  + bdx*bdx + bdy*bdy + bdz*bdz + cdx*cdx + cdy*cdy + cdz*cdz;
   const float cb = cbrtf(0.5f * fabsf(det));          /* (3 |det| / 6)^(1/3) */
   const float q = 12.0f * cb * cb / l2;
   *inv = !pos;
   return pos ? q : -q;
}

/* per-thread accumulators of the statistics */
struct QAcc
{
   unsigned long long kmin, kmax;
   float s, c;
   unsigned ninv, nf64;
};

__device__ __forceinline__ void qacc_add(QAcc &a, float q, int t, int f64, unsigned *hist)
{
   int bin = (int)(q * 64.0f);
   bin = bin < 0 ? 0 : (bin > 63 ? 63 : bin);
   atomicAdd(&hist[bin], 1u);
   const unsigned k = mk_fkey(q);
   const unsigned long long a64 = ((unsigned long long)k << 32) | (unsigned)t;
   const unsigned long long b64 = ((unsigned long long)(~k) << 32) | (unsigned)t;
   a.kmin = a64 < a.kmin ? a64 : a.kmin;
   a.kmax = b64 < a.kmax ? b64 : a.kmax;
   const float tt = a.s + q, bp = tt - a.s;
   a.c += (a.s - (tt - bp)) + (q - bp);
   a.s = tt;
   a.nf64 += f64;
}

/* block reduction of the accumulators into the global statistics */
__device__ __forceinline__ void qacc_flush(QAcc &a, unsigned *hist, GmlxQualStats *st)
{
   __shared__ unsigned long long smin[MK_THREADS / 32], smax[MK_THREADS / 32];
   __shared__ double ssum[MK_THREADS / 32];
   __shared__ unsigned sinv[MK_THREADS / 32], sf64[MK_THREADS / 32];
   const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
   double dsum = (double)a.s + (double)a.c;
   unsigned long long kmin = a.kmin, kmax = a.kmax;
   unsigned ninv = a.ninv, nf64 = a.nf64;

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

/* non-blocking probe of the phase with the given parity */
__device__ __forceinline__ int mbar_try_wait(unsigned long long *bar, unsigned parity)
{
   unsigned ok;
   asm volatile("{\n\t.reg .pred p;\n\t"
                "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
   return (int)ok;
}

/* bounded wait: gives up after QK_SPIN polls (well under a second), so a
   lost transfer ends the kernel with an error flag instead of hanging it */
#define QK_SPIN (1 << 22)

__device__ __forceinline__ int mbar_wait_bounded(unsigned long long *bar, unsigned parity)
{
   for(int i=0;i<QK_SPIN;i++)
      if(mbar_try_wait(bar, parity))
         return 1;
   return 0;
}

#define QK_CHUNK  1024                     /* tets per stage: 16 KB */
#define QK_STAGES 3
#define QK_SMEM   (QK_STAGES * QK_CHUNK * 16)

/* The tetrahedron stream (16 bytes per tet, read once) is staged through
   shared memory by TMA bulk copies, QK_STAGES chunks ahead; the coordinate
   gathers (16 V bytes, L2 resident) are issued from registers, two tets per
   thread at a time.  Each warp handles 32 consecutive tets per pass, so its
   ballot is one word of the inverted-element bit flags. */
__global__ void __launch_bounds__(MK_THREADS, 4)
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
   QAcc a = { ~0ULL, ~0ULL, 0.f, 0.f, 0u, 0u };

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
         tma_bulk_g2s(stage + s * QK_CHUNK, tet + start, bytes, &bar[s]);
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

      /* 4 passes of 256 tets; a thread takes tets j and j + 512 together */
#pragma unroll 1
      for(int pass=0;pass<2;pass++)
      {
         const int j0 = pass * 2 * MK_THREADS + wid * 32 + lane;
         const int j1 = j0 + MK_THREADS;
         int inv0 = 0, inv1 = 0, f0 = 0, f1 = 0;
         float q0 = 0.f, q1 = 0.f;
         if(j0 < n) q0 = tet_mean_ratio(chunk[j0], crd, thr, &inv0, &f0);
         if(j1 < n) q1 = tet_mean_ratio(chunk[j1], crd, thr, &inv1, &f1);
         if(j0 < n)
         {
            qacc_add(a, q0, start + j0, f0, hist);
            if(qout) qout[start + j0] = q0;
         }
         if(j1 < n)
         {
            qacc_add(a, q1, start + j1, f1, hist);
            if(qout) qout[start + j1] = q1;
         }
         const unsigned w0 = __ballot_sync(0xffffffffu, inv0);
         const unsigned w1 = __ballot_sync(0xffffffffu, inv1);
         if(lane == 0)
         {
            const int b0 = pass * 2 * MK_THREADS + wid * 32, b1 = b0 + MK_THREADS;
            a.ninv += __popc(w0) + __popc(w1);
            if(flags && b0 < n) flags[ (start + b0) >> 5 ] = w0;
            if(flags && b1 < n) flags[ (start + b1) >> 5 ] = w1;
         }
      }

      /* every thread is done with stage s: refill it */
      __syncthreads();
      if(threadIdx.x == 0 && i + QK_STAGES < mine)
      {
         const int nstart = (blockIdx.x + (i + QK_STAGES) * gridDim.x) * QK_CHUNK;
         const unsigned bytes = (unsigned)(min(QK_CHUNK, nt - nstart) * 16);
         mbar_expect_tx(&bar[s], bytes);
         tma_bulk_g2s(stage + s * QK_CHUNK, tet + nstart, bytes, &bar[s]);
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
                                    const int *vt, const int *fixed, int *pdeg, int *pptr,
                                    int *err)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   point_count_kernel<<<nblk(nv, 128), 128, 0, st>>>(nv, (const int4 *)tet, ptr, vt, fixed, pdeg, err);
   scan_excl_kernel<int><<<1, 1024, 0, st>>>(pdeg, pptr, nv);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_point_fill(GmdCtx *ctx, const void *tet, int nv, const int *ptr,
                                   const int *vt, const int *pptr, int *pcol)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   point_fill_kernel<<<nblk(nv, 128), 128, 0, st>>>(nv, (const int4 *)tet, ptr, vt, pptr, pcol);
   return cudaGetLastError() == cudaSuccess;
}

extern "C" int gmd_mesh_laplace(GmdCtx *ctx, int nv, const int *pptr, const int *pcol,
                                const void *in, void *out, float omega)
{
   cudaStream_t st = (cudaStream_t)gmd_stream(ctx);
   laplace_warp_kernel<<<nblk(nv, MK_THREADS), MK_THREADS, 0, st>>>(nv, pptr, pcol,
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
                                float *qout, unsigned *flags, GmlxQualStats *st, int *err)
{
   static int attr_set = 0;
   cudaStream_t s = (cudaStream_t)gmd_stream(ctx);
   long long need = nblk(nt, QK_CHUNK);
   long long cap = (long long)gmd_num_sms(ctx) * 4;
   unsigned g = (unsigned)(need < cap ? need : cap);
   if(nt <= 0)
      return 1;
   if(!attr_set)
   {
      if(cudaFuncSetAttribute(tet_quality_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              QK_SMEM) != cudaSuccess)
         return 0;
      attr_set = 1;
   }
   tet_quality_tma_kernel<<<g, MK_THREADS, QK_SMEM, s>>>(nt, (const int4 *)tet, (const float4 *)crd,
                                                         thr, qout, flags, st, err);
   return cudaGetLastError() == cudaSuccess;
}
