/*
 * gmlib3_gb300.h -- extensions of the GB300-native GMlib.
 *
 * Everything here is additive: gmlib3.h alone is the drop-in interface of the
 * reference.  These entry points give foreign-function callers non-variadic
 * forms of the variadic calls, expose the native mesh kernels, the solvers,
 * the batched and served paths, and the controls of the launch machinery.
 * Each declaration names the reference function it extends, or says that it
 * has no counterpart in the reference.
 */
#ifndef GMLIB3_GB300_H
#define GMLIB3_GB300_H

#include <stddef.h>
#include <stdint.h>
#include "gmlib3.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Instance control
 * ------------------------------------------------------------------------- */

/* Instance without a GPU: datatypes live in host memory, GmlCompileKernel
   generates and compiles (NVRTC, sm_103a) but nothing can be launched.  For
   checking generated kernels on machines without a GPU.  No counterpart in
   the reference. */
size_t   GmlxInitOffline      (void);

/* 0 disables the per-launch CUDA events behind GmlGetKernelRunTime (needed
   while capturing CUDA graphs by hand); 1 (default) enables them.  Extends
   the reference's event recording of RunOclKrn (gmlib3.c:3207). */
int      GmlxSetTiming        (size_t, int on);

/* 0 disables block-size calibration (every generated kernel then uses
   `block`, or 256 when block <= 0); 1 re-enables it.  Extends the reference's
   work-group calibration (gmlib3.c:3142-3190). */
int      GmlxSetTuning        (size_t, int on, int block);

/* Block size chosen for a generated kernel (0 while still calibrating). */
int      GmlxKernelBlockSize  (size_t, int KrnIdx);

/* Generated CUDA source of a kernel (NULL for library kernels) and whether
   its uplink gathers are lazy accessors (1) or eager arrays (0). */
const char *GmlxKernelSource  (size_t, int KrnIdx);
int      GmlxKernelIsLazy     (size_t, int KrnIdx);

/* Number of 32-bit registers per thread of a generated kernel. */
int      GmlxKernelRegisters  (size_t, int KrnIdx);

/* 0: generated uplink gathers use the reference's eager per-thread arrays;
   1 (default): lazy accessors, eager only when the body needs arrays. */
int      GmlxSetLazy          (size_t, int on);

/* Datatype indices of the link between two mesh types built by
   GmlCompileKernel (base ball table, degree table, high-degree table; 0 when
   absent).  Extends GmlGetLinkInfo (gmlib3.c:4307-4336). */
int      GmlxLinkData         (size_t, int SrcTyp, int DstTyp, int *BalIdx, int *DegIdx,
                               int *HghIdx);

/* Wait for all work of the instance. */
int      GmlxSynchronize      (size_t);

/* CUDA stream (cudaStream_t) that orders all work of the instance. */
void    *GmlxStream           (size_t);

/* CUDA events recorded on the instance stream, for timing device work from
   foreign callers: create, record, elapsed seconds between two recorded
   events (waits for the second), destroy.  No counterpart in the reference
   (its per-kernel events are internal, gmlib3.c:3207-3208). */
void    *GmlxEventCreate      (void);
int      GmlxEventRecord      (size_t, void *evt);
double   GmlxEventElapsed     (void *beg, void *end);
void     GmlxEventDestroy     (void *evt);

/* ---------------------------------------------------------------------------
 * Non-variadic forms for foreign-function interfaces
 * ------------------------------------------------------------------------- */

/* GmlCompileKernel (gmlib3.c:2217) with the (index, flags, link) triplets
   given as three arrays of NmbTyp entries. */
int      GmlxCompileKernelV   (size_t, const char *src, const char *name, int MshTyp,
                               int NmbTyp, const int *IdxTab, const int *FlgTab,
                               const int *LnkTab);

/* Whole-datatype copies between a caller buffer and a datatype, bytes equal
   to the datatype size (lines x line size).  Set uploads (asynchronously),
   Get downloads (blocking).  Bulk counterparts of GmlSetDataLine /
   GmlGetDataLine (gmlib3.c:1841, 1910). */
int      GmlxSetData          (size_t, int DatIdx, const void *buf, size_t bytes);
int      GmlxGetData          (size_t, int DatIdx, void *buf, size_t bytes);

/* Size in bytes, number of lines and device address of a datatype. */
size_t   GmlxDataBytes        (size_t, int DatIdx);
int      GmlxDataLines        (size_t, int DatIdx);
void    *GmlxDevicePtr        (size_t, int DatIdx);

/* ---------------------------------------------------------------------------
 * Reductions with indices.  No counterpart in the reference (GmlReduceVector
 * returns values only).  Ties go to the smallest line index.
 * ------------------------------------------------------------------------- */
int      GmlxReduceArg        (size_t, int DatIdx, float *MinVal, int *MinIdx,
                               float *MaxVal, int *MaxIdx);

/* ---------------------------------------------------------------------------
 * Reduction that allocates nothing.  No counterpart in the reference.
 *
 * GmlReduceVector needs an instance (GmlInit allocates its buffers) and a
 * datatype.  Some callers cannot allocate device memory at the point where
 * they need a reduction: a host whose own memory pool has reserved the free
 * device memory (cudaMalloc then fails), or a time-critical loop that must
 * not take the device-wide synchronisation cudaFree implies.  They pass a
 * device pointer of their own instead.
 *
 * RedOpp is GmlMin..GmlLinf, computed as GmlReduceVector does (FP64
 * combine; L2 is the sum of squares, no square root); *res (host) receives
 * the result, and NmbLin = 0 gives the operation's identity.  The call
 * launches on `stream` (a cudaStream_t, NULL for the legacy default stream)
 * of the CURRENT device, where DevVec must live, and returns when the result
 * is on the host: 1 on success, 0 on failure with a one-line message on
 * stderr.  NmbLin above GMLX_NOALLOC_MAX_LINES is rejected that way.
 *
 * Scratch: a static device array of GMLX_NOALLOC_SCRATCH_BYTES, one per
 * device.  It is zero when the library's device code loads and every
 * completed call leaves it in that state; nothing needs clearing by the
 * caller.  Its address is looked up on the first call on each device, so
 * make that first call outside any stream capture.  Calls on one stream run
 * one after the other and are safe; calls that overlap on one device (two
 * streams, two host threads) share the scratch and race.
 * ------------------------------------------------------------------------- */
#define GMLX_NOALLOC_MAX_LINES      2147483647      /* 32-bit line index */
#define GMLX_NOALLOC_SCRATCH_BYTES  8208            /* (2 + 1024) x 8 bytes */
int      GmlxReduceNoAlloc    (const float *DevVec, size_t NmbLin, int RedOpp,
                               double *res, void *stream);

/* ---------------------------------------------------------------------------
 * Native tetrahedral mesh kernels: Laplacian smoothing over the ball of
 * points and mean-ratio quality statistics.  They work on the instance's
 * GmlVertices and GmlTetrahedra datatypes in place, without generated
 * scatter/gather pairs.  No counterpart in the reference API (its
 * NodeSmoothing example smooths through generated kernels,
 * examples/NodeSmoothing/NodeSmoothing.c:128-171).
 * ------------------------------------------------------------------------- */

/* Device-side statistics of one quality pass (keys pack an order-preserving
   image of the float quality in the high word and the tet index in the low
   word; MaxKey stores the complemented image). */
typedef struct
{
   unsigned long long MinKey, MaxKey;
   double   Sum;
   unsigned NmbInv, NmbF64;
   unsigned Hist[64];
}GmlxQualStats;

/* Decoded statistics. */
typedef struct
{
   float    MinQal, MaxQal;       /* signed mean-ratio quality */
   int      MinIdx, MaxIdx;       /* smallest index on ties */
   double   SumQal;               /* FP64 sum of the qualities */
   unsigned NmbInv;              /* tets with det <= 0 (FP64 sign) */
   unsigned NmbF64;              /* tets whose sign needed the FP64 determinant */
   unsigned Hist[64];            /* bin = clamp(floor(64 q), 0, 63) */
}GmlxQuality;

/* Build the topology the native kernels need (vertex->tet lists and the
   ball of points in SELL-32 form) on the GPU.  fix: 0 no vertex fixed,
   1 vertices with a non-zero reference fixed, 2 vertices on the topological
   boundary (faces owned by one tet) fixed.  Returns 1, or 0 on error (a ball
   of more than 64 points). */
int      GmlxMeshSetup        (size_t, int fix);

/* Number of ball-of-points entries stored (sum of slice widths x 32) and
   used (sum of degrees). */
int      GmlxMeshBallInfo     (size_t, long long *stored, long long *used, int *maxdeg);

/* nsweeps Jacobi sweeps x <- x + omega (mean of the ball of points - x) of
   the vertex coordinates, in place; fixed vertices do not move. */
int      GmlxSmooth           (size_t, int nsweeps, float omega);

/* Mean-ratio quality q = 12 (3|V|)^(2/3) / sum of squared edge lengths of
   every tet, negative when det <= 0; determinants whose FP32 magnitude is
   below max(1e-6 h^3, the FP32 error bound) are recomputed in FP64.  QalIdx
   (optional, 0 for none) receives q per tet (float tet solution).  The
   inverted-element bit flags (bit t%32 of word t/32) are kept and returned
   by GmlxInvertedFlags. */
int      GmlxQualityStats     (size_t, double h, int QalIdx, GmlxQuality *res);
int      GmlxInvertedFlags    (size_t, unsigned *flags, size_t nwords);

/* The smoothing workload as one unit: nsweeps times (one sweep, then the
   quality statistics), captured once as a CUDA graph and replayed; res
   receives nsweeps results (may be NULL). */
int      GmlxSmoothQualityLoop(size_t, int nsweeps, float omega, double h, GmlxQuality *res);

/* Algorithmic (unique) bytes of one sweep and of one quality pass for the
   current mesh, the numerators of the roofline figures. */
int      GmlxMeshBytes        (size_t, double *sweep_bytes, double *quality_bytes);

/* ---------------------------------------------------------------------------
 * Synthetic meshes and renumbering (host utilities).  No counterpart in the
 * reference library; the reference renumbers meshes with an external Hilbert
 * tool (README.md, todolist.md:44).
 * ------------------------------------------------------------------------- */

/* Unit cube of n^3 hexahedra split into 6 tetrahedra each.  split = 0: all
   hexes split around the same main diagonal (Kuhn/Freudenthal, interior
   vertex degree 24); split = 1: the diagonal of each hex goes through its
   all-even corner (reflected split, ragged degrees 16/48).  Interior vertices
   are jittered uniformly by +-jitter*h (h = 1/n) from a seed; boundary
   vertices get reference 1, interior 0.  crd receives 4 floats per vertex
   (w = 0), tet 4 ints per tetrahedron, ref one int per vertex.  Returns 1. */
void     GmlxCubeSizes        (int n, int *NmbVer, int *NmbTet);
int      GmlxCubeMesh         (int n, int split, double jitter, uint64_t seed,
                               float *crd, int *tet, int *ref);

/* Renumber vertices along a 3-D Hilbert curve of their coordinates and
   tetrahedra along the curve of their centroids; arrays are permuted in
   place.  VerPrm (optional) receives the new index of each old vertex. */
int      GmlxHilbertRenumber  (int NmbVer, float *crd, int *ref, int NmbTet, int *tet,
                               int *VerPrm);

#ifdef __cplusplus
}
#endif

/* internal helpers shared by the host files (not part of the public API) */
#ifdef GML_INTERNAL_H
const char *gmlx_intern(GmlSct *gml, const char *s);
int      gmlx_cache_lookup(const char *src, const char *opts, const char *name, void **cubin, size_t *size);
void     gmlx_cache_store(const char *src, const char *opts, const char *name, const void *cubin, size_t size);
int      gmlx_timing_off(GmlSct *gml);
void     gmlx_release_extensions(GmlSct *gml);
#endif

#endif
