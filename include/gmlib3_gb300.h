/*
 * gmlib3_gb300.h -- extensions of the GB300-native GMlib.
 *
 * Everything here is additive: gmlib3.h alone is the drop-in interface of the
 * reference.  These entry points give foreign-function callers non-variadic
 * forms of the variadic calls, expose the native mesh kernels, the solvers,
 * the batched and served paths, and the controls of the launch machinery.
 * Each declaration names the reference function it extends, or says that it
 * has no counterpart in the reference.
 *
 * Environment variables read by the library (none changes a result):
 *   GML_TUNE      at GmlInit: <= 0 turns block-size calibration off (block
 *                 256), >= 32 fixes the block size; as GmlxSetTuning.
 *   GML_LAZY      at GmlInit: 0 makes GmlCompileKernel always emit the
 *                 reference's eager gather prologue; as GmlxSetLazy(0).
 *   GML_DIRECT    at GmlInit: 0 keeps whole-datatype transfers on the staged
 *                 path (host mirror, then DMA) instead of the one-kernel copy.
 *   GML_CACHE_DIR a directory where compiled generated kernels are also kept
 *                 on disk between processes (unset: in memory only).
 *   GML_CG_TRACE  1 prints each GmlxSolveCG phase's wall and device time, 2
 *                 each kernel's (timed one by one, without graphs).
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
   to the datatype size (lines x line size).  Bulk counterparts of
   GmlSetDataLine / GmlGetDataLine (gmlib3.c:1841, 1910): the host mirror
   that the line accessors read holds the data set or downloaded.  Set has
   consumed buf when it returns; it uploads asynchronously from the mirror,
   or, for a large datatype on an idle instance whose device can address
   buf (pinned memory, or pageable memory where the device has pageable
   memory access), copies buf to the device and the mirror with one kernel
   before returning.  Get is blocking; on the kernel path it writes buf
   only, and the mirror is downloaded at the next call on the instance,
   before that call reads the mirror or changes the device data (a Set of
   the same datatype, which rewrites the mirror, skips the download). */
int      GmlxSetData          (size_t, int DatIdx, const void *buf, size_t bytes);
int      GmlxGetData          (size_t, int DatIdx, void *buf, size_t bytes);

/* Datatype index holding the lines of a GmlNewVector vector (padded lines
   of the vector's lane count), for GmlxGetData / GmlxSetData.  Extends
   GmlNewVector (gmlib3.c:1434-1560), which keeps that index private. */
int      GmlxVectorData       (size_t, int VecIdx);

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
 * make that first call outside any stream capture.  The looked-up address
 * is kept for the life of the process: after cudaDeviceReset on a device
 * the entry point must not be called on that device again.  Calls on one
 * stream run one after the other and are safe; calls that overlap on one
 * device (two streams, two host threads) share the scratch and race.
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
   1 vertices with a non-zero reference fixed (the device copy of the
   references, as the kernels see them), 2 vertices on the topological
   boundary (faces owned by one tet) fixed.  Returns 1, or 0 on error (a ball
   of more than 64 points). */
int      GmlxMeshSetup        (size_t, int fix);

/* Number of ball-of-points entries stored (sum of slice widths x 32) and
   used (sum of degrees). */
int      GmlxMeshBallInfo     (size_t, long long *stored, long long *used, int *maxdeg);

/* The ball-of-points layout sorts rows by ball size inside windows of 32,
   64, 128 or 256 consecutive vertices: wider windows pad less, narrower ones
   keep rows nearer their Hilbert neighbours.  GmlxSetBallWindow fixes the
   window of the next GmlxMeshSetup (0: the tuning table's choice for meshes
   of that size, else 256); GmlxBallWindow returns the window in use.
   GmlxMeshTune times nsweeps sweeps with each window on the current mesh,
   keeps the fastest (rebuilding the layout; coordinates restored), records
   it in the tuning table and returns it (0 on error).  The results do not
   depend on the window. */
int      GmlxSetBallWindow    (size_t, int window);
int      GmlxBallWindow       (size_t);
int      GmlxMeshTune         (size_t, int nsweeps, float omega);

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
 * Batched meshes: many tetrahedral meshes of uneven size in one instance,
 * smoothed and measured together.  No counterpart in the reference (one
 * mesh per instance, one launch per kernel call, gmlib3.c:3064-3222).
 * ------------------------------------------------------------------------- */

enum GmlxBatchMode { GmlxBatchQueue = 0, GmlxBatchLoop = 1 };

/* Declare NmbMsh meshes (vertex and tet counts, edge length h of each for
   the FP64 determinant threshold 1e-6 h^3).  Creates the instance's vertex
   and tetrahedron datatypes holding all meshes packed (each mesh's vertices
   start on a multiple of 256); the instance must not have them yet. */
int      GmlxBatchCreate      (size_t, int NmbMsh, const int *NmbVer, const int *NmbTet,
                               const double *h);

/* Mesh MshIdx (0-based): crd 4 floats per vertex, ref one int per vertex
   (NULL: 0), tet 4 local vertex indices per tet. */
int      GmlxBatchSetMesh     (size_t, int MshIdx, const float *crd, const int *ref,
                               const int *tet);

/* Upload the packed meshes and build their topology (GmlxMeshSetup on the
   packed mesh, fix as there). */
int      GmlxBatchSetup       (size_t, int fix);

/* nsweeps Jacobi sweeps then the quality statistics of every mesh.
   GmlxBatchQueue: one persistent launch drains a (mesh, range) tile queue,
   captured once as a CUDA graph and replayed; GmlxBatchLoop: the per-mesh
   launch loop.  res (may be NULL) receives NmbMsh results, tet indices local
   to each mesh.  The coordinates are updated in place. */
int      GmlxBatchRun         (size_t, int nsweeps, float omega, int mode, GmlxQuality *res);

/* The queue's dependency wait: a tile of sweep s + 1 waits on the device
   until every sweep-s tile of its mesh is done, at most `spin` tries of
   about 256 ns (0: the default 2^22, about 1 s); past that the launch stops,
   GmlxBatchRun (given res) returns 0 and prints why, and the instance can
   run again.  hold > 0 adds that many never-finished tiles to the first
   sweep of mesh 0, so that its second-sweep tiles wait until the limit: a
   host-side way to exercise the timeout (hold 0 restores the queue).  The
   coordinates of a stopped run are incomplete.  No counterpart in the
   reference. */
int      GmlxBatchSetWaitLimit(size_t, int spin, int hold);

/* Coordinates (4 floats per vertex) and inverted-element flags of a mesh. */
int      GmlxBatchGetMesh     (size_t, int MshIdx, float *crd);
int      GmlxBatchFlags       (size_t, int MshIdx, unsigned *flags, size_t nwords);

/* Time the queue on the packed meshes with tiles claimed per block or per
   warp, several tile sizes and grid sizes, and keep the fastest (the
   coordinates are restored afterwards); read back the choice (WarpTiles 1:
   per-warp tiles) and the tile count. */
int      GmlxBatchTune        (size_t, int nsweeps, float omega);

/* Set the queue's configuration by hand: tiles per warp (1) or per block
   (0), slices per sweep tile, tets per quality tile (a multiple of 32),
   grid (0: keep). */
int      GmlxBatchSetTiles    (size_t, int WarpTiles, int TileSlices, int TileTets, int grid);
int      GmlxBatchInfo        (size_t, int *TileSlices, int *TileTets, int *grid, int *ntile,
                               int *WarpTiles);

/* ---------------------------------------------------------------------------
 * Request loop: quality, smoothing and solve requests on registered meshes
 * and systems, served from one GPU with continuous batching against a
 * device-memory budget.  No counterpart in the reference.
 * ------------------------------------------------------------------------- */

enum GmlxReqKind   { GmlxReqQuality = 0, GmlxReqSmooth = 1, GmlxReqSolve = 2 };
enum GmlxServeMode { GmlxServeBatching = 0, GmlxServeSerial = 1 };

typedef struct
{
   int      kind, target;       /* GmlxReqKind; index from GmlxServeAdd* */
   double   arrival;            /* seconds from the start of the run, non-decreasing */
   double   start, finish;      /* filled in: seconds from the start of the run */
   int      status;             /* filled in: 1 done, 0 failed */
   int      NmbIte;             /* solve: CG iterations */
   double   RelRes;             /* solve: |b - A x| / |b| */
   GmlxQuality qal;             /* quality, or quality after the 10th smoothing sweep */
}GmlxRequest;

typedef struct
{
   int      completed, failed, loads, evictions;
   double   seconds, throughput, mean, p50, p99, max, peak_bytes;
}GmlxServeStats;

/* Server on device dev with a device-memory budget (bytes) for resident
   targets and NmbSlot concurrent requests (1..64).  It runs a small mesh and
   a small system through every request kind before returning (device
   context and kernels loaded up front, a few hundred ms on a cold process). */
size_t   GmlxServeNew         (int dev, double BudgetBytes, int NmbSlot);

/* Register a tet mesh (crd 4 floats per vertex, ref per vertex or NULL;
   vertices with a non-zero ref stay fixed when smoothing; h for the FP64
   determinant threshold) or a 3x3-block SPD system (CSR as GmlNewMatrix,
   FP64 values, rhs 3 per row).  The arrays are used in place and must
   outlive the server.  Returns the target index, or -1. */
int      GmlxServeAddMesh     (size_t srv, int NmbVer, const float *crd, const int *ref,
                               int NmbTet, const int *tet, double h);
int      GmlxServeAddSystem   (size_t srv, int NmbLin, int NmbBlk, const int *lin,
                               const int *col, const double *val, const double *rhs);

/* Serve NmbReq requests arriving at their times.  GmlxReqQuality: mean-ratio
   statistics; GmlxReqSmooth: 10 sweeps (omega 1) each followed by the
   statistics, the mesh's registered coordinates restored afterwards;
   GmlxReqSolve: FP32 CG in FP64 refinement to 1e-10.  GmlxServeBatching:
   continuous batching over NmbSlot slots with resident targets;
   GmlxServeSerial: one request at a time, each on a fresh instance.
   Returns 1 when the loop ran (individual failures are in status). */
int      GmlxServeRun         (size_t srv, GmlxRequest *req, int NmbReq, int mode,
                               GmlxServeStats *st);

/* Estimated device bytes of a target when resident (what admission
   charges against the budget); number of resident targets and their bytes. */
double   GmlxServeTargetBytes (size_t srv, int target);
int      GmlxServeResident    (size_t srv, double *bytes);
void     GmlxServeFree        (size_t srv);

/* ---------------------------------------------------------------------------
 * Conjugate gradients on a GmlNewMatrix block matrix.  No counterpart in the
 * reference: its LinearSolver example runs a fixed-point loop with
 * GmlMultMatVec / GmlMultDiagMatVec / GmlAddVec3
 * (examples/LinearSolver/LinearSolver.c:300-338).
 * ------------------------------------------------------------------------- */

enum GmlxCgMode { GmlxCgFp64 = 0, GmlxCgMixed = 1 };

typedef struct
{
   int      NmbIte;        /* CG iterations (FP32 iterations in GmlxCgMixed) */
   int      NmbOut;        /* refinement steps (1 for GmlxCgFp64) */
   double   RelRes;        /* |b - A x| / |b|, recomputed in FP64 at the end */
   double   Seconds;       /* device time of the solve (CUDA events) */
}GmlxSolveInfo;

/* Solve A x = b for a symmetric positive definite matrix MatIdx (GmlDbl,
   diagonal blocks stored in the matrix), RhsIdx and SolIdx being GmlDbl
   vectors of the matrix's size and block size.  x starts at 0.
   GmlxCgFp64: CG in FP64.  GmlxCgMixed: CG in FP32 (FP32 copy of the matrix,
   FP32 vectors, FP64 dot products) inside FP64 iterative refinement with
   the true residual b - A x in FP64.  Stops when |b - A x| <= tol |b| or after
   MaxIte CG iterations.  Returns 1 when converged, 0 when not, negative on
   errors (-1 matrix, -2 vectors, -3 types or sizes, -4 arguments, -5 memory,
   -6 device, -7 breakdown: p.Ap <= 0). */
int      GmlxSolveCG          (size_t, int MatIdx, int RhsIdx, int SolIdx, int mode,
                               double tol, int MaxIte, GmlxSolveInfo *info);

/* Symmetric positive definite 3x3-block system on the vertex graph of the
   n^3-hex cube of GmlxCubeMesh (no jitter, Hilbert order): row v holds v and
   the vertices sharing a tet with v, columns ascending; off-diagonal block
   entries uniform in [-1, 0] from the seed, A_ji = A_ij^T; diagonal block
   diag(1 + sum of |off-diagonal entries| of each scalar row); rhs uniform in
   [-1, 1].  lin has NmbLin + 1 entries, col NmbBlk, val 9 NmbBlk (row-major
   blocks), rhs 3 NmbLin (may be NULL).  Returns 1, or 0 on bad sizes. */
int      GmlxCubeSpdSizes     (int n, int split, int *NmbLin, int *NmbBlk);
int      GmlxCubeSpdMatrix    (int n, int split, uint64_t seed, int *lin, int *col,
                               double *val, double *rhs);

/* ---------------------------------------------------------------------------
 * Mesh files without libMeshb.  GmlImportMesh / GmlExportSolution (declared
 * in gmlib3.h under WITH_LIBMESHB as in the reference, gmlib3.c:4480-4738)
 * are always provided, on the library's own reader and writer of the Gamma
 * mesh format (.meshb binary versions 1-4, .mesh ASCII).  These are their
 * non-variadic forms plus a mesh writer.
 * ------------------------------------------------------------------------- */

/* Read the keywords of KwdTab (libMeshb codes: Vertices 4, Edges 5,
   Triangles 6, Quadrilaterals 7, Tetrahedra 8, Prisms 9, Hexahedra 10,
   Pyramids 49) and create their mesh datatypes.  Returns NmbKwd, 0 when the
   file cannot be read. */
int      GmlxImportMesh       (size_t, const char *MshNam, int NmbKwd, const int *KwdTab);

/* Write the mesh types of TypTab (GmlVertices ...) to a .meshb (binary
   version 2) or .mesh (ASCII) file.  Returns 1. */
int      GmlxExportMesh       (size_t, const char *MshNam, int NmbTyp, const int *TypTab);

/* Write float datatypes as ASCII solution fields (.sol), one SolAt keyword
   per mesh type.  Returns the number of keywords written. */
int      GmlxExportSolution   (size_t, const char *SolNam, int NmbDat, const int *DatTab);

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

/* Stable partition of the vertices by the number of tetrahedra they belong
   to: those in at most BalSiz tetrahedra first, then the others, each group
   keeping its order (call it after GmlxHilbertRenumber).  This is the
   numbering the reference's ball tables expect (low degrees first,
   Documentation/GMlib3_en.tex:401); BalSiz is the base ball width, 32 for
   vertex -> tetrahedron balls.  Arrays are permuted in place; VerPrm
   (optional) receives the new index of each old vertex.  Returns the size
   of the first group, or -1 on bad arguments (a tet index out of range). */
int      GmlxDegreeSort       (int NmbVer, float *crd, int *ref, int NmbTet, int *tet,
                               int BalSiz, int *VerPrm);

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
int      gmlx_tune_get(const char *kind, uint64_t hash, long long count, int nsm);
void     gmlx_tune_set(const char *kind, uint64_t hash, long long count, int nsm, int val);
#endif

#endif
