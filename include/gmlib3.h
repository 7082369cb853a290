/*
 * gmlib3.h -- GB300-native GMlib, drop-in public interface.
 *
 * Same limits, flags, enums and prototypes as the reference header
 * (sources/gmlib3.h:46-122), so an existing C solver or mesher compiles and
 * links unchanged against libgmlib3.so.  The one difference: this header does
 * not include <CL/opencl.h> (reference sources/gmlib3.h:25-35); a client that
 * relied on that transitive include must include it itself.
 *
 * Each prototype cites the reference definition it replaces.
 */
#ifndef GMLIB3_H
#define GMLIB3_H

#include <stddef.h>

#ifdef WITH_LIBMESHB
#include <libmeshb8.h>
#endif

/* Limits and flags: sources/gmlib3.h:46-60 */
#define GmlMaxDat    100
#define GmlMaxMat    10
#define GmlMaxVec    10
#define GmlMaxKrn    100
#define GmlMaxSrcSiz 50000
#define GmlMaxStrSiz 200
#define MaxGpu       10
#define GmlRefFlag   1
#define GmlReadMode  2
#define GmlWriteMode 4
#define GmlVoyeurs   8
#define GmlManual    16
#ifndef MAX_WORKGROUP_SIZE
#define MAX_WORKGROUP_SIZE 1024
#endif

/* Enums: sources/gmlib3.h:62-70 */
enum  element_type   {GmlVertices, GmlEdges, GmlTriangles, GmlQuadrilaterals,
                      GmlTetrahedra, GmlPyramids, GmlPrisms, GmlHexahedra,
                      GmlMaxEleTyp};
enum  opencl_type    {GmlInt, GmlInt2, GmlInt4, GmlInt8, GmlInt16,
                      GmlFlt, GmlFlt2, GmlFlt4, GmlFlt8, GmlFlt16,
                      GmlDbl, GmlDbl2, GmlDbl4, GmlDbl8, GmlDbl16,
                      GmlByt, GmlByt2, GmlByt4, GmlByt8, GmlByt16,
                      GmlMaxOclTyp};
enum reduction_opp   {GmlMin, GmlMax, GmlSum, GmlL0, GmlL1, GmlL2, GmlLinf, GmlMaxRed};

#ifdef __cplusplus
extern "C" {
#endif

size_t   GmlInit              (int);                          /* gmlib3.c:385-454   */
void     GmlStop              (size_t);                       /* gmlib3.c:461-479   */
void     GmlListGPU           ();                             /* gmlib3.c:486-518   */
void    *GmlNewParameters     (size_t, int, char *);          /* gmlib3.c:525-564   */
int      GmlNewMeshData       (size_t, int, int);             /* gmlib3.c:571-639   */
int      GmlNewSolutionData   (size_t, int, int, int, char *);/* gmlib3.c:646-686   */
int      GmlNewLinkData       (size_t, int, int, int, char *);/* gmlib3.c:693-736   */
int      GmlNewMatrix         (size_t, int, int, int, void *, int *, int *, int); /* gmlib3.c:1175-1427 */
int      GmlNewVector         (size_t, int, int, void *, int);/* gmlib3.c:1434-1560 */
int      GmlFreeData          (size_t, int);                  /* gmlib3.c:1812-1834 */
int      GmlSetDataLine       (size_t, int, int, ...);        /* gmlib3.c:1841-1903 */
int      GmlGetDataLine       (size_t, int, int, ...);        /* gmlib3.c:1910-1961 */
void     GmlSetCompilerOptions(size_t, char *);               /* gmlib3.c:2206-2210 */
int      GmlCompileKernel     (size_t, char *, char *, int, int, ...); /* gmlib3.c:2217-2590 */
int      GmlLaunchKernel      (size_t, int);                  /* gmlib3.c:3064-3082 */
int      GmlReduceVector      (size_t, int, int, double *);   /* gmlib3.c:3229-3332 */
size_t   GmlGetMemoryUsage    (size_t);                       /* gmlib3.c:3648-3652 */
size_t   GmlGetMemoryTransfer (size_t);                       /* gmlib3.c:3659-3663 */
float    GmlGetMemoryAccess   (size_t);                       /* gmlib3.c:3670-3674 */
float    GmlGetFlops          (size_t);                       /* gmlib3.c:3681-3685 */
void     GmlDebugOn           (size_t);                       /* gmlib3.c:3691-3695 */
void     GmlDebugOff          (size_t);                       /* gmlib3.c:3697-3701 */
int      GmlExtractEdges      (size_t);                       /* gmlib3.c:3719-3873 */
int      GmlExtractFaces      (size_t);                       /* gmlib3.c:3880-4171 */
int      GmlSetNeighbours     (size_t, int);                  /* gmlib3.c:4178-4267 */
int      GmlCheckFP64         (size_t);                       /* gmlib3.c:3708-3712 */
int      GmlGetMeshInfo       (size_t, int, int *, int *);    /* gmlib3.c:4274-4300 */
int      GmlGetLinkInfo       (size_t, int, int, int *, int *, int *, int *); /* gmlib3.c:4307-4336 */
int      GmlSetDataBlock      (size_t, int, int, int, void *, void *, int *, int *); /* gmlib3.c:1968-2035 */
int      GmlGetDataBlock      (size_t, int, int, int, void *, void *, int *, int *); /* gmlib3.c:2042-2105 */
double   GmlGetKernelRunTime  (size_t, int);                  /* gmlib3.c:4343-4366 */
double   GmlGetReduceRunTime  (size_t, int);                  /* gmlib3.c:4373-4384 */
double   GmlGetWallClock      ();                             /* gmlib3.c:4391-4402 */
int      GmlUploadParameters  (size_t);                       /* gmlib3.c:2177-2185 */
int      GmlDownloadParameters(size_t);                       /* gmlib3.c:2192-2200 */
float    GmlEvaluateNumbering (size_t);                       /* gmlib3.c:4409-4442 */
void     GmlIncludeUserToolkit(size_t, char *);               /* gmlib3.c:4449-4453 */
int      GmlMultMatVec        (size_t, int, int, int);        /* gmlib3.c:3339-3404 */
int      GmlMultDiagMatVec    (size_t, int, int, int);        /* gmlib3.c:3582-3641 */
int      GmlAddVec3           (size_t, int, int, int, int);   /* gmlib3.c:3411-3488 */
int      GmlScaleVec          (size_t, int, double *);        /* gmlib3.c:3495-3527 */
int      GmlNormVec           (size_t, int, int, double *);   /* gmlib3.c:3534-3575 */

#ifdef WITH_LIBMESHB
int      GmlImportMesh        (size_t, char *, ...);          /* gmlib3.c:4480-4584 */
int      GmlExportSolution    (size_t, char *, ...);          /* gmlib3.c:4591-4738 */
#endif

#ifdef __cplusplus
}
#endif

#endif
