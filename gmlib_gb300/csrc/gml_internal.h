/*
 * gml_internal.h -- instance state of the GB300 GMlib host layer.
 *
 * The slot model follows the reference's public contract (sources/gmlib3.c:
 * 76-156): an instance is a calloc'd structure whose address is the size_t
 * handle; data, kernels, matrices and vectors live in 1-based slots limited by
 * GmlMaxDat/GmlMaxKrn/GmlMaxMat/GmlMaxVec; every datatype has a device buffer
 * and a host mirror; element types link to each other through the LnkMat /
 * LnkHgh / CntMat / SizMatHgh tables.  The device side is reached only through
 * gml_device.h.
 */
#ifndef GML_INTERNAL_H
#define GML_INTERNAL_H

#include <stddef.h>
#include <stdint.h>
#include "gmlib3.h"
#include "gml_device.h"

#define GML_MAXSLC     5
#define GML_MAXARG     (2 * GmlMaxDat + 8)
#define GML_TUNE_STEPS 16

enum gml_data_kind   { GmlArgDat, GmlRawDat, GmlLnkDat, GmlEleDat, GmlRefDat,
                       GmlMatDat = 100, GmlVecDat = 101 };
enum gml_mem_access  { GmlInternal, GmlInput, GmlOutput, GmlInout };
enum gml_kernel_kind { GmlKrnGenerated = 1, GmlKrnReduce, GmlKrnMatVec,
                       GmlKrnVecAdd, GmlKrnVecScale, GmlKrnVecDiag, GmlKrnVecNorm };

typedef struct
{
   int         use, AloTyp, MshTyp, LnkTyp, MemAcs, ItmTyp, RedIdx;
   int         NmbItm, ItmLen, ItmSiz, NmbLin, LinSiz;
   size_t      MemSiz;
   const char  *nam, *VoyNam;
   char        *src;
   void        *GpuMem, *CpuMem;
   int         pinned;
   void        *UpEvt;        /* event recorded after the last async upload */
   int         MirOld;        /* mirror still to be refreshed from the device (GmlxGetData) */
}GmlDatSct;

/* One generated-kernel argument; fields and meanings follow ArgSct of the
   reference (sources/gmlib3.c:91-96). */
typedef struct
{
   int         ArgIdx, MshTyp, DatIdx, LnkTyp, LnkIdx, LnkDir, CntIdx;
   int         LnkDeg, MaxDeg, NmbItm, ItmLen, ItmTyp, FlgTab;
   const char  *nam, *VoyNam;
}GmlArgSct;

typedef struct
{
   int         use, kind, idx, HghIdx, NmbLin[2], NmbDat;
   int         DatTab[ GML_MAXARG ];
   int         LibOp;                 /* library kernel: operation code */
   /* generated kernels */
   void        *module, *func;
   char        *name, *source;
   uint64_t    hash;
   int         MaxSiz, NumReg, lazy;
   /* block-size calibration (reference: sources/gmlib3.c:3142-3190) */
   int         GrpSiz, OptSiz, TunStp;
   double      TunTim[ GML_TUNE_STEPS ];
   void        *TunBeg, *TunEnd;
   /* per-launch timing (reference: events per launch, sources/gmlib3.c:3207) */
   int         NmbEvt, EvtCap;
   void        **EvtBeg, **EvtEnd;
   double      RunTim;                /* time of launches already folded in */
}GmlKrnSct;

typedef struct
{
   int         use, NmbLin, NmbBlk, BlkSiz, FltTyp, NmbSlc;
   int         MatSlc[ GML_MAXSLC + 1 ][5];
   int         KrnIdx;
   /* device BSR storage: row pointers, block columns, block values */
   int         *RowPtr, *ColIdx;
   void        *Val;
   float       FltOpp, MemAcc;
   void        *Sol;                  /* solver work space (gml_solver.c) */
}GmlMatSct;

typedef struct
{
   int         use, NmbLin, BlkSiz, FltTyp, FltSiz, idx, NmbValTyp, VecValSiz;
   int         AddKrnIdx, SclKrnIdx, MulDiaKrnIdx, NrmKrnIdx;
}GmlVecSct;

typedef struct
{
   int         NmbKrn, ParIdx, CurDev, DbgFlg, DblExt;
   int         TypIdx[ GmlMaxEleTyp ];
   int         RefIdx[ GmlMaxEleTyp ];
   int         NmbEle[ GmlMaxEleTyp ];
   int         LnkMat[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
   int         LnkHgh[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
   int         CntMat[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
   int         SizMatHgh[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
   int         RedKrn[ GmlMaxRed ];
   char        *UsrTlk, cflags[1024];
   size_t      MemSiz, MovSiz;
   float       MemAcc, FltOpp;
   GmlDatSct   dat[ GmlMaxDat + 1 ];
   GmlMatSct   mat[ GmlMaxMat + 1 ];
   GmlVecSct   vec[ GmlMaxVec + 1 ];
   GmlKrnSct   krn[ GmlMaxKrn + 1 ];
   GmdCtx      *dev;
   void        *RedScr;               /* reduction scratch (device) */
   size_t      RedScrSiz;
   int         TunOff;                /* 1: no calibration, fixed block size */
   int         TunBlk;                /* block size used when TunOff */
   int         LazyOff;               /* 1: always emit eager prologues */
   int         TimOff;                /* 1: no per-launch timing events */
   int         Offline;               /* 1: no GPU, code generation only */
   int         Quiet;                 /* 1: no informational messages */
   int         PinOff;                /* 1: pageable host mirrors (no page locking) */
   int         MirOff;                /* 1: whole-datatype sets write the device only and
                                         the host mirrors are never read (the request
                                         loop's own instances); mirrors stay pageable */
   char        **Names;               /* interned strings owned by the instance */
   int         NmbNames, CapNames;
   int         NmbMirOld;             /* datatypes whose MirOld is set */
   void        *ext;                  /* state of the native extensions */
   void        *bat;                  /* batched meshes (gml_batch.c) */
}GmlSct;

/* Every entry point starts here.  A bulk read (GmlxGetData) leaves the host
   mirror of its datatype to be refreshed; the next call on the instance
   refreshes it before anything can read the mirror or change the device
   data (gml_settle), so the mirror holds the data of the read, as after a
   download.  GmlxSetData and GmlxGetData, which rewrite or keep that data,
   use GETGMLPTR_NOSETTLE. */
#define GETGMLPTR_NOSETTLE(p,i)  GmlSct *p = (GmlSct *)(i)
#define GETGMLPTR(p,i)  GmlSct *p = (GmlSct *)(i); gml_settle(p)
void  gml_settle(GmlSct *gml);

/* shared tables (gml_tables.c) */
extern const int   GmlOclTypSiz[ GmlMaxOclTyp ];
extern const char *GmlOclTypStr[ GmlMaxOclTyp ];
extern const int   GmlTypVecSiz[ GmlMaxOclTyp ];
extern const int   GmlMshItmTyp[ GmlMaxEleTyp ];
extern const int   GmlEleNmbNod[ GmlMaxEleTyp ];
extern const int   GmlMshTypDim[ GmlMaxEleTyp ];
extern const char *GmlBalTypStr[ GmlMaxEleTyp ];
extern const char *GmlMshTypStr[ GmlMaxEleTyp ];
extern const char *GmlMshRefStr[ GmlMaxEleTyp ];
extern const int   GmlLenMatBas[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
extern const int   GmlLenMatMax[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
extern const int   GmlNmbTpoLnk[ GmlMaxEleTyp ][ GmlMaxEleTyp ];
extern const int   GmlNgbTyp[8];
extern const int   GmlItmNmbVer[8];
extern const int   GmlItmNmbEdg[8];
extern const int   GmlItmNmbFac[8];
extern const int   GmlItmEdgNod[8][12][2];
extern const int   GmlItmFacNod[8][6][4];
extern const int   GmlItmFacDeg[8][6];
extern const int   GmlOclVecPow[5];

/* gmlib3.c internals shared with the other host files */
int   gml_new_data_idx(GmlSct *gml);
int   gml_alloc_data(GmlSct *gml, GmlDatSct *dat);
int   gml_upload(GmlSct *gml, int idx);
int   gml_download(GmlSct *gml, int idx);
void  gml_wait_upload(GmlSct *gml, GmlDatSct *dat);
int   gml_new_kernel_slot(GmlSct *gml, int kind, const char *name);
void  gml_host_copy(void *dst, const void *src, size_t n);     /* gml_hostcopy.c */
int   gml_timed_launch(GmlSct *gml, GmlKrnSct *krn, unsigned grid, unsigned block, void **args);
void  gml_lib_timer_begin(GmlSct *gml, GmlKrnSct *krn);
void  gml_lib_timer_end(GmlSct *gml, GmlKrnSct *krn);
void  gml_get_cnt_vec(int siz, int *cnt, int *vec, int *typ);

/* topology (gml_topo.c) */
int   gml_new_ball_data(GmlSct *gml, int SrcTyp, int DstTyp,
                        const char *BalNam, const char *DegNam, const char *VoyNam);

/* code generation (gml_codegen.c) and dialect rewriting (gml_dialect.c) */
int   gml_generate(char **out, const char *PrcNam, int MshTyp, int NmbArg,
                   const GmlArgSct *ArgTab, const char *KrnSrc, const char *UsrTlk,
                   const char *ParSrc, int lazy);
char *gml_rewrite_opencl(const char *src);
char *gml_nvrtc_options(const char *cflags);
uint64_t gml_hash64(const void *p, size_t n, uint64_t seed);

#endif
