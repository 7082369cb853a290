/*
 * gmlib3.c -- GB300-native GMlib host layer (C99).
 *
 * Implements the gmlib3.h API (reference sources/gmlib3.c) on top of the thin
 * CUDA ABI of gml_device.h.  Behaviour follows the reference function by
 * function: slot allocation, implicit whole-buffer upload when the last line
 * is set and download when line 0 is read, argument tables of generated
 * kernels, error codes and messages.  What changes is the execution model:
 *
 *   - one non-blocking CUDA stream per instance and no device drain before
 *     each launch (the reference calls clFinish before every enqueue,
 *     sources/gmlib3.c:3200); every host-visible read point (GmlGetData*,
 *     GmlReduceVector, GmlNormVec, GmlGetKernelRunTime) synchronises;
 *   - host mirrors of large datatypes are pinned, so uploads are truly
 *     asynchronous; a mirror is not rewritten while its upload is in flight;
 *   - generated kernels are CUDA C++ compiled by NVRTC for sm_103a;
 *   - library kernels (reductions, block sparse mat-vec, vector algebra) are
 *     hand-written CUDA.
 *
 * Deviations from the reference that fix defects are listed where they occur
 * and gathered in the design notes of the repository.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdarg.h>
#include <math.h>
#include <float.h>
#include <sys/time.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"
#include "gml_linalg.h"

#define MB 1048576
#define PIN_THRESHOLD (1 << 20)

static const char *sep = "\n\n############################################################\n";

/* ========================================================================= */
/* data slots                                                                 */
/* ========================================================================= */

int gml_new_data_idx(GmlSct *gml)
{
   for(int i=1;i<=GmlMaxDat;i++)
      if(!gml->dat[i].use)
      {
         memset(&gml->dat[i], 0, sizeof(GmlDatSct));
         gml->dat[i].use = 1;
         return i;
      }
   return 0;
}

int gml_alloc_data(GmlSct *gml, GmlDatSct *dat)
{
   dat->GpuMem = gmd_alloc(gml->dev, dat->MemSiz);

   if(!dat->GpuMem)
   {
      printf("Cannot allocate %zd MB on the GPU (%zd MB already used)\n",
             dat->MemSiz / MB, gml->MemSiz / MB);
      return 0;
   }

   if(dat->MemAcs != GmlInternal)
   {
      if(!gml->PinOff && !gml->MirOff && dat->AloTyp != GmlArgDat && dat->MemSiz >= PIN_THRESHOLD
      && (dat->CpuMem = gmd_host_alloc(dat->MemSiz)))
         dat->pinned = 1;
      else
      {
         dat->pinned = 0;
         dat->CpuMem = calloc(1, dat->MemSiz ? dat->MemSiz : 1);
      }

      if(!dat->CpuMem)
      {
         printf("Cannot allocate %zd MB on the CPU\n", dat->MemSiz / MB);
         gmd_free(gml->dev, dat->GpuMem);
         dat->GpuMem = NULL;
         return 0;
      }
   }

   gml->MemSiz += dat->MemSiz;
   return 1;
}

static void release_data(GmlSct *gml, GmlDatSct *dat)
{
   if(dat->UpEvt)
   {
      gmd_event_wait(dat->UpEvt);
      gmd_event_free(dat->UpEvt);
   }
   if(dat->GpuMem)
      gmd_free(gml->dev, dat->GpuMem);
   if(dat->CpuMem)
   {
      if(dat->pinned)
         gmd_host_free(dat->CpuMem);
      else
         free(dat->CpuMem);
   }
   gml->MemSiz -= dat->MemSiz;
   memset(dat, 0, sizeof(GmlDatSct));
}

void gml_wait_upload(GmlSct *gml, GmlDatSct *dat)
{
   (void)gml;
   if(dat->UpEvt && dat->pinned)
      gmd_event_wait(dat->UpEvt);
}

/* Copy a whole host mirror to the device (reference UploadData, :2112-2139).
   The reference adds the size to the transfer counter twice (inside and in
   every caller); here it is counted once. */
int gml_upload(GmlSct *gml, int idx)
{
   GmlDatSct *dat;

   if(idx < 1 || idx > GmlMaxDat)
      return 0;

   dat = &gml->dat[ idx ];

   if(!dat->GpuMem || !dat->CpuMem || dat->MemAcs == GmlOutput)
      return 0;

   if(!gmd_h2d_async(gml->dev, dat->GpuMem, dat->CpuMem, dat->MemSiz))
   {
      printf("Uploading the data to the GPu failed with error %s\n", gmd_last_error(gml->dev));
      return 0;
   }

   if(dat->pinned)
   {
      if(!dat->UpEvt)
         dat->UpEvt = gmd_event_new();
      if(dat->UpEvt)
         gmd_event_record(gml->dev, dat->UpEvt);
   }

   gml->MovSiz += dat->MemSiz;
   return (int)(dat->MemSiz > 0x7fffffff ? 0x7fffffff : dat->MemSiz);
}

/* Blocking copy of a whole device buffer to its host mirror (reference
   DownloadData, :2146-2170). */
int gml_download(GmlSct *gml, int idx)
{
   GmlDatSct *dat;

   if(idx < 1 || idx > GmlMaxDat)
      return 0;

   dat = &gml->dat[ idx ];

   if(!dat->GpuMem || !dat->CpuMem)
      return 0;

   if(!gmd_d2h(gml->dev, dat->CpuMem, dat->GpuMem, dat->MemSiz))
   {
      printf("Downloading the data from the GPu failed with error %s\n", gmd_last_error(gml->dev));
      return 0;
   }

   gml->MovSiz += dat->MemSiz;
   return (int)(dat->MemSiz > 0x7fffffff ? 0x7fffffff : dat->MemSiz);
}

/* Refresh the host mirrors that bulk reads left to the next call (see
   GETGMLPTR): one blocking download each, of device data that nothing has
   changed since the read. */
void gml_settle(GmlSct *gml)
{
   int i;

   if(!gml || !gml->NmbMirOld)
      return;
   for(i=1;i<=GmlMaxDat;i++)
      if(gml->dat[i].use && gml->dat[i].MirOld)
      {
         gml->dat[i].MirOld = 0;
         gml_download(gml, i);
      }
   gml->NmbMirOld = 0;
}

/* Spread an arbitrary vector size over power-of-two OpenCL vectors of at most
   16 lanes (reference GetCntVec, :2945-2964). */
void gml_get_cnt_vec(int siz, int *cnt, int *vec, int *typ)
{
   int p = 0;

   while((1 << p) < siz)
      p++;
   if(p > 7)
      p = 7;

   if(p > 4)
   {
      *cnt = 1 << (p - 4);
      *vec = 16;
      *typ = GmlOclVecPow[4];
   }
   else
   {
      *cnt = 1;
      *vec = 1 << p;
      *typ = GmlOclVecPow[p];
   }
}

/* ========================================================================= */
/* instance                                                                   */
/* ========================================================================= */

size_t GmlInit(int DevIdx)
{
   GmlSct *gml;
   char err[256] = "";
   const char *env;

   if(!(gml = calloc(1, sizeof(GmlSct))))
      return 0;

   gml->CurDev = DevIdx;
   gml->dev = gmd_init(DevIdx, &gml->DblExt, err, sizeof(err));

   if(!gml->dev)
   {
      puts(err[0] ? err : "Could not initialise the CUDA device.");
      free(gml);
      return 0;
   }

   gml->RedScrSiz = gmd_reduce_scratch_bytes(0);
   gml->RedScr = gmd_alloc(gml->dev, gml->RedScrSiz);

   if(!gml->RedScr)
   {
      gmd_stop(gml->dev);
      free(gml);
      return 0;
   }

   if((env = getenv("GML_TUNE")) && atoi(env) <= 0)
      gml->TunOff = 1;
   else if(env && atoi(env) >= 32)
   {
      gml->TunOff = 1;
      gml->TunBlk = atoi(env);
   }
   if((env = getenv("GML_LAZY")) && atoi(env) == 0)
      gml->LazyOff = 1;

   return (size_t)gml;
}

static void free_kernel(GmlSct *gml, GmlKrnSct *krn)
{
   int i;
   (void)gml;
   for(i=0;i<krn->EvtCap;i++)
   {
      gmd_event_free(krn->EvtBeg[i]);
      gmd_event_free(krn->EvtEnd[i]);
   }
   free(krn->EvtBeg);
   free(krn->EvtEnd);
   gmd_event_free(krn->TunBeg);
   gmd_event_free(krn->TunEnd);
   if(krn->module)
      gmd_module_unload(krn->module);
   free(krn->name);
   free(krn->source);
   memset(krn, 0, sizeof(GmlKrnSct));
}

void GmlStop(size_t GmlIdx)
{
   int i;
   GETGMLPTR_NOSETTLE(gml, GmlIdx);

   if(!gml)
      return;

   gmd_sync(gml->dev);

   for(i=1;i<=GmlMaxDat;i++)
      if(gml->dat[i].use)
         release_data(gml, &gml->dat[i]);

   gml_release_solvers(gml);
   gml_release_matrices(gml);

   for(i=1;i<=gml->NmbKrn && i<=GmlMaxKrn;i++)
      free_kernel(gml, &gml->krn[i]);

   gmd_free(gml->dev, gml->RedScr);
   gmlx_release_extensions(gml);
   gmd_stop(gml->dev);
   free(gml);
}

void GmlListGPU()
{
   int i, n = gmd_device_count();
   char nam[ GmlMaxStrSiz ];

   for(i=0;i<n;i++)
      if(gmd_device_name(i, nam, sizeof(nam)))
         printf("      %d      : %s\n", i, nam);
}

int GmlCheckFP64(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   return gml->DblExt;
}

/* ========================================================================= */
/* datatypes                                                                  */
/* ========================================================================= */

/* The shape of a datatype: what kind of data it is, which entities its lines
   follow, and how a line is made (cnt items of the OpenCL type `typ`, `len`
   scalars each, `siz` bytes each).  Every creator below describes its
   datatype with one of these and hands it to new_datatype(). */
typedef struct
{
   int         kind, msh, lnk, typ, cnt, len, siz, lines;
   const char  *name;
   char        *src;
}GmlShape;

/* Take a free slot, give it the shape, allocate the device buffer and the
   host mirror.  `what` names the datatype in the debug trace, which opens a
   new block unless `more` (a second datatype of the same call). */
static int new_datatype(GmlSct *gml, const GmlShape *shp, const char *what, int more)
{
   const int idx = gml_new_data_idx(gml);
   GmlDatSct *d;

   if(!idx)
      return 0;

   d = &gml->dat[ idx ];
   d->AloTyp = shp->kind;
   d->MshTyp = shp->msh;
   d->LnkTyp = shp->lnk;
   d->MemAcs = GmlInout;
   d->ItmTyp = shp->typ;
   d->NmbItm = shp->cnt;
   d->ItmLen = shp->len;
   d->ItmSiz = shp->siz;
   d->NmbLin = shp->lines;
   d->LinSiz = shp->cnt * shp->siz;
   d->MemSiz = (size_t)shp->lines * (size_t)d->LinSiz;
   d->nam    = shp->name;
   d->src    = shp->src;

   if(!gml_alloc_data(gml, d))
   {
      d->use = 0;
      return 0;
   }

   if(gml->DbgFlg)
   {
      if(!more)
         puts(sep);
      printf("Allocated %s: index=%2d, size=%zu bytes\n", what, idx, d->MemSiz);
   }
   return idx;
}

/* the shape of a mesh datatype's lines: one OpenCL vector wide enough for
   an element's nodes (vertices: float4 coordinates) */
static GmlShape element_shape(int MshTyp, int NmbLin)
{
   const int typ = GmlMshItmTyp[ MshTyp ];
   return (GmlShape){ GmlEleDat, MshTyp, 0, typ, 1, GmlTypVecSiz[ typ ], GmlOclTypSiz[ typ ],
                      NmbLin, GmlMshTypStr[ MshTyp ], NULL };
}

void *GmlNewParameters(size_t GmlIdx, int siz, char *src)
{
   GETGMLPTR(gml, GmlIdx);
   const GmlShape shp = { GmlArgDat, 0, 0, 0, 1, 0, siz, 1, "GmlParSct", src };
   const int idx = siz >= 0 ? new_datatype(gml, &shp, "a parameters data", 0) : 0;

   if(!idx)
      return NULL;
   gml->ParIdx = idx;
   return gml->dat[ idx ].CpuMem;
}

int GmlNewMeshData(size_t GmlIdx, int MshTyp, int NmbLin)
{
   GETGMLPTR(gml, GmlIdx);
   int EleIdx, RefIdx;

   if(MshTyp < 0 || MshTyp >= GmlMaxEleTyp || NmbLin < 0)
      return 0;

   /* the element (or coordinate) lines, then one int reference per line */
   {
      const GmlShape ele = element_shape(MshTyp, NmbLin);
      const GmlShape ref = { GmlRefDat, MshTyp, 0, GmlInt, 1, 0, 4, NmbLin,
                             GmlMshRefStr[ MshTyp ], NULL };
      if(!(EleIdx = new_datatype(gml, &ele, "mesh data", 0))
      || !(RefIdx = new_datatype(gml, &ref, "ref  data", 1)))
         return 0;
   }

   gml->NmbEle[ MshTyp ] = NmbLin;
   gml->TypIdx[ MshTyp ] = EleIdx;
   gml->RefIdx[ MshTyp ] = RefIdx;
   gml->LnkMat[ MshTyp ][ GmlVertices ] = EleIdx;    /* the element table is the downlink */
   return EleIdx;
}

int GmlNewSolutionData(size_t GmlIdx, int MshTyp, int NmbDat, int ItmTyp, char *nam)
{
   GETGMLPTR(gml, GmlIdx);

   if(MshTyp < 0 || MshTyp >= GmlMaxEleTyp || ItmTyp < GmlInt || ItmTyp >= GmlMaxOclTyp || NmbDat < 1)
      return 0;

   {
      const GmlShape shp = { GmlRawDat, MshTyp, 0, ItmTyp, NmbDat, GmlTypVecSiz[ ItmTyp ],
                             GmlOclTypSiz[ ItmTyp ], gml->NmbEle[ MshTyp ], nam, NULL };
      return new_datatype(gml, &shp, "solutions data", 0);
   }
}

/* User link table (reference :693-736).  A line holds NmbDat entity indices
   padded to the OpenCL vector width; GmlSetDataLine sets a line from a
   pointer to NmbDat ints (the documented usage, also what the reference's own
   GmlSetNeighbours passes). */
int GmlNewLinkData(size_t GmlIdx, int MshTyp, int LnkTyp, int NmbDat, char *nam)
{
   GETGMLPTR(gml, GmlIdx);
   int cnt, width, typ, idx;

   if(MshTyp < 0 || MshTyp >= GmlMaxEleTyp || LnkTyp < 0 || LnkTyp >= GmlMaxEleTyp || NmbDat < 1)
      return 0;

   gml_get_cnt_vec(NmbDat, &cnt, &width, &typ);
   {
      const GmlShape shp = { GmlLnkDat, MshTyp, LnkTyp, typ, cnt, NmbDat, GmlOclTypSiz[ typ ],
                             gml->NmbEle[ MshTyp ], nam, NULL };
      if(!(idx = new_datatype(gml, &shp, "link data", 0)))
         return 0;
   }
   gml->LnkMat[ MshTyp ][ LnkTyp ] = idx;
   return idx;
}

int GmlFreeData(size_t GmlIdx, int idx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat;
   int t, u;

   if(idx < 1 || idx > GmlMaxDat)
      return 0;

   dat = &gml->dat[ idx ];

   if(!dat->use || !dat->GpuMem)
      return 0;

   /* forget links that point at the freed slot */
   for(t=0;t<GmlMaxEleTyp;t++)
   {
      if(gml->TypIdx[t] == idx)
      {
         gml->TypIdx[t] = 0;
         gml->NmbEle[t] = 0;
      }
      if(gml->RefIdx[t] == idx)
         gml->RefIdx[t] = 0;
      for(u=0;u<GmlMaxEleTyp;u++)
      {
         if(gml->LnkMat[t][u] == idx) gml->LnkMat[t][u] = 0;
         if(gml->LnkHgh[t][u] == idx) gml->LnkHgh[t][u] = 0;
         if(gml->CntMat[t][u] == idx) gml->CntMat[t][u] = 0;
      }
   }
   if(gml->ParIdx == idx)
      gml->ParIdx = 0;

   gmd_sync(gml->dev);
   release_data(gml, dat);
   return 1;
}

/* ========================================================================= */
/* line and block transfers                                                   */
/* ========================================================================= */

static GmlDatSct *chk_dat(GmlSct *gml, int idx)
{
   if(idx < 1 || idx > GmlMaxDat || !gml->dat[idx].use)
      return NULL;
   return &gml->dat[idx];
}

int GmlSetDataLine(size_t GmlIdx, int idx, int lin, ...)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = chk_dat(gml, idx), *RefDat;
   int i, RefIdx = 0, *tab, *RefTab;
   float *CrdTab;
   va_list VarArg;

   if(!dat || lin < 0 || lin >= dat->NmbLin || !dat->CpuMem)
      return 0;

   gml_wait_upload(gml, dat);
   va_start(VarArg, lin);

   if(dat->AloTyp == GmlRawDat || dat->AloTyp == GmlArgDat)
   {
      memcpy((char *)dat->CpuMem + (size_t)lin * dat->LinSiz, va_arg(VarArg, void *), dat->LinSiz);
   }
   else if(dat->AloTyp == GmlLnkDat)
   {
      const int *src = va_arg(VarArg, const int *);
      int RowLen = dat->LinSiz / 4;
      tab = (int *)dat->CpuMem + (size_t)lin * RowLen;
      for(i=0;i<RowLen;i++)
         tab[i] = (i < dat->ItmLen && src) ? src[i] : 0;
   }
   else if(dat->AloTyp == GmlEleDat && dat->MshTyp == GmlVertices)
   {
      CrdTab = (float *)dat->CpuMem;
      RefIdx = gml->RefIdx[ GmlVertices ];
      RefDat = &gml->dat[ RefIdx ];
      gml_wait_upload(gml, RefDat);
      RefTab = (int *)RefDat->CpuMem;
      for(i=0;i<3;i++)
         CrdTab[ (size_t)lin * 4 + i ] = (float)va_arg(VarArg, double);
      CrdTab[ (size_t)lin * 4 + 3 ] = 0.f;
      RefTab[ lin ] = va_arg(VarArg, int);
   }
   else if(dat->AloTyp == GmlEleDat)
   {
      int siz = GmlTypVecSiz[ GmlMshItmTyp[ dat->MshTyp ] ];
      tab = (int *)dat->CpuMem;
      RefIdx = gml->RefIdx[ dat->MshTyp ];
      RefDat = &gml->dat[ RefIdx ];
      gml_wait_upload(gml, RefDat);
      RefTab = (int *)RefDat->CpuMem;
      for(i=0;i<GmlEleNmbNod[ dat->MshTyp ];i++)
         tab[ (size_t)lin * siz + i ] = va_arg(VarArg, int);
      RefTab[ lin ] = va_arg(VarArg, int);
   }

   va_end(VarArg);

   if(lin == dat->NmbLin - 1)
   {
      gml_upload(gml, idx);
      if(RefIdx)
         gml_upload(gml, RefIdx);
   }

   return 1;
}

/* Reading line 0 downloads the whole buffer (reference :1921-1922).  For
   vertices the reference reads coordinates with a stride of LinSiz floats
   instead of 4 (:1937); here line lin returns its own coordinates.  Element
   lines also refresh their reference table from the device. */
int GmlGetDataLine(size_t GmlIdx, int idx, int lin, ...)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat = chk_dat(gml, idx);
   int i, *RefTab;
   va_list VarArg;

   if(!dat || lin < 0 || lin >= dat->NmbLin || !dat->CpuMem)
      return 0;

   if(lin == 0)
   {
      gml_download(gml, idx);
      if(dat->AloTyp == GmlEleDat && gml->RefIdx[ dat->MshTyp ])
         gml_download(gml, gml->RefIdx[ dat->MshTyp ]);
   }

   va_start(VarArg, lin);

   if(dat->AloTyp == GmlRawDat || dat->AloTyp == GmlArgDat)
   {
      memcpy(va_arg(VarArg, void *), (char *)dat->CpuMem + (size_t)lin * dat->LinSiz, dat->LinSiz);
   }
   else if(dat->AloTyp == GmlLnkDat)
   {
      int *dst = va_arg(VarArg, int *);
      int RowLen = dat->LinSiz / 4, n = dat->ItmLen < RowLen ? dat->ItmLen : RowLen;
      if(dst)
         memcpy(dst, (int *)dat->CpuMem + (size_t)lin * RowLen, (size_t)(n > 0 ? n : RowLen) * 4);
   }
   else if(dat->AloTyp == GmlEleDat && dat->MshTyp == GmlVertices)
   {
      const float *crd = (const float *)dat->CpuMem;
      for(i=0;i<3;i++)
         *va_arg(VarArg, double *) = (double)crd[ (size_t)lin * 4 + i ];
   }
   else if(dat->AloTyp == GmlEleDat)
   {
      int siz = GmlTypVecSiz[ GmlMshItmTyp[ dat->MshTyp ] ];
      const int *tab = (const int *)dat->CpuMem;
      RefTab = (int *)gml->dat[ gml->RefIdx[ dat->MshTyp ] ].CpuMem;
      for(i=0;i<GmlEleNmbNod[ dat->MshTyp ];i++)
         *va_arg(VarArg, int *) = tab[ (size_t)lin * siz + i ];
      *va_arg(VarArg, int *) = RefTab ? RefTab[ lin ] : 0;
   }

   va_end(VarArg);
   return 1;
}

/* Inclusive line range BegIdx..EndIdx; the user strides are deduced from the
   first and last line pointers (reference :1968-2035). */
int GmlSetDataBlock(size_t GmlIdx, int TypIdx, int BegIdx, int EndIdx,
                    void *DatBeg, void *DatEnd, int *RefBeg, int *RefEnd)
{
   GETGMLPTR(gml, GmlIdx);
   int DatIdx, RefIdx, i, j;
   GmlDatSct *dat, *RefDat;
   size_t DatLen, RefLen;
   int *RefTab;

   if(TypIdx < 0 || TypIdx >= GmlMaxEleTyp)
      return 0;

   DatIdx = gml->TypIdx[ TypIdx ];
   RefIdx = gml->RefIdx[ TypIdx ];

   if(!DatIdx)
      return 0;

   dat = &gml->dat[ DatIdx ];
   RefDat = &gml->dat[ RefIdx ];

   if(EndIdx <= BegIdx || dat->AloTyp != GmlEleDat || BegIdx < 0 || EndIdx >= dat->NmbLin)
      return 0;

   gml_wait_upload(gml, dat);
   gml_wait_upload(gml, RefDat);
   RefTab = (int *)RefDat->CpuMem;
   RefLen = RefBeg ? (size_t)(RefEnd - RefBeg) / (size_t)(EndIdx - BegIdx) : 0;

   if(dat->MshTyp == GmlVertices)
   {
      float *CrdTab = (float *)dat->CpuMem;
      const float *UsrCrd = (const float *)DatBeg;
      DatLen = (size_t)((const float *)DatEnd - (const float *)DatBeg) / (size_t)(EndIdx - BegIdx);

      for(i=BegIdx;i<=EndIdx;i++)
      {
         const float *u = &UsrCrd[ (size_t)(i - BegIdx) * DatLen ];
         float *c = &CrdTab[ (size_t)i * 4 ];
         c[0] = u[0]; c[1] = u[1]; c[2] = u[2]; c[3] = 0.f;
      }
   }
   else
   {
      int *EleTab = (int *)dat->CpuMem;
      const int *UsrEle = (const int *)DatBeg;
      int siz = GmlTypVecSiz[ GmlMshItmTyp[ dat->MshTyp ] ], nn = GmlEleNmbNod[ dat->MshTyp ];
      DatLen = (size_t)((const int *)DatEnd - (const int *)DatBeg) / (size_t)(EndIdx - BegIdx);

      if(DatLen == (size_t)siz && nn == siz)
         memcpy(&EleTab[ (size_t)BegIdx * siz ], UsrEle, (size_t)(EndIdx - BegIdx + 1) * siz * sizeof(int));
      else
         for(i=BegIdx;i<=EndIdx;i++)
            for(j=0;j<nn;j++)
               EleTab[ (size_t)i * siz + j ] = UsrEle[ (size_t)(i - BegIdx) * DatLen + j ];
   }

   if(RefBeg)
   {
      if(RefLen == 1)
         memcpy(&RefTab[ BegIdx ], RefBeg, (size_t)(EndIdx - BegIdx + 1) * sizeof(int));
      else
         for(i=BegIdx;i<=EndIdx;i++)
            RefTab[i] = RefBeg[ (size_t)(i - BegIdx) * RefLen ];
   }

   if(EndIdx == dat->NmbLin - 1)
   {
      gml_upload(gml, DatIdx);
      gml_upload(gml, RefIdx);
   }

   return 1;
}

/* The reference writes 4 floats per vertex line whatever the user stride
   (:2081-2082), overrunning a 3-float layout; here min(4, stride) floats. */
int GmlGetDataBlock(size_t GmlIdx, int TypIdx, int BegIdx, int EndIdx,
                    void *DatBeg, void *DatEnd, int *RefBeg, int *RefEnd)
{
   GETGMLPTR(gml, GmlIdx);
   int DatIdx, RefIdx, i, j;
   GmlDatSct *dat, *RefDat;
   size_t DatLen, RefLen;
   const int *RefTab;

   if(TypIdx < 0 || TypIdx >= GmlMaxEleTyp)
      return 0;

   DatIdx = gml->TypIdx[ TypIdx ];
   RefIdx = gml->RefIdx[ TypIdx ];

   if(!DatIdx)
      return 0;

   dat = &gml->dat[ DatIdx ];
   RefDat = &gml->dat[ RefIdx ];

   if(EndIdx <= BegIdx || dat->AloTyp != GmlEleDat || BegIdx < 0 || EndIdx >= dat->NmbLin)
      return 0;

   if(BegIdx == 0)
   {
      gml_download(gml, DatIdx);
      gml_download(gml, RefIdx);
   }

   RefTab = (const int *)RefDat->CpuMem;
   RefLen = RefBeg ? (size_t)(RefEnd - RefBeg) / (size_t)(EndIdx - BegIdx) : 0;

   if(dat->MshTyp == GmlVertices)
   {
      const float *CrdTab = (const float *)dat->CpuMem;
      float *UsrCrd = (float *)DatBeg;
      size_t nc;
      DatLen = (size_t)((float *)DatEnd - (float *)DatBeg) / (size_t)(EndIdx - BegIdx);
      nc = DatLen < 4 ? DatLen : 4;

      if(DatLen == 4)
         memcpy(UsrCrd, &CrdTab[ (size_t)BegIdx * 4 ], (size_t)(EndIdx - BegIdx + 1) * 16);
      else
         for(i=BegIdx;i<=EndIdx;i++)
            for(j=0;j<(int)nc;j++)
               UsrCrd[ (size_t)(i - BegIdx) * DatLen + j ] = CrdTab[ (size_t)i * 4 + j ];
   }
   else
   {
      const int *EleTab = (const int *)dat->CpuMem;
      int *UsrEle = (int *)DatBeg;
      int siz = GmlTypVecSiz[ GmlMshItmTyp[ dat->MshTyp ] ], nn = GmlEleNmbNod[ dat->MshTyp ];
      DatLen = (size_t)((int *)DatEnd - (int *)DatBeg) / (size_t)(EndIdx - BegIdx);

      for(i=BegIdx;i<=EndIdx;i++)
         for(j=0;j<nn;j++)
            UsrEle[ (size_t)(i - BegIdx) * DatLen + j ] = EleTab[ (size_t)i * siz + j ];
   }

   if(RefBeg)
      for(i=BegIdx;i<=EndIdx;i++)
         RefBeg[ (size_t)(i - BegIdx) * RefLen ] = RefTab[i];

   return 1;
}

int GmlUploadParameters(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   return gml_upload(gml, gml->ParIdx) ? 1 : 0;
}

int GmlDownloadParameters(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   return gml_download(gml, gml->ParIdx) ? 1 : 0;
}

int GmlGetMeshInfo(size_t GmlIdx, int typ, int *NmbLin, int *DatIdx)
{
   GETGMLPTR(gml, GmlIdx);
   int idx;

   if(typ < 0 || typ >= GmlMaxEleTyp)
      return 0;
   if(NmbLin) *NmbLin = 0;
   if(DatIdx) *DatIdx = 0;
   if(!(idx = gml->TypIdx[ typ ]))
      return 0;
   if(!gml->dat[ idx ].NmbLin)
      return 0;
   if(NmbLin) *NmbLin = gml->dat[ idx ].NmbLin;
   if(DatIdx) *DatIdx = idx;
   return 1;
}

int GmlGetLinkInfo(size_t GmlIdx, int SrcTyp, int DstTyp, int *n, int *w, int *N, int *W)
{
   GETGMLPTR(gml, GmlIdx);
   int BalIdx, HghIdx;

   if(SrcTyp < 0 || SrcTyp >= GmlMaxEleTyp || DstTyp < 0 || DstTyp >= GmlMaxEleTyp)
      return 0;

   BalIdx = gml->LnkMat[ SrcTyp ][ DstTyp ];
   HghIdx = gml->LnkHgh[ SrcTyp ][ DstTyp ];

   if(!BalIdx)
      return 0;

   *n = gml->dat[ BalIdx ].NmbLin;
   *w = gml->dat[ BalIdx ].ItmLen;

   if(HghIdx)
   {
      *N = gml->dat[ HghIdx ].NmbLin;
      *W = gml->dat[ HghIdx ].ItmLen;
   }
   else
      *N = *W = 0;

   return 1;
}

/* ========================================================================= */
/* kernels: slots, timing, calibration                                        */
/* ========================================================================= */

int gml_new_kernel_slot(GmlSct *gml, int kind, const char *name)
{
   int idx = ++gml->NmbKrn;
   GmlKrnSct *krn;

   if(idx > GmlMaxKrn)
   {
      gml->NmbKrn = GmlMaxKrn;
      return 0;
   }

   krn = &gml->krn[ idx ];
   memset(krn, 0, sizeof(GmlKrnSct));
   krn->use  = 1;
   krn->kind = kind;
   krn->idx  = idx;
   krn->name = strdup(name ? name : "");
   return idx;
}

static int grow_events(GmlKrnSct *krn)
{
   int cap = krn->EvtCap ? 2 * krn->EvtCap : 64, i;
   void **b = realloc(krn->EvtBeg, cap * sizeof(void *));
   void **e;
   if(!b) return 0;
   krn->EvtBeg = b;
   e = realloc(krn->EvtEnd, cap * sizeof(void *));
   if(!e) return 0;
   krn->EvtEnd = e;
   for(i=krn->EvtCap;i<cap;i++)
   {
      krn->EvtBeg[i] = gmd_event_new();
      krn->EvtEnd[i] = gmd_event_new();
   }
   krn->EvtCap = cap;
   return 1;
}

/* fold the recorded launch events into RunTim */
static void fold_events(GmlKrnSct *krn)
{
   int i;
   for(i=0;i<krn->NmbEvt;i++)
      krn->RunTim += gmd_event_elapsed_s(krn->EvtBeg[i], krn->EvtEnd[i]);
   krn->NmbEvt = 0;
}

static void *evt_begin(GmlSct *gml, GmlKrnSct *krn)
{
   if(gmd_capturing(gml->dev) || gmlx_timing_off(gml))
      return NULL;
   if(krn->NmbEvt >= 4096)
      fold_events(krn);
   if(krn->NmbEvt == krn->EvtCap && !grow_events(krn))
      return NULL;
   gmd_event_record(gml->dev, krn->EvtBeg[ krn->NmbEvt ]);
   return krn->EvtEnd[ krn->NmbEvt ];
}

static void evt_end(GmlSct *gml, GmlKrnSct *krn, void *end)
{
   if(!end)
      return;
   gmd_event_record(gml->dev, end);
   krn->NmbEvt++;
}

static void *lib_end_evt;

void gml_lib_timer_begin(GmlSct *gml, GmlKrnSct *krn)
{
   lib_end_evt = evt_begin(gml, krn);
}

void gml_lib_timer_end(GmlSct *gml, GmlKrnSct *krn)
{
   evt_end(gml, krn, lib_end_evt);
   lib_end_evt = NULL;
}

int gml_timed_launch(GmlSct *gml, GmlKrnSct *krn, unsigned grid, unsigned block, void **args)
{
   void *end = evt_begin(gml, krn);
   int res = gmd_launch(gml->dev, krn->func, grid, block, 0, args);
   evt_end(gml, krn, end);
   return res;
}

static const int TunCand[] = { 64, 128, 256, 512, 1024, 32 };
#define NMB_TUNCAND ((int)(sizeof(TunCand) / sizeof(TunCand[0])))
#define NMB_TUNRND  2            /* timings of each candidate; the fastest counts */

/* Block-size calibration.  Like the reference (:3142-3190) the first launches
   of a kernel try several work-group sizes and keep the fastest; here the
   candidates are warp multiples timed with CUDA events instead of a host
   clock around clFinish: launch 0 warms up with 256, launches 1 to
   NMB_TUNRND x NMB_TUNCAND time the candidates in turn, each NMB_TUNRND
   times (a kernel's launches do the caller's work, so the rounds are spread
   over its first launches), and each candidate's best time counts.  The
   choice is kept in the process-wide tuning table under the kernel's source
   hash, line count and SM count, and persisted when GML_CACHE_DIR is set:
   a later kernel with the same key starts with the choice. */
static int pick_block(GmlSct *gml, GmlKrnSct *krn)
{
   const int lim = krn->MaxSiz > 0 ? krn->MaxSiz : 1024;
   const int nstep = NMB_TUNRND * NMB_TUNCAND;
   int c, best = -1;
   double tbest = 1e30;

   if(krn->OptSiz)
      return krn->OptSiz;

   if(gml->TunOff || gmd_capturing(gml->dev) || krn->NmbLin[0] < 4096)
   {
      int b = (gml->TunOff && gml->TunBlk > 0) ? gml->TunBlk : 256;
      krn->OptSiz = lim < b ? lim : b;
      return krn->OptSiz;
   }

   if(krn->TunStp == 0)
   {
      const int known = gmlx_tune_get("k", krn->hash, krn->NmbLin[0], gmd_num_sms(gml->dev));
      if(known >= 32 && known <= lim)
         return krn->OptSiz = known;
   }

   if(krn->TunStp <= nstep)
   {
      c = krn->TunStp == 0 ? 2 : (krn->TunStp - 1) % NMB_TUNCAND;
      krn->TunStp++;
      while(TunCand[c] > lim && c > 0)
         c--;
      return TunCand[c];
   }

   for(c=0;c<NMB_TUNCAND;c++)
      if(TunCand[c] <= lim && krn->TunTim[c] > 0. && krn->TunTim[c] < tbest)
      {
         tbest = krn->TunTim[c];
         best = TunCand[c];
      }

   krn->OptSiz = best > 0 ? best : (lim < 256 ? lim : 256);
   if(best > 0)
      gmlx_tune_set("k", krn->hash, krn->NmbLin[0], gmd_num_sms(gml->dev), krn->OptSiz);
   return krn->OptSiz;
}

static int run_generated(GmlSct *gml, GmlKrnSct *krn)
{
   void *ptrs[ GML_MAXARG ], *args[ GML_MAXARG + 2 ], *par;
   int cnt[2], i, blk, tuning, step;
   unsigned grid;
   GmlDatSct *dat;

   for(i=0;i<krn->NmbDat;i++)
   {
      dat = &gml->dat[ krn->DatTab[i] ];
      if(krn->DatTab[i] < 1 || krn->DatTab[i] > GmlMaxDat || !dat->GpuMem)
      {
         printf("Invalid user argument %d, DatTab[i]=%d, GpuMem=%p\n", i, krn->DatTab[i], dat->GpuMem);
         return -1;
      }
      ptrs[i] = dat->GpuMem;
      args[i] = &ptrs[i];
   }

   par = gml->ParIdx ? gml->dat[ gml->ParIdx ].GpuMem : NULL;
   args[ krn->NmbDat ] = &par;
   cnt[0] = krn->NmbLin[0];
   cnt[1] = krn->NmbLin[1];
   args[ krn->NmbDat + 1 ] = cnt;

   if(cnt[0] <= 0)
      return 1;

   step = krn->TunStp;
   tuning = !krn->OptSiz;
   blk = pick_block(gml, krn);
   grid = (unsigned)((cnt[0] + blk - 1) / blk);

   if(tuning && step >= 1 && step <= NMB_TUNRND * NMB_TUNCAND && krn->OptSiz == 0)
   {
      const int c = (step - 1) % NMB_TUNCAND;
      int res;
      double t;
      if(!krn->TunBeg) krn->TunBeg = gmd_event_new();
      if(!krn->TunEnd) krn->TunEnd = gmd_event_new();
      gmd_event_record(gml->dev, krn->TunBeg);
      res = gml_timed_launch(gml, krn, grid, (unsigned)blk, args);
      gmd_event_record(gml->dev, krn->TunEnd);
      t = TunCand[c] == blk ? gmd_event_elapsed_s(krn->TunBeg, krn->TunEnd) : 0.;
      if(t > 0. && (krn->TunTim[c] <= 0. || t < krn->TunTim[c]))
         krn->TunTim[c] = t;
      return res ? 1 : -6;
   }

   return gml_timed_launch(gml, krn, grid, (unsigned)blk, args) ? 1 : -6;
}

int GmlLaunchKernel(size_t GmlIdx, int idx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *krn;
   int res;

   if(idx < 1 || idx > gml->NmbKrn || idx > GmlMaxKrn)
      return -1;

   krn = &gml->krn[ idx ];

   if(!krn->use || krn->kind != GmlKrnGenerated || !krn->func)
      return -1;

   res = run_generated(gml, krn);

   if(res != 1)
      return res;

   if(krn->HghIdx)
      res = run_generated(gml, &gml->krn[ krn->HghIdx ]);

   return res;
}

double GmlGetKernelRunTime(size_t GmlIdx, int KrnIdx)
{
   GETGMLPTR(gml, GmlIdx);
   GmlKrnSct *krn;

   if(KrnIdx < 1 || KrnIdx > gml->NmbKrn || KrnIdx > GmlMaxKrn)
      return -1;

   krn = &gml->krn[ KrnIdx ];

   if(!krn->use)
      return -1;

   fold_events(krn);
   return krn->RunTim;
}

double GmlGetReduceRunTime(size_t GmlIdx, int RedOpp)
{
   GETGMLPTR(gml, GmlIdx);

   if(RedOpp < 0 || RedOpp >= GmlMaxRed)
   {
      printf("Invalid operation code %d\n", RedOpp);
      return -1.;
   }

   if(!gml->RedKrn[ RedOpp ])
      return 0.;

   return GmlGetKernelRunTime(GmlIdx, gml->RedKrn[ RedOpp ]);
}

double GmlGetWallClock()
{
   struct timeval tp;
   gettimeofday(&tp, NULL);
   return tp.tv_sec + tp.tv_usec / 1000000.;
}

/* ========================================================================= */
/* kernel generation and compilation                                          */
/* ========================================================================= */

void GmlSetCompilerOptions(size_t GmlIdx, char *OptStr)
{
   GETGMLPTR(gml, GmlIdx);
   snprintf(gml->cflags, sizeof(gml->cflags), "%s", OptStr ? OptStr : "");
}

void GmlIncludeUserToolkit(size_t GmlIdx, char *PtrSrc)
{
   GETGMLPTR(gml, GmlIdx);
   gml->UsrTlk = PtrSrc;
}

/* Compile one generated source into a kernel slot; returns the slot or 0. */
static int compile_into_slot(GmlSct *gml, const char *src, const char *PrcNam, int quiet, char **logout)
{
   void *cubin = NULL, *mod = NULL, *fn = NULL;
   size_t cs = 0;
   char *log = NULL, *opts;
   int idx, maxthr = 1024, nreg = 0;

   opts = gml_nvrtc_options(gml->cflags);

   if(!gmlx_cache_lookup(src, opts, PrcNam, &cubin, &cs))
   {
      if(!gmd_compile(src, PrcNam, opts, &cubin, &cs, &log))
      {
         if(!quiet)
         {
            printf("Compiling the kernel %s failed at step 2\n", PrcNam);
            printf("%s\n", log ? log : "");
            fflush(stdout);
         }
         if(logout) *logout = log; else free(log);
         free(opts);
         return 0;
      }
      gmlx_cache_store(src, opts, PrcNam, cubin, cs);
   }
   free(log);
   free(opts);

   if(gml->Offline)
   {
      /* code generation only: keep the source, nothing to load */
      free(cubin);
      if(!(idx = gml_new_kernel_slot(gml, GmlKrnGenerated, PrcNam)))
         return 0;
      gml->krn[ idx ].source = strdup(src);
      gml->krn[ idx ].hash = gml_hash64(src, strlen(src), 0x9e3779b97f4a7c15ULL);
      return idx;
   }

   if(!gmd_module_load(gml->dev, cubin, PrcNam, &mod, &fn, &maxthr, &nreg))
   {
      printf("Compiling the kernel %s failed at step 3: %s\n", PrcNam, gmd_last_error(gml->dev));
      free(cubin);
      return 0;
   }
   free(cubin);

   if(!(idx = gml_new_kernel_slot(gml, GmlKrnGenerated, PrcNam)))
   {
      gmd_module_unload(mod);
      return 0;
   }

   gml->krn[ idx ].module = mod;
   gml->krn[ idx ].func   = fn;
   gml->krn[ idx ].MaxSiz = maxthr;
   gml->krn[ idx ].NumReg = nreg;
   gml->krn[ idx ].source = strdup(src);
   gml->krn[ idx ].hash = gml_hash64(src, strlen(src), 0x9e3779b97f4a7c15ULL);
   return idx;
}

/* Generate (lazy ball gathers first, the reference's eager arrays when the
   body needs real arrays) and compile. */
static int build_kernel(GmlSct *gml, char *KrnSrc, char *PrcNam, int MshTyp,
                        int NmbArg, GmlArgSct *ArgTab, const char *ParSrc)
{
   char *src = NULL;
   int idx = 0, lazy;

   for(lazy = gml->LazyOff ? 0 : 1; lazy >= 0 && !idx; lazy--)
   {
      if(!gml_generate(&src, PrcNam, MshTyp, NmbArg, ArgTab, KrnSrc, gml->UsrTlk, ParSrc, lazy))
         return 0;
      idx = compile_into_slot(gml, src, PrcNam, lazy, NULL);
      if(idx)
      {
         gml->krn[ idx ].lazy = lazy;
         if(gml->DbgFlg)
         {
            puts(sep);
            printf("Generated source for kernel=%s, index=%2d\n", PrcNam, idx);
            puts(src);
         }
      }
      free(src);
      src = NULL;
   }

   return idx;
}

/* ------------------------------------------------------------------------- */
/* Kernel argument planning.                                                  */
/*                                                                           */
/* The generated kernel's parameter list is part of the naming contract      */
/* (reference sources/gmlib3.c:2635-2663): first the link tables the kernel  */
/* needs, each uplink followed by its degree table, then the user's          */
/* datatypes in call order, each followed by its reference array when        */
/* GmlRefFlag asks for it.  A kernel runs over entities of type `run`; a     */
/* datatype of type `dst` is reached directly (same type), through a         */
/* downlink (run has more dimensions, e.g. tet -> vertex: the element        */
/* table), a same-dimension user link (e.g. neighbours), or an uplink (the   */
/* ball of dst entities around each run entity).  The plan below is built    */
/* from these rules; gml_codegen.c turns it into source.                     */
/* ------------------------------------------------------------------------- */

typedef struct
{
   int         dat, flags, link, count;   /* one user datatype of the kernel */
}GmlUse;

typedef struct
{
   GmlArgSct   arg[ GML_MAXARG ];
   int         n;
   int         up;                        /* index of the uplink argument, -1 if none */
   int         high;                      /* its high-degree table, 0 if none */
   int         width;                     /* that table's width */
}GmlPlan;

/* -1 downlink, 0 same dimension, +1 uplink */
static int reach(int run, int dst)
{
   const int a = GmlMshTypDim[ run ], b = GmlMshTypDim[ dst ];
   return a > b ? -1 : a < b ? 1 : 0;
}

static int plan_push(GmlPlan *p, GmlArgSct a)
{
   a.ArgIdx = p->n;
   p->arg[ p->n ] = a;
   return p->n++;
}

/* the latest argument bound to datatype `dat`, or -1 */
static int plan_find(const GmlPlan *p, int dat)
{
   for(int j=p->n-1;j>=0;j--)
      if(p->arg[j].DatIdx == dat)
         return j;
   return -1;
}

/* The default link of a run -> dst pair, built on first use under the
   contract's names: <Run><Dst>Lnk/Deg for a downlink, <Run><Dst>Bal/Deg/Voy
   for an uplink. */
static int default_link(GmlSct *gml, int run, int dst, int dir)
{
   static const char *suffix[2][3] = { { "Lnk", "Deg", NULL }, { "Bal", "Deg", "Voy" } };
   const char *nam[3] = { NULL, NULL, NULL };
   char buf[ GmlMaxStrSiz ];

   if(gml->LnkMat[ run ][ dst ])
      return gml->LnkMat[ run ][ dst ];

   for(int k=0;k<3;k++)
      if(suffix[ dir > 0 ][k])
      {
         snprintf(buf, sizeof(buf), "%s%s%s", GmlBalTypStr[ run ], GmlBalTypStr[ dst ], suffix[ dir > 0 ][k]);
         nam[k] = gmlx_intern(gml, buf);
      }
   if(!gml_new_ball_data(gml, run, dst, nam[0], nam[1], nam[2]))
      return 0;
   return gml->LnkMat[ run ][ dst ];
}

/* A link table as an argument: `width` entity indices per line, packed in
   OpenCL int vectors. */
static GmlArgSct link_arg(GmlSct *gml, int dat, int dst, int dir, int width)
{
   int cnt, len, typ;
   gml_get_cnt_vec(width, &cnt, &len, &typ);
   return (GmlArgSct){ .MshTyp = dst, .DatIdx = dat, .LnkTyp = -1, .LnkIdx = -1, .CntIdx = -1,
                       .LnkDir = dir, .LnkDeg = dir > 0 ? -1 : width, .MaxDeg = width,
                       .NmbItm = cnt, .ItmLen = len, .ItmTyp = typ, .FlgTab = GmlReadMode,
                       .nam = gml->dat[ dat ].nam };
}

/* A user datatype (or its reference array) read through link argument `lk`
   and count argument `ct` (either may be -1). */
static GmlArgSct data_arg(const GmlPlan *p, const GmlDatSct *d, int dat, int lk, int ct, int flags)
{
   const GmlArgSct *l = lk >= 0 ? &p->arg[ lk ] : NULL;
   return (GmlArgSct){ .MshTyp = d->MshTyp, .DatIdx = dat, .LnkDir = 0, .LnkTyp = d->MshTyp,
                       .LnkIdx = lk, .CntIdx = ct,
                       .LnkDeg = l && ct < 0 ? l->LnkDeg : -1, .MaxDeg = l ? l->MaxDeg : -1,
                       .NmbItm = d->NmbItm, .ItmLen = d->ItmLen, .ItmTyp = d->ItmTyp,
                       .FlgTab = flags, .nam = d->nam };
}

/* Link arguments, in the order of their first user.  Returns 0 when two
   different uplinks would meet in one kernel (one high-degree twin only). */
static int plan_links(GmlSct *gml, GmlPlan *p, int run, GmlUse *use, int nuse)
{
   for(int i=0;i<nuse;i++)
   {
      const int dst = gml->dat[ use[i].dat ].MshTyp;
      const GmlDatSct *lnk;
      int dir, width, at;

      if(!use[i].link || plan_find(p, use[i].link) >= 0)
         continue;

      lnk   = &gml->dat[ use[i].link ];
      dir   = reach(run, dst);
      width = (lnk->AloTyp == GmlLnkDat && lnk->MshTyp == run && run == dst)
            ? lnk->ItmLen : GmlLenMatBas[ run ][ dst ];
      at    = plan_push(p, link_arg(gml, use[i].link, dst, dir, width));

      if(dir <= 0)
         continue;

      /* an uplink: one kind per kernel, its voyeurs, then its degrees */
      if(p->up >= 0 && p->high != gml->LnkHgh[ run ][ dst ])
      {
         puts("Current limitation prevents mixing two different kinds of uplink in the same kernel.");
         return 0;
      }
      p->up    = at;
      p->high  = gml->LnkHgh[ run ][ dst ];
      p->width = gml->SizMatHgh[ run ][ dst ];
      if(use[i].flags & GmlVoyeurs)
      {
         p->arg[ at ].VoyNam  = lnk->VoyNam;
         p->arg[ at ].FlgTab |= GmlVoyeurs;
         use[i].flags        &= ~GmlVoyeurs;
      }
      {
         const int deg = gml->CntMat[ run ][ dst ];
         plan_push(p, (GmlArgSct){ .MshTyp = dst, .DatIdx = deg, .LnkDir = 0, .LnkTyp = -1,
                                   .LnkIdx = -1, .CntIdx = -1, .LnkDeg = 1, .MaxDeg = 1,
                                   .NmbItm = 1, .ItmLen = 1, .ItmTyp = GmlInt,
                                   .FlgTab = GmlReadMode, .nam = gml->dat[ deg ].nam });
      }
   }
   return 1;
}

/* The user's datatypes, each with its reference array on request (not for
   data read through a variable-degree uplink). */
static void plan_data(GmlSct *gml, GmlPlan *p, const GmlUse *use, int nuse)
{
   for(int i=0;i<nuse;i++)
   {
      const GmlDatSct *d = &gml->dat[ use[i].dat ];
      const int lk = use[i].link ? plan_find(p, use[i].link) : -1;
      const int ct = use[i].count ? plan_find(p, use[i].count) : -1;
      const int flags = use[i].flags & ~GmlRefFlag;
      const int ref = gml->RefIdx[ d->MshTyp ];

      plan_push(p, data_arg(p, d, use[i].dat, lk, ct, flags));
      if((use[i].flags & GmlRefFlag) && ct < 0 && ref)
         plan_push(p, data_arg(p, &gml->dat[ ref ], ref, lk, ct, flags));
   }
}

/* bind a compiled kernel to the plan's datatypes and line range */
static void bind_kernel(GmlKrnSct *krn, const GmlPlan *p, int lines, int first)
{
   krn->NmbDat    = p->n;
   krn->NmbLin[0] = lines;
   krn->NmbLin[1] = first;
   for(int i=0;i<p->n;i++)
      krn->DatTab[i] = p->arg[i].DatIdx;
}

int GmlCompileKernel(size_t GmlIdx, char *KrnSrc, char *PrcNam, int MshTyp, int NmbTyp, ...)
{
   GETGMLPTR(gml, GmlIdx);
   GmlUse use[ GmlMaxDat ];
   GmlPlan plan;
   const char *ParSrc;
   int base, twin, lines, hlines;
   va_list ap;

   if(MshTyp < 0 || MshTyp >= GmlMaxEleTyp || NmbTyp < 0 || NmbTyp > GmlMaxDat || !KrnSrc || !PrcNam)
      return 0;

   /* (datatype, flags, link) triplets, as the reference's varargs */
   va_start(ap, NmbTyp);
   for(int i=0;i<NmbTyp;i++)
   {
      use[i].dat   = va_arg(ap, int);
      use[i].flags = va_arg(ap, int);
      use[i].link  = va_arg(ap, int);
      use[i].count = 0;
   }
   va_end(ap);

   for(int i=0;i<NmbTyp;i++)
   {
      int dst, dir;

      if(!chk_dat(gml, use[i].dat))
      {
         printf("Invalid datatype index %d in kernel %s\n", use[i].dat, PrcNam);
         return 0;
      }
      dst = gml->dat[ use[i].dat ].MshTyp;
      dir = reach(MshTyp, dst);
      if(use[i].link || dst == MshTyp || !dir)
         continue;
      if(!(use[i].link = default_link(gml, MshTyp, dst, dir)))
         return 0;
      if(dir > 0)
         use[i].count = gml->CntMat[ MshTyp ][ dst ];
   }

   memset(&plan, 0, sizeof(plan));
   plan.up = -1;
   if(!plan_links(gml, &plan, MshTyp, use, NmbTyp))
      return 0;
   plan_data(gml, &plan, use, NmbTyp);

   ParSrc = gml->ParIdx ? gml->dat[ gml->ParIdx ].src : NULL;
   lines  = gml->dat[ gml->TypIdx[ MshTyp ] ].NmbLin;
   hlines = plan.up >= 0 && plan.high > 0 ? gml->dat[ plan.high ].NmbLin : 0;

   if(!(base = build_kernel(gml, KrnSrc, PrcNam, MshTyp, plan.n, plan.arg, ParSrc)))
      return 0;
   bind_kernel(&gml->krn[ base ], &plan, lines - hlines, 0);
   if(!(plan.up >= 0 && plan.high > 0))
      return base;

   /* The high-degree twin (reference :2543-2589): the same kernel over the
      last hlines lines, reading the wide table; data gathered through it with
      a variable degree get the wider bound. */
   {
      GmlArgSct *up = &plan.arg[ plan.up ];
      int cnt, len, typ;
      gml_get_cnt_vec(plan.width, &cnt, &len, &typ);
      up->DatIdx = plan.high;
      up->MaxDeg = plan.width;
      up->NmbItm = cnt;
      up->ItmLen = len;
      up->ItmTyp = typ;
      for(int i=0;i<plan.n;i++)
         if(plan.arg[i].LnkIdx == plan.up && plan.arg[i].CntIdx != -1)
            plan.arg[i].MaxDeg = plan.width;
   }
   if(!(twin = build_kernel(gml, KrnSrc, PrcNam, MshTyp, plan.n, plan.arg, ParSrc)))
      return 0;
   gml->krn[ base ].HghIdx = twin;
   bind_kernel(&gml->krn[ twin ], &plan, hlines, lines - hlines);
   return base;
}

/* ========================================================================= */
/* reductions (reference :3229-3332)                                          */
/* ========================================================================= */

static const char *RedNam[] = { "reduce_min", "reduce_max", "reduce_sum",
                                "reduce_L0", "reduce_L1", "reduce_L2", "reduce_Linf" };

int GmlReduceVector(size_t GmlIdx, int DatIdx, int RedOpp, double *nrm)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct *dat;
   GmlKrnSct *krn;
   int res;

   if(DatIdx < 1 || DatIdx > GmlMaxDat || !gml->dat[ DatIdx ].use)
   {
      printf("Invalid data index: %d\n", DatIdx);
      return -1;
   }

   dat = &gml->dat[ DatIdx ];

   if(dat->ItmTyp != GmlFlt || dat->NmbItm != 1 || dat->ItmLen != 1)
   {
      printf("Invalid data structure: count %d, type %s, length %d\n",
             dat->NmbItm, GmlOclTypStr[ dat->ItmTyp ], dat->ItmLen);
      return -2;
   }

   if(RedOpp < 0 || RedOpp >= GmlMaxRed)
   {
      printf("Invalid operation code %d\n", RedOpp);
      return -3;
   }

   /* The reference allocates an output vector the size of the input on first
      use; the slot is kept so that datatype indices evolve the same way. */
   if(!dat->RedIdx)
      dat->RedIdx = GmlNewSolutionData(GmlIdx, dat->MshTyp, 1, GmlFlt, "reduce");

   if(!dat->RedIdx)
   {
      printf("Failed to allocate a reduction vector of %d bytes\n", 4 * dat->NmbLin);
      return -4;
   }

   if(!gml->RedKrn[ RedOpp ])
      gml->RedKrn[ RedOpp ] = gml_new_kernel_slot(gml, GmlKrnReduce, RedNam[ RedOpp ]);

   if(!gml->RedKrn[ RedOpp ])
   {
      printf("Failed to compile the %s reduction kernel\n", RedNam[ RedOpp ]);
      return -5;
   }

   krn = &gml->krn[ gml->RedKrn[ RedOpp ] ];
   gml_lib_timer_begin(gml, krn);
   res = gmd_reduce_f32(gml->dev, RedOpp, (const float *)dat->GpuMem, dat->NmbLin, nrm, gml->RedScr);
   gml_lib_timer_end(gml, krn);

   return res ? 1 : -6;
}

/* ========================================================================= */
/* observability                                                              */
/* ========================================================================= */

size_t GmlGetMemoryUsage(size_t GmlIdx)    { GETGMLPTR(gml, GmlIdx); return gml->MemSiz; }
size_t GmlGetMemoryTransfer(size_t GmlIdx) { GETGMLPTR(gml, GmlIdx); return gml->MovSiz; }
float  GmlGetMemoryAccess(size_t GmlIdx)   { GETGMLPTR(gml, GmlIdx); return gml->MemAcc; }
float  GmlGetFlops(size_t GmlIdx)          { GETGMLPTR(gml, GmlIdx); return gml->FltOpp; }
void   GmlDebugOn(size_t GmlIdx)           { GETGMLPTR(gml, GmlIdx); gml->DbgFlg = 1; }
void   GmlDebugOff(size_t GmlIdx)          { GETGMLPTR(gml, GmlIdx); gml->DbgFlg = 0; }

/* Share of element-to-vertex accesses that hit a 16-entry direct-mapped
   cache of 1 KB lines (reference :4409-4442).  Like the reference, only the
   first node of each element line is looked at (it iterates j < NmbItm = 1). */
/* How well the element -> vertex accesses of the mesh reuse a cache, in
   percent of hits, by the reference's model (sources/gmlib3.c:4409-4442): a
   direct-mapped cache of 16 sets; vertex v falls in set (v >> 4) mod 16 and is
   tagged v >> 10 (bits 8-9 of v stay out of the tag); one lookup per item of
   each element line, i.e. the line's first node, the mesh datatypes holding
   one item per line; element types in increasing order from the edges. */
float GmlEvaluateNumbering(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   int tag[16] = { 0 };
   long long look = 0, hit = 0;

   for(int typ=GmlEdges; typ<GmlMaxEleTyp; typ++)
   {
      const GmlDatSct *d = gml->TypIdx[ typ ] ? &gml->dat[ gml->TypIdx[ typ ] ] : NULL;
      const int *node = d ? (const int *)d->CpuMem : NULL;

      for(size_t e=0; node && e<(size_t)d->NmbLin; e++)
         for(int k=0;k<d->NmbItm;k++, look++)
         {
            const int v = node[ e * d->ItmLen + k ];
            int *t = &tag[ (v >> 4) & 15 ];
            hit += (*t == (v >> 10));
            *t = v >> 10;
         }
   }
   return look ? 100 * (float)hit / (float)look : 0.f;
}
