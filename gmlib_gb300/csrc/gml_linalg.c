/*
 * gml_linalg.c -- block sparse matrices and block vectors (host side).
 *
 * Reference: GmlNewMatrix (sources/gmlib3.c:1175-1427), GmlNewVector
 * (:1434-1560), GmlMultMatVec (:3339-3404), GmlAddVec3 (:3411-3488),
 * GmlScaleVec (:3495-3527), GmlNormVec (:3534-3575), GmlMultDiagMatVec
 * (:3582-3641).
 *
 * Matrix layout.  The reference sorts rows into degree classes (<=16, 32,
 * 64, 128, 256 blocks) and stores each class as block-ELL with one OpenCL
 * kernel per class; rows must already be sorted by degree class or they
 * overflow into their neighbours (:1351, :1386), and block size 7 has no
 * kernel at all (multmatvec.cl:1645-1662).  Here the CSR input is repacked
 * into SELL-32: rows are grouped by 32 in their given order, a slice is as
 * wide as its longest row, and inside a slice entry k of all 32 rows is
 * stored contiguously (column index, then each of the b*b block values as a
 * run of 32).  One thread per row then reads everything with 128-byte
 * coalesced loads and no degree sorting is required.  Block sizes 3, 4, 5
 * and 7 are accepted, in FP32 or FP64.
 *
 * Vector layout is the reference's: each line holds BlkSiz values padded to
 * 1, 2, 4, 8, 16 (or 2, 3, 4 times 16) lanes (:1462-1501), so 3- and
 * 4-blocks are one float4/double4 per line.
 *
 * Semantics kept from the reference code:
 *   GmlMultMatVec(mat, V1, V2)      V1 = A . V2   (the kernel writes its fourth
 *                                   argument, which is V1, :3389-3390)
 *   GmlMultDiagMatVec(D, U, V)      V  = D_line . U_line
 *   GmlAddVec3(U, V, W, Y)          Y  = U + V + W
 *   GmlNormVec(V, R, &n)            R_line = |V_line|_2 ; n = sqrt(sum_line R)
 * GmlScaleVec multiplies by *mul; the reference kernel ignores *mul and
 * reads a `scale` field from the caller's parameter structure instead
 * (scalevec.cl:14-29), which exists only if the caller declared it.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"
#include "gml_linalg.h"

static int get_mat_idx(GmlSct *gml)
{
   for(int i=1;i<=GmlMaxMat;i++)
      if(!gml->mat[i].use)
      {
         memset(&gml->mat[i], 0, sizeof(GmlMatSct));
         gml->mat[i].use = 1;
         return i;
      }
   return 0;
}

static int get_vec_idx(GmlSct *gml)
{
   for(int i=1;i<=GmlMaxVec;i++)
      if(!gml->vec[i].use)
      {
         memset(&gml->vec[i], 0, sizeof(GmlVecSct));
         gml->vec[i].use = 1;
         return i;
      }
   return 0;
}

/* number of lanes of one vector line for a block of BlkSiz values */
static void vec_lanes(int BlkSiz, int *NmbValTyp, int *VecValSiz)
{
   if(BlkSiz == 1)       { *NmbValTyp = 1; *VecValSiz = 1; }
   else if(BlkSiz == 2)  { *NmbValTyp = 1; *VecValSiz = 2; }
   else if(BlkSiz <= 4)  { *NmbValTyp = 1; *VecValSiz = 4; }
   else if(BlkSiz <= 8)  { *NmbValTyp = 1; *VecValSiz = 8; }
   else if(BlkSiz <= 16) { *NmbValTyp = 1; *VecValSiz = 16; }
   else if(BlkSiz <= 32) { *NmbValTyp = 2; *VecValSiz = 16; }
   else if(BlkSiz <= 48) { *NmbValTyp = 3; *VecValSiz = 16; }
   else                  { *NmbValTyp = 4; *VecValSiz = 16; }
}

void gml_sell_dev_free(GmlSct *gml, GmlSellDev *d)
{
   gmd_free(gml->dev, d->SlcOff);
   gmd_free(gml->dev, d->Deg);
   gmd_free(gml->dev, d->Col);
   gmd_free(gml->dev, d->Val);
   memset(d, 0, sizeof(GmlSellDev));
}

/* SELL-32 image built on the device from the caller's CSR arrays: they are
   uploaded once, the slice widths and offsets are computed and scanned on
   the device, and a fill kernel scatters the blocks.  Returns 1, or 0 with
   a message (bad row pointers or columns, no memory). */
static int sell_build_device(GmlSct *gml, int NmbLin, int NmbBlk, int BlkSiz, int FltSiz,
                             const void *val, const int *col, const int *lin, GmlSellDev *d)
{
   const size_t bb = (size_t)BlkSiz * BlkSiz;
   const int nsl = (NmbLin + 31) / 32;
   int *dlin, *dcol, *err, herr = 0, ok = 0;
   void *dval;
   long long *width, tot = 0;

   memset(d, 0, sizeof(GmlSellDev));
   d->NmbLin = NmbLin;
   d->BlkSiz = BlkSiz;
   d->FltSiz = FltSiz;
   d->NmbSlc = nsl;
   dlin = gmd_alloc(gml->dev, (size_t)(NmbLin + 1) * 4);
   dcol = gmd_alloc(gml->dev, (size_t)NmbBlk * 4);
   dval = gmd_alloc(gml->dev, (size_t)NmbBlk * bb * FltSiz);
   err = gmd_alloc(gml->dev, sizeof(int));
   width = gmd_alloc(gml->dev, (size_t)(nsl + 1) * 8);
   d->Deg = gmd_alloc(gml->dev, (size_t)NmbLin * 4);
   d->SlcOff = gmd_alloc(gml->dev, (size_t)(nsl + 1) * 8);
   if(!dlin || !dcol || !dval || !err || !width || !d->Deg || !d->SlcOff)
      goto done;
   /* the caller's arrays are pageable: each copy is staged before it returns */
   if(!gmd_h2d_async(gml->dev, dlin, lin, (size_t)(NmbLin + 1) * 4)
   || !gmd_h2d_async(gml->dev, dcol, col, (size_t)NmbBlk * 4)
   || !gmd_h2d_async(gml->dev, dval, val, (size_t)NmbBlk * bb * FltSiz)
   || !gmd_sell_widths(gml->dev, NmbLin, dlin, d->Deg, width, err)
   || !gmd_scan_excl_i64(gml->dev, width, (long long *)d->SlcOff, nsl)
   || !gmd_d2h(gml->dev, &tot, (long long *)d->SlcOff + nsl, sizeof(long long))
   || !gmd_d2h(gml->dev, &herr, err, sizeof(int)))
      goto done;
   if(herr)
   {
      printf("GmlNewMatrix: row pointers decrease\n");
      goto done;
   }
   d->NmbCol = (size_t)tot;
   d->Col = gmd_alloc(gml->dev, (size_t)tot * 32 * 4);
   d->Val = gmd_alloc(gml->dev, (size_t)tot * 32 * bb * FltSiz);
   if(!d->Col || !d->Val)
      goto done;
   if(!gmd_sell_fill(gml->dev, NmbLin, (int)bb, FltSiz, dlin, dcol, dval,
                     (const long long *)d->SlcOff, d->Col,
                     d->Val, err)
   || !gmd_d2h(gml->dev, &herr, err, sizeof(int)))
      goto done;
   if(herr)
   {
      printf("GmlNewMatrix: column index out of range\n");
      goto done;
   }
   d->bytes = (size_t)(nsl + 1) * 8 + (size_t)NmbLin * 4 + (size_t)tot * 32 * 4
            + (size_t)tot * 32 * bb * FltSiz;
   ok = 1;
done:
   gmd_free(gml->dev, dlin);
   gmd_free(gml->dev, dcol);
   gmd_free(gml->dev, dval);
   gmd_free(gml->dev, err);
   gmd_free(gml->dev, width);
   if(!ok)
      gml_sell_dev_free(gml, d);
   return ok;
}

/* ========================================================================= */
/* GmlNewMatrix                                                               */
/* ========================================================================= */

int GmlNewMatrix(size_t GmlIdx, int NmbLin, int NmbBlk, int BlkSiz, void *val,
                 int *col, int *lin, int FltTyp)
{
   GETGMLPTR(gml, GmlIdx);
   int MatIdx, FltSiz;
   GmlMatSct *mat;
   GmlSellDev *dev;

   if(NmbLin < 1 || NmbBlk < 1 || BlkSiz < 1 || BlkSiz > 10)
      return 0;
   if(BlkSiz != 3 && BlkSiz != 4 && BlkSiz != 5 && BlkSiz != 7)
      return 0;
   if(FltTyp != GmlFlt && FltTyp != GmlDbl)
      return 0;
   /* row pointers start at 0 and end at NmbBlk; the device build checks
      that they never decrease and that every column is a row index */
   if(!val || !col || !lin || lin[0] != 0 || lin[NmbLin] != NmbBlk)
      return 0;
   if(!(MatIdx = get_mat_idx(gml)))
      return 0;

   mat = &gml->mat[ MatIdx ];
   FltSiz = FltTyp == GmlFlt ? 4 : 8;
   mat->NmbLin = NmbLin;
   mat->NmbBlk = NmbBlk;
   mat->BlkSiz = BlkSiz;
   mat->FltTyp = FltTyp;

   dev = calloc(1, sizeof(GmlSellDev));
   if(!dev || !sell_build_device(gml, NmbLin, NmbBlk, BlkSiz, FltSiz, val, col, lin, dev))
   {
      printf("Cannot build the sparse matrix on the GPU\n");
      free(dev);
      mat->use = 0;
      return 0;
   }

   if(!gml->Quiet)
   {
      printf(" Matrix slices = %d (SELL-32)\n", dev->NmbSlc);
      printf("  sparse nnz = %d, vectorized nnz = %zu, occupency = %.1f%%\n",
             NmbBlk, dev->NmbCol * 32, (100. * NmbBlk) / (double)(dev->NmbCol * 32));
   }

   mat->Val = dev;
   gml->MemSiz += dev->bytes;
   mat->KrnIdx = gml_new_kernel_slot(gml, GmlKrnMatVec, "MulMatVecSell");

   mat->MemAcc = ((float)NmbLin * BlkSiz + (float)NmbBlk * BlkSiz * (BlkSiz + 1)) * FltSiz;
   mat->FltOpp = (float)NmbBlk * BlkSiz * BlkSiz * 2;
   if(!gml->Quiet)
      printf("  swipe = %.2f GB, %.2f GFlops\n", mat->MemAcc / 1.E9, mat->FltOpp / 1.E9);

   return MatIdx;
}

/* ========================================================================= */
/* GmlNewVector                                                               */
/* ========================================================================= */

int GmlNewVector(size_t GmlIdx, int NmbLin, int BlkSiz, void *val, int FltTyp)
{
   GETGMLPTR(gml, GmlIdx);
   int VecIdx, DatIdx, i;
   GmlVecSct *vec;
   GmlDatSct *dat;
   char *dst;

   if(NmbLin < 1 || BlkSiz < 1 || BlkSiz > 64)
      return 0;
   if(FltTyp != GmlFlt && FltTyp != GmlDbl)
      return 0;
   if(!(VecIdx = get_vec_idx(gml)))
      return 0;

   vec = &gml->vec[ VecIdx ];
   vec->NmbLin = NmbLin;
   vec->BlkSiz = BlkSiz;
   vec->FltTyp = FltTyp;
   vec->FltSiz = FltTyp == GmlFlt ? 4 : 8;
   vec_lanes(BlkSiz, &vec->NmbValTyp, &vec->VecValSiz);

   if(!(DatIdx = gml_new_data_idx(gml)))
   {
      vec->use = 0;
      return 0;
   }

   dat = &gml->dat[ DatIdx ];
   dat->AloTyp = GmlRawDat;
   dat->MshTyp = GmlVecDat;
   dat->MemAcs = GmlInput;
   dat->ItmTyp = FltTyp;
   dat->NmbItm = vec->NmbValTyp * vec->VecValSiz;
   dat->ItmSiz = vec->FltSiz;
   dat->ItmLen = 1;
   dat->NmbLin = NmbLin;
   dat->LinSiz = dat->NmbItm * dat->ItmSiz;
   dat->MemSiz = (size_t)NmbLin * (size_t)dat->LinSiz;
   dat->nam    = "vector";

   if(!gml_alloc_data(gml, dat))
   {
      dat->use = 0;
      vec->use = 0;
      return 0;
   }

   dst = (char *)dat->CpuMem;
   if(val)
      for(i=0;i<NmbLin;i++)
         memcpy(dst + (size_t)i * dat->LinSiz, (const char *)val + (size_t)i * BlkSiz * vec->FltSiz,
                (size_t)BlkSiz * vec->FltSiz);

   vec->idx = DatIdx;
   gml_upload(gml, DatIdx);
   return VecIdx;
}

/* datatype holding the lines of a vector (the reference keeps it in
   vec->idx, sources/gmlib3.c:1504, without exposing it) */
int GmlxVectorData(size_t GmlIdx, int VecIdx)
{
   GETGMLPTR(gml, GmlIdx);
   if(VecIdx < 1 || VecIdx > GmlMaxVec || !gml->vec[VecIdx].use)
      return 0;
   return gml->vec[VecIdx].idx;
}

/* ========================================================================= */
/* operations                                                                 */
/* ========================================================================= */

static GmlVecSct *chk_vec(GmlSct *gml, int idx)
{
   if(idx < 1 || idx > GmlMaxVec || !gml->vec[idx].use)
      return NULL;
   return &gml->vec[idx];
}

static void *vec_ptr(GmlSct *gml, GmlVecSct *v)
{
   return gml->dat[ v->idx ].GpuMem;
}

static int vec_stride(GmlVecSct *v)
{
   return v->NmbValTyp * v->VecValSiz;
}

int GmlMultMatVec(size_t GmlIdx, int MatIdx, int VecIdx1, int VecIdx2)
{
   GETGMLPTR(gml, GmlIdx);
   GmlMatSct *mat;
   GmlVecSct *v1, *v2;
   GmlKrnSct *krn;
   int res;

   if(MatIdx < 1 || MatIdx > GmlMaxMat || !gml->mat[MatIdx].use)
   {
      printf("Invalid data index: %d\n", MatIdx);
      return -1;
   }
   mat = &gml->mat[ MatIdx ];

   if(!(v1 = chk_vec(gml, VecIdx1)))
   {
      printf("Invalid data index: %d\n", VecIdx1);
      return -2;
   }
   if(!(v2 = chk_vec(gml, VecIdx2)))
   {
      printf("Invalid data index: %d\n", VecIdx2);
      return -3;
   }
   if(mat->NmbLin != v1->NmbLin || mat->NmbLin != v2->NmbLin
   || v1->FltTyp != mat->FltTyp || v2->FltTyp != mat->FltTyp
   || vec_stride(v1) < mat->BlkSiz || vec_stride(v2) < mat->BlkSiz)
   {
      printf("vectors and matrix size differ: %d(%d) %d(%d) %d(%d)\n",
             MatIdx, mat->NmbLin, VecIdx1, v1->NmbLin, VecIdx2, v2->NmbLin);
      return -4;
   }

   krn = &gml->krn[ mat->KrnIdx ];
   gml_lib_timer_begin(gml, krn);
   res = gmd_sell_spmv(gml->dev, (const GmlSellDev *)mat->Val, vec_ptr(gml, v2), vec_stride(v2),
                       vec_ptr(gml, v1), vec_stride(v1), 1.0, 0.0, NULL, 0);
   gml_lib_timer_end(gml, krn);

   if(!res)
      return -6;

   gml->MemAcc += mat->MemAcc;
   gml->FltOpp += mat->FltOpp;
   return 1;
}

int GmlAddVec3(size_t GmlIdx, int VecIdx1, int VecIdx2, int VecIdx3, int VecIdx4)
{
   GETGMLPTR(gml, GmlIdx);
   GmlVecSct *v1, *v2, *v3, *v4;

   if(!(v1 = chk_vec(gml, VecIdx1))) { printf("Invalid data index: %d\n", VecIdx1); return -1; }
   if(!(v2 = chk_vec(gml, VecIdx2))) { printf("Invalid data index: %d\n", VecIdx2); return -2; }
   if(!(v3 = chk_vec(gml, VecIdx3))) { printf("Invalid data index: %d\n", VecIdx3); return -3; }
   if(!(v4 = chk_vec(gml, VecIdx4))) { printf("Invalid data index: %d\n", VecIdx4); return -4; }

   if(v1->NmbLin != v2->NmbLin || v1->BlkSiz != v2->BlkSiz)
   {
      printf("vector sizes differ: ID %d (%d x %d) and ID %d (%d x %d)\n",
             VecIdx1, v1->NmbLin, v1->BlkSiz, VecIdx2, v2->NmbLin, v2->BlkSiz);
      return -4;
   }
   if(v1->NmbLin != v4->NmbLin || v1->BlkSiz != v4->BlkSiz
   || v1->NmbLin != v3->NmbLin || v1->BlkSiz != v3->BlkSiz
   || v1->FltTyp != v2->FltTyp || v1->FltTyp != v3->FltTyp || v1->FltTyp != v4->FltTyp)
   {
      printf("vector sizes differ: ID %d (%d x %d) and ID %d (%d x %d)\n",
             VecIdx1, v1->NmbLin, v1->BlkSiz, VecIdx4, v4->NmbLin, v4->BlkSiz);
      return -5;
   }

   if(!gmd_vec_add3(gml->dev, vec_ptr(gml, v1), vec_ptr(gml, v2), vec_ptr(gml, v3),
                    vec_ptr(gml, v4), (size_t)v1->NmbLin * vec_stride(v1), v1->FltSiz))
      return -6;

   gml->MemAcc += (float)v1->NmbLin * v1->BlkSiz * v1->FltSiz * 3;
   gml->FltOpp += (float)v1->NmbLin * v1->BlkSiz;
   return 1;
}

int GmlScaleVec(size_t GmlIdx, int VecIdx, double *mul)
{
   GETGMLPTR(gml, GmlIdx);
   GmlVecSct *v;
   double s = 1.0;

   if(!(v = chk_vec(gml, VecIdx)))
   {
      printf("Invalid data index: %d\n", VecIdx);
      return -2;
   }
   if(mul)
      s = *mul;

   if(!gmd_vec_scale(gml->dev, vec_ptr(gml, v), (size_t)v->NmbLin * vec_stride(v), v->FltSiz, s))
      return -6;

   gml->MemAcc += (float)v->NmbLin * v->BlkSiz * v->FltSiz * 2;
   gml->FltOpp += (float)v->NmbLin * v->BlkSiz;
   return 1;
}

int GmlNormVec(size_t GmlIdx, int VecIdx, int RedIdx, double *nrm)
{
   GETGMLPTR(gml, GmlIdx);
   GmlVecSct *v;
   GmlDatSct *red;
   int res;

   if(!(v = chk_vec(gml, VecIdx)))
   {
      printf("Invalid data index: %d\n", VecIdx);
      return -2;
   }
   if(RedIdx < 1 || RedIdx > GmlMaxDat || !gml->dat[RedIdx].use)
   {
      printf("Invalid data index: %d\n", RedIdx);
      return -1;
   }
   red = &gml->dat[ RedIdx ];
   if(red->ItmTyp != GmlFlt || red->NmbItm != 1 || red->NmbLin < v->NmbLin)
   {
      printf("Invalid data structure: count %d, type %s, length %d\n",
             red->NmbItm, GmlOclTypStr[ red->ItmTyp ], red->ItmLen);
      return -2;
   }

   if(!gmd_vec_rownorm(gml->dev, vec_ptr(gml, v), vec_stride(v), v->BlkSiz < 7 ? v->BlkSiz : 7,
                       v->FltSiz, v->NmbLin, (float *)red->GpuMem))
      return -6;

   *nrm = 0.;
   res = GmlReduceVector(GmlIdx, RedIdx, GmlL1, nrm);
   if(res != 1)
      return res;
   *nrm = sqrt(*nrm);

   gml->MemAcc += (float)v->NmbLin * v->BlkSiz * v->FltSiz * 2;
   gml->FltOpp += (float)v->NmbLin * v->BlkSiz * 2;
   return 1;
}

int GmlMultDiagMatVec(size_t GmlIdx, int VecIdx1, int VecIdx2, int VecIdx3)
{
   GETGMLPTR(gml, GmlIdx);
   GmlVecSct *v1, *v2, *v3;

   if(!(v1 = chk_vec(gml, VecIdx1))) { printf("Invalid data index: %d\n", VecIdx1); return -1; }
   if(!(v2 = chk_vec(gml, VecIdx2))) { printf("Invalid data index: %d\n", VecIdx2); return -2; }
   if(!(v3 = chk_vec(gml, VecIdx3))) { printf("Invalid data index: %d\n", VecIdx3); return -3; }

   if(v1->NmbLin != v3->NmbLin || v1->BlkSiz != v3->BlkSiz * v3->BlkSiz
   || v2->NmbLin != v3->NmbLin || v2->BlkSiz != v3->BlkSiz
   || v1->FltTyp != v2->FltTyp || v1->FltTyp != v3->FltTyp)
   {
      printf("vector sizes differ: ID %d (%d x %d) and ID %d (%d x %d)\n",
             VecIdx1, v1->NmbLin, v1->BlkSiz, VecIdx2, v3->NmbLin, v3->BlkSiz);
      return -4;
   }

   if(!gmd_vec_diag(gml->dev, vec_ptr(gml, v1), vec_stride(v1), vec_ptr(gml, v2),
                    vec_ptr(gml, v3), vec_stride(v3), v3->BlkSiz, v1->FltSiz, v1->NmbLin))
      return -6;

   gml->MemAcc += (float)v1->NmbLin * (v1->BlkSiz + 2 * v2->BlkSiz) * v1->FltSiz;
   gml->FltOpp += (float)v1->NmbLin * 2 * v1->BlkSiz;
   return 1;
}

void gml_release_matrices(GmlSct *gml)
{
   for(int i=1;i<=GmlMaxMat;i++)
      if(gml->mat[i].use && gml->mat[i].Val)
      {
         gml_sell_dev_free(gml, (GmlSellDev *)gml->mat[i].Val);
         free(gml->mat[i].Val);
         gml->mat[i].Val = NULL;
      }
}
