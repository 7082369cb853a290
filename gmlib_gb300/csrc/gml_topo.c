/*
 * gml_topo.c -- topological links: vertex balls, edge/face shells, downlinks,
 * unique edge extraction and element neighbours.
 *
 * Reference: NewBallData (sources/gmlib3.c:743-1168) with its hash helpers
 * GetItmNod/CalHshKey/AddHsh/GetHsh (:1567-1721), GmlExtractEdges
 * (:3719-3873) and GmlSetNeighbours (:4178-4267).
 *
 * The reference inserts every (element, local item) pair into a chained hash
 * table keyed by the item's sorted node tuple, inserting at the chain head,
 * and reads a ball back by walking the chain.  A ball therefore lists its
 * elements in DESCENDING insertion order, each entry coded
 * (element << 4) | local item index.  This file produces the same tables
 * without chains: items are matched through an open-addressing tuple map (or
 * directly by vertex index), counted, and written by a reverse sweep over the
 * elements, which yields exactly the reverse insertion order.
 *
 * Table shapes follow the reference: a degree table, a base table of width
 * LenMatBas[src][dst] for lines 0..MaxPos and, when some degree exceeds it, a
 * high table of width min(2^ceil(log2 maxdeg), LenMatMax[src][dst]) for lines
 * MaxPos..NmbLin-1, MaxPos being the first line whose degree exceeds the base
 * width.  Two documented deviations:
 *   - the reference never fills row 0 of the high table (the line MaxPos is
 *     written into the base table instead, overflowing it,
 *     sources/gmlib3.c:1126-1129), yet the high kernel reads that row for line
 *     MaxPos; here row 0 of the high table holds line MaxPos's ball and the
 *     base row MaxPos holds its first base-width entries;
 *   - the reference's MaxPos search restarts when line 0 is a high-degree line
 *     (`!MaxPos` test, :932); here MaxPos is the first high-degree line,
 *     whichever it is.
 * A degree above LenMatMax makes the link fail instead of overflowing rows.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "gml_internal.h"

/* ------------------------------------------------------------------------- */
/* sub-entity node tuples (reference GetItmNod, sources/gmlib3.c:1567-1620)   */
/* ------------------------------------------------------------------------- */

static int item_nodes(const int *EleNod, int EleTyp, int ItmTyp, int ItmIdx, int *tab)
{
   int i, j, t, n = 0;

   switch(ItmTyp)
   {
      case GmlVertices :
         tab[0] = EleNod[ ItmIdx ];
         return 1;
      case GmlEdges :
         i = EleNod[ GmlItmEdgNod[ EleTyp ][ ItmIdx ][0] ];
         j = EleNod[ GmlItmEdgNod[ EleTyp ][ ItmIdx ][1] ];
         tab[0] = i < j ? i : j;
         tab[1] = i < j ? j : i;
         return 2;
      case GmlTriangles : n = 3; break;
      case GmlQuadrilaterals : n = 4; break;
      default : return 0;
   }

   for(i=0;i<n;i++)
      tab[i] = EleNod[ GmlItmFacNod[ EleTyp ][ ItmIdx ][i] ];

   for(i=0;i<n;i++)
      for(j=i+1;j<n;j++)
         if(tab[i] > tab[j])
         {
            t = tab[i]; tab[i] = tab[j]; tab[j] = t;
         }

   return n;
}

/* ------------------------------------------------------------------------- */
/* open-addressing map from a sorted node tuple (<= 4 ints) to an int value   */
/* ------------------------------------------------------------------------- */

typedef struct
{
   int      len;
   size_t   cap, mask, cnt;
   int      *key;       /* cap * len node indices, key[0] == -1: empty */
   int      *val;
}TupMap;

static uint64_t tup_hash(const int *t, int len)
{
   uint64_t h = 0x9e3779b97f4a7c15ULL;
   for(int i=0;i<len;i++)
   {
      h ^= (uint64_t)(uint32_t)t[i] + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
      h *= 0xbf58476d1ce4e5b9ULL;
   }
   return h ^ (h >> 31);
}

static int tup_init(TupMap *m, int len, size_t n)
{
   size_t cap = 16;
   while(cap < 2 * n + 16) cap <<= 1;
   m->len = len; m->cap = cap; m->mask = cap - 1; m->cnt = 0;
   m->key = malloc(cap * len * sizeof(int));
   m->val = malloc(cap * sizeof(int));
   if(!m->key || !m->val) return 0;
   for(size_t i=0;i<cap;i++) m->key[ i * len ] = -1;
   return 1;
}

static void tup_free(TupMap *m) { free(m->key); free(m->val); }

/* returns the value of tuple t, or inserts it with value v and returns -1 */
static int tup_get_or_put(TupMap *m, const int *t, int v)
{
   size_t p = tup_hash(t, m->len) & m->mask;
   for(;;)
   {
      int *k = &m->key[ p * m->len ];
      if(k[0] == -1)
      {
         memcpy(k, t, m->len * sizeof(int));
         m->val[p] = v;
         m->cnt++;
         return -1;
      }
      if(!memcmp(k, t, m->len * sizeof(int)))
         return m->val[p];
      p = (p + 1) & m->mask;
   }
}

static int tup_get(const TupMap *m, const int *t)
{
   size_t p = tup_hash(t, m->len) & m->mask;
   for(;;)
   {
      const int *k = &m->key[ p * m->len ];
      if(k[0] == -1) return -1;
      if(!memcmp(k, t, m->len * sizeof(int))) return m->val[p];
      p = (p + 1) & m->mask;
   }
}

/* ------------------------------------------------------------------------- */
/* link data allocation helper                                                */
/* ------------------------------------------------------------------------- */

static int new_link_dat(GmlSct *gml, int SrcTyp, int DstTyp, int ItmTyp,
                        int NmbItm, int ItmLen, int NmbLin, const char *nam,
                        const char *VoyNam)
{
   int idx = gml_new_data_idx(gml);
   GmlDatSct *dat;

   if(!idx)
      return 0;

   dat = &gml->dat[ idx ];
   dat->AloTyp = GmlLnkDat;
   dat->MshTyp = SrcTyp;
   dat->LnkTyp = DstTyp;
   dat->MemAcs = GmlInout;
   dat->ItmTyp = ItmTyp;
   dat->NmbItm = NmbItm;
   dat->ItmSiz = GmlOclTypSiz[ ItmTyp ];
   dat->ItmLen = ItmLen;
   dat->NmbLin = NmbLin;
   dat->LinSiz = NmbItm * dat->ItmSiz;
   dat->MemSiz = (size_t)NmbLin * (size_t)dat->LinSiz;
   dat->nam    = nam;
   dat->VoyNam = VoyNam;

   if(!gml_alloc_data(gml, dat))
   {
      dat->use = 0;
      return 0;
   }

   return idx;
}

/* ------------------------------------------------------------------------- */
/* uplinks (balls, shells) and downlinks                                      */
/* ------------------------------------------------------------------------- */

int gml_new_ball_data(GmlSct *gml, int SrcTyp, int DstTyp,
                      const char *BalNam, const char *DegNam, const char *VoyNam)
{
   GmlDatSct   *src, *dst;
   int         HshTyp, dir, i, j, k, n, tab[4];
   int         DstNmbItm, SrcNmbItm, DstLen, SrcLen;
   const int   *SrcNod, *DstNod;
   TupMap      map;
   int         use_map;

   if(SrcTyp < 0 || SrcTyp >= GmlMaxEleTyp || DstTyp < 0 || DstTyp >= GmlMaxEleTyp)
      return 0;

   if(!gml->TypIdx[ SrcTyp ] || !gml->TypIdx[ DstTyp ])
   {
      printf("Cannot build a link %s -> %s: mesh data missing\n",
             GmlBalTypStr[ SrcTyp ], GmlBalTypStr[ DstTyp ]);
      return 0;
   }

   src = &gml->dat[ gml->TypIdx[ SrcTyp ] ];
   dst = &gml->dat[ gml->TypIdx[ DstTyp ] ];
   SrcNod = (const int *)src->CpuMem;
   DstNod = (const int *)dst->CpuMem;
   SrcLen = src->ItmLen;
   DstLen = dst->ItmLen;

   if(SrcTyp < DstTyp)       { dir =  1; HshTyp = SrcTyp; }
   else if(SrcTyp > DstTyp)  { dir = -1; HshTyp = DstTyp; }
   else
   {
      puts("Intra-type links are built by GmlSetNeighbours or GmlNewLinkData.");
      return 0;
   }

   SrcNmbItm = (SrcTyp != HshTyp) ? GmlNmbTpoLnk[ SrcTyp ][ HshTyp ] : 1;
   DstNmbItm = (DstTyp != HshTyp) ? GmlNmbTpoLnk[ DstTyp ][ HshTyp ] : 1;

   if(gml->DbgFlg)
      printf("Building %s link %s -> %s\n", dir == 1 ? "up" : "down",
             GmlBalTypStr[ SrcTyp ], GmlBalTypStr[ DstTyp ]);

   /* Map each hashed-type entity (the source for uplinks, the destination for
      downlinks) to its line index.  Vertices are their own key. */
   use_map = (HshTyp != GmlVertices);

   if(dir == 1)
   {
      int   BalSiz = GmlLenMatBas[ SrcTyp ][ DstTyp ];
      int   MaxSiz = GmlLenMatMax[ SrcTyp ][ DstTyp ];
      int   MaxDeg = 0, MaxPos = -1, HghSiz = 0, DegIdx, BalIdx, HghIdx = 0;
      int   VecCnt, VecSiz, ItmTyp, NmbSrc = src->NmbLin;
      int   *DegTab, *fill, *BalTab, *HghTab = NULL;

      if(use_map)
      {
         if(!tup_init(&map, GmlItmNmbVer[ HshTyp ], NmbSrc))
            return 0;
         for(i=0;i<NmbSrc;i++)
         {
            n = item_nodes(&SrcNod[ i * SrcLen ], SrcTyp, HshTyp, 0, tab);
            (void)n;
            tup_get_or_put(&map, tab, i);
         }
      }

      DegIdx = new_link_dat(gml, SrcTyp, DstTyp, GmlInt, 1, 0, NmbSrc, DegNam, NULL);
      if(!DegIdx)
         goto fail_map;
      DegTab = (int *)gml->dat[ DegIdx ].CpuMem;
      gml->CntMat[ SrcTyp ][ DstTyp ] = DegIdx;

      /* degrees */
      for(i=0;i<dst->NmbLin;i++)
         for(j=0;j<DstNmbItm;j++)
         {
            item_nodes(&DstNod[ i * DstLen ], DstTyp, HshTyp, j, tab);
            k = use_map ? tup_get(&map, tab) : tab[0];
            if(k >= 0 && k < NmbSrc)
               DegTab[k]++;
         }

      for(i=0;i<NmbSrc;i++)
      {
         if(DegTab[i] > MaxDeg) MaxDeg = DegTab[i];
         if(MaxPos < 0 && DegTab[i] > BalSiz) MaxPos = i;
      }

      if(BalSiz == MaxSiz || MaxDeg <= BalSiz)
      {
         HghSiz = 0;
         MaxPos = NmbSrc;
      }
      else
      {
         int p2 = 1;
         while(p2 < MaxDeg) p2 <<= 1;
         if(MaxDeg > MaxSiz)
         {
            printf("Link %s -> %s: degree %d exceeds the maximum width %d\n",
                   GmlBalTypStr[ SrcTyp ], GmlBalTypStr[ DstTyp ], MaxDeg, MaxSiz);
            goto fail_map;
         }
         HghSiz = p2 < MaxSiz ? p2 : MaxSiz;
      }

      gml->SizMatHgh[ SrcTyp ][ DstTyp ] = HghSiz;

      gml_get_cnt_vec(BalSiz, &VecCnt, &VecSiz, &ItmTyp);
      BalIdx = new_link_dat(gml, SrcTyp, DstTyp, ItmTyp, VecCnt, BalSiz,
                            MaxPos + 1, BalNam, VoyNam);
      if(!BalIdx)
         goto fail_map;
      gml->LnkMat[ SrcTyp ][ DstTyp ] = BalIdx;
      BalTab = (int *)gml->dat[ BalIdx ].CpuMem;

      if(HghSiz)
      {
         gml_get_cnt_vec(HghSiz, &VecCnt, &VecSiz, &ItmTyp);
         HghIdx = new_link_dat(gml, SrcTyp, DstTyp, ItmTyp, VecCnt, HghSiz,
                               NmbSrc - MaxPos, BalNam, VoyNam);
         if(!HghIdx)
            goto fail_map;
         gml->LnkHgh[ SrcTyp ][ DstTyp ] = HghIdx;
         HghTab = (int *)gml->dat[ HghIdx ].CpuMem;
      }

      /* reverse sweep: entries land in descending (element, item) order */
      fill = calloc(NmbSrc, sizeof(int));
      if(!fill)
         goto fail_map;

      for(i=dst->NmbLin-1;i>=0;i--)
         for(j=DstNmbItm-1;j>=0;j--)
         {
            int cod = (i << 4) | j, f;
            item_nodes(&DstNod[ i * DstLen ], DstTyp, HshTyp, j, tab);
            k = use_map ? tup_get(&map, tab) : tab[0];
            if(k < 0 || k >= NmbSrc)
               continue;
            f = fill[k]++;
            if(k < MaxPos)
               BalTab[ (size_t)k * BalSiz + f ] = cod;
            else
            {
               if(k == MaxPos && f < BalSiz)
                  BalTab[ (size_t)k * BalSiz + f ] = cod;
               HghTab[ (size_t)(k - MaxPos) * HghSiz + f ] = cod;
            }
         }

      free(fill);

      gml_upload(gml, BalIdx);
      gml_upload(gml, DegIdx);
      if(HghIdx)
         gml_upload(gml, HghIdx);

      if(gml->DbgFlg)
         printf("Ball %s -> %s: base %d lines x %d, high %d lines x %d, max degree %d\n",
                GmlBalTypStr[ SrcTyp ], GmlBalTypStr[ DstTyp ], MaxPos + 1, BalSiz,
                HghIdx ? NmbSrc - MaxPos : 0, HghSiz, MaxDeg);

      if(use_map) tup_free(&map);
      return 1;

fail_map:
      if(use_map) tup_free(&map);
      return 0;
   }
   else
   {
      /* downlink: each source element lists the indices of its sub-entities
         of the destination type, 0 when absent (reference :1041-1071) */
      int   NmbDat = GmlLenMatBas[ SrcTyp ][ DstTyp ];
      int   VecCnt, VecSiz, ItmTyp, BalIdx, *BalTab, RowLen;

      if(use_map)
      {
         if(!tup_init(&map, GmlItmNmbVer[ HshTyp ], dst->NmbLin))
            return 0;
         for(i=0;i<dst->NmbLin;i++)
         {
            item_nodes(&DstNod[ i * DstLen ], DstTyp, HshTyp, 0, tab);
            tup_get_or_put(&map, tab, i);
         }
      }

      gml_get_cnt_vec(NmbDat, &VecCnt, &VecSiz, &ItmTyp);
      BalIdx = new_link_dat(gml, SrcTyp, DstTyp, ItmTyp, VecCnt, NmbDat,
                            src->NmbLin, BalNam, NULL);
      if(!BalIdx)
      {
         if(use_map) tup_free(&map);
         return 0;
      }
      gml->LnkMat[ SrcTyp ][ DstTyp ] = BalIdx;
      BalTab = (int *)gml->dat[ BalIdx ].CpuMem;
      RowLen = VecCnt * VecSiz;

      for(i=0;i<src->NmbLin;i++)
         for(j=0;j<SrcNmbItm && j<RowLen;j++)
         {
            item_nodes(&SrcNod[ i * SrcLen ], SrcTyp, HshTyp, j, tab);
            k = use_map ? tup_get(&map, tab) : tab[0];
            BalTab[ (size_t)i * RowLen + j ] = k > 0 ? k : 0;
         }

      if(use_map) tup_free(&map);
      gml_upload(gml, BalIdx);
      return 1;
   }
}

/* ------------------------------------------------------------------------- */
/* GmlExtractEdges (reference sources/gmlib3.c:3719-3873)                     */
/* ------------------------------------------------------------------------- */

/* Unique edges of every element type, numbered in order of first appearance
   (element types ascending, elements ascending, local edges in ItmEdgNod
   order), stored as (min node, max node, ref 0).  Edges that already exist in
   the GmlEdges data keep their position and reference at the front of the new
   table (the reference intends this but writes the new volume edges past the
   end of the table it allocated, :3808-3866). */
int GmlExtractEdges(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   TupMap   map;
   int      typ, i, j, tab[4], NmbEdg = 0, OldNmb = 0, OldIdx, EdgIdx;
   int      *OldTab = NULL, *OldRef = NULL, *EdgTab, *RefTab;
   size_t   tot = 0;

   for(typ=GmlEdges+1; typ<GmlMaxEleTyp; typ++)
      if(gml->TypIdx[ typ ])
         tot += (size_t)gml->dat[ gml->TypIdx[ typ ] ].NmbLin * GmlItmNmbEdg[ typ ];

   OldIdx = gml->TypIdx[ GmlEdges ];
   if(OldIdx)
   {
      GmlDatSct *old = &gml->dat[ OldIdx ];
      OldNmb = old->NmbLin;
      tot += OldNmb;
   }

   if(!tup_init(&map, 2, tot / 2 + 16))
      return 0;

   if(OldNmb)
   {
      GmlDatSct *old = &gml->dat[ OldIdx ];
      gml_download(gml, OldIdx);
      gml_download(gml, gml->RefIdx[ GmlEdges ]);
      OldTab = malloc((size_t)OldNmb * 2 * sizeof(int));
      OldRef = malloc((size_t)OldNmb * sizeof(int));
      if(!OldTab || !OldRef) { tup_free(&map); free(OldTab); free(OldRef); return 0; }
      for(i=0;i<OldNmb;i++)
      {
         const int *e = &((const int *)old->CpuMem)[ i * 2 ];
         tab[0] = e[0] < e[1] ? e[0] : e[1];
         tab[1] = e[0] < e[1] ? e[1] : e[0];
         OldTab[ 2*i ] = tab[0];
         OldTab[ 2*i+1 ] = tab[1];
         OldRef[i] = ((const int *)gml->dat[ gml->RefIdx[ GmlEdges ] ].CpuMem)[i];
         if(tup_get_or_put(&map, tab, NmbEdg) < 0)
            NmbEdg++;
      }
   }

   for(typ=GmlEdges+1; typ<GmlMaxEleTyp; typ++)
   {
      GmlDatSct *dat;
      const int *nod;
      if(!gml->TypIdx[ typ ])
         continue;
      dat = &gml->dat[ gml->TypIdx[ typ ] ];
      nod = (const int *)dat->CpuMem;
      for(i=0;i<dat->NmbLin;i++)
         for(j=0;j<GmlItmNmbEdg[ typ ];j++)
         {
            item_nodes(&nod[ i * dat->ItmLen ], typ, GmlEdges, j, tab);
            if(tup_get_or_put(&map, tab, NmbEdg) < 0)
               NmbEdg++;
         }
   }

   if(OldIdx)
      GmlFreeData(GmlIdx, OldIdx), GmlFreeData(GmlIdx, gml->RefIdx[ GmlEdges ]);

   EdgIdx = GmlNewMeshData(GmlIdx, GmlEdges, NmbEdg);
   if(!EdgIdx)
   {
      tup_free(&map); free(OldTab); free(OldRef);
      return 0;
   }

   /* write the table in numbering order by replaying the same sweep */
   EdgTab = (int *)gml->dat[ EdgIdx ].CpuMem;
   RefTab = (int *)gml->dat[ gml->RefIdx[ GmlEdges ] ].CpuMem;
   tup_free(&map);
   if(!tup_init(&map, 2, tot / 2 + 16))
      return 0;
   NmbEdg = 0;

   for(i=0;i<OldNmb;i++)
      if(tup_get_or_put(&map, &OldTab[ 2*i ], NmbEdg) < 0)
      {
         EdgTab[ 2*NmbEdg ] = OldTab[ 2*i ];
         EdgTab[ 2*NmbEdg+1 ] = OldTab[ 2*i+1 ];
         RefTab[ NmbEdg ] = OldRef[i];
         NmbEdg++;
      }

   for(typ=GmlEdges+1; typ<GmlMaxEleTyp; typ++)
   {
      GmlDatSct *dat;
      const int *nod;
      if(!gml->TypIdx[ typ ])
         continue;
      dat = &gml->dat[ gml->TypIdx[ typ ] ];
      nod = (const int *)dat->CpuMem;
      for(i=0;i<dat->NmbLin;i++)
         for(j=0;j<GmlItmNmbEdg[ typ ];j++)
         {
            item_nodes(&nod[ i * dat->ItmLen ], typ, GmlEdges, j, tab);
            if(tup_get_or_put(&map, tab, NmbEdg) < 0)
            {
               EdgTab[ 2*NmbEdg ] = tab[0];
               EdgTab[ 2*NmbEdg+1 ] = tab[1];
               RefTab[ NmbEdg ] = 0;
               NmbEdg++;
            }
         }
   }

   tup_free(&map);
   free(OldTab);
   free(OldRef);

   gml_upload(gml, EdgIdx);
   gml_upload(gml, gml->RefIdx[ GmlEdges ]);

   if(gml->DbgFlg)
      printf("Extracted %d unique edges\n", NmbEdg);

   return NmbEdg;
}

/* ------------------------------------------------------------------------- */
/* GmlExtractFaces (reference sources/gmlib3.c:3880-4171)                     */
/* ------------------------------------------------------------------------- */

/* Every distinct triangle and quadrilateral face of the mesh.  Faces are
   visited in the reference's order: existing triangles, existing
   quadrilaterals, then the faces of tetrahedra, pyramids, prisms and
   hexahedra, element by element and face by face; the first visit of a
   node set defines the face.  As in the reference the face's nodes are
   stored sorted (GetItmNod sorts them for hashing), existing surface faces
   keep their reference and new faces get 0.  The triangle and quadrilateral
   datatypes are replaced by the extracted ones.  Returns the number of
   triangles plus quadrilaterals.  Deviation: the reference gives an
   existing quadrilateral its fourth node as reference (QadTab[i][3],
   :4093); here it keeps its reference. */
static int faces_to_datatype(GmlSct *gml, size_t GmlIdx, int typ, const int *tab, const int *ref,
                             int n)
{
   const int nn = typ == GmlTriangles ? 3 : 4;
   int idx, *row, *rt, w;
   GmlDatSct *d;
   if(gml->TypIdx[typ])
   {
      int old = gml->TypIdx[typ];
      GmlFreeData(GmlIdx, gml->RefIdx[typ]);
      GmlFreeData(GmlIdx, old);
      gml->TypIdx[typ] = gml->RefIdx[typ] = 0;
   }
   if(!n)
      return 1;
   if(!(idx = GmlNewMeshData(GmlIdx, typ, n)))
      return 0;
   d = &gml->dat[idx];
   w = GmlTypVecSiz[ d->ItmTyp ];
   row = (int *)d->CpuMem;
   rt = (int *)gml->dat[ gml->RefIdx[typ] ].CpuMem;
   for(int i=0;i<n;i++)
   {
      for(int c=0;c<w;c++)
         row[(size_t)i * w + c] = c < nn ? tab[(size_t)i * nn + c] : 0;
      rt[i] = ref[i];
   }
   return gml_upload(gml, idx) && gml_upload(gml, gml->RefIdx[typ]);
}

int GmlExtractFaces(size_t GmlIdx)
{
   GETGMLPTR(gml, GmlIdx);
   size_t cap[2] = { 0, 0 };
   int n[2] = { 0, 0 }, *tab[2] = { NULL, NULL }, *ref[2] = { NULL, NULL }, ok = 0;
   TupMap map[2];
   int have[2] = { 0, 0 };

   for(int typ=GmlTriangles;typ<GmlMaxEleTyp;typ++)
      if(gml->TypIdx[typ])
         for(int j=0;j<GmlItmNmbFac[typ];j++)
            cap[ GmlItmFacDeg[typ][j] == 4 ] += (size_t)gml->dat[ gml->TypIdx[typ] ].NmbLin;

   for(int k=0;k<2;k++)
   {
      const int len = k ? 4 : 3;
      if(!cap[k])
         continue;
      if(!tup_init(&map[k], len, cap[k]))
         goto done;
      have[k] = 1;
      tab[k] = malloc(cap[k] * len * sizeof(int));
      ref[k] = malloc(cap[k] * sizeof(int));
      if(!tab[k] || !ref[k])
         goto done;
   }

   for(int typ=GmlTriangles;typ<GmlMaxEleTyp;typ++)
   {
      GmlDatSct *d;
      const int *nod, *rt;
      int w;
      if(!gml->TypIdx[typ])
         continue;
      d = &gml->dat[ gml->TypIdx[typ] ];
      gml_wait_upload(gml, d);
      nod = (const int *)d->CpuMem;
      rt = (const int *)gml->dat[ gml->RefIdx[typ] ].CpuMem;
      w = GmlTypVecSiz[ d->ItmTyp ];
      for(int i=0;i<d->NmbLin;i++)
         for(int j=0;j<GmlItmNmbFac[typ];j++)
         {
            const int k = GmlItmFacDeg[typ][j] == 4, len = k ? 4 : 3;
            int t[4];
            item_nodes(nod + (size_t)i * w, typ, k ? GmlQuadrilaterals : GmlTriangles, j, t);
            if(tup_get_or_put(&map[k], t, n[k]) < 0)
            {
               memcpy(tab[k] + (size_t)n[k] * len, t, len * sizeof(int));
               ref[k][ n[k] ] = (typ == GmlTriangles || typ == GmlQuadrilaterals) && rt ? rt[i] : 0;
               n[k]++;
            }
         }
   }

   ok = faces_to_datatype(gml, GmlIdx, GmlTriangles, tab[0], ref[0], n[0])
     && faces_to_datatype(gml, GmlIdx, GmlQuadrilaterals, tab[1], ref[1], n[1]);

done:
   for(int k=0;k<2;k++)
   {
      if(have[k])
         tup_free(&map[k]);
      free(tab[k]);
      free(ref[k]);
   }
   return ok ? n[0] + n[1] : 0;
}

/* ------------------------------------------------------------------------- */
/* GmlSetNeighbours (reference sources/gmlib3.c:4178-4267)                    */
/* ------------------------------------------------------------------------- */

/* Element-to-element neighbours through shared faces (tets, hexes) or edges
   (triangles, quads): for each element and each of its NmbTpoLnk[typ][NgbTyp]
   sub-entities, the index of the other element sharing it, 0 when none
   (0 is also element 0: the reference uses the same convention).  When more
   than two elements share a sub-entity, the last one found that is not the
   element itself is kept, as the reference does. */
int GmlSetNeighbours(size_t GmlIdx, int typ)
{
   GETGMLPTR(gml, GmlIdx);
   GmlDatSct   *dat;
   const int   *nod;
   int         HshTyp, NmbItm, i, j, tab[4], NgbIdx, *cnt, *own, *lst;
   int         *NgbTab, RowLen;
   TupMap      map;

   if(typ == GmlPyramids || typ == GmlPrisms)
   {
      puts("Neighbours calculation between prisms or pyramids is not yet implemented.");
      return 0;
   }
   if(typ <= GmlVertices || typ >= GmlMaxEleTyp || !gml->TypIdx[ typ ])
      return 0;

   dat    = &gml->dat[ gml->TypIdx[ typ ] ];
   nod    = (const int *)dat->CpuMem;
   HshTyp = GmlNgbTyp[ typ ];
   NmbItm = GmlNmbTpoLnk[ typ ][ HshTyp ];

   if(!tup_init(&map, GmlItmNmbVer[ HshTyp ], (size_t)dat->NmbLin * NmbItm))
      return 0;

   /* first pass: number the distinct sub-entities and count their users */
   cnt = calloc((size_t)dat->NmbLin * NmbItm, sizeof(int));
   own = malloc((size_t)dat->NmbLin * NmbItm * sizeof(int));
   if(!cnt || !own) { tup_free(&map); free(cnt); free(own); return 0; }
   {
      int nb = 0, id;
      for(i=0;i<dat->NmbLin;i++)
         for(j=0;j<NmbItm;j++)
         {
            item_nodes(&nod[ i * dat->ItmLen ], typ, HshTyp, j, tab);
            id = tup_get_or_put(&map, tab, nb);
            if(id < 0) id = nb++;
            own[ (size_t)i * NmbItm + j ] = id;
            cnt[id]++;
         }
   }

   /* CSR of users per sub-entity, filled in ascending element order */
   {
      size_t ns = map.cnt, s, acc = 0;
      size_t *ptr = malloc((ns + 1) * sizeof(size_t));
      size_t *pos;
      if(!ptr) { tup_free(&map); free(cnt); free(own); return 0; }
      for(s=0;s<ns;s++) { ptr[s] = acc; acc += cnt[s]; }
      ptr[ns] = acc;
      lst = malloc(acc * sizeof(int));
      pos = malloc(ns * sizeof(size_t));
      if(!lst || !pos) { free(ptr); free(lst); free(pos); tup_free(&map); free(cnt); free(own); return 0; }
      for(s=0;s<ns;s++) pos[s] = ptr[s];
      for(i=0;i<dat->NmbLin;i++)
         for(j=0;j<NmbItm;j++)
            lst[ pos[ own[ (size_t)i * NmbItm + j ] ]++ ] = i;

      NgbIdx = GmlNewLinkData(GmlIdx, typ, typ, GmlItmNmbFac[ typ ] ? GmlItmNmbFac[ typ ] : NmbItm, "ngb");
      if(!NgbIdx) { free(ptr); free(lst); free(pos); tup_free(&map); free(cnt); free(own); return 0; }
      NgbTab = (int *)gml->dat[ NgbIdx ].CpuMem;
      RowLen = gml->dat[ NgbIdx ].LinSiz / (int)sizeof(int);

      for(i=0;i<dat->NmbLin;i++)
         for(j=0;j<NmbItm && j<RowLen;j++)
         {
            size_t id = own[ (size_t)i * NmbItm + j ], u;
            int ngb = 0;
            /* the reference keeps the earliest-inserted other element */
            for(u=ptr[id];u<ptr[id+1];u++)
               if(lst[u] != i)
               {
                  ngb = lst[u];
                  break;
               }
            NgbTab[ (size_t)i * RowLen + j ] = ngb;
         }

      free(ptr); free(pos); free(lst);
   }

   tup_free(&map);
   free(cnt);
   free(own);
   gml_upload(gml, NgbIdx);
   return NgbIdx;
}
