/*
 * gml_codegen.c -- CUDA C++ generation for GmlCompileKernel.
 *
 * Input: the argument plan built by GmlCompileKernel (link tables, degree
 * tables, datatypes and reference arrays in the contract's order) and the
 * user's OpenCL-C body.
 * Output: one CUDA kernel source with the reference's naming contract, so the
 * body compiles unchanged:
 *
 *   parameters   <nam>Tab per argument, in argument order, then
 *                GmlParSct *GmlPar and const int2 count   (ref :2635-2663)
 *   counters     int cnt; int <Ent>Idx = cnt + count.s1;  (ref :2739-2748)
 *   locals       <nam>, <nam>[MaxDeg][NmbItm], <nam>Deg, <nam>Nul,
 *                #define <nam>DegMax, voyeurs <Voy>[]      (ref :2670-2732)
 *   reads        downlinks, neighbour links, balls with voyeurs (ref :2755-2885)
 *   body         verbatim after dialect rewriting           (ref :2892-2896)
 *   writes       <nam>Tab[cnt + count.s1] = <nam>            (ref :2903-2938)
 *
 * The GB300 difference is in the uplink (ball/shell) gathers.  The reference
 * fills, for every ball entry k < DegMax and every item j, a per-thread array
 * X[k][j] with a conditional global load (128 float4 loads and 2 KB of
 * private memory per vertex for the NodeSmoothing gather).  In "lazy" mode
 * the generator declares X as an accessor object (gml_up / gml_up1 in
 * gml_cl.h) whose operator[] performs the load the body actually asks for,
 * with the same value (null beyond the degree).  The ball row, the voyeur
 * indices and the link vectors are accessors too.  Bodies that need real
 * arrays (writing into a gathered local, taking its address) fail to compile
 * in lazy mode and are regenerated in "eager" mode, which reproduces the
 * reference's prologue statement by statement.
 *
 * Read-only arguments are passed as const __restrict__ pointers so that the
 * compiler can route their loads through the read-only data path.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_internal.h"

typedef struct { char *buf; size_t len, cap; } Out;

static void emit(Out *o, const char *fmt, ...)
{
   va_list ap;
   int n;
   for(;;)
   {
      size_t room = o->cap - o->len;
      va_start(ap, fmt);
      n = vsnprintf(o->buf + o->len, room, fmt, ap);
      va_end(ap);
      if(n >= 0 && (size_t)n < room)
      {
         o->len += n;
         return;
      }
      o->cap = o->cap * 2 + (size_t)n + 1024;
      o->buf = realloc(o->buf, o->cap);
   }
}

static const char HexDig[] = "0123456789abcdef";

static int is_read_only(const GmlArgSct *a)
{
   return !(a->FlgTab & GmlWriteMode) && !(a->FlgTab & GmlManual);
}

/* lazy accessor for an uplinked (count-linked) datatype? */
static int lazy_data(const GmlArgSct *a, const GmlArgSct *cpt, int lazy)
{
   return lazy && cpt && (a->FlgTab & GmlReadMode) && is_read_only(a);
}

/* The row object <link>Row that the lazy accessors of one ball link share
   (gml_balrow in gml_cl.h), declared once before its first user.  Rows
   whose width is a multiple of four codes are read in 16-byte pieces
   (V = 4), others one code at a time (V = 1).  Its degree is the count of
   a datatype uplinked through this link, else the row width.  Returns V. */
static int ensure_row(Out *o, const GmlArgSct *ArgTab, int NmbArg, int li, int *RowDone)
{
   const GmlArgSct *l = &ArgTab[li];
   const int W = GmlTypVecSiz[ l->ItmTyp ] * l->NmbItm, V = (W % 4) ? 1 : 4;
   const char *deg = NULL;
   char DegStr[16];
   int j;

   if(RowDone[li])
      return RowDone[li];
   for(j=0;j<NmbArg && !deg;j++)
      if(ArgTab[j].LnkIdx == li && ArgTab[j].CntIdx != -1)
         deg = ArgTab[ ArgTab[j].CntIdx ].nam;
   if(!deg)
   {
      snprintf(DegStr, sizeof(DegStr), "%d", W);
      deg = DegStr;
   }
   emit(o, "   gml_balrow<%d> %sRow = { (const int *)(%sTab + cnt), %s%s };\n",
        V, l->nam, l->nam, deg, V == 4 ? ", -1" : "");
   RowDone[li] = V;
   return V;
}

/* ------------------------------------------------------------------------- */
/* Eager reads: the text of the reference's read prologue (sources/gmlib3.c:  */
/* 2755-2885), which bodies needing real arrays compile against.  Item j of   */
/* a datatype is read for every gather slot k of its link: the slot's index   */
/* is link component k (vector k/16 of the line, lane k%16), guarded by the   */
/* degree (counted uplinks) or by the component itself (neighbour links),    */
/* and shifted right by 4 for ball entries, whose low bits are the voyeur.   */
/* ------------------------------------------------------------------------- */

/* buf = "[v]" when on, else "" */
static const char *sub(char *buf, size_t n, int on, int v)
{
   if(on)
      snprintf(buf, n, "[%d]", v);
   else
      buf[0] = 0;
   return buf;
}

/* where line `cnt` of the kernel finds slot k of its link */
static void slot_index(char *buf, size_t n, const GmlArgSct *a, const GmlArgSct *lnk, int k)
{
   char vec[16];
   if(!lnk)
      snprintf(buf, n, "%s", a->LnkDir == 1 ? "cnt" : "cnt + count.s1");
   else if(lnk->ItmLen > 1)
      snprintf(buf, n, "%s%s.s%c", lnk->nam, sub(vec, sizeof vec, lnk->NmbItm > 1, k / 16),
               HexDig[ k & 15 ]);
   else
      snprintf(buf, n, "%s%s", lnk->nam, sub(vec, sizeof vec, lnk->NmbItm > 1, k / 16));
}

static void emit_eager_item(Out *o, const GmlArgSct *a, const GmlArgSct *lnk,
                            const GmlArgSct *cpt, int j)
{
   const int slots = (lnk && lnk->NmbItm * lnk->ItmLen > 1) ? lnk->NmbItm * lnk->ItmLen : 1;
   const int nul = cpt || (lnk && lnk->LnkDir == 0);
   char item[32], idx[300];

   sub(item, sizeof item, a->NmbItm > 1, j);
   if(cpt)
      emit(o, "   %sDeg = %s;\n", a->nam, cpt->nam);
   if(nul)
      emit(o, "   %sNul = gml_zero<%s>();\n", a->nam, GmlOclTypStr[ a->ItmTyp ]);

   if(a->FlgTab & GmlVoyeurs)
   {
      /* a ball row: load it, split off the voyeurs, keep the entities */
      if(lnk)
         snprintf(idx, sizeof idx, "%s", lnk->nam);
      else
         slot_index(idx, sizeof idx, a, NULL, 0);
      emit(o, "   %s%s = %sTab[ %s ]%s;\n", a->nam, item, a->nam, idx, item);
      for(int l=0;l<a->ItmLen;l++)
         emit(o, "   %s[%d] = %s%s.s%c & 7;\n", a->VoyNam, j * a->ItmLen + l, a->nam, item, HexDig[l]);
      emit(o, "   %s%s = %s%s >> 4;\n", a->nam, item, a->nam, item);
      return;
   }

   for(int k=0;k<slots;k++)
   {
      char slot[32], pre[300] = "", post[300] = "";

      slot_index(idx, sizeof idx, a, lnk, k);
      if(cpt)
      {
         snprintf(pre, sizeof pre, "(%sDeg >= %d) ?", a->nam, k + 1);
         snprintf(post, sizeof post, ": %sNul", a->nam);
      }
      else if(lnk && lnk->LnkDir == 0)
      {
         char lane[16] = "";
         if(lnk->ItmLen > 1)
            snprintf(lane, sizeof lane, ".s%c", HexDig[ k & 15 ]);
         snprintf(pre, sizeof pre, "%s%s ?", lnk->nam, lane);
         snprintf(post, sizeof post, ": %sNul", a->nam);
      }
      emit(o, "   %s%s%s = %s %sTab[ %s ]%s %s %s;\n",
           a->nam, sub(slot, sizeof slot, slots > 1, k), item, pre, a->nam, idx, item,
           a->LnkDir == 1 ? ">> 4" : "", post);
   }
}

/* Argument i is a table of links read at the thread's own line (one item
   of 4, 8, 16 or 32 bytes) through which other arguments are gathered. */
static int stream_link(const GmlArgSct *ArgTab, int NmbArg, int i)
{
   const GmlArgSct *a = &ArgTab[i];
   const int siz = GmlOclTypSiz[ a->ItmTyp ];
   int j;

   if(a->LnkIdx != -1 || a->CntIdx != -1 || a->LnkDir == 1 || a->NmbItm != 1
   || (a->FlgTab & GmlVoyeurs) || !is_read_only(a)
   || (siz != 4 && siz != 8 && siz != 16 && siz != 32))
      return 0;
   for(j=0;j<NmbArg;j++)
      if(j != i && ArgTab[j].LnkIdx == i)
         return 1;
   return 0;
}

int gml_generate(char **res, const char *PrcNam, int MshTyp, int NmbArg,
                 const GmlArgSct *ArgTab, const char *KrnSrc, const char *UsrTlk,
                 const char *ParSrc, int lazy)
{
   Out o;
   int i, j, V;
   char *tmp;

   o.cap = 16384;
   o.len = 0;
   o.buf = malloc(o.cap);
   o.buf[0] = 0;

   emit(&o, "// GMlib GB300 generated kernel: %s (%s prologue)\n", PrcNam, lazy ? "lazy" : "eager");
   emit(&o, "#include \"gml_cl.h\"\n");
   emit(&o, "// GMlib MESHING AND GEOMETRICAL TOOLKIT\n#include \"gml_toolkit.h\"\n");

   if(UsrTlk)
   {
      tmp = gml_rewrite_opencl(UsrTlk);
      emit(&o, "// USER'S TOOLKIT\n%s\n", tmp);
      free(tmp);
   }

   emit(&o, "// USER'S ARGUMENTS STRUCTURE\n");
   if(ParSrc)
   {
      tmp = gml_rewrite_opencl(ParSrc);
      emit(&o, "%s\n", tmp);
      free(tmp);
   }
   else
      emit(&o, "typedef struct { int foo; float res; } GmlParSct;\n");

   /* ---------------- header ---------------- */
   emit(&o, "// KERNEL HEADER\nextern \"C\" __global__ void %s(", PrcNam);

   for(i=0;i<NmbArg;i++)
   {
      const GmlArgSct *a = &ArgTab[i];
      const char *cq = is_read_only(a) ? "const " : "";
      const char *rq = is_read_only(a) ? "__restrict__ " : "";
      if(a->NmbItm <= 1)
         emit(&o, "\n   %s%s *%s%sTab,", cq, GmlOclTypStr[ a->ItmTyp ], rq, a->nam);
      else
         emit(&o, "\n   %s%s (*%s%sTab)[%d],", cq, GmlOclTypStr[ a->ItmTyp ], rq, a->nam, a->NmbItm);
   }
   emit(&o, "\n   GmlParSct *GmlPar,\n   const int2 count )\n{\n");

   /* ---------------- counters ---------------- */
   emit(&o, "// KERNEL COUNTERS\n");
   emit(&o, "   int cnt = get_global_id(0);\n");
   emit(&o, "   int %sIdx = cnt + count.s1;\n\n", GmlBalTypStr[ MshTyp ]);
   emit(&o, "   if(cnt >= count.s0)\n      return;\n\n");

   /* ---------------- variables ---------------- */
   emit(&o, "// KERNEL VARIABLES DEFINITION\n");

   for(i=0;i<NmbArg;i++)
   {
      const GmlArgSct *a = &ArgTab[i];
      const GmlArgSct *lnk = a->LnkIdx != -1 ? &ArgTab[ a->LnkIdx ] : NULL;
      const GmlArgSct *cpt = a->CntIdx != -1 ? &ArgTab[ a->CntIdx ] : NULL;
      const char *T = GmlOclTypStr[ a->ItmTyp ];

      if(a->FlgTab & GmlManual)
         continue;

      /* accessors are declared after the eager reads they depend on */
      if(lazy_data(a, cpt, lazy))
         continue;
      if(lazy && a->LnkDir == 1 && a->NmbItm > 1 && (a->FlgTab & GmlReadMode))
         continue;

      if(lnk && lnk->MaxDeg > 1)
      {
         if(a->NmbItm > 1)
            emit(&o, "   %s %s[%d][%d];\n", T, a->nam, lnk->MaxDeg, a->NmbItm);
         else
            emit(&o, "   %s %s[%d];\n", T, a->nam, lnk->MaxDeg);
      }
      else
      {
         if(a->NmbItm > 1)
            emit(&o, "   %s %s[%d];\n", T, a->nam, a->NmbItm);
         else
            emit(&o, "   %s %s;\n", T, a->nam);
      }

      if(cpt)
      {
         emit(&o, "   %s %sDeg;\n", GmlOclTypStr[ cpt->ItmTyp ], a->nam);
         emit(&o, "   %s %sNul;\n", T, a->nam);
         emit(&o, "   #define   %sDegMax %d\n", a->nam, lnk->MaxDeg);
      }
      else if(lnk && lnk->LnkDir == 0)
         emit(&o, "   %s %sNul;\n", T, a->nam);

      if(a->FlgTab & GmlVoyeurs)
         emit(&o, "   char      %s[%d];\n", a->VoyNam, a->NmbItm * a->ItmLen);
   }

   /* ---------------- reads ---------------- */
   emit(&o, "\n// KERNEL MEMORY READINGS\n");

   for(i=0;i<NmbArg;i++)
   {
      const GmlArgSct *a = &ArgTab[i];
      const GmlArgSct *lnk = a->LnkIdx != -1 ? &ArgTab[ a->LnkIdx ] : NULL;
      const GmlArgSct *cpt = a->CntIdx != -1 ? &ArgTab[ a->CntIdx ] : NULL;

      if(!(a->FlgTab & GmlReadMode) || (a->FlgTab & GmlManual))
         continue;
      if(lazy_data(a, cpt, lazy))
         continue;
      if(lazy && a->LnkDir == 1 && a->NmbItm > 1)
         continue;

      if(lazy && stream_link(ArgTab, NmbArg, i))
         /* an element table that other arguments gather through, read once
            per launch at the thread's own line: evict-first, so that it
            does not push the gathered data out of L2 */
         emit(&o, "   %s = gml_ld_cs(&%sTab[ cnt + count.s1 ]);\n", a->nam, a->nam);
      else if(lazy && !lnk && !cpt && a->LnkDir != 1 && !(a->FlgTab & GmlVoyeurs)
      && GmlOclTypSiz[ a->ItmTyp ] == 16 && (a->NmbItm == 2 || a->NmbItm == 4))
         /* the entity's own 32- or 64-byte line: 32-byte loads */
         emit(&o, "   gml_load_line(%s, %sTab[ cnt + count.s1 ]);\n", a->nam, a->nam);
      else
         for(j=0;j<a->NmbItm;j++)
            emit_eager_item(&o, a, lnk, cpt, j);
      emit(&o, "\n");
   }

   /* ---------------- lazy accessors ---------------- */
   if(lazy)
   {
      int RowDone[ GML_MAXARG ] = { 0 };
      for(i=0;i<NmbArg;i++)
      {
         const GmlArgSct *a = &ArgTab[i];
         const GmlArgSct *lnk = a->LnkIdx != -1 ? &ArgTab[ a->LnkIdx ] : NULL;
         const GmlArgSct *cpt = a->CntIdx != -1 ? &ArgTab[ a->CntIdx ] : NULL;
         const char *T = GmlOclTypStr[ a->ItmTyp ];

         if(a->FlgTab & GmlManual)
            continue;

         if(lazy_data(a, cpt, lazy))
         {
            /* uplinked datatype: degree, null value, bound and accessor */
            emit(&o, "   %s %sDeg = %s;\n", GmlOclTypStr[ cpt->ItmTyp ], a->nam, cpt->nam);
            emit(&o, "   %s %sNul = gml_zero<%s>();\n", T, a->nam, T);
            emit(&o, "   #define   %sDegMax %d\n", a->nam, lnk->MaxDeg);
            V = ensure_row(&o, ArgTab, NmbArg, a->LnkIdx, RowDone);
            if(a->NmbItm > 1)
               emit(&o, "   const gml_up<%s,%d,%d> %s = { %sTab, &%sRow, %sDeg };\n",
                    T, a->NmbItm, V, a->nam, a->nam, lnk->nam, a->nam);
            else
               emit(&o, "   const gml_up1<%s,%d> %s = { %sTab, &%sRow, %sDeg };\n",
                    T, V, a->nam, a->nam, lnk->nam, a->nam);
         }
         else if(a->LnkDir == 1 && a->NmbItm > 1 && (a->FlgTab & GmlReadMode))
         {
            /* ball row as link vectors shifted on access */
            emit(&o, "   const gml_ballink<%s> %s = { (const %s *)(%sTab + cnt) };\n", T, a->nam, T, a->nam);
            if(a->FlgTab & GmlVoyeurs)
            {
               V = ensure_row(&o, ArgTab, NmbArg, i, RowDone);
               emit(&o, "   const gml_voy<%d> %s = { &%sRow };\n", V, a->VoyNam, a->nam);
            }
         }
      }
   }

   /* ---------------- user body ---------------- */
   tmp = gml_rewrite_opencl(KrnSrc);
   emit(&o, "// USER'S KERNEL CODE\n%s\n", tmp);
   free(tmp);

   /* ---------------- writes ---------------- */
   emit(&o, "\n// KERNEL MEMORY WRITINGS\n");

   for(i=0;i<NmbArg;i++)
   {
      const GmlArgSct *a = &ArgTab[i];

      if(!(a->FlgTab & GmlWriteMode) || (a->FlgTab & GmlManual))
         continue;

      if(a->NmbItm == 1)
         emit(&o, "   %sTab[ cnt + count.s1 ] = %s;\n", a->nam, a->nam);
      else if(GmlOclTypSiz[ a->ItmTyp ] == 16 && (a->NmbItm == 2 || a->NmbItm == 4))
         /* a 32- or 64-byte line of 16-byte items: 32-byte stores */
         emit(&o, "   gml_store_line(%sTab[ cnt + count.s1 ], %s);\n", a->nam, a->nam);
      else
         for(j=0;j<a->NmbItm;j++)
            emit(&o, "   %sTab[ cnt + count.s1 ][%d] = %s[%d];\n", a->nam, j, a->nam, j);
   }

   emit(&o, "}\n");

   *res = o.buf;
   return 1;
}
