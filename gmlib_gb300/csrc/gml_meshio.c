/*
 * gml_meshio.c -- mesh files: GmlImportMesh and GmlExportSolution of the
 * reference (sources/gmlib3.c:4480-4738, built there on libMeshb), without
 * libMeshb.
 *
 * Formats.  The Gamma mesh format in its two encodings:
 *
 *   .meshb  binary: int32 code 1 (byte order), int32 version, then keyword
 *           records: int32 keyword, the file position of the next record
 *           (int32 for versions 1-2, int64 for 3-4), and for data keywords
 *           the line count (int32, int64 for version 4) followed by the
 *           lines.  Reals are float32 in version 1 and float64 from version
 *           2; integers are int32 up to version 3 and int64 in version 4.
 *           A vertex line is `dim` reals and a reference, an element line
 *           its 1-based vertex indices and a reference.  Keyword 3 holds
 *           the dimension (one int32), keyword 54 ends the file.
 *   .mesh   ASCII: the same content with keyword names ("Dimension",
 *           "Vertices", "Tetrahedra", ...) and "End".
 *
 * Keyword codes (the libMeshb numbering the reference's callers pass to
 * GmlImportMesh): Vertices 4, Edges 5, Triangles 6, Quadrilaterals 7,
 * Tetrahedra 8, Prisms 9, Hexahedra 10, Pyramids 49.
 *
 * GmlExportSolution writes the solution format, ASCII (.sol) or binary
 * (.solb): one SolAtVertices / SolAtTetrahedra / ... keyword per mesh type,
 * the field count and a type code per field (1 scalar), one line per entity.
 * The keyword codes are libMeshb's (the library the reference links for its
 * files, absent here; the Gamma Mesh Format as libMeshb 7 numbers it).
 */
#include <ctype.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"

#define MIO_DIM   3
#define MIO_END   54

/* libMeshb keyword of each GMlib mesh type (enum element_type order) */
static const int MioKwd[ GmlMaxEleTyp ] = { 4, 5, 6, 7, 8, 49, 9, 10 };
static const char *MioName[ GmlMaxEleTyp ] = { "Vertices", "Edges", "Triangles",
   "Quadrilaterals", "Tetrahedra", "Pyramids", "Prisms", "Hexahedra" };
static const char *MioSolName[ GmlMaxEleTyp ] = { "SolAtVertices", "SolAtEdges",
   "SolAtTriangles", "SolAtQuadrilaterals", "SolAtTetrahedra", "SolAtPyramids",
   "SolAtPrisms", "SolAtHexahedra" };

static int kwd_to_type(int kwd)
{
   for(int i=0;i<GmlMaxEleTyp;i++)
      if(MioKwd[i] == kwd)
         return i;
   return -1;
}

static int ends_with(const char *s, const char *suf)
{
   size_t n = strlen(s), m = strlen(suf);
   return n >= m && !strcmp(s + n - m, suf);
}

/* ------------------------------------------------------------------------- */
/* reading                                                                    */
/* ------------------------------------------------------------------------- */

typedef struct
{
   int      nlin, dim;            /* lines; dimension for vertices */
   float    *crd;                 /* 4 floats per vertex (w = 0) */
   int      *ele;                 /* nodes per element, 0-based */
   int      *ref;
}MioBlock;

static void block_free(MioBlock *b)
{
   free(b->crd); free(b->ele); free(b->ref);
   memset(b, 0, sizeof(*b));
}

static int rd(FILE *f, void *p, size_t n)
{
   return fread(p, 1, n, f) == n;
}

static int rd_int(FILE *f, int ver, long long *v)
{
   if(ver >= 4)
   {
      int64_t x;
      if(!rd(f, &x, 8)) return 0;
      *v = x;
   }
   else
   {
      int32_t x;
      if(!rd(f, &x, 4)) return 0;
      *v = x;
   }
   return 1;
}

static int rd_real(FILE *f, int ver, double *v)
{
   if(ver == 1)
   {
      float x;
      if(!rd(f, &x, 4)) return 0;
      *v = x;
   }
   else if(!rd(f, v, 8))
      return 0;
   return 1;
}

/* binary: fill blk[type] for every requested type present in the file */
static int read_meshb(const char *name, const int *want, MioBlock *blk)
{
   FILE *f = fopen(name, "rb");
   int32_t code, ver, kwd;
   int dim = 3, ok = 1;
   if(!f)
      return 0;
   if(!rd(f, &code, 4) || !rd(f, &ver, 4) || code != 1 || ver < 1 || ver > 4)
   {
      printf("%s: not a native-endian meshb file (code %d, version %d)\n", name, code, ver);
      fclose(f);
      return 0;
   }
   for(;;)
   {
      long long next, n;
      int typ;
      if(!rd(f, &kwd, 4))
         break;
      if(ver >= 3)
      {
         int64_t p;
         if(!rd(f, &p, 8)) { ok = 0; break; }
         next = p;
      }
      else
      {
         int32_t p;
         if(!rd(f, &p, 4)) { ok = 0; break; }
         next = (uint32_t)p;
      }
      if(kwd == MIO_END || next == 0)
         break;
      if(kwd == MIO_DIM)
      {
         int32_t d;
         if(!rd(f, &d, 4)) { ok = 0; break; }
         dim = d;
      }
      else if((typ = kwd_to_type(kwd)) >= 0 && want[typ])
      {
         MioBlock *b = &blk[typ];
         const int nn = GmlEleNmbNod[typ];
         if(!rd_int(f, ver, &n) || n < 0 || n > 2147483647LL) { ok = 0; break; }
         b->nlin = (int)n;
         b->dim = dim;
         b->ref = malloc((size_t)(n ? n : 1) * sizeof(int));
         if(typ == GmlVertices)
            b->crd = calloc((size_t)(n ? n : 1) * 4, sizeof(float));
         else
            b->ele = malloc((size_t)(n ? n : 1) * nn * sizeof(int));
         if(!b->ref || (typ == GmlVertices ? !b->crd : !b->ele)) { ok = 0; break; }
         for(long long i=0;i<n && ok;i++)
         {
            long long r;
            if(typ == GmlVertices)
            {
               for(int c=0;c<dim;c++)
               {
                  double x;
                  if(!rd_real(f, ver, &x)) { ok = 0; break; }
                  if(c < 3) b->crd[4*i + c] = (float)x;
               }
            }
            else
               for(int c=0;c<nn;c++)
               {
                  long long v;
                  if(!rd_int(f, ver, &v)) { ok = 0; break; }
                  b->ele[(size_t)i * nn + c] = (int)(v - 1);
               }
            if(ok && rd_int(f, ver, &r))
               b->ref[i] = (int)r;
            else
               ok = 0;
         }
         if(!ok)
            break;
      }
      if(fseek(f, (long)next, SEEK_SET) != 0) { ok = 0; break; }
   }
   fclose(f);
   return ok;
}

static int next_token(FILE *f, char *buf, int len)
{
   int c, n = 0;
   do { c = fgetc(f); } while(c != EOF && isspace(c));
   if(c == EOF)
      return 0;
   if(c == '#')
   {
      while(c != EOF && c != '\n') c = fgetc(f);
      return next_token(f, buf, len);
   }
   while(c != EOF && !isspace(c) && n < len - 1)
   {
      buf[n++] = (char)c;
      c = fgetc(f);
   }
   buf[n] = '\0';
   return 1;
}

/* ASCII: known keywords are read (kept when requested), an unknown keyword
   ends the scan */
static int read_mesh_ascii(const char *name, const int *want, MioBlock *blk)
{
   FILE *f = fopen(name, "r");
   char tok[128];
   int dim = 3, ok = 1;
   if(!f)
      return 0;
   while(ok && next_token(f, tok, sizeof(tok)))
   {
      int typ = -1;
      if(!strcmp(tok, "End"))
         break;
      if(!strcmp(tok, "MeshVersionFormatted"))
      {
         ok = next_token(f, tok, sizeof(tok));
         continue;
      }
      if(!strcmp(tok, "Dimension"))
      {
         ok = next_token(f, tok, sizeof(tok));
         dim = atoi(tok);
         continue;
      }
      for(int i=0;i<GmlMaxEleTyp;i++)
         if(!strcmp(tok, MioName[i]))
            typ = i;
      if(typ < 0)
         break;
      {
         const int nn = typ == GmlVertices ? dim : GmlEleNmbNod[typ];
         long long n;
         MioBlock *b = &blk[typ];
         if(!next_token(f, tok, sizeof(tok)) || (n = atoll(tok)) < 0 || n > 2147483647LL)
         {
            ok = 0;
            break;
         }
         if(want[typ])
         {
            b->nlin = (int)n;
            b->dim = dim;
            b->ref = malloc((size_t)(n ? n : 1) * sizeof(int));
            if(typ == GmlVertices)
               b->crd = calloc((size_t)(n ? n : 1) * 4, sizeof(float));
            else
               b->ele = malloc((size_t)(n ? n : 1) * nn * sizeof(int));
            if(!b->ref || (typ == GmlVertices ? !b->crd : !b->ele)) { ok = 0; break; }
         }
         for(long long i=0;i<n && ok;i++)
         {
            for(int c=0;c<=nn && ok;c++)
            {
               ok = next_token(f, tok, sizeof(tok));
               if(!ok || !want[typ])
                  continue;
               if(c == nn)
                  b->ref[i] = atoi(tok);
               else if(typ == GmlVertices)
               {
                  if(c < 3) b->crd[4*i + c] = (float)atof(tok);
               }
               else
                  b->ele[(size_t)i * nn + c] = atoi(tok) - 1;
            }
         }
      }
   }
   fclose(f);
   return ok;
}

/* Read the requested keywords and create one mesh datatype per keyword
   found (vertices first, so element indices can be checked). */
static int import_mesh(size_t GmlIdx, const char *name, int NmbKwd, const int *KwdTab)
{
   MioBlock blk[ GmlMaxEleTyp ];
   int want[ GmlMaxEleTyp ] = { 0 }, ok, typ, created = 0;

   memset(blk, 0, sizeof(blk));
   for(int k=0;k<NmbKwd;k++)
      if((typ = kwd_to_type(KwdTab[k])) >= 0)
         want[typ] = 1;
   ok = ends_with(name, ".meshb") ? read_meshb(name, want, blk) : read_mesh_ascii(name, want, blk);
   if(!ok)
   {
      printf("Could not read file %s\n", name);
      fflush(stdout);
      for(typ=0;typ<GmlMaxEleTyp;typ++)
         block_free(&blk[typ]);
      return 0;
   }
   for(typ=0;typ<GmlMaxEleTyp;typ++)
   {
      MioBlock *b = &blk[typ];
      const int nn = GmlEleNmbNod[typ];
      if(!want[typ] || b->nlin < 1)
         continue;
      if(typ != GmlVertices)
      {
         const int nv = blk[GmlVertices].nlin;
         size_t i, tot = (size_t)b->nlin * nn;
         for(i=0;i<tot;i++)
            if(b->ele[i] < 0 || (nv > 0 && b->ele[i] >= nv))
               break;
         if(i < tot)
         {
            printf("%s: %s line %zu refers to vertex %d of %d\n", name, MioName[typ], i / nn + 1,
                   b->ele[i] + 1, nv);
            fflush(stdout);
            continue;
         }
      }
      if(!GmlNewMeshData(GmlIdx, typ, b->nlin))
         continue;
      if(b->nlin == 1)
      {
         /* GmlSetDataBlock needs two lines to deduce the strides */
         if(typ == GmlVertices)
            GmlSetDataLine(GmlIdx, typ, 0, (double)b->crd[0], (double)b->crd[1], (double)b->crd[2],
                           b->ref[0]);
         else
         {
            GmlSct *gml = (GmlSct *)GmlIdx;
            GmlDatSct *d = &gml->dat[ gml->TypIdx[typ] ];
            memcpy(d->CpuMem, b->ele, (size_t)nn * sizeof(int));
            ((int *)gml->dat[ gml->RefIdx[typ] ].CpuMem)[0] = b->ref[0];
            gml_upload(gml, gml->TypIdx[typ]);
            gml_upload(gml, gml->RefIdx[typ]);
         }
      }
      else if(typ == GmlVertices)
         GmlSetDataBlock(GmlIdx, typ, 0, b->nlin - 1, b->crd, b->crd + 4 * (size_t)(b->nlin - 1),
                         b->ref, b->ref + b->nlin - 1);
      else
         GmlSetDataBlock(GmlIdx, typ, 0, b->nlin - 1, b->ele, b->ele + (size_t)nn * (b->nlin - 1),
                         b->ref, b->ref + b->nlin - 1);
      created++;
   }
   for(typ=0;typ<GmlMaxEleTyp;typ++)
      block_free(&blk[typ]);
   GmlxSynchronize(GmlIdx);
   (void)created;
   return NmbKwd;
}

int GmlxImportMesh(size_t GmlIdx, const char *MshNam, int NmbKwd, const int *KwdTab)
{
   if(!MshNam || NmbKwd < 0 || (NmbKwd && !KwdTab))
      return 0;
   return import_mesh(GmlIdx, MshNam, NmbKwd, KwdTab);
}

int GmlImportMesh(size_t GmlIdx, char *MshNam, ...)
{
   int KwdTab[10], NmbKwd = 0, kwd;
   va_list VarArg;
   va_start(VarArg, MshNam);
   while((kwd = va_arg(VarArg, int)) && NmbKwd < 10)
      if(kwd_to_type(kwd) >= 0)
         KwdTab[ NmbKwd++ ] = kwd;
   va_end(VarArg);
   return import_mesh(GmlIdx, MshNam, NmbKwd, KwdTab);
}

/* ------------------------------------------------------------------------- */
/* writing                                                                    */
/* ------------------------------------------------------------------------- */

/* binary version 2: float64 reals, int32 integers and positions */
static int write_meshb(const char *name, GmlSct *gml, int NmbTyp, const int *TypTab)
{
   FILE *f = fopen(name, "wb");
   int32_t hdr[2] = { 1, 2 }, dimrec[3] = { MIO_DIM, 20, 3 }, endrec[2] = { MIO_END, 0 };
   int ok = 1;
   if(!f)
      return 0;
   ok = fwrite(hdr, 4, 2, f) == 2 && fwrite(dimrec, 4, 3, f) == 3;
   for(int k=0;k<NmbTyp && ok;k++)
   {
      const int typ = TypTab[k], di = gml->TypIdx[typ], ri = gml->RefIdx[typ];
      const int nn = GmlEleNmbNod[typ];
      GmlDatSct *d, *r;
      long pos = ftell(f);
      int32_t rec[3];
      size_t line;
      if(typ < 0 || typ >= GmlMaxEleTyp || !di)
         continue;
      d = &gml->dat[di];
      r = &gml->dat[ri];
      gml_download(gml, di);
      gml_download(gml, ri);
      line = typ == GmlVertices ? 3 * 8 + 4 : (size_t)nn * 4 + 4;
      if((double)pos + 12. + (double)line * d->NmbLin > 2147483000.)
      {
         printf("%s: more than 2 GB, beyond the 32-bit positions of this encoding\n", name);
         ok = 0;
         break;
      }
      rec[0] = MioKwd[typ];
      rec[1] = (int32_t)(pos + 12 + (long)line * d->NmbLin);
      rec[2] = d->NmbLin;
      ok = fwrite(rec, 4, 3, f) == 3;
      for(int i=0;i<d->NmbLin && ok;i++)
      {
         const int32_t ref = ((const int *)r->CpuMem)[i];
         if(typ == GmlVertices)
         {
            const float *c = (const float *)d->CpuMem + 4 * (size_t)i;
            const double x[3] = { c[0], c[1], c[2] };
            ok = fwrite(x, 8, 3, f) == 3;
         }
         else
         {
            const int *e = (const int *)d->CpuMem + (size_t)i * GmlTypVecSiz[ d->ItmTyp ];
            int32_t v[8];
            for(int c=0;c<nn;c++)
               v[c] = e[c] + 1;
            ok = fwrite(v, 4, nn, f) == (size_t)nn;
         }
         ok = ok && fwrite(&ref, 4, 1, f) == 1;
      }
      ok = ok && ftell(f) == rec[1];
   }
   ok = ok && fwrite(endrec, 4, 2, f) == 2;
   return (fclose(f) == 0) && ok;
}

static int write_mesh_ascii(const char *name, GmlSct *gml, int NmbTyp, const int *TypTab)
{
   FILE *f = fopen(name, "w");
   int ok;
   if(!f)
      return 0;
   ok = fprintf(f, "MeshVersionFormatted 2\n\nDimension 3\n") > 0;
   for(int k=0;k<NmbTyp && ok;k++)
   {
      const int typ = TypTab[k], di = gml->TypIdx[typ], ri = gml->RefIdx[typ];
      const int nn = GmlEleNmbNod[typ];
      GmlDatSct *d, *r;
      if(typ < 0 || typ >= GmlMaxEleTyp || !di)
         continue;
      d = &gml->dat[di];
      r = &gml->dat[ri];
      gml_download(gml, di);
      gml_download(gml, ri);
      fprintf(f, "\n%s\n%d\n", MioName[typ], d->NmbLin);
      for(int i=0;i<d->NmbLin;i++)
      {
         const int ref = ((const int *)r->CpuMem)[i];
         if(typ == GmlVertices)
         {
            const float *c = (const float *)d->CpuMem + 4 * (size_t)i;
            fprintf(f, "%.9g %.9g %.9g %d\n", c[0], c[1], c[2], ref);
         }
         else
         {
            const int *e = (const int *)d->CpuMem + (size_t)i * GmlTypVecSiz[ d->ItmTyp ];
            for(int c=0;c<nn;c++)
               fprintf(f, "%d ", e[c] + 1);
            fprintf(f, "%d\n", ref);
         }
      }
   }
   fprintf(f, "\nEnd\n");
   return (fclose(f) == 0) && ok;
}

int GmlxExportMesh(size_t GmlIdx, const char *MshNam, int NmbTyp, const int *TypTab)
{
   GETGMLPTR(gml, GmlIdx);
   if(!MshNam || NmbTyp < 1 || !TypTab)
      return 0;
   return ends_with(MshNam, ".meshb") ? write_meshb(MshNam, gml, NmbTyp, TypTab)
                                      : write_mesh_ascii(MshNam, gml, NmbTyp, TypTab);
}

/* libMeshb's solution keywords (SolAtVertices ... SolAtHexahedra), in the
   enum element_type order, and its scalar field type code */
static const int MioSolKwd[ GmlMaxEleTyp ] = { 62, 63, 64, 65, 66, 26, 67, 68 };
#define MIO_SCA 1

/* The float datatypes among DatTab that live on mesh type typ (at most 10,
   all with the first one's line count): their indices in sel, the scalar
   field count in *nfld, the line count returned (-1: none). */
static int solution_fields(GmlSct *gml, int typ, int NmbDat, const int *DatTab, int *sel, int *ns,
                           int *nfld)
{
   int nlin = -1;
   *ns = *nfld = 0;
   for(int k=0;k<NmbDat && *ns<10;k++)
   {
      const int di = DatTab[k];
      const GmlDatSct *d;
      if(di < 1 || di > GmlMaxDat || !gml->dat[di].use)
         continue;
      d = &gml->dat[di];
      if(d->MshTyp != typ || (d->ItmTyp != GmlFlt && d->ItmTyp != GmlFlt2 && d->ItmTyp != GmlFlt4
                              && d->ItmTyp != GmlFlt8 && d->ItmTyp != GmlFlt16))
         continue;
      if(nlin >= 0 && d->NmbLin != nlin)
         continue;
      nlin = d->NmbLin;
      sel[ (*ns)++ ] = di;
      *nfld += d->NmbItm * GmlTypVecSiz[ d->ItmTyp ];
   }
   for(int s=0;s<*ns;s++)
      gml_download(gml, sel[s]);
   return nlin;
}

/* the scalar fields of line i, in datatype then component order */
static int line_values(GmlSct *gml, const int *sel, int ns, int i, double *out)
{
   int n = 0;
   for(int s=0;s<ns;s++)
   {
      const GmlDatSct *d = &gml->dat[ sel[s] ];
      const int nv = d->NmbItm * GmlTypVecSiz[ d->ItmTyp ];
      const float *v = (const float *)((const char *)d->CpuMem + (size_t)i * d->LinSiz);
      for(int c=0;c<nv;c++)
         out[n++] = v[c];
   }
   return n;
}

/* Solution fields of the given datatypes, grouped by mesh type: each float
   component of each datatype is one scalar field of its SolAt keyword.
   Written in the ASCII encoding (.sol) or, for a .solb name, the binary one
   of libMeshb's version 3 (int32 byte-order code 1 and version, then per
   keyword: int32 code, int64 position of the next keyword, and for a SolAt
   keyword the int32 line count, the int32 field count and one int32 type
   code per field (1, scalar), then the lines as float64; Dimension 3 holds
   int32 3; End (54) closes the file).  The reference writes through libMeshb
   with the same keywords (sources/gmlib3.c:4591-4738); its ReferenceStrings
   keyword, naming the fields, is not written here. */
static int export_solution(size_t GmlIdx, const char *name, int NmbDat, const int *DatTab)
{
   GETGMLPTR(gml, GmlIdx);
   const int bin = ends_with(name, ".solb");
   FILE *f = fopen(name, bin ? "wb" : "w");
   int done = 0, ok = 1;
   double *line = NULL;

   if(!f)
   {
      printf("Could not create file %s\n", name);
      return 0;
   }
   if(bin)
   {
      const int32_t hdr[2] = { 1, 3 }, dim[2] = { MIO_DIM, 0 };
      const int64_t next = 8 + 4 + 8 + 4;
      ok = fwrite(hdr, 4, 2, f) == 2 && fwrite(dim, 4, 1, f) == 1 && fwrite(&next, 8, 1, f) == 1
        && fwrite(&(int32_t){ 3 }, 4, 1, f) == 1;
   }
   else
      fprintf(f, "MeshVersionFormatted 2\n\nDimension 3\n");

   for(int typ=0;typ<GmlMaxEleTyp && ok;typ++)
   {
      int sel[10], ns, nfld;
      const int nlin = solution_fields(gml, typ, NmbDat, DatTab, sel, &ns, &nfld);
      if(nlin < 0)
         continue;
      free(line);
      if(!(line = malloc((size_t)nfld * sizeof(double))))
      {
         ok = 0;
         break;
      }
      if(bin)
      {
         const int64_t here = ftell(f);
         const int64_t next = here + 4 + 8 + 4 + 4 + 4 * (int64_t)nfld + 8 * (int64_t)nfld * nlin;
         const int32_t kwd = MioSolKwd[typ], nl = nlin, nf = nfld;
         ok = fwrite(&kwd, 4, 1, f) == 1 && fwrite(&next, 8, 1, f) == 1 && fwrite(&nl, 4, 1, f) == 1
           && fwrite(&nf, 4, 1, f) == 1;
         for(int k=0;k<nfld && ok;k++)
            ok = fwrite(&(int32_t){ MIO_SCA }, 4, 1, f) == 1;
         for(int i=0;i<nlin && ok;i++)
            ok = fwrite(line, 8, line_values(gml, sel, ns, i, line), f) == (size_t)nfld;
         ok = ok && ftell(f) == next;
      }
      else
      {
         fprintf(f, "\n%s\n%d\n%d", MioSolName[typ], nlin, nfld);
         for(int k=0;k<nfld;k++)
            fprintf(f, " 1");
         fprintf(f, "\n");
         for(int i=0;i<nlin;i++)
         {
            const int n = line_values(gml, sel, ns, i, line);
            for(int c=0;c<n;c++)
               fprintf(f, "%.9g ", line[c]);
            fprintf(f, "\n");
         }
      }
      done++;
   }
   free(line);
   if(bin)
   {
      const int32_t end = MIO_END;
      const int64_t zero = 0;
      ok = ok && fwrite(&end, 4, 1, f) == 1 && fwrite(&zero, 8, 1, f) == 1;
   }
   else
      fprintf(f, "\nEnd\n");
   ok = (fclose(f) == 0) && ok;
   return ok ? done : 0;
}

int GmlxExportSolution(size_t GmlIdx, const char *SolNam, int NmbDat, const int *DatTab)
{
   if(!SolNam || NmbDat < 1 || !DatTab)
      return 0;
   return export_solution(GmlIdx, SolNam, NmbDat, DatTab);
}

int GmlExportSolution(size_t GmlIdx, char *SolNam, ...)
{
   int DatTab[10], NmbDat = 0, idx;
   va_list VarArg;
   va_start(VarArg, SolNam);
   while((idx = va_arg(VarArg, int)) && NmbDat < 10)
      DatTab[ NmbDat++ ] = idx;
   va_end(VarArg);
   return export_solution(GmlIdx, SolNam, NmbDat, DatTab);
}
