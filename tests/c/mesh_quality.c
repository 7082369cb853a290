/*
 * mesh_quality.c -- a C99 client of gmlib3.h written the way the reference's
 * MeshQuality example drives the library: vertices and tetrahedra set line by
 * line with the variadic GmlSetDataLine, a kernel compiled with the variadic
 * GmlCompileKernel, launched, reduced with GmlReduceVector and read back with
 * GmlGetDataLine.  The mesh is a jittered cube from the extension header.
 *
 * usage: mesh_quality n split out.bin
 * prints: "sum min" ; writes the per-tet quality (float) to out.bin
 */
#include <stdio.h>
#include <stdlib.h>
#include <gmlib3.h>
#include <gmlib3_gb300.h>

static char *params =
   "typedef struct {\n"
   "   int   foo;\n"
   "   float res;\n"
   "}GmlParSct;\n";

static char *quality =
   "   float len, area, vol;\n"
   "   float4 e01 = VerCrd[0] - VerCrd[1], e02 = VerCrd[0] - VerCrd[2];\n"
   "   float4 e03 = VerCrd[0] - VerCrd[3], e12 = VerCrd[1] - VerCrd[2];\n"
   "   float4 e13 = VerCrd[1] - VerCrd[3], e23 = VerCrd[2] - VerCrd[3];\n"
   "   len = max(max(max(dot(e01,e01), dot(e02,e02)), max(dot(e03,e03), dot(e12,e12))),\n"
   "             max(dot(e13,e13), dot(e23,e23)));\n"
   "   area = CalTriSrf(VerCrd[0], VerCrd[1], VerCrd[2]) + CalTriSrf(VerCrd[0], VerCrd[1], VerCrd[3]);\n"
   "   vol = CalTetVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]);\n"
   "   qal = 7.348469 * vol / (area * sqrt(len));\n";

typedef struct { int foo; float res; } GmlParSct;

int main(int argc, char **argv)
{
   int n, split, nv, nt, i, VerIdx, TetIdx, QalIdx, krn, res;
   float *crd, *q;
   int *tet, *ref;
   size_t GmlIdx;
   double sum, mn;
   FILE *f;

   if(argc != 4)
      return 2;
   n = atoi(argv[1]);
   split = atoi(argv[2]);

   GmlxCubeSizes(n, &nv, &nt);
   crd = malloc((size_t)nv * 4 * sizeof(float));
   tet = malloc((size_t)nt * 4 * sizeof(int));
   ref = malloc((size_t)nv * sizeof(int));
   q   = malloc((size_t)nt * sizeof(float));
   GmlxCubeMesh(n, split, 0.25, 12345, crd, tet, ref);
   GmlxHilbertRenumber(nv, crd, ref, nt, tet, NULL);

   if(!(GmlIdx = GmlInit(0)))
      return 1;

   if(!GmlNewParameters(GmlIdx, sizeof(GmlParSct), params))
      return 1;

   VerIdx = GmlNewMeshData(GmlIdx, GmlVertices, nv);
   TetIdx = GmlNewMeshData(GmlIdx, GmlTetrahedra, nt);

   for(i=0;i<nv;i++)
      GmlSetDataLine(GmlIdx, VerIdx, i, (double)crd[4*i], (double)crd[4*i+1],
                     (double)crd[4*i+2], ref[i]);
   for(i=0;i<nt;i++)
      GmlSetDataLine(GmlIdx, TetIdx, i, tet[4*i], tet[4*i+1], tet[4*i+2], tet[4*i+3], 0);

   if(!(QalIdx = GmlNewSolutionData(GmlIdx, GmlTetrahedra, 1, GmlFlt, "qal")))
      return 1;

   krn = GmlCompileKernel(GmlIdx, quality, "quality", GmlTetrahedra, 2,
                          VerIdx, GmlReadMode,  NULL,
                          QalIdx, GmlWriteMode, NULL);
   if(!krn)
      return 1;

   if((res = GmlLaunchKernel(GmlIdx, krn)) < 0)
   {
      printf("launch failed %d\n", res);
      return 1;
   }

   if(GmlReduceVector(GmlIdx, QalIdx, GmlSum, &sum) < 0
   || GmlReduceVector(GmlIdx, QalIdx, GmlMin, &mn) < 0)
      return 1;

   for(i=0;i<nt;i++)
      GmlGetDataLine(GmlIdx, QalIdx, i, &q[i]);

   printf("%.17g %.17g\n", sum, mn);

   if(!(f = fopen(argv[3], "wb")))
      return 1;
   fwrite(q, sizeof(float), nt, f);
   fclose(f);

   GmlFreeData(GmlIdx, VerIdx);
   GmlFreeData(GmlIdx, TetIdx);
   GmlFreeData(GmlIdx, QalIdx);
   GmlStop(GmlIdx);
   return 0;
}
