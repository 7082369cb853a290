/*
 * gml_native.h -- state of the native mesh kernels shared by gml_native.c
 * (one mesh per instance) and gml_batch.c (many meshes packed in the
 * instance's mesh).
 */
#ifndef GML_NATIVE_H
#define GML_NATIVE_H

#include "gml_internal.h"
#include "gmlib3_gb300.h"
#include "gml_mesh.h"

#define GML_MAXSTATS 64

typedef struct
{
   int         nv, nt, fix, ready;
   int         nrow;                  /* rows of the SELL layout (a multiple of 256) */
   int         window;                /* rows sorted by ball size together (32..256) */
   int         wreq;                  /* window asked for by GmlxSetBallWindow, 0: auto */
   int         *ptr, *vt, *tmp, *err, *fixed, *pdeg, *pcol;
   unsigned    *rowv;
   long long   *width, *soff;
   long long   used, stored;
   int         maxdeg;
   void        *crd2;                 /* second coordinate buffer */
   unsigned    *flags;                /* inverted-element bits */
   GmlxQualStats *stats;              /* device, GML_MAXSTATS entries */
   int         nstats;
   void        *graph;                /* smoothing workload graph */
   int         gsweeps;
   float       gomega;
   double      gh;
   void        *gver, *gtet;          /* buffers the graph was captured on */
   void        *evL[GML_MAXSTATS + 1], *evQ[GML_MAXSTATS + 1];   /* graph ordering */
   int         NmbLoopKrn, NmbSweepKrn, NmbQalKrn;
}NatSct;

NatSct *gmlx_nat(GmlSct *gml);
void    gmlx_decode_stats(const GmlxQualStats *s, GmlxQuality *r);
float   gmlx_det_threshold(double h);
void    gmlx_batch_release(GmlSct *gml);

#endif
