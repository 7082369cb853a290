/*
 * refcl.cpp -- the reference's own kernel bodies run on the CPU.
 *
 * Test infrastructure.  Includes, from the reference tree (REF_ROOT), the
 * geometry toolkit (sources/toolkit.cl, found through -I) and the example kernel bodies
 * (examples/MeshQuality/compute_quality.cl, examples/NodeSmoothing/scatter.cl
 * and gather.cl, examples/P2Quality/quality.cl), and wraps each body in the gather prologue and scatter
 * epilogue that the reference's generator writes around it
 * (sources/gmlib3.c:2739-2938), one loop iteration per work-item; and a table
 * of every toolkit function on given point sets (tests/kernels/toolkit_table.cl,
 * this project's body, found through -I).  Built with
 * -fsingle-precision-constant like the reference's OpenCL build
 * (sources/gmlib3.c:2993).  Nothing from the reference is copied: the files
 * are compiled where they lie.
 */
#include "cl_host.h"

#include "toolkit.cl"

extern "C" {

/* MeshQuality: loop over tetrahedra, VerCrd[4] gathered through TetVer */
void ref_compute_quality(const float *crd, int nt, const int *tet, float *out)
{
   #pragma omp parallel for schedule(static)
   for(int cnt=0;cnt<nt;cnt++)
   {
      float4 VerCrd[4];
      float qal;
      for(int k=0;k<4;k++)
      {
         const float *c = &crd[ 4 * tet[ 4*cnt + k ] ];
         VerCrd[k] = float4(c[0], c[1], c[2], c[3]);
      }
      {
#include "MeshQuality/compute_quality.cl"
      }
      out[cnt] = qal;
   }
}

/* NodeSmoothing scatter: per tetrahedron, four optimal points */
void ref_scatter(const float *crd, int nt, const int *tet, float *opt)
{
   #pragma omp parallel for schedule(static)
   for(int cnt=0;cnt<nt;cnt++)
   {
      float4 VerCrd[4], OptCrd[4];
      for(int k=0;k<4;k++)
      {
         const float *c = &crd[ 4 * tet[ 4*cnt + k ] ];
         VerCrd[k] = float4(c[0], c[1], c[2], c[3]);
      }
#include "NodeSmoothing/scatter.cl"
      for(int k=0;k<4;k++)
         for(int c=0;c<4;c++)
            opt[ 16 * (size_t)cnt + 4*k + c ] = OptCrd[k].v[c];
   }
}

/* P2Quality: loop over tetrahedra, VerCrd[4] gathered through TetVer and
   MidCrd[6] through the tetrahedron -> edge downlink TetEdg (6 edge lines
   per tet in the local edge order of the edge table) */
void ref_p2_quality(const float *crd, const float *mid, int nt, const int *tet,
                    const int *tedg, float *out)
{
   #pragma omp parallel for schedule(static)
   for(int cnt=0;cnt<nt;cnt++)
   {
      float4 VerCrd[4], MidCrd[6];
      float qal;
      for(int k=0;k<4;k++)
      {
         const float *c = &crd[ 4 * (size_t)tet[ 4*(size_t)cnt + k ] ];
         VerCrd[k] = float4(c[0], c[1], c[2], c[3]);
      }
      for(int k=0;k<6;k++)
      {
         const float *c = &mid[ 4 * (size_t)tedg[ 6*(size_t)cnt + k ] ];
         MidCrd[k] = float4(c[0], c[1], c[2], c[3]);
      }
      {
#include "P2Quality/quality.cl"
      }
      out[cnt] = qal;
   }
}

/* NodeSmoothing gather: per vertex, over its tetrahedron ball (codes
   (tet << 4) | local index, `width` entries per row), with voyeurs.  The
   prologue fills OptCrd[k][j] for every k < OptCrdDegMax as the reference's
   generated code does (:2844-2879). */
void ref_gather(float *crd, int nv, const int *deg, const int *ball, int width,
                const float *opt, float *res_out)
{
   #pragma omp parallel for schedule(static)
   for(int cnt=0;cnt<nv;cnt++)
   {
#define OptCrdDegMax 64
      float4 OptCrd[ OptCrdDegMax ][4], OptCrdNul(0.f), VerCrd;
      char VerTetVoy[ OptCrdDegMax ];
      int OptCrdDeg = deg[cnt];
      float res;
      for(int k=0;k<OptCrdDegMax;k++)
      {
         int code = k < width ? ball[ (size_t)cnt * width + k ] : 0;
         VerTetVoy[k] = (char)(code & 7);
         for(int j=0;j<4;j++)
         {
            const float *p = &opt[ 16 * (size_t)(code >> 4) + 4*j ];
            OptCrd[k][j] = (OptCrdDeg >= k + 1) ? float4(p[0], p[1], p[2], p[3]) : OptCrdNul;
         }
      }
      {
         const float *c = &crd[ 4 * (size_t)cnt ];
         VerCrd = float4(c[0], c[1], c[2], c[3]);
      }
#include "NodeSmoothing/gather.cl"
      res_out[cnt] = res;
      for(int c=0;c<4;c++)
         crd[ 4 * (size_t)cnt + c ] = VerCrd.v[c];
#undef OptCrdDegMax
   }
}

/* every toolkit function on n point sets of 8 float4 (tests/kernels/
   toolkit_table.cl), 64 results per set */
void ref_toolkit_table(const float *pts, int n, float *res)
{
   #pragma omp parallel for schedule(static)
   for(int cnt=0;cnt<n;cnt++)
   {
      float4 Pts[8];
      float Res[64];
      for(int k=0;k<8;k++)
      {
         const float *c = &pts[ 32 * (size_t)cnt + 4 * k ];
         Pts[k] = float4(c[0], c[1], c[2], c[3]);
      }
#include "toolkit_table.cl"
      for(int k=0;k<64;k++)
         res[ 64 * (size_t)cnt + k ] = Res[k];
   }
}

}
