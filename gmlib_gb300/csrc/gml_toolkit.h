/*
 * gml_toolkit.h -- device geometry toolkit available to every generated kernel.
 *
 * Same function names, argument orders and results as the reference toolkit
 * that GMlib prepends to user kernels (sources/toolkit.cl:1-342): vertices are
 * float4 with w = 0, lengths and areas use the fast_ forms, and the quality
 * formulas keep their normalisation constants, which are part of the
 * observable results (for instance CalTetVol multiplies by .166666 and
 * CalTetQal sums the b-c edge twice, toolkit.cl:130-133 and 203-222).
 * Constants are single precision, as under -cl-single-precision-constant.
 */
#ifndef GML_TOOLKIT_H
#define GML_TOOLKIT_H

#include "gml_cl.h"

/* projections and distances (toolkit.cl:32-98) */
GML_FN float4 PrjVerLin(float4 VerCrd, float4 LinCrd, float4 LinTng)
{ return LinCrd + dot(LinTng, VerCrd - LinCrd) * LinTng; }

GML_FN float4 PrjVerPla(float4 VerCrd, float4 PlaCrd, float4 PlaNrm)
{ return VerCrd + dot(PlaNrm, PlaCrd - VerCrd) * PlaNrm; }

GML_FN float DisVerLin(float4 VerCrd, float4 LinCrd, float4 LinTng)
{ return distance(VerCrd, PrjVerLin(VerCrd, LinCrd, LinTng)); }

GML_FN float DisVerPla(float4 VerCrd, float4 PlaCrd, float4 PlaNrm)
{ return dot(VerCrd - PlaCrd, PlaNrm); }

GML_FN float4 LinIntLin(float4 LinCrd1, float4 LinTng1, float4 LinCrd2, float4 LinTng2)
{
   float4 img = PrjVerLin(LinCrd2, LinCrd1, LinTng1);
   return img - (distance(img, LinCrd2) / dot(LinCrd2 - img, LinTng2)) * LinTng1;
}

GML_FN float4 LinIntPla(float4 LinCrd, float4 LinTng, float4 PlaCrd, float4 PlaNrm)
{ return LinCrd - (dot(PlaNrm, LinCrd - PlaCrd) / dot(PlaNrm, LinTng)) * LinTng; }

GML_FN void PlaIntPla(float4 PlaCrd1, float4 PlaNrm1, float4 PlaCrd2, float4 PlaNrm2,
                      float4 *LinCrd1, float4 *LinTng1)
{
   *LinTng1 = normalize(cross(PlaNrm1, PlaNrm2));
   *LinCrd1 = LinIntPla(PlaCrd2, normalize(cross(*LinTng1, PlaNrm2)), PlaCrd1, PlaNrm1);
}

/* elementary measures */
GML_FN float DisPow(float4 a, float4 b)             { return dot(a - b, a - b); }
GML_FN float CalLen(float4 a, float4 b)             { return fast_distance(a, b); }
GML_FN float CalSrf(float4 a, float4 b, float4 c)   { return fast_length(cross(c - a, b - a)); }
GML_FN float CalVol(float4 a, float4 b, float4 c, float4 d) { return dot(cross(b - a, c - a), d - a); }

GML_FN float DisVerEdg(float4 VerCrd, float4 EdgCrd1, float4 EdgCrd2, float4 EdgTng)
{
   float dis = fminf(DisPow(VerCrd, EdgCrd1), DisPow(VerCrd, EdgCrd2));
   float4 img = PrjVerLin(VerCrd, EdgCrd1, EdgTng);
   return sqrtf(fminf(dis, DisPow(VerCrd, img)));
}

GML_FN float4 GetEdgTng(float4 a, float4 b)                  { return fast_normalize(b - a); }
GML_FN float4 GetTriNrm(float4 a, float4 b, float4 c)        { return fast_normalize(cross(c - a, b - a)); }
GML_FN float4 GetQadNrm(float4 a, float4 b, float4 c, float4 d) { return fast_normalize(cross(c - a, d - b)); }
GML_FN float  CalEdgLen(float4 a, float4 b)                  { return CalLen(a, b); }
GML_FN float  CalTriSrf(float4 a, float4 b, float4 c)        { return .5f * CalSrf(a, b, c); }
GML_FN float  CalQadSrf(float4 a, float4 b, float4 c, float4 d) { return .5f * fast_length(cross(c - a, d - b)); }
GML_FN float  CalTetVol(float4 a, float4 b, float4 c, float4 d) { return .166666f * CalVol(a, b, c, d); }

GML_FN float CalPyrVol(float4 a, float4 b, float4 c, float4 d, float4 e)
{
   return .083333f * (CalVol(a,b,c,e) + CalVol(c,d,a,e) + CalVol(b,c,d,e) + CalVol(d,a,b,e));
}

GML_FN float CalPriVol(float4 a, float4 b, float4 c, float4 d, float4 e, float4 f)
{
   return .833333f * (CalVol(a,b,c,d) + CalVol(b,c,a,e) + CalVol(c,a,b,f)
                    + CalVol(d,f,e,a) + CalVol(e,d,f,b) + CalVol(f,e,d,c));
}

GML_FN float CalHexVol(float4 a, float4 b, float4 c, float4 d,
                       float4 e, float4 f, float4 g, float4 h)
{
   return .125f * (CalVol(a,b,d,e) + CalVol(b,c,a,f) + CalVol(c,d,b,g) + CalVol(d,a,c,h)
                 + CalVol(e,h,f,a) + CalVol(f,e,g,b) + CalVol(g,f,h,c) + CalVol(h,g,e,d));
}

/* element qualities (toolkit.cl:166-330) */
GML_FN float CalTriQal(float4 a, float4 b, float4 c)
{
   float ha = CalLen(b,c), hb = CalLen(c,a), hc = CalLen(a,b);
   float hmax = fmaxf(fmaxf(ha, hb), hc);
   return 3.46410f * CalSrf(a,b,c) / (hmax * (ha + hb + hc));
}

GML_FN float CalQadQal(float4 a, float4 b, float4 c, float4 d)
{
   float h1 = CalLen(a,b), h2 = CalLen(b,c), h3 = CalLen(c,d), h4 = CalLen(d,a);
   float h5 = CalLen(a,c) * .707106f, h6 = CalLen(b,d) * .707106f;
   float hmax = fmaxf(fmaxf(fmaxf(h1, h2), fmaxf(h3, h4)), fmaxf(h5, h6));
   float smin = fminf(fminf(CalSrf(a,b,c), CalSrf(b,c,d)), fminf(CalSrf(c,d,a), CalSrf(d,a,b)));
   return 4.f * smin / (hmax * (h1 + h2 + h3 + h4));
}

GML_FN float CalTetQal(float4 a, float4 b, float4 c, float4 d)
{
   /* the b-c edge is counted twice and c-d once, as in the reference */
   float h = CalLen(a,b) + CalLen(a,c) + CalLen(a,d) + CalLen(b,c) + CalLen(b,c) + CalLen(c,d);
   float s = CalSrf(a,b,c) + CalSrf(c,a,d) + CalSrf(b,c,d) + CalSrf(d,a,b);
   return 176.363f * CalVol(a,b,c,d) / (h * s);
}

GML_FN float CalPyrQal(float4 a, float4 b, float4 c, float4 d, float4 e)
{
   float h = CalLen(a,b) + CalLen(b,c) + CalLen(c,d) + CalLen(d,a)
           + CalLen(e,a) + CalLen(e,b) + CalLen(e,c) + CalLen(e,d);
   float s = CalTriSrf(e,a,b) + CalTriSrf(e,b,c) + CalTriSrf(e,c,d) + CalTriSrf(e,d,a)
           + CalQadSrf(d,c,b,a);
   float v = CalVol(a,b,c,e);
   v = fminf(v, CalVol(c,d,a,e));
   v = fminf(v, CalVol(a,b,d,e));
   v = fminf(v, CalVol(b,c,d,e));
   return 141.516f * v / (h * s);
}

GML_FN float CalPriQal(float4 a, float4 b, float4 c, float4 d, float4 e, float4 f)
{
   float h = CalLen(a,b) + CalLen(b,c) + CalLen(c,a) + CalLen(d,e) + CalLen(e,f)
           + CalLen(f,d) + CalLen(a,d) + CalLen(b,e) + CalLen(c,f);
   float s = CalTriSrf(c,b,a) + CalTriSrf(d,e,f) + CalQadSrf(d,f,c,a)
           + CalQadSrf(a,d,e,b) + CalQadSrf(e,f,c,b);
   float v = CalVol(a,b,c,d);
   v = fminf(v, CalVol(e,c,d,f)); v = fminf(v, CalVol(d,b,c,e)); v = fminf(v, CalVol(a,b,c,f));
   v = fminf(v, CalVol(a,b,f,e)); v = fminf(v, CalVol(a,e,f,d)); v = fminf(v, CalVol(d,b,f,e));
   v = fminf(v, CalVol(f,a,b,d)); v = fminf(v, CalVol(c,a,b,e)); v = fminf(v, CalVol(c,a,e,d));
   v = fminf(v, CalVol(e,c,a,f)); v = fminf(v, CalVol(b,c,d,f));
   return 98.3538f * v / (h * s);
}

GML_FN float CalHexQal(float4 a, float4 b, float4 c, float4 d,
                       float4 e, float4 f, float4 g, float4 h)
{
   float l = CalLen(d,c) + CalLen(a,b) + CalLen(e,f) + CalLen(h,g) + CalLen(d,h) + CalLen(c,g)
           + CalLen(b,f) + CalLen(a,e) + CalLen(d,a) + CalLen(h,e) + CalLen(g,f) + CalLen(c,b);
   float s = CalQadSrf(d,a,e,h) + CalQadSrf(g,f,b,c) + CalQadSrf(d,c,b,a)
           + CalQadSrf(e,f,g,h) + CalQadSrf(d,h,g,c) + CalQadSrf(b,f,e,a);
   float v = CalVol(a,b,d,e);
   v = fminf(v, CalVol(b,c,d,g)); v = fminf(v, CalVol(e,d,h,g)); v = fminf(v, CalVol(e,f,b,g));
   v = fminf(v, CalVol(e,b,d,g)); v = fminf(v, CalVol(e,f,a,h)); v = fminf(v, CalVol(h,f,c,g));
   v = fminf(v, CalVol(a,c,d,h)); v = fminf(v, CalVol(a,b,c,f)); v = fminf(v, CalVol(a,f,c,h));
   return 72.f * v / (l * s);
}

/* 4x4 row-major block times a 4-vector (toolkit.cl:332-342) */
GML_FN float4 MulMatVec(float16 a, float4 b)
{
   float4 x;
   x.s0 = a.s0 * b.s0 + a.s1 * b.s1 + a.s2 * b.s2 + a.s3 * b.s3;
   x.s1 = a.s4 * b.s0 + a.s5 * b.s1 + a.s6 * b.s2 + a.s7 * b.s3;
   x.s2 = a.s8 * b.s0 + a.s9 * b.s1 + a.sa * b.s2 + a.sb * b.s3;
   x.s3 = a.sc * b.s0 + a.sd * b.s1 + a.se * b.s2 + a.sf * b.s3;
   return x;
}

#endif
