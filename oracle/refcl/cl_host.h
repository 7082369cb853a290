/*
 * cl_host.h -- minimal OpenCL C vocabulary for compiling the reference's
 * kernel bodies as host C++ (oracle/refcl/refcl.cpp).  Test infrastructure,
 * written independently of the library's device header so that a mistake in
 * one is caught by the other.  Only what sources/toolkit.cl and the example
 * kernels use is provided.
 */
#ifndef CL_HOST_H
#define CL_HOST_H

#include <cmath>

struct float4
{
   union { struct { float x, y, z, w; }; struct { float s0, s1, s2, s3; }; float v[4]; };
   float4() : x(0), y(0), z(0), w(0) {}
   float4(double s) : x((float)s), y((float)s), z((float)s), w((float)s) {}
   float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
};

struct float16
{
   union {
      struct { float s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; };
      float v[16];
   };
};

inline float4 operator+(float4 a, float4 b) { return float4(a.x+b.x, a.y+b.y, a.z+b.z, a.w+b.w); }
inline float4 operator-(float4 a, float4 b) { return float4(a.x-b.x, a.y-b.y, a.z-b.z, a.w-b.w); }
inline float4 operator*(float4 a, float4 b) { return float4(a.x*b.x, a.y*b.y, a.z*b.z, a.w*b.w); }
inline float4 operator*(float4 a, float s)  { return float4(a.x*s, a.y*s, a.z*s, a.w*s); }
inline float4 operator*(float s, float4 a)  { return float4(a.x*s, a.y*s, a.z*s, a.w*s); }
inline float4 operator/(float4 a, float s)  { return float4(a.x/s, a.y/s, a.z/s, a.w/s); }
inline float4 &operator+=(float4 &a, float4 b) { a = a + b; return a; }
inline float4 &operator*=(float4 &a, float4 b) { a = a * b; return a; }

inline float dot(float4 a, float4 b) { return a.x*b.x + a.y*b.y + a.z*b.z + a.w*b.w; }
inline float4 cross(float4 a, float4 b)
{ return float4(a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x, 0.f); }
inline float length(float4 a)        { return std::sqrt(dot(a, a)); }
inline float fast_length(float4 a)   { return std::sqrt(dot(a, a)); }
inline float distance(float4 a, float4 b)      { return length(a - b); }
inline float fast_distance(float4 a, float4 b) { return length(a - b); }
inline float4 normalize(float4 a)      { float l = length(a); return l > 0 ? a / l : a; }
inline float4 fast_normalize(float4 a) { return normalize(a); }
inline float4 mix(float4 x, float4 y, float a) { return x + (y - x) * a; }
inline float rsqrt(float a) { return 1.f / std::sqrt(a); }
using std::sqrt;
inline float min(float a, float b) { return a < b ? a : b; }
inline float max(float a, float b) { return a > b ? a : b; }

#endif
