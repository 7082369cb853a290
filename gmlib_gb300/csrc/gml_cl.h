/*
 * gml_cl.h -- OpenCL C 1.2 kernel-language layer for CUDA C++ (NVRTC, sm_103a).
 *
 * GMlib user kernels are bare OpenCL-C loop bodies (for example
 * examples/MeshQuality/compute_quality.cl and examples/NodeSmoothing/gather.cl
 * in the reference).  The code generator (gml_codegen.c) wraps such a body in a
 * CUDA kernel and compiles it with NVRTC.  This header gives the body the
 * OpenCL vocabulary it expects:
 *
 *   - vector types charN/ucharN/shortN/ushortN/intN/uintN/longN/ulongN/floatN/
 *     doubleN for N = 2,3,4,8,16 with OpenCL layout (size = alignment, 3-vectors
 *     occupy 4 slots), component names .x .y .z .w, .s0 ... .sf (and .sA ... .sF),
 *     the halves .lo/.hi and the pairs .xy/.zw;
 *   - component-wise arithmetic, bit and shift operators, vector/scalar mixing;
 *   - OpenCL built-ins used by mesh kernels: dot, cross, length, distance,
 *     normalize and their fast_ forms, mix, clamp, min/max, fmin/fmax, step,
 *     sign, select, rsqrt, native_* and half_* forms, convert_T, as_T,
 *     get_global_id ... and the address-space qualifiers.
 *
 * The vector types are named gml_vec<T,N> and bound to the OpenCL spellings by
 * macros, because NVRTC predeclares CUDA's own float4/int4 types.  Vector
 * literals `(float4)(a,b,c,d)` and `(float4){...}` are C++-incompatible; the
 * source rewriter (gml_dialect.c) turns them into `float4(a,b,c,d)` and
 * `float4{...}` before compilation, and suffixes unsuffixed floating literals
 * with `f` (the reference always builds with -cl-single-precision-constant,
 * sources/gmlib3.c:2993).
 *
 * The accessor templates at the end implement the generated gather prologues:
 * instead of materialising a per-thread array of up to 64 x NmbItm values for a
 * vertex ball (the reference declares e.g. float4 OptCrd[32][4] and fills all
 * of it, sources/gmlib3.c:2689-2697 and 2844-2879), an uplinked datatype is an
 * object whose operator[] loads exactly the entry the body asks for.
 */
#ifndef GML_CL_H
#define GML_CL_H

#if !defined(__CUDACC_RTC__) && !defined(__CUDACC__)
#error "gml_cl.h is compiled by NVRTC or nvcc only"
#endif
#define GML_ON_DEVICE 1
#define GML_FN __host__ __device__ __forceinline__

/* ------------------------------------------------------------------------- */
/* scalar types and traits                                                    */
/* ------------------------------------------------------------------------- */

typedef unsigned char  uchar;
typedef unsigned short ushort;
typedef unsigned int   uint;
typedef unsigned long  ulong;

template<class T> struct gml_is_scalar { enum { value = 0 }; };
#define GML_SCALAR(T) template<> struct gml_is_scalar<T> { enum { value = 1 }; };
GML_SCALAR(bool) GML_SCALAR(char) GML_SCALAR(signed char) GML_SCALAR(unsigned char)
GML_SCALAR(short) GML_SCALAR(unsigned short) GML_SCALAR(int) GML_SCALAR(unsigned int)
GML_SCALAR(long) GML_SCALAR(unsigned long) GML_SCALAR(long long)
GML_SCALAR(unsigned long long) GML_SCALAR(float) GML_SCALAR(double)
#undef GML_SCALAR

template<bool B, class R = void> struct gml_enable_if {};
template<class R> struct gml_enable_if<true, R> { typedef R type; };

/* ------------------------------------------------------------------------- */
/* vector types                                                               */
/* ------------------------------------------------------------------------- */

template<class T, int N> struct gml_vec;

/* number of storage slots (3-vectors are stored as 4) and byte alignment */
template<int N> struct gml_slots { enum { value = N == 3 ? 4 : N }; };

/* Flattening constructor helpers: count components of each argument and copy
   them into consecutive slots, as OpenCL vector literals do. */
template<class A> struct gml_ncomp { enum { value = 1 }; };
template<class T, int N> struct gml_ncomp< gml_vec<T,N> > { enum { value = N }; };
template<class... A> struct gml_sumcomp;
template<> struct gml_sumcomp<> { enum { value = 0 }; };
template<class A, class... R> struct gml_sumcomp<A, R...>
{ enum { value = gml_ncomp<A>::value + gml_sumcomp<R...>::value }; };

template<class T, class A> GML_FN void gml_put(T *v, int &k, const A &a) { v[k++] = (T)a; }
template<class T, class U, int M> GML_FN void gml_put(T *v, int &k, const gml_vec<U,M> &a)
{ for(int i=0;i<M;i++) v[k++] = (T)a.v[i]; }
template<class T> GML_FN void gml_fill(T *, int &) {}
template<class T, class A, class... R> GML_FN void gml_fill(T *v, int &k, const A &a, const R &... r)
{ gml_put(v, k, a); gml_fill(v, k, r...); }

#define GML_VEC_COMMON(N)                                                         \
   typedef T elem_type;                                                           \
   enum { size = N };                                                             \
   gml_vec() = default;                                                           \
   template<class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type> \
   GML_FN gml_vec(S s) { for(int i=0;i<gml_slots<N>::value;i++) v[i] = (T)s; }    \
   template<class A, class B, class... R,                                         \
            class = typename gml_enable_if<gml_sumcomp<A,B,R...>::value == N>::type> \
   GML_FN gml_vec(const A &a, const B &b, const R &... r)                         \
   { int k = 0; gml_fill(v, k, a, b, r...); for(;k<gml_slots<N>::value;k++) v[k] = (T)0; } \
   GML_FN T &operator[](int i) { return v[i]; }                                   \
   GML_FN const T &operator[](int i) const { return v[i]; }

template<class T> struct alignas(2*sizeof(T)) gml_vec<T,2>
{
   union { struct { T x, y; }; struct { T s0, s1; }; struct { T lo, hi; }; T v[2]; };
   GML_VEC_COMMON(2)
};

template<class T> struct alignas(4*sizeof(T)) gml_vec<T,3>
{
   union { struct { T x, y, z, pad_; }; struct { T s0, s1, s2, s3_; }; T v[4]; };
   GML_VEC_COMMON(3)
};

template<class T> struct alignas(4*sizeof(T)) gml_vec<T,4>
{
   union {
      struct { T x, y, z, w; };
      struct { T s0, s1, s2, s3; };
      struct { gml_vec<T,2> lo, hi; };
      struct { gml_vec<T,2> xy, zw; };
      T v[4];
   };
   GML_VEC_COMMON(4)
};

template<class T> struct alignas(8*sizeof(T) > 64 ? 64 : 8*sizeof(T)) gml_vec<T,8>
{
   union {
      struct { T s0, s1, s2, s3, s4, s5, s6, s7; };
      struct { T x, y, z, w, s4_, s5_, s6_, s7_; };
      struct { gml_vec<T,4> lo, hi; };
      T v[8];
   };
   GML_VEC_COMMON(8)
};

template<class T> struct alignas(16*sizeof(T) > 128 ? 128 : 16*sizeof(T)) gml_vec<T,16>
{
   union {
      struct { T s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; };
      struct { T x, y, z, w, s4_, s5_, s6_, s7_, s8_, s9_, sA, sB, sC, sD, sE, sF; };
      struct { gml_vec<T,8> lo, hi; };
      T v[16];
   };
   GML_VEC_COMMON(16)
};

#undef GML_VEC_COMMON

/* ------------------------------------------------------------------------- */
/* operators                                                                  */
/* ------------------------------------------------------------------------- */

#define GML_SLOTS(N) gml_slots<N>::value

#define GML_BINOP(OP)                                                                   \
template<class T, int N> GML_FN gml_vec<T,N> operator OP(const gml_vec<T,N> &a, const gml_vec<T,N> &b) \
{ gml_vec<T,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = a.v[i] OP b.v[i]; return r; } \
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type> \
GML_FN gml_vec<T,N> operator OP(const gml_vec<T,N> &a, S s)                               \
{ gml_vec<T,N> r; T t = (T)s; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = a.v[i] OP t; return r; } \
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type> \
GML_FN gml_vec<T,N> operator OP(S s, const gml_vec<T,N> &a)                               \
{ gml_vec<T,N> r; T t = (T)s; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = t OP a.v[i]; return r; } \
template<class T, int N> GML_FN gml_vec<T,N> &operator OP##=(gml_vec<T,N> &a, const gml_vec<T,N> &b) \
{ for(int i=0;i<GML_SLOTS(N);i++) a.v[i] = a.v[i] OP b.v[i]; return a; }                 \
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type> \
GML_FN gml_vec<T,N> &operator OP##=(gml_vec<T,N> &a, S s)                                \
{ T t = (T)s; for(int i=0;i<GML_SLOTS(N);i++) a.v[i] = a.v[i] OP t; return a; }

GML_BINOP(+) GML_BINOP(-) GML_BINOP(*) GML_BINOP(/)
GML_BINOP(%) GML_BINOP(&) GML_BINOP(|) GML_BINOP(^) GML_BINOP(<<) GML_BINOP(>>)
#undef GML_BINOP

template<class T, int N> GML_FN gml_vec<T,N> operator-(const gml_vec<T,N> &a)
{ gml_vec<T,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = -a.v[i]; return r; }
template<class T, int N> GML_FN gml_vec<T,N> operator+(const gml_vec<T,N> &a) { return a; }
template<class T, int N> GML_FN gml_vec<T,N> operator~(const gml_vec<T,N> &a)
{ gml_vec<T,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = ~a.v[i]; return r; }

/* ------------------------------------------------------------------------- */
/* OpenCL spellings                                                           */
/* ------------------------------------------------------------------------- */

#define GML_DECLARE_VECS(T, NAME)                                        \
   typedef gml_vec<T,2> gml_##NAME##2;  typedef gml_vec<T,3> gml_##NAME##3; \
   typedef gml_vec<T,4> gml_##NAME##4;  typedef gml_vec<T,8> gml_##NAME##8; \
   typedef gml_vec<T,16> gml_##NAME##16;

GML_DECLARE_VECS(char, char)     GML_DECLARE_VECS(uchar, uchar)
GML_DECLARE_VECS(short, short)   GML_DECLARE_VECS(ushort, ushort)
GML_DECLARE_VECS(int, int)       GML_DECLARE_VECS(uint, uint)
GML_DECLARE_VECS(long, long)     GML_DECLARE_VECS(ulong, ulong)
GML_DECLARE_VECS(float, float)   GML_DECLARE_VECS(double, double)
#undef GML_DECLARE_VECS

#define char2 gml_char2
#define char3 gml_char3
#define char4 gml_char4
#define char8 gml_char8
#define char16 gml_char16
#define uchar2 gml_uchar2
#define uchar3 gml_uchar3
#define uchar4 gml_uchar4
#define uchar8 gml_uchar8
#define uchar16 gml_uchar16
#define short2 gml_short2
#define short3 gml_short3
#define short4 gml_short4
#define short8 gml_short8
#define short16 gml_short16
#define ushort2 gml_ushort2
#define ushort3 gml_ushort3
#define ushort4 gml_ushort4
#define ushort8 gml_ushort8
#define ushort16 gml_ushort16
#define int2 gml_int2
#define int3 gml_int3
#define int4 gml_int4
#define int8 gml_int8
#define int16 gml_int16
#define uint2 gml_uint2
#define uint3 gml_uint3
#define uint4 gml_uint4
#define uint8 gml_uint8
#define uint16 gml_uint16
#define long2 gml_long2
#define long3 gml_long3
#define long4 gml_long4
#define long8 gml_long8
#define long16 gml_long16
#define ulong2 gml_ulong2
#define ulong3 gml_ulong3
#define ulong4 gml_ulong4
#define ulong8 gml_ulong8
#define ulong16 gml_ulong16
#define float2 gml_float2
#define float3 gml_float3
#define float4 gml_float4
#define float8 gml_float8
#define float16 gml_float16
#define double2 gml_double2
#define double3 gml_double3
#define double4 gml_double4
#define double8 gml_double8
#define double16 gml_double16

/* ------------------------------------------------------------------------- */
/* scalar math not provided by CUDA under the OpenCL names                    */
/* ------------------------------------------------------------------------- */

GML_FN float  gml_sqrtf(float a)  { return sqrtf(a); }
GML_FN double gml_sqrtd(double a) { return ::sqrt(a); }
GML_FN float  gml_rsqrtf(float a) { return rsqrtf(a); }
GML_FN double gml_rsqrtd(double a){ return ::rsqrt(a); }
GML_FN float  native_sqrt(float a)   { return sqrtf(a); }
GML_FN float  native_rsqrt(float a)  { return rsqrtf(a); }
GML_FN float  native_recip(float a)  { return __frcp_rn(a); }
GML_FN float  native_divide(float a, float b) { return __fdividef(a, b); }
GML_FN float  native_exp(float a)    { return __expf(a); }
GML_FN float  native_log(float a)    { return __logf(a); }
GML_FN float  native_sin(float a)    { return __sinf(a); }
GML_FN float  native_cos(float a)    { return __cosf(a); }
GML_FN float  native_powr(float a, float b) { return __powf(a, b); }
GML_FN float  half_sqrt(float a)   { return native_sqrt(a); }
GML_FN float  half_rsqrt(float a)  { return native_rsqrt(a); }
GML_FN float  half_recip(float a)  { return native_recip(a); }
GML_FN float  half_divide(float a, float b) { return native_divide(a, b); }
GML_FN float  mad(float a, float b, float c)    { return a * b + c; }
GML_FN double mad(double a, double b, double c) { return a * b + c; }
GML_FN float  mix(float x, float y, float a)    { return x + (y - x) * a; }
GML_FN double mix(double x, double y, double a) { return x + (y - x) * a; }
GML_FN float  clamp(float x, float lo, float hi)   { return fminf(fmaxf(x, lo), hi); }
GML_FN double clamp(double x, double lo, double hi){ return fmin(fmax(x, lo), hi); }
GML_FN int    clamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }
GML_FN float  step(float e, float x)   { return x < e ? 0.0f : 1.0f; }
GML_FN double step(double e, double x) { return x < e ? 0.0 : 1.0; }
GML_FN float  sign(float x)  { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
GML_FN double sign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }
GML_FN float  dot(float a, float b)   { return a * b; }
GML_FN double dot(double a, double b) { return a * b; }
GML_FN float  length(float a)  { return fabsf(a); }
GML_FN float  pown(float x, int n) { float r = 1.0f; int m = n < 0 ? -n : n; while(m--) r *= x; return n < 0 ? 1.0f / r : r; }
GML_FN float  as_float(int i)  { return __int_as_float(i); }
GML_FN int    as_int(float f)  { return __float_as_int(f); }
GML_FN uint   as_uint(float f) { return (uint)__float_as_int(f); }

/* ------------------------------------------------------------------------- */
/* geometric built-ins (OpenCL 1.2 section 6.12.5): all N components count   */
/* ------------------------------------------------------------------------- */

template<class T, int N> GML_FN T dot(const gml_vec<T,N> &a, const gml_vec<T,N> &b)
{ T s = a.v[0] * b.v[0]; for(int i=1;i<N;i++) s += a.v[i] * b.v[i]; return s; }

template<class T> GML_FN gml_vec<T,4> cross(const gml_vec<T,4> &a, const gml_vec<T,4> &b)
{
   gml_vec<T,4> r;
   r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
   r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
   r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
   r.v[3] = (T)0;
   return r;
}
template<class T> GML_FN gml_vec<T,3> cross(const gml_vec<T,3> &a, const gml_vec<T,3> &b)
{
   gml_vec<T,3> r;
   r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
   r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
   r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
   r.v[3] = (T)0;
   return r;
}

template<int N> GML_FN float  length(const gml_vec<float,N> &a)  { return gml_sqrtf(dot(a, a)); }
template<int N> GML_FN double length(const gml_vec<double,N> &a) { return gml_sqrtd(dot(a, a)); }
template<int N> GML_FN float  fast_length(const gml_vec<float,N> &a) { return native_sqrt(dot(a, a)); }
template<class T, int N> GML_FN T distance(const gml_vec<T,N> &a, const gml_vec<T,N> &b) { return length(a - b); }
template<int N> GML_FN float fast_distance(const gml_vec<float,N> &a, const gml_vec<float,N> &b) { return fast_length(a - b); }
template<int N> GML_FN gml_vec<float,N> normalize(const gml_vec<float,N> &a)
{ float d = dot(a, a); return d > 0.0f ? a * gml_rsqrtf(d) : a; }
template<int N> GML_FN gml_vec<double,N> normalize(const gml_vec<double,N> &a)
{ double d = dot(a, a); return d > 0.0 ? a * gml_rsqrtd(d) : a; }
template<int N> GML_FN gml_vec<float,N> fast_normalize(const gml_vec<float,N> &a)
{ float d = dot(a, a); return d > 0.0f ? a * native_rsqrt(d) : a; }

/* ------------------------------------------------------------------------- */
/* component-wise math                                                        */
/* ------------------------------------------------------------------------- */

#define GML_MAP1(NAME, FF, FD)                                                        \
template<int N> GML_FN gml_vec<float,N> NAME(const gml_vec<float,N> &a)                 \
{ gml_vec<float,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = FF(a.v[i]); return r; }  \
template<int N> GML_FN gml_vec<double,N> NAME(const gml_vec<double,N> &a)               \
{ gml_vec<double,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = FD(a.v[i]); return r; }

GML_MAP1(sqrt, gml_sqrtf, gml_sqrtd)      GML_MAP1(rsqrt, gml_rsqrtf, gml_rsqrtd)
GML_MAP1(fabs, fabsf, ::fabs)             GML_MAP1(floor, floorf, ::floor)
GML_MAP1(ceil, ceilf, ::ceil)             GML_MAP1(exp, expf, ::exp)
GML_MAP1(log, logf, ::log)                GML_MAP1(sin, sinf, ::sin)
GML_MAP1(cos, cosf, ::cos)                GML_MAP1(round, roundf, ::round)
GML_MAP1(trunc, truncf, ::trunc)          GML_MAP1(sign, sign, sign)
GML_MAP1(native_sqrt, native_sqrt, gml_sqrtd) GML_MAP1(native_rsqrt, native_rsqrt, gml_rsqrtd)
GML_MAP1(half_sqrt, native_sqrt, gml_sqrtd)   GML_MAP1(native_recip, native_recip, 1.0/)
#undef GML_MAP1

#define GML_MAP2(NAME, F)                                                                 \
template<class T, int N> GML_FN gml_vec<T,N> NAME(const gml_vec<T,N> &a, const gml_vec<T,N> &b) \
{ gml_vec<T,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = F(a.v[i], b.v[i]); return r; }   \
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type> \
GML_FN gml_vec<T,N> NAME(const gml_vec<T,N> &a, S s)                                           \
{ gml_vec<T,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = F(a.v[i], (T)s); return r; }

template<class T> GML_FN T gml_min(T a, T b) { return b < a ? b : a; }
template<class T> GML_FN T gml_max(T a, T b) { return a < b ? b : a; }
template<class T> GML_FN T gml_pow(T a, T b) { return ::pow(a, b); }
GML_MAP2(min, gml_min) GML_MAP2(max, gml_max) GML_MAP2(fmin, gml_min) GML_MAP2(fmax, gml_max)
GML_MAP2(pow, gml_pow) GML_MAP2(step, step)
#undef GML_MAP2

template<class T, int N> GML_FN gml_vec<T,N> mix(const gml_vec<T,N> &x, const gml_vec<T,N> &y, const gml_vec<T,N> &a)
{ return x + (y - x) * a; }
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type>
GML_FN gml_vec<T,N> mix(const gml_vec<T,N> &x, const gml_vec<T,N> &y, S a)
{ return x + (y - x) * (T)a; }
template<class T, int N, class S, class = typename gml_enable_if<gml_is_scalar<S>::value>::type>
GML_FN gml_vec<T,N> clamp(const gml_vec<T,N> &x, S lo, S hi)
{ return min(max(x, (T)lo), (T)hi); }
template<class T, int N> GML_FN gml_vec<T,N> clamp(const gml_vec<T,N> &x, const gml_vec<T,N> &lo, const gml_vec<T,N> &hi)
{ return min(max(x, lo), hi); }
template<class T, int N> GML_FN gml_vec<T,N> mad(const gml_vec<T,N> &a, const gml_vec<T,N> &b, const gml_vec<T,N> &c)
{ return a * b + c; }

/* conversions: convert_floatN(x), convert_intN(x), ... */
template<class D, class T, int N> GML_FN gml_vec<D,N> gml_convert(const gml_vec<T,N> &a)
{ gml_vec<D,N> r; for(int i=0;i<GML_SLOTS(N);i++) r.v[i] = (D)a.v[i]; return r; }
#define GML_CONV(NAME, D) \
   template<class T, int N> GML_FN gml_vec<D,N> NAME(const gml_vec<T,N> &a) { return gml_convert<D>(a); } \
   template<class T> GML_FN D NAME##_s(T a) { return (D)a; }
GML_CONV(gml_convert_float, float) GML_CONV(gml_convert_double, double)
GML_CONV(gml_convert_int, int)     GML_CONV(gml_convert_uint, uint)
GML_CONV(gml_convert_char, char)   GML_CONV(gml_convert_uchar, uchar)
GML_CONV(gml_convert_long, long)
#undef GML_CONV
#define convert_float(x)  ((float)(x))
#define convert_double(x) ((double)(x))
#define convert_int(x)    ((int)(x))
#define convert_uint(x)   ((uint)(x))
#define convert_float2  gml_convert_float
#define convert_float3  gml_convert_float
#define convert_float4  gml_convert_float
#define convert_float8  gml_convert_float
#define convert_float16 gml_convert_float
#define convert_double2  gml_convert_double
#define convert_double3  gml_convert_double
#define convert_double4  gml_convert_double
#define convert_double8  gml_convert_double
#define convert_double16 gml_convert_double
#define convert_int2  gml_convert_int
#define convert_int3  gml_convert_int
#define convert_int4  gml_convert_int
#define convert_int8  gml_convert_int
#define convert_int16 gml_convert_int
#define convert_char4 gml_convert_char
#define convert_uchar4 gml_convert_uchar

/* ------------------------------------------------------------------------- */
/* work-item functions, qualifiers and constants                              */
/* ------------------------------------------------------------------------- */

__device__ __forceinline__ size_t get_global_id(int d)
{ return d == 0 ? (size_t)blockIdx.x * blockDim.x + threadIdx.x : d == 1 ? (size_t)blockIdx.y * blockDim.y + threadIdx.y : (size_t)blockIdx.z * blockDim.z + threadIdx.z; }
__device__ __forceinline__ size_t get_local_id(int d)   { return d == 0 ? threadIdx.x : d == 1 ? threadIdx.y : threadIdx.z; }
__device__ __forceinline__ size_t get_group_id(int d)   { return d == 0 ? blockIdx.x : d == 1 ? blockIdx.y : blockIdx.z; }
__device__ __forceinline__ size_t get_local_size(int d) { return d == 0 ? blockDim.x : d == 1 ? blockDim.y : blockDim.z; }
__device__ __forceinline__ size_t get_num_groups(int d) { return d == 0 ? gridDim.x : d == 1 ? gridDim.y : gridDim.z; }
__device__ __forceinline__ size_t get_global_size(int d){ return get_num_groups(d) * get_local_size(d); }
#define CLK_LOCAL_MEM_FENCE  1
#define CLK_GLOBAL_MEM_FENCE 2
#define barrier(f) __syncthreads()
#define mem_fence(f) __threadfence()
#define atomic_add(p, v)  atomicAdd((p), (v))
#define atomic_sub(p, v)  atomicSub((p), (v))
#define atomic_inc(p)     atomicAdd((p), 1)
#define atomic_dec(p)     atomicSub((p), 1)
#define atomic_min(p, v)  atomicMin((p), (v))
#define atomic_max(p, v)  atomicMax((p), (v))
#define atomic_xchg(p, v) atomicExch((p), (v))
#define atomic_cmpxchg(p, c, v) atomicCAS((p), (c), (v))
#define atom_add  atomic_add
#define atom_inc  atomic_inc
#define atom_min  atomic_min
#define atom_max  atomic_max
#define __local    __shared__

#define __global
#define __constant const
#define __private
#define __kernel
#define __read_only
#define __write_only

#ifndef M_PI_F
#define M_PI_F 3.14159265358979323846f
#endif
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef MAXFLOAT
#define MAXFLOAT 3.402823466e+38f
#endif
#ifndef FLT_MAX
#define FLT_MAX 3.402823466e+38f
#endif
#ifndef FLT_MIN
#define FLT_MIN 1.175494351e-38f
#endif
#ifndef FLT_EPSILON
#define FLT_EPSILON 1.192092896e-07f
#endif
#ifndef DBL_MAX
#define DBL_MAX 1.7976931348623158e+308
#endif
#ifndef INT_MAX
#define INT_MAX 2147483647
#endif

/* ------------------------------------------------------------------------- */
/* lazy gather accessors used by generated prologues                          */
/* ------------------------------------------------------------------------- */

/* One ball entry k of an uplinked datatype with NI items per line:
   X[k][j] is XTab[ball_k][j] when k < deg, else the null value. */
template<class T> GML_FN T gml_zero() { T z; z = (T)0; return z; }

/* Evict-first load (ld.global.cs) of a 4- or 16-byte item: the ball rows
   are read once per launch, and with plain loads they pushed the uplinked
   lines, which each line's other readers still need, out of L2 (NodeSmoothing
   gather on the 128^3 cube: 608 -> 527 us).  Gathered data keep the default
   policy: loading them at L2 only (ld.global.cg) measured no faster. */
template<class T> GML_FN T gml_ld_cs(const T *p)
{
#if defined(__CUDA_ARCH__)
   if(sizeof(T) == 16)
   {
      unsigned u[4];
      asm("ld.global.cs.v4.u32 {%0,%1,%2,%3}, [%4];"
          : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]) : "l"(p));
      T r;
      unsigned *d = (unsigned *)&r;
      d[0] = u[0]; d[1] = u[1]; d[2] = u[2]; d[3] = u[3];
      return r;
   }
   if(sizeof(T) == 4)
   {
      unsigned u;
      asm("ld.global.cs.u32 %0, [%1];" : "=r"(u) : "l"(p));
      T r;
      *(unsigned *)&r = u;
      return r;
   }
   if(sizeof(T) == 8)
   {
      unsigned u[2];
      asm("ld.global.cs.v2.u32 {%0,%1}, [%2];" : "=r"(u[0]), "=r"(u[1]) : "l"(p));
      T r;
      memcpy(&r, u, 8);
      return r;
   }
#if __CUDA_ARCH__ >= 1000
   if(sizeof(T) == 32)
   {
      unsigned u[8];
      asm("ld.global.cs.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
          : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]),
            "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]) : "l"(p));
      T r;
      memcpy(&r, u, 32);
      return r;
   }
#endif
#endif
   return *p;
}

/* Write a line of NI 16-byte items (NI = 2 or 4) with 32-byte stores
   (st.global.v8.b32): one full sector per store, where 16-byte stores from
   the lanes of a warp, a line apart, each wrote half sectors.  The values
   written are the items' bytes unchanged.  Lines that are not 32-byte
   aligned are written item by item. */
template<class T, int NI> GML_FN void gml_store_line(T (&dst)[NI], const T (&v)[NI])
{
   static_assert(sizeof(T) == 16 && (NI == 2 || NI == 4), "16-byte items, 2 or 4 per line");
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
   if((((unsigned long long)(&dst[0])) & 31) == 0)
   {
#pragma unroll
      for(int h=0;h<NI;h+=2)
      {
         uint4 a, b;
         memcpy(&a, &v[h], 16);
         memcpy(&b, &v[h + 1], 16);
         asm volatile("st.global.v8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                      :: "l"(&dst[h]), "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w),
                         "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w) : "memory");
      }
      return;
   }
#endif
#pragma unroll
   for(int j=0;j<NI;j++)
      dst[j] = v[j];
}

/* Read a line of NI 16-byte items (NI = 2 or 4) with 32-byte loads
   (ld.global.v8.b32), the counterpart of gml_store_line. */
template<class T, int NI> GML_FN void gml_load_line(T (&v)[NI], const T (&src)[NI])
{
   static_assert(sizeof(T) == 16 && (NI == 2 || NI == 4), "16-byte items, 2 or 4 per line");
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
   if((((unsigned long long)(&src[0])) & 31) == 0)
   {
#pragma unroll
      for(int h=0;h<NI;h+=2)
      {
         uint4 a, b;
         asm volatile("ld.global.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                      : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w),
                        "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w) : "l"(&src[h]));
         memcpy(&v[h], &a, 16);
         memcpy(&v[h + 1], &b, 16);
      }
      return;
   }
#endif
#pragma unroll
   for(int j=0;j<NI;j++)
      v[j] = src[j];
}

template<class T, int NI> struct gml_up_row
{
   const T *p;
   int ok;
   GML_FN const T operator[](int j) const { return ok ? p[j] : gml_zero<T>(); }
};

/* The ball row of the current entity: its codes (element << 4) | local
   index, read through the row object shared by the entity's accessors.
   With V = 4 the row is read in 16-byte pieces, kept in registers while a
   loop walks through them: one load serves four consecutive codes, where
   one load per code and per accessor touched the same 128-byte line of
   every lane's row again and again.  Codes at or beyond the degree are the
   table's zero padding and are returned without a load.  V = 1 reads one
   code at a time (rows whose width is not a multiple of four codes). */
template<int V> struct gml_balrow;

struct __align__(16) gml_codes4 { int a, b, c, d; };

template<> struct gml_balrow<4>
{
   const int *row;
   int deg;
   int q;               /* index of the piece held in c, -1 for none */
   gml_codes4 c;
   GML_FN int code(int k)
   {
      if(k >= deg)
         return 0;
      const int p = k >> 2;
      if(p != q)
      {
         c = gml_ld_cs((const gml_codes4 *)(row + 4 * p));
         q = p;
      }
      const int e = k & 3;
      return e == 0 ? c.a : e == 1 ? c.b : e == 2 ? c.c : c.d;
   }
};

template<> struct gml_balrow<1>
{
   const int *row;
   int deg;
   GML_FN int code(int k) { return k < deg ? gml_ld_cs(row + k) : 0; }
};

/* Uplinked datatype with NI items per line: X[k][j] is XTab[ball_k][j]
   when k < deg, else the null value. */
template<class T, int NI, int V> struct gml_up
{
   const T (*tab)[NI];
   gml_balrow<V> *row;
   int deg;
   GML_FN gml_up_row<T,NI> operator[](int k) const
   {
      gml_up_row<T,NI> r;
      r.ok = k < deg;
      r.p = tab[r.ok ? (row->code(k) >> 4) : 0];
      return r;
   }
};

/* Uplinked datatype with one item per line: X[k] is XTab[ball_k] or null. */
template<class T, int V> struct gml_up1
{
   const T *tab;
   gml_balrow<V> *row;
   int deg;
   GML_FN const T operator[](int k) const
   {
      return k < deg ? tab[row->code(k) >> 4] : gml_zero<T>();
   }
};

/* Voyeurs: local index (0..7) of the looping entity inside ball element k
   (0 beyond the degree, the value of the table's padding). */
template<int V> struct gml_voy
{
   gml_balrow<V> *row;
   GML_FN char operator[](int k) const { return (char)(row->code(k) & 7); }
};

/* Ball link vector j of the current row, already shifted right by 4. */
template<class V> struct gml_ballink
{
   const V *row;
   GML_FN const V operator[](int j) const { return row[j] >> 4; }
};

#endif
