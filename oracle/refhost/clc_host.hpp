/*
 * clc_host.hpp -- the OpenCL C vocabulary as host C++, so that the kernels
 * the reference host library generates and builds at run time (and its
 * library kernels: reduce.cl, multmatvec.cl, addvec.cl, scalevec.cl,
 * normvec.cl, multdiagmatvec.cl, toolkit.cl) compile with g++ and run on the
 * CPU.  Test infrastructure, used only by oracle/refhost/mockcl.cpp, which
 * prepends this header to each program it is asked to build.
 *
 * Work-items: a launch sets `clc_cur` (per OS thread) before each work-item;
 * barrier() hands control back to the launcher, which runs the other
 * work-items of the group up to the same barrier (one fiber per work-item).
 * __local arrays become static storage, shared by the work-items of a group,
 * because a group with barriers runs on one OS thread.
 */
#ifndef GML_CLC_HOST_HPP
#define GML_CLC_HOST_HPP

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <type_traits>
#include <utility>

/* ---- address spaces and qualifiers -------------------------------------- */
#define __kernel
#define __global
#define __constant const
#define __private
#define __local static
#define CLK_LOCAL_MEM_FENCE  1
#define CLK_GLOBAL_MEM_FENCE 2

typedef unsigned char  uchar;
typedef unsigned short ushort;
typedef unsigned int   uint;
typedef unsigned long  ulong;

/* ---- work-item state ----------------------------------------------------- */
struct clc_wi
{
   size_t gid, lid, grp, lsz, gsz, ngrp;
   void (*yield)(clc_wi *);       /* barrier: back to the group scheduler */
};

static thread_local clc_wi *clc_cur;

static inline size_t get_global_id(int)   { return clc_cur->gid; }
static inline size_t get_local_id(int)    { return clc_cur->lid; }
static inline size_t get_group_id(int)    { return clc_cur->grp; }
static inline size_t get_local_size(int)  { return clc_cur->lsz; }
static inline size_t get_global_size(int) { return clc_cur->gsz; }
static inline size_t get_num_groups(int)  { return clc_cur->ngrp; }
static inline void barrier(int)
{
   clc_wi *me = clc_cur;
   if(me->yield)
      me->yield(me);
   clc_cur = me;
}

/* ---- vector types --------------------------------------------------------- */
template<class V> struct clc_vt { static const bool ok = false; };

#define CLC_F2(T)  struct { T x, y; }; struct { T s0, s1; };
#define CLC_F4(T)  struct { T x, y, z, w; }; struct { T s0, s1, s2, s3; };
#define CLC_F8(T)  struct { T s0, s1, s2, s3, s4, s5, s6, s7; };
#define CLC_F16(T) struct { T s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf; }; \
                   struct { T S0_, S1_, S2_, S3_, S4_, S5_, S6_, S7_, S8_, S9_, sA, sB, sC, sD, sE, sF; };

#define CLC_VEC(NAME, T, N, FIELDS)                                                  \
   struct NAME                                                                       \
   {                                                                                 \
      union { T v[N]; FIELDS(T) };                                                   \
      NAME() { for(int i=0;i<N;i++) v[i] = (T)0; }                                   \
      template<class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type> \
      NAME(S s) { for(int i=0;i<N;i++) v[i] = (T)s; }                                \
      template<class A, class B, class... R>                                         \
      NAME(A a, B b, R... r) { T t[] = { (T)a, (T)b, (T)r... }; for(int i=0;i<N;i++) v[i] = t[i]; } \
      T &operator[](int i) { return v[i]; }                                          \
      const T &operator[](int i) const { return v[i]; }                              \
   };                                                                                \
   template<> struct clc_vt<NAME> { static const bool ok = true; typedef T elem; enum { n = N }; };

#define CLC_FAMILY(P, T) \
   CLC_VEC(P##2, T, 2, CLC_F2) CLC_VEC(P##4, T, 4, CLC_F4) \
   CLC_VEC(P##8, T, 8, CLC_F8) CLC_VEC(P##16, T, 16, CLC_F16)

CLC_FAMILY(char, signed char)
CLC_FAMILY(uchar, unsigned char)
CLC_FAMILY(short, short)
CLC_FAMILY(ushort, unsigned short)
CLC_FAMILY(int, int)
CLC_FAMILY(uint, unsigned int)
CLC_FAMILY(long, long)
CLC_FAMILY(ulong, unsigned long)
CLC_FAMILY(float, float)
CLC_FAMILY(double, double)

#define CLC_ISV(V) clc_vt<typename std::decay<V>::type>::ok
#define CLC_ISS(S) std::is_arithmetic<typename std::decay<S>::type>::value

#define CLC_BINOP(OP, AOP)                                                           \
   template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>              \
   V operator OP(V a, const V &b) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] AOP b.v[i]; return a; } \
   template<class V, class S, class = typename std::enable_if<CLC_ISV(V) && CLC_ISS(S)>::type> \
   V operator OP(V a, S s)                                                           \
   { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] AOP (typename clc_vt<V>::elem)s; return a; } \
   template<class S, class V, class = typename std::enable_if<CLC_ISV(V) && CLC_ISS(S)>::type, class = void> \
   V operator OP(S s, const V &b)                                                    \
   { V a(s); for(int i=0;i<clc_vt<V>::n;i++) a.v[i] AOP b.v[i]; return a; }         \
   template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>              \
   V &operator AOP(V &a, const V &b) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] AOP b.v[i]; return a; } \
   template<class V, class S, class = typename std::enable_if<CLC_ISV(V) && CLC_ISS(S)>::type> \
   V &operator AOP(V &a, S s)                                                        \
   { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] AOP (typename clc_vt<V>::elem)s; return a; }

CLC_BINOP(+, +=)
CLC_BINOP(-, -=)
CLC_BINOP(*, *=)
CLC_BINOP(/, /=)
CLC_BINOP(%, %=)
CLC_BINOP(>>, >>=)
CLC_BINOP(<<, <<=)
CLC_BINOP(&, &=)
CLC_BINOP(|, |=)
CLC_BINOP(^, ^=)

template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
V operator-(V a) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] = -a.v[i]; return a; }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
V operator+(V a) { return a; }

/* ---- math built-ins -------------------------------------------------------- */
using std::sqrt;
using std::fabs;
using std::pow;
using std::fmin;
using std::fmax;
using std::exp;
using std::log;
using std::cbrt;
using std::floor;
using std::ceil;

static inline float  rsqrt(float a)  { return 1.0f / std::sqrt(a); }
static inline double rsqrt(double a) { return 1.0 / std::sqrt(a); }

template<class A, class B, class = typename std::enable_if<CLC_ISS(A) && CLC_ISS(B)>::type>
typename std::common_type<A, B>::type min(A a, B b) { return b < a ? b : a; }
template<class A, class B, class = typename std::enable_if<CLC_ISS(A) && CLC_ISS(B)>::type>
typename std::common_type<A, B>::type max(A a, B b) { return a < b ? b : a; }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type, class = void>
V min(V a, const V &b) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] = b.v[i] < a.v[i] ? b.v[i] : a.v[i]; return a; }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type, class = void>
V max(V a, const V &b) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] = a.v[i] < b.v[i] ? b.v[i] : a.v[i]; return a; }

template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
typename clc_vt<V>::elem dot(const V &a, const V &b)
{
   typename clc_vt<V>::elem s = 0;
   for(int i=0;i<clc_vt<V>::n;i++)
      s += a.v[i] * b.v[i];
   return s;
}
static inline float  dot(float a, float b)   { return a * b; }
static inline double dot(double a, double b) { return a * b; }

template<class V, class = typename std::enable_if<CLC_ISV(V) && clc_vt<V>::n == 4>::type>
V cross(const V &a, const V &b)
{
   V r;
   r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
   r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
   r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
   r.v[3] = 0;
   return r;
}

template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
typename clc_vt<V>::elem length(const V &a) { return std::sqrt(dot(a, a)); }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
typename clc_vt<V>::elem fast_length(const V &a) { return std::sqrt(dot(a, a)); }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
typename clc_vt<V>::elem distance(const V &a, const V &b) { return length(a - b); }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
typename clc_vt<V>::elem fast_distance(const V &a, const V &b) { return length(a - b); }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
V normalize(const V &a) { typename clc_vt<V>::elem l = length(a); return l > 0 ? a / l : a; }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
V fast_normalize(const V &a) { return normalize(a); }
template<class V, class S, class = typename std::enable_if<CLC_ISV(V) && CLC_ISS(S)>::type>
V mix(const V &x, const V &y, S a) { return x + (y - x) * a; }
template<class V, class = typename std::enable_if<CLC_ISV(V)>::type>
V fabs(V a) { for(int i=0;i<clc_vt<V>::n;i++) a.v[i] = std::fabs(a.v[i]); return a; }

/* ---- calling a kernel with its arguments given as addresses of values ---- */
template<class... A, size_t... I>
static void clc_invoke_(void (*f)(A...), void **a, std::index_sequence<I...>)
{
   f(*static_cast<typename std::decay<A>::type *>(a[I])...);
}

template<class... A>
static void clc_invoke(void (*f)(A...), void **a)
{
   clc_invoke_(f, a, std::index_sequence_for<A...>{});
}

#endif
