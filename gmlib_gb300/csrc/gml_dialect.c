/*
 * gml_dialect.c -- OpenCL C to CUDA C++ source rewriting for user kernels.
 *
 * User bodies, user toolkits and the parameter typedef are OpenCL C.  Three
 * constructs mean something else (or nothing) in C++ and are rewritten token
 * by token, leaving comments, strings and everything else untouched:
 *
 *   (float4)(a, b, c, d)   vector literal  -> float4(a, b, c, d)
 *   (float4){a, b, c, d}   vector literal  -> float4{a, b, c, d}
 *   (float){0.}            scalar literal  -> float{0.f}
 *   1.5, .25, 3e2          unsuffixed floating constants get an `f`, which is
 *                          what the reference's -cl-single-precision-constant
 *                          build option does (sources/gmlib3.c:2993).
 *
 * A C++ cast of a parenthesised list would silently evaluate the comma
 * operator, so the vector-literal rewrite is required for correctness, not
 * only for compilation.  Scalar casts such as (float)(x) are left alone.
 *
 * A `for` loop whose header names a `...DegMax` bound (a loop over a ball
 * or shell, whose entries past the degree read as null values) gets a
 * `#pragma unroll 4` line, unless a pragma precedes it already or it sits in
 * a preprocessor directive (continuation lines included).  With the loop unrolled the compiler issues four
 * of the ball's gathers before it uses them; one dependent load per
 * iteration held the NodeSmoothing gather to 536 us on the 128^3 cube, four
 * take it to 483 us (the reference's own gather body: 793 to 702 us).
 * Unrolling changes no result.
 *
 * gml_nvrtc_options maps the OpenCL build options a caller can pass through
 * GmlSetCompilerOptions (-D, -I, -cl-fast-relaxed-math, ...) to NVRTC ones.
 */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_internal.h"

typedef struct { char *buf; size_t len, cap; } Str;

static void put(Str *s, const char *p, size_t n)
{
   if(s->len + n + 1 > s->cap)
   {
      size_t cap = s->cap ? s->cap : 1024;
      while(cap < s->len + n + 1) cap *= 2;
      s->buf = realloc(s->buf, cap);
      s->cap = cap;
   }
   memcpy(s->buf + s->len, p, n);
   s->len += n;
   s->buf[ s->len ] = 0;
}

static int is_vec_type(const char *p, size_t n)
{
   static const char *base[] = { "char", "uchar", "short", "ushort", "int", "uint",
                                 "long", "ulong", "float", "double", NULL };
   static const char *suf[] = { "2", "3", "4", "8", "16", NULL };
   int i, j;
   for(i=0;base[i];i++)
   {
      size_t b = strlen(base[i]);
      if(n <= b || strncmp(p, base[i], b))
         continue;
      for(j=0;suf[j];j++)
         if(n - b == strlen(suf[j]) && !strncmp(p + b, suf[j], n - b))
            return 1;
   }
   return 0;
}

static int is_scalar_type(const char *p, size_t n)
{
   static const char *sc[] = { "char", "uchar", "short", "ushort", "int", "uint",
                               "long", "ulong", "float", "double", "bool", NULL };
   for(int i=0;sc[i];i++)
      if(strlen(sc[i]) == n && !strncmp(p, sc[i], n))
         return 1;
   return 0;
}

static const char *skip_ws(const char *p)
{
   for(;;)
   {
      while(*p && isspace((unsigned char)*p)) p++;
      if(p[0] == '/' && p[1] == '/') { while(*p && *p != '\n') p++; continue; }
      if(p[0] == '/' && p[1] == '*') { p += 2; while(*p && !(p[0] == '*' && p[1] == '/')) p++; if(*p) p += 2; continue; }
      return p;
   }
}

/* length of a numeric literal at p; *isflt tells if it is a floating
   constant without suffix */
static size_t number_len(const char *p, int *isflt)
{
   const char *q = p;
   int flt = 0, hex = 0;

   if(q[0] == '0' && (q[1] == 'x' || q[1] == 'X'))
   {
      hex = 1;
      q += 2;
      while(isxdigit((unsigned char)*q) || *q == '.') q++;
      if(*q == 'p' || *q == 'P') { flt = 1; q++; if(*q == '+' || *q == '-') q++; while(isdigit((unsigned char)*q)) q++; }
   }
   else
   {
      while(isdigit((unsigned char)*q)) q++;
      if(*q == '.') { flt = 1; q++; while(isdigit((unsigned char)*q)) q++; }
      if(*q == 'e' || *q == 'E')
      {
         const char *r = q + 1;
         if(*r == '+' || *r == '-') r++;
         if(isdigit((unsigned char)*r))
         {
            flt = 1;
            q = r;
            while(isdigit((unsigned char)*q)) q++;
         }
      }
   }

   /* suffixes */
   if(*q == 'f' || *q == 'F' || *q == 'h' || *q == 'H')
   {
      if(flt || !hex) { q++; flt = 0; }
   }
   else if(*q == 'l' || *q == 'L')
   {
      /* 1.0L: long double, keep as is; 10L, 10UL integers */
      q++;
      flt = 0;
   }
   while(*q == 'u' || *q == 'U' || *q == 'l' || *q == 'L') q++;

   *isflt = flt;
   return (size_t)(q - p);
}

/* p points just after the keyword `for`: does its parenthesised header
   contain an identifier ending in "DegMax"? */
static int ball_loop_header(const char *p)
{
   const char *q = skip_ws(p);
   int depth = 0;
   if(*q != '(')
      return 0;
   for(;*q;q++)
   {
      if(*q == '(')
         depth++;
      else if(*q == ')' && --depth == 0)
         return 0;
      else if(isalpha((unsigned char)*q) || *q == '_')
      {
         const char *e = q;
         while(isalnum((unsigned char)e[1]) || e[1] == '_') e++;
         if(e - q + 1 >= 6 && !strncmp(e - 5, "DegMax", 6))
            return 1;
         q = e;
      }
   }
   return 0;
}

/* the output's current line is a preprocessor directive, or the last
   non-blank line before it is a pragma */
static int pragma_context(const Str *out)
{
   const char *b = out->buf, *e = out->buf + out->len, *l = e;
   while(l > b && l[-1] != '\n') l--;
   {
      const char *t = skip_ws(l);
      if(t < e && *t == '#')
         return 1;
   }
   /* a continuation line (the line before ends with a backslash) belongs
      to a directive or to a macro definition */
   if(l > b)
   {
      const char *c = l - 1;                 /* the '\n' ending the previous line */
      while(c > b && (c[-1] == '\r' || c[-1] == ' ' || c[-1] == '\t')) c--;
      if(c > b && c[-1] == '\\')
         return 1;
   }
   /* previous non-blank lines */
   while(l > b)
   {
      const char *pe = l - 1, *ps = pe;
      while(ps > b && ps[-1] != '\n') ps--;
      {
         const char *t = ps;
         while(t < pe && (*t == ' ' || *t == '\t' || *t == '\r')) t++;
         if(t < pe)
            return *t == '#';
      }
      l = ps;
   }
   return 0;
}

char *gml_rewrite_opencl(const char *src)
{
   Str out = { NULL, 0, 0 };
   const char *p = src;

   put(&out, "", 0);
   if(!src)
      return out.buf;

   while(*p)
   {
      /* comments */
      if(p[0] == '/' && p[1] == '/')
      {
         const char *q = p;
         while(*q && *q != '\n') q++;
         put(&out, p, q - p);
         p = q;
         continue;
      }
      if(p[0] == '/' && p[1] == '*')
      {
         const char *q = p + 2;
         while(*q && !(q[0] == '*' && q[1] == '/')) q++;
         if(*q) q += 2;
         put(&out, p, q - p);
         p = q;
         continue;
      }
      /* string and character literals */
      if(*p == '"' || *p == '\'')
      {
         char d = *p;
         const char *q = p + 1;
         while(*q && *q != d) { if(*q == '\\' && q[1]) q++; q++; }
         if(*q) q++;
         put(&out, p, q - p);
         p = q;
         continue;
      }
      /* identifiers (a number inside an identifier is not a literal) */
      if(isalpha((unsigned char)*p) || *p == '_')
      {
         const char *q = p;
         while(isalnum((unsigned char)*q) || *q == '_') q++;
         if(q - p == 3 && !strncmp(p, "for", 3) && ball_loop_header(q) && !pragma_context(&out))
         {
            static const char pr[] = "\n#pragma unroll 4\n";
            put(&out, pr, sizeof(pr) - 1);
         }
         put(&out, p, q - p);
         p = q;
         continue;
      }
      /* numeric literals */
      if(isdigit((unsigned char)*p) || (*p == '.' && isdigit((unsigned char)p[1])))
      {
         int flt;
         size_t n = number_len(p, &flt);
         put(&out, p, n);
         if(flt)
            put(&out, "f", 1);
         p += n;
         continue;
      }
      /* (type)( or (type){ */
      if(*p == '(')
      {
         const char *a = skip_ws(p + 1), *b = a, *c;
         while(isalnum((unsigned char)*b) || *b == '_') b++;
         c = skip_ws(b);
         if(b > a && *c == ')')
         {
            const char *d = skip_ws(c + 1);
            int vec = is_vec_type(a, b - a), sca = is_scalar_type(a, b - a);
            if((vec && (*d == '(' || *d == '{')) || (sca && *d == '{'))
            {
               put(&out, a, b - a);
               p = d;
               continue;
            }
         }
      }
      put(&out, p, 1);
      p++;
   }

   return out.buf;
}

/* OpenCL build options -> NVRTC options */
char *gml_nvrtc_options(const char *cflags)
{
   Str out = { NULL, 0, 0 };
   char *buf, *tok, *save = NULL;

   put(&out, "", 0);
   if(!cflags || !*cflags)
      return out.buf;

   buf = strdup(cflags);
   for(tok = strtok_r(buf, " \t\n", &save); tok; tok = strtok_r(NULL, " \t\n", &save))
   {
      if(!strncmp(tok, "-D", 2) || !strncmp(tok, "-U", 2) || !strncmp(tok, "-I", 2))
      {
         put(&out, tok, strlen(tok));
         put(&out, " ", 1);
      }
      else if(!strcmp(tok, "-cl-fast-relaxed-math") || !strcmp(tok, "-cl-unsafe-math-optimizations"))
         put(&out, "--use_fast_math ", 16);
      else if(!strcmp(tok, "-cl-denorms-are-zero"))
         put(&out, "--ftz=true ", 11);
      else if(!strcmp(tok, "-cl-opt-disable"))
         put(&out, "-G ", 3);
      /* other -cl-* options (mad-enable, single-precision-constant,
         no-signed-zeros, finite-math-only, ...) are the default behaviour of
         the generated code or have no NVRTC counterpart */
   }
   free(buf);
   return out.buf;
}

/* 64-bit FNV-1a variant with a final mix, for cache keys */
uint64_t gml_hash64(const void *p, size_t n, uint64_t seed)
{
   const unsigned char *c = (const unsigned char *)p;
   uint64_t h = 0xcbf29ce484222325ULL ^ seed;
   for(size_t i=0;i<n;i++)
   {
      h ^= c[i];
      h *= 0x100000001b3ULL;
   }
   h ^= h >> 33;
   h *= 0xff51afd7ed558ccdULL;
   h ^= h >> 33;
   return h;
}
