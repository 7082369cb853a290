/*
 * mockcl.cpp -- an OpenCL 1.2 runtime on the host CPU, written for this
 * project, that runs the reference's host library (sources/gmlib3.c, compiled
 * unmodified against oracle/refhost/CL/opencl.h) end to end.
 *
 * Test infrastructure only: it turns the reference into an executable oracle
 * for the integer tables (balls, links, edges, faces, neighbours, matrix
 * slices) and for the results of its generated and library kernels, on
 * machines with no OpenCL runtime.
 *
 *   buffers     clCreateBuffer -> calloc; writes/reads are memcpy.
 *   programs    clBuildProgram writes the program source after
 *               #include "clc_host.hpp", with one C entry per __kernel, and
 *               builds it with g++ (-fsingle-precision-constant, the
 *               -D options of the build string); the shared object is cached
 *               by a hash of source and options and loaded with dlopen.
 *   launches    clEnqueueNDRangeKernel runs every work-item: kernels without
 *               barrier() as an OpenMP loop, kernels with barrier() one group
 *               at a time, each work-item a ucontext fiber that yields at the
 *               barrier.
 *   events      carry the wall-clock start and end of their launch.
 *   records     every program source and options, and each kernel's last
 *               argument list, are kept for the refhost_* queries below.
 */
#include <dlfcn.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <ucontext.h>
#include <unistd.h>

#include <algorithm>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "CL/opencl.h"

#ifndef REFHOST_HDR_DIR
#define REFHOST_HDR_DIR "."
#endif

struct clc_wi
{
   size_t gid, lid, grp, lsz, gsz, ngrp;
   void (*yield)(clc_wi *);
};

typedef void (*entry_fn)(void **, clc_wi *);

struct _cl_platform_id { int dummy; };
struct _cl_device_id { int dummy; };
struct _cl_context { int dummy; };
struct _cl_command_queue { int dummy; };
struct _cl_mem { void *data; size_t size; };
struct _cl_event { double beg, end; };

struct _cl_program
{
   std::string src, opt, log;
   void *dl;
   bool barriers;
};

struct _cl_kernel
{
   _cl_program *prg;
   std::string name;
   entry_fn fn;
   std::vector<std::vector<unsigned char> > args;
};

static _cl_platform_id the_platform;
static _cl_device_id the_device;
static _cl_context the_context;
static _cl_command_queue the_queue;
static std::set<_cl_mem *> live_mems;
static std::vector<_cl_program *> programs;
static std::vector<_cl_kernel *> kernels;                 /* in creation order */
static size_t max_group = 256;

static double now_s()
{
   struct timespec t;
   clock_gettime(CLOCK_MONOTONIC, &t);
   return t.tv_sec + 1e-9 * t.tv_nsec;
}

static const char *cache_dir()
{
   const char *d = getenv("REFHOST_CACHE");
   return d ? d : "/tmp/refhost_jit";
}

/* ---- platform, device, context, queue ------------------------------------ */

extern "C" cl_int clGetPlatformIDs(cl_uint n, cl_platform_id *p, cl_uint *num)
{
   if(p && n) p[0] = &the_platform;
   if(num) *num = 1;
   return CL_SUCCESS;
}

extern "C" cl_int clGetDeviceIDs(cl_platform_id, cl_device_type, cl_uint n, cl_device_id *d,
                                 cl_uint *num)
{
   if(d && n) d[0] = &the_device;
   if(num) *num = 1;
   return CL_SUCCESS;
}

extern "C" cl_int clGetDeviceInfo(cl_device_id, cl_device_info what, size_t sz, void *val,
                                  size_t *ret)
{
   const char *s = what == CL_DEVICE_EXTENSIONS ? "cl_khr_fp64 cl_khr_byte_addressable_store"
                                                : "refhost CPU (mock OpenCL runtime)";
   size_t n = strlen(s) + 1;
   if(val && sz)
   {
      strncpy((char *)val, s, sz);
      ((char *)val)[sz - 1] = 0;
   }
   if(ret) *ret = n;
   return CL_SUCCESS;
}

extern "C" cl_context clCreateContext(const cl_context_properties *, cl_uint, const cl_device_id *,
                                      void (*)(const char *, const void *, size_t, void *), void *,
                                      cl_int *err)
{
   if(err) *err = CL_SUCCESS;
   return &the_context;
}

extern "C" cl_command_queue clCreateCommandQueue(cl_context, cl_device_id,
                                                 cl_command_queue_properties, cl_int *err)
{
   if(err) *err = CL_SUCCESS;
   return &the_queue;
}

extern "C" cl_int clFinish(cl_command_queue) { return CL_SUCCESS; }
extern "C" cl_int clReleaseCommandQueue(cl_command_queue) { return CL_SUCCESS; }
extern "C" cl_int clReleaseContext(cl_context) { return CL_SUCCESS; }

/* ---- buffers -------------------------------------------------------------- */

extern "C" cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t size, void *host, cl_int *err)
{
   _cl_mem *m = new _cl_mem;
   m->size = size;
   m->data = calloc(size ? size : 1, 1);
   if(host && size)
      memcpy(m->data, host, size);
   live_mems.insert(m);
   if(err) *err = m->data ? CL_SUCCESS : CL_INVALID_VALUE;
   return m;
}

extern "C" cl_int clReleaseMemObject(cl_mem m)
{
   if(!live_mems.count(m))
      return CL_INVALID_VALUE;
   live_mems.erase(m);
   free(m->data);
   delete m;
   return CL_SUCCESS;
}

static cl_event new_event(cl_event *out, double beg, double end)
{
   if(!out) return 0;
   _cl_event *e = new _cl_event;   /* never released by the reference: kept */
   e->beg = beg;
   e->end = end;
   *out = e;
   return e;
}

extern "C" cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem m, cl_bool, size_t off, size_t sz,
                                       const void *src, cl_uint, const cl_event *, cl_event *ev)
{
   if(!live_mems.count(m) || off + sz > m->size)
      return CL_INVALID_VALUE;
   double t = now_s();
   memcpy((char *)m->data + off, src, sz);
   new_event(ev, t, now_s());
   return CL_SUCCESS;
}

extern "C" cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem m, cl_bool, size_t off, size_t sz,
                                      void *dst, cl_uint, const cl_event *, cl_event *ev)
{
   if(!live_mems.count(m) || off + sz > m->size)
      return CL_INVALID_VALUE;
   double t = now_s();
   memcpy(dst, (char *)m->data + off, sz);
   new_event(ev, t, now_s());
   return CL_SUCCESS;
}

extern "C" cl_int clGetEventProfilingInfo(cl_event e, cl_profiling_info what, size_t sz, void *val,
                                          size_t *ret)
{
   if(ret) *ret = sizeof(cl_ulong);
   if(!e || !val || sz < sizeof(cl_ulong))
      return CL_INVALID_VALUE;
   double t = what == CL_PROFILING_COMMAND_END ? e->end : e->beg;
   *(cl_ulong *)val = (cl_ulong)(t * 1e9);
   return CL_SUCCESS;
}

/* ---- programs --------------------------------------------------------------- */

extern "C" cl_program clCreateProgramWithSource(cl_context, cl_uint n, const char **src,
                                                const size_t *len, cl_int *err)
{
   _cl_program *p = new _cl_program;
   p->dl = 0;
   p->barriers = false;
   for(cl_uint i=0;i<n;i++)
      p->src += len && len[i] ? std::string(src[i], len[i]) : std::string(src[i]);
   programs.push_back(p);
   if(err) *err = CL_SUCCESS;
   return p;
}

static unsigned long long fnv1a(const std::string &s, unsigned long long h)
{
   for(unsigned char c : s)
      h = (h ^ c) * 1099511628211ULL;
   return h;
}

/* names of the __kernel functions of a program, in order */
static std::vector<std::string> kernel_names(const std::string &src)
{
   std::vector<std::string> out;
   size_t pos = 0;
   while((pos = src.find("__kernel", pos)) != std::string::npos)
   {
      size_t p = pos + 8, q;
      pos = p;
      while(p < src.size() && isspace((unsigned char)src[p])) p++;
      if(src.compare(p, 4, "void")) continue;
      p += 4;
      while(p < src.size() && isspace((unsigned char)src[p])) p++;
      q = p;
      while(q < src.size() && (isalnum((unsigned char)src[q]) || src[q] == '_')) q++;
      /* one entry per name: #if branches of a library kernel reuse it */
      if(q > p && std::find(out.begin(), out.end(), src.substr(p, q - p)) == out.end())
         out.push_back(src.substr(p, q - p));
   }
   return out;
}

/* the -D options of an OpenCL build string, as g++ options */
static std::string defines(const std::string &opt)
{
   std::string out;
   size_t p = 0;
   while((p = opt.find("-D", p)) != std::string::npos)
   {
      size_t q = p;
      while(q < opt.size() && !isspace((unsigned char)opt[q])) q++;
      out += " '" + opt.substr(p, q - p) + "'";
      p = q;
   }
   return out;
}

extern "C" cl_int clBuildProgram(cl_program p, cl_uint, const cl_device_id *, const char *opt,
                                 void (*)(cl_program, void *), void *)
{
   char base[1024], cpp[1100], so[1100], log[1100], cmd[8192];
   std::vector<std::string> names = kernel_names(p->src);
   const char *extra = getenv("REFHOST_CXXFLAGS");   /* e.g. a sanitizer */
   unsigned long long h;

   p->opt = opt ? opt : "";
   p->barriers = p->src.find("barrier(") != std::string::npos;
   h = fnv1a(extra ? extra : "", fnv1a(p->opt, fnv1a(p->src, 1469598103934665603ULL)));
   mkdir(cache_dir(), 0755);
   snprintf(base, sizeof base, "%s/prg_%016llx", cache_dir(), h);
   snprintf(cpp, sizeof cpp, "%s.cpp", base);
   snprintf(so, sizeof so, "%s.so", base);
   snprintf(log, sizeof log, "%s.log", base);

   if(access(so, R_OK))
   {
      FILE *f = fopen(cpp, "w");
      if(!f) return CL_BUILD_PROGRAM_FAILURE;
      fputs("#include \"clc_host.hpp\"\n", f);
      fputs(p->src.c_str(), f);
      fputs("\n", f);
      for(const std::string &k : names)
         fprintf(f, "extern \"C\" void %s__refhost(void **a, clc_wi *wi)"
                    " { clc_cur = wi; clc_invoke(%s, a); }\n", k.c_str(), k.c_str());
      fclose(f);
      snprintf(cmd, sizeof cmd,
               "g++ -O2 -std=c++17 -shared -fPIC -w -fsingle-precision-constant"
               " -ffp-contract=off %s -I'%s' %s '%s' -o '%s.tmp' > '%s' 2>&1 && mv '%s.tmp' '%s'",
               extra ? extra : "", REFHOST_HDR_DIR, defines(p->opt).c_str(), cpp, so, log, so, so);
      if(system(cmd))
      {
         FILE *g = fopen(log, "r");
         char buf[4096];
         size_t n = g ? fread(buf, 1, sizeof buf - 1, g) : 0;
         if(g) fclose(g);
         buf[n] = 0;
         p->log = std::string("g++ failed on ") + cpp + "\n" + buf;
         return CL_BUILD_PROGRAM_FAILURE;
      }
   }
   p->dl = dlopen(so, RTLD_NOW | RTLD_LOCAL);
   if(!p->dl)
   {
      p->log = dlerror();
      return CL_BUILD_PROGRAM_FAILURE;
   }
   return CL_SUCCESS;
}

extern "C" cl_int clGetProgramBuildInfo(cl_program p, cl_device_id, cl_program_build_info,
                                        size_t sz, void *val, size_t *ret)
{
   if(ret) *ret = p->log.size() + 1;
   if(val && sz)
   {
      strncpy((char *)val, p->log.c_str(), sz);
      ((char *)val)[sz - 1] = 0;
   }
   return CL_SUCCESS;
}

extern "C" cl_int clGetProgramInfo(cl_program p, cl_program_info, size_t sz, void *val,
                                   size_t *ret)
{
   if(ret) *ret = sizeof(size_t);
   if(val && sz >= sizeof(size_t))
      *(size_t *)val = p->src.size();
   return CL_SUCCESS;
}

extern "C" cl_int clReleaseProgram(cl_program) { return CL_SUCCESS; }

/* ---- kernels ---------------------------------------------------------------- */

extern "C" cl_kernel clCreateKernel(cl_program p, const char *name, cl_int *err)
{
   std::string sym = std::string(name) + "__refhost";
   entry_fn fn = p->dl ? (entry_fn)dlsym(p->dl, sym.c_str()) : 0;
   if(!fn)
   {
      if(err) *err = CL_INVALID_KERNEL_NAME;
      return 0;
   }
   _cl_kernel *k = new _cl_kernel;
   k->prg = p;
   k->name = name;
   k->fn = fn;
   kernels.push_back(k);
   if(err) *err = CL_SUCCESS;
   return k;
}

extern "C" cl_int clReleaseKernel(cl_kernel) { return CL_SUCCESS; }

extern "C" cl_int clGetKernelWorkGroupInfo(cl_kernel, cl_device_id, cl_kernel_work_group_info,
                                           size_t sz, void *val, size_t *ret)
{
   if(ret) *ret = sizeof(size_t);
   if(val && sz >= sizeof(size_t))
      *(size_t *)val = max_group;
   return CL_SUCCESS;
}

extern "C" cl_int clSetKernelArg(cl_kernel k, cl_uint i, size_t sz, const void *val)
{
   if(!k)
      return CL_INVALID_KERNEL;
   if(i >= 256)
      return CL_INVALID_ARG_INDEX;
   if(k->args.size() <= i)
      k->args.resize(i + 1);
   k->args[i].assign((const unsigned char *)val, (const unsigned char *)val + sz);
   return CL_SUCCESS;
}

/* argument value addresses: a cl_mem argument becomes its data pointer */
static void arg_values(_cl_kernel *k, std::vector<void *> &ptrs, std::vector<void *> &slots)
{
   size_t n = k->args.size();
   ptrs.resize(n);
   slots.resize(n);
   for(size_t i=0;i<n;i++)
   {
      std::vector<unsigned char> &a = k->args[i];
      _cl_mem *m = 0;
      if(a.size() == sizeof(cl_mem))
         memcpy(&m, a.data(), sizeof m);
      if(m && live_mems.count(m))
      {
         ptrs[i] = m->data;
         slots[i] = &ptrs[i];
      }
      else
         slots[i] = a.data();
   }
}

/* a group with barriers: one fiber per work-item, resumed in turn */
struct fiber
{
   clc_wi wi;                /* first member: the wi pointer is the fiber pointer */
   ucontext_t ctx;
   ucontext_t *sched;
   entry_fn fn;
   void **args;
   bool done;
};

static void fiber_yield(clc_wi *wi)
{
   fiber *f = (fiber *)wi;
   swapcontext(&f->ctx, f->sched);
}

static void fiber_start(unsigned hi, unsigned lo)
{
   fiber *f = (fiber *)(((uintptr_t)hi << 32) | (uintptr_t)lo);
   f->fn(f->args, &f->wi);
   f->done = true;
   swapcontext(&f->ctx, f->sched);
}

static void run_groups_with_barriers(entry_fn fn, void **args, size_t gsz, size_t lsz)
{
   const size_t stack = 256 * 1024;
   std::vector<fiber> fib(lsz);
   std::vector<char> stacks(lsz * stack);
   ucontext_t sched;
   size_t ngrp = gsz / lsz;

   for(size_t g=0;g<ngrp;g++)
   {
      for(size_t l=0;l<lsz;l++)
      {
         fiber &f = fib[l];
         f.wi.gid = g * lsz + l;
         f.wi.lid = l;
         f.wi.grp = g;
         f.wi.lsz = lsz;
         f.wi.gsz = gsz;
         f.wi.ngrp = ngrp;
         f.wi.yield = fiber_yield;
         f.sched = &sched;
         f.fn = fn;
         f.args = args;
         f.done = false;
         getcontext(&f.ctx);
         f.ctx.uc_stack.ss_sp = &stacks[l * stack];
         f.ctx.uc_stack.ss_size = stack;
         f.ctx.uc_link = 0;
         uintptr_t p = (uintptr_t)&f;
         makecontext(&f.ctx, (void (*)())fiber_start, 2, (unsigned)(p >> 32),
                     (unsigned)(p & 0xffffffffu));
      }
      for(;;)
      {
         bool alive = false;
         for(size_t l=0;l<lsz;l++)
            if(!fib[l].done)
            {
               swapcontext(&sched, &fib[l].ctx);
               alive |= !fib[l].done;
            }
         if(!alive)
            break;
      }
   }
}

extern "C" cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel k, cl_uint dim,
                                         const size_t *, const size_t *gsz, const size_t *lsz,
                                         cl_uint, const cl_event *, cl_event *ev)
{
   std::vector<void *> ptrs, slots;
   size_t G, L;

   if(!k)
      return CL_INVALID_KERNEL;
   if(dim != 1 || !gsz)
      return CL_INVALID_VALUE;
   G = gsz[0];
   L = lsz && lsz[0] ? lsz[0] : 1;
   if(G % L)
      return CL_INVALID_VALUE;
   arg_values(k, ptrs, slots);
   double t0 = now_s();

   if(k->prg->barriers)
      run_groups_with_barriers(k->fn, slots.data(), G, L);
   else
   {
      entry_fn fn = k->fn;
      void **a = slots.data();
      const long long n = (long long)G;
      #pragma omp parallel for schedule(static)
      for(long long i=0;i<n;i++)
      {
         clc_wi wi;
         wi.gid = (size_t)i;
         wi.lid = (size_t)i % L;
         wi.grp = (size_t)i / L;
         wi.lsz = L;
         wi.gsz = G;
         wi.ngrp = G / L;
         wi.yield = 0;
         fn(a, &wi);
      }
   }
   new_event(ev, t0, now_s());
   return CL_SUCCESS;
}

/* ---- queries for the fixture scripts ------------------------------------ */

extern "C" int refhost_nprograms(void) { return (int)programs.size(); }

extern "C" const char *refhost_program_source(int i)
{
   return i >= 0 && i < (int)programs.size() ? programs[i]->src.c_str() : 0;
}

extern "C" const char *refhost_program_options(int i)
{
   return i >= 0 && i < (int)programs.size() ? programs[i]->opt.c_str() : 0;
}

extern "C" int refhost_nkernels(void) { return (int)kernels.size(); }

extern "C" const char *refhost_kernel_name(int i)
{
   return i >= 0 && i < (int)kernels.size() ? kernels[i]->name.c_str() : 0;
}

/* the argument list bound to kernel object i (creation order): ptr[a] is a
   buffer's data (size[a] its bytes) or 0 for a value argument (size[a] its
   bytes); returns the argument count, or -1 for an unknown kernel */
extern "C" int refhost_kernel_args(int i, void **ptr, size_t *size, int max)
{
   if(i < 0 || i >= (int)kernels.size())
      return -1;
   _cl_kernel *k = kernels[i];
   int n = (int)k->args.size();
   for(int a=0;a<n && a<max;a++)
   {
      std::vector<unsigned char> &v = k->args[a];
      _cl_mem *m = 0;
      if(v.size() == sizeof(cl_mem))
         memcpy(&m, v.data(), sizeof m);
      if(m && live_mems.count(m))
      {
         ptr[a] = m->data;
         size[a] = m->size;
      }
      else
      {
         ptr[a] = 0;
         size[a] = v.size();
      }
   }
   return n;
}

/* the program index of kernel object i, or -1 */
extern "C" int refhost_kernel_program(int i)
{
   if(i < 0 || i >= (int)kernels.size())
      return -1;
   for(size_t p=0;p<programs.size();p++)
      if(programs[p] == kernels[i]->prg)
         return (int)p;
   return -1;
}

extern "C" void refhost_set_max_group(int n) { if(n > 0) max_group = (size_t)n; }
