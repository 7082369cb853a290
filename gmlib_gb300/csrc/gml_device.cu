/*
 * gml_device.cu -- CUDA side of the thin C ABI declared in gml_device.h.
 *
 * One GmlInit instance owns one non-blocking CUDA stream on the selected
 * device; every copy and launch of the instance is ordered on that stream
 * (the reference uses one in-order OpenCL queue per instance,
 * sources/gmlib3.c:437-438).  Generated kernels are compiled by NVRTC straight
 * to an sm_103a cubin and loaded through the driver API, whose entry points
 * are fetched from the runtime (cudaGetDriverEntryPoint) so that the library
 * loads on hosts without a GPU driver.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include <cuda.h>
#include <nvrtc.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gml_device.h"

/* embedded headers for NVRTC (generated at build time from gml_cl.h and
   gml_toolkit.h) */
extern "C" const char *gml_embedded_cl_h;
extern "C" const char *gml_embedded_toolkit_h;

struct GmdCtx
{
   int            dev, nsm;
   cudaStream_t   stream;
   cudaStream_t   side;          /* second stream for concurrent graph branches */
   int            use_side;      /* 1: gmd_stream returns the side stream */
   int            pageable;      /* kernels can address pageable host memory */
   char           err[512];
};

/* ------------------------------------------------------------------------- */
/* driver API entry points                                                    */
/* ------------------------------------------------------------------------- */

typedef CUresult (*PFN_ModuleLoadData)(CUmodule *, const void *);
typedef CUresult (*PFN_ModuleGetFunction)(CUfunction *, CUmodule, const char *);
typedef CUresult (*PFN_ModuleUnload)(CUmodule);
typedef CUresult (*PFN_LaunchKernel)(CUfunction, unsigned, unsigned, unsigned,
                                     unsigned, unsigned, unsigned, unsigned,
                                     CUstream, void **, void **);
typedef CUresult (*PFN_FuncGetAttribute)(int *, CUfunction_attribute, CUfunction);
typedef CUresult (*PFN_FuncSetAttribute)(CUfunction, CUfunction_attribute, int);

static PFN_ModuleLoadData     p_cuModuleLoadData;
static PFN_ModuleGetFunction  p_cuModuleGetFunction;
static PFN_ModuleUnload       p_cuModuleUnload;
static PFN_LaunchKernel       p_cuLaunchKernel;
static PFN_FuncGetAttribute   p_cuFuncGetAttribute;
static PFN_FuncSetAttribute   p_cuFuncSetAttribute;

static int load_driver_api(char *err, int errlen)
{
   cudaDriverEntryPointQueryResult q;
   if(p_cuLaunchKernel)
      return 1;
#define GET(sym, ptr) \
   if(cudaGetDriverEntryPointByVersion(sym, (void **)&ptr, 12000, cudaEnableDefault, &q) != cudaSuccess \
      || q != cudaDriverEntryPointSuccess || !ptr) \
   { snprintf(err, errlen, "driver entry point %s unavailable", sym); return 0; }
   GET("cuModuleLoadData", p_cuModuleLoadData);
   GET("cuModuleGetFunction", p_cuModuleGetFunction);
   GET("cuModuleUnload", p_cuModuleUnload);
   GET("cuFuncGetAttribute", p_cuFuncGetAttribute);
   GET("cuFuncSetAttribute", p_cuFuncSetAttribute);
   GET("cuLaunchKernel", p_cuLaunchKernel);
#undef GET
   return 1;
}

static int ok(GmdCtx *ctx, cudaError_t e, const char *what)
{
   if(e == cudaSuccess)
      return 1;
   if(ctx)
      snprintf(ctx->err, sizeof(ctx->err), "%s: %s", what, cudaGetErrorString(e));
   fprintf(stderr, "GMlib CUDA error in %s: %s\n", what, cudaGetErrorString(e));
   return 0;
}

/* ------------------------------------------------------------------------- */
/* device and context                                                         */
/* ------------------------------------------------------------------------- */

extern "C" int gmd_device_count(void)
{
   int n = 0;
   if(cudaGetDeviceCount(&n) != cudaSuccess)
   {
      cudaGetLastError();
      return 0;
   }
   return n;
}

extern "C" int gmd_device_name(int dev, char *buf, int len)
{
   cudaDeviceProp p;
   if(cudaGetDeviceProperties(&p, dev) != cudaSuccess)
      return 0;
   snprintf(buf, len, "%s", p.name);
   return 1;
}

extern "C" GmdCtx *gmd_init(int dev, int *fp64, char *err, int errlen)
{
   GmdCtx *ctx;
   int n = gmd_device_count();
   cudaDeviceProp p;

   if(dev < 0 || dev >= n)
   {
      snprintf(err, errlen, "Selected device Id is out of bounds (0 -> %d)", n - 1);
      return NULL;
   }
   if(cudaSetDevice(dev) != cudaSuccess || cudaFree(0) != cudaSuccess)
   {
      snprintf(err, errlen, "cannot initialise device %d", dev);
      return NULL;
   }
   if(!load_driver_api(err, errlen))
      return NULL;

   ctx = (GmdCtx *)calloc(1, sizeof(GmdCtx));
   if(!ctx)
      return NULL;
   ctx->dev = dev;
   cudaGetDeviceProperties(&p, dev);
   ctx->nsm = p.multiProcessorCount;
   {
      /* GML_DIRECT=0 keeps whole-datatype transfers on the staged path */
      const char *e = getenv("GML_DIRECT");
      int v = 0;
      if(cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess)
      {
         cudaGetLastError();
         v = 0;
      }
      ctx->pageable = v && !(e && *e == '0');
   }

   if(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
   {
      snprintf(err, errlen, "cannot create a CUDA stream");
      free(ctx);
      return NULL;
   }
   if(fp64)
      *fp64 = 1;   /* every sm_103a device has FP64 units */
   return ctx;
}

extern "C" void gmd_stop(GmdCtx *ctx)
{
   if(!ctx)
      return;
   cudaSetDevice(ctx->dev);
   cudaStreamSynchronize(ctx->stream);
   cudaStreamDestroy(ctx->stream);
   if(ctx->side)
   {
      cudaStreamSynchronize(ctx->side);
      cudaStreamDestroy(ctx->side);
   }
   free(ctx);
}

extern "C" int gmd_sync(GmdCtx *ctx)
{
   if(!ctx)
      return 1;
   return ok(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize");
}

extern "C" void *gmd_stream(GmdCtx *ctx)
{
   if(!ctx)
      return NULL;
   return ctx->use_side ? (void *)ctx->side : (void *)ctx->stream;
}

/* route subsequent work of the instance to its side stream (1) or back to
   the main stream (0) */
extern "C" int gmd_use_side(GmdCtx *ctx, int on)
{
   if(!ctx)
      return 0;
   if(on && !ctx->side
   && cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess)
      return 0;
   ctx->use_side = on ? 1 : 0;
   return 1;
}

/* event without timing, for ordering streams (also inside graph capture) */
extern "C" void *gmd_event_new_sync(void)
{
   cudaEvent_t e;
   if(cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return NULL;
   return (void *)e;
}

/* the current stream of the instance waits for an event */
extern "C" int gmd_stream_wait(GmdCtx *ctx, void *evt)
{
   if(!ctx || !evt)
      return 0;
   return ok(ctx, cudaStreamWaitEvent((cudaStream_t)gmd_stream(ctx), (cudaEvent_t)evt, 0),
             "stream wait");
}
/* ------------------------------------------------------------------------- */
/* direct whole-buffer transfers                                              */
/* ------------------------------------------------------------------------- */

/* 1 when kernels of the instance can read and write host memory at p:
   any host memory where the device has pageable memory access (on this
   platform, through the CPU's page tables over the chip-to-chip link), else
   only pinned or registered memory mapped at the same address */
extern "C" int gmd_host_addressable(GmdCtx *ctx, const void *p)
{
   cudaPointerAttributes a;
   if(!ctx || !p)
      return 0;
   if(ctx->pageable)
      return 1;
   if(cudaPointerGetAttributes(&a, p) != cudaSuccess)
   {
      cudaGetLastError();
      return 0;
   }
   return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

/* 1 when no work is pending on the instance's streams */
extern "C" int gmd_idle(GmdCtx *ctx)
{
   cudaError_t r;
   if(!ctx)
      return 0;
   r = cudaStreamQuery(ctx->stream);
   if(r == cudaSuccess && ctx->side)
      r = cudaStreamQuery(ctx->side);
   if(r != cudaSuccess && r != cudaErrorNotReady)
      return ok(ctx, r, "stream query");
   return r == cudaSuccess;
}

/* n 16-byte words from src to d0 and, when d1 is given, to d1 as well: one
   read of the source however many copies are written.  Block b copies the
   contiguous words [b chunk, (b + 1) chunk): over the chip-to-chip link a
   few long sequential streams measured faster than a grid-stride spread
   (34 MB from pageable memory to the device and a pinned mirror: 0.21 ms
   with 1 MB per block, 0.27 ms grid-stride). */
__global__ void __launch_bounds__(256)
fanout_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ d0, uint4 *__restrict__ d1,
              size_t n, size_t chunk)
{
   const size_t beg = (size_t)blockIdx.x * chunk;
   const size_t end = beg + chunk < n ? beg + chunk : n;
   size_t i = beg + threadIdx.x;
   for(;i+3*256<end;i+=4*256)
   {
      const uint4 a = src[i], b = src[i + 256], c = src[i + 512], d = src[i + 768];
      d0[i] = a; d0[i + 256] = b; d0[i + 512] = c; d0[i + 768] = d;
      if(d1)
      {
         d1[i] = a; d1[i + 256] = b; d1[i + 512] = c; d1[i + 768] = d;
      }
   }
   for(;i<end;i+=256)
   {
      const uint4 a = src[i];
      d0[i] = a;
      if(d1)
         d1[i] = a;
   }
}

/* copy bytes from src to d0 (and d1 unless NULL) with one kernel on the
   instance's stream; every pointer is device memory or host memory the
   device can address (gmd_host_addressable), 16-byte aligned, and bytes a
   multiple of 16.  Returns 0 (nothing launched) when those do not hold. */
extern "C" int gmd_fanout(GmdCtx *ctx, const void *src, void *d0, void *d1, size_t bytes)
{
   const size_t n = bytes / 16;
   size_t chunk;
   if(!ctx || !src || !d0 || (bytes & 15)
   || (((uintptr_t)src | (uintptr_t)d0 | (uintptr_t)d1) & 15))
      return 0;
   if(!n)
      return 1;
   /* 1 MB per block, at least 32 blocks, at least 64 KB per block */
   chunk = (n + 31) / 32;
   if(chunk > 65536) chunk = 65536;
   if(chunk < 4096) chunk = 4096;
   fanout_kernel<<<(unsigned)((n + chunk - 1) / chunk), 256, 0, ctx->stream>>>(
      (const uint4 *)src, (uint4 *)d0, (uint4 *)d1, n, chunk);
   return ok(ctx, cudaGetLastError(), "fan-out copy");
}

extern "C" const char *gmd_last_error(GmdCtx *ctx) { return ctx ? ctx->err : ""; }
extern "C" int gmd_num_sms(GmdCtx *ctx) { return ctx ? ctx->nsm : 1; }

extern "C" size_t gmd_free_memory(GmdCtx *ctx)
{
   size_t f = 0, t = 0;
   (void)ctx;
   cudaMemGetInfo(&f, &t);
   return f;
}

/* ------------------------------------------------------------------------- */
/* memory                                                                     */
/* ------------------------------------------------------------------------- */

extern "C" void *gmd_alloc(GmdCtx *ctx, size_t bytes)
{
   void *p = NULL;
   if(!bytes)
      bytes = 16;
   if(!ctx)                       /* offline instance: host memory */
      return calloc(1, bytes);
   if(!ok(ctx, cudaMallocAsync(&p, bytes, ctx->stream), "device allocation"))
      return NULL;
   if(!ok(ctx, cudaMemsetAsync(p, 0, bytes, ctx->stream), "device clear"))
      return NULL;
   return p;
}

extern "C" void gmd_free(GmdCtx *ctx, void *ptr)
{
   if(ptr && !ctx)
      free(ptr);
   else if(ptr)
      cudaFreeAsync(ptr, ctx->stream);
}

extern "C" void *gmd_host_alloc(size_t bytes)
{
   void *p = NULL;
   if(!bytes)
      bytes = 16;
   if(cudaMallocHost(&p, bytes) != cudaSuccess)
   {
      cudaGetLastError();
      return NULL;
   }
   memset(p, 0, bytes);
   return p;
}

extern "C" void gmd_host_free(void *ptr)
{
   if(ptr)
      cudaFreeHost(ptr);
}

extern "C" int gmd_h2d_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes)
{
   if(!ctx) { memcpy(dst, src, bytes); return 1; }
   return ok(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "upload");
}

extern "C" int gmd_d2h(GmdCtx *ctx, void *dst, const void *src, size_t bytes)
{
   if(!ctx) { memcpy(dst, src, bytes); return 1; }
   if(!ok(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download"))
      return 0;
   return ok(ctx, cudaStreamSynchronize(ctx->stream), "download synchronize");
}

extern "C" int gmd_d2h_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes)
{
   if(!ctx) { memcpy(dst, src, bytes); return 1; }
   return ok(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream), "download");
}

extern "C" int gmd_d2d_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes)
{
   if(!ctx) { memmove(dst, src, bytes); return 1; }
   return ok(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream), "device copy");
}

extern "C" int gmd_memset_async(GmdCtx *ctx, void *dst, int val, size_t bytes)
{
   if(!ctx) { memset(dst, val, bytes); return 1; }
   return ok(ctx, cudaMemsetAsync(dst, val, bytes, ctx->stream), "device memset");
}

/* ------------------------------------------------------------------------- */
/* events                                                                     */
/* ------------------------------------------------------------------------- */

extern "C" void *gmd_event_new(void)
{
   cudaEvent_t e;
   if(cudaEventCreate(&e) != cudaSuccess)
      return NULL;
   return (void *)e;
}

extern "C" void gmd_event_free(void *evt)
{
   if(evt)
      cudaEventDestroy((cudaEvent_t)evt);
}

extern "C" int gmd_event_record(GmdCtx *ctx, void *evt)
{
   if(!ctx || !evt)
      return 0;
   return ok(ctx, cudaEventRecord((cudaEvent_t)evt, (cudaStream_t)gmd_stream(ctx)), "event record");
}

extern "C" int gmd_event_wait(void *evt)
{
   if(!evt)
      return 1;
   return cudaEventSynchronize((cudaEvent_t)evt) == cudaSuccess;
}

extern "C" double gmd_event_elapsed_s(void *beg, void *end)
{
   float ms = 0.f;
   if(!beg || !end)
      return 0.;
   if(cudaEventSynchronize((cudaEvent_t)end) != cudaSuccess)
      return 0.;
   if(cudaEventElapsedTime(&ms, (cudaEvent_t)beg, (cudaEvent_t)end) != cudaSuccess)
   {
      cudaGetLastError();
      return 0.;
   }
   return 1e-3 * (double)ms;
}

extern "C" int gmd_capturing(GmdCtx *ctx)
{
   cudaStreamCaptureStatus s = cudaStreamCaptureStatusNone;
   if(!ctx)
      return 0;
   cudaStreamIsCapturing(ctx->stream, &s);
   return s != cudaStreamCaptureStatusNone;
}

/* ------------------------------------------------------------------------- */
/* NVRTC                                                                      */
/* ------------------------------------------------------------------------- */

extern "C" int gmd_compile(const char *src, const char *name, const char *opts,
                           void **cubin, size_t *cubin_size, char **log)
{
   nvrtcProgram prog;
   const char *hdr[2]  = { gml_embedded_cl_h, gml_embedded_toolkit_h };
   const char *hnam[2] = { "gml_cl.h", "gml_toolkit.h" };
   const char *argv[64];
   char *optbuf = NULL, *tok, *save = NULL;
   int argc = 0, okres;
   size_t n;
   nvrtcResult r;

   *cubin = NULL;
   *cubin_size = 0;
   if(log)
      *log = NULL;

   argv[argc++] = "--gpu-architecture=sm_103a";
   argv[argc++] = "-std=c++17";
   argv[argc++] = "--fmad=true";
   argv[argc++] = "-default-device";
   argv[argc++] = "-lineinfo";

   if(opts && *opts)
   {
      optbuf = strdup(opts);
      for(tok = strtok_r(optbuf, " \t\n", &save); tok && argc < 60;
          tok = strtok_r(NULL, " \t\n", &save))
         argv[argc++] = tok;
   }

   if(nvrtcCreateProgram(&prog, src, name, 2, hdr, hnam) != NVRTC_SUCCESS)
   {
      free(optbuf);
      return 0;
   }

   r = nvrtcCompileProgram(prog, argc, argv);
   okres = (r == NVRTC_SUCCESS);

   if(log && nvrtcGetProgramLogSize(prog, &n) == NVRTC_SUCCESS && n > 1)
   {
      *log = (char *)malloc(n + 1);
      nvrtcGetProgramLog(prog, *log);
   }

   if(okres && nvrtcGetCUBINSize(prog, &n) == NVRTC_SUCCESS && n)
   {
      *cubin = malloc(n);
      nvrtcGetCUBIN(prog, (char *)*cubin);
      *cubin_size = n;
   }
   else
      okres = 0;

   nvrtcDestroyProgram(&prog);
   free(optbuf);
   return okres;
}

extern "C" int gmd_module_load(GmdCtx *ctx, const void *cubin, const char *name,
                               void **module, void **func, int *max_threads, int *num_regs)
{
   CUmodule m;
   CUfunction f;
   CUresult r;

   if(!ctx)
      return 0;
   cudaSetDevice(ctx->dev);
   if((r = p_cuModuleLoadData(&m, cubin)) != CUDA_SUCCESS)
   {
      snprintf(ctx->err, sizeof(ctx->err), "cuModuleLoadData failed (%d)", (int)r);
      return 0;
   }
   if((r = p_cuModuleGetFunction(&f, m, name)) != CUDA_SUCCESS)
   {
      snprintf(ctx->err, sizeof(ctx->err), "kernel %s not found (%d)", name, (int)r);
      p_cuModuleUnload(m);
      return 0;
   }
   if(max_threads)
      p_cuFuncGetAttribute(max_threads, CU_FUNC_ATTRIBUTE_MAX_THREADS_PER_BLOCK, f);
   if(num_regs)
      p_cuFuncGetAttribute(num_regs, CU_FUNC_ATTRIBUTE_NUM_REGS, f);
   *module = (void *)m;
   *func = (void *)f;
   return 1;
}

extern "C" void gmd_module_unload(void *module)
{
   if(module && p_cuModuleUnload)
      p_cuModuleUnload((CUmodule)module);
}

/* ------------------------------------------------------------------------- */
/* CUDA graphs                                                                */
/* ------------------------------------------------------------------------- */

extern "C" int gmd_graph_begin(GmdCtx *ctx)
{
   if(!ctx)
      return 0;
   return ok(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
             "begin graph capture");
}

extern "C" int gmd_graph_end(GmdCtx *ctx, void **exec)
{
   cudaGraph_t g = NULL;
   cudaGraphExec_t e = NULL;
   *exec = NULL;
   if(!ctx)
      return 0;
   if(!ok(ctx, cudaStreamEndCapture(ctx->stream, &g), "end graph capture"))
      return 0;
   if(!ok(ctx, cudaGraphInstantiate(&e, g, 0), "graph instantiate"))
   {
      cudaGraphDestroy(g);
      return 0;
   }
   cudaGraphDestroy(g);
   *exec = (void *)e;
   return 1;
}

extern "C" int gmd_graph_launch(GmdCtx *ctx, void *exec)
{
   if(!ctx || !exec)
      return 0;
   return ok(ctx, cudaGraphLaunch((cudaGraphExec_t)exec, ctx->stream), "graph launch");
}

extern "C" void gmd_graph_free(void *exec)
{
   if(exec)
      cudaGraphExecDestroy((cudaGraphExec_t)exec);
}

extern "C" int gmd_launch(GmdCtx *ctx, void *func, unsigned grid, unsigned block,
                          unsigned smem, void **args)
{
   CUresult r;
   if(!grid)
      return 1;
   if(!ctx)
      return 0;
   r = p_cuLaunchKernel((CUfunction)func, grid, 1, 1, block, 1, 1, smem,
                        (CUstream)ctx->stream, args, NULL);
   if(r != CUDA_SUCCESS)
   {
      snprintf(ctx->err, sizeof(ctx->err), "cuLaunchKernel failed (%d)", (int)r);
      fprintf(stderr, "GMlib: %s\n", ctx->err);
      return 0;
   }
   return 1;
}
