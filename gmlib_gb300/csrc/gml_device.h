/*
 * gml_device.h -- thin C ABI between the C99 GMlib host layer and CUDA.
 *
 * Everything that touches the GPU goes through these calls: device and stream
 * setup, device/pinned allocations, host<->device copies, NVRTC compilation of
 * generated kernels, module loading and launches, CUDA events, and the
 * hand-written library kernels (reductions, block sparse mat-vec, vector
 * algebra, native mesh kernels).  The implementation is gml_device.cu plus the
 * kernel files; the host layer never includes a CUDA header.
 *
 * In the reference these roles are played by OpenCL calls made directly from
 * sources/gmlib3.c (clCreateBuffer, clEnqueueWriteBuffer/ReadBuffer,
 * clBuildProgram, clEnqueueNDRangeKernel, clGetEventProfilingInfo).
 */
#ifndef GML_DEVICE_H
#define GML_DEVICE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct GmdCtx GmdCtx;

/* device and context ------------------------------------------------------- */
int      gmd_device_count(void);
int      gmd_device_name(int dev, char *buf, int len);
GmdCtx  *gmd_init(int dev, int *fp64, char *err, int errlen);
void     gmd_stop(GmdCtx *ctx);
int      gmd_sync(GmdCtx *ctx);
void    *gmd_stream(GmdCtx *ctx);          /* cudaStream_t of the instance */
const char *gmd_last_error(GmdCtx *ctx);
int      gmd_num_sms(GmdCtx *ctx);
size_t   gmd_free_memory(GmdCtx *ctx);

/* memory -------------------------------------------------------------------- */
void    *gmd_alloc(GmdCtx *ctx, size_t bytes);           /* device, zeroed */
void     gmd_free(GmdCtx *ctx, void *ptr);
void    *gmd_host_alloc(size_t bytes);                    /* pinned, zeroed */
void     gmd_host_free(void *ptr);
int      gmd_h2d_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes);
int      gmd_d2h(GmdCtx *ctx, void *dst, const void *src, size_t bytes);
int      gmd_d2h_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes);
int      gmd_d2d_async(GmdCtx *ctx, void *dst, const void *src, size_t bytes);
int      gmd_memset_async(GmdCtx *ctx, void *dst, int val, size_t bytes);
int      gmd_host_addressable(GmdCtx *ctx, const void *p);  /* kernels can use host pointer p */
int      gmd_idle(GmdCtx *ctx);                               /* no work pending */
/* one-kernel copy of bytes from src to d0 and d1 (d1 may be NULL); 0 when
   the pointers are not 16-byte aligned or bytes is not a multiple of 16 */
int      gmd_fanout(GmdCtx *ctx, const void *src, void *d0, void *d1, size_t bytes);

/* events ------------------------------------------------------------------- */
void    *gmd_event_new(void);
void     gmd_event_free(void *evt);
int      gmd_event_record(GmdCtx *ctx, void *evt);
int      gmd_event_wait(void *evt);
double   gmd_event_elapsed_s(void *beg, void *end);    /* synchronises on end */
int      gmd_capturing(GmdCtx *ctx);                   /* stream under graph capture */
int      gmd_use_side(GmdCtx *ctx, int on);            /* work goes to the side stream */
void    *gmd_event_new_sync(void);                     /* event without timing */
int      gmd_stream_wait(GmdCtx *ctx, void *evt);      /* current stream waits for evt */

/* NVRTC + modules ----------------------------------------------------------- */
/* Compile a generated CUDA source to an sm_103a cubin.  Returns 1 on success;
   on failure *log holds the compiler log (malloc'd).  opts is a blank
   separated list of extra NVRTC options. */
int      gmd_compile(const char *src, const char *name, const char *opts,
                     void **cubin, size_t *cubin_size, char **log);
int      gmd_module_load(GmdCtx *ctx, const void *cubin, const char *name,
                         void **module, void **func, int *max_threads, int *num_regs);
void     gmd_module_unload(void *module);
int      gmd_launch(GmdCtx *ctx, void *func, unsigned grid, unsigned block,
                    unsigned smem, void **args);

/* library kernels ------------------------------------------------------------ */
/* Reduction of a float field of n lines: op is GmlMin..GmlLinf (gmlib3.h).
   The result is accumulated in FP64 (sums) and written to *res (host). */
int      gmd_reduce_f32(GmdCtx *ctx, int op, const float *in, int n, double *res,
                        void *scratch);
size_t   gmd_reduce_scratch_bytes(int n);

/* exclusive prefix sums: out[0..n-1] and the total in out[n] (gml_scan.cu) */
int      gmd_scan_excl_i32(GmdCtx *ctx, const int *in, int *out, int n);
int      gmd_scan_excl_i64(GmdCtx *ctx, const long long *in, long long *out, int n);

/* min/argmin/max/argmax of a float field, smallest index wins ties. */
int      gmd_minmax_arg_f32(GmdCtx *ctx, const float *in, int n,
                            float *vmin, int *imin, float *vmax, int *imax,
                            void *scratch);

#ifdef __cplusplus
}
#endif

#endif
