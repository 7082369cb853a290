/*
 * CL/opencl.h -- a stand-in for the OpenCL 1.2 host header, written for this
 * project from the public Khronos specification (types, sizes, enumerants).
 *
 * Test infrastructure.  It lets the reference's host library
 * (sources/gmlib3.c, which includes <CL/opencl.h> through sources/gmlib3.h)
 * compile unmodified on a machine with no OpenCL SDK; oracle/refhost/mockcl.cpp
 * provides the entry points.  Only the part of the API that the reference
 * host file calls is declared.
 */
#ifndef GML_REFHOST_OPENCL_H
#define GML_REFHOST_OPENCL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- scalar types (Khronos cl_platform.h sizes) ------------------------- */
typedef int8_t   cl_char;
typedef uint8_t  cl_uchar;
typedef int16_t  cl_short;
typedef uint16_t cl_ushort;
typedef int32_t  cl_int;
typedef uint32_t cl_uint;
typedef int64_t  cl_long;
typedef uint64_t cl_ulong;
typedef float    cl_float;
typedef double   cl_double;
typedef cl_uint  cl_bool;
typedef cl_ulong cl_bitfield;

/* ---- vector types: N lanes, aligned to their size (N*sizeof(T)) --------- */
#define GML_CLVEC(T, N) \
   typedef union { T s[N]; } __attribute__((aligned(N * sizeof(T)))) T##N;

GML_CLVEC(cl_char, 2)   GML_CLVEC(cl_char, 4)   GML_CLVEC(cl_char, 8)   GML_CLVEC(cl_char, 16)
GML_CLVEC(cl_uchar, 2)  GML_CLVEC(cl_uchar, 4)  GML_CLVEC(cl_uchar, 8)  GML_CLVEC(cl_uchar, 16)
GML_CLVEC(cl_int, 2)    GML_CLVEC(cl_int, 4)    GML_CLVEC(cl_int, 8)    GML_CLVEC(cl_int, 16)
GML_CLVEC(cl_uint, 2)   GML_CLVEC(cl_uint, 4)   GML_CLVEC(cl_uint, 8)   GML_CLVEC(cl_uint, 16)
GML_CLVEC(cl_float, 2)  GML_CLVEC(cl_float, 4)  GML_CLVEC(cl_float, 8)  GML_CLVEC(cl_float, 16)
GML_CLVEC(cl_double, 2) GML_CLVEC(cl_double, 4) GML_CLVEC(cl_double, 8) GML_CLVEC(cl_double, 16)
#undef GML_CLVEC

/* ---- opaque objects ------------------------------------------------------ */
typedef struct _cl_platform_id   *cl_platform_id;
typedef struct _cl_device_id     *cl_device_id;
typedef struct _cl_context       *cl_context;
typedef struct _cl_command_queue *cl_command_queue;
typedef struct _cl_mem           *cl_mem;
typedef struct _cl_program       *cl_program;
typedef struct _cl_kernel        *cl_kernel;
typedef struct _cl_event         *cl_event;

typedef cl_bitfield cl_device_type;
typedef cl_uint     cl_device_info;
typedef intptr_t    cl_context_properties;
typedef cl_bitfield cl_command_queue_properties;
typedef cl_bitfield cl_mem_flags;
typedef cl_uint     cl_program_info;
typedef cl_uint     cl_program_build_info;
typedef cl_uint     cl_kernel_work_group_info;
typedef cl_uint     cl_profiling_info;

/* ---- enumerants (values from the specification) ------------------------- */
#define CL_SUCCESS                   0
#define CL_INVALID_VALUE             (-30)
#define CL_INVALID_KERNEL_NAME       (-46)
#define CL_INVALID_KERNEL            (-48)
#define CL_INVALID_ARG_INDEX         (-49)
#define CL_BUILD_PROGRAM_FAILURE     (-11)
#define CL_FALSE                     0
#define CL_TRUE                      1
#define CL_DEVICE_TYPE_ALL           0xFFFFFFFF
#define CL_DEVICE_NAME               0x102B
#define CL_DEVICE_EXTENSIONS         0x1030
#define CL_QUEUE_PROFILING_ENABLE    (1 << 1)
#define CL_MEM_READ_WRITE            (1 << 0)
#define CL_MEM_WRITE_ONLY            (1 << 1)
#define CL_MEM_READ_ONLY             (1 << 2)
#define CL_PROGRAM_BINARY_SIZES      0x1165
#define CL_PROGRAM_BUILD_LOG         0x1183
#define CL_KERNEL_WORK_GROUP_SIZE    0x11B0
#define CL_PROFILING_COMMAND_QUEUED  0x1280
#define CL_PROFILING_COMMAND_END     0x1283

/* ---- entry points used by the reference host library -------------------- */
cl_int clGetPlatformIDs(cl_uint, cl_platform_id *, cl_uint *);
cl_int clGetDeviceIDs(cl_platform_id, cl_device_type, cl_uint, cl_device_id *, cl_uint *);
cl_int clGetDeviceInfo(cl_device_id, cl_device_info, size_t, void *, size_t *);
cl_context clCreateContext(const cl_context_properties *, cl_uint, const cl_device_id *,
                           void (*)(const char *, const void *, size_t, void *), void *, cl_int *);
cl_command_queue clCreateCommandQueue(cl_context, cl_device_id, cl_command_queue_properties,
                                      cl_int *);
cl_mem clCreateBuffer(cl_context, cl_mem_flags, size_t, void *, cl_int *);
cl_program clCreateProgramWithSource(cl_context, cl_uint, const char **, const size_t *, cl_int *);
cl_int clBuildProgram(cl_program, cl_uint, const cl_device_id *, const char *,
                      void (*)(cl_program, void *), void *);
cl_int clGetProgramBuildInfo(cl_program, cl_device_id, cl_program_build_info, size_t, void *,
                             size_t *);
cl_int clGetProgramInfo(cl_program, cl_program_info, size_t, void *, size_t *);
cl_kernel clCreateKernel(cl_program, const char *, cl_int *);
cl_int clGetKernelWorkGroupInfo(cl_kernel, cl_device_id, cl_kernel_work_group_info, size_t,
                                void *, size_t *);
cl_int clSetKernelArg(cl_kernel, cl_uint, size_t, const void *);
cl_int clEnqueueNDRangeKernel(cl_command_queue, cl_kernel, cl_uint, const size_t *,
                              const size_t *, const size_t *, cl_uint, const cl_event *,
                              cl_event *);
cl_int clEnqueueWriteBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t, const void *,
                            cl_uint, const cl_event *, cl_event *);
cl_int clEnqueueReadBuffer(cl_command_queue, cl_mem, cl_bool, size_t, size_t, void *,
                           cl_uint, const cl_event *, cl_event *);
cl_int clGetEventProfilingInfo(cl_event, cl_profiling_info, size_t, void *, size_t *);
cl_int clFinish(cl_command_queue);
cl_int clReleaseMemObject(cl_mem);
cl_int clReleaseKernel(cl_kernel);
cl_int clReleaseProgram(cl_program);
cl_int clReleaseCommandQueue(cl_command_queue);
cl_int clReleaseContext(cl_context);

#ifdef __cplusplus
}
#endif

#endif
