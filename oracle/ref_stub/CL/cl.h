/*
 * Inert stand-in for <CL/cl.h> -- oracle build only.
 *
 * The reference's src/tools.h includes <CL/cl.h> and src/tools.cpp carries
 * OpenCL platform helpers next to the CPU code the oracle needs (load,
 * calculate_rmse_directly, cdmf_ref).  This image has no OpenCL headers or
 * ICD, so this header declares just enough types and entry points for those
 * two files to compile.  Every entry point reports "no platform"; the oracle
 * never calls them.
 */
#ifndef CDMF_ORACLE_CL_STUB_H
#define CDMF_ORACLE_CL_STUB_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef uint64_t cl_ulong;
typedef int8_t cl_char;
typedef cl_uint cl_bool;
typedef cl_ulong cl_bitfield;
typedef cl_bitfield cl_device_type;
typedef cl_uint cl_platform_info;
typedef cl_uint cl_device_info;
typedef cl_uint cl_profiling_info;
typedef struct _cl_platform_id *cl_platform_id;
typedef struct _cl_device_id *cl_device_id;
typedef struct _cl_event *cl_event;

#define CL_SUCCESS 0
#define CL_DEVICE_NOT_FOUND -1
#define CL_DEVICE_TYPE_CPU (1 << 1)
#define CL_DEVICE_TYPE_GPU (1 << 2)
#define CL_DEVICE_TYPE_ACCELERATOR (1 << 3)
#define CL_DEVICE_TYPE_ALL 0xFFFFFFFF
#define CL_PLATFORM_PROFILE 0x0900
#define CL_PLATFORM_VERSION 0x0901
#define CL_PLATFORM_NAME 0x0902
#define CL_PLATFORM_VENDOR 0x0903
#define CL_PLATFORM_EXTENSIONS 0x0904
#define CL_DEVICE_MAX_COMPUTE_UNITS 0x1002
#define CL_DEVICE_NAME 0x102B
#define CL_DEVICE_VENDOR 0x102C
#define CL_DRIVER_VERSION 0x102D
#define CL_DEVICE_PROFILE 0x102E
#define CL_DEVICE_VERSION 0x102F
#define CL_DEVICE_EXTENSIONS 0x1030
#define CL_DEVICE_OPENCL_C_VERSION 0x103D
#define CL_PROFILING_COMMAND_START 0x1282
#define CL_PROFILING_COMMAND_END 0x1283

static inline cl_int clGetPlatformIDs(cl_uint, cl_platform_id *, cl_uint *n) {
    if (n) *n = 0;
    return CL_DEVICE_NOT_FOUND;
}
static inline cl_int clGetPlatformInfo(cl_platform_id, cl_platform_info, size_t, void *, size_t *s) {
    if (s) *s = 0;
    return CL_DEVICE_NOT_FOUND;
}
static inline cl_int clGetDeviceIDs(cl_platform_id, cl_device_type, cl_uint, cl_device_id *, cl_uint *n) {
    if (n) *n = 0;
    return CL_DEVICE_NOT_FOUND;
}
static inline cl_int clGetDeviceInfo(cl_device_id, cl_device_info, size_t, void *, size_t *s) {
    if (s) *s = 0;
    return CL_DEVICE_NOT_FOUND;
}
static inline cl_int clGetEventProfilingInfo(cl_event, cl_profiling_info, size_t, void *, size_t *) {
    return CL_DEVICE_NOT_FOUND;
}
#ifdef __cplusplus
}
#endif
#endif
