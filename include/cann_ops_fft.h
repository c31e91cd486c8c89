/*
 * cann_ops_fft.h - public C API of the GB300 (sm_103a) aclfft library.
 *
 * Drop-in replacement for the ops-fft public header (include/cann_ops_fft.h of
 * the reference).  Symbol names, enum values, struct layouts and argument
 * orders are kept identical so that code written against the reference links
 * against libops_fft.so unchanged.  The one type change is the stream:
 * aclfftSetStream takes a cudaStream_t (the reference takes an aclrtStream,
 * include/cann_ops_fft.h:429).
 *
 * Pointer semantics (deliberate divergence, see aclfftExecC2C below):
 *   - device or managed pointers: the transform is enqueued on the plan's
 *     stream and the call returns without synchronising (cuFFT style, can be
 *     captured in a CUDA graph);
 *   - host pointers (pageable or pinned): the library stages the data through
 *     device memory owned by the plan and synchronises the plan's stream
 *     before returning, which is the reference's "return means done"
 *     contract for host buffers.
 */
#ifndef CANN_OPS_FFT_H
#define CANN_OPS_FFT_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime_api.h>

#if defined(_WIN32) || defined(__CYGWIN__)
#define ACLFFT_API __declspec(dllexport)
#else
#define ACLFFT_API __attribute__((visibility("default")))
#endif

/* Result codes.  Values match include/cann_ops_fft.h:32-66 of the reference
 * (15 is unused there as well). */
typedef enum aclfftResult_t {
    ACLFFT_SUCCESS = 0,
    ACLFFT_INVALID_PLAN = 1,
    ACLFFT_ALLOC_FAILED = 2,
    ACLFFT_INVALID_TYPE = 3,
    ACLFFT_INVALID_VALUE = 4,
    ACLFFT_INTERNAL_ERROR = 5,
    ACLFFT_EXEC_FAILED = 6,
    ACLFFT_SETUP_FAILED = 7,
    ACLFFT_INVALID_SIZE = 8,
    ACLFFT_UNALIGNED_DATA = 9,
    ACLFFT_INCOMPLETE_PARAMETER_LIST = 10,
    ACLFFT_INVALID_DEVICE = 11,
    ACLFFT_PARSE_ERROR = 12,
    ACLFFT_NO_WORKSPACE = 13,
    ACLFFT_NOT_IMPLEMENTED = 14,
    ACLFFT_NOT_SUPPORTED = 16
} aclfftResult;

/* Transform types, include/cann_ops_fft.h:80-94 of the reference. */
typedef enum aclfftType_t {
    ACLFFT_R2C = 0x2a,
    ACLFFT_C2R = 0x2c,
    ACLFFT_C2C = 0x29,
    ACLFFT_D2Z = 0x6a,
    ACLFFT_Z2D = 0x6c,
    ACLFFT_Z2Z = 0x69
} aclfftType;

typedef enum aclfftLibraryPropertyType_t {
    ACLFFT_MAJOR_VERSION,
    ACLFFT_MINOR_VERSION,
    ACLFFT_PATCH_LEVEL
} aclfftLibraryPropertyType;

/* Direction: forward is exp(-2*pi*i*k*n/N), backward exp(+2*pi*i*k*n/N).
 * Neither is scaled by default (the backward result is N * ifft). */
#define ACLFFT_FORWARD (-1)
#define ACLFFT_BACKWARD 1

/* 1D layout: HORIZONTAL = one transform per contiguous row;
 * VERTICAL = transforms run down the columns of a row-major (nx, batch)
 * array, consecutive samples of one transform are `batch` elements apart. */
#define ACLFFT_HORIZONTAL 0
#define ACLFFT_VERTICAL 1

typedef struct aclfftHandle_t* aclfftHandle;

typedef struct {
    float x; /* real */
    float y; /* imaginary */
} aclfftComplex;

typedef struct {
    double x;
    double y;
} aclfftDoubleComplex;

typedef float aclfftReal;
typedef double aclfftDoubleReal;

#ifdef __cplusplus
extern "C" {
#endif

/* Plan creation.  Validation order and error codes follow
 * lib/fft_plan_api.cpp:47-85 (1D) and :90-122 (2D) of the reference. */
ACLFFT_API aclfftResult aclfftPlan1d(aclfftHandle* plan, int nx, aclfftType type, int batch, int dimType);
ACLFFT_API aclfftResult aclfftPlan2d(aclfftHandle* plan, int batch, int nx, int ny, aclfftType type);
ACLFFT_API aclfftResult aclfftPlan3d(aclfftHandle* plan, int nx, int ny, int nz, aclfftType type);
ACLFFT_API aclfftResult aclfftCreate(aclfftHandle* plan);

/* Plan initialisation (lib/fft_plan_init_api.cpp:118-176, :189-236).
 * Here it also factorises the length, generates the FP64-accurate twiddle
 * tables on the GPU and reports the device workspace the plan owns. */
ACLFFT_API aclfftResult aclfftMakePlan1d(aclfftHandle plan, int nx, aclfftType type, int batch, int dimType,
                                         size_t* workSize);
ACLFFT_API aclfftResult aclfftMakePlan2d(aclfftHandle plan, int batch, int nx, int ny, aclfftType type,
                                         size_t* workSize);
ACLFFT_API aclfftResult aclfftMakePlan3d(aclfftHandle plan, int nx, int ny, int nz, aclfftType type,
                                         size_t* workSize);

/* Work-area queries and control: not implemented in the reference either
 * (lib/fft_utils_api.cpp:66-109); they return ACLFFT_NOT_IMPLEMENTED. */
ACLFFT_API aclfftResult aclfftGetSize1d(aclfftHandle plan, int nx, aclfftType type, int batch, size_t* workSize);
ACLFFT_API aclfftResult aclfftGetSize2d(aclfftHandle plan, int nx, int ny, aclfftType type, size_t* workSize);
ACLFFT_API aclfftResult aclfftGetSize3d(aclfftHandle plan, int nx, int ny, int nz, aclfftType type,
                                        size_t* workSize);
ACLFFT_API aclfftResult aclfftGetSize(aclfftHandle plan, size_t* workSize);
ACLFFT_API aclfftResult aclfftSetAutoAllocation(aclfftHandle plan, int autoAllocate);
ACLFFT_API aclfftResult aclfftSetWorkArea(aclfftHandle plan, void* workArea);

/* Execution (lib/fft_exec_api.cpp:32-85).  idata == odata is an in-place
 * transform; an in-place R2C needs 2*(nx/2+1)*batch floats of storage. */
ACLFFT_API aclfftResult aclfftExecC2C(aclfftHandle plan, aclfftComplex* idata, aclfftComplex* odata,
                                      int direction);
ACLFFT_API aclfftResult aclfftExecR2C(aclfftHandle plan, aclfftReal* idata, aclfftComplex* odata);
ACLFFT_API aclfftResult aclfftExecC2R(aclfftHandle plan, aclfftComplex* idata, aclfftReal* odata);

/* Double precision (stubs in the reference, lib/fft_exec_api.cpp:87-116):
 * Z2Z, D2Z and Z2D of rank 1-3 (Z2Z HORIZONTAL or VERTICAL in 1D), same
 * argument checks, layouts and pointer semantics as the FP32 entries, with
 * FP64 arithmetic and FP64 twiddles throughout. */
ACLFFT_API aclfftResult aclfftExecZ2Z(aclfftHandle plan, aclfftDoubleComplex* idata, aclfftDoubleComplex* odata,
                                      int direction);
ACLFFT_API aclfftResult aclfftExecD2Z(aclfftHandle plan, aclfftDoubleReal* idata, aclfftDoubleComplex* odata);
ACLFFT_API aclfftResult aclfftExecZ2D(aclfftHandle plan, aclfftDoubleComplex* idata, aclfftDoubleReal* odata);

/* Stream binding (lib/fft_stream_api.cpp:22-32), here a CUDA stream.
 * nullptr selects the legacy default stream. */
ACLFFT_API aclfftResult aclfftSetStream(aclfftHandle plan, cudaStream_t stream);
ACLFFT_API aclfftResult aclfftSetStride(aclfftHandle plan, int32_t stride);

/* Releases the plan and every device buffer it owns
 * (lib/fft_plan_destroy_api.cpp:24-40).  Destroying twice is undefined. */
ACLFFT_API aclfftResult aclfftDestroy(aclfftHandle plan);

ACLFFT_API aclfftResult aclfftGetVersion(int* version);
ACLFFT_API aclfftResult aclfftGetProperty(aclfftLibraryPropertyType type, int* value);

/* Static description string, "Unknown error" for unknown codes
 * (lib/fft_utils_api.cpp:19-56). */
ACLFFT_API const char* aclfftGetErrorString(aclfftResult result);

#ifdef __cplusplus
}
#endif

#endif /* CANN_OPS_FFT_H */
