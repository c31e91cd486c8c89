/*
 * aclfft_ops.h - the reference's per-operator direct entries.
 *
 * The reference exports, next to the plan API, one entry per Ascend kernel
 * family (src/fft1_d/fft1_d.h, src/rfft1_d/rfft1_d.h, src/irfft1_d/irfft1_d.h,
 * src/fft2_d/fft2_d.h).  Its own C++ operator tests call them directly.  They
 * are kept here with the same names, argument orders, validation and return
 * codes; each one runs the transform on this library's GB300 kernels (a plan
 * cached per calling thread and shape), so the kernel family the name refers
 * to no longer matters, only its documented domain does.
 *
 * Common contract (as in the reference):
 *   - x / y hold interleaved complex (re, im) floats or real floats;
 *     x == y is an in-place call;
 *   - host pointers: the call copies in, computes and copies out, and returns
 *     when done (the reference's behaviour); device pointers of the current
 *     GPU are also accepted and then run asynchronously on `stream`;
 *   - `stream` is a cudaStream_t (NULL: the legacy default stream);
 *   - isForward: 1 forward (exp(-2 pi i kn/N)), 0 backward (exp(+...),
 *     unnormalised); R2C entries accept only 1, C2R entries only 0;
 *   - norm: 0 (no scaling) only, except aclfftRfft1D (0 none, 1 ortho
 *     1/sqrt(n), 2 forward 1/n);
 *   - return ACL_SUCCESS, ACL_ERROR_INVALID_PARAM for an argument outside the
 *     entry's domain or a length this library cannot transform (a prime
 *     factor above 47), ACL_ERROR_BAD_ALLOC when device memory runs out, and
 *     ACL_ERROR_INTERNAL_ERROR for any other failure.
 */
#ifndef ACLFFT_OPS_H
#define ACLFFT_OPS_H

#include <stdint.h>

#include "cann_ops_fft.h"

#ifndef ACL_SUCCESS
typedef int aclError;
#define ACL_SUCCESS 0
#define ACL_ERROR_INVALID_PARAM 100000
#define ACL_ERROR_BAD_ALLOC 200000
#define ACL_ERROR_INTERNAL_ERROR 500000
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D C2C (src/fft1_d/fft1_d.h:37-58) ---------------------------------- */
/* n in [1, 1024]; batches in [1, INT32_MAX]   (src/fft1_d/arch32/dft/fft1_d_dft.cpp:79-125) */
ACLFFT_API aclError aclfftFft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream);
/* n a power of two in [64, 2^27]              (src/fft1_d/arch32/fft_n/fft1_d_n.cpp:208-250) */
ACLFFT_API aclError aclfftFft1DN(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                 void* stream);
/* VERTICAL: transform down the columns of one n x stride matrix (column b is
 * transform b); batches must be 1, stride a multiple of 4, n * stride <=
 * 2^30, n a power of two in [256, 2^18]     (src/fft1_d/arch32/fft_stride/fft1_d_stride.cpp:46-100,
 *                                              src/fft1_d/arch32/fft1_d_exec_api.cpp:88-99) */
ACLFFT_API aclError aclfftFft1DStride(float* x, float* y, uint32_t n, int32_t norm, uint32_t stride, uint32_t batches,
                                      int isForward, void* stream);
/* n a power of two in [256, 16384]            (src/fft1_d/arch32/fft_b/fft1_d_b.cpp:27-48,199-215) */
ACLFFT_API aclError aclfftFft1DB(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                 void* stream);
/* n in [1, 2^27]                              (src/fft1_d/arch32/fft_mix/fft1_d_mix.cpp:23-65,190) */
ACLFFT_API aclError aclfftFft1DMix(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream);
/* n in [1, 2^27]                              (src/fft1_d/arch35/fft/fft1_d_c2c.cpp:138-175) */
ACLFFT_API aclError aclfftFft1DC2C(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream);
/* n in [1, 2^27]                              (src/fft1_d/arch35/mix/fft1_d_c2c_mix.cpp:127-165) */
ACLFFT_API aclError aclfftFft1DC2CMix(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                      void* stream);

/* ---- 1D R2C (src/rfft1_d/rfft1_d.h:47-74): n reals in, n/2+1 bins out ----- */
/* n in [1, 4096], norm 0/1/2, no isForward    (src/rfft1_d/arch35/fast_dft/rfft1_d_fast_dft.cpp:29,165-200) */
ACLFFT_API aclError aclfftRfft1D(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, void* stream);
/* n in [1, 2^27]                              (src/rfft1_d/arch32/r2c_fft/rfft1_d_r2c_fft.cpp:86-127,159) */
ACLFFT_API aclError aclfftRfft1DR2CFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                       void* stream);
/* n in [1, 2^27]                              (src/rfft1_d/arch35/fft/rfft1_d_fft.cpp:151-190) */
ACLFFT_API aclError aclfftRfft1DFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                    void* stream);
/* n in [1, 1024]; batches <= INT32_MAX        (src/rfft1_d/arch32/dft/rfft1_d_dft.cpp:45-90) */
ACLFFT_API aclError aclfftRfft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                    void* stream);
/* Power-of-two families (src/rfft1_d/arch32/rfft1_d_r2c_host_common.h:318-343):
 * n a power of two, batches * (n + 2) <= 2^31, and per family
 *   Fft1: n >= 2 (src/rfft1_d/arch32/r2c_fft1/rfft1_d_r2c_fft1.cpp:82-90)
 *   Fft2: 128 < n <= 16384 (src/rfft1_d/arch32/r2c_fft2/rfft1_d_r2c_fft2.cpp:90-100)
 *   Fft5: n >= 4 (src/rfft1_d/arch32/r2c_fft5/rfft1_d_r2c_fft5.cpp:48-60) */
ACLFFT_API aclError aclfftRfft1DR2CFft1(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);
ACLFFT_API aclError aclfftRfft1DR2CFft2(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);
ACLFFT_API aclError aclfftRfft1DR2CFft31(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);
ACLFFT_API aclError aclfftRfft1DR2CFft32(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);
ACLFFT_API aclError aclfftRfft1DR2CFft4(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);
ACLFFT_API aclError aclfftRfft1DR2CFft5(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream);

/* ---- 1D C2R (src/irfft1_d/irfft1_d.h:32-39): n/2+1 bins in, n reals out, no 1/n */
/* n in [1, 2^27]                              (src/irfft1_d/arch35/fft/irfft1_d_fft.cpp:125-160) */
ACLFFT_API aclError aclfftIrfft1DFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                     void* stream);
/* n in [1, 1024]; batches <= INT32_MAX        (src/irfft1_d/arch32/dft/irfft1_d_dft.cpp:58-100) */
ACLFFT_API aclError aclfftIrfft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                     void* stream);
/* n in [1, 2^27]                              (src/irfft1_d/arch32/c2r_fft/irfft1_d_c2r_fft.cpp:123-165,196) */
ACLFFT_API aclError aclfftIrfft1DC2RFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                        void* stream);

/* ---- 2D C2C (src/fft2_d/fft2_d.h:27): batches of fftX x fftY (fftY fastest),
 * unnormalised both ways; fftX, fftY >= 1, batches in [1, INT32_MAX]
 *                                             (src/fft2_d/arch32/dd/fft2_d_dd.cpp:68-110) */
ACLFFT_API aclError aclfftFft2DDd(float* x, float* y, uint32_t fftX, uint32_t fftY, uint32_t batches, int isForward,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ACLFFT_OPS_H */
