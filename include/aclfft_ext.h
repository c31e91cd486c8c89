/*
 * aclfft_ext.h - GB300 extensions to the aclfft C API.
 *
 * Everything here is new relative to the reference (which has no adjoints,
 * no configurable normalisation, no precision modes and no plan
 * introspection); the reference-compatible surface is cann_ops_fft.h.
 */
#ifndef ACLFFT_EXT_H
#define ACLFFT_EXT_H

#include "cann_ops_fft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Library version reported by aclfftGetVersion (MAJOR*10000 + MINOR*100 +
 * PATCH) and aclfftGetProperty. */
#define ACLFFT_GB300_VERSION_MAJOR 1
#define ACLFFT_GB300_VERSION_MINOR 1
#define ACLFFT_GB300_VERSION_PATCH 0
#define ACLFFT_GB300_VERSION \
    (ACLFFT_GB300_VERSION_MAJOR * 10000 + ACLFFT_GB300_VERSION_MINOR * 100 + ACLFFT_GB300_VERSION_PATCH)

/* Normalisation.  The reference fixes normMode = 0 (lib/fft_handle_impl.h:36):
 * neither direction is scaled.  The other modes scale by the total number
 * of points n of one transform (nx for 1D, nx*ny for 2D). */
typedef enum aclfftNormMode_t {
    ACLFFT_NORM_NONE = 0,     /* reference behaviour: no scaling */
    ACLFFT_NORM_BACKWARD = 1, /* backward (and C2R) scaled by 1/n */
    ACLFFT_NORM_ORTHO = 2,    /* both directions scaled by 1/sqrt(n) */
    ACLFFT_NORM_FORWARD = 3   /* forward (and R2C) scaled by 1/n */
} aclfftNormMode;

/* Sets the plan's normalisation (before or after MakePlan).  Returns
 * ACLFFT_INVALID_VALUE for an unknown mode, ACLFFT_INVALID_PLAN for NULL. */
ACLFFT_API aclfftResult aclfftSetNormMode(aclfftHandle plan, int normMode);
ACLFFT_API aclfftResult aclfftGetNormMode(aclfftHandle plan, int* normMode);

/* Arithmetic of the C2C DFT stages.  ACLFFT_PREC_FP32 (default) runs the
 * FP32 Stockham kernels.  The split-precision forms run the on-chip
 * 64- and 256-point sub-transforms as tensor-core DFT-matrix stages (8- and
 * 16-point real-embedded DFT matrices on tcgen05) with both the data and the
 * matrices split into hi + lo parts of the operand type and three products
 * accumulated in FP32: TF32x3 keeps plain-FP32 accuracy, BF16x3 about 1e-5
 * relative.  They apply to 1D HORIZONTAL C2C plans of length 64, 256, or a
 * product of two of {64, 256} (4096, 16384, 65536); other plans keep the
 * FP32 kernels (aclfftGetPlanInfo reports which ran via tc_stages).
 * Settable before or after MakePlan (a made plan is re-planned; returns
 * ACLFFT_ALLOC_FAILED / ACLFFT_SETUP_FAILED if that fails, leaving the old
 * plan in place).  The mode is not part of the reference API. */
typedef enum aclfftPrecisionMode_t {
    ACLFFT_PREC_FP32 = 0,
    ACLFFT_PREC_TF32X3 = 1,
    ACLFFT_PREC_BF16X3 = 2
} aclfftPrecisionMode;

ACLFFT_API aclfftResult aclfftSetPrecisionMode(aclfftHandle plan, int mode);
ACLFFT_API aclfftResult aclfftGetPrecisionMode(aclfftHandle plan, int* mode);

/* Adjoint (vector-Jacobian) transforms, using the complex-gradient convention
 * g = dL/dRe + i dL/dIm.  Same pointer and stream semantics as the Exec
 * calls; the plan's normalisation scale carries over unchanged.
 *   C2C: the adjoint of direction d is the transform of direction -d.
 *   R2C: gradIn[n] = Re sum_{k<=N/2} gradOut[k] exp(+2 pi i k n / N), i.e. a
 *        C2R of gradOut with interior bins halved.
 *   C2R: gradIn[k] = w_k * R2C(gradOut)[k], w = 1 at DC and Nyquist, 2 on
 *        interior bins. */
ACLFFT_API aclfftResult aclfftExecC2CAdjoint(aclfftHandle plan, aclfftComplex* gradOut, aclfftComplex* gradIn,
                                             int direction);
ACLFFT_API aclfftResult aclfftExecR2CAdjoint(aclfftHandle plan, aclfftComplex* gradOut, aclfftReal* gradIn);
ACLFFT_API aclfftResult aclfftExecC2RAdjoint(aclfftHandle plan, aclfftReal* gradOut, aclfftComplex* gradIn);

/* Weighted R2C adjoint (no counterpart in the reference): gradIn = the R2C
 * adjoint of (weights * gradOut), weights real with the layout of the
 * transform's output ([batch][nx/2+1] floats), multiplied in as the bins are
 * loaded instead of by a separate elementwise pass.  For the loss
 * sum(w*|X|^2) of X = R2C(x), gradOut = X and weights = 2w give dL/dx in one
 * launch.  Device pointers only, out of place, asynchronous on the plan's
 * stream; results are identical to scaling gradOut first and calling
 * aclfftExecR2CAdjoint.  Available for even nx whose adjoint runs as one
 * specialised row launch (aclfftGetPlanInfo: nsteps == 1 and kernel >= 0;
 * e.g. nx = 1024, 2048, 3000, 4096, 8192; longer even lengths run on
 * thread-block clusters or column passes);
 * ACLFFT_NOT_IMPLEMENTED otherwise. */
ACLFFT_API aclfftResult aclfftExecR2CAdjointWeighted(aclfftHandle plan, const aclfftComplex* gradOut,
                                                     const aclfftReal* weights, aclfftReal* gradIn);

/* Plan introspection (for tests and tooling). */
typedef struct aclfftPlanInfo_t {
    int supported;        /* 1 when the plan can execute on the GPU */
    int nsteps;           /* kernel launches per out-of-place exec */
    int nradix;           /* passes of the first on-chip transform */
    int radix[12];        /* their radices */
    int onchip_length;    /* length of the first on-chip transform */
    int threads_per_transform;
    int transforms_per_cta;
    long long twiddle_entries; /* complex entries generated on the GPU */
    size_t workspace_bytes;    /* device workspace owned by the plan */
    int kernel;                /* first step: -1 generic row/column kernel, >= 0 specialised codelet id */
    int groups_per_cta;        /* codelets: independent transform groups per CTA */
    int stages;                /* input prefetch stages */
    int smem_bytes;            /* dynamic shared memory per CTA */
    int tc_stages;             /* tensor-core DFT-matrix launches per exec (0: FP32 kernels only) */
    int cluster_ctas;          /* CTAs per thread-block cluster of a cluster transform (0: none) */
    int cluster_count;         /* clusters resident at once on the plan's device (0: not prepared) */
    int tuned;                 /* 1 when the launches were chosen by the autotuner (timed or cached) */
    int tune_candidates;       /* distinct candidates the last tuning timed (0: taken from the cache) */
} aclfftPlanInfo;

ACLFFT_API aclfftResult aclfftGetPlanInfo(aclfftHandle plan, aclfftPlanInfo* info);

/* Autotuning (no counterpart in the reference, whose radix choices are
 * fixed tables).  mode 1 times the planner's candidate choices for this
 * plan - every specialised row-kernel build of its length, their transform
 * groups per CTA and prefetch stages, the thread-block-cluster sizes and
 * cluster-or-row-kernel for 4096-point transforms, no specialised kernels -
 * on scratch buffers of the plan's shape (batch capped at 256 MB of input)
 * and re-plans with the fastest; the planner's own choice is kept unless
 * another is at least 2 % faster.  Called on a made plan it tunes at once,
 * before MakePlan it makes MakePlan tune (OPS_FFT_AUTOTUNE=1 does this for
 * every plan).  Needs a device; allocates scratch for the duration, so call
 * it outside stream capture.  Choices are cached per (device, type, lengths,
 * batch, layout) for the process and in the file named by
 * OPS_FFT_PLAN_TUNE_CACHE (a damaged line is ignored).  Split-precision
 * and VERTICAL plans have nothing to tune.  mode 0 (default) plans by the
 * static rules. */
ACLFFT_API aclfftResult aclfftSetAutotune(aclfftHandle plan, int mode);

/* Copies the plan's FP32 twiddle blob (as generated on the GPU) to host
 * memory: at most maxEntries complex values; *entries receives the total. */
ACLFFT_API aclfftResult aclfftGetTwiddles(aclfftHandle plan, aclfftComplex* host, long long maxEntries,
                                          long long* entries);

/* Layout of the twiddle blob returned by aclfftGetTwiddles (for tests):
 * per segment five values {offset, count, M, param, kind}; entry i of the
 * segment (at blob index offset + i) is exp(-2 pi i m / M) evaluated in
 * FP64 and rounded to FP32, with m = (i / param) * (i % param) mod M for a
 * pass table (kind 2, layout [r][k] with param = k's extent) and
 * m = i * param mod M for a linear table (kind 1); kind 3 segments hold
 * tensor-core DFT-matrix operand images.  Writes at most maxSegs segments;
 * *nsegs receives the total. */
ACLFFT_API aclfftResult aclfftDebugGetTwiddleSegments(aclfftHandle plan, long long* segs, int maxSegs, int* nsegs);

/* Allocation-free long C2C (no counterpart in the reference).  For callers
 * that cannot allocate device memory - code running while another component
 * owns the device memory pool, or that must avoid cudaMalloc/cudaFree and
 * the synchronisation they may cause.  No plan object: the transform of
 * `batch` contiguous rows of length nx (nx = L1 * L2, both factors <= 2048
 * with prime factors <= 47) runs as two column passes whose intermediate is
 * a fixed 16 MiB device array built into the library, so nx * batch must not
 * exceed 2^21 (ACLFFT_INVALID_SIZE otherwise).  idata/odata are device
 * pointers; the call is asynchronous on `stream` and unscaled.  The fixed
 * arrays are shared by all calls on a device: calls that overlap on the GPU
 * race.  The first call on each device looks up the arrays' device addresses
 * (cudaGetSymbolAddress) and should therefore come before any stream
 * capture. */
ACLFFT_API aclfftResult aclfftExecC2CNoAlloc(const aclfftComplex* idata, aclfftComplex* odata, int nx, int batch,
                                             int direction, cudaStream_t stream);

/* Ragged batches (no counterpart in the reference, which runs one exec per
 * (length, kind) plan): `count` 1D transforms of different lengths and kinds
 * executed by ONE persistent kernel launch driven by a device work-descriptor
 * table.  Transform i is C2C or R2C (types[i]) of length lengths[i] (2 ..
 * 2^24, prime factors <= 13); its input starts inOffsets[i] bytes and its
 * output outOffsets[i] bytes after the pointers given to aclfftRaggedExec
 * (both offsets multiples of 8; C2C: n complex in and out; R2C: n reals in,
 * n/2 + 1 complex out).  Lengths above 4096 (complex) run as two dependent
 * steps inside the same launch using a plan-owned workspace.  Per (kind,
 * length) the radix order and threads per transform come from an autotuner
 * (timed candidates, cached per process and in the file named by
 * OPS_FFT_TUNE_CACHE) that runs on the first exec unless disabled.  Execs
 * replay a CUDA graph captured per (input, output, direction); inside a
 * caller's stream capture they are recorded into that capture instead.
 * Unnormalised; direction applies to the C2C transforms (R2C transforms are
 * always forward). */
typedef struct aclfftRaggedPlan_t* aclfftRaggedPlan;

typedef struct aclfftRaggedInfo_t {
    int transforms;
    int classes;          /* distinct (kind, length) */
    int long_transforms;  /* transforms run as two dependent steps */
    int items;            /* work items per exec */
    int tuned_classes;    /* classes whose plan came from the autotuner */
    int graph;            /* 1 when execs replay a captured CUDA graph */
    int smem_bytes;       /* shared memory per CTA */
    long long twiddle_entries;
    size_t workspace_bytes;
    size_t in_bytes_min;  /* input extent implied by the offsets */
    size_t out_bytes_min; /* output extent implied by the offsets */
} aclfftRaggedInfo;

ACLFFT_API aclfftResult aclfftRaggedPlanCreate(aclfftRaggedPlan* plan, int count, const int* lengths,
                                               const aclfftType* types, const long long* inOffsets,
                                               const long long* outOffsets);
ACLFFT_API aclfftResult aclfftRaggedSetStream(aclfftRaggedPlan plan, cudaStream_t stream);
/* autotune: tune on the first exec (default 1); useGraph: replay a captured
 * CUDA graph (default 1). */
ACLFFT_API aclfftResult aclfftRaggedSetOptions(aclfftRaggedPlan plan, int autotune, int useGraph);
ACLFFT_API aclfftResult aclfftRaggedAutotune(aclfftRaggedPlan plan);
/* idata/odata: device pointers; asynchronous on the plan's stream. */
ACLFFT_API aclfftResult aclfftRaggedExec(aclfftRaggedPlan plan, void* idata, void* odata, int direction);
ACLFFT_API aclfftResult aclfftRaggedGetInfo(aclfftRaggedPlan plan, aclfftRaggedInfo* info);
/* Device error flags of the plan's launches (bit 2: a dependency wait ran
 * out of time, the items behind it were skipped and the output is
 * incomplete).  Synchronises the plan's stream, stores the flags in *flags,
 * clears them and returns ACLFFT_EXEC_FAILED when any was set. */
ACLFFT_API aclfftResult aclfftRaggedGetError(aclfftRaggedPlan plan, int* flags);
/* Upper bound, in SM clock cycles, of each dependency wait inside the
 * ragged kernel (default 2^31, about a second; must be > 0).  Takes effect
 * at the next exec. */
ACLFFT_API aclfftResult aclfftRaggedSetWaitLimit(aclfftRaggedPlan plan, long long cycles);
/* Test hook: every dependency wait of the next execs waits for `extra` more
 * completed items than exist (0 restores normal operation), so a wait runs
 * out of time by construction and the failure path can be exercised without
 * faulting the GPU. */
ACLFFT_API aclfftResult aclfftRaggedDebugHoldDependencies(aclfftRaggedPlan plan, int extra);
ACLFFT_API aclfftResult aclfftRaggedDestroy(aclfftRaggedPlan plan);
/* Host replay of every work item's index ranges (0 = all in bounds). */
ACLFFT_API int aclfftRaggedDebugCheck(aclfftRaggedPlan plan, char* msg, int msglen);

/* Replays the address arithmetic of every launch the plan can make against
 * the buffer sizes of each call variant (no kernel runs).  Returns 0 when
 * all launches stay in bounds; msg receives a description. */
ACLFFT_API int aclfftDebugCheckPlan(aclfftHandle plan, char* msg, int msglen);

/* Device-side failure reporting (no counterpart in the reference, whose
 * execs are synchronous and map a failed kernel to ACLFFT_EXEC_FAILED,
 * src/fft1_d/arch32/fft1_d_exec_api.cpp:148-152).  Every wait inside the
 * kernels is bounded; a wait that runs out sets a bit in the plan's device
 * error word and the kernel returns early, leaving the output incomplete:
 *   bit 0  row kernel: an input copy did not arrive
 *   bit 1  tensor-core stage: an MMA did not complete
 *   bit 3  cluster kernel: a distributed-shared-memory exchange did not arrive
 * Execs on host buffers read the word before returning (they synchronise
 * anyway) and return ACLFFT_EXEC_FAILED when a bit is set.  Execs on device
 * buffers are asynchronous: aclfftGetExecError synchronises the plan's
 * stream, stores the word in *flags, clears it and returns
 * ACLFFT_EXEC_FAILED when it was non-zero (ACLFFT_SUCCESS otherwise).  The
 * word accumulates over execs until it is read. */
ACLFFT_API aclfftResult aclfftGetExecError(aclfftHandle plan, int* flags);
/* Test hook: overwrites the plan's device error word with `flags` (on the
 * plan's stream, synchronously), as a kernel whose wait ran out would. */
ACLFFT_API aclfftResult aclfftDebugSetExecError(aclfftHandle plan, int flags);

/* Test hook for allocation failures: after `after` more successful device
 * allocations (after >= 0) every device allocation the library makes fails
 * as if cudaMalloc had run out of memory, so that ACLFFT_ALLOC_FAILED paths
 * can be exercised; a negative value switches the hook off (the default).
 * Process-wide. */
ACLFFT_API aclfftResult aclfftDebugFailAllocations(int after);

/* Test hook: the in-register butterfly of radix R (1 <= R <= 48) that the
 * kernels use, evaluated on the host (the same operation sequence and
 * rounding as the device's paired FP32 instructions): in and out hold R
 * interleaved complex values (forward DFT, natural order).  Returns
 * ACLFFT_INVALID_SIZE for other R. */
ACLFFT_API aclfftResult aclfftDebugButterfly(int R, const float* in, float* out);

/* Human-readable reason of the last failure on this thread ("" if none). */
ACLFFT_API const char* aclfftGetLastErrorDetail(void);

#ifdef __cplusplus
}
#endif

#endif /* ACLFFT_EXT_H */
