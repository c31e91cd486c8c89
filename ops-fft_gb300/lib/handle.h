// handle.h - the plan object behind aclfftHandle.
//
// The reference keeps only the transform description in the handle
// (lib/fft_handle_impl.h:23-59).  Those fields are kept with the same names
// and defaults; the GB300 plan additionally owns its device state: the FP32
// twiddle blob generated on the GPU, the kernel step lists for each call
// variant, the workspace and (lazily) host-staging buffers.
#pragma once
#include <cuda_runtime_api.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "../../include/aclfft_ext.h"
#include "../../include/cann_ops_fft.h"
#include "planner.h"

struct aclfftHandle_t;

namespace gfft {

struct PlanImpl {
    Problem prob{};
    // step lists: [0] primary out-of-place, [1] primary in-place,
    //             [2] adjoint out-of-place, [3] adjoint in-place
    StepList lists[4];
    TwiddleBuilder tb;
    int64_t ws_bytes = 0, ws2_bytes = 0;
    // device state (created at plan time when a device is present)
    bool device_ready = false;
    int device = -1;
    void* tw = nullptr;
    void* ws = nullptr;
    void* ws2 = nullptr;
    // workspace ownership: with auto allocation (the default) the plan
    // allocates ws/ws2 itself; otherwise they point into the caller's work
    // area (aclfftSetWorkArea), or are NULL until one is set
    bool auto_ws = true;
    void* user_ws = nullptr;
    int* err = nullptr;  // device error word written by bounded waits
    // host staging (allocated on the first exec with host pointers)
    void* stage_a = nullptr;
    void* stage_b = nullptr;
    size_t stage_bytes = 0;
    // chunked host pipeline (created on the first exec with host buffers)
    bool pipe_ready = false;
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_start = nullptr;
    static constexpr int kMaxHostChunks = 32;
    cudaEvent_t ev_in[kMaxHostChunks] = {};
    cudaEvent_t ev_k[kMaxHostChunks] = {};
};

void plan_impl_free(PlanImpl* p);
// Rebuilds a made plan after a setting that changes its steps; the old
// state is kept on failure.
aclfftResult replan(aclfftHandle_t* h);
aclfftResult plan_device_setup(PlanImpl* p);

void set_last_error(const std::string& s);
bool log_enabled();

// cudaMalloc behind a failure-injection hook (aclfftDebugFailAllocations):
// every device allocation of the library goes through here.
cudaError_t dev_alloc(void** p, size_t bytes);

// Bytes of the caller-provided work area a plan needs: ws, then ws2 at a
// 256-byte aligned offset.
size_t work_area_bytes(const PlanImpl* p);
size_t ws2_offset(const PlanImpl* p);
// Points the plan's workspaces into a caller-owned area (NULL unbinds),
// freeing any workspace the plan allocated itself.
void bind_work_area(PlanImpl* p, void* area);
void release_workspace(PlanImpl* p);
aclfftResult allocate_workspace(PlanImpl* p);
// Work area of a transform description without creating any device state
// (aclfftGetSize1d/2d).
aclfftResult estimate_work_area(const aclfftHandle_t* desc, size_t* bytes);

// Plans the handle's transform on the host with the handle's hints (no
// device state); NULL on failure with the reason in *why.
PlanImpl* plan_steps(const aclfftHandle_t* h, aclfftResult* why);

// Launches the out-of-place primary step list of a device-ready plan on
// `st` (forward direction, no scaling); 0 or a CUDA error.
int launch_primary(PlanImpl* impl, void* in, void* out, cudaStream_t st);

// Times the planner's candidate choices for a made plan and re-plans it
// with the fastest (aclfftSetAutotune).
aclfftResult autotune_plan(aclfftHandle_t* h);

}  // namespace gfft

struct aclfftHandle_t {
    int32_t rank;
    int32_t lengths[3];
    int32_t stride[3];
    int32_t batch;
    aclfftType type;
    int32_t normMode;
    cudaStream_t stream;
    bool is_initialized;
    gfft::PlanImpl* impl;
    int32_t precision;    // aclfftPrecisionMode (extension)
    bool auto_allocate;   // aclfftSetAutoAllocation (default: the plan allocates its workspace)
    int32_t autotune;     // aclfftSetAutotune: 0 off, 1 tune when made
    gfft::PlanHints hints;  // planner choices (defaults, or the autotuner's)
    int32_t tuned;        // 1 when `hints` came from the autotuner (timed or cached)
    int32_t tune_candidates;  // candidates timed by the last tuning (0: cache hit)

    aclfftHandle_t()
        : rank(0), lengths{0, 0, 0}, stride{0, 0, 0}, batch(1), type(ACLFFT_C2C), normMode(0), stream(nullptr),
          is_initialized(false), impl(nullptr), precision(0), auto_allocate(true), autotune(0), tuned(0),
          tune_candidates(0)
    {
    }
    ~aclfftHandle_t()
    {
        if (impl) {
            gfft::plan_impl_free(impl);
            delete impl;
        }
    }
};

#define GFFT_LOG(...)                                   \
    do {                                                \
        if (gfft::log_enabled()) {                      \
            std::fprintf(stderr, "[ops-fft] ");         \
            std::fprintf(stderr, __VA_ARGS__);          \
            std::fprintf(stderr, "\n");                 \
        }                                               \
    } while (0)

#define ACLFFT_CHECK_PARAM(cond, code) \
    do {                               \
        if (!(cond)) return (code);    \
    } while (0)
#define ACLFFT_CHECK_NULL(p) ACLFFT_CHECK_PARAM((p) != nullptr, ACLFFT_INVALID_VALUE)
