// api_plan.cpp - plan creation, initialisation, stream binding, destruction.
//
// Validation order and error codes follow the reference API layer:
//   aclfftCreate       lib/fft_plan_api.cpp:24-36
//   aclfftPlan1d       lib/fft_plan_api.cpp:47-85
//   aclfftPlan2d       lib/fft_plan_api.cpp:90-122
//   aclfftPlan3d       lib/fft_plan_api.cpp:127-150
//   aclfftMakePlan1d   lib/fft_plan_init_api.cpp:118-176 (VERTICAL encodes
//                      batch = 1, stride[0] = batch, :154-159)
//   aclfftMakePlan2d   lib/fft_plan_init_api.cpp:189-236
//   size domain        lib/fft_plan_validate.h:20-47
//   overflow checks    lib/fft_plan_init_api.cpp:25-105
//   aclfftSetStream    lib/fft_stream_api.cpp:22-32
//   aclfftDestroy      lib/fft_plan_destroy_api.cpp:24-40
// Deliberate differences: MakePlan also plans the GPU execution (radix
// sequence, twiddles generated on the GPU, workspace), *workSize reports the
// workspace the plan owns, 2D plans accept any C2C size (the reference only
// has {32,64,128}^2 kernels and returns ACLFFT_NOT_SUPPORTED otherwise) and
// R2C/C2R (the reference rejects them until its 2D real path lands,
// lib/fft_plan_init_api.cpp:200-209), and 3D plans exist for every type
// (the reference's MakePlan3d returns ACLFFT_NOT_IMPLEMENTED, :250-254).  Double
// precision is planned too (the reference rejects it at plan time,
// lib/fft_plan_init_api.cpp:132-136), at every rank.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>

#include "handle.h"

using gfft::Kind;
using gfft::PlanImpl;
using gfft::Problem;

namespace {

constexpr int kHorizontalMaxN = 1 << 27;
constexpr int kVerticalMinN = 256;
constexpr int kVerticalMaxN = 1 << 18;

bool valid_type(aclfftType t)
{
    switch (t) {
    case ACLFFT_C2C:
    case ACLFFT_R2C:
    case ACLFFT_C2R:
    case ACLFFT_Z2Z:
    case ACLFFT_D2Z:
    case ACLFFT_Z2D:
        return true;
    default:
        return false;
    }
}

aclfftResult validate_1d_size(int dimType, int nx, const char* entry)
{
    if (dimType == ACLFFT_HORIZONTAL) {
        if (nx > kHorizontalMaxN) {
            GFFT_LOG("%s: nx=%d exceeds 2^27 for horizontal FFT", entry, nx);
            return ACLFFT_INVALID_SIZE;
        }
    } else {
        const bool pow2 = nx > 0 && (nx & (nx - 1)) == 0;
        if (nx < kVerticalMinN || nx > kVerticalMaxN || !pow2) {
            GFFT_LOG("%s: nx=%d out of [256, 262144] or not a power of 2 for vertical FFT", entry, nx);
            return ACLFFT_INVALID_SIZE;
        }
    }
    return ACLFFT_SUCCESS;
}

// Overflow-checked element counts of the plan's input and output.
aclfftResult check_sizes(const aclfftHandle_t* p)
{
    size_t full = 1, packed = 1, tmp = 0;
    for (int i = 0; i < p->rank; ++i)
        if (__builtin_mul_overflow(full, (size_t)p->lengths[i], &full)) return ACLFFT_INVALID_SIZE;
    if (__builtin_mul_overflow(full, (size_t)p->batch, &full)) return ACLFFT_INVALID_SIZE;
    for (int i = 0; i < p->rank - 1; ++i)
        if (__builtin_mul_overflow(packed, (size_t)p->lengths[i], &packed)) return ACLFFT_INVALID_SIZE;
    if (__builtin_mul_overflow(packed, (size_t)(p->lengths[p->rank - 1] / 2 + 1), &packed) ||
        __builtin_mul_overflow(packed, (size_t)p->batch, &packed))
        return ACLFFT_INVALID_SIZE;
    const size_t elem = (p->type == ACLFFT_Z2Z || p->type == ACLFFT_D2Z || p->type == ACLFFT_Z2D) ? 8 : 4;
    if (__builtin_mul_overflow(full, (size_t)2 * elem, &tmp) || __builtin_mul_overflow(packed, (size_t)2 * elem, &tmp))
        return ACLFFT_INVALID_SIZE;
    return ACLFFT_SUCCESS;
}

}  // namespace

namespace gfft {

// Plans every call variant of the transform described by the handle on the
// host (kernel steps, twiddle segments, workspace sizes); NULL on failure.
PlanImpl* plan_steps(const aclfftHandle_t* h, aclfftResult* why)
{
    PlanImpl* impl = new (std::nothrow) PlanImpl();
    if (!impl) {
        *why = ACLFFT_ALLOC_FAILED;
        return nullptr;
    }
    Problem pr;
    pr.rank = h->rank;
    pr.dbl = h->type == ACLFFT_Z2Z || h->type == ACLFFT_D2Z || h->type == ACLFFT_Z2D;
    pr.kind = (h->type == ACLFFT_C2C || h->type == ACLFFT_Z2Z)
                  ? Kind::C2C
                  : ((h->type == ACLFFT_R2C || h->type == ACLFFT_D2Z) ? Kind::R2C : Kind::C2R);
    pr.n0 = h->lengths[0];
    pr.n1 = h->rank >= 2 ? h->lengths[1] : 1;
    pr.n2 = h->rank == 3 ? h->lengths[2] : 1;
    pr.batch = h->batch;
    pr.stride = h->rank == 1 ? h->stride[0] : 1;
    pr.prec = pr.kind == Kind::C2C && pr.rank == 1 && !pr.dbl ? h->precision : 0;
    pr.hints = h->hints;
    impl->prob = pr;
    impl->auto_ws = h->auto_allocate;
    Problem adj = pr;
    if (pr.kind == Kind::R2C) {
        adj.kind = Kind::C2R;
        adj.weight = gfft::WEIGHT_LOAD_HALF;
    } else if (pr.kind == Kind::C2R) {
        adj.kind = Kind::R2C;
        adj.weight = gfft::WEIGHT_STORE_X2;
    }
    bool ok = true;
    for (int v = 0; v < 4 && ok; ++v) {
        int64_t ws = 0, ws2 = 0;
        ok = gfft::build_steps(v < 2 ? pr : adj, (v & 1) != 0, impl->tb, impl->lists[v], ws, ws2);
        impl->ws_bytes = std::max<int64_t>(impl->ws_bytes, ws);
        impl->ws2_bytes = std::max<int64_t>(impl->ws2_bytes, ws2);
    }
    if (!ok) {
        delete impl;
        gfft::set_last_error("internal planning failure");
        *why = ACLFFT_INTERNAL_ERROR;
        return nullptr;
    }
    return impl;
}

}  // namespace gfft

namespace {

using gfft::plan_steps;

// Plans every call variant of the transform described by the handle.
aclfftResult plan_execution(aclfftHandle_t* h, size_t* workSize)
{
    aclfftResult why = ACLFFT_SUCCESS;
    PlanImpl* impl = plan_steps(h, &why);
    if (!impl) return why;
    const aclfftResult r = gfft::plan_device_setup(impl);
    if (r != ACLFFT_SUCCESS) {
        gfft::plan_impl_free(impl);
        delete impl;
        return r;
    }
    if (h->impl) {  // re-plan of a made plan: the new state replaces the old
        // a caller's work area stays bound when it is still large enough
        if (!impl->auto_ws && h->impl->user_ws && gfft::work_area_bytes(impl) <= gfft::work_area_bytes(h->impl))
            gfft::bind_work_area(impl, h->impl->user_ws);
        gfft::plan_impl_free(h->impl);
        delete h->impl;
    }
    h->impl = impl;
    if (workSize) *workSize = gfft::work_area_bytes(impl);
    return ACLFFT_SUCCESS;
}

// MakePlan tunes when the plan asked for it (aclfftSetAutotune) or
// OPS_FFT_AUTOTUNE=1 is set; a tuning failure keeps the planner's choices.
void maybe_autotune(aclfftHandle_t* h, size_t* workSize)
{
    static const bool env_on = [] {
        const char* v = std::getenv("OPS_FFT_AUTOTUNE");
        return v && v[0] == '1';
    }();
    if (!(h->autotune || env_on)) return;
    if (gfft::autotune_plan(h) == ACLFFT_SUCCESS && workSize && h->impl) *workSize = gfft::work_area_bytes(h->impl);
}

}  // namespace

namespace gfft {

aclfftResult replan(aclfftHandle_t* h)
{
    if (!h->is_initialized || !h->impl) return ACLFFT_SUCCESS;
    const int dev = h->impl->device;
    int cur = -1;
    if (h->impl->device_ready && cudaGetDevice(&cur) == cudaSuccess && cur != dev) {
        if (cudaSetDevice(dev) != cudaSuccess) {
            cudaGetLastError();
            return ACLFFT_INVALID_DEVICE;
        }
        const aclfftResult r = plan_execution(h, nullptr);
        cudaSetDevice(cur);
        return r;
    }
    return plan_execution(h, nullptr);
}

aclfftResult estimate_work_area(const aclfftHandle_t* desc, size_t* bytes)
{
    aclfftResult why = ACLFFT_SUCCESS;
    PlanImpl* impl = plan_steps(desc, &why);
    if (!impl) return why;
    *bytes = work_area_bytes(impl);
    delete impl;
    return ACLFFT_SUCCESS;
}

size_t ws2_offset(const PlanImpl* p) { return ((size_t)p->ws_bytes + 255) & ~(size_t)255; }

size_t work_area_bytes(const PlanImpl* p)
{
    return p->ws2_bytes > 0 ? ws2_offset(p) + (size_t)p->ws2_bytes : (size_t)p->ws_bytes;
}

void release_workspace(PlanImpl* p)
{
    if (!p->user_ws) {
        if (p->ws) cudaFree(p->ws);
        if (p->ws2) cudaFree(p->ws2);
    }
    p->ws = p->ws2 = p->user_ws = nullptr;
}

void bind_work_area(PlanImpl* p, void* area)
{
    release_workspace(p);
    if (!area) return;
    p->user_ws = area;
    p->ws = p->ws_bytes > 0 ? area : nullptr;
    p->ws2 = p->ws2_bytes > 0 ? static_cast<char*>(area) + ws2_offset(p) : nullptr;
}

aclfftResult allocate_workspace(PlanImpl* p)
{
    if (p->ws_bytes > 0 && dev_alloc(&p->ws, (size_t)p->ws_bytes) != cudaSuccess) {
        cudaGetLastError();
        p->ws = nullptr;
        set_last_error("cudaMalloc of the workspace failed");
        return ACLFFT_ALLOC_FAILED;
    }
    if (p->ws2_bytes > 0 && dev_alloc(&p->ws2, (size_t)p->ws2_bytes) != cudaSuccess) {
        cudaGetLastError();
        p->ws2 = nullptr;
        release_workspace(p);
        set_last_error("cudaMalloc of the second workspace failed");
        return ACLFFT_ALLOC_FAILED;
    }
    return ACLFFT_SUCCESS;
}

void plan_impl_free(PlanImpl* p)
{
    if (!p) return;
    if (p->tw) cudaFree(p->tw);
    release_workspace(p);
    if (p->stage_a) cudaFree(p->stage_a);
    if (p->stage_b) cudaFree(p->stage_b);
    if (p->err) cudaFree(p->err);
    p->err = nullptr;
    if (p->pipe_ready) {
        cudaStreamDestroy(p->s_in);
        cudaStreamDestroy(p->s_out);
        cudaEventDestroy(p->ev_start);
        for (int c = 0; c < PlanImpl::kMaxHostChunks; ++c) {
            cudaEventDestroy(p->ev_in[c]);
            cudaEventDestroy(p->ev_k[c]);
        }
        p->pipe_ready = false;
    }
    p->tw = p->stage_a = p->stage_b = nullptr;
    p->device_ready = false;
}

// Allocates the twiddle blob and workspace on the current device and fills
// the blob with the FP64-evaluated, FP32-rounded unit roots.  Without a CUDA
// device the plan stays host-only and the setup is retried at exec time.
aclfftResult plan_device_setup(PlanImpl* p)
{
    if (p->device_ready) return ACLFFT_SUCCESS;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return ACLFFT_SUCCESS;  // deferred
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_SETUP_FAILED;
    }
    const size_t tw_bytes = (size_t)std::max<int64_t>(p->tb.count, 2) * 8;
    if (dev_alloc(&p->tw, tw_bytes) != cudaSuccess) {
        cudaGetLastError();
        p->tw = nullptr;
        set_last_error("cudaMalloc of the twiddle table failed");
        return ACLFFT_ALLOC_FAILED;
    }
    if (p->auto_ws && !p->user_ws) {
        const aclfftResult r = allocate_workspace(p);
        if (r != ACLFFT_SUCCESS) {
            plan_impl_free(p);
            return r;
        }
    }
    if (dev_alloc(reinterpret_cast<void**>(&p->err), sizeof(int)) != cudaSuccess ||
        cudaMemset(p->err, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        p->err = nullptr;
        plan_impl_free(p);
        set_last_error("cudaMalloc of the error word failed");
        return ACLFFT_ALLOC_FAILED;
    }
    if (!p->tb.segs.empty() || !p->tb.dsegs.empty()) {
        int rc = p->tb.segs.empty() ? 0 : gfft_gen_twiddles(p->tw, p->tb.segs.data(), (int)p->tb.segs.size(), nullptr);
        for (const auto& d : p->tb.dsegs) {
            if (rc != 0) break;
            rc = gfft_gen_dtwiddles(static_cast<float2*>(p->tw) + d.first, d.second, nullptr);
        }
        if (rc != 0 || cudaStreamSynchronize(nullptr) != cudaSuccess) {
            cudaGetLastError();
            plan_impl_free(p);
            set_last_error("twiddle generation failed");
            return ACLFFT_SETUP_FAILED;
        }
    }
    // cluster kernels: attributes and co-resident clusters, once per plan
    // (outside any stream capture)
    for (StepList& sl : p->lists) {
        for (Step& s : sl.steps) {
            if (s.kind != Step::CLUSTER) continue;
            const int n = gfft_cluster_prepare(s.cl.kid, s.cl.io_mode);
            if (n < 1) {
                cudaGetLastError();
                plan_impl_free(p);
                set_last_error(std::string("cluster kernel setup failed: ") +
                               cudaGetErrorString((cudaError_t)(n < 0 ? -n : (int)cudaErrorInvalidConfiguration)));
                return ACLFFT_SETUP_FAILED;
            }
            // OPS_FFT_CLUSTER_COUNT=<k> launches at most k clusters (tuning)
            const char* env_cc = std::getenv("OPS_FFT_CLUSTER_COUNT");
            const int cap = env_cc ? std::atoi(env_cc) : 0;
            s.cl.clusters = (cap > 0 && cap < n) ? cap : n;
        }
    }
    p->device = dev;
    p->device_ready = true;
    return ACLFFT_SUCCESS;
}

}  // namespace gfft

extern "C" {

ACLFFT_API aclfftResult aclfftCreate(aclfftHandle* plan)
{
    ACLFFT_CHECK_NULL(plan);
    aclfftHandle_t* p = new (std::nothrow) aclfftHandle_t();
    if (!p) return ACLFFT_ALLOC_FAILED;
    *plan = p;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftMakePlan1d(aclfftHandle plan, int nx, aclfftType type, int batch, int dimType,
                                         size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(!plan->is_initialized, ACLFFT_INVALID_VALUE);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(batch > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(dimType == ACLFFT_HORIZONTAL || dimType == ACLFFT_VERTICAL, ACLFFT_INVALID_VALUE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    if (validate_1d_size(dimType, nx, "aclfftMakePlan1d") != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    plan->rank = 1;
    plan->lengths[0] = nx;
    plan->batch = batch;
    plan->type = type;
    if (dimType == ACLFFT_VERTICAL) {
        plan->batch = 1;
        plan->stride[0] = batch;
    } else {
        plan->stride[0] = 1;
    }
    if (check_sizes(plan) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    const aclfftResult r = plan_execution(plan, workSize);
    if (r != ACLFFT_SUCCESS) return r;
    plan->is_initialized = true;
    maybe_autotune(plan, workSize);
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftMakePlan2d(aclfftHandle plan, int batch, int nx, int ny, aclfftType type,
                                         size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(!plan->is_initialized, ACLFFT_INVALID_VALUE);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(batch > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    plan->rank = 2;
    plan->lengths[0] = nx;
    plan->lengths[1] = ny;
    plan->batch = batch;
    plan->type = type;
    plan->stride[0] = 1;
    plan->stride[1] = 1;
    if (check_sizes(plan) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    const aclfftResult r = plan_execution(plan, workSize);
    if (r != ACLFFT_SUCCESS) return r;
    plan->is_initialized = true;
    maybe_autotune(plan, workSize);
    return ACLFFT_SUCCESS;
}

// 3D transform of one nx x ny x nz volume (nz fastest; every type),
// the reference's signature (include/cann_ops_fft.h:260; no batch argument).
ACLFFT_API aclfftResult aclfftMakePlan3d(aclfftHandle plan, int nx, int ny, int nz, aclfftType type,
                                         size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(!plan->is_initialized, ACLFFT_INVALID_VALUE);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(nz > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    plan->rank = 3;
    plan->lengths[0] = nx;
    plan->lengths[1] = ny;
    plan->lengths[2] = nz;
    plan->batch = 1;
    plan->type = type;
    plan->stride[0] = plan->stride[1] = plan->stride[2] = 1;
    if (check_sizes(plan) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    const aclfftResult r = plan_execution(plan, workSize);
    if (r != ACLFFT_SUCCESS) return r;
    plan->is_initialized = true;
    maybe_autotune(plan, workSize);
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftPlan1d(aclfftHandle* plan, int nx, aclfftType type, int batch, int dimType)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(batch > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(dimType == ACLFFT_HORIZONTAL || dimType == ACLFFT_VERTICAL, ACLFFT_INVALID_VALUE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    if (validate_1d_size(dimType, nx, "aclfftPlan1d") != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    aclfftResult r = aclfftCreate(plan);
    if (r != ACLFFT_SUCCESS) return r;
    r = aclfftMakePlan1d(*plan, nx, type, batch, dimType, nullptr);
    if (r != ACLFFT_SUCCESS) {
        aclfftDestroy(*plan);
        *plan = nullptr;
    }
    return r;
}

ACLFFT_API aclfftResult aclfftPlan2d(aclfftHandle* plan, int batch, int nx, int ny, aclfftType type)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(batch > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    aclfftResult r = aclfftCreate(plan);
    if (r != ACLFFT_SUCCESS) return r;
    r = aclfftMakePlan2d(*plan, batch, nx, ny, type, nullptr);
    if (r != ACLFFT_SUCCESS) {
        aclfftDestroy(*plan);
        *plan = nullptr;
    }
    return r;
}

ACLFFT_API aclfftResult aclfftPlan3d(aclfftHandle* plan, int nx, int ny, int nz, aclfftType type)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(nz > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    aclfftResult r = aclfftCreate(plan);
    if (r != ACLFFT_SUCCESS) return r;
    r = aclfftMakePlan3d(*plan, nx, ny, nz, type, nullptr);
    if (r != ACLFFT_SUCCESS) {
        aclfftDestroy(*plan);
        *plan = nullptr;
    }
    return r;
}

// ------------------------------------------------------------ work area
// The reference declares these and leaves them as stubs (lib/fft_utils_api.cpp:
// 66-89); its roadmap describes them (docs/implementation.md:90-100,176-212):
// query the work area a plan needs, let the plan allocate it (default) or
// let the caller provide it.  Here the work area is the device scratch the
// kernels use between passes (long 1D transforms split into column passes,
// in-place calls whose rows change pitch, 2D transforms); many plans need
// none.  Host-pointer execs additionally stage the data through plan-owned
// buffers allocated at their first call; device-pointer execs never
// allocate.

ACLFFT_API aclfftResult aclfftGetSize1d(aclfftHandle plan, int nx, aclfftType type, int batch, size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_NULL(workSize);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(batch > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    if (validate_1d_size(ACLFFT_HORIZONTAL, nx, "aclfftGetSize1d") != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    aclfftHandle_t d;
    d.rank = 1;
    d.lengths[0] = nx;
    d.stride[0] = 1;
    d.batch = batch;
    d.type = type;
    d.precision = plan->precision;
    if (check_sizes(&d) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    return gfft::estimate_work_area(&d, workSize);
}

ACLFFT_API aclfftResult aclfftGetSize2d(aclfftHandle plan, int nx, int ny, aclfftType type, size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_NULL(workSize);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    aclfftHandle_t d;
    d.rank = 2;
    d.lengths[0] = nx;
    d.lengths[1] = ny;
    d.stride[0] = d.stride[1] = 1;
    d.batch = 1;
    d.type = type;
    if (check_sizes(&d) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    return gfft::estimate_work_area(&d, workSize);
}

ACLFFT_API aclfftResult aclfftGetSize3d(aclfftHandle plan, int nx, int ny, int nz, aclfftType type,
                                        size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_NULL(workSize);
    ACLFFT_CHECK_PARAM(nx > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(ny > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(nz > 0, ACLFFT_INVALID_SIZE);
    ACLFFT_CHECK_PARAM(valid_type(type), ACLFFT_INVALID_TYPE);
    aclfftHandle_t d;
    d.rank = 3;
    d.lengths[0] = nx;
    d.lengths[1] = ny;
    d.lengths[2] = nz;
    d.stride[0] = d.stride[1] = d.stride[2] = 1;
    d.batch = 1;
    d.type = type;
    if (check_sizes(&d) != ACLFFT_SUCCESS) return ACLFFT_INVALID_SIZE;
    return gfft::estimate_work_area(&d, workSize);
}

ACLFFT_API aclfftResult aclfftGetSize(aclfftHandle plan, size_t* workSize)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_NULL(workSize);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    *workSize = gfft::work_area_bytes(plan->impl);
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftSetAutoAllocation(aclfftHandle plan, int autoAllocate)
{
    ACLFFT_CHECK_NULL(plan);
    const bool on = autoAllocate != 0;
    plan->auto_allocate = on;
    PlanImpl* impl = plan->impl;
    if (!plan->is_initialized || !impl || impl->auto_ws == on) {
        if (impl) impl->auto_ws = on;
        return ACLFFT_SUCCESS;
    }
    impl->auto_ws = on;
    if (!on) {
        // the plan's own workspace is released; a caller's area stays bound
        if (!impl->user_ws) gfft::release_workspace(impl);
        return ACLFFT_SUCCESS;
    }
    if (impl->user_ws || !impl->device_ready) return ACLFFT_SUCCESS;
    const aclfftResult r = gfft::allocate_workspace(impl);
    if (r != ACLFFT_SUCCESS) {
        impl->auto_ws = false;
        plan->auto_allocate = false;
    }
    return r;
}

ACLFFT_API aclfftResult aclfftSetWorkArea(aclfftHandle plan, void* workArea)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    PlanImpl* impl = plan->impl;
    if (!workArea) {
        // unbinds a caller's area; an auto-allocating plan gets its own back
        gfft::bind_work_area(impl, nullptr);
        if (impl->auto_ws && impl->device_ready) return gfft::allocate_workspace(impl);
        return ACLFFT_SUCCESS;
    }
    if (reinterpret_cast<uintptr_t>(workArea) % 256 != 0) {
        gfft::set_last_error("the work area must be 256-byte aligned");
        return ACLFFT_UNALIGNED_DATA;
    }
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, workArea) != cudaSuccess) {
        cudaGetLastError();
        at.type = cudaMemoryTypeUnregistered;
    }
    const bool ok = at.type == cudaMemoryTypeManaged ||
                    (at.type == cudaMemoryTypeDevice && (!impl->device_ready || at.device == impl->device));
    if (!ok) {
        gfft::set_last_error("the work area must be device memory of the plan's device");
        return ACLFFT_INVALID_VALUE;
    }
    gfft::bind_work_area(impl, workArea);
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftSetStream(aclfftHandle plan, cudaStream_t stream)
{
    ACLFFT_CHECK_NULL(plan);
    plan->stream = stream;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftDestroy(aclfftHandle plan)
{
    ACLFFT_CHECK_NULL(plan);
    delete plan;
    return ACLFFT_SUCCESS;
}

}  // extern "C"
