// api_utils.cpp - error strings, the reference's NOT_IMPLEMENTED stubs and
// the GB300 extension getters/setters.
//
// aclfftGetErrorString follows lib/fft_utils_api.cpp:19-56 of the reference
// (same strings, "Unknown error" otherwise).  The version queries are stubs
// in the reference (lib/fft_utils_api.cpp:95-109) and its roadmap lists them
// as library information (docs/implementation.md:101-106); here they report
// this library's version.  aclfftSetStride stays a stub as in the reference
// (lib/fft_utils_api.cpp:90-94).
#include <algorithm>
#include <atomic>
#include <cstring>
#include <math.h>
#include <utility>

#include "../csrc/butterfly.cuh"
#include "handle.h"

namespace gfft {

// Failure injection for device allocations: -1 off, k >= 0 lets k more
// allocations succeed and fails every one after them.
std::atomic<int> g_fail_alloc_after{-1};

cudaError_t dev_alloc(void** p, size_t bytes)
{
    int k = g_fail_alloc_after.load();
    while (k >= 0) {
        if (k == 0) {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
        if (g_fail_alloc_after.compare_exchange_weak(k, k - 1)) break;
    }
    return cudaMalloc(p, bytes);
}

bool log_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("OPS_FFT_LOG");
        return !(v && (std::strcmp(v, "0") == 0 || std::strcmp(v, "off") == 0));
    }();
    return on;
}

}  // namespace gfft

namespace {

template <int R>
void butterfly_host(const float* in, float* out)
{
    float2 v[R];
    for (int i = 0; i < R; ++i) v[i] = make_float2(in[2 * i], in[2 * i + 1]);
    gfft::DFT<R>::run(v);
    for (int i = 0; i < R; ++i) {
        out[2 * i] = v[i].x;
        out[2 * i + 1] = v[i].y;
    }
}

template <int... Rs>
bool butterfly_dispatch(int R, const float* in, float* out, std::integer_sequence<int, Rs...>)
{
    bool done = false;
    ((R == Rs + 1 ? (butterfly_host<Rs + 1>(in, out), done = true) : false), ...);
    return done;
}

}  // namespace

extern "C" {

ACLFFT_API const char* aclfftGetErrorString(aclfftResult result)
{
    switch (result) {
    case ACLFFT_SUCCESS: return "Success";
    case ACLFFT_INVALID_PLAN: return "Invalid plan handle";
    case ACLFFT_ALLOC_FAILED: return "Memory allocation failed";
    case ACLFFT_INVALID_TYPE: return "Invalid data type";
    case ACLFFT_INVALID_VALUE: return "Invalid parameter value";
    case ACLFFT_INTERNAL_ERROR: return "Internal error";
    case ACLFFT_EXEC_FAILED: return "Execution failed";
    case ACLFFT_SETUP_FAILED: return "Setup failed";
    case ACLFFT_INVALID_SIZE: return "Invalid size parameter";
    case ACLFFT_UNALIGNED_DATA: return "Data not aligned";
    case ACLFFT_INCOMPLETE_PARAMETER_LIST: return "Incomplete parameter list";
    case ACLFFT_INVALID_DEVICE: return "Invalid device";
    case ACLFFT_PARSE_ERROR: return "Parse error";
    case ACLFFT_NO_WORKSPACE: return "No workspace available";
    case ACLFFT_NOT_IMPLEMENTED: return "Feature not implemented";
    case ACLFFT_NOT_SUPPORTED: return "Feature not supported";
    default: return "Unknown error";
    }
}

ACLFFT_API aclfftResult aclfftSetStride(aclfftHandle plan, int32_t stride)
{
    (void)plan; (void)stride;
    return ACLFFT_NOT_IMPLEMENTED;
}

ACLFFT_API aclfftResult aclfftGetVersion(int* version)
{
    ACLFFT_CHECK_NULL(version);
    *version = ACLFFT_GB300_VERSION;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftGetProperty(aclfftLibraryPropertyType type, int* value)
{
    ACLFFT_CHECK_NULL(value);
    switch (type) {
    case ACLFFT_MAJOR_VERSION: *value = ACLFFT_GB300_VERSION_MAJOR; return ACLFFT_SUCCESS;
    case ACLFFT_MINOR_VERSION: *value = ACLFFT_GB300_VERSION_MINOR; return ACLFFT_SUCCESS;
    case ACLFFT_PATCH_LEVEL: *value = ACLFFT_GB300_VERSION_PATCH; return ACLFFT_SUCCESS;
    default: return ACLFFT_INVALID_TYPE;
    }
}

ACLFFT_API aclfftResult aclfftDebugFailAllocations(int after)
{
    gfft::g_fail_alloc_after.store(after < 0 ? -1 : after);
    return ACLFFT_SUCCESS;
}

// ------------------------------------------------------------- extensions
ACLFFT_API aclfftResult aclfftSetNormMode(aclfftHandle plan, int normMode)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_PARAM(normMode >= ACLFFT_NORM_NONE && normMode <= ACLFFT_NORM_FORWARD, ACLFFT_INVALID_VALUE);
    plan->normMode = normMode;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftSetPrecisionMode(aclfftHandle plan, int mode)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_PARAM(mode >= ACLFFT_PREC_FP32 && mode <= ACLFFT_PREC_BF16X3, ACLFFT_INVALID_VALUE);
    if (plan->precision == mode) return ACLFFT_SUCCESS;
    const int old = plan->precision;
    plan->precision = mode;
    const aclfftResult r = gfft::replan(plan);
    if (r != ACLFFT_SUCCESS) plan->precision = old;
    return r;
}

ACLFFT_API aclfftResult aclfftGetPrecisionMode(aclfftHandle plan, int* mode)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(mode);
    *mode = plan->precision;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftGetNormMode(aclfftHandle plan, int* normMode)
{
    ACLFFT_CHECK_PARAM(plan != nullptr, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(normMode);
    *normMode = plan->normMode;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftGetPlanInfo(aclfftHandle plan, aclfftPlanInfo* info)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(info);
    std::memset(info, 0, sizeof(*info));
    const gfft::StepList& sl = plan->impl->lists[0];
    info->supported = sl.supported ? 1 : 0;
    info->nsteps = (int)sl.steps.size();
    for (const gfft::Step& s : sl.steps)
        if (s.kind == gfft::Step::TC) ++info->tc_stages;
    for (const gfft::Step& s : sl.steps)
        if (s.kind == gfft::Step::CLUSTER) {
            info->cluster_ctas = s.cl.csize;
            info->cluster_count = s.cl.clusters;
        }
    for (const gfft::Step& s : sl.steps) {
        const gfft::InnerPlan* ip = nullptr;
        int tf = 0;
        info->kernel = -1;
        if (s.kind == gfft::Step::ROW) {
            ip = &s.row.ip;
            tf = s.row.tfpc;
            info->kernel = s.row.codelet;
            info->groups_per_cta = s.row.ngroups;
            info->stages = s.row.nstage;
            info->smem_bytes = s.row.smem_bytes;
        } else if (s.kind == gfft::Step::COL) {
            ip = &s.col.ip;
            tf = s.col.tfpc;
        } else if (s.kind == gfft::Step::CLUSTER) {
            // column radices then row radices; threads = all CTAs of a cluster
            int C = 0, Q = 0, P = 0, Q0 = 0, P0 = 0, nt = 0, smem = 0;
            if (gfft_cluster_lookup(s.cl.length, s.cl.csize, &C, &Q, &P, &Q0, &P0, &nt, &smem) == s.cl.kid) {
                info->nradix = 4;
                info->radix[0] = Q0;
                info->radix[1] = Q / Q0;
                info->radix[2] = P0;
                info->radix[3] = P / P0;
                info->onchip_length = Q * P;
                info->threads_per_transform = nt * C;
                info->transforms_per_cta = 1;
                info->smem_bytes = smem;
            }
            break;
        }
        if (!ip) continue;
        info->nradix = ip->npass;
        for (int p = 0; p < ip->npass && p < 12; ++p) info->radix[p] = ip->pass[p].radix;
        info->onchip_length = ip->L;
        info->threads_per_transform = ip->nthr;
        info->transforms_per_cta = tf;
        break;
    }
    info->twiddle_entries = plan->impl->tb.count;
    info->workspace_bytes = gfft::work_area_bytes(plan->impl);
    info->tuned = plan->tuned;
    info->tune_candidates = plan->tune_candidates;
    return ACLFFT_SUCCESS;
}

ACLFFT_API aclfftResult aclfftDebugGetTwiddleSegments(aclfftHandle plan, long long* segs, int maxSegs, int* nsegs)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(nsegs);
    const auto& v = plan->impl->tb.segs;
    *nsegs = (int)v.size();
    for (int i = 0; segs && i < maxSegs && i < (int)v.size(); ++i) {
        segs[5 * i + 0] = v[i].offset;
        segs[5 * i + 1] = v[i].count;
        segs[5 * i + 2] = v[i].M;
        segs[5 * i + 3] = v[i].R_or_mult;
        segs[5 * i + 4] = v[i].kind;
    }
    return ACLFFT_SUCCESS;
}


ACLFFT_API aclfftResult aclfftDebugButterfly(int R, const float* in, float* out)
{
    ACLFFT_CHECK_NULL(in);
    ACLFFT_CHECK_NULL(out);
    ACLFFT_CHECK_PARAM(R >= 1 && R <= 48, ACLFFT_INVALID_SIZE);
    return butterfly_dispatch(R, in, out, std::make_integer_sequence<int, 48>{}) ? ACLFFT_SUCCESS
                                                                                 : ACLFFT_INVALID_SIZE;
}

ACLFFT_API aclfftResult aclfftGetTwiddles(aclfftHandle plan, aclfftComplex* host, long long maxEntries,
                                          long long* entries)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(entries);
    gfft::PlanImpl* impl = plan->impl;
    *entries = impl->tb.count;
    if (!host || maxEntries <= 0) return ACLFFT_SUCCESS;
    if (!impl->device_ready && gfft::plan_device_setup(impl) != ACLFFT_SUCCESS) return ACLFFT_EXEC_FAILED;
    if (!impl->device_ready) return ACLFFT_EXEC_FAILED;
    const long long n = std::min<long long>(maxEntries, impl->tb.count);
    if (n > 0 && cudaMemcpy(host, impl->tw, (size_t)n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    return ACLFFT_SUCCESS;
}

}  // extern "C"
