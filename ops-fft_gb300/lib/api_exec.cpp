// api_exec.cpp - transform execution.
//
// Entry checks mirror lib/fft_exec_api.cpp:32-85 of the reference (plan
// initialised, non-NULL buffers, matching plan type, valid direction) and the
// 1D op-layer checks of src/common/host/fft_exec_helper.h:37-47 (R2C/C2R
// reject VERTICAL plans with ACLFFT_NOT_IMPLEMENTED).  Lengths outside the
// supported domain (a prime factor > 47) also return ACLFFT_NOT_IMPLEMENTED,
// like the reference's dispatchers (src/fft1_d/arch35/fft1_d_exec_api.cpp:
// 42-74).  Device failures map to ACLFFT_EXEC_FAILED as in
// src/fft1_d/arch32/fft1_d_exec_api.cpp:148-152.
//
// Pointer semantics: device/managed pointers run asynchronously on the
// plan's stream (capturable in CUDA graphs); host pointers are staged
// through plan-owned device buffers and the call synchronises the stream
// before returning, which is the reference's contract for host buffers.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <thread>

#include "handle.h"

using gfft::Kind;
using gfft::PlanImpl;
using gfft::Step;
using gfft::StepList;

namespace {

thread_local std::string g_last_error;

// Where a caller's buffer lives: host memory (pageable or pinned) is staged
// through the plan's device buffers; device memory must belong to the device
// the call runs on (another GPU's memory would be dereferenced as a peer
// address, which faults without peer access); managed memory is reachable
// from every device.
enum class Mem { HOST, DEVICE, FOREIGN };

Mem classify(const void* p, int dev)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return Mem::HOST;
    }
    if (a.type == cudaMemoryTypeManaged) return Mem::DEVICE;
    if (a.type == cudaMemoryTypeDevice) return a.device == dev ? Mem::DEVICE : Mem::FOREIGN;
    return Mem::HOST;
}

// Reads (and clears) the plan's device error word after the work queued on
// `st`; every bounded wait in the kernels sets a bit there when it gives up
// (bit 0 row-kernel copy wait, bit 1 tensor-core MMA wait, bit 3 cluster
// exchange wait).  Synchronises `st`.
aclfftResult drain_error_word(PlanImpl* impl, cudaStream_t st, int* flags_out)
{
    int v = 0;
    if (cudaMemcpyAsync(&v, impl->err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        gfft::set_last_error("reading the device error word failed");
        return ACLFFT_EXEC_FAILED;
    }
    if (flags_out) *flags_out = v;
    if (v == 0) return ACLFFT_SUCCESS;
    if (cudaMemsetAsync(impl->err, 0, sizeof(int), st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
        cudaGetLastError();
    char msg[96];
    std::snprintf(msg, sizeof msg, "a device wait ran out of time (error flags 0x%x); the output is incomplete", v);
    gfft::set_last_error(msg);
    GFFT_LOG("exec: %s", msg);
    return ACLFFT_EXEC_FAILED;
}

double points(const aclfftHandle_t* h)
{
    double n = 1.0;
    for (int a = 0; a < h->rank; ++a) n *= (double)h->lengths[a];
    return n;
}

// The plan's output scale (FP32 kernels take it rounded to float).
double norm_scale(const aclfftHandle_t* h, bool backward_like)
{
    const double n = points(h);
    switch (h->normMode) {
    case ACLFFT_NORM_BACKWARD: return backward_like ? 1.0 / n : 1.0;
    case ACLFFT_NORM_ORTHO: return 1.0 / std::sqrt(n);
    case ACLFFT_NORM_FORWARD: return backward_like ? 1.0 : 1.0 / n;
    default: return 1.0;
    }
}

int launch_list(PlanImpl* impl, const StepList& sl, void* in, void* out, cudaStream_t st, bool c2c, bool inverse,
                double dscale, const float* wload = nullptr, bool host_in = false)
{
    void* bufs[4] = {in, out, impl->ws, impl->ws2};
    const float2* tw = static_cast<const float2*>(impl->tw);
    const float scale = (float)dscale;
    const size_t n = sl.steps.size();
    // the first and last computing steps (copies move data only)
    size_t i_first = 0, i_last = n ? n - 1 : 0;
    while (i_first + 1 < n && sl.steps[i_first].kind == Step::COPY) ++i_first;
    while (i_last > 0 && sl.steps[i_last].kind == Step::COPY) --i_last;
    for (size_t i = 0; i < n; ++i) {
        Step s = sl.steps[i];
        const bool first = i == i_first, last = i == i_last;
        void* src = bufs[s.src];
        void* dst = bufs[s.dst];
        int rc = 0;
        switch (s.kind) {
        case Step::ROW:
            s.row.tw = tw;
            s.row.post_tw = s.post_off >= 0 ? tw + s.post_off : nullptr;
            s.row.in = src;
            s.row.out = dst;
            s.row.err = impl->err;
            s.row.host_in = (first && host_in) ? 1 : 0;
            if (c2c) {
                s.row.conj_in = first && inverse;
                s.row.conj_out = last && inverse;
            }
            if (last) s.row.scale = scale;
            if (first && wload) {
                s.row.wload = wload;
                s.row.wdist = s.row.in_dist;
            }
            rc = gfft_launch_row(&s.row, st);
            break;
        case Step::COL:
            s.col.tw = tw;
            s.col.otw_hi = s.hi_off >= 0 ? tw + s.hi_off : nullptr;
            s.col.otw_lo = s.lo_off >= 0 ? tw + s.lo_off : nullptr;
            s.col.in = src;
            s.col.out = dst;
            if (c2c) {
                s.col.conj_in = first && inverse;
                s.col.conj_out = last && inverse;
            }
            if (last) s.col.scale = scale;
            rc = gfft_launch_col(&s.col, st);
            break;
        case Step::PACK:
            s.pack.post_tw = tw + s.post_off;
            s.pack.in = src;
            s.pack.out = dst;
            if (last) s.pack.scale = scale;
            rc = gfft_launch_pack(&s.pack, st);
            break;
        case Step::COPY:
            rc = (int)cudaMemcpyAsync(dst, src, (size_t)s.copy_bytes, cudaMemcpyDeviceToDevice, st);
            break;
        case Step::DPASS:
            s.dp.in = src;
            s.dp.out = dst;
            s.dp.tw = tw + s.dtw_off;
            if (c2c) {
                s.dp.conj_in = first && inverse;
                s.dp.conj_out = last && inverse;
            }
            if (last) s.dp.scale = dscale;
            rc = gfft_launch_dpass(&s.dp, st);
            break;
        case Step::TC:
            s.tc.in = src;
            s.tc.out = dst;
            s.tc.bmat = tw + s.bmat_off;
            s.tc.twl = tw + s.tw_off;
            s.tc.otw_hi = s.hi_off >= 0 ? tw + s.hi_off : nullptr;
            s.tc.otw_lo = s.lo_off >= 0 ? tw + s.lo_off : nullptr;
            s.tc.err = impl->err;
            if (c2c) {
                s.tc.conj_in = first && inverse;
                s.tc.conj_out = last && inverse;
            }
            if (last) s.tc.scale = scale;
            rc = gfft_launch_tc(&s.tc, st);
            break;
        case Step::CLUSTER:
            s.cl.in = src;
            s.cl.out = dst;
            s.cl.tw = tw;
            s.cl.err = impl->err;
            if (c2c) {
                s.cl.conj_in = first && inverse;
                s.cl.conj_out = last && inverse;
            }
            if (last) s.cl.scale = scale;
            rc = gfft_launch_cluster(&s.cl, st);
            break;
        }
        if (rc != 0) {
            gfft::set_last_error(std::string("kernel launch failed: ") + cudaGetErrorString((cudaError_t)rc));
            cudaGetLastError();
            return rc;
        }
    }
    return 0;
}

// True when a step of `sl` reads or writes a workspace the plan does not
// have (auto allocation off and no work area set).
bool missing_workspace(const PlanImpl* impl, const StepList& sl)
{
    for (const Step& s : sl.steps) {
        for (int b : {s.src, s.dst}) {
            if ((b == 2 && !impl->ws) || (b == 3 && !impl->ws2)) return true;
        }
    }
    return false;
}

aclfftResult no_workspace()
{
    gfft::set_last_error("the plan has no work area: auto allocation is off and aclfftSetWorkArea was not called");
    return ACLFFT_NO_WORKSPACE;
}

// Host buffers, one row-kernel step: the batch is cut into chunks whose
// host-to-device copy, kernel and device-to-host copy run on three streams,
// so copies in both directions overlap the kernels of neighbouring chunks.
// Returns 0 on success, 1 on failure, -1 when the transform is too small to
// be worth chunking (the caller then runs the plain staged path).
int exec_host_pipelined(PlanImpl* impl, const Step& step, const void* in, void* out, size_t in_bytes,
                        size_t out_bytes, cudaStream_t st, bool c2c, bool inverse, float scale)
{
    const int64_t ntf = step.row.ntf;
    // chunks per exec (OPS_FFT_HOST_CHUNKS, 2..32, default 4): more chunks
    // shorten the pipeline's fill and drain but cost more per chunk; measured
    // on the R2C/C2R N=3000/1024 batch-4096 round trip with pinned buffers:
    // 4 chunks 230 GB/s, 8 224, 16 209, 32 178
    static const int kChunks = [] {
        const char* v = std::getenv("OPS_FFT_HOST_CHUNKS");
        return v ? std::max(2, std::min(PlanImpl::kMaxHostChunks, std::atoi(v))) : 4;
    }();
    if (ntf < 2 * kChunks || in_bytes + out_bytes < (size_t)(8u << 20)) return -1;
    if (in_bytes % (size_t)ntf || out_bytes % (size_t)ntf) return -1;
    const size_t rin = in_bytes / (size_t)ntf, rout = out_bytes / (size_t)ntf;
    if (!impl->pipe_ready) {
        bool ok = cudaStreamCreateWithFlags(&impl->s_in, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&impl->s_out, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&impl->ev_start, cudaEventDisableTiming) == cudaSuccess;
        for (int c = 0; ok && c < PlanImpl::kMaxHostChunks; ++c)
            ok = cudaEventCreateWithFlags(&impl->ev_in[c], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&impl->ev_k[c], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return -1;
        }
        impl->pipe_ready = true;
    }
    if (cudaEventRecord(impl->ev_start, st) != cudaSuccess || cudaStreamWaitEvent(impl->s_in, impl->ev_start, 0) != cudaSuccess)
        return 1;
    const int64_t per = (ntf + kChunks - 1) / kChunks;
    const float2* tw = static_cast<const float2*>(impl->tw);
    int used = 0;
    for (int c = 0; c < kChunks; ++c) {
        const int64_t t0 = c * per, t1 = std::min<int64_t>(ntf, t0 + per);
        if (t0 >= t1) break;
        ++used;
        char* din = static_cast<char*>(impl->stage_a) + t0 * rin;
        if (cudaMemcpyAsync(din, static_cast<const char*>(in) + t0 * rin, (t1 - t0) * rin, cudaMemcpyHostToDevice,
                            impl->s_in) != cudaSuccess ||
            cudaEventRecord(impl->ev_in[c], impl->s_in) != cudaSuccess)
            return 1;
    }
    // When the caller's input and output ranges overlap (an in-place call),
    // a chunk's output rows can cover input rows of later chunks (R2C rows
    // grow from n reals to n/2+1 complex values), so no result is copied
    // back before the whole input has been read.
    const bool overlap = static_cast<const char*>(in) < static_cast<const char*>(out) + out_bytes &&
                         static_cast<const char*>(out) < static_cast<const char*>(in) + in_bytes;
    if (overlap && cudaStreamWaitEvent(impl->s_out, impl->ev_in[used - 1], 0) != cudaSuccess) return 1;
    for (int c = 0; c < used; ++c) {
        const int64_t t0 = c * per, t1 = std::min<int64_t>(ntf, t0 + per);
        char* din = static_cast<char*>(impl->stage_a) + t0 * rin;
        char* dout = static_cast<char*>(impl->stage_b) + t0 * rout;
        if (cudaStreamWaitEvent(st, impl->ev_in[c], 0) != cudaSuccess) return 1;
        gfft::RowArgs a = step.row;
        a.tw = tw;
        a.post_tw = step.post_off >= 0 ? tw + step.post_off : nullptr;
        a.in = din;
        a.out = dout;
        a.err = impl->err;
        a.ntf = t1 - t0;
        if (c2c) {
            a.conj_in = inverse;
            a.conj_out = inverse;
        }
        a.scale = scale;
        if (gfft_launch_row(&a, st) != 0 || cudaEventRecord(impl->ev_k[c], st) != cudaSuccess ||
            cudaStreamWaitEvent(impl->s_out, impl->ev_k[c], 0) != cudaSuccess ||
            cudaMemcpyAsync(static_cast<char*>(out) + t0 * rout, dout, (t1 - t0) * rout, cudaMemcpyDeviceToHost,
                            impl->s_out) != cudaSuccess)
            return 1;
    }
    if (cudaStreamSynchronize(impl->s_out) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return 0;
}

// The device address of pinned (page-locked, mapped) host memory, or
// nullptr for any other pointer.
void* mapped_host(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Host buffers the kernel may use in place: both pinned, the plan one
// codelet launch from the input to the output (the only kernel whose input
// pipeline runs on host-mapped memory), the ranges disjoint and aligned to
// the kernel's element.  By default only calls of at most kHostDirectBytes
// (input + output) run in place: measured per call on GB300 (pinned
// buffers, NVLink-C2C host link), in place beats the staged pipeline on
// small calls (C2C 4096 x 256, 16.8 MB: 164 vs 149 GB/s) and loses on large
// ones (R2C 1024 x 4096, 33.6 MB: 168 vs 190; R2C 3000 x 4096, 98 MB: 218 vs
// 239), where the staged pipeline's copy engines move both directions at
// once.  OPS_FFT_HOST_DIRECT=1 runs every eligible call in place, =0 none.
constexpr size_t kHostDirectBytes = 24u << 20;

bool host_direct(const StepList& sl, const void* in, const void* out, size_t in_bytes, size_t out_bytes,
                 size_t in_align, size_t out_align, void** din, void** dout)
{
    const char* env = std::getenv("OPS_FFT_HOST_DIRECT");
    if (env && env[0] == '0') return false;
    if (!(env && env[0] == '1') && in_bytes + out_bytes > kHostDirectBytes) return false;
    if (sl.steps.size() != 1) return false;
    const Step& s = sl.steps[0];
    if (s.kind != Step::ROW || s.row.codelet < 0 || s.src != 0 || s.dst != 1) return false;
    const char* i0 = static_cast<const char*>(in);
    const char* o0 = static_cast<const char*>(out);
    if (i0 < o0 + out_bytes && o0 < i0 + in_bytes) return false;
    *din = mapped_host(in);
    *dout = mapped_host(out);
    return *din && *dout && reinterpret_cast<uintptr_t>(*din) % in_align == 0 &&
           reinterpret_cast<uintptr_t>(*dout) % out_align == 0;
}

struct CallShape {
    size_t in_bytes;
    size_t out_bytes;
    // alignment the kernels need of device pointers: the complex element
    // (8 bytes FP32, 16 FP64); real FP64 rows are read as double pairs (8)
    size_t in_align = 8;
    size_t out_align = 8;
};

// variant 0 = primary transform, 2 = adjoint transform
aclfftResult exec_common(aclfftHandle_t* h, int variant, void* in, void* out, CallShape shape, bool c2c,
                         bool inverse, bool backward_like)
{
    PlanImpl* impl = h->impl;
    if (!impl) return ACLFFT_INTERNAL_ERROR;
    const StepList& primary = impl->lists[variant];
    if (!primary.supported) {
        GFFT_LOG("exec: %s", primary.why.c_str());
        gfft::set_last_error(primary.why);
        return ACLFFT_NOT_IMPLEMENTED;
    }
    if (!impl->device_ready) {
        if (gfft::plan_device_setup(impl) != ACLFFT_SUCCESS || !impl->device_ready) {
            gfft::set_last_error("no usable CUDA device");
            return ACLFFT_EXEC_FAILED;
        }
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    if (dev != impl->device) {
        gfft::set_last_error("plan executed on a different device than it was created on");
        return ACLFFT_INVALID_DEVICE;
    }
    const double scale = norm_scale(h, backward_like);
    cudaStream_t st = h->stream;
    const Mem min = classify(in, dev), mout = classify(out, dev);
    if (min == Mem::FOREIGN || mout == Mem::FOREIGN) {
        gfft::set_last_error("a data pointer is device memory of another GPU than the current one");
        return ACLFFT_INVALID_VALUE;
    }
    const bool din = min == Mem::DEVICE, dout = mout == Mem::DEVICE;
    if ((din && reinterpret_cast<uintptr_t>(in) % shape.in_align) ||
        (dout && reinterpret_cast<uintptr_t>(out) % shape.out_align)) {
        gfft::set_last_error("a device data pointer is not aligned to the transform's complex element");
        return ACLFFT_UNALIGNED_DATA;
    }
    if (din && dout) {
        const StepList& sl = (in == out) ? impl->lists[variant + 1] : primary;
        if (!sl.supported) return ACLFFT_NOT_IMPLEMENTED;
        if (missing_workspace(impl, sl)) return no_workspace();
        return launch_list(impl, sl, in, out, st, c2c, inverse, scale) == 0 ? ACLFFT_SUCCESS : ACLFFT_EXEC_FAILED;
    }
    // host buffers: stage through device memory, return when done
    if (missing_workspace(impl, primary)) return no_workspace();
    void* hin = nullptr;
    void* hout = nullptr;
    if (!din && !dout &&
        host_direct(primary, in, out, shape.in_bytes, shape.out_bytes, shape.in_align, shape.out_align, &hin, &hout)) {
        // pinned host buffers: the kernel reads and writes them over the
        // host link, with the transfers of both directions overlapping for
        // the whole call (no staging copies, no pipeline fill or drain)
        if (launch_list(impl, primary, hin, hout, st, c2c, inverse, scale, nullptr, true) != 0) {
            cudaStreamSynchronize(st);
            cudaGetLastError();
            return ACLFFT_EXEC_FAILED;
        }
        return drain_error_word(impl, st, nullptr);
    }
    const size_t need = std::max(shape.in_bytes, shape.out_bytes);
    if (impl->stage_bytes < need) {
        if (impl->stage_a) cudaFree(impl->stage_a);
        if (impl->stage_b) cudaFree(impl->stage_b);
        impl->stage_a = impl->stage_b = nullptr;
        impl->stage_bytes = 0;
        if (gfft::dev_alloc(&impl->stage_a, need) != cudaSuccess || gfft::dev_alloc(&impl->stage_b, need) != cudaSuccess) {
            cudaGetLastError();
            if (impl->stage_a) cudaFree(impl->stage_a);
            impl->stage_a = impl->stage_b = nullptr;
            gfft::set_last_error("cudaMalloc of the host staging buffers failed");
            return ACLFFT_ALLOC_FAILED;
        }
        impl->stage_bytes = need;
    }
    void* dev_in = din ? in : impl->stage_a;
    void* dev_out = dout ? out : impl->stage_b;
    if (!din && !dout && primary.steps.size() == 1 && primary.steps[0].kind == Step::ROW) {
        const int rc = exec_host_pipelined(impl, primary.steps[0], in, out, shape.in_bytes, shape.out_bytes, st, c2c,
                                           inverse, (float)scale);
        if (rc > 0) return ACLFFT_EXEC_FAILED;
        if (rc == 0) return drain_error_word(impl, st, nullptr);
    }
    if (!din && cudaMemcpyAsync(dev_in, in, shape.in_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    const StepList& sl = (dev_in == dev_out) ? impl->lists[variant + 1] : primary;
    if (launch_list(impl, sl, dev_in, dev_out, st, c2c, inverse, scale) != 0) {
        cudaStreamSynchronize(st);
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    if (!dout && cudaMemcpyAsync(out, dev_out, shape.out_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    // host buffers: the call has waited for the device anyway, so a wait
    // that ran out is reported here
    return drain_error_word(impl, st, nullptr);
}

// Rows along the fastest axis (batch x the slower axes) and that axis' length.
size_t outer_rows(const aclfftHandle_t* h)
{
    size_t r = (size_t)h->batch;
    for (int a = 0; a + 1 < h->rank; ++a) r *= (size_t)h->lengths[a];
    return r;
}
size_t last_len(const aclfftHandle_t* h) { return (size_t)h->lengths[h->rank - 1]; }

size_t complex_elems(const aclfftHandle_t* h)
{
    if (h->rank >= 2) return outer_rows(h) * last_len(h);
    return (size_t)h->batch * (size_t)h->lengths[0] * (size_t)(h->stride[0] > 1 ? h->stride[0] : 1);
}

size_t real_elems(const aclfftHandle_t* h) { return outer_rows(h) * last_len(h); }
size_t half_elems(const aclfftHandle_t* h) { return outer_rows(h) * (last_len(h) / 2 + 1); }

#define EXEC_PLAN_CHECKS(plan, a, b, expected)                                \
    ACLFFT_CHECK_NULL(plan);                                                  \
    ACLFFT_CHECK_PARAM((plan)->is_initialized, ACLFFT_INVALID_PLAN);          \
    ACLFFT_CHECK_NULL(a);                                                     \
    ACLFFT_CHECK_NULL(b);                                                     \
    ACLFFT_CHECK_PARAM((plan)->type == (expected), ACLFFT_INVALID_TYPE)

}  // namespace

namespace gfft {
void set_last_error(const std::string& s) { g_last_error = s; }

int launch_primary(PlanImpl* impl, void* in, void* out, cudaStream_t st)
{
    const StepList& sl = impl->lists[0];
    if (!sl.supported || missing_workspace(impl, sl)) return (int)cudaErrorInvalidValue;
    return launch_list(impl, sl, in, out, st, impl->prob.kind == Kind::C2C, false, 1.f);
}
}  // namespace gfft

extern "C" {

ACLFFT_API aclfftResult aclfftExecC2C(aclfftHandle plan, aclfftComplex* idata, aclfftComplex* odata, int direction)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_C2C);
    ACLFFT_CHECK_PARAM(direction == ACLFFT_FORWARD || direction == ACLFFT_BACKWARD, ACLFFT_INVALID_VALUE);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    const size_t bytes = complex_elems(plan) * 8;
    const bool inv = direction == ACLFFT_BACKWARD;
    return exec_common(plan, 0, idata, odata, {bytes, bytes}, true, inv, inv);
}

ACLFFT_API aclfftResult aclfftExecR2C(aclfftHandle plan, aclfftReal* idata, aclfftComplex* odata)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_R2C);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 0, idata, odata, {real_elems(plan) * 4, half_elems(plan) * 8}, false, false, false);
}

ACLFFT_API aclfftResult aclfftExecC2R(aclfftHandle plan, aclfftComplex* idata, aclfftReal* odata)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_C2R);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 0, idata, odata, {half_elems(plan) * 8, real_elems(plan) * 4}, false, false, true);
}

ACLFFT_API aclfftResult aclfftExecC2CAdjoint(aclfftHandle plan, aclfftComplex* gradOut, aclfftComplex* gradIn,
                                             int direction)
{
    EXEC_PLAN_CHECKS(plan, gradOut, gradIn, ACLFFT_C2C);
    ACLFFT_CHECK_PARAM(direction == ACLFFT_FORWARD || direction == ACLFFT_BACKWARD, ACLFFT_INVALID_VALUE);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    const size_t bytes = complex_elems(plan) * 8;
    const bool primary_inv = direction == ACLFFT_BACKWARD;
    // adjoint of direction d is direction -d with the primary's scale
    return exec_common(plan, 0, gradOut, gradIn, {bytes, bytes}, true, !primary_inv, primary_inv);
}

ACLFFT_API aclfftResult aclfftExecR2CAdjoint(aclfftHandle plan, aclfftComplex* gradOut, aclfftReal* gradIn)
{
    EXEC_PLAN_CHECKS(plan, gradOut, gradIn, ACLFFT_R2C);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 2, gradOut, gradIn, {half_elems(plan) * 8, real_elems(plan) * 4}, false, false,
                       false);
}

ACLFFT_API aclfftResult aclfftExecR2CAdjointWeighted(aclfftHandle plan, const aclfftComplex* gradOut,
                                                     const aclfftReal* weights, aclfftReal* gradIn)
{
    EXEC_PLAN_CHECKS(plan, gradOut, gradIn, ACLFFT_R2C);
    ACLFFT_CHECK_NULL(weights);
    if (plan->rank != 1) return ACLFFT_NOT_IMPLEMENTED;
    PlanImpl* impl = plan->impl;
    if (!impl) return ACLFFT_INTERNAL_ERROR;
    const StepList& sl = impl->lists[2];
    // the weights ride on the even-C2R pre-process of a single codelet launch
    if (!sl.supported || sl.steps.size() != 1 || sl.steps[0].kind != Step::ROW || sl.steps[0].row.codelet < 0 ||
        sl.steps[0].row.io_mode != gfft::IO_C2R_EVEN) {
        gfft::set_last_error("weighted adjoint: this length's adjoint is not one codelet launch");
        return ACLFFT_NOT_IMPLEMENTED;
    }
    if (static_cast<const void*>(gradOut) == static_cast<const void*>(gradIn)) {
        gfft::set_last_error("weighted adjoint: in-place calls are not supported");
        return ACLFFT_INVALID_VALUE;
    }
    if (!impl->device_ready) {
        if (gfft::plan_device_setup(impl) != ACLFFT_SUCCESS || !impl->device_ready) {
            gfft::set_last_error("no usable CUDA device");
            return ACLFFT_EXEC_FAILED;
        }
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    if (dev != impl->device) return ACLFFT_INVALID_DEVICE;
    if (classify(gradOut, dev) != Mem::DEVICE || classify(gradIn, dev) != Mem::DEVICE ||
        classify(weights, dev) != Mem::DEVICE) {
        gfft::set_last_error("weighted adjoint: device pointers of the plan's device only");
        return ACLFFT_INVALID_VALUE;
    }
    const double scale = norm_scale(plan, false);
    return launch_list(impl, sl, const_cast<aclfftComplex*>(gradOut), gradIn, plan->stream, false, false, scale,
                       weights) == 0
               ? ACLFFT_SUCCESS
               : ACLFFT_EXEC_FAILED;
}

ACLFFT_API aclfftResult aclfftExecC2RAdjoint(aclfftHandle plan, aclfftReal* gradOut, aclfftComplex* gradIn)
{
    EXEC_PLAN_CHECKS(plan, gradOut, gradIn, ACLFFT_C2R);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 2, gradOut, gradIn, {real_elems(plan) * 4, half_elems(plan) * 8}, false, false,
                       true);
}

// Double precision (the reference declares these and returns
// ACLFFT_NOT_IMPLEMENTED, lib/fft_exec_api.cpp:87-116): the same checks and
// pointer semantics as the single-precision entries.
ACLFFT_API aclfftResult aclfftExecZ2Z(aclfftHandle plan, aclfftDoubleComplex* idata, aclfftDoubleComplex* odata,
                                      int direction)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_Z2Z);
    ACLFFT_CHECK_PARAM(direction == ACLFFT_FORWARD || direction == ACLFFT_BACKWARD, ACLFFT_INVALID_VALUE);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    const size_t bytes = complex_elems(plan) * 16;
    const bool inv = direction == ACLFFT_BACKWARD;
    return exec_common(plan, 0, idata, odata, {bytes, bytes, 16, 16}, true, inv, inv);
}

ACLFFT_API aclfftResult aclfftExecD2Z(aclfftHandle plan, aclfftDoubleReal* idata, aclfftDoubleComplex* odata)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_D2Z);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 0, idata, odata, {real_elems(plan) * 8, half_elems(plan) * 16, 8, 16}, false, false,
                       false);
}

ACLFFT_API aclfftResult aclfftExecZ2D(aclfftHandle plan, aclfftDoubleComplex* idata, aclfftDoubleReal* odata)
{
    EXEC_PLAN_CHECKS(plan, idata, odata, ACLFFT_Z2D);
    if (plan->rank < 1 || plan->rank > 3) return ACLFFT_NOT_IMPLEMENTED;
    return exec_common(plan, 0, idata, odata, {half_elems(plan) * 16, real_elems(plan) * 8, 16, 8}, false, false,
                       true);
}

ACLFFT_API aclfftResult aclfftGetExecError(aclfftHandle plan, int* flags)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    ACLFFT_CHECK_NULL(flags);
    *flags = 0;
    PlanImpl* impl = plan->impl;
    if (!impl->device_ready || !impl->err) return ACLFFT_SUCCESS;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != impl->device) {
        cudaGetLastError();
        return ACLFFT_INVALID_DEVICE;
    }
    return drain_error_word(impl, plan->stream, flags);
}

ACLFFT_API aclfftResult aclfftDebugSetExecError(aclfftHandle plan, int flags)
{
    ACLFFT_CHECK_NULL(plan);
    ACLFFT_CHECK_PARAM(plan->is_initialized && plan->impl, ACLFFT_INVALID_PLAN);
    PlanImpl* impl = plan->impl;
    if (!impl->device_ready || !impl->err) return ACLFFT_EXEC_FAILED;
    if (cudaMemcpyAsync(impl->err, &flags, sizeof(int), cudaMemcpyHostToDevice, plan->stream) != cudaSuccess ||
        cudaStreamSynchronize(plan->stream) != cudaSuccess) {
        cudaGetLastError();
        return ACLFFT_EXEC_FAILED;
    }
    return ACLFFT_SUCCESS;
}

ACLFFT_API const char* aclfftGetLastErrorDetail(void) { return g_last_error.c_str(); }

}  // extern "C"
