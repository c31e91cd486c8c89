// noalloc.cu - an allocation-free entry point for long batched C2C.
//
// aclfftExecC2CNoAlloc runs the same two column passes as a plan for a long
// C2C (length n = L1 * L2 split over two on-chip factors), but without any
// plan object or device allocation: the intermediate between the two passes
// lives in a fixed file-scope device array, and the FP64-evaluated twiddle
// tables are regenerated into a second fixed array at every call.  It exists
// for callers that cannot call cudaMalloc: code running while another
// component owns the device memory pool (a host framework whose caching
// allocator has reserved the memory, a real-time loop that must not touch
// the allocator), or code that has to stay clear of the implicit
// synchronisation cudaMalloc/cudaFree can cause.
//
// Limits and sharing rules:
//   * n * batch <= kScratchElems (2^21 complex values, 16 MiB of scratch) and
//     the twiddle tables must fit kTwiddleElems (2^16 complex values);
//   * both arrays exist once per device for the lifetime of the process and
//     are shared by every call: calls that overlap on the GPU (different
//     streams, no ordering) race on them.  Nothing in them has to start at
//     zero: the twiddle kernel rewrites every table entry and the first pass
//     writes every scratch element before the second pass reads it;
//   * the first call on a device resolves the arrays' device addresses with
//     cudaGetSymbolAddress (once per device), so that first call should
//     happen before any stream capture;
//   * idata and odata must be device pointers of the current device (or
//     managed pointers); idata == odata is allowed because the intermediate
//     never touches the caller's buffers.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/aclfft_ext.h"
#include "../lib/planner.h"
#include "kernel_args.h"

namespace gfft {
void set_last_error(const std::string& s);
}

namespace {

constexpr long long kScratchElems = 1ll << 21;  // complex values
constexpr long long kTwiddleElems = 1ll << 16;  // complex values
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float2 g_noalloc_scratch[kScratchElems];
static __device__ __align__(256) float2 g_noalloc_twiddles[kTwiddleElems];

struct DeviceAddrs {
    float2* scratch = nullptr;
    float2* twiddles = nullptr;
};

DeviceAddrs g_addrs[kMaxDevices];
std::mutex g_addrs_mu;
thread_local std::string g_noalloc_error;

// Once per device, with that device current: host-side names of the arrays
// are stand-ins, the kernels need their device addresses.
cudaError_t device_addrs(int dev, DeviceAddrs& out)
{
    std::lock_guard<std::mutex> lk(g_addrs_mu);
    DeviceAddrs& a = g_addrs[dev];
    if (!a.scratch) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        void* q = nullptr;
        e = cudaGetSymbolAddress(&q, g_noalloc_twiddles);
        if (e != cudaSuccess) return e;
        a.scratch = static_cast<float2*>(p);
        a.twiddles = static_cast<float2*>(q);
    }
    out = a;
    return cudaSuccess;
}

// Device memory of the current device `dev`, or managed memory.  Device
// memory of another GPU is refused: the kernels would dereference it as a
// peer address, which faults when peer access is not enabled.
bool is_local_device_pointer(const void* p, int dev)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    return at.type == cudaMemoryTypeDevice && at.device == dev;
}

aclfftResult fail(aclfftResult code, const std::string& why)
{
    g_noalloc_error = why;
    gfft::set_last_error(why);
    return code;
}

}  // namespace

extern "C" ACLFFT_API aclfftResult aclfftExecC2CNoAlloc(const aclfftComplex* idata, aclfftComplex* odata, int nx,
                                                        int batch, int direction, cudaStream_t stream)
{
    if (!idata || !odata) return fail(ACLFFT_INVALID_VALUE, "NULL data pointer");
    if (nx <= 0 || batch <= 0) return fail(ACLFFT_INVALID_SIZE, "nx and batch must be positive");
    if (direction != ACLFFT_FORWARD && direction != ACLFFT_BACKWARD)
        return fail(ACLFFT_INVALID_VALUE, "direction must be ACLFFT_FORWARD or ACLFFT_BACKWARD");
    if ((long long)nx * (long long)batch > kScratchElems)
        return fail(ACLFFT_INVALID_SIZE, "nx * batch exceeds the 2^21-element scratch of the allocation-free entry");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(ACLFFT_EXEC_FAILED, "no current CUDA device");
    }
    if (!is_local_device_pointer(idata, dev) || !is_local_device_pointer(odata, dev))
        return fail(ACLFFT_INVALID_VALUE,
                    "the allocation-free entry takes device pointers of the current device only");

    gfft::TwiddleBuilder tb;
    std::vector<gfft::Step> steps;
    if (!gfft::build_scratch_c2c_steps(nx, batch, tb, steps))
        return fail(ACLFFT_NOT_IMPLEMENTED, "nx does not split into two on-chip factors (prime factors <= 47)");
    if (tb.count > kTwiddleElems) return fail(ACLFFT_INVALID_SIZE, "twiddle tables exceed the fixed table size");

    DeviceAddrs a;
    const cudaError_t e = device_addrs(dev, a);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(ACLFFT_EXEC_FAILED, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    }
    if (gfft_gen_twiddles(a.twiddles, tb.segs.data(), (int)tb.segs.size(), stream) != 0) {
        cudaGetLastError();
        return fail(ACLFFT_EXEC_FAILED, "twiddle generation launch failed");
    }
    const bool inverse = direction == ACLFFT_BACKWARD;
    void* bufs[4] = {const_cast<aclfftComplex*>(idata), odata, a.scratch, nullptr};
    for (size_t i = 0; i < steps.size(); ++i) {
        gfft::ColArgs c = steps[i].col;
        c.tw = a.twiddles;
        c.otw_hi = steps[i].hi_off >= 0 ? a.twiddles + steps[i].hi_off : nullptr;
        c.otw_lo = steps[i].lo_off >= 0 ? a.twiddles + steps[i].lo_off : nullptr;
        c.in = bufs[steps[i].src];
        c.out = bufs[steps[i].dst];
        c.conj_in = (i == 0) && inverse;
        c.conj_out = (i + 1 == steps.size()) && inverse;
        c.scale = 1.f;
        if (gfft_launch_col(&c, stream) != 0) {
            cudaGetLastError();
            return fail(ACLFFT_EXEC_FAILED, "column pass launch failed");
        }
    }
    return ACLFFT_SUCCESS;
}
