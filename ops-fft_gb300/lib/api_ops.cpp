// api_ops.cpp - the reference's per-operator direct entries (aclfft_ops.h).
//
// Each entry checks its arguments in the reference's order and with its
// codes (the file:line of every rule is in aclfft_ops.h), then runs the
// transform through a plan of this library, cached per calling thread and
// shape so repeated calls do not re-plan.  The reference maps an entry's
// ACL_ERROR_INVALID_PARAM to ACLFFT_NOT_IMPLEMENTED in its dispatchers
// (src/fft1_d/arch32/fft1_d_exec_api.cpp:148-152); the reverse mapping is
// used here for the plan results.
#include <climits>
#include <cstdint>
#include <list>
#include <tuple>

#include "../../include/aclfft_ops.h"
#include "handle.h"

namespace {

struct PlanKey {
    int type, rank, n0, n1, batch, dim, norm;
    bool operator==(const PlanKey& o) const
    {
        return std::tie(type, rank, n0, n1, batch, dim, norm) ==
               std::tie(o.type, o.rank, o.n0, o.n1, o.batch, o.dim, o.norm);
    }
};

// Least-recently-used plans of this thread (a plan is not thread-safe, and
// one thread's calls are ordered).
class PlanCache {
public:
    ~PlanCache()
    {
        for (auto& e : plans_) aclfftDestroy(e.second);
    }
    aclfftResult get(const PlanKey& k, aclfftHandle* out)
    {
        for (auto it = plans_.begin(); it != plans_.end(); ++it) {
            if (it->first == k) {
                plans_.splice(plans_.begin(), plans_, it);
                *out = plans_.front().second;
                return ACLFFT_SUCCESS;
            }
        }
        aclfftHandle h = nullptr;
        aclfftResult r = k.rank == 2 ? aclfftPlan2d(&h, k.batch, k.n0, k.n1, (aclfftType)k.type)
                                     : aclfftPlan1d(&h, k.n0, (aclfftType)k.type, k.batch, k.dim);
        if (r != ACLFFT_SUCCESS) return r;
        if (k.norm != ACLFFT_NORM_NONE && (r = aclfftSetNormMode(h, k.norm)) != ACLFFT_SUCCESS) {
            aclfftDestroy(h);
            return r;
        }
        plans_.emplace_front(k, h);
        if (plans_.size() > kMax) {
            aclfftDestroy(plans_.back().second);
            plans_.pop_back();
        }
        *out = h;
        return ACLFFT_SUCCESS;
    }

private:
    static constexpr size_t kMax = 8;
    std::list<std::pair<PlanKey, aclfftHandle>> plans_;
};

thread_local PlanCache t_plans;

aclError to_acl(aclfftResult r)
{
    switch (r) {
    case ACLFFT_SUCCESS: return ACL_SUCCESS;
    case ACLFFT_NOT_IMPLEMENTED:
    case ACLFFT_NOT_SUPPORTED:
    case ACLFFT_INVALID_SIZE:
    case ACLFFT_INVALID_VALUE:
    case ACLFFT_INVALID_TYPE: return ACL_ERROR_INVALID_PARAM;
    case ACLFFT_ALLOC_FAILED: return ACL_ERROR_BAD_ALLOC;
    default: return ACL_ERROR_INTERNAL_ERROR;
    }
}

aclError reject(const char* entry, const char* why)
{
    GFFT_LOG("%s: %s", entry, why);
    gfft::set_last_error(std::string(entry) + ": " + why);
    return ACL_ERROR_INVALID_PARAM;
}

bool pow2(uint32_t n) { return n != 0 && (n & (n - 1)) == 0; }

enum class Op { C2C, R2C, C2R };

// Runs one transform through the calling thread's cached plan.
aclError run(Op op, const PlanKey& k, float* x, float* y, int isForward, void* stream)
{
    aclfftHandle h = nullptr;
    aclfftResult r = t_plans.get(k, &h);
    if (r != ACLFFT_SUCCESS) return to_acl(r);
    if ((r = aclfftSetStream(h, static_cast<cudaStream_t>(stream))) != ACLFFT_SUCCESS) return to_acl(r);
    switch (op) {
    case Op::C2C:
        r = aclfftExecC2C(h, reinterpret_cast<aclfftComplex*>(x), reinterpret_cast<aclfftComplex*>(y),
                          isForward ? ACLFFT_FORWARD : ACLFFT_BACKWARD);
        break;
    case Op::R2C: r = aclfftExecR2C(h, x, reinterpret_cast<aclfftComplex*>(y)); break;
    case Op::C2R: r = aclfftExecC2R(h, reinterpret_cast<aclfftComplex*>(x), y); break;
    }
    return to_acl(r);
}

PlanKey key1d(aclfftType t, uint32_t n, uint32_t batches, int norm = ACLFFT_NORM_NONE)
{
    return PlanKey{(int)t, 1, (int)n, 1, (int)batches, ACLFFT_HORIZONTAL, norm};
}

// Checks shared by the C2C entries with a norm argument (NULL pointers, norm,
// isForward, batches = 0), in the reference's order.
aclError c2c_common(const char* entry, const float* x, const float* y, int32_t norm, uint32_t batches, int isForward)
{
    if (!x || !y) return reject(entry, "input/output pointer is null");
    if (norm != 0) return reject(entry, "norm is not supported (only 0 = no scaling)");
    if (isForward != 0 && isForward != 1) return reject(entry, "isForward invalid (expected 0 or 1)");
    (void)batches;
    return ACL_SUCCESS;
}

aclError c2c_plain(const char* entry, float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                   void* stream, uint32_t nmax)
{
    const aclError e = c2c_common(entry, x, y, norm, batches, isForward);
    if (e != ACL_SUCCESS) return e;
    if (n == 0 || n > nmax) return reject(entry, "n out of the supported range");
    if (batches == 0) return reject(entry, "batches=0 is not supported");
    if (batches > (uint32_t)INT32_MAX) return reject(entry, "batches exceeds INT32_MAX");
    return run(Op::C2C, key1d(ACLFFT_C2C, n, batches), x, y, isForward, stream);
}

// R2C / C2R entries with norm and isForward (norm 0 only; isForward fixed).
aclError real_entry(Op op, const char* entry, float* x, float* y, uint32_t n, int32_t norm, uint32_t batches,
                    int isForward, void* stream, uint32_t nmax, bool isf_first)
{
    if (!x || !y) return reject(entry, "input/output pointer is null");
    const int want = op == Op::R2C ? 1 : 0;
    if (isf_first && isForward != want) return reject(entry, op == Op::R2C ? "R2C is always forward (isForward must be 1)"
                                                                           : "C2R is always backward (isForward must be 0)");
    if (norm != 0) return reject(entry, "norm is not supported (only 0 = no scaling)");
    if (!isf_first && isForward != want) return reject(entry, op == Op::R2C ? "R2C is always forward (isForward must be 1)"
                                                                            : "C2R is always backward (isForward must be 0)");
    if (n == 0 || n > nmax) return reject(entry, "n out of the supported range");
    if (batches == 0) return reject(entry, "batches=0 is not supported");
    if (batches > (uint32_t)INT32_MAX) return reject(entry, "batches exceeds INT32_MAX");
    return run(op, key1d(op == Op::R2C ? ACLFFT_R2C : ACLFFT_C2R, n, batches), x, y, isForward, stream);
}

// Power-of-two R2C families: rfft1_d_r2c_host_common.h:318-343, then the
// family's own bound.
aclError r2c_pow2(const char* entry, float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream,
                  uint32_t nmin_exclusive, uint32_t nmax)
{
    if (!x || !y) return reject(entry, "input/output pointer is null");
    if (isForward != 1) return reject(entry, "R2C is always forward (isForward must be 1)");
    if (n == 0 || batches == 0) return reject(entry, "n and batches must be positive");
    if (!pow2(n)) return reject(entry, "n is not a power of two");
    if ((uint64_t)batches * ((uint64_t)n + 2) > (1ull << 31)) return reject(entry, "batches*(n+2) exceeds 2^31");
    if (n <= nmin_exclusive || n > nmax) return reject(entry, "n outside this family's range");
    return run(Op::R2C, key1d(ACLFFT_R2C, n, batches), x, y, 1, stream);
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------- C2C
ACLFFT_API aclError aclfftFft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream)
{
    return c2c_plain("aclfftFft1DDft", x, y, n, norm, batches, isForward, stream, 1024);
}

ACLFFT_API aclError aclfftFft1DN(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                 void* stream)
{
    const char* e = "aclfftFft1DN";
    const aclError c = c2c_common(e, x, y, norm, batches, isForward);
    if (c != ACL_SUCCESS) return c;
    if (!pow2(n)) return reject(e, "n must be a power of 2");
    if (n < 64) return reject(e, "n below the minimum 64");
    if (batches == 0) return reject(e, "batches=0 is not supported");
    if (batches > (uint32_t)INT32_MAX) return reject(e, "batches exceeds INT32_MAX");
    if (n > (1u << 27)) return reject(e, "n out of (0, 2^27]");
    return run(Op::C2C, key1d(ACLFFT_C2C, n, batches), x, y, isForward, stream);
}

ACLFFT_API aclError aclfftFft1DStride(float* x, float* y, uint32_t n, int32_t norm, uint32_t stride, uint32_t batches,
                                      int isForward, void* stream)
{
    const char* e = "aclfftFft1DStride";
    const aclError c = c2c_common(e, x, y, norm, batches, isForward);
    if (c != ACL_SUCCESS) return c;
    if (batches != 1) return reject(e, "only a single matrix (batches=1) is supported");
    if (stride == 0) return reject(e, "stride=0 is not supported");
    if (stride % 4 != 0) return reject(e, "stride must be a multiple of 4 (32-byte rows)");
    if ((uint64_t)n * stride > (1ull << 30)) return reject(e, "n*stride exceeds 2^30");
    if (!pow2(n) || n < 256 || n > (1u << 18)) return reject(e, "n must be a power of 2 in [2^8, 2^18]");
    // the VERTICAL encoding of aclfftMakePlan1d: columns = stride
    const PlanKey k{(int)ACLFFT_C2C, 1, (int)n, 1, (int)stride, ACLFFT_VERTICAL, ACLFFT_NORM_NONE};
    return run(Op::C2C, k, x, y, isForward, stream);
}

ACLFFT_API aclError aclfftFft1DB(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                 void* stream)
{
    const char* e = "aclfftFft1DB";
    const aclError c = c2c_common(e, x, y, norm, batches, isForward);
    if (c != ACL_SUCCESS) return c;
    if (batches == 0) return reject(e, "batches=0 is not supported");
    if (!pow2(n) || n < 256 || n > 16384) return reject(e, "n must be a power of 2 in [2^8, 2^14]");
    return run(Op::C2C, key1d(ACLFFT_C2C, n, batches), x, y, isForward, stream);
}

ACLFFT_API aclError aclfftFft1DMix(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream)
{
    return c2c_plain("aclfftFft1DMix", x, y, n, norm, batches, isForward, stream, 1u << 27);
}

ACLFFT_API aclError aclfftFft1DC2C(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                   void* stream)
{
    return c2c_plain("aclfftFft1DC2C", x, y, n, norm, batches, isForward, stream, 1u << 27);
}

ACLFFT_API aclError aclfftFft1DC2CMix(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                      void* stream)
{
    return c2c_plain("aclfftFft1DC2CMix", x, y, n, norm, batches, isForward, stream, 1u << 27);
}

// ------------------------------------------------------------------- R2C
ACLFFT_API aclError aclfftRfft1D(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, void* stream)
{
    const char* e = "aclfftRfft1D";
    if (!x || !y) return reject(e, "input/output pointer is null");
    if (n == 0) return reject(e, "n=0 is not supported");
    if (n > 4096) return reject(e, "n exceeds 4096");
    if (norm < 0 || norm > 2) return reject(e, "norm must be 0 (none), 1 (ortho) or 2 (forward)");
    if (batches == 0) return reject(e, "batches=0 is not supported");
    const int mode = norm == 1 ? ACLFFT_NORM_ORTHO : (norm == 2 ? ACLFFT_NORM_FORWARD : ACLFFT_NORM_NONE);
    return run(Op::R2C, key1d(ACLFFT_R2C, n, batches, mode), x, y, 1, stream);
}

ACLFFT_API aclError aclfftRfft1DR2CFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                       void* stream)
{
    return real_entry(Op::R2C, "aclfftRfft1DR2CFft", x, y, n, norm, batches, isForward, stream, 1u << 27, true);
}

ACLFFT_API aclError aclfftRfft1DFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                    void* stream)
{
    return real_entry(Op::R2C, "aclfftRfft1DFft", x, y, n, norm, batches, isForward, stream, 1u << 27, false);
}

ACLFFT_API aclError aclfftRfft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                    void* stream)
{
    return real_entry(Op::R2C, "aclfftRfft1DDft", x, y, n, norm, batches, isForward, stream, 1024, true);
}

ACLFFT_API aclError aclfftRfft1DR2CFft1(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft1", x, y, n, batches, isForward, stream, 1, 1u << 27);
}

ACLFFT_API aclError aclfftRfft1DR2CFft2(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft2", x, y, n, batches, isForward, stream, 128, 16384);
}

ACLFFT_API aclError aclfftRfft1DR2CFft31(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft31", x, y, n, batches, isForward, stream, 0, 1u << 27);
}

ACLFFT_API aclError aclfftRfft1DR2CFft32(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft32", x, y, n, batches, isForward, stream, 0, 1u << 27);
}

ACLFFT_API aclError aclfftRfft1DR2CFft4(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft4", x, y, n, batches, isForward, stream, 0, 1u << 27);
}

ACLFFT_API aclError aclfftRfft1DR2CFft5(float* x, float* y, uint32_t n, uint32_t batches, int isForward, void* stream)
{
    return r2c_pow2("aclfftRfft1DR2CFft5", x, y, n, batches, isForward, stream, 3, 1u << 27);
}

// ------------------------------------------------------------------- C2R
ACLFFT_API aclError aclfftIrfft1DFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                     void* stream)
{
    return real_entry(Op::C2R, "aclfftIrfft1DFft", x, y, n, norm, batches, isForward, stream, 1u << 27, false);
}

ACLFFT_API aclError aclfftIrfft1DDft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                     void* stream)
{
    return real_entry(Op::C2R, "aclfftIrfft1DDft", x, y, n, norm, batches, isForward, stream, 1024, false);
}

ACLFFT_API aclError aclfftIrfft1DC2RFft(float* x, float* y, uint32_t n, int32_t norm, uint32_t batches, int isForward,
                                        void* stream)
{
    return real_entry(Op::C2R, "aclfftIrfft1DC2RFft", x, y, n, norm, batches, isForward, stream, 1u << 27, true);
}

// -------------------------------------------------------------------- 2D
ACLFFT_API aclError aclfftFft2DDd(float* x, float* y, uint32_t fftX, uint32_t fftY, uint32_t batches, int isForward,
                                  void* stream)
{
    const char* e = "aclfftFft2DDd";
    if (!x || !y) return reject(e, "input/output pointer is null");
    if (isForward != 0 && isForward != 1) return reject(e, "isForward invalid (expected 0 or 1)");
    if (batches == 0) return reject(e, "batches=0 is not supported");
    if (batches > (uint32_t)INT32_MAX) return reject(e, "batches exceeds INT32_MAX");
    if (fftX == 0 || fftY == 0) return reject(e, "fftX and fftY must be positive");
    if (fftX > (uint32_t)INT32_MAX || fftY > (uint32_t)INT32_MAX) return reject(e, "size exceeds INT32_MAX");
    const PlanKey k{(int)ACLFFT_C2C, 2, (int)fftX, (int)fftY, (int)batches, ACLFFT_HORIZONTAL, ACLFFT_NORM_NONE};
    return run(Op::C2C, k, x, y, isForward, stream);
}

}  // extern "C"
