// stockham.cuh - batched on-chip Stockham FFT kernels for sm_103a.
//
// Algorithm (autosort Stockham, the same index maps as the reference's
// arch35 mixed-radix kernel, src/fft1_d/arch35/mix/fft1_d_c2c_mix_kernel.h:
// 29-120, where len = ns*R, prev = ns, part = L/R): a length-L transform is
// L = R_0 * R_1 * ... ; pass p with radix R and ns = R_0*...*R_{p-1} takes
// butterfly j (0 <= j < L/R), reads x[j + r*L/R], multiplies input r by
// W_{ns*R}^{(j%ns)*r}, runs an in-register R-point DFT and writes output r to
// y[(j/ns)*ns*R + j%ns + r*ns].  After the last pass y is in natural order.
//
// GB300 mapping:
//   * the whole transform lives in shared memory (one HBM read, one HBM
//     write per element); a pass streams butterflies from one shared buffer
//     to the other (ping-pong), one R-point butterfly in registers at a time;
//   * the first pass reads HBM directly and the last pass writes HBM
//     directly: both access patterns (x[j + r*L/R] and y[j + r*L/R]) are
//     unit-stride across consecutive threads, i.e. fully coalesced;
//   * shared memory is padded by one float2 every 16 (pad(i) = i + i/16),
//     which makes the stride-R Stockham writes of the early passes
//     bank-conflict free for power-of-two radices;
//   * backward transforms are conj(F(conj(x))) so only forward butterflies
//     and forward twiddle tables exist;
//   * real-data transforms (R2C/C2R) run an L = N/2 complex transform with
//     the even/odd packing fused into the shared-memory phase before the
//     first pass (C2R) or after the last pass (R2C).
//
// Row kernel: one transform per batch item, consecutive threads walk along
// the transform.  Column kernel: TF strided transforms per CTA, consecutive
// threads walk across neighbouring columns so strided HBM accesses still
// coalesce; it also carries the inter-pass twiddle of multi-pass (four-step
// style) transforms, 2D column passes and VERTICAL layouts.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterfly.cuh"
#include "kernel_args.h"
#include "pdl.cuh"

namespace gfft {

__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }

__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }

// Fast j / ns for j, ns < 2^16 (ns > 1).
__device__ __forceinline__ int fdiv(int j, const PassDesc& pd)
{
    return pd.ns == 1 ? j : (int)__umulhi((unsigned)j, pd.ns_magic);
}

// e / L for e < 2^22 using a single float multiply (error < 0.5/L).
__device__ __forceinline__ int fdivf(int e, float invL) { return __float2int_rz(((float)e + 0.5f) * invL); }

// --------------------------------------------------------------- one pass
// c.tw may point to shared memory (row kernel) or global memory (column
// kernel), so twiddles are read with generic loads.
// Buffers: 0 = HBM (the Ctx's gload/gstore), 1 = shared buffer A,
// 2 = shared buffer B.  Each thread walks butterflies j = tid, tid+nthr, ...
// and streams them from the source to the destination buffer, so a pass
// never holds more than one butterfly (R values) in registers and source and
// destination must differ (ping-pong).
template <int R, class Ctx>
__device__ __forceinline__ void stockham_pass(const Ctx& c, const PassDesc& pd, int src, int dst)
{
    const int nbf = c.L / R;
    const bool act_g = c.ok_io;
    const bool act_s = c.ok_sm;
    for (int j = c.tid; j < nbf; j += c.nthr) {
        float2 u[R];
        if (src == 0) {
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                u[r] = act_g ? c.gload(j + r * nbf) : make_float2(0.f, 0.f);
            });
        } else {
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                u[r] = act_s ? c.sget(src, j + r * nbf) : make_float2(0.f, 0.f);
            });
        }
        if (pd.ns > 1) {
            const int q = fdiv(j, pd);
            const int k = j - q * pd.ns;
            const float2* w = c.tw + pd.tw_off + k;  // entry r*ns + k
            sfor<R - 1>([&](auto rr) {
                constexpr int r = decltype(rr)::value + 1;
                u[r] = cmul(u[r], w[r * pd.ns]);
            });
        }
        DFT<R>::run(u);
        if (dst == 0) {
            // only the last pass writes HBM: ns == L/R, so the output of
            // butterfly j sits at j + r*ns (unit stride across threads)
            if (act_g) {
                sfor<R>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    c.gstore(j + r * pd.ns, u[r]);
                });
            }
        } else if (act_s) {
            const int q = fdiv(j, pd);
            const int k = j - q * pd.ns;
            const int base = q * pd.ns * R + k;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                c.sput(dst, base + r * pd.ns, u[r]);
            });
        }
    }
    __syncthreads();
}

// Passes of the large primes (17..47) are rare; keeping them out of line
// keeps the radix-47 kernels' code size and compile time bounded.
template <int R, class Ctx>
__device__ __noinline__ void stockham_pass_outlined(const Ctx& c, const PassDesc& pd, int src, int dst)
{
    stockham_pass<R>(c, pd, src, dst);
}

#define GFFT_RADIX_CASE(RV)                                                 \
    case RV:                                                                \
        if constexpr (RV <= RMAX) {                                         \
            if constexpr (RV > 16) stockham_pass_outlined<RV>(c, pd, src, dst); \
            else stockham_pass<RV>(c, pd, src, dst);                        \
        }                                                                   \
        break;

// Runs all passes.  `start` is where the data is (0 = HBM, 1 = buffer A);
// when `last_global` the final pass writes HBM, otherwise the result ends in
// the shared buffer that is returned (1 or 2).
template <int RMAX, class Ctx>
__device__ __forceinline__ int run_passes(const Ctx& c, const InnerPlan& ip, int start, bool last_global,
                                          int p_begin = 0, int p_end = kMaxPass)
{
    int cur = start;
    const int pe = p_end < ip.npass ? p_end : ip.npass;
    for (int p = p_begin; p < pe; ++p) {
        const PassDesc pd = ip.pass[p];
        const int src = cur;
        const int dst = (last_global && p == ip.npass - 1) ? 0 : (cur == 1 ? 2 : 1);
        switch (pd.radix) {
            GFFT_RADIX_CASE(1)
            GFFT_RADIX_CASE(2)
            GFFT_RADIX_CASE(3)
            GFFT_RADIX_CASE(4)
            GFFT_RADIX_CASE(5)
            GFFT_RADIX_CASE(6)
            GFFT_RADIX_CASE(7)
            GFFT_RADIX_CASE(8)
            GFFT_RADIX_CASE(9)
            GFFT_RADIX_CASE(10)
            GFFT_RADIX_CASE(11)
            GFFT_RADIX_CASE(12)
            GFFT_RADIX_CASE(13)
            GFFT_RADIX_CASE(14)
            GFFT_RADIX_CASE(15)
            GFFT_RADIX_CASE(16)
            GFFT_RADIX_CASE(17)
            GFFT_RADIX_CASE(19)
            GFFT_RADIX_CASE(23)
            GFFT_RADIX_CASE(29)
            GFFT_RADIX_CASE(31)
            GFFT_RADIX_CASE(37)
            GFFT_RADIX_CASE(41)
            GFFT_RADIX_CASE(43)
            GFFT_RADIX_CASE(47)
        default:
            break;
        }
        cur = dst;
    }
    return cur;
}
#undef GFFT_RADIX_CASE

template <int RMAX>
constexpr int kernel_max_threads()
{
    return RMAX <= 16 ? 512 : 256;
}

// ========================================================= column kernel
struct ColCtx {
    int L, nthr, tid, tl, tfp;
    bool ok_sm, ok_io;
    const float2* tw;
    float2* sA;
    float2* sB;
    const float2* gin;  // column base, element r at gin[r*in_stride]
    float2* gout;
    int64_t in_stride, out_stride;
    int conj_in, conj_out;
    float scale;
    // outer twiddle
    bool otw;
    int jm;  // (j / tw_div) % ons
    const float2* hi;
    const float2* lo;
    int shift;
    unsigned mask;

    __device__ __forceinline__ float2* buf(int b) const { return b == 1 ? sA : sB; }
    __device__ __forceinline__ float2 sget(int b, int i) const { return buf(b)[i * tfp + tl]; }
    __device__ __forceinline__ void sput(int b, int i, float2 x) const { buf(b)[i * tfp + tl] = x; }
    __device__ __forceinline__ float2 gload(int i) const
    {
        float2 x = ldg2(gin + (int64_t)i * in_stride);
        if (conj_in) x = cconj(x);
        if (otw) {
            const unsigned m = (unsigned)jm * (unsigned)i;
            x = cmul(x, cmul(ldg2(hi + (m >> shift)), ldg2(lo + (m & mask))));
        }
        return x;
    }
    __device__ __forceinline__ void gstore(int i, float2 x) const
    {
        if (conj_out) x = cconj(x);
        gout[(int64_t)i * out_stride] = cscale(x, scale);
    }
};

// Shared-memory layout: buffer A = [L][tfp] at smem, buffer B right after.
template <int RMAX>
__device__ __forceinline__ void col_body(const ColArgs& A)
{
    extern __shared__ float2 smem[];
    const int tf = A.tfpc;
    const int tl = threadIdx.x % tf;
    const int tid = threadIdx.x / tf;
    const int64_t c0 = (int64_t)blockIdx.x * tf;
    const int64_t col = c0 + tl;

    ColCtx c;
    c.L = A.ip.L;
    c.nthr = A.ip.nthr;
    c.tid = tid;
    c.tl = tl;
    c.tfp = A.tfp;
    c.ok_sm = tid < c.nthr;
    c.ok_io = c.ok_sm && col < A.ncols;
    c.tw = reinterpret_cast<const float2*>(A.tw);
    c.sA = smem;
    c.sB = smem + (int64_t)A.ip.L * A.tfp;
    c.in_stride = A.in_stride;
    c.out_stride = A.out_stride;
    c.conj_in = A.conj_in;
    c.conj_out = A.conj_out;
    c.scale = A.scale;
    const int64_t cc = c.ok_io ? col : 0;
    const int64_t item = cc / A.cpi;
    const int64_t j = cc - item * A.cpi;
    c.gin = reinterpret_cast<const float2*>(A.in) + item * A.in_dist + (j / A.in_split) * A.in_hi +
            (j % A.in_split) * A.in_lo;
    c.gout = reinterpret_cast<float2*>(A.out) + item * A.out_dist + (j / A.out_split) * A.out_hi +
             (j % A.out_split) * A.out_lo;
    c.otw = A.ons > 1;
    c.jm = c.otw ? (int)((j / A.tw_div) % A.ons) : 0;
    c.hi = reinterpret_cast<const float2*>(A.otw_hi);
    c.lo = reinterpret_cast<const float2*>(A.otw_lo);
    c.shift = A.otw_shift;
    c.mask = (1u << A.otw_shift) - 1u;

    const bool staged = A.staged_out != 0;
    const int fin = run_passes<RMAX>(c, A.ip, 0, !staged);
    if (staged) {
        // column c's L outputs are contiguous at out + c*L: copy the CTA's
        // block column by column so consecutive threads write consecutive bins
        const int L = c.L;
        const float2* s = c.buf(fin);
        float2* g = reinterpret_cast<float2*>(A.out) + c0 * L;
        const int ncol = (int)min((int64_t)tf, A.ncols - c0);
        for (int q = 0; q < ncol; ++q) {
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                float2 x = s[k * A.tfp + q];
                if (A.conj_out) x = cconj(x);
                g[(int64_t)q * L + k] = cscale(x, A.scale);
            }
        }
    }
}

template <int RMAX>
__global__ void __launch_bounds__(kernel_max_threads<RMAX>()) col_kernel(const __grid_constant__ ColArgs A)
{
    pdl_wait();  // every access below may touch the caller's buffers
    col_body<RMAX>(A);
}

}  // namespace gfft
