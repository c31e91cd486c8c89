// ragged.cu - ragged batches of transforms in one persistent launch.
//
// Every CTA loops: claim the next work item from the queue head (one atomic
// per item), read its descriptor and class from the device tables, run it,
// and for the steps of long transforms publish completion on the
// transform's counter.  Items are the on-chip Stockham transforms of the
// row / column kernels (the same pass code, run_passes), parameterised per
// item instead of per launch:
//
//   RAG_SINGLE  `count` same-class transforms, one thread group each, rows
//               in shared memory at a padded pitch; even R2C fuses the
//               even/odd post-process, odd R2C reads reals and keeps bins
//               k <= n/2.
//   RAG_P1      `count` adjacent columns j of a long transform (length
//               L1 = ip.L transforms of x[j + L2*i]) into the workspace.
//   RAG_P2      `count` rows k1 of the workspace, each multiplied by
//               W_L^{k1*n2} and transformed (length L2), written to
//               X[k1 + L1*k2] (or to the second workspace half for R2C).
//   RAG_POST    the even/odd post-process of a long even R2C.
//
// Waits (P2 on P1, POST on P2) are done by one thread with a clock bound;
// the queue order guarantees the awaited items are already running.
#include <cuda_runtime.h>

#include "butterfly.cuh"
#include "kernel_args.h"
#include "stockham.cuh"

namespace gfft {
namespace {

constexpr int kRagThreads = 256;

struct RagCtx {
    int L, nthr, tid, tl;
    bool ok_sm, ok_io;
    bool rows;  // shared layout: rows [tl][spad(i)] at `pitch`, else columns [i][tl] at `tfp`
    int pitch, tfp;
    const float2* tw;
    float2* sA;
    float2* sB;
    const float2* gin;  // complex input, element i at gin[i * in_stride]
    const float* rin;   // real input (odd R2C), element i at rin[i * in_stride]
    bool real_in, coherent;
    float2* gout;
    int64_t in_stride, out_stride;
    bool conj_in, conj_out;
    float scale;
    // input twiddle W^{jm*i} = hi[e >> shift] * lo[e & mask]
    bool otw;
    unsigned jm;
    const float2* hi;
    const float2* lo;
    int shift;
    unsigned mask;
    // output bins kept: k = kb + km*i <= kmax (kmax < 0: all)
    int kb, km, kmax;

    __device__ __forceinline__ float2* buf(int b) const { return b == 1 ? sA : sB; }
    __device__ __forceinline__ int sidx(int i) const { return rows ? tl * pitch + spad(i) : i * tfp + tl; }
    __device__ __forceinline__ float2 sget(int b, int i) const { return buf(b)[sidx(i)]; }
    __device__ __forceinline__ void sput(int b, int i, float2 x) const { buf(b)[sidx(i)] = x; }
    __device__ __forceinline__ float2 gload(int i) const
    {
        float2 x;
        if (real_in) x = make_float2(__ldg(rin + (int64_t)i * in_stride), 0.f);
        else if (coherent) x = __ldcg(gin + (int64_t)i * in_stride);
        else x = ldg2(gin + (int64_t)i * in_stride);
        if (conj_in) x = cconj(x);
        if (otw) {
            const unsigned e = jm * (unsigned)i;
            x = cmul(x, cmul(ldg2(hi + (e >> shift)), ldg2(lo + (e & mask))));
        }
        return x;
    }
    __device__ __forceinline__ void gstore(int i, float2 x) const
    {
        if (kmax >= 0 && kb + km * i > kmax) return;
        if (conj_out) x = cconj(x);
        gout[(int64_t)i * out_stride] = cscale(x, scale);
    }
};

// Even/odd post-process of an even-length R2C: Z (L = n/2 complex) -> the
// n/2 + 1 bins X, bins k and L - k from Z[k] and Z[L - k].
template <class GetZ>
__device__ __forceinline__ void r2c_post(GetZ getz, const float2* post, float2* out, int L, int t0, int tstep)
{
    for (int k = t0; k <= L / 2; k += tstep) {
        if (k == 0) {
            const float2 z0 = getz(0);
            out[0] = make_float2(z0.x + z0.y, 0.f);
            out[L] = make_float2(z0.x - z0.y, 0.f);
            continue;
        }
        const float2 zk = getz(k), zc = cconj(getz(L - k));
        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
        const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
        const float2 wo = cmul(ldg2(post + k), o);
        out[k] = cadd(e, wo);
        if (L - k != k) out[L - k] = cconj(csub(e, wo));
    }
}

// Copies a class's pass-table window into shared memory and returns the
// pointer that makes `tw + pass.tw_off` address it (the window starts at
// blob offset lo).
__device__ __forceinline__ const float2* stage_twiddles(const float2* tw, int64_t lo, int cnt, float2* dst)
{
    if (cnt <= 0) return tw;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) dst[i] = ldg2(tw + lo + i);
    __syncthreads();
    return dst - lo;
}

__device__ __forceinline__ bool wait_count(int* ctr, int need, int* err, long long budget)
{
    if (budget <= 0) budget = 1ll << 31;
    const long long t0 = clock64();
    while (atomicAdd(ctr, 0) < need) {
        if (*reinterpret_cast<volatile int*>(err) & 4) return false;
        __nanosleep(128);
        if (clock64() - t0 > budget) {
            atomicOr(err, 4);
            return false;
        }
    }
    __threadfence();
    return true;
}

template <int RMAX>
__global__ void __launch_bounds__(kRagThreads, 2) ragged_kernel(const __grid_constant__ RagArgs A)
{
    extern __shared__ float2 smem[];
    __shared__ int s_item;
    __shared__ int s_ok;
    const float2* tw = static_cast<const float2*>(A.tw);
    float2* const ws = static_cast<float2*>(A.ws);
    for (;;) {
        __syncthreads();  // the previous item is done with shared memory and s_item
        if (threadIdx.x == 0) s_item = atomicAdd(A.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= A.nitems) break;
        const RagItem item = A.items[it];
        const RagClass& C = A.cls[item.cls];
        const int type = C.type;
        if (item.kind == RAG_P2 || item.kind == RAG_POST) {
            if (threadIdx.x == 0) s_ok = wait_count(A.queue + 1 + item.xform, item.need + A.need_bias, A.err, A.wait_cycles) ? 1 : 0;
            __syncthreads();
            if (!s_ok) continue;
        }

        RagCtx c;
        c.tw = tw;
        c.sA = smem;
        c.real_in = false;
        c.rin = nullptr;
        c.coherent = false;
        c.otw = false;
        c.jm = 0;
        c.hi = c.lo = nullptr;
        c.shift = 0;
        c.mask = 0;
        c.kb = 0;
        c.km = 0;
        c.kmax = -1;
        c.scale = 1.f;
        const bool c2c = type == RAG_C2C;
        const bool odd_r2c = type == RAG_R2C && (C.n & 1);

        if (item.kind == RAG_SINGLE) {
            c.tw = stage_twiddles(tw, C.tw_lo, C.tw_cnt, smem + C.tw_smem);
            const int nthr = C.ip.nthr;
            c.L = C.L;
            c.nthr = nthr;
            c.tid = threadIdx.x % nthr;
            c.tl = threadIdx.x / nthr;
            c.rows = true;
            c.pitch = C.pitch;
            c.tfp = 1;
            c.sB = smem + C.group * C.pitch;
            c.ok_sm = c.tl < C.group;
            c.ok_io = c.tl < item.count;
            const RagXform x = A.xf[A.order[item.first + (c.ok_io ? c.tl : 0)]];
            const char* ib = static_cast<const char*>(A.in) + x.in_off;
            char* ob = static_cast<char*>(A.out) + x.out_off;
            c.gin = reinterpret_cast<const float2*>(ib);
            c.rin = reinterpret_cast<const float*>(ib);
            c.real_in = odd_r2c;
            c.in_stride = c.out_stride = 1;
            c.gout = reinterpret_cast<float2*>(ob);
            c.conj_in = c2c && A.inverse;
            c.conj_out = c2c && A.inverse;
            if (c2c) c.scale = A.scale_c2c;
            if (c2c) {
                run_passes<RMAX>(c, C.ip, 0, true);
            } else if (!odd_r2c) {
                const int fin = run_passes<RMAX>(c, C.ip, 0, false);
                if (c.ok_io) {
                    const float2* z = c.buf(fin);
                    const int base = c.tl * c.pitch;
                    r2c_post([&](int k) { return z[base + spad(k)]; }, tw + C.post_off, c.gout, C.L, c.tid, nthr);
                }
            } else {
                const int fin = run_passes<RMAX>(c, C.ip, 0, false);
                if (c.ok_io) {
                    const float2* z = c.buf(fin);
                    for (int k = c.tid; k <= C.n / 2; k += nthr) c.gout[k] = z[c.tl * c.pitch + spad(k)];
                }
            }
        } else if (item.kind == RAG_P1) {
            c.tw = stage_twiddles(tw, C.tw_lo, C.tw_cnt, smem + C.tw_smem);
            const int tf = C.group;
            const RagXform x = A.xf[item.xform];
            c.L = C.L1;
            c.nthr = C.ip.nthr;
            c.tl = threadIdx.x % tf;
            c.tid = threadIdx.x / tf;
            c.rows = false;
            c.pitch = 0;
            c.tfp = tf + 1;
            c.sB = smem + (int64_t)C.L1 * c.tfp;
            c.ok_sm = c.tid < c.nthr;
            c.ok_io = c.ok_sm && c.tl < item.count;
            const int j = item.first + (c.ok_io ? c.tl : 0);
            const char* ib = static_cast<const char*>(A.in) + x.in_off;
            c.gin = reinterpret_cast<const float2*>(ib) + j;
            c.rin = reinterpret_cast<const float*>(ib) + j;
            c.real_in = odd_r2c;
            c.in_stride = C.L2;
            c.gout = ws + x.ws_off + j;
            c.out_stride = C.L2;
            c.conj_in = c2c && A.inverse;
            c.conj_out = false;
            run_passes<RMAX>(c, C.ip, 0, true);
        } else if (item.kind == RAG_P2) {
            c.tw = stage_twiddles(tw, C.tw2_lo, C.tw2_cnt, smem + C.tw2_smem);
            const int nthr = C.ip2.nthr;
            const RagXform x = A.xf[item.xform];
            c.L = C.L2;
            c.nthr = nthr;
            c.tid = threadIdx.x % nthr;
            c.tl = threadIdx.x / nthr;
            c.rows = true;
            c.pitch = C.pitch;
            c.tfp = 1;
            c.sB = smem + C.group2 * C.pitch;
            c.ok_sm = c.tl < C.group2;
            c.ok_io = c.tl < item.count;
            const int k1 = item.first + (c.ok_io ? c.tl : 0);
            c.gin = ws + x.ws_off + (int64_t)k1 * C.L2;
            c.coherent = true;
            c.in_stride = 1;
            c.otw = true;
            c.jm = (unsigned)k1;
            c.hi = tw + C.hi_off;
            c.lo = tw + C.lo_off;
            c.shift = C.otw_shift;
            c.mask = (1u << C.otw_shift) - 1u;
            c.out_stride = C.L1;
            c.conj_in = false;
            if (c2c) {
                c.gout = reinterpret_cast<float2*>(static_cast<char*>(A.out) + x.out_off) + k1;
                c.conj_out = A.inverse != 0;
                c.scale = A.scale_c2c;
            } else if (!odd_r2c) {
                c.gout = ws + x.ws_off + C.L + k1;
                c.conj_out = false;
            } else {
                c.gout = reinterpret_cast<float2*>(static_cast<char*>(A.out) + x.out_off) + k1;
                c.conj_out = false;
                c.kb = k1;
                c.km = C.L1;
                c.kmax = C.n / 2;
            }
            run_passes<RMAX>(c, C.ip2, 0, true);
        } else {  // RAG_POST
            const RagXform x = A.xf[item.xform];
            const float2* z = ws + x.ws_off + C.L;
            float2* out = reinterpret_cast<float2*>(static_cast<char*>(A.out) + x.out_off);
            r2c_post([&](int k) { return __ldcg(z + k); }, tw + C.post_off, out, C.L, threadIdx.x, kRagThreads);
        }

        if (item.kind == RAG_P1 || item.kind == RAG_P2) {
            // release: the CTA barrier orders every thread's stores before
            // thread 0's fence, which orders them before the counter update
            __syncthreads();
            if (threadIdx.x == 0) {
                __threadfence();
                atomicAdd(A.queue + 1 + item.xform, 1);
            }
        }
    }
}

}  // namespace
}  // namespace gfft

using namespace gfft;

extern "C" int gfft_ragged_ctas(int smem_bytes)
{
    // the kernel's static shared memory counts against the opt-in limit, so
    // the attribute is the dynamic size actually launched with
    int occ = 0;
    cudaError_t e = cudaFuncSetAttribute(ragged_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ragged_kernel<16>, kRagThreads, (size_t)smem_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return -(int)e;
    }
    return occ;
}

extern "C" int gfft_launch_ragged(const RagArgs* a, void* stream)
{
    // stream-ordered work only (capturable): attributes and residency come
    // from gfft_ragged_ctas, called beforehand
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (a->nitems <= 0) return 0;
    if (a->smem_bytes <= 0 || a->smem_bytes > kMaxSmemBytes || a->ctas <= 0) return (int)cudaErrorInvalidValue;
    const int grid = a->ctas < a->nitems ? a->ctas : a->nitems;
    ragged_kernel<16><<<(unsigned)grid, kRagThreads, (size_t)a->smem_bytes, st>>>(*a);
    return (int)cudaGetLastError();
}
