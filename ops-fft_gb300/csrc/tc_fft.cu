// tc_fft.cu - split-precision tensor-core sub-transforms (tcgen05 + TMEM).
//
// A launch computes L = R*R point DFTs (R = 16: 256 points, R = 8: 64 points)
// of many sequences, as one pass of a multi-pass C2C transform.  Index split
// n = n_a + R*n_b, k = k_b + R*k_a:
//
//   stage A   y[n_a][k_b] = sum_{n_b} x[n_a + R*n_b] W_R^{n_b*k_b}
//   twiddle   y[n_a][k_b] *= W_L^{n_a*k_b}
//   stage B   X[k_b + R*k_a] = sum_{n_a} y[n_a][k_b] W_R^{n_a*k_a}
//
// Each stage is one real GEMM D[128 x 2R] = A[128 x 2R] * B[2R x 2R]: a row
// of A holds one R-point input vector (real parts, then imaginary parts), B
// is the real-embedded DFT matrix, and a row of D the R-point output.  A tile
// is TS = 128/R sequences: stage A rows are (n_a, t) = n_a*TS + t, stage B
// rows (k_b, t) = k_b*TS + t.  A and B are split into hi + lo parts of the
// operand type (TF32 or BF16) and D = Ahi*Blo + Alo*Bhi + Ahi*Bhi is
// accumulated in FP32 in tensor memory, which keeps about 2^-22 (TF32) or
// 2^-16 (BF16) of relative precision per product.
//
// Per CTA (128 threads, persistent over tiles): cp.async double-buffered
// loads of the next tile into shared memory while the current one runs;
// thread m gathers row m, splits it and writes the K-major operand tile;
// thread 0 issues the MMAs and commits them to an mbarrier; every thread
// reads its D row back from tensor memory (tcgen05.ld), applies the
// twiddles and writes the next operand tile or the output staging tile;
// the output tile is written to HBM with 16-byte coalesced stores.
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices, row r
// of a core matrix at +16*r, the next core matrix along K at +128 (leading
// byte offset) and the next 8-row group at +SBO (stride byte offset).
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterfly.cuh"
#include "kernel_args.h"
#include "pipe_ptx.cuh"
#include "tc_ptx.cuh"

namespace gfft {
namespace {

template <int R_, bool BF16_>
struct TcCfg {
    static constexpr int R = R_;
    static constexpr bool BF16 = BF16_;
    static constexpr int L = R * R;
    static constexpr int TS = 128 / R;               // sequences per tile
    static constexpr int K = 2 * R;                  // GEMM K (= GEMM N)
    static constexpr int ES = BF16 ? 2 : 4;          // operand element bytes
    static constexpr int EPC = 16 / ES;              // elements per core-matrix row
    static constexpr int KSTEP = BF16 ? 16 : 8;      // K of one MMA instruction
    static constexpr uint32_t LBO = 128;
    static constexpr uint32_t SBO = (K / EPC) * 128;
    static constexpr int A_BYTES = 16 * SBO;         // 128 rows
    static constexpr int B_BYTES = (K / 8) * SBO;    // K rows
    static constexpr int PAD = R / 4;                // keeps [t][n] gathers conflict-free
    static constexpr int P = L + PAD;                // [t][n] staging pitch (float2)
    static constexpr int STG = TS * P;               // float2 per staging buffer
    static constexpr int TMEM_COLS = 32;
    static constexpr uint32_t IDESC = BF16 ? tc::idesc_f32acc(tc::kFmtBF16, tc::kFmtBF16, 128, K)
                                           : tc::idesc_f32acc(tc::kFmtTF32, tc::kFmtTF32, 128, K);
    static_assert(K <= TMEM_COLS, "accumulator must fit the allocation");
    static_assert(R % EPC == 0 || EPC % R == 0, "chunks must not straddle the re/im halves");
};

template <class C>
__device__ __forceinline__ uint32_t op_off(int row, int k)
{
    return (uint32_t)(row >> 3) * C::SBO + (uint32_t)(k / C::EPC) * C::LBO + (uint32_t)(row & 7) * 16u +
           (uint32_t)(k % C::EPC) * C::ES;
}

template <class C>
__device__ __forceinline__ size_t smem_bytes_for(int hi_n, int lo_n)
{
    return 2 * C::A_BYTES + 2 * C::B_BYTES + 2 * C::STG * sizeof(float2) +
           (size_t)(C::L + hi_n + lo_n) * sizeof(float2) + 16;
}

// Row m of a stage-A operand tile from R complex values (K index k < R: real
// part of x[k], k >= R: imaginary part of x[k - R]).
template <class C>
__device__ __forceinline__ void put_row(uint8_t* hi, uint8_t* lo, int m, const float2* x)
{
    if constexpr (!C::BF16) {
#pragma unroll
        for (int j = 0; j < C::K / 4; ++j) {
            float h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int k = 4 * j + e;
                const float v = k < C::R ? x[k].x : x[k - C::R].y;
                h[e] = tc::to_tf32(v);
                l[e] = tc::to_tf32(v - h[e]);
            }
            *reinterpret_cast<float4*>(hi + op_off<C>(m, 4 * j)) = make_float4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<float4*>(lo + op_off<C>(m, 4 * j)) = make_float4(l[0], l[1], l[2], l[3]);
        }
    } else {
#pragma unroll
        for (int j = 0; j < C::K / 8; ++j) {
            uint32_t h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                __nv_bfloat16 hv[2], lv[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int k = 8 * j + 2 * e + u;
                    const float v = k < C::R ? x[k].x : x[k - C::R].y;
                    hv[u] = __float2bfloat16_rn(v);
                    lv[u] = __float2bfloat16_rn(v - __bfloat162float(hv[u]));
                }
                h[e] = (uint32_t)__bfloat16_as_ushort(hv[0]) | ((uint32_t)__bfloat16_as_ushort(hv[1]) << 16);
                l[e] = (uint32_t)__bfloat16_as_ushort(lv[0]) | ((uint32_t)__bfloat16_as_ushort(lv[1]) << 16);
            }
            *reinterpret_cast<uint4*>(hi + op_off<C>(m, 8 * j)) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4*>(lo + op_off<C>(m, 8 * j)) = make_uint4(l[0], l[1], l[2], l[3]);
        }
    }
}

// One split element at (row, k) of an operand tile.
template <class C>
__device__ __forceinline__ void put_elem(uint8_t* hi, uint8_t* lo, int row, int k, float v)
{
    const uint32_t off = op_off<C>(row, k);
    if constexpr (!C::BF16) {
        const float h = tc::to_tf32(v);
        *reinterpret_cast<float*>(hi + off) = h;
        *reinterpret_cast<float*>(lo + off) = tc::to_tf32(v - h);
    } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
        *reinterpret_cast<__nv_bfloat16*>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}

// D (tensor memory) = Ahi*Blo + Alo*Bhi + Ahi*Bhi; one thread issues.
template <class C>
__device__ __forceinline__ void issue_gemm(uint32_t tmem, uint32_t ahi, uint32_t alo, uint32_t bhi, uint32_t blo)
{
#pragma unroll
    for (int kk = 0; kk < C::K / C::KSTEP; ++kk) {
        const uint32_t ko = (uint32_t)kk * (C::KSTEP / C::EPC) * C::LBO;
        const uint64_t a_h = tc::sdesc_noswizzle(ahi + ko, C::LBO, C::SBO);
        const uint64_t a_l = tc::sdesc_noswizzle(alo + ko, C::LBO, C::SBO);
        const uint64_t b_h = tc::sdesc_noswizzle(bhi + ko, C::LBO, C::SBO);
        const uint64_t b_l = tc::sdesc_noswizzle(blo + ko, C::LBO, C::SBO);
        if constexpr (C::BF16) {
            tc::mma_f16(tmem, a_h, b_l, C::IDESC, kk > 0);
            tc::mma_f16(tmem, a_l, b_h, C::IDESC, true);
            tc::mma_f16(tmem, a_h, b_h, C::IDESC, true);
        } else {
            tc::mma_tf32(tmem, a_h, b_l, C::IDESC, kk > 0);
            tc::mma_tf32(tmem, a_l, b_h, C::IDESC, true);
            tc::mma_tf32(tmem, a_h, b_h, C::IDESC, true);
        }
    }
}

// This thread's D row (2R columns: real parts, then imaginary parts).
template <class C>
__device__ __forceinline__ void read_row(uint32_t taddr, float2* v)
{
    float f[C::K];
#pragma unroll
    for (int c = 0; c < C::K; c += 16) tc::tmem_ld16_wait(taddr + (uint32_t)c, f + c);
#pragma unroll
    for (int i = 0; i < C::R; ++i) v[i] = make_float2(f[i], f[C::R + i]);
}

// Issues the cp.async copies of tile (first sequence q0) into stg.  All TS
// sequences of a tile belong to the same batch item (checked by the host).
template <class C>
__device__ __forceinline__ void load_tile(const TcArgs& a, int64_t q0, float2* stg, int tid)
{
    const float2* in = static_cast<const float2*>(a.in);
    const int64_t b = q0 / a.S;
    const int64_t s0 = q0 - b * a.S;
    const float2* base = in + b * a.in_dist;
    const int nvalid = (int)((a.nseq - q0) < C::TS ? (a.nseq - q0) : C::TS);
    if (a.in_mode == TC_IO_INTERLEAVED) {
        constexpr int CPN = C::TS / 2;
        for (int c = tid; c < C::L * CPN; c += 128) {
            const int n = c / CPN, tp = c - n * CPN;
            tc::cp_async16(stg + n * C::TS + 2 * tp, base + s0 + 2 * tp + (int64_t)n * a.in_n);
        }
    } else if (a.in_mode == TC_IO_CONTIG) {
        constexpr int CPS = C::L / 2;
        for (int c = tid; c < C::TS * CPS; c += 128) {
            const int t = c / CPS, np = c - t * CPS;
            if (t < nvalid) tc::cp_async16(stg + t * C::P + 2 * np, base + (s0 + t) * a.in_s + 2 * np);
        }
    } else {
        for (int c = tid; c < C::TS * C::L; c += 128) {
            const int t = c / C::L, n = c - t * C::L;
            if (t < nvalid) tc::cp_async8(stg + t * C::P + n, base + (s0 + t) * a.in_s + (int64_t)n * a.in_n);
        }
    }
}

template <class C>
__device__ __forceinline__ void store_tile(const TcArgs& a, int64_t q0, const float2* stg, int tid)
{
    float2* out = static_cast<float2*>(a.out);
    const int64_t b = q0 / a.S;
    const int64_t s0 = q0 - b * a.S;
    float2* base = out + b * a.out_dist;
    const int nvalid = (int)((a.nseq - q0) < C::TS ? (a.nseq - q0) : C::TS);
    if (a.out_mode == TC_IO_INTERLEAVED) {
        constexpr int CPN = C::TS / 2;
        for (int c = tid; c < C::L * CPN; c += 128) {
            const int n = c / CPN, tp = c - n * CPN;
            *reinterpret_cast<float4*>(base + s0 + 2 * tp + (int64_t)n * a.out_n) =
                *reinterpret_cast<const float4*>(stg + n * C::TS + 2 * tp);
        }
    } else if (a.out_mode == TC_IO_CONTIG) {
        constexpr int CPS = C::L / 2;
        for (int c = tid; c < C::TS * CPS; c += 128) {
            const int t = c / CPS, np = c - t * CPS;
            if (t < nvalid)
                *reinterpret_cast<float4*>(base + (s0 + t) * a.out_s + 2 * np) =
                    *reinterpret_cast<const float4*>(stg + t * C::P + 2 * np);
        }
    } else {
        for (int c = tid; c < C::TS * C::L; c += 128) {
            const int t = c / C::L, n = c - t * C::L;
            if (t < nvalid) base[(s0 + t) * a.out_s + (int64_t)n * a.out_n] = stg[t * C::P + n];
        }
    }
}

template <class C>
__global__ void __launch_bounds__(128) tc_fft_kernel(const TcArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* s_ahi = smem;
    uint8_t* s_alo = s_ahi + C::A_BYTES;
    uint8_t* s_bhi = s_alo + C::A_BYTES;
    uint8_t* s_blo = s_bhi + C::B_BYTES;
    float2* stg = reinterpret_cast<float2*>(s_blo + C::B_BYTES);
    float2* twl = stg + 2 * C::STG;
    float2* ohi = twl + C::L;
    float2* olo = ohi + a.otw_hi_n;
    uint64_t* bar = reinterpret_cast<uint64_t*>(olo + a.otw_lo_n);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int64_t ntiles = (a.nseq + C::TS - 1) / C::TS;
    int64_t tile = blockIdx.x;

    // first tile's loads go out before the table setup
    if (tile < ntiles) load_tile<C>(a, tile * C::TS, stg, tid);
    tc::cp_async_commit();

    {
        const uint4* src = static_cast<const uint4*>(a.bmat);
        uint4* dst = reinterpret_cast<uint4*>(s_bhi);
        for (int i = tid; i < 2 * C::B_BYTES / 16; i += 128) dst[i] = src[i];
        const float2* tl = static_cast<const float2*>(a.twl);
        for (int i = tid; i < C::L; i += 128) twl[i] = tl[i];
        if (a.otw_hi) {
            const float2* th = static_cast<const float2*>(a.otw_hi);
            const float2* tlo = static_cast<const float2*>(a.otw_lo);
            for (int i = tid; i < a.otw_hi_n; i += 128) ohi[i] = th[i];
            for (int i = tid; i < a.otw_lo_n; i += 128) olo[i] = tlo[i];
        }
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, C::TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t u_ahi = tc::smem_u32(s_ahi), u_alo = tc::smem_u32(s_alo);
    const uint32_t u_bhi = tc::smem_u32(s_bhi), u_blo = tc::smem_u32(s_blo);

    // stage-A rows (n_a, t) and stage-B rows (k_b, t) of this thread
    const int ra = tid / C::TS;
    const int rt = tid - ra * C::TS;
    const int mask = (1 << a.otw_shift) - 1;
    uint32_t phase = 0;
    int buf = 0;
    bool failed = false;

    for (; tile < ntiles; tile += gridDim.x) {
        const int64_t q0 = tile * C::TS;
        const int64_t next = tile + gridDim.x;
        if (next < ntiles) load_tile<C>(a, next * C::TS, stg + (buf ^ 1) * C::STG, tid);
        tc::cp_async_commit();
        tc::cp_async_wait<1>();
        __syncthreads();
        float2* cur = stg + buf * C::STG;

        // ---- stage A: DFT over n_b
        {
            float2 x[C::R];
            if (a.in_mode == TC_IO_INTERLEAVED) {
#pragma unroll
                for (int nb = 0; nb < C::R; ++nb) x[nb] = cur[(ra + C::R * nb) * C::TS + rt];
            } else {
#pragma unroll
                for (int nb = 0; nb < C::R; ++nb) x[nb] = cur[rt * C::P + ra + C::R * nb];
            }
            if (a.conj_in) {
#pragma unroll
                for (int nb = 0; nb < C::R; ++nb) x[nb].y = -x[nb].y;
            }
            put_row<C>(s_ahi, s_alo, tid, x);
        }
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_gemm<C>(tmem, u_ahi, u_alo, u_bhi, u_blo);
            tc::mma_commit(bar);
        }
        failed = !mbar_wait_bounded(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(failed)) break;
        tc::fence_after_sync();

        // ---- twiddle, then the stage-B operand (rows k_b*TS + t, K index n_a)
        {
            float2 y[C::R];
            read_row<C>(taddr, y);
#pragma unroll
            for (int kb = 0; kb < C::R; ++kb) {
                const float2 w = twl[ra * kb];
                const float2 v = kb == 0 ? y[kb] : cmul(y[kb], w);
                const int row = kb * C::TS + rt;
                put_elem<C>(s_ahi, s_alo, row, ra, v.x);
                put_elem<C>(s_ahi, s_alo, row, C::R + ra, v.y);
            }
        }
        tc::fence_async_shared();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            issue_gemm<C>(tmem, u_ahi, u_alo, u_bhi, u_blo);
            tc::mma_commit(bar);
        }
        failed = !mbar_wait_bounded(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(failed)) break;
        tc::fence_after_sync();

        // ---- outputs X[k_b + R*k_a] of sequence rt, outer twiddle, staging
        {
            float2 z[C::R];
            read_row<C>(taddr, z);
            const int kb = ra;
            const int64_t s = (q0 + rt) % a.S;
#pragma unroll
            for (int ka = 0; ka < C::R; ++ka) {
                const int k = kb + C::R * ka;
                float2 v = z[ka];
                if (a.otw_hi) {
                    const int64_t e = s * k;
                    const float2 w = cmul(ohi[e >> a.otw_shift], olo[e & mask]);
                    v = cmul(v, w);
                }
                v = cscale(v, a.scale);
                if (a.conj_out) v.y = -v.y;
                if (a.out_mode == TC_IO_INTERLEAVED) cur[k * C::TS + rt] = v;
                else cur[rt * C::P + k] = v;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        store_tile<C>(a, q0, cur, tid);
        __syncthreads();
        buf ^= 1;
    }

    tc::cp_async_wait<0>();
    if (failed && tid == 0 && a.err) atomicOr(a.err, 2);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
}

// Real-embedded R-point DFT matrix as the B operand (row n: output real
// parts n < R, imaginary parts n >= R; K index k: input real parts k < R,
// imaginary parts k >= R), evaluated in FP64 and split into hi and lo images.
template <class C>
__global__ void tc_bmat_kernel(uint8_t* dst)
{
    constexpr int K = C::K, R = C::R;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < K * K; idx += gridDim.x * blockDim.x) {
        const int n = idx / K, k = idx - n * K;
        const int o = n < R ? n : n - R;
        const int j = k < R ? k : k - R;
        double s, c;
        sincospi(2.0 * (double)((o * j) % R) / (double)R, &s, &c);  // W_R^{o*j} = c - i*s
        const double v = n < R ? (k < R ? c : s) : (k < R ? -s : c);
        const uint32_t off = op_off<C>(n, k);
        if constexpr (!C::BF16) {
            const float h = tc::to_tf32((float)v);
            *reinterpret_cast<float*>(dst + off) = h;
            *reinterpret_cast<float*>(dst + C::B_BYTES + off) = tc::to_tf32((float)(v - (double)h));
        } else {
            const __nv_bfloat16 h = __float2bfloat16_rn((float)v);
            *reinterpret_cast<__nv_bfloat16*>(dst + off) = h;
            *reinterpret_cast<__nv_bfloat16*>(dst + C::B_BYTES + off) =
                __float2bfloat16_rn((float)(v - (double)__bfloat162float(h)));
        }
    }
}

int num_sms()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    int& c = cached[dev & 63];
    if (c == 0 && cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) c = 0;
    return c;
}

template <class C>
int launch_tc_t(const TcArgs* a, cudaStream_t st)
{
    static int occ_cached[64] = {0};
    static size_t smem_cached[64] = {0};
    if (a->nseq <= 0) return 0;
    if (a->S <= 0 || (a->S % C::TS != 0 && a->S < a->nseq)) return (int)cudaErrorInvalidValue;
    const size_t smem = smem_bytes_for<C>(a->otw_hi_n, a->otw_lo_n);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    int& occ = occ_cached[dev & 63];
    if (occ == 0 || smem_cached[dev & 63] != smem) {
        e = cudaFuncSetAttribute(tc_fft_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tc_fft_kernel<C>, 128, smem);
        if (e != cudaSuccess) return (int)e;
        if (occ < 1) return (int)cudaErrorInvalidConfiguration;
        smem_cached[dev & 63] = smem;
    }
    // a CTA holds C::TMEM_COLS of the 512 tensor-memory columns of its SM
    const int per_sm = occ < 512 / C::TMEM_COLS ? occ : 512 / C::TMEM_COLS;
    const int64_t ntiles = (a->nseq + C::TS - 1) / C::TS;
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (grid < 1) grid = 1;
    if (grid > ntiles) grid = ntiles;
    tc_fft_kernel<C><<<(unsigned)grid, 128, smem, st>>>(*a);
    return (int)cudaGetLastError();
}

bool host_aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace
}  // namespace gfft

using namespace gfft;

extern "C" long long gfft_tc_bmat_entries(int R, int prec)
{
    if (R != 8 && R != 16) return -1;
    const int es = prec == TC_PREC_BF16X3 ? 2 : 4;
    return 2ll * (2 * R) * (2 * R) * es / 8;  // two images, float2 units
}

extern "C" int gfft_tc_gen_bmat(void* dst, int R, int prec, void* stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t* d = static_cast<uint8_t*>(dst);
    if (prec == TC_PREC_TF32X3 && R == 16) tc_bmat_kernel<TcCfg<16, false>><<<4, 256, 0, st>>>(d);
    else if (prec == TC_PREC_TF32X3 && R == 8) tc_bmat_kernel<TcCfg<8, false>><<<1, 256, 0, st>>>(d);
    else if (prec == TC_PREC_BF16X3 && R == 16) tc_bmat_kernel<TcCfg<16, true>><<<4, 256, 0, st>>>(d);
    else if (prec == TC_PREC_BF16X3 && R == 8) tc_bmat_kernel<TcCfg<8, true>><<<1, 256, 0, st>>>(d);
    else return (int)cudaErrorInvalidValue;
    return (int)cudaGetLastError();
}

extern "C" int gfft_launch_tc(const TcArgs* in_args, void* stream)
{
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    TcArgs a = *in_args;
    if (!a.in || !a.out || !a.bmat || !a.twl) return (int)cudaErrorInvalidValue;
    if (a.otw_hi && (a.otw_shift < 0 || a.otw_shift > 20 || a.otw_hi_n <= 0 || a.otw_lo_n <= 0))
        return (int)cudaErrorInvalidValue;
    if (!a.otw_hi) a.otw_hi_n = a.otw_lo_n = 0;
    // 16-byte paths need aligned pointers; fall back to element accesses
    if (a.in_mode != TC_IO_GENERIC && !host_aligned16(a.in)) a.in_mode = TC_IO_GENERIC;
    if (a.out_mode != TC_IO_GENERIC && !host_aligned16(a.out)) a.out_mode = TC_IO_GENERIC;
    if (a.prec == TC_PREC_TF32X3 && a.R == 16) return launch_tc_t<TcCfg<16, false>>(&a, st);
    if (a.prec == TC_PREC_TF32X3 && a.R == 8) return launch_tc_t<TcCfg<8, false>>(&a, st);
    if (a.prec == TC_PREC_BF16X3 && a.R == 16) return launch_tc_t<TcCfg<16, true>>(&a, st);
    if (a.prec == TC_PREC_BF16X3 && a.R == 8) return launch_tc_t<TcCfg<8, true>>(&a, st);
    return (int)cudaErrorInvalidValue;
}
