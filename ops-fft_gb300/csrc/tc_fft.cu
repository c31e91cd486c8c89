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
// Per CTA (256 threads, persistent over tiles): two threads per GEMM row,
// thread (m, h) owning row m (tensor-memory lane m) and the column half h.
// The DFT-matrix rows are ordered so that half h of a D row - the real and
// imaginary parts of outputs h*R/2 .. h*R/2 + R/2 - 1 - is R contiguous
// tensor-memory columns.  The input tile is staged in shared memory by
// cp.async and, once gathered into registers, the staging buffer receives
// the next tile while this one is computed; each thread splits its values
// and writes them into the K-major operand tile; thread 0 issues the MMAs
// and commits them to an mbarrier; every thread reads its D row half back
// (tcgen05.ld), applies the twiddles and writes the next operand tile or the
// output staging tile (which reuses the operand tiles), and the output tile
// goes to HBM with 16-byte coalesced stores.
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

constexpr int kTcThreads = 256;

template <int R_, bool BF16_>
struct TcCfg {
    static constexpr int R = R_;
    static constexpr bool BF16 = BF16_;
    static constexpr int L = R * R;
    static constexpr int HALF = R / 2;               // outputs per thread and GEMM row
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
    static_assert((HALF * ES) % 8 == 0, "a thread's K range is whole 8-byte units");
};

template <class C>
__host__ __device__ constexpr uint32_t op_off(int row, int k)
{
    return (uint32_t)(row >> 3) * C::SBO + (uint32_t)(k / C::EPC) * C::LBO + (uint32_t)(row & 7) * 16u +
           (uint32_t)(k % C::EPC) * C::ES;
}

// D column c of the ordered DFT matrix: half c / R, then R/2 real parts and
// R/2 imaginary parts of outputs half*R/2 + j.
template <class C>
__host__ __device__ constexpr void dcol(int c, int& index, bool& imag)
{
    const int h = c / C::R, j = c % C::R;
    imag = j >= C::HALF;
    index = h * C::HALF + (j % C::HALF);
}

// Split v into operand parts (hi, lo), stored at byte offset off of each tile.
template <class C>
__device__ __forceinline__ void put_split(uint8_t* hi, uint8_t* lo, uint32_t off, float v)
{
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

// Packs n (4 or 8) consecutive operand elements of the split parts.
template <class C, int N>
__device__ __forceinline__ void put_run(uint8_t* hi, uint8_t* lo, uint32_t off, const float* v)
{
    if constexpr (!C::BF16) {
        static_assert(N == 4, "tf32 runs are one 16-byte core-matrix row");
        float h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            h[e] = tc::to_tf32(v[e]);
            l[e] = tc::to_tf32(v[e] - h[e]);
        }
        *reinterpret_cast<float4*>(hi + off) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4*>(lo + off) = make_float4(l[0], l[1], l[2], l[3]);
    } else {
        uint32_t h[N / 2], l[N / 2];
#pragma unroll
        for (int e = 0; e < N / 2; ++e) {
            const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * e]), h1 = __float2bfloat16_rn(v[2 * e + 1]);
            const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * e] - __bfloat162float(h0));
            const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * e + 1] - __bfloat162float(h1));
            h[e] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
            l[e] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        if constexpr (N == 8) {
            *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
        } else {
            *reinterpret_cast<uint2*>(hi + off) = make_uint2(h[0], h[1]);
            *reinterpret_cast<uint2*>(lo + off) = make_uint2(l[0], l[1]);
        }
    }
}

// Stage-A operand: row m, K range of half h (real parts at K = h*R/2 ..,
// imaginary parts at K = R + h*R/2 ..) from this thread's R/2 values.
template <class C>
__device__ __forceinline__ void put_half_row(uint8_t* hi, uint8_t* lo, int m, int h, const float2* x)
{
    constexpr int RUN = C::BF16 ? (C::HALF < 8 ? C::HALF : 8) : 4;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
#pragma unroll
        for (int r0 = 0; r0 < C::HALF; r0 += RUN) {
            float v[RUN];
#pragma unroll
            for (int e = 0; e < RUN; ++e) v[e] = part ? x[r0 + e].y : x[r0 + e].x;
            put_run<C, RUN>(hi, lo, op_off<C>(m, part * C::R + h * C::HALF + r0), v);
        }
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

// This thread's half of its D row: R/2 complex outputs.
template <class C>
__device__ __forceinline__ void read_half(uint32_t taddr, float2* v)
{
    float f[C::R];
    if constexpr (C::R == 16) tc::tmem_ld16_wait(taddr, f);
    else tc::tmem_ld8_wait(taddr, f);
#pragma unroll
    for (int i = 0; i < C::HALF; ++i) v[i] = make_float2(f[i], f[C::HALF + i]);
}

// Shared-memory layout of one CTA: the operand tiles (hi, lo) - reused as
// the output staging tile once the second GEMM has completed - the DFT
// matrix images, the input staging tile, W_L, the barrier words and the
// outer-twiddle tables (their size is per launch).
template <class C>
struct TcSmem {
    static constexpr int OUTSTG = (2 * C::A_BYTES > C::STG * 8) ? 2 * C::A_BYTES : C::STG * 8;
    static constexpr int OFF_A = 0;
    static constexpr int OFF_B = OUTSTG;
    static constexpr int OFF_STG = OFF_B + 2 * C::B_BYTES;
    static constexpr int OFF_TWL = OFF_STG + C::STG * 8;
    static constexpr int OFF_BAR = OFF_TWL + C::L * 8;
    static constexpr int OFF_OTW = OFF_BAR + 16;
    static constexpr int FIXED = OFF_OTW;
};

template <class C>
__host__ __device__ inline size_t smem_bytes_for(int hi_n, int lo_n)
{
    return (size_t)TcSmem<C>::FIXED + (size_t)(hi_n + lo_n) * 8;
}

// TF32: the first GEMM's A operand lives in tensor memory (columns
// [K, 2K) hi, [2K, 3K) lo, after the accumulator [0, K)); BF16 keeps it in
// shared memory.
template <class C>
struct TcTmem {
    static constexpr bool A_IN_TMEM = !C::BF16;
    static constexpr int COLS = A_IN_TMEM ? 128 : 32;
    static constexpr uint32_t A_HI = C::K;
    static constexpr uint32_t A_LO = 2 * C::K;
};

// Stage-A operand row half from this thread's R/2 complex values into
// tensor memory: real parts at K = h*R/2 .., imaginary parts at R + h*R/2 ...
template <class C>
__device__ __forceinline__ void put_half_row_tmem(uint32_t trow, int h, const float2* x)
{
    float hr[C::HALF], lr[C::HALF], hi[C::HALF], li[C::HALF];
#pragma unroll
    for (int j = 0; j < C::HALF; ++j) {
        hr[j] = tc::to_tf32(x[j].x);
        lr[j] = tc::to_tf32(x[j].x - hr[j]);
        hi[j] = tc::to_tf32(x[j].y);
        li[j] = tc::to_tf32(x[j].y - hi[j]);
    }
    const uint32_t kre = (uint32_t)(h * C::HALF), kim = (uint32_t)(C::R + h * C::HALF);
    tc::tmem_st<C::HALF>(trow + TcTmem<C>::A_HI + kre, hr);
    tc::tmem_st<C::HALF>(trow + TcTmem<C>::A_HI + kim, hi);
    tc::tmem_st<C::HALF>(trow + TcTmem<C>::A_LO + kre, lr);
    tc::tmem_st<C::HALF>(trow + TcTmem<C>::A_LO + kim, li);
    tc::tmem_wait_st();
}

// First GEMM with A in tensor memory: D = Ahi*Blo + Alo*Bhi + Ahi*Bhi.
template <class C>
__device__ __forceinline__ void issue_gemm_ta(uint32_t tmem, uint32_t bhi, uint32_t blo)
{
#pragma unroll
    for (int kk = 0; kk < C::K / C::KSTEP; ++kk) {
        const uint32_t ko = (uint32_t)kk * (C::KSTEP / C::EPC) * C::LBO;
        const uint64_t b_h = tc::sdesc_noswizzle(bhi + ko, C::LBO, C::SBO);
        const uint64_t b_l = tc::sdesc_noswizzle(blo + ko, C::LBO, C::SBO);
        const uint32_t a_h = tmem + TcTmem<C>::A_HI + (uint32_t)(kk * C::KSTEP);
        const uint32_t a_l = tmem + TcTmem<C>::A_LO + (uint32_t)(kk * C::KSTEP);
        tc::mma_tf32_ta(tmem, a_h, b_l, C::IDESC, kk > 0);
        tc::mma_tf32_ta(tmem, a_l, b_h, C::IDESC, true);
        tc::mma_tf32_ta(tmem, a_h, b_h, C::IDESC, true);
    }
}

// Per-thread constants of a tile copy.  Interleaved layouts move 16-byte
// pairs of neighbouring sequences (staging [n][t], pitch TS); contiguous ones
// 16-byte pairs along each sequence (staging [t][n], pitch P); the generic
// path single elements (staging [t][n]).
template <class C, int MODE>
struct TileCopy {
    static constexpr int NT = kTcThreads;
    static constexpr int CPN = C::TS / 2;  // interleaved chunks per element row
    static constexpr int CPS = C::L / 2;   // contiguous chunks per sequence
    static constexpr int ITER = MODE == TC_IO_GENERIC ? C::TS * C::L / NT : C::TS * C::L / (2 * NT);
    static_assert(NT % CPN == 0 && NT % CPS == 0, "whole chunk rows per iteration");
    int soff, sstep;   // staging offsets (float2)
    int t0, tstep;     // sequence of the first chunk, and per iteration
    int64_t goff;      // element offset inside the tile, first chunk (generic: sequence stride)
    int64_t gstep;     // per iteration (generic: element stride)
    __device__ __forceinline__ TileCopy(int tid, int64_t ss, int64_t sn)
    {
        if constexpr (MODE == TC_IO_INTERLEAVED) {
            const int n0 = tid / CPN, tp = tid % CPN;
            soff = n0 * C::TS + 2 * tp;
            sstep = (NT / CPN) * C::TS;
            t0 = 2 * tp;
            tstep = 0;
            goff = 2 * tp + (int64_t)n0 * sn;
            gstep = (int64_t)(NT / CPN) * sn;
        } else if constexpr (MODE == TC_IO_CONTIG) {
            const int tt = tid / CPS, np = tid % CPS;
            soff = tt * C::P + 2 * np;
            sstep = (NT / CPS) * C::P;
            t0 = tt;
            tstep = NT / CPS;
            goff = (int64_t)tt * ss + 2 * np;
            gstep = (int64_t)(NT / CPS) * ss;
        } else {
            soff = tid;
            sstep = 0;
            t0 = 0;
            tstep = 0;
            goff = ss;
            gstep = sn;
        }
    }
};

template <class C, int MODE>
__device__ __forceinline__ void load_tile(const TileCopy<C, MODE>& tcp, const float2* gbase, float2* stg, int nvalid)
{
    const float2* g = gbase + tcp.goff;
    int so = tcp.soff, t = tcp.t0;
#pragma unroll
    for (int i = 0; i < TileCopy<C, MODE>::ITER; ++i) {
        if constexpr (MODE == TC_IO_INTERLEAVED) {
            tc::cp_async16(stg + so, g);
        } else if constexpr (MODE == TC_IO_CONTIG) {
            if (t < nvalid) tc::cp_async16(stg + so, g);
        } else {
            const int c = tcp.soff + kTcThreads * i, tt = c / C::L, n = c % C::L;
            if (tt < nvalid) tc::cp_async8(stg + tt * C::P + n, gbase + tt * tcp.goff + n * tcp.gstep);
        }
        g += tcp.gstep;
        so += tcp.sstep;
        t += tcp.tstep;
    }
}

template <class C, int MODE>
__device__ __forceinline__ void store_tile(const TileCopy<C, MODE>& tcp, float2* gbase, const float2* stg, int nvalid)
{
    float2* g = gbase + tcp.goff;
    int so = tcp.soff, t = tcp.t0;
#pragma unroll
    for (int i = 0; i < TileCopy<C, MODE>::ITER; ++i) {
        if constexpr (MODE == TC_IO_INTERLEAVED) {
            __stcs(reinterpret_cast<float4*>(g), *reinterpret_cast<const float4*>(stg + so));
        } else if constexpr (MODE == TC_IO_CONTIG) {
            if (t < nvalid) __stcs(reinterpret_cast<float4*>(g), *reinterpret_cast<const float4*>(stg + so));
        } else {
            const int c = tcp.soff + kTcThreads * i, tt = c / C::L, n = c % C::L;
            if (tt < nvalid) gbase[tt * tcp.goff + n * tcp.gstep] = stg[tt * C::P + n];
        }
        g += tcp.gstep;
        so += tcp.sstep;
        t += tcp.tstep;
    }
}

// Staging offset (float2) of element n of tile sequence t for a layout.
template <class C, int MODE>
__host__ __device__ constexpr int stg_index(int t, int n)
{
    return MODE == TC_IO_INTERLEAVED ? n * C::TS + t : t * C::P + n;
}

template <class C, int IN, int OUT, bool OUTER>
__global__ void __launch_bounds__(kTcThreads) tc_fft_kernel(const TcArgs a)
{
    using SM = TcSmem<C>;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* s_ahi = smem + SM::OFF_A;
    uint8_t* s_alo = s_ahi + C::A_BYTES;
    float2* ostg = reinterpret_cast<float2*>(smem + SM::OFF_A);  // after the second GEMM
    uint8_t* s_bhi = smem + SM::OFF_B;
    uint8_t* s_blo = s_bhi + C::B_BYTES;
    float2* stg = reinterpret_cast<float2*>(smem + SM::OFF_STG);
    float2* twl = reinterpret_cast<float2*>(smem + SM::OFF_TWL);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + SM::OFF_BAR);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    float2* ohi = reinterpret_cast<float2*>(smem + SM::OFF_OTW);
    float2* olo = ohi + a.otw_hi_n;

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int m = tid & 127;   // GEMM row / tensor-memory lane
    const int hh = tid >> 7;   // column half
    const int64_t ntiles = (a.nseq + C::TS - 1) / C::TS;
    int64_t tile = blockIdx.x;
    const int64_t tstride = (int64_t)gridDim.x * C::TS;  // sequences per grid step

    const TileCopy<C, IN> lcp(tid, a.in_s, a.in_n);
    const TileCopy<C, OUT> scp(tid, a.out_s, a.out_n);
    const float2* gin = static_cast<const float2*>(a.in);
    float2* gout = static_cast<float2*>(a.out);

    // batch item and sequence of the tile's first sequence, kept incrementally
    int64_t q0 = tile * C::TS;
    int64_t bi = q0 / a.S;
    int64_t s0 = q0 - bi * a.S;
    auto nvalid_of = [&](int64_t q) { return (int)((a.nseq - q) < C::TS ? (a.nseq - q) : C::TS); };
    if (tile < ntiles) load_tile<C, IN>(lcp, gin + bi * a.in_dist + s0 * a.in_s, stg, nvalid_of(q0));
    tc::cp_async_commit();

    {
        const uint4* src = static_cast<const uint4*>(a.bmat);
        uint4* dst = reinterpret_cast<uint4*>(s_bhi);
        for (int i = tid; i < 2 * C::B_BYTES / 16; i += kTcThreads) dst[i] = src[i];
        const float2* tl = static_cast<const float2*>(a.twl);
        for (int i = tid; i < C::L; i += kTcThreads) twl[i] = tl[i];
        if constexpr (OUTER) {
            const float2* th = static_cast<const float2*>(a.otw_hi);
            const float2* tlo = static_cast<const float2*>(a.otw_lo);
            for (int i = tid; i < a.otw_hi_n; i += kTcThreads) ohi[i] = th[i];
            for (int i = tid; i < a.otw_lo_n; i += kTcThreads) olo[i] = tlo[i];
        }
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tslot, TcTmem<C>::COLS);
        tc::tmem_relinquish();
    }
    tc::fence_async_shared();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tslot;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t taddr = trow + (uint32_t)(hh * C::R);
    const uint32_t u_ahi = tc::smem_u32(s_ahi), u_alo = tc::smem_u32(s_alo);
    const uint32_t u_bhi = tc::smem_u32(s_bhi), u_blo = tc::smem_u32(s_blo);

    // stage-A row (n_a, t) = (ra, rt); stage-B row (k_b, t) = (ra, rt)
    const int ra = m / C::TS;
    const int rt = m - ra * C::TS;
    const int hb = hh * C::HALF;                              // first n_b / k_b / k_a of this half
    const int g0 = stg_index<C, IN>(rt, ra + C::R * hb);      // x[n_a + R*n_b], n_b = hb + j
    constexpr int GSTEP = IN == TC_IO_INTERLEAVED ? C::R * C::TS : C::R;
    const int o0 = stg_index<C, OUT>(rt, ra + C::R * hb);     // X[k_b + R*k_a], k_a = hb + j
    constexpr int OSTEP = OUT == TC_IO_INTERLEAVED ? C::R * C::TS : C::R;
    // stage-B operand: row k_b*TS + rt (k_b = hb + j), K index n_a (real) and R + n_a (imaginary)
    const uint32_t bb_re = op_off<C>(hb * C::TS + rt, ra);
    constexpr uint32_t BB_IM = (uint32_t)(C::R / C::EPC) * C::LBO;
    constexpr uint32_t BB_KB = (uint32_t)(C::TS / 8) * C::SBO;
    static_assert(C::R % C::EPC == 0 || C::EPC % C::R == 0, "");
    const uint32_t omask = (1u << a.otw_shift) - 1u;
    const bool conj_in = a.conj_in != 0, conj_out = a.conj_out != 0;
    const float scale = a.scale;
    uint32_t phase = 0;
    bool failed = false;

    for (; tile < ntiles; tile += gridDim.x) {
        const int nv = nvalid_of(q0);
        const int64_t cb = bi, cs0 = s0;  // this tile
        s0 += tstride;
        if (s0 >= a.S) {
            const int64_t d = s0 / a.S;
            bi += d;
            s0 -= d * a.S;
        }
        const int64_t qn = q0 + tstride;

        tc::cp_async_wait<0>();
        __syncthreads();
        float2 x[C::HALF];
#pragma unroll
        for (int j = 0; j < C::HALF; ++j) x[j] = stg[g0 + j * GSTEP];
        __syncthreads();  // staging free: prefetch the next tile into it
        if (tile + gridDim.x < ntiles) load_tile<C, IN>(lcp, gin + bi * a.in_dist + s0 * a.in_s, stg, nvalid_of(qn));
        tc::cp_async_commit();

        // ---- stage A: DFT over n_b
        if (conj_in) {
#pragma unroll
            for (int j = 0; j < C::HALF; ++j) x[j].y = -x[j].y;
        }
        if constexpr (TcTmem<C>::A_IN_TMEM) {
            put_half_row_tmem<C>(trow, hh, x);
        } else {
            put_half_row<C>(s_ahi, s_alo, m, hh, x);
            tc::fence_async_shared();
        }
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
            if constexpr (TcTmem<C>::A_IN_TMEM) issue_gemm_ta<C>(tmem, u_bhi, u_blo);
            else issue_gemm<C>(tmem, u_ahi, u_alo, u_bhi, u_blo);
            tc::mma_commit(bar);
        }
        failed = !mbar_wait_bounded(bar, phase);
        phase ^= 1;
        if (__syncthreads_or(failed)) break;
        tc::fence_after_sync();

        // ---- twiddle W_L^{n_a k_b}, stage-B operand
        {
            float2 y[C::HALF];
            read_half<C>(taddr, y);
            uint32_t off = bb_re;
#pragma unroll
            for (int j = 0; j < C::HALF; ++j) {
                const int kb = hb + j;
                const float2 v = cmul(y[j], twl[ra * kb]);
                put_split<C>(s_ahi, s_alo, off, v.x);
                put_split<C>(s_ahi, s_alo, off + BB_IM, v.y);
                off += BB_KB;
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

        // ---- outputs X[k_b + R*k_a] of sequence rt (outer twiddle W_N^{s*k})
        {
            float2 z[C::HALF];
            read_half<C>(taddr, z);
            uint32_t e = 0, de = 0;
            if constexpr (OUTER) {
                const uint32_t s = (uint32_t)(cs0 + rt);
                e = s * (uint32_t)(ra + C::R * hb);
                de = s * (uint32_t)C::R;
            }
#pragma unroll
            for (int j = 0; j < C::HALF; ++j) {
                float2 v = z[j];
                if constexpr (OUTER) {
                    v = cmul(v, cmul(ohi[e >> a.otw_shift], olo[e & omask]));
                    e += de;
                }
                if (scale != 1.0f) v = cscale(v, scale);
                if (conj_out) v.y = -v.y;
                ostg[o0 + j * OSTEP] = v;
            }
        }
        tc::fence_before_sync();
        __syncthreads();
        store_tile<C, OUT>(scp, gout + cb * a.out_dist + cs0 * a.out_s, ostg, nv);
        q0 = qn;
    }

    tc::cp_async_wait<0>();
    if (failed && tid == 0 && a.err) atomicOr(a.err, 2);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TcTmem<C>::COLS);
}

// Real-embedded R-point DFT matrix as the B operand, rows in D-column order
// (see dcol) and K index k: input real parts k < R, imaginary parts k >= R;
// evaluated in FP64 and split into hi and lo images.
template <class C>
__global__ void tc_bmat_kernel(uint8_t* dst)
{
    constexpr int K = C::K, R = C::R;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < K * K; idx += gridDim.x * blockDim.x) {
        const int n = idx / K, k = idx - n * K;
        int o = 0;
        bool oim = false;
        dcol<C>(n, o, oim);
        const int j = k < R ? k : k - R;
        double s, c;
        sincospi(2.0 * (double)((o * j) % R) / (double)R, &s, &c);  // W_R^{o*j} = c - i*s
        const double v = !oim ? (k < R ? c : s) : (k < R ? -s : c);
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

template <class C, int IN, int OUT, bool OUTER>
int launch_tc_k(const TcArgs* a, cudaStream_t st)
{
    static int smem_set[64] = {0};
    static int resident[64][8] = {};  // CTAs per SM by shared-memory size bucket
    const size_t smem = smem_bytes_for<C>(a->otw_hi_n, a->otw_lo_n);
    if (smem > (size_t)kMaxSmemBytes) return (int)cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    if (smem_set[dev & 63] == 0) {
        e = cudaFuncSetAttribute(tc_fft_kernel<C, IN, OUT, OUTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kMaxSmemBytes);
        if (e != cudaSuccess) return (int)e;
        e = cudaFuncSetAttribute(tc_fft_kernel<C, IN, OUT, OUTER>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return (int)e;
        smem_set[dev & 63] = 1;
    }
    // Resident CTAs per SM from shared memory, registers and warps.  The
    // occupancy API reports one CTA per SM for kernels that allocate tensor
    // memory, so the limits are applied here directly.
    const int bucket = (int)((smem >> 12) & 7);
    int& occ = resident[dev & 63][bucket];
    if (occ == 0) {
        cudaFuncAttributes fa{};
        e = cudaFuncGetAttributes(&fa, tc_fft_kernel<C, IN, OUT, OUTER>);
        if (e != cudaSuccess) return (int)e;
        int sm_smem = 0, blk_res = 0, sm_regs = 0;
        if (cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&blk_res, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sm_regs, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess)
            return (int)cudaGetLastError();
        const int by_smem = sm_smem / (int)(smem + (size_t)blk_res + fa.sharedSizeBytes);
        const int regs_per_warp = ((fa.numRegs * 32 + 255) / 256) * 256;
        const int warps = kTcThreads / 32;
        const int by_regs = regs_per_warp > 0 ? sm_regs / (regs_per_warp * warps) : 64 / warps;
        int o = by_smem < by_regs ? by_smem : by_regs;
        if (o > 64 / warps) o = 64 / warps;
        if (o > 512 / TcTmem<C>::COLS) o = 512 / TcTmem<C>::COLS;
        if (o < 1) return (int)cudaErrorInvalidConfiguration;
        occ = o;
    }
    const int64_t ntiles = (a->nseq + C::TS - 1) / C::TS;
    int64_t grid = (int64_t)num_sms() * occ;
    if (grid < 1) grid = 1;
    if (grid > ntiles) grid = ntiles;
    tc_fft_kernel<C, IN, OUT, OUTER><<<(unsigned)grid, kTcThreads, smem, st>>>(*a);
    return (int)cudaGetLastError();
}

// Layout-specialised instantiations: the passes of the planner's two-pass
// split (interleaved -> interleaved with the outer twiddle, contiguous ->
// interleaved), single-pass contiguous rows, and an element-wise fallback.
template <class C>
int launch_tc_t(const TcArgs* a, cudaStream_t st)
{
    if (a->nseq <= 0) return 0;
    if (a->S <= 0 || (a->S % C::TS != 0 && a->S < a->nseq)) return (int)cudaErrorInvalidValue;
    const bool outer = a->otw_hi != nullptr;
    if (outer && a->in_mode == TC_IO_INTERLEAVED && a->out_mode == TC_IO_INTERLEAVED)
        return launch_tc_k<C, TC_IO_INTERLEAVED, TC_IO_INTERLEAVED, true>(a, st);
    if (!outer && a->in_mode == TC_IO_CONTIG && a->out_mode == TC_IO_INTERLEAVED)
        return launch_tc_k<C, TC_IO_CONTIG, TC_IO_INTERLEAVED, false>(a, st);
    if (!outer && a->in_mode == TC_IO_CONTIG && a->out_mode == TC_IO_CONTIG)
        return launch_tc_k<C, TC_IO_CONTIG, TC_IO_CONTIG, false>(a, st);
    if (outer) return launch_tc_k<C, TC_IO_GENERIC, TC_IO_GENERIC, true>(a, st);
    return launch_tc_k<C, TC_IO_GENERIC, TC_IO_GENERIC, false>(a, st);
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
