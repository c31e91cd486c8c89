// codelet.cuh - compile-time specialised row kernels ("codelets").
//
// Same persistent, bulk-copy-fed tile loop as row_pipe.cuh, but the length,
// the thread count per transform and the radix sequence are template
// parameters, so every index, stride and twiddle-row computation folds to
// constants and each thread keeps its butterflies in registers:
//   * pass p: each thread owns NB_p = ceil(L/R_p / NTHR) butterflies
//     j = tid + b*NTHR and holds their R_p inputs in registers;
//   * passes run in place in ONE shared buffer per transform: all reads of
//     a pass complete (barrier) before any write, so half the shared memory
//     of the ping-pong kernel is needed;
//   * the first pass reads the raw stage copy of the input, the last pass
//     writes HBM directly (or shared memory for the R2C post-process).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "row_pipe.cuh"

namespace gfft {

template <int L_, int NTHR_, int... Rs>
struct CSpec {
    static constexpr int L = L_;
    static constexpr int NTHR = NTHR_;
    static constexpr int NP = sizeof...(Rs);
    static constexpr int R[NP] = {Rs...};
    __host__ __device__ static constexpr int ns(int p)
    {
        int n = 1;
        for (int i = 0; i < p; ++i) n *= R[i];
        return n;
    }
    __host__ __device__ static constexpr int nbf(int p) { return L / R[p]; }
    __host__ __device__ static constexpr int nb(int p) { return (L / R[p] + NTHR - 1) / NTHR; }
    __host__ __device__ static constexpr int emax()
    {
        int e = 0;
        for (int p = 0; p < NP; ++p) e = nb(p) * R[p] > e ? nb(p) * R[p] : e;
        return e;
    }
    static constexpr int E = emax();
    static constexpr int PSHIFT = (R[0] % 2 == 0) ? 4 : 30;
    __host__ __device__ static constexpr int product()
    {
        int n = 1;
        for (int i = 0; i < NP; ++i) n *= R[i];
        return n;
    }
    static_assert(product() == L, "radix product must equal L");
};

template <class S>
__device__ __forceinline__ int cpad(int i)
{
    return i + (i >> S::PSHIFT);
}

// One in-place pass P of codelet S on the transform held in W (shared) or,
// for P == 0 with from_stage, read from the stage copy through c.gload.
template <class S, int P>
__device__ __forceinline__ void codelet_pass(const PipeCtx& c, float2* W, float2 (&v)[S::E], const float2* tw,
                                             int tw_off, bool from_stage, bool last_global)
{
    constexpr int R = S::R[P];
    constexpr int NS = S::ns(P);
    constexpr int NBF = S::nbf(P);
    constexpr int NB = S::nb(P);
    constexpr bool FULL = (NBF % S::NTHR) == 0;
    constexpr bool LAST = P == S::NP - 1;
    const int tid = c.tid;
    // ---- load
    if (P == 0 && from_stage) {
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = tid + b * S::NTHR;
            const bool act = (FULL || j < NBF) && c.ok_io;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b * R + r] = act ? c.gload(j + r * NBF) : make_float2(0.f, 0.f);
            });
        });
    } else {
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = tid + b * S::NTHR;
            const bool act = FULL || j < NBF;
            sfor<R>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b * R + r] = act ? W[cpad<S>(j + r * NBF)] : make_float2(0.f, 0.f);
            });
        });
        __syncthreads();  // in place: every read of this pass precedes any write
    }
    // ---- twiddle + butterfly
    sfor<NB>([&](auto bb) {
        constexpr int b = decltype(bb)::value;
        const int j = tid + b * S::NTHR;
        if constexpr (NS > 1) {
            const int k = j % NS;
            const float2* w = tw + tw_off + k * R;
            if constexpr (R % 2 == 0) {
                sfor<R / 2>([&](auto hh) {
                    constexpr int h = decltype(hh)::value;
                    const float4 ww = reinterpret_cast<const float4*>(w)[h];
                    if constexpr (h > 0) v[b * R + 2 * h] = cmul(v[b * R + 2 * h], make_float2(ww.x, ww.y));
                    v[b * R + 2 * h + 1] = cmul(v[b * R + 2 * h + 1], make_float2(ww.z, ww.w));
                });
            } else {
                sfor<R - 1>([&](auto rr) {
                    constexpr int r = decltype(rr)::value + 1;
                    v[b * R + r] = cmul(v[b * R + r], w[r]);
                });
            }
        }
        DFT<R>::run(&v[b * R]);
    });
    // ---- store
    if (LAST && last_global) {
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = tid + b * S::NTHR;
            if ((FULL || j < NBF) && c.ok_io) {
                sfor<R>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    c.gstore(j + r * NS, v[b * R + r]);
                });
            }
        });
    } else {
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = tid + b * S::NTHR;
            if (FULL || j < NBF) {
                const int q = j / NS;
                const int k = j - q * NS;
                const int base = q * NS * R + k;
                sfor<R>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    W[cpad<S>(base + r * NS)] = v[b * R + r];
                });
            }
        });
        __syncthreads();
    }
}

template <class S>
__device__ __forceinline__ void codelet_passes(const PipeCtx& c, float2* W, float2 (&v)[S::E], const float2* tw,
                                               const RowArgs& A, bool from_stage, bool last_global)
{
    sfor<S::NP>([&](auto pp) {
        constexpr int P = decltype(pp)::value;
        codelet_pass<S, P>(c, W, v, tw, A.ip.pass[P].tw_off - A.tw_lo, from_stage, last_global);
    });
}

template <class S>
__global__ void __launch_bounds__(512) codelet_kernel(const __grid_constant__ RowArgs A)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smraw);
    volatile int* flags = reinterpret_cast<int*>(smraw + 64);  // [0] abort, [1+s] manual copy of stage s
    float2* stw = reinterpret_cast<float2*>(smraw + A.smem_tw);
    float2* spost = reinterpret_cast<float2*>(smraw + A.smem_post);
    unsigned char* stages = smraw + A.smem_stage;
    float2* work = reinterpret_cast<float2*>(smraw + A.smem_work);

    constexpr int L = S::L;
    const int tl = threadIdx.x / S::NTHR;
    const int tid = threadIdx.x - tl * S::NTHR;
    const int NST = A.nstage;
    const int64_t ntiles = (A.ntf + A.tfpc - 1) / A.tfpc;
    const int64_t row_bytes = A.in_dist * A.in_esize;
    const float2* gtw = reinterpret_cast<const float2*>(A.tw);
    const float2* gpost = reinterpret_cast<const float2*>(A.post_tw);

    for (int i = threadIdx.x; i < A.tw_cnt; i += blockDim.x) stw[i] = ldg2(gtw + A.tw_lo + i);
    for (int i = threadIdx.x; i < A.post_cnt; i += blockDim.x) spost[i] = ldg2(gpost + i);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) mbar_init(&bars[s], 1);
        flags[0] = 0;
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int s, int64_t tile) {
        const int64_t t0 = tile * A.tfpc;
        const int64_t rows = min((int64_t)A.tfpc, A.ntf - t0);
        const unsigned char* src = reinterpret_cast<const unsigned char*>(A.in) + t0 * row_bytes;
        const int64_t bytes = rows * row_bytes;
        if (((reinterpret_cast<uintptr_t>(src) | (uintptr_t)bytes) & 15) == 0) {
            flags[1 + s] = 0;
            mbar_expect_tx(&bars[s], (uint32_t)bytes);
            bulk_copy_g2s(stages + (int64_t)s * A.stage_bytes, src, (uint32_t)bytes, &bars[s]);
        } else {
            flags[1 + s] = 1;
        }
    };
    uint32_t phase = 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            const int64_t tile = blockIdx.x + (int64_t)s * gridDim.x;
            if (tile < ntiles) issue(s, tile);
        }
    }
    // pass tables: shared window (the planner guarantees it fits)
    const float2* tw = stw;
    const float2* post = A.post_cnt > 0 ? spost : gpost;
    const bool staged = A.staged != 0;
    const bool last_global = !(A.io_mode == IO_R2C_EVEN || (A.io_mode == IO_C2C && staged));
    float2* W = work + tl * A.lpad;
    float2 v[S::E];

    for (int64_t it = 0;; ++it) {
        const int64_t tile = blockIdx.x + it * gridDim.x;
        if (tile >= ntiles) break;
        const int s = (int)(it % NST);
        if (threadIdx.x == 0 && !flags[1 + s]) {
            if (!mbar_wait_bounded(&bars[s], (phase >> s) & 1u)) flags[0] = 1;
            phase ^= 1u << s;
        }
        __syncthreads();
        if (flags[0]) {
            if (threadIdx.x == 0) {
                atomicOr(A.err, 1);
                for (int k = 1; k < NST; ++k) {
                    const int s2 = (s + k) % NST;
                    const int64_t t2 = blockIdx.x + (it + k) * gridDim.x;
                    if (t2 < ntiles && !flags[1 + s2]) mbar_wait_bounded(&bars[s2], (phase >> s2) & 1u);
                }
            }
            return;
        }
        unsigned char* stg = stages + (int64_t)s * A.stage_bytes;
        const int64_t t0 = tile * A.tfpc;
        const int rows = (int)min((int64_t)A.tfpc, A.ntf - t0);
        if (flags[1 + s]) {
            coop_copy(stg, reinterpret_cast<const unsigned char*>(A.in) + t0 * row_bytes, rows * row_bytes);
            __syncthreads();
        }
        PipeCtx c;
        c.L = L;
        c.nthr = S::NTHR;
        c.tid = tid;
        c.ok_sm = true;
        c.ok_io = tl < rows;
        c.pshift = S::PSHIFT;
        c.tw = tw;
        c.sA = W;
        c.sB = W;
        c.st2 = reinterpret_cast<const float2*>(stg + (int64_t)tl * row_bytes);
        c.st1 = reinterpret_cast<const float*>(c.st2);
        c.mode = A.io_mode;
        c.conj_in = A.conj_in;
        c.conj_out = A.conj_out;
        c.weight = A.weight;
        c.nreal = A.nreal;
        c.scale = A.scale;
        const int64_t tt = c.ok_io ? t0 + tl : 0;
        c.out2 = reinterpret_cast<float2*>(A.out) + tt * A.out_dist;
        c.out1 = reinterpret_cast<float*>(A.out) + tt * A.out_dist;

        bool from_stage = true;
        if (A.io_mode == IO_C2R_EVEN) {
            // pre-process pairs (k, L-k) from the stage into W (see row_pipe.cuh)
            const bool half = A.weight == WEIGHT_LOAD_HALF;
            for (int k = tid; k <= (L >> 1); k += S::NTHR) {
                if (k == 0) {
                    const float x0 = c.st2[0].x, xl = c.st2[L].x;
                    W[0] = make_float2(x0 + xl, -(x0 - xl));
                } else {
                    float2 a = c.st2[k], b = c.st2[L - k];
                    if (half) {
                        a = cscale(a, 0.5f);
                        b = cscale(b, 0.5f);
                    }
                    const float2 w = post[k];
                    const float2 bc = cconj(b);
                    const float2 e = cadd(a, bc);
                    const float2 o = cmulc(csub(a, bc), w);
                    W[cpad<S>(k)] = cconj(make_float2(e.x - o.y, e.y + o.x));
                    if (L - k != k) W[cpad<S>(L - k)] = cconj(make_float2(e.x + o.y, -e.y + o.x));
                }
            }
            __syncthreads();
            from_stage = false;
        }
        // the first pass (or the pre-process) consumes the stage: it is
        // refilled once pass 0 has loaded its registers
        if (from_stage) {
            codelet_pass<S, 0>(c, W, v, tw, A.ip.pass[0].tw_off - A.tw_lo, true, last_global);
        }
        if (threadIdx.x == 0) {
            const int64_t nt = blockIdx.x + (it + NST) * gridDim.x;
            if (nt < ntiles) {
                fence_proxy_async_smem();
                issue(s, nt);
            }
        }
        if (!from_stage) {
            codelet_pass<S, 0>(c, W, v, tw, A.ip.pass[0].tw_off - A.tw_lo, false, last_global);
        }
        sfor<S::NP - 1>([&](auto pp) {
            constexpr int P = decltype(pp)::value + 1;
            codelet_pass<S, P>(c, W, v, tw, A.ip.pass[P].tw_off - A.tw_lo, false, last_global);
        });

        if (A.io_mode == IO_C2C && staged) {
            rows_to_global(work, A.lpad, S::PSHIFT, reinterpret_cast<float2*>(A.out) + t0 * A.out_dist, A.out_dist,
                           rows, L, A.conj_out != 0, A.scale);
        } else if (A.io_mode == IO_R2C_EVEN) {
            const float sc = A.scale;
            const float s2 = A.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
            if (c.ok_io) {
                for (int k = tid; k <= (L >> 1); k += S::NTHR) {
                    if (k == 0) {
                        const float2 z0 = W[0];
                        c.out2[0] = make_float2((z0.x + z0.y) * sc, 0.f);
                        c.out2[L] = make_float2((z0.x - z0.y) * sc, 0.f);
                    } else {
                        const float2 zk = W[cpad<S>(k)], zc = cconj(W[cpad<S>(L - k)]);
                        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
                        const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
                        const float2 wo = cmul(post[k], o);
                        c.out2[k] = cscale(cadd(e, wo), s2);
                        if (L - k != k) c.out2[L - k] = cscale(cconj(csub(e, wo)), s2);
                    }
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace gfft
