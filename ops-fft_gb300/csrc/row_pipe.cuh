// row_pipe.cuh - persistent, TMA-fed row kernel (contiguous batched
// transforms whose whole length fits one CTA).
//
// Each CTA loops over tiles b, b + grid, b + 2*grid, ... where a tile is
// `tfpc` consecutive transforms.  The raw input of a tile (one contiguous
// range in HBM) is brought into one of `nstage` shared stage buffers by a
// single bulk asynchronous copy (cp.async.bulk, completion counted on an
// mbarrier), issued `nstage` tiles ahead, so HBM reads of later tiles
// overlap the shared-memory passes of the current one.  Ranges that are not
// 16-byte aligned (possible for odd row lengths) fall back to a cooperative
// copy.  The pass tables and the real-data post-process twiddles live in
// shared memory for the CTA's lifetime.
//
// Every mbarrier wait is bounded by a clock budget (~2 s); on expiry the CTA
// records bit 0 in the plan's error word, drains its outstanding copies
// (again bounded) and returns, leaving the context usable.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pipe_ptx.cuh"
#include "pdl.cuh"
#include "stockham.cuh"

namespace gfft {

// -------------------------------------------------------------- context
struct PipeCtx {
    int L, nthr, tid;
    bool ok_sm, ok_io;
    int pshift;
    const float2* tw;
    float2* sA;
    float2* sB;
    const float2* st2;  // this transform's raw input in the stage buffer
    const float* st1;
    float2* out2;
    float* out1;
    int mode, conj_in, conj_out, weight, nreal;
    float scale;
    const float* wl;  // codelets, even C2R: per-bin input weights of this transform (or nullptr)

    __device__ __forceinline__ int pad(int i) const { return i + (i >> pshift); }
    __device__ __forceinline__ float2* buf(int b) const { return b == 1 ? sA : sB; }
    __device__ __forceinline__ float2 sget(int b, int i) const { return buf(b)[pad(i)]; }
    __device__ __forceinline__ void sput(int b, int i, float2 x) const { buf(b)[pad(i)] = x; }

    // "buffer 0" source: the raw stage copy of the input row
    __device__ __forceinline__ float2 gload(int i) const
    {
        if (mode == IO_R2C_ODD) return make_float2(st1[i], 0.f);
        if (mode == IO_C2R_ODD) {
            // Hermitian expansion of bins 0..N/2 to N bins, conjugated for the
            // backward-as-forward trick; interior bins optionally halved.
            const int h = nreal >> 1;
            float2 x = (i <= h) ? st2[i] : cconj(st2[nreal - i]);
            if (weight == WEIGHT_LOAD_HALF && i != 0) x = cscale(x, 0.5f);
            return cconj(x);
        }
        const float2 x = st2[i];
        return conj_in ? cconj(x) : x;
    }
    // "buffer 0" destination: HBM (last pass only)
    __device__ __forceinline__ void gstore(int i, float2 x) const
    {
        if (mode == IO_R2C_ODD) {
            if (i <= (nreal >> 1)) {
                float sc = scale;
                if (weight == WEIGHT_STORE_X2 && i != 0) sc *= 2.f;
                out2[i] = cscale(x, sc);
            }
            return;
        }
        if (mode == IO_C2R_ODD) {
            out1[i] = x.x * scale;  // Re(conj(x)) == Re(x)
            return;
        }
        if (conj_out) x = cconj(x);
        out2[i] = cscale(x, scale);
    }
};

// Coalesced copy of `rows` results of `len` float2 from shared work buffers
// (row r at base + r*pitch, padded) to HBM rows `dist` apart.
__device__ __forceinline__ void rows_to_global(const float2* base, int pitch, int pshift, float2* g, int64_t dist,
                                               int rows, int len, bool conj, float scale)
{
    const int total = rows * len;
    const float inv = 1.0f / (float)len;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int r = fdivf(e, inv);
        const int i = e - r * len;
        float2 x = base[r * pitch + i + (i >> pshift)];
        if (conj) x = cconj(x);
        g[(int64_t)r * dist + i] = cscale(x, scale);
    }
}

// Cooperative copy of `bytes` bytes (multiple of 4) HBM -> shared.
__device__ __forceinline__ void coop_copy(void* dst, const void* src, int64_t bytes)
{
    if ((((uintptr_t)src | (uintptr_t)dst | (uintptr_t)bytes) & 7) == 0) {
        const float2* s = reinterpret_cast<const float2*>(src);
        float2* d = reinterpret_cast<float2*>(dst);
        for (int64_t i = threadIdx.x; i < bytes / 8; i += blockDim.x) d[i] = ldg2(s + i);
    } else {
        const float* s = reinterpret_cast<const float*>(src);
        float* d = reinterpret_cast<float*>(dst);
        for (int64_t i = threadIdx.x; i < bytes / 4; i += blockDim.x) d[i] = __ldg(s + i);
    }
}

// ---------------------------------------------------------------- kernel
template <int RMAX>
__global__ void __launch_bounds__(kernel_max_threads<RMAX>()) row_kernel(const __grid_constant__ RowArgs A)
{
    pdl_wait();  // every access below may touch the caller's buffers
    extern __shared__ __align__(128) unsigned char smraw[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smraw);   // up to 4 stages
    volatile int* flags = reinterpret_cast<int*>(smraw + 64);  // [0] abort, [1+s] manual copy of stage s
    float2* stw = reinterpret_cast<float2*>(smraw + A.smem_tw);
    float2* spost = reinterpret_cast<float2*>(smraw + A.smem_post);
    unsigned char* stages = smraw + A.smem_stage;
    float2* work = reinterpret_cast<float2*>(smraw + A.smem_work);

    const int nthr = A.ip.nthr;
    const int tl = threadIdx.x / nthr;
    const int tid = threadIdx.x - tl * nthr;
    const int L = A.ip.L;
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

    // Thread 0 only: start the copy of `tile` into stage s.
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

    uint32_t phase = 0;  // thread 0: parity bit per stage
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            const int64_t tile = blockIdx.x + (int64_t)s * gridDim.x;
            if (tile < ntiles) issue(s, tile);
        }
    }

    const float2* twp = A.tw_cnt > 0 ? stw - A.tw_lo : gtw;
    const float2* post = A.post_cnt > 0 ? spost : gpost;
    const int pitch = A.nbuf * A.lpad;

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
            // a copy did not complete in time: record it, drain the other
            // stages (bounded) and leave
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
        c.wl = nullptr;
        c.L = L;
        c.nthr = nthr;
        c.tid = tid;
        c.ok_sm = tl < A.tfpc;
        c.ok_io = c.ok_sm && tl < rows;
        c.pshift = A.pshift;
        c.tw = twp;
        c.sA = work + (c.ok_sm ? tl : 0) * pitch;
        c.sB = c.sA + A.lpad;
        c.st2 = reinterpret_cast<const float2*>(stg + (int64_t)(c.ok_sm ? tl : 0) * row_bytes);
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

        const bool staged = A.staged != 0;
        const bool last_global = !(A.io_mode == IO_R2C_EVEN || (A.io_mode == IO_C2C && staged));
        int cur;
        int p_next;
        if (A.io_mode == IO_C2R_EVEN) {
            // pre-process pairs (k, L-k) from the stage into buffer A:
            //   Z'[k] = E + i*O,  E = X[k] + conj(X[L-k]),
            //   O = (X[k] - conj(X[L-k])) * conj(W_N^k), stored conjugated.
            if (c.ok_sm) {
                const bool half = A.weight == WEIGHT_LOAD_HALF;
                for (int k = tid; k <= (L >> 1); k += nthr) {
                    if (k == 0) {
                        const float x0 = c.st2[0].x, xl = c.st2[L].x;  // imaginary parts of DC/Nyquist ignored
                        c.sput(1, 0, make_float2(x0 + xl, -(x0 - xl)));
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
                        c.sput(1, k, cconj(make_float2(e.x - o.y, e.y + o.x)));
                        if (L - k != k) c.sput(1, L - k, cconj(make_float2(e.x + o.y, -e.y + o.x)));
                    }
                }
            }
            __syncthreads();
            cur = 1;
            p_next = 0;
        } else {
            cur = run_passes<RMAX>(c, A.ip, 0, last_global, 0, 1);
            p_next = 1;
        }
        // the stage is consumed: refill it with the tile NST iterations ahead
        if (threadIdx.x == 0) {
            const int64_t nt = blockIdx.x + (it + NST) * gridDim.x;
            if (nt < ntiles) {
                fence_proxy_async_smem();
                issue(s, nt);
            }
        }
        cur = run_passes<RMAX>(c, A.ip, cur, last_global, p_next, kMaxPass);

        if (A.io_mode == IO_C2C && staged) {
            rows_to_global(work + (cur == 2 ? A.lpad : 0), pitch, A.pshift,
                           reinterpret_cast<float2*>(A.out) + t0 * A.out_dist, A.out_dist, rows, L,
                           A.conj_out != 0, A.scale);
        } else if (A.io_mode == IO_R2C_EVEN) {
            // post-process pairs:
            //   E = (Z[k] + conj Z[L-k])/2, O = (Z[k] - conj Z[L-k])/(2i)
            //   X[k] = E + W^k O, X[L-k] = conj(E - W^k O),
            //   X[0] = Re Z0 + Im Z0, X[L] = Re Z0 - Im Z0 (zero imaginary parts)
            const float sc = A.scale;
            const float s2 = A.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
            if (!staged) {
                if (c.ok_io) {
                    for (int k = tid; k <= (L >> 1); k += nthr) {
                        if (k == 0) {
                            const float2 z0 = c.sget(cur, 0);
                            c.out2[0] = make_float2((z0.x + z0.y) * sc, 0.f);
                            c.out2[L] = make_float2((z0.x - z0.y) * sc, 0.f);
                        } else {
                            const float2 zk = c.sget(cur, k), zc = cconj(c.sget(cur, L - k));
                            const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
                            const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
                            const float2 wo = cmul(post[k], o);
                            c.out2[k] = cscale(cadd(e, wo), s2);
                            if (L - k != k) c.out2[L - k] = cscale(cconj(csub(e, wo)), s2);
                        }
                    }
                }
            } else {
                if (c.ok_sm) {
                    for (int k = tid; k <= (L >> 1); k += nthr) {
                        if (k == 0) {
                            const float2 z0 = c.sget(cur, 0);
                            c.sput(cur, 0, make_float2((z0.x + z0.y) * sc, 0.f));
                            c.sput(cur, L, make_float2((z0.x - z0.y) * sc, 0.f));
                        } else {
                            const float2 zk = c.sget(cur, k), zc = cconj(c.sget(cur, L - k));
                            const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
                            const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
                            const float2 wo = cmul(post[k], o);
                            c.sput(cur, k, cscale(cadd(e, wo), s2));
                            if (L - k != k) c.sput(cur, L - k, cscale(cconj(csub(e, wo)), s2));
                        }
                    }
                }
                __syncthreads();
                rows_to_global(work + (cur == 2 ? A.lpad : 0), pitch, A.pshift,
                               reinterpret_cast<float2*>(A.out) + t0 * A.out_dist, A.out_dist, rows, L + 1, false,
                               1.f);
            }
        }
        __syncthreads();
    }
}

}  // namespace gfft
