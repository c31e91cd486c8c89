// codelet.cuh - compile-time specialised row kernels ("codelets").
//
// The length, the threads per transform and the radix sequence are template
// parameters, so every index, stride and twiddle-row computation folds to
// constants and each thread keeps its butterflies in registers.
//
// Execution model (per CTA):
//   * the CTA holds NG independent transform GROUPS of NTHR threads
//     (NTHR a multiple of 32); groups synchronise only among themselves with
//     a named barrier (bar.sync 1+g, NTHR), never CTA-wide, so one group's
//     passes overlap another group's loads and stores;
//   * each group owns a ring of NST shared SLOTS; a slot holds TPS
//     consecutive transforms, filled by ONE bulk asynchronous copy
//     (cp.async.bulk, completion counted on the slot's mbarrier) issued by
//     the group leader NST slots ahead.  TPS is chosen so a slot is a 16-byte
//     aligned, 16-byte multiple range (2 for rows of an odd number of float2);
//   * pass p: thread owns NB_p = ceil(L/R_p / NTHR) butterflies
//     j = tid + b*NTHR and holds their R_p inputs in registers; the first
//     pass reads the slot, the last pass writes HBM directly (or shared
//     memory for the R2C post-process).  Without a work buffer (nbuf 1) the
//     passes run in place in the slot (all reads of a pass finish before any
//     write: two group barriers per pass); with one (nbuf 2, ping-pong) they
//     alternate between the slot and the group's work buffer, ending in the
//     work buffer, so each pass needs one barrier and the slot is refilled
//     as soon as the last pass that reads it is done;
//   * twiddle tables and the real-data post-process twiddles are copied to
//     shared memory once per CTA.
// Every mbarrier wait is bounded (~2 s); on expiry the group records bit 0 in
// the plan's error word, drains its own outstanding copies (bounded) and
// stops, leaving the context usable.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pdl.cuh"
#include "row_pipe.cuh"

namespace gfft {

template <int MAXT_, int MINB_, int L_, int NTHR_, int... Rs>
struct CSpec {
    static constexpr int MAXT = MAXT_;  // launch bound: threads per CTA
    static constexpr int MINB = MINB_;  // CTAs per SM the register budget must allow
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
    // transform groups a CTA can hold (launch bound / group size, at most 15)
    static constexpr int NGMAX = (MAXT_ / NTHR_) < 15 ? (MAXT_ / NTHR_) : 15;
    static constexpr int PSHIFT = (R[0] % 2 == 0) ? 4 : 30;
    __host__ __device__ static constexpr int product()
    {
        int n = 1;
        for (int i = 0; i < NP; ++i) n *= R[i];
        return n;
    }
    static_assert(product() == L, "radix product must equal L");
    static_assert(NTHR % 32 == 0, "transform groups are whole warps");
    static_assert(NGMAX >= 1, "launch bound below one transform group");
};

template <class S>
__device__ __forceinline__ int cpad(int i)
{
    if constexpr (S::PSHIFT >= 30) {
        return i;  // odd first radix: stride-R writes are already conflict free
    } else {
        return i + (i >> S::PSHIFT);
    }
}

// bar.sync of transform group barrier `id` (1 .. NG) with an immediate
// barrier operand, selected by a uniform branch.  With a register operand
// ptxas reserves all 16 hardware barriers of the CTA, and ncu's occupancy
// limit for 3 barriers per CTA is 21 CTAs per SM (a pool of ~64), so 16
// barriers alone cap residency at 4 CTAs per SM; immediates reserve NG + 1.
template <int NT, int I, int NG>
__device__ __forceinline__ void bar_sync_id(int id)
{
    if constexpr (I >= NG) {
        asm volatile("bar.sync %0, %1;" ::"n"(NG), "n"(NT) : "memory");
    } else {
        if (id == I) {
            asm volatile("bar.sync %0, %1;" ::"n"(I), "n"(NT) : "memory");
        } else {
            bar_sync_id<NT, I + 1, NG>(id);
        }
    }
}

template <class S>
__device__ __forceinline__ void group_sync(int id)
{
    bar_sync_id<S::NTHR, 1, S::NGMAX>(id);
}

// One in-place pass P of codelet S on the transform held in W (shared) or,
// for P == 0 with from_slot, read from the slot copy through c.gload.
// Win: input buffer (ignored when the pass reads the slot); Wout: output
// buffer; sync_loaded: a group barrier between the loads and the stores
// (in-place passes, and passes whose input buffer must be free afterwards).
template <class S, int P, bool FC2R = false>
__device__ __forceinline__ void codelet_pass(const PipeCtx& c, const float2* Win, float2* Wout, float2 (&v)[S::E],
                                             const float2* tw, int tw_off, bool from_slot, bool last_global,
                                             bool sync_loaded, int bar_id, const float2* post = nullptr)
{
    constexpr int R = S::R[P];
    constexpr int NS = S::ns(P);
    constexpr int NBF = S::nbf(P);
    constexpr int NB = S::nb(P);
    constexpr bool FULL = (NBF % S::NTHR) == 0;
    constexpr bool LAST = P == S::NP - 1;
    const int tid = c.tid;
    // ---- load (the io mode is uniform: branch once, outside the unrolled loops)
    if (P == 0 && from_slot) {
        auto load_all = [&](auto getter) {
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                const int j = tid + b * S::NTHR;
                if (FULL || j < NBF) {
                    sfor<R>([&](auto rr) {
                        constexpr int r = decltype(rr)::value;
                        v[b * R + r] = getter(j + r * NBF);
                    });
                }
            });
        };
        if constexpr (FC2R) {
            // even C2R with the Hermitian pre-process fused into this first
            // pass: Z'[i] from the raw bins X[i] and X[L-i] of the slot
            // (X[L] for i = 0), stored conjugated for the forward transform:
            //   k = min(i, L-i), E = X[k] + conj X[L-k],
            //   O = (X[k] - conj X[L-k]) * conj W_N^k,
            //   Z'[k] = conj(E + iO), Z'[L-k] = conj(conj(E) + i conj(O)),
            //   Z'[0] = (x0 + xL, -(x0 - xL)) (imaginary parts of DC and Nyquist ignored)
            constexpr int L = S::L;
            const bool half = c.weight == WEIGHT_LOAD_HALF;
            const float* wl = c.wl;
            load_all([&](int i) {
                float2 xi = c.st2[i], xm = c.st2[L - i];
                if (wl) {
                    xi = cscale(xi, __ldg(wl + i));
                    xm = cscale(xm, __ldg(wl + (L - i)));
                }
                if (i == 0) return make_float2(xi.x + xm.x, -(xi.x - xm.x));
                const bool lo = i <= (L >> 1);
                float2 a = lo ? xi : xm, b = lo ? xm : xi;  // a = X[k], b = X[L-k]
                if (half) {
                    a = cscale(a, 0.5f);
                    b = cscale(b, 0.5f);
                }
                const float2 bc = cconj(b);
                const float2 e = cadd(a, bc);
                const float2 o = cmulc(csub(a, bc), post[lo ? i : L - i]);
                return lo ? cconj(make_float2(e.x - o.y, e.y + o.x)) : cconj(make_float2(e.x + o.y, -e.y + o.x));
            });
        } else if (c.mode == IO_R2C_ODD) {
            load_all([&](int i) { return make_float2(c.st1[i], 0.f); });
        } else if (c.mode == IO_C2R_ODD) {
            load_all([&](int i) { return c.gload(i); });
        } else if (c.conj_in) {
            load_all([&](int i) { return cconj(c.st2[i]); });
        } else {
            load_all([&](int i) { return c.st2[i]; });
        }
        if (sync_loaded) group_sync<S>(bar_id);  // e.g. the raw row and an in-slot output share the slot
    } else {
        sfor<NB>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = tid + b * S::NTHR;
            if (FULL || j < NBF) {
                sfor<R>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    v[b * R + r] = Win[cpad<S>(j + r * NBF)];
                });
            }
        });
        if (sync_loaded) group_sync<S>(bar_id);  // in place: every read of this pass precedes any write
    }
    // ---- twiddle + butterfly
    sfor<NB>([&](auto bb) {
        constexpr int b = decltype(bb)::value;
        const int j = tid + b * S::NTHR;
        if (FULL || j < NBF) {
            if constexpr (NS > 1) {
                const int k = j % NS;
                const float2* w = tw + tw_off + k;  // entry r*NS + k: consecutive k, consecutive banks
                sfor<R - 1>([&](auto rr) {
                    constexpr int r = decltype(rr)::value + 1;
                    v[b * R + r] = cmul(v[b * R + r], w[r * NS]);
                });
            }
            DFT<R>::run(&v[b * R]);
        }
    });
    // ---- store
    if (LAST && last_global) {
        auto store_all = [&](auto putter) {
            sfor<NB>([&](auto bb) {
                constexpr int b = decltype(bb)::value;
                const int j = tid + b * S::NTHR;
                if (FULL || j < NBF) {
                    sfor<R>([&](auto rr) {
                        constexpr int r = decltype(rr)::value;
                        putter(j + r * NS, v[b * R + r]);
                    });
                }
            });
        };
        if (c.ok_io) {
            const float sc = c.scale;
            if (c.mode == IO_C2C || c.mode == IO_C2R_EVEN) {
                if (c.conj_out) {
                    store_all([&](int i, float2 x) { c.out2[i] = make_float2(x.x * sc, -x.y * sc); });
                } else if (sc == 1.f) {
                    store_all([&](int i, float2 x) { c.out2[i] = x; });
                } else {
                    store_all([&](int i, float2 x) { c.out2[i] = cscale(x, sc); });
                }
            } else {
                store_all([&](int i, float2 x) { c.gstore(i, x); });
            }
        }
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
                    Wout[cpad<S>(base + r * NS)] = v[b * R + r];
                });
            }
        });
        group_sync<S>(bar_id);
    }
}

// Whether the even-R2C launches of codelet S use the instance whose last
// pass is fused with the even/odd post-process (codelet_last_r2c): the last
// radix at most 8 (two butterflies per unit in registers), its NS = L/R
// even, and the NS/2 units dividing evenly over the group's threads; 1024
// to 4096 points (shorter transforms were measured slower with it, and the
// 8192-point build's tables do not fit its row plans).
template <class S>
__host__ __device__ constexpr bool fuse_r2c_spec()
{
    constexpr int RL = S::R[S::NP - 1];
    constexpr int NSL = S::L / RL;
    return S::NP >= 2 && S::L >= 1024 && S::L <= 4096 && RL <= 8 && NSL % 2 == 0 && (NSL / 2) % S::NTHR == 0;
}

// The last pass of an even R2C fused with the even/odd post-process.  The
// last pass (radix R, NS = L/R) has butterfly j write Z[j + r*NS]; the
// mirror of that bin, L - j - r*NS, is output R-1-r of butterfly NS - j.
// So unit u (1 <= u < NS/2) runs butterflies u and NS - u and holds every
// pair (k, L - k) of their 2R outputs in registers; unit 0 runs butterflies
// 0 (bins r*NS: DC/Nyquist, the self-paired L/2, and pairs r, R - r) and
// NS/2 (pairs r, R-1-r).  Each pair is post-processed and stored to HBM
// directly:
//   E = (Z[k] + conj Z[L-k])/2, O = (Z[k] - conj Z[L-k])/(2i),
//   X[k] = E + W_N^k O, X[L-k] = conj(E - W_N^k O),
//   X[0] = Re Z0 + Im Z0, X[L] = Re Z0 - Im Z0,
// so the pass's output never goes through shared memory and no separate
// post-process loop reads it back.  Win: the previous pass's output.
template <class S>
__device__ __forceinline__ void codelet_last_r2c(const PipeCtx& c, const float2* Win, const float2* tw, int tw_off,
                                                 const float2* post)
{
    constexpr int P = S::NP - 1;
    constexpr int R = S::R[P];
    constexpr int NS = S::L / R;
    constexpr int L = S::L;
    constexpr int UPT = (NS / 2) / S::NTHR;  // units per thread
    const float sc = c.scale;
    const float s2 = c.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
    float2* out = c.out2;
    auto load = [&](int j, float2 (&z)[R]) {
        sfor<R>([&](auto rr) {
            constexpr int r = decltype(rr)::value;
            z[r] = Win[cpad<S>(j + r * NS)];
        });
    };
    // pair (k, L - k) with k < L/2, or the self-paired k = L/2
    auto pair = [&](int k, float2 zk, float2 zn) {
        const float2 zc = cconj(zn);
        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
        const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
        const float2 wo = cmul(post[k], o);
        out[k] = cscale(cadd(e, wo), s2);
        if (L - k != k) out[L - k] = cscale(cconj(csub(e, wo)), s2);
    };
    sfor<UPT>([&](auto ii) {
        constexpr int i = decltype(ii)::value;
        const int u = c.tid + i * S::NTHR;
        float2 a[R], b[R];
        if (u == 0) {
            // butterfly 0 has no twiddles; butterfly NS/2 has the constants
            // W_L^{(NS/2) r} = W_{2R}^r
            load(0, a);
            load(NS / 2, b);
            sfor<R - 1>([&](auto rr) {
                constexpr int r = decltype(rr)::value + 1;
                b[r] = twc<2 * R, r>(b[r]);
            });
            DFT<R>::run(a);
            DFT<R>::run(b);
            const float2 z0 = a[0];
            out[0] = make_float2((z0.x + z0.y) * sc, 0.f);
            out[L] = make_float2((z0.x - z0.y) * sc, 0.f);
            sfor<R / 2>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                if constexpr (r > 0) pair(r * NS, a[r], a[R - r]);
            });
            pair(L / 2, a[R / 2], a[R / 2]);
            sfor<R / 2>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                pair(NS / 2 + r * NS, b[r], b[R - 1 - r]);
            });
        } else {
            // butterfly NS-u's twiddles from butterfly u's table entries:
            // W_L^{(NS-u) r} = W_R^r conj(W_L^{u r})
            load(u, a);
            load(NS - u, b);
            sfor<R - 1>([&](auto rr) {
                constexpr int r = decltype(rr)::value + 1;
                const float2 w = tw[tw_off + u + r * NS];
                a[r] = cmul(a[r], w);
                b[r] = twc<R, r>(cmulc(b[r], w));
            });
            DFT<R>::run(a);
            DFT<R>::run(b);
            sfor<R / 2>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                pair(u + r * NS, a[r], b[R - 1 - r]);
                pair(NS - u + r * NS, b[r], a[R - 1 - r]);
            });
        }
    });
}

// Shared-memory layout (byte offsets from the dynamic shared base):
//   [0, 8)                         mbarrier of the table copies
//   [smem_tw, ...)                 pass tables (CTA-wide), at smem_tw + (src % 16)
//   [smem_post, ...)               post-process twiddles (CTA-wide), likewise
//   [smem_stage + g*group_bytes)   group g: 64 B barriers/flags, then NST
//                                  slots of stage_bytes.  A slot holds one
//                                  transform: its raw input row at offset
//                                  src % 16, then (in place, from offset 16)
//                                  the padded work layout WA; with nbuf 2
//                                  the group's work buffer WB (lpad float2)
//                                  follows at group offset smem_work.
//
// Slot fill: the row of transform t starts at src = in + t*row_bytes and is
// placed at slot + (src % 16), so the 16-byte aligned superset
// [src - src%16, ceil16(src + row_bytes)) is copied by one bulk copy.  The
// superset only touches bytes of the neighbouring rows of the same buffer;
// when it would reach outside the buffer (first/last row with unaligned
// ends) the group copies the row with ordinary loads instead.
// FC2R: the even-C2R instance (pre-process fused into the first pass, see
// codelet_pass); FR2C: the even-R2C instance (post-process fused into the
// last pass, see codelet_last_r2c); the plain instance serves every mode.
template <class S, bool FC2R = false, bool FR2C = false>
__global__ void __launch_bounds__(S::MAXT, S::MINB) codelet_kernel(const __grid_constant__ RowArgs A)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    const float2* gtw = reinterpret_cast<const float2*>(A.tw);
    const float2* gpost = reinterpret_cast<const float2*>(A.post_tw);
    // tables: bulk copies of the 16-byte aligned supersets of the pass-table
    // window and of the post-process twiddles; each lands at its region's
    // start, so a table sits (src % 16) bytes in
    const uintptr_t tw_src = reinterpret_cast<uintptr_t>(gtw + A.tw_lo);
    const uintptr_t post_src = reinterpret_cast<uintptr_t>(gpost);
    float2* stw = reinterpret_cast<float2*>(smraw + A.smem_tw + (tw_src & 15));
    float2* spost = reinterpret_cast<float2*>(smraw + A.smem_post + (post_src & 15));
    uint64_t* tbar = reinterpret_cast<uint64_t*>(smraw);
    constexpr int L = S::L;
    const int g = threadIdx.x / S::NTHR;
    const int tid = threadIdx.x - g * S::NTHR;
    const int NG = A.ngroups;
    const int NST = A.nstage;
    const int bar_id = 1 + g;
    const bool leader = tid == 0;
    unsigned char* gbase = smraw + A.smem_stage + (int64_t)g * A.group_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase);
    volatile int* flags = reinterpret_cast<int*>(gbase + 32);  // [0] abort, [1+s] manual copy
    unsigned char* slots = gbase + 64;

    const int64_t row_bytes = A.in_dist * A.in_esize;
    const int64_t gstride = (int64_t)gridDim.x * NG;
    const int64_t gfirst = (int64_t)blockIdx.x * NG + g;
    const uintptr_t buf_lo = reinterpret_cast<uintptr_t>(A.in);
    const uintptr_t buf_hi = buf_lo + (uintptr_t)(A.ntf * row_bytes);

    auto issue = [&](int s, int64_t t) {  // group leader only
        const uintptr_t src = buf_lo + (uintptr_t)(t * row_bytes);
        const uintptr_t c0 = src & ~(uintptr_t)15;
        const uintptr_t c1 = (src + (uintptr_t)row_bytes + 15) & ~(uintptr_t)15;
        if (c0 >= buf_lo && c1 <= buf_hi) {
            flags[1 + s] = 0;
            mbar_expect_tx(&bars[s], (uint32_t)(c1 - c0));
            bulk_copy_g2s(slots + (int64_t)s * A.stage_bytes, reinterpret_cast<const void*>(c0),
                          (uint32_t)(c1 - c0), &bars[s]);
        } else {
            flags[1 + s] = 1;
        }
    };
    // host-mapped input: every thread of the group copies its share of the
    // same superset with 16-byte cp.async and commits one group per slot
    // fill (an empty one when there is no transform left), so that waiting
    // for all but the newest NST-1 groups completes the oldest slot
    const bool host_in = A.host_in != 0;
    auto issue_all = [&](int s, int64_t t) {  // every thread of the group
        if (t < A.ntf) {
            const uintptr_t src = buf_lo + (uintptr_t)(t * row_bytes);
            const uintptr_t c0 = src & ~(uintptr_t)15;
            const uintptr_t c1 = (src + (uintptr_t)row_bytes + 15) & ~(uintptr_t)15;
            const bool inside = c0 >= buf_lo && c1 <= buf_hi;
            if (inside) {
                unsigned char* dst = slots + (int64_t)s * A.stage_bytes;
                const int nch = (int)((c1 - c0) >> 4);
                for (int i = tid; i < nch; i += S::NTHR)
                    cp_async16(dst + 16 * i, reinterpret_cast<const void*>(c0 + 16 * (uintptr_t)i));
            }
            if (leader) flags[1 + s] = inside ? 0 : 1;
        }
        cp_async_commit();
    };
    // prologue: thread 0 starts the table copies (plan-owned memory, safe
    // before the wait for the preceding grid), then each group leader starts
    // its input prefetches once that grid is complete; no thread reads the
    // tables before the table barrier completes
    uint32_t phase = 0;
    if (threadIdx.x == 0) {
        const uint32_t tw_bytes = A.tw_cnt > 0 ? (uint32_t)(((tw_src + (uintptr_t)A.tw_cnt * 8 + 15) & ~(uintptr_t)15) -
                                                           (tw_src & ~(uintptr_t)15))
                                               : 0u;
        const uint32_t post_bytes =
            A.post_cnt > 0 ? (uint32_t)(((post_src + (uintptr_t)A.post_cnt * 8 + 15) & ~(uintptr_t)15) -
                                        (post_src & ~(uintptr_t)15))
                           : 0u;
        mbar_init(tbar, 1);
        fence_mbar_init();
        mbar_expect_tx(tbar, tw_bytes + post_bytes);
        if (tw_bytes)
            bulk_copy_g2s(smraw + A.smem_tw, reinterpret_cast<const void*>(tw_src & ~(uintptr_t)15), tw_bytes, tbar);
        if (post_bytes)
            bulk_copy_g2s(smraw + A.smem_post, reinterpret_cast<const void*>(post_src & ~(uintptr_t)15), post_bytes,
                          tbar);
    }
    pdl_wait();
    if (leader) {
        for (int s = 0; s < NST; ++s) mbar_init(&bars[s], 1);
        flags[0] = 0;
        fence_mbar_init();
        if (!host_in) {
            for (int s = 0; s < NST; ++s) {
                const int64_t t = gfirst + (int64_t)s * gstride;
                if (t < A.ntf) issue(s, t);
            }
        }
    }
    if (host_in) {
        for (int s = 0; s < NST; ++s) issue_all(s, gfirst + (int64_t)s * gstride);
    }
    __syncthreads();  // the only CTA-wide barrier: barriers initialised
    if (!mbar_wait_bounded(tbar, 0)) {
        if (host_in) cp_async_wait_all();
        // the tables never arrived: record it and leave after the group's
        // own copies have landed (or their wait ran out as well)
        if (leader) {
            atomicOr(A.err, 1);
            for (int s = 0; s < NST; ++s) {
                const int64_t t = gfirst + (int64_t)s * gstride;
                if (t < A.ntf && !flags[1 + s]) mbar_wait_bounded(&bars[s], 0);
            }
        }
        return;
    }
    const float2* tw = stw - A.tw_lo;
    const float2* post = spost;
    const bool last_global = A.io_mode != IO_R2C_EVEN;
    const bool pp = A.nbuf == 2;  // the group has a work buffer at gbase + smem_work
    float2 v[S::E];
    constexpr int NPP = (L / 2 + 1 + S::NTHR - 1) / S::NTHR;  // C2R pre-process pairs per thread

    for (int64_t it = 0;; ++it) {
        const int64_t t = gfirst + it * gstride;
        if (t >= A.ntf) break;
        const int s = (int)(it % NST);
        if (host_in) {
            cp_async_wait_pending(NST - 1);  // this thread's copies into slot s have landed
        } else if (leader && !flags[1 + s]) {
            if (!mbar_wait_bounded(&bars[s], (phase >> s) & 1u)) flags[0] = 1;
            phase ^= 1u << s;
        }
        group_sync<S>(bar_id);
        if (flags[0]) {
            if (leader) {
                atomicOr(A.err, 1);
                for (int k = 1; k < NST; ++k) {
                    const int s2 = (s + k) % NST;
                    const int64_t t2 = gfirst + (it + k) * gstride;
                    if (t2 < A.ntf && !flags[1 + s2]) mbar_wait_bounded(&bars[s2], (phase >> s2) & 1u);
                }
            }
            break;
        }
        const uintptr_t src = buf_lo + (uintptr_t)(t * row_bytes);
        unsigned char* row = slots + (int64_t)s * A.stage_bytes + (src & 15);
        if (flags[1 + s]) {
            const float* gs = reinterpret_cast<const float*>(src);
            for (int64_t i = tid; i < row_bytes / 4; i += S::NTHR)
                reinterpret_cast<float*>(row)[i] = host_in ? gs[i] : __ldg(gs + i);
            group_sync<S>(bar_id);
        }
        // work layouts (padded, 16-byte aligned): WA inside the slot (it
        // overlaps the raw row), WB the group's work buffer (nbuf 2)
        float2* WA = reinterpret_cast<float2*>(slots + (int64_t)s * A.stage_bytes + 16);
        float2* WB = pp ? reinterpret_cast<float2*>(gbase + A.smem_work) : WA;
        PipeCtx c;
        c.L = L;
        c.nthr = S::NTHR;
        c.tid = tid;
        c.ok_sm = true;
        c.ok_io = true;
        c.pshift = S::PSHIFT;
        c.tw = tw;
        c.sA = WA;
        c.sB = WB;
        c.st2 = reinterpret_cast<const float2*>(row);
        c.st1 = reinterpret_cast<const float*>(row);
        c.mode = A.io_mode;
        c.conj_in = A.conj_in;
        c.conj_out = A.conj_out;
        c.weight = A.weight;
        c.nreal = A.nreal;
        c.scale = A.scale;
        c.out2 = reinterpret_cast<float2*>(A.out) + t * A.out_dist;
        c.out1 = reinterpret_cast<float*>(A.out) + t * A.out_dist;
        c.wl = A.wload ? A.wload + t * A.wdist : nullptr;

        // the slot is free once no later stage reads it: refill it with the
        // transform NST iterations ahead (group leader, after a group barrier
        // that follows the last read of the slot)
        bool refilled = false;
        auto refill = [&]() {
            refilled = true;
            if (host_in) {
                issue_all(s, gfirst + (it + NST) * gstride);
            } else if (leader) {
                const int64_t nt = gfirst + (it + NST) * gstride;
                if (nt < A.ntf) {
                    fence_proxy_async_smem();
                    issue(s, nt);
                }
            }
        };
        // shared-writing stages: the C2R pre-process, then every pass but a
        // last one that writes HBM.  With a work buffer, stage i writes WB
        // when K-1-i is even (so the last one writes WB) and WA otherwise;
        // without one, every stage runs in place in WA.
        const bool pre = !FC2R && A.io_mode == IO_C2R_EVEN;
        const int K = (pre ? 1 : 0) + S::NP - ((last_global || FR2C) ? 1 : 0);
        auto out_of = [&](int i) { return (pp && ((K - 1 - i) & 1) == 0) ? WB : WA; };
        int stage = 0;
        const float2* cur = WA;  // input of the next stage once the raw row is consumed
        bool from_slot = true;
        if (pre) {
            // pre-process pairs (k, L-k):
            //   Z'[k] = E + i*O,  E = X[k] + conj(X[L-k]),
            //   O = (X[k] - conj(X[L-k])) * conj(W_N^k), stored conjugated.
            // All pairs are read into registers before any is written when
            // the output overlaps the raw row.
            float2* Wo = out_of(0);
            const bool half = A.weight == WEIGHT_LOAD_HALF;
            float2 pa[NPP], pb[NPP];
            sfor<NPP>([&](auto qq) {
                constexpr int q = decltype(qq)::value;
                const int k = tid + q * S::NTHR;
                if (k <= (L >> 1)) {
                    pa[q] = c.st2[k];
                    pb[q] = c.st2[L - k];
                    if (c.wl) {
                        pa[q] = cscale(pa[q], __ldg(c.wl + k));
                        pb[q] = cscale(pb[q], __ldg(c.wl + (L - k)));
                    }
                }
            });
            if (Wo == WA) group_sync<S>(bar_id);
            sfor<NPP>([&](auto qq) {
                constexpr int q = decltype(qq)::value;
                const int k = tid + q * S::NTHR;
                if (k == 0) {
                    const float x0 = pa[q].x, xl = pb[q].x;  // Im of DC/Nyquist ignored
                    Wo[0] = make_float2(x0 + xl, -(x0 - xl));
                } else if (k <= (L >> 1)) {
                    float2 a = pa[q], b = pb[q];
                    if (half) {
                        a = cscale(a, 0.5f);
                        b = cscale(b, 0.5f);
                    }
                    const float2 w = post[k];
                    const float2 bc = cconj(b);
                    const float2 e = cadd(a, bc);
                    const float2 o = cmulc(csub(a, bc), w);
                    Wo[cpad<S>(k)] = cconj(make_float2(e.x - o.y, e.y + o.x));
                    if (L - k != k) Wo[cpad<S>(L - k)] = cconj(make_float2(e.x + o.y, -e.y + o.x));
                }
            });
            group_sync<S>(bar_id);
            cur = Wo;
            from_slot = false;
            if (pp && ++stage == K) refill();
        }
        sfor<S::NP>([&](auto pidx) {
            constexpr int P = decltype(pidx)::value;
            if constexpr (FR2C && P == S::NP - 1) {
                codelet_last_r2c<S>(c, cur, tw, A.ip.pass[P].tw_off, post);
                return;
            }
            const bool global_last = P == S::NP - 1 && last_global;
            float2* Wo = global_last ? WA : out_of(stage);
            // a barrier between loads and stores: in place (the output is the
            // input, or overlaps the slot's raw row), or after the loads of a
            // last pass that reads the slot, before the slot is refilled
            const bool sync_loaded = global_last ? (from_slot || cur == WA) : (from_slot ? Wo == WA : cur == Wo);
            codelet_pass<S, P, FC2R && P == 0>(c, cur, Wo, v, tw, A.ip.pass[P].tw_off, from_slot, last_global,
                                                sync_loaded, bar_id, post);
            from_slot = false;
            if (!global_last) {
                cur = Wo;
                if (pp && ++stage == K) refill();
            }
        });
        if constexpr (FR2C) {
            // the fused last pass read the previous pass's output, which may
            // sit in the slot: every read precedes its refill
            if (!refilled) group_sync<S>(bar_id);
        } else if (A.io_mode == IO_R2C_EVEN) {
            // post-process pairs:
            //   E = (Z[k] + conj Z[L-k])/2, O = (Z[k] - conj Z[L-k])/(2i)
            //   X[k] = E + W^k O, X[L-k] = conj(E - W^k O),
            //   X[0] = Re Z0 + Im Z0, X[L] = Re Z0 - Im Z0 (zero imaginary parts)
            // every pair of the thread is read (and its twiddle) before any
            // is stored, so the shared loads of all its pairs are in flight
            // together
            const float sc = A.scale;
            const float s2 = A.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
            constexpr int NPO = (L / 2 + 1 + S::NTHR - 1) / S::NTHR;  // pairs per thread
            // pairs are handled in chunks of PCH (all of them when few), every
            // pair of a chunk read before any is stored; the reads only touch
            // shared memory and the stores only global memory, so chunks need
            // no barrier
            constexpr int PCH = NPO <= 8 ? NPO : 4;
            const float2* Z = cur;
            sfor<(NPO + PCH - 1) / PCH>([&](auto cc) {
                constexpr int q0 = decltype(cc)::value * PCH;
                float2 za[PCH], zb[PCH], wk[PCH];
                sfor<PCH>([&](auto qq) {
                    constexpr int q = q0 + decltype(qq)::value;
                    const int k = tid + q * S::NTHR;
                    if (q < NPO && k <= (L >> 1)) {
                        za[q - q0] = Z[cpad<S>(k)];
                        zb[q - q0] = Z[cpad<S>(L - k)];  // k = 0: entry L, unused
                        wk[q - q0] = post[k];
                    }
                });
                sfor<PCH>([&](auto qq) {
                    constexpr int q = q0 + decltype(qq)::value;
                    const int k = tid + q * S::NTHR;
                    if (q >= NPO) return;
                    if (k == 0) {
                        const float2 z0 = za[q - q0];
                        c.out2[0] = make_float2((z0.x + z0.y) * sc, 0.f);
                        c.out2[L] = make_float2((z0.x - z0.y) * sc, 0.f);
                    } else if (k <= (L >> 1)) {
                        const float2 zk = za[q - q0], zc = cconj(zb[q - q0]);
                        const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
                        const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
                        const float2 wo = cmul(wk[q - q0], o);
                        c.out2[k] = cscale(cadd(e, wo), s2);
                        if (L - k != k) c.out2[L - k] = cscale(cconj(csub(e, wo)), s2);
                    }
                });
            });
            // the slot is read here when there is no work buffer: all reads
            // precede its refill (a work buffer is protected by the barrier
            // at the next transform's start)
            if (!refilled) group_sync<S>(bar_id);
        }
        if (!refilled) refill();
    }
    if (host_in) cp_async_wait_all();
}

// Column tiles: tfpc adjacent columns of a strided axis (column c, element
// r at base(c) + r*in_stride, base as in the column kernel) per tile, one
// codelet transform group per column.  The tile is loaded cooperatively
// (consecutive threads take consecutive columns of a row, so every row of
// the tile is one contiguous HBM segment), each group runs the codelet's
// in-place passes on its column, and the tile is stored back the same way.
// Persistent over tiles; in-place calls are safe (a tile is fully read
// before it is written).
template <class S>
__global__ void __launch_bounds__(S::MAXT, S::MINB) coltile_kernel(const __grid_constant__ ColArgs A)
{
    extern __shared__ __align__(128) unsigned char smraw[];
    pdl_wait();
    constexpr int L = S::L;
    const int TF = A.tfpc;
    const int g = threadIdx.x / S::NTHR;
    const int tid = threadIdx.x - g * S::NTHR;
    const int bar_id = 1 + g;
    float2* stw = reinterpret_cast<float2*>(smraw);
    float2* tile = reinterpret_cast<float2*>(smraw + (((int64_t)A.tw_cnt * 8 + 127) & ~(int64_t)127));
    const float2* gtw = reinterpret_cast<const float2*>(A.tw);
    for (int i = threadIdx.x; i < A.tw_cnt; i += blockDim.x) stw[i] = ldg2(gtw + A.tw_lo + i);
    const float2* tw = A.tw_cnt > 0 ? stw - A.tw_lo : gtw;
    __syncthreads();

    PipeCtx c;
    c.L = L;
    c.nthr = S::NTHR;
    c.tid = tid;
    c.ok_sm = true;
    c.ok_io = true;
    c.pshift = S::PSHIFT;
    c.tw = tw;
    c.mode = IO_C2C;
    c.conj_in = 0;
    c.conj_out = 0;
    c.scale = 1.f;
    c.wl = nullptr;
    float2 v[S::E];
    float2* W = tile + (int64_t)g * A.wsize;

    // this thread's column within a tile and its first row; rows step by NTHR
    const int cc = threadIdx.x % TF;
    const int r0 = threadIdx.x / TF;
    const int rstep = blockDim.x / TF;
    const int64_t ntiles = (A.ncols + TF - 1) / TF;
    const float2* gin = reinterpret_cast<const float2*>(A.in);
    float2* gout = reinterpret_cast<float2*>(A.out);
    const float sc = A.scale;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t col = t * TF + cc;
        const bool ok = col < A.ncols;
        const int64_t cl = ok ? col : 0;
        const int64_t item = cl / A.cpi;
        const int64_t j = cl - item * A.cpi;
        const float2* ib = gin + item * A.in_dist + (j / A.in_split) * A.in_hi + (j % A.in_split) * A.in_lo;
        float2* ob = gout + item * A.out_dist + (j / A.out_split) * A.out_hi + (j % A.out_split) * A.out_lo;
        float2* Wc = tile + (int64_t)cc * A.wsize;
        if (ok) {
            // batches of 8 independent loads per thread keep enough bytes in
            // flight for the strided rows (one load at a time leaves the SM
            // waiting on HBM latency)
            for (int r = r0; r < L; r += 8 * rstep) {
                float2 x[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int rr = r + u * rstep;
                    x[u] = rr < L ? ldg2(ib + (int64_t)rr * A.in_stride) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int rr = r + u * rstep;
                    if (rr < L) Wc[cpad<S>(rr)] = A.conj_in ? cconj(x[u]) : x[u];
                }
            }
        }
        __syncthreads();
        if (g < TF) {
            sfor<S::NP>([&](auto pp) {
                constexpr int P = decltype(pp)::value;
                codelet_pass<S, P>(c, W, W, v, tw, A.ip.pass[P].tw_off, false, false, true, bar_id);
            });
        }
        __syncthreads();
        if (ok) {
            for (int r = r0; r < L; r += rstep) {
                float2 x = Wc[cpad<S>(r)];
                if (A.conj_out) x.y = -x.y;
                ob[(int64_t)r * A.out_stride] = sc == 1.f ? x : cscale(x, sc);
            }
        }
        __syncthreads();
    }
}

}  // namespace gfft
