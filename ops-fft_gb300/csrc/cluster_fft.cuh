// cluster_fft.cuh - long transforms (complex length N = Q*P up to 65536) on
// one thread-block cluster per transform, with a single HBM read and a
// single HBM write per element.  MODE 0 is a C2C transform; MODE 1 an even
// R2C of length 2N (real input viewed as N complex values, the even/odd
// post-process fused after the row phase); MODE 2 an even C2R of length 2N
// (the Hermitian pre-process fused into the column loads).
//
// View the input of one transform as Q rows of P (x[q*P + p]).  Then
//   X[k_q + Q*k_p] = sum_p W_P^{p*k_p} W_N^{p*k_q} sum_q x[q*P + p] W_Q^{q*k_q}.
// The C CTAs of a cluster split the work:
//   column phase (CTA c): columns p in [c*P/C, (c+1)*P/C).  Each thread owns
//     one column lane and loads its radix-Q0 butterfly inputs straight from
//     HBM into registers (consecutive lanes read consecutive columns, so
//     every warp load covers whole row segments; the loads of the next
//     transform are issued before the row phase of the current one), runs
//     the Q-point Stockham transform (radix Q0 then Q1, one exchange through
//     shared memory), multiplies bin k_q = j + r*Q0 by
//     W_N^{p*k_q} = W_N^{p*j} * W_N^{p*Q0*r} (two small tables laid out
//     [index][column], so lanes read consecutive entries) and stores the
//     value into receive buffer b (b = transform parity) of CTA
//     d = k_q / (Q/C): row k_q % (Q/C), column p, rows padded to P+1 float2.
//     Remote values travel as st.async with a byte count on d's "full[b]"
//     mbarrier; values for the CTA itself are plain shared stores followed
//     by one arrival per thread on the same mbarrier;
//   row phase (CTA d): waits for full[b] (all M elements delivered), reads
//     its radix-P0 inputs from the receive buffer, runs the P-point
//     transform (one exchange through shared memory) and writes bin
//     k_q + Q*k_p; consecutive lanes hold consecutive k_q, so every warp
//     store covers whole Q/C-element output runs.
// Buffer release: one extra "signal" warp per CTA meets the compute warps
// at a named barrier once they have read receive buffer b, executes one
// fence.acq_rel.cluster and arrives (lane r on CTA r) on every CTA's
// "free[b]" mbarrier; a producer
// waits for all C arrivals before it writes buffer b again.  The fence of
// that release pattern therefore stalls only the signal warp, never the compute
// warps, while the bar.sync + release/acquire chain still orders every read
// of buffer b before the next writes into it.
// There is no cluster-wide barrier inside the loop: the mbarriers carry the
// data dependences, so a fast CTA runs ahead until it needs a slower one's
// data.  Every mbarrier wait is bounded (~2 s); on expiry the thread sets
// bit 3 of the error word and a CTA-wide abort flag that makes every later
// wait return at once, so the loop ends (with garbage output) and all CTAs
// meet at the final cluster barrier.  The hardware co-schedules the CTAs of
// a cluster, so that barrier always completes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterfly.cuh"
#include "cluster_list.h"
#include "kernel_args.h"
#include "pdl.cuh"

namespace gfft {
namespace {

template <int ID_, int N_, int C_, int Q_, int P_, int NT_, int MINB_, int Q0_, int Q1_, int P0_, int P1_>
struct ClSpec {
    static constexpr int N = N_, C = C_, Q = Q_, P = P_, NT = NT_, MINB = MINB_;
    static constexpr int Q0 = Q0_, Q1 = Q1_, P0 = P0_, P1 = P1_;
    static constexpr int PC = P / C;   // columns per CTA
    static constexpr int QC = Q / C;   // rows per CTA
    static constexpr int M = N / C;    // elements per CTA
    static constexpr int RP = P + 1;   // receive-row pitch (float2)
    static constexpr int NSA = NT / PC;  // butterfly slots per column
    static constexpr int NSB = NT / QC;  // butterfly slots per row
    static constexpr int NBA0 = (Q / Q0) / NSA, NBA1 = (Q / Q1) / NSA;
    static constexpr int NBB0 = (P / P0) / NSB, NBB1 = (P / P1) / NSB;
    static constexpr int mx(int a, int b) { return a > b ? a : b; }
    static constexpr int E = mx(mx(NBA0 * Q0, NBA1 * Q1), mx(NBB0 * P0, NBB1 * P1));
    // shared memory, float2 offsets: header (4 mbarriers + abort flag),
    // pass tables, outer-twiddle tables, exchange buffer, 2 receive buffers
    static constexpr int O_HDR = 0;
    static constexpr int O_TQ = 8;
    static constexpr int O_TP = O_TQ + Q;
    static constexpr int O_TA = O_TP + P;       // W_N^{p*j}, j < Q0: [j][column]
    static constexpr int O_TB = O_TA + Q0 * PC;  // W_N^{p*Q0*r}, r < Q1: [r][column]
    static constexpr int O_X = O_TB + Q1 * PC;   // real modes: post/pre twiddles (Q + P + QC)
    static constexpr int O_S = O_X + Q + P + QC;
    static constexpr int RBUF = QC * RP;
    static constexpr int O_R = O_S + M;          // receive buffer b at O_R + b*RBUF
    static constexpr int TOTAL = O_R + 2 * RBUF;
    static constexpr int SMEM = TOTAL * 8;
    static constexpr uint32_t RX_BYTES = (uint32_t)((C - 1) * QC * PC * 8);  // remote bytes per transform
    static constexpr int H = QC / 2;  // R2C: rows k_q (and their mirrors Q - k_q) per CTA
    static_assert(QC % 2 == 0 && (NT / (QC / 2)) <= P && P % (NT / (QC / 2)) == 0, "R2C post-process split");
    static_assert(Q * P == N && Q0 * Q1 == Q && P0 * P1 == P, "factorisation");
    static_assert(P % C == 0 && Q % C == 0, "cluster split");
    static_assert(NT % PC == 0 && NT % QC == 0, "lanes per line");
    static_assert(NBA0 >= 1 && NBA1 >= 1 && NBB0 >= 1 && NBB1 >= 1, "butterflies per thread");
    static_assert(NBA0 * NSA == Q / Q0 && NBA1 * NSA == Q / Q1, "column butterflies divide evenly");
    static_assert(NBB0 * NSB == P / P0 && NBB1 * NSB == P / P1, "row butterflies divide evenly");
    static_assert(NT % 32 == 0 && NT <= 1024, "block size");
    static_assert(SMEM <= 227 * 1024, "shared memory");
    static_assert(C >= 2 && C <= 16, "cluster size");
};

__device__ __forceinline__ uint32_t cl_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_id()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_count()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire;" ::: "memory"); }
__device__ __forceinline__ uint32_t shared_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
// address of the same shared-memory offset in CTA `rank` of this cluster
__device__ __forceinline__ uint32_t cl_map(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

__device__ __forceinline__ void named_sync(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void mb_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mb_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// arrival of this thread on a barrier of its own CTA, ordering its earlier
// shared-memory stores before the phase completes
__device__ __forceinline__ void mb_arrive_local(uint32_t bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// arrival on a barrier of another CTA (shared::cluster address); ordering
// comes from a preceding fence.acq_rel.cluster
__device__ __forceinline__ void mb_arrive_remote_relaxed(uint32_t bar_cl)
{
    asm volatile("mbarrier.arrive.relaxed.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cl) : "memory");
}
__device__ __forceinline__ bool mb_try_wait_cluster(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// asynchronous store into another CTA's shared memory; completion counts
// 8 bytes on that CTA's mbarrier
__device__ __forceinline__ void st_async(uint32_t addr_cl, float2 v, uint32_t bar_cl)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(addr_cl),
                 "f"(v.x), "f"(v.y), "r"(bar_cl)
                 : "memory");
}

template <class K, int MODE>
__global__ void __launch_bounds__(K::NT + 32, K::MINB) cluster_kernel(const __grid_constant__ ClusterArgs A)
{
    extern __shared__ __align__(16) float2 sm[];
    constexpr int Q = K::Q, P = K::P, PC = K::PC, QC = K::QC;
    constexpr int NA0 = K::NBA0 * K::Q0;  // column-phase inputs per thread
    constexpr int NTT = K::NT + 32;       // compute threads + the signal warp
    const int tid = threadIdx.x;
    const uint32_t rank = cl_rank();
    const int64_t cid = cl_id();
    const int64_t ncl = cl_count();
    const float2* gtw = static_cast<const float2*>(A.tw);
    float2* TQ = sm + K::O_TQ;
    float2* TP = sm + K::O_TP;
    float2* TA = sm + K::O_TA;
    float2* TB = sm + K::O_TB;
    float2* S = sm + K::O_S;
    float2* TX = sm + K::O_X;
    const float2* gpost = gtw + A.post_off;  // real modes: W_{2N}^i, i <= N
    constexpr int H = K::H;
    // header: full[0], full[1], free[0], free[1], abort flag
    const uint32_t hdr = shared_u32(sm + K::O_HDR);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + K::O_HDR + 4);

    // the first transform's column inputs are requested right after the
    // table loads, before the barrier set-up (compute threads only; pf
    // stays in registers)
    const int ca = tid % PC, sa = tid / PC;  // column lane, butterfly slot
    const float2* gin = static_cast<const float2*>(A.in);
    float2 pf[NA0];
    auto load_columns = [&](int64_t t) {
        const float2* x = gin + t * A.in_dist + rank * PC + ca;
        sfor<K::NBA0>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sa + b * K::NSA;
            sfor<K::Q0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                pf[b * K::Q0 + r] = __ldcs(x + (int64_t)(j + r * (Q / K::Q0)) * P);
            });
        });
    };
    for (int i = tid; i < Q; i += NTT) TQ[i] = __ldg(gtw + A.twq_off + i);
    for (int i = tid; i < P; i += NTT) TP[i] = __ldg(gtw + A.twp_off + i);
    for (int i = tid; i < (K::Q0 + K::Q1) * PC; i += NTT) {
        const int row = i / PC;
        const int64_t p = (int64_t)rank * PC + (i - row * PC);
        const int64_t m = row < K::Q0 ? row : (int64_t)(row - K::Q0) * K::Q0;
        TA[i] = __ldg(gtw + A.outer_off + (p * m) % K::N);  // TB follows TA contiguously
    }
    if constexpr (MODE == 2) {
        for (int i = tid; i < Q; i += NTT) TX[i] = __ldg(gpost + (int64_t)i * P);  // W_{2N}^{q*P}
    }
    if constexpr (MODE == 1) {
        for (int i = tid; i < P; i += NTT) TX[i] = __ldg(gpost + (int64_t)i * Q);  // W_{2N}^{Q*k_p}
        for (int i = tid; i <= H; i += NTT) TX[P + i] = __ldg(gpost + (i < H ? (int)rank * H + i : Q / 2));
    }
    // the tables above belong to the plan; everything below touches the
    // caller's buffers, so it waits for the grids this launch depends on
    // (the first column loads then overlap the barrier set-up)
    pdl_wait();
    if (tid < K::NT && cid < A.ntf) load_columns(cid);
    if (tid == 0) {
        mb_init(hdr + 0, 1 + K::NT);
        mb_init(hdr + 8, 1 + K::NT);
        mb_init(hdr + 16, K::C);
        mb_init(hdr + 24, K::C);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mb_expect_tx(hdr + 0, K::RX_BYTES);
        mb_expect_tx(hdr + 8, K::RX_BYTES);
    }
    // every CTA of the cluster has started and initialised its barriers
    // (its shared memory may be written remotely from now on)
    cl_arrive();
    cl_wait();

    if (tid >= K::NT) {
        // signal warp: after the compute warps have read receive buffer b of
        // transform it, re-arm full[b] for transform it+2 and release
        // buffer b to every producer
        int64_t it = 0;
        for (int64_t t = cid; t < A.ntf; t += ncl, ++it) {
            const uint32_t b = (uint32_t)(it & 1);
            named_sync(2, NTT);
            const int lane = tid - K::NT;
            if (lane == 0) mb_expect_tx(hdr + 8 * b, K::RX_BYTES);
            __syncwarp();
            // one release fence, then relaxed arrivals (lane r -> CTA r): a
            // release pattern for each of them, one fence per transform
            asm volatile("fence.acq_rel.cluster;" ::: "memory");
            if (lane < K::C) mb_arrive_remote_relaxed(cl_map(hdr + 16 + 8 * b, (uint32_t)lane));
        }
        cl_arrive();
        cl_wait();
        return;
    }

    auto wait = [&](uint32_t bar, uint32_t parity) {
        if (*abort_flag) return;
        const long long t0 = clock64();
        while (!mb_try_wait_cluster(bar, parity)) {
            if (*abort_flag) return;
            if (clock64() - t0 > (1ll << 32)) {
                *abort_flag = 1;
                atomicOr(A.err, 8);
                return;
            }
        }
    };

    const int cb = tid % QC, sb = tid / QC;  // row lane, butterfly slot
    const uint32_t r_col = shared_u32(sm + K::O_R + rank * PC + ca);  // this lane's column, buffer 0
    float2* gout = static_cast<float2*>(A.out);
    const float sc = A.scale;
    float2 v[K::E];
    int64_t it = 0;
    for (int64_t t = cid; t < A.ntf; t += ncl, ++it) {
        const uint32_t b = (uint32_t)(it & 1);
        const uint32_t u = (uint32_t)(it >> 1);
        const uint32_t full_b = hdr + 8 * b, free_b = hdr + 16 + 8 * b;
        // ---- column phase, pass 0 (radix Q0, ns = 1): prefetched inputs
        if constexpr (MODE == 2) {
            // Hermitian pre-process of bin k = q*P + p from X[k] and X[N-k]
            // (X[N] for k = 0), stored conjugated for the forward transform:
            //   e = X[k] + conj X[N-k], o = (X[k] - conj X[N-k]) * conj W_{2N}^k,
            //   Z'[k] = conj(e.x - o.y, e.y + o.x);  Z'[0] = (x0 + xN, -(x0 - xN))
            const float2* xin = gin + t * A.in_dist;
            const int p = (int)rank * PC + ca;
            float2 bv[NA0];
            sfor<K::NBA0>([&](auto bb) {
                constexpr int b2 = decltype(bb)::value;
                const int j = sa + b2 * K::NSA;
                sfor<K::Q0>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    const int k = (j + r * (Q / K::Q0)) * P + p;
                    bv[b2 * K::Q0 + r] = __ldcs(xin + (k == 0 ? K::N : K::N - k));
                });
            });
            const float2 wp = __ldg(gpost + p);
            const bool half = A.weight == WEIGHT_LOAD_HALF;
            sfor<K::NBA0>([&](auto bb) {
                constexpr int b2 = decltype(bb)::value;
                const int j = sa + b2 * K::NSA;
                sfor<K::Q0>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    constexpr int i = b2 * K::Q0 + r;
                    const int q = j + r * (Q / K::Q0);
                    float2 a = pf[i], bq = bv[i];
                    if (q == 0 && p == 0) {
                        v[i] = make_float2(a.x + bq.x, -(a.x - bq.x));
                    } else {
                        if (half) {
                            a = cscale(a, 0.5f);
                            bq = cscale(bq, 0.5f);
                        }
                        const float2 w = cmul(TX[q], wp);
                        const float2 bc = cconj(bq);
                        const float2 e = cadd(a, bc);
                        const float2 o = cmulc(csub(a, bc), w);
                        v[i] = make_float2(e.x - o.y, -(e.y + o.x));
                    }
                });
            });
        } else {
            sfor<NA0>([&](auto ii) {
                constexpr int i = decltype(ii)::value;
                v[i] = pf[i];
                if (A.conj_in) v[i].y = -v[i].y;
            });
        }
        sfor<K::NBA0>([&](auto bb) { DFT<K::Q0>::run(&v[decltype(bb)::value * K::Q0]); });
        named_sync(1, K::NT);  // the previous transform's row-phase reads of S are done
        sfor<K::NBA0>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sa + b2 * K::NSA;
            sfor<K::Q0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                S[(j * K::Q0 + r) * PC + ca] = v[b2 * K::Q0 + r];
            });
        });
        named_sync(1, K::NT);
        // ---- column phase, pass 1 (radix Q1, ns = Q0): j < Q0, bin k_q = j + r*Q0
        sfor<K::NBA1>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sa + b2 * K::NSA;
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                float2 w = S[(j + r * K::Q0) * PC + ca];
                if constexpr (r > 0) w = cmul(w, TQ[r * K::Q0 + j]);
                v[b2 * K::Q1 + r] = w;
            });
            DFT<K::Q1>::run(&v[b2 * K::Q1]);
            const float2 wj = TA[j * PC + ca];
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                if constexpr (r == 0) {
                    v[b2 * K::Q1] = cmul(v[b2 * K::Q1], wj);
                } else {
                    v[b2 * K::Q1 + r] = cmul(v[b2 * K::Q1 + r], cmul(wj, TB[r * PC + ca]));
                }
            });
        });
        if (it >= 2) wait(free_b, (u - 1) & 1u);  // every CTA has read buffer b of transform it-2
        const uint32_t r_col_b = r_col + b * (uint32_t)(K::RBUF * 8);
        sfor<K::NBA1>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sa + b2 * K::NSA;
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const int kq = j + r * K::Q0;
                uint32_t d;
                int l;
                if constexpr (MODE == 1) {
                    // rows k_q and Q - k_q on the same CTA: [d*H, (d+1)*H) and
                    // their mirrors; CTA 0 also holds row Q/2 (mirror slot 0)
                    if (kq == 0) {
                        d = 0;
                        l = 0;
                    } else if (kq == Q / 2) {
                        d = 0;
                        l = H;
                    } else if (kq < Q / 2) {
                        d = (uint32_t)(kq / H);
                        l = kq - (int)d * H;
                    } else {
                        const int m = Q - kq;
                        d = (uint32_t)(m / H);
                        l = H + m - (int)d * H;
                    }
                } else {
                    d = (uint32_t)(kq / QC);
                    l = kq - (int)d * QC;
                }
                const uint32_t addr = r_col_b + (uint32_t)(l * K::RP) * 8u;
                if (d == rank) {
                    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v[b2 * K::Q1 + r].x),
                                 "f"(v[b2 * K::Q1 + r].y)
                                 : "memory");
                } else {
                    st_async(cl_map(addr, d), v[b2 * K::Q1 + r], cl_map(full_b, d));
                }
            });
        });
        mb_arrive_local(full_b);  // this thread's own-CTA values are stored
        if (t + ncl < A.ntf) load_columns(t + ncl);
        wait(full_b, u & 1u);  // all M values of this CTA's rows have arrived
        // ---- row phase, pass 0 (radix P0, ns = 1): inputs from receive buffer b
        const float2* Rrow = sm + K::O_R + b * K::RBUF + cb * K::RP;
        sfor<K::NBB0>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sb + b2 * K::NSB;
            sfor<K::P0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b2 * K::P0 + r] = Rrow[j + r * (P / K::P0)];
            });
        });
        sfor<K::NBB0>([&](auto bb) { DFT<K::P0>::run(&v[decltype(bb)::value * K::P0]); });
        sfor<K::NBB0>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sb + b2 * K::NSB;
            sfor<K::P0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                S[(j * K::P0 + r) * QC + cb] = v[b2 * K::P0 + r];
            });
        });
        named_sync(2, NTT);  // receive buffer b fully read (the signal warp releases it); S written
        // ---- row phase, pass 1 (radix P1, ns = P0): bin k_p = j + r*P0
        sfor<K::NBB1>([&](auto bb) {
            constexpr int b2 = decltype(bb)::value;
            const int j = sb + b2 * K::NSB;
            sfor<K::P1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                float2 w = S[(j + r * K::P0) * QC + cb];
                if constexpr (r > 0) w = cmul(w, TP[r * K::P0 + j]);
                v[b2 * K::P1 + r] = w;
            });
            DFT<K::P1>::run(&v[b2 * K::P1]);
        });
        if constexpr (MODE != 1) {
            float2* y = gout + t * A.out_dist + rank * QC + cb;
            sfor<K::NBB1>([&](auto bb) {
                constexpr int b2 = decltype(bb)::value;
                const int j = sb + b2 * K::NSB;
                sfor<K::P1>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    float2 o = v[b2 * K::P1 + r];
                    if (A.conj_out) o.y = -o.y;
                    if (sc != 1.f) o = cscale(o, sc);
                    __stcs(y + (int64_t)(j + r * K::P0) * Q, o);
                });
            });
        } else {
            // Z of every owned row to S ([k_p][row]), then the even/odd
            // post-process of the pairs (k, N - k), both rows on this CTA:
            //   E = (Z[k] + conj Z[N-k])/2, O = (Z[k] - conj Z[N-k])/(2i),
            //   X[k] = E + W_{2N}^k O, X[N-k] = conj(E - W_{2N}^k O),
            //   X[0] = Re Z0 + Im Z0, X[N] = Re Z0 - Im Z0.
            named_sync(1, K::NT);  // every read of S above is done
            sfor<K::NBB1>([&](auto bb) {
                constexpr int b2 = decltype(bb)::value;
                const int j = sb + b2 * K::NSB;
                sfor<K::P1>([&](auto rr) {
                    constexpr int r = decltype(rr)::value;
                    S[(j + r * K::P0) * QC + cb] = v[b2 * K::P1 + r];
                });
            });
            named_sync(1, K::NT);
            float2* y = gout + t * A.out_dist;
            const float s2 = A.weight == WEIGHT_STORE_X2 ? 2.f * sc : sc;
            constexpr int NS2 = K::NT / H;
            const int l = tid % H, s0 = tid / H;
            // pair (k, N - k): Z values zk, zn; twiddle w = W_{2N}^k
            auto pair = [&](int64_t k, int64_t kn, float2 zk, float2 zn, float2 w) {
                const float2 zc = cconj(zn);
                const float2 e = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
                const float2 o = make_float2(0.5f * (zk.y - zc.y), 0.5f * (zc.x - zk.x));
                const float2 wo = cmul(w, o);
                __stcs(y + k, cscale(cadd(e, wo), s2));
                if (kn != k) __stcs(y + kn, cscale(cconj(csub(e, wo)), s2));
            };
            if (rank != 0 || l != 0) {
                const int kq = (int)rank * H + l;
                const float2 wl = TX[P + l];
                for (int kp = s0; kp < P; kp += NS2) {
                    const int kpn = P - 1 - kp;
                    pair(kq + (int64_t)Q * kp, (Q - kq) + (int64_t)Q * kpn, S[kp * QC + l], S[kpn * QC + H + l],
                         cmul(wl, TX[kp]));
                }
            } else {
                // rows 0 (pairs k_p, P - k_p) and Q/2 (pairs k_p, P - 1 - k_p)
                const float2 wh = TX[P + H];
                for (int kp = s0; kp < P; kp += NS2) {
                    if (kp == 0) {
                        const float2 z0 = S[0];
                        __stcs(y, make_float2((z0.x + z0.y) * sc, 0.f));
                        __stcs(y + K::N, make_float2((z0.x - z0.y) * sc, 0.f));
                        const int m = P / 2 - 1;  // the row-Q/2 pair no k_p > P/2 covers
                        pair(Q / 2 + (int64_t)Q * m, Q / 2 + (int64_t)Q * (P - 1 - m), S[m * QC + H],
                             S[(P - 1 - m) * QC + H], cmul(wh, TX[m]));
                    } else if (kp <= P / 2) {
                        pair((int64_t)Q * kp, (int64_t)Q * (P - kp), S[kp * QC], S[(P - kp) * QC], TX[kp]);
                    } else {
                        const int m = kp - P / 2 - 1;
                        pair(Q / 2 + (int64_t)Q * m, Q / 2 + (int64_t)Q * (P - 1 - m), S[m * QC + H],
                             S[(P - 1 - m) * QC + H], cmul(wh, TX[m]));
                    }
                }
            }
        }
    }
    // no CTA leaves while another may still access its shared memory
    cl_arrive();
    cl_wait();
}

struct ClState {
    int prepared[64];
    int clusters[64];
};

template <class K, int MODE>
int prepare_t(ClState& s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return -(int)e;
    dev &= 63;
    if (s.prepared[dev]) return s.clusters[dev];
    e = cudaFuncSetAttribute(cluster_kernel<K, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM);
    if (e == cudaSuccess && K::C > 8)
        e = cudaFuncSetAttribute(cluster_kernel<K, MODE>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return -(int)e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(K::C * 1024, 1, 1);
    cfg.blockDim = dim3(K::NT + 32, 1, 1);
    cfg.dynamicSmemBytes = K::SMEM;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, cluster_kernel<K, MODE>, &cfg);
    if (e != cudaSuccess) return -(int)e;
    if (n < 1) return -(int)cudaErrorInvalidConfiguration;
    s.clusters[dev] = n;
    s.prepared[dev] = 1;
    return n;
}

template <class K, int MODE>
int launch_t(const ClusterArgs* a, cudaStream_t st)
{
    if (a->csize != K::C || a->smem_bytes != K::SMEM || a->clusters < 1 || a->ntf < 1 || a->io_mode != MODE)
        return (int)cudaErrorInvalidValue;
    const int64_t ncl = a->ntf < a->clusters ? a->ntf : a->clusters;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    (void)cfg;
    return (int)launch_pdl(cluster_kernel<K, MODE>, dim3((unsigned)(ncl * K::C)), dim3(K::NT + 32), (size_t)K::SMEM,
                           st, *a, &attr[0]);
}

#define GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) ClSpec<ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1>

// Per-mode dispatch over the configurations of cluster_list.h (one
// translation unit per mode instantiates these).
template <int MODE>
int prepare_mode(int kid, ClState* st)
{
#define GFFT_CL_PREP(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) \
    if (kid == ID) return prepare_t<GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1), MODE>(st[ID]);
    GFFT_CLUSTERS(GFFT_CL_PREP)
#undef GFFT_CL_PREP
    return -(int)cudaErrorInvalidValue;
}

template <int MODE>
int launch_mode(const ClusterArgs* a, cudaStream_t st)
{
#define GFFT_CL_LAUNCH(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) \
    if (a->kid == ID) return launch_t<GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1), MODE>(a, st);
    GFFT_CLUSTERS(GFFT_CL_LAUNCH)
#undef GFFT_CL_LAUNCH
    return (int)cudaErrorInvalidValue;
}

}  // namespace
}  // namespace gfft
