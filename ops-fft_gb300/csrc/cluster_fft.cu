// cluster_fft.cu - long C2C transforms (N = Q*P up to 65536) on one
// thread-block cluster per transform, with a single HBM read and a single
// HBM write per element.
//
// View the input of one transform as Q rows of P (x[q*P + p]).  Then
//   X[k_q + Q*k_p] = sum_p W_P^{p*k_p} W_N^{p*k_q} sum_q x[q*P + p] W_Q^{q*k_q}.
// The C CTAs of a cluster split the work:
//   column phase (CTA c): columns p in [c*P/C, (c+1)*P/C).  Each thread owns
//     one column lane and loads its radix-Q0 butterfly inputs straight from
//     HBM into registers (consecutive lanes read consecutive columns, so
//     every warp load covers whole row segments), runs the Q-point Stockham
//     transform (radix Q0 then Q1, one exchange through shared memory),
//     multiplies bin k_q by W_N^{p*k_q} (a per-CTA table in shared memory,
//     laid out [k_q][column] so lanes read consecutive entries) and stores the
//     value into the receive buffer of CTA d = k_q / (Q/C) over distributed
//     shared memory (row k_q % (Q/C), column p; rows padded to P+1 float2);
//   row phase (CTA d): rows k_q in [d*Q/C, (d+1)*Q/C).  Each thread owns one
//     row lane, reads its radix-P0 inputs from the receive buffer, runs the
//     P-point transform (one exchange through shared memory) and writes bin
//     k_q + Q*k_p; consecutive lanes hold consecutive k_q, so every warp
//     store covers whole Q/C-element output runs.
// Synchronisation per transform: cluster barrier X (all blocks delivered)
// and cluster barrier Y (every CTA has read its receive buffer, so the next
// transform may overwrite it), split into arrive/wait halves; two CTA-wide
// barriers protect the shared exchange buffer.  The hardware co-schedules
// the CTAs of a cluster, so the barriers always complete.
#include <cuda_runtime.h>
#include <stdint.h>

#include "butterfly.cuh"
#include "cluster_list.h"
#include "kernel_args.h"

namespace gfft {
namespace {

template <int ID_, int N_, int C_, int Q_, int P_, int NT_, int MINB_, int Q0_, int Q1_, int P0_, int P1_>
struct ClSpec {
    static constexpr int ID = ID_, N = N_, C = C_, Q = Q_, P = P_, NT = NT_, MINB = MINB_;
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
    // shared memory, float2 offsets
    static constexpr int O_TQ = 0;
    static constexpr int O_TP = O_TQ + Q;
    static constexpr int O_T = O_TP + P;
    static constexpr int O_S = O_T + M;
    static constexpr int O_R = O_S + M;
    static constexpr int TOTAL = O_R + QC * RP;
    static constexpr int SMEM = TOTAL * 8;
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
__device__ __forceinline__ void cl_store(uint32_t addr, float2 v)
{
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}

template <class K>
__global__ void __launch_bounds__(K::NT, K::MINB) cluster_kernel(const __grid_constant__ ClusterArgs A)
{
    extern __shared__ __align__(16) float2 sm[];
    constexpr int Q = K::Q, P = K::P, PC = K::PC, QC = K::QC;
    const int tid = threadIdx.x;
    const uint32_t rank = cl_rank();
    const int64_t cid = cl_id();
    const int64_t ncl = cl_count();
    const float2* gtw = static_cast<const float2*>(A.tw);
    float2* TQ = sm + K::O_TQ;
    float2* TP = sm + K::O_TP;
    float2* T = sm + K::O_T;
    float2* S = sm + K::O_S;
    float2* R = sm + K::O_R;

    for (int i = tid; i < Q; i += K::NT) TQ[i] = __ldg(gtw + A.twq_off + i);
    for (int i = tid; i < P; i += K::NT) TP[i] = __ldg(gtw + A.twp_off + i);
    for (int i = tid; i < K::M; i += K::NT) {
        const int kq = i / PC;
        const int c = i - kq * PC;
        const int e = (int)(((int64_t)rank * PC + c) * kq % K::N);
        T[i] = __ldg(gtw + A.outer_off + e);
    }
    // every CTA of the cluster has started (its shared memory may be
    // written remotely from now on) and the tables are in place
    cl_arrive();
    cl_wait();

    const int ca = tid % PC, sa = tid / PC;  // column lane, butterfly slot
    const int cb = tid % QC, sb = tid / QC;  // row lane, butterfly slot
    const uint32_t r_col = shared_u32(R + rank * PC + ca);  // this lane's column in any receive buffer
    const float2* gin = static_cast<const float2*>(A.in);
    float2* gout = static_cast<float2*>(A.out);
    const float sc = A.scale;
    float2 v[K::E];
    int64_t it = 0;
    for (int64_t t = cid; t < A.ntf; t += ncl, ++it) {
        // ---- column phase, pass 0 (radix Q0, ns = 1): inputs from HBM
        const float2* x = gin + t * A.in_dist + rank * PC + ca;
        sfor<K::NBA0>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sa + b * K::NSA;
            sfor<K::Q0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b * K::Q0 + r] = __ldcs(x + (int64_t)(j + r * (Q / K::Q0)) * P);
            });
        });
        if (A.conj_in) {
            sfor<K::NBA0 * K::Q0>([&](auto ii) { v[decltype(ii)::value].y = -v[decltype(ii)::value].y; });
        }
        sfor<K::NBA0>([&](auto bb) { DFT<K::Q0>::run(&v[decltype(bb)::value * K::Q0]); });
        __syncthreads();  // the previous transform's row-phase reads of S are done
        sfor<K::NBA0>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sa + b * K::NSA;
            sfor<K::Q0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                S[(j * K::Q0 + r) * PC + ca] = v[b * K::Q0 + r];
            });
        });
        __syncthreads();
        // ---- column phase, pass 1 (radix Q1, ns = Q0): j < Q0, bin k_q = j + r*Q0
        sfor<K::NBA1>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sa + b * K::NSA;
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                float2 u = S[(j + r * K::Q0) * PC + ca];
                if constexpr (r > 0) u = cmul(u, TQ[r * K::Q0 + j]);
                v[b * K::Q1 + r] = u;
            });
            DFT<K::Q1>::run(&v[b * K::Q1]);
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b * K::Q1 + r] = cmul(v[b * K::Q1 + r], T[(j + r * K::Q0) * PC + ca]);
            });
        });
        if (it > 0) cl_wait();  // Y of the previous transform: receive buffers are free
        sfor<K::NBA1>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sa + b * K::NSA;
            sfor<K::Q1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                const int kq = j + r * K::Q0;
                const uint32_t d = (uint32_t)(kq / QC);
                const uint32_t off = (uint32_t)((kq - (int)d * QC) * K::RP) * 8u;
                cl_store(cl_map(r_col + off, d), v[b * K::Q1 + r]);
            });
        });
        cl_arrive();  // X: this thread's blocks are delivered
        cl_wait();
        // ---- row phase, pass 0 (radix P0, ns = 1): inputs from the receive buffer
        const float2* Rrow = R + cb * K::RP;
        sfor<K::NBB0>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sb + b * K::NSB;
            sfor<K::P0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                v[b * K::P0 + r] = Rrow[j + r * (P / K::P0)];
            });
        });
        cl_arrive();  // Y: this thread has read its receive-buffer inputs
        sfor<K::NBB0>([&](auto bb) { DFT<K::P0>::run(&v[decltype(bb)::value * K::P0]); });
        sfor<K::NBB0>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sb + b * K::NSB;
            sfor<K::P0>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                S[(j * K::P0 + r) * QC + cb] = v[b * K::P0 + r];
            });
        });
        __syncthreads();
        // ---- row phase, pass 1 (radix P1, ns = P0): bin k_p = j + r*P0
        float2* y = gout + t * A.out_dist + rank * QC + cb;
        sfor<K::NBB1>([&](auto bb) {
            constexpr int b = decltype(bb)::value;
            const int j = sb + b * K::NSB;
            sfor<K::P1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                float2 u = S[(j + r * K::P0) * QC + cb];
                if constexpr (r > 0) u = cmul(u, TP[r * K::P0 + j]);
                v[b * K::P1 + r] = u;
            });
            DFT<K::P1>::run(&v[b * K::P1]);
            sfor<K::P1>([&](auto rr) {
                constexpr int r = decltype(rr)::value;
                float2 o = v[b * K::P1 + r];
                if (A.conj_out) o.y = -o.y;
                if (sc != 1.f) o = cscale(o, sc);
                __stcs(y + (int64_t)(j + r * K::P0) * Q, o);
            });
        });
    }
    if (it > 0) cl_wait();  // no CTA leaves while another may still read or write its shared memory
}

struct ClState {
    int prepared[64];
    int clusters[64];
};

template <class K>
int prepare_t(ClState& s)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return -(int)e;
    dev &= 63;
    if (s.prepared[dev]) return s.clusters[dev];
    e = cudaFuncSetAttribute(cluster_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, K::SMEM);
    if (e == cudaSuccess && K::C > 8)
        e = cudaFuncSetAttribute(cluster_kernel<K>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return -(int)e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(K::C * 1024, 1, 1);
    cfg.blockDim = dim3(K::NT, 1, 1);
    cfg.dynamicSmemBytes = K::SMEM;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, cluster_kernel<K>, &cfg);
    if (e != cudaSuccess) return -(int)e;
    if (n < 1) return -(int)cudaErrorInvalidConfiguration;
    s.clusters[dev] = n;
    s.prepared[dev] = 1;
    return n;
}

template <class K>
int launch_t(const ClusterArgs* a, cudaStream_t st)
{
    if (a->csize != K::C || a->smem_bytes != K::SMEM || a->clusters < 1 || a->ntf < 1)
        return (int)cudaErrorInvalidValue;
    const int64_t ncl = a->ntf < a->clusters ? a->ntf : a->clusters;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(ncl * K::C), 1, 1);
    cfg.blockDim = dim3(K::NT, 1, 1);
    cfg.dynamicSmemBytes = K::SMEM;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, cluster_kernel<K>, *a);
    return (int)e;
}

#define GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) ClSpec<ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1>

ClState g_state[GFFT_NUM_CLUSTER_CFGS];

}  // namespace
}  // namespace gfft

using namespace gfft;

extern "C" int gfft_cluster_lookup(long long n, int want_c, int* csize, int* q, int* p, int* q0, int* p0,
                                   int* nt, int* smem_bytes)
{
#define GFFT_CL_LOOKUP(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)                \
    if (n == N && (want_c <= 0 || want_c == C)) {                            \
        if (csize) *csize = C;                                               \
        if (q) *q = Q;                                                       \
        if (p) *p = P;                                                       \
        if (q0) *q0 = Q0;                                                    \
        if (p0) *p0 = P0;                                                    \
        if (nt) *nt = NT;                                                    \
        if (smem_bytes) *smem_bytes = GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)::SMEM; \
        return ID;                                                           \
    }
    GFFT_CLUSTERS(GFFT_CL_LOOKUP)
#undef GFFT_CL_LOOKUP
    return -1;
}

extern "C" int gfft_cluster_prepare(int kid)
{
#define GFFT_CL_PREP(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) \
    if (kid == ID) return prepare_t<GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)>(g_state[ID]);
    GFFT_CLUSTERS(GFFT_CL_PREP)
#undef GFFT_CL_PREP
    return -(int)cudaErrorInvalidValue;
}

extern "C" int gfft_launch_cluster(const ClusterArgs* a, void* stream)
{
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
#define GFFT_CL_LAUNCH(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1) \
    if (a->kid == ID) return launch_t<GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)>(a, st);
    GFFT_CLUSTERS(GFFT_CL_LAUNCH)
#undef GFFT_CL_LAUNCH
    return (int)cudaErrorInvalidValue;
}
