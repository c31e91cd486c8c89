// launch_common.cuh - host-side launch helpers for the Stockham kernels.
#pragma once
#include <cuda_runtime.h>

#include "codelet.cuh"
#include "pdl.cuh"
#include "codelet_list.h"
#include "row_pipe.cuh"
#include "stockham.cuh"

namespace gfft {

// Opt a kernel into >48 KB of dynamic shared memory once per device.
template <class K>
inline cudaError_t ensure_smem_attr(K kernel, unsigned long long& done_mask, size_t bytes)
{
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done_mask & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMaxSmemBytes);
    if (e == cudaSuccess) done_mask |= bit;
    return e;
}

inline int sm_count()
{
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    int& c = cached[dev & 63];
    if (c == 0 && cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) c = 0;
    return c;
}

template <int RMAX>
int launch_row_t(const RowArgs* a, cudaStream_t st)
{
    static unsigned long long attr_mask = 0;
    static thread_local int last_threads = -1, last_smem = -1, last_occ = 1;
    const int threads = a->ip.nthr * a->tfpc;
    if (threads <= 0 || threads > kernel_max_threads<RMAX>() || a->ntf <= 0) return (int)cudaErrorInvalidValue;
    if (a->smem_bytes <= 0 || a->smem_bytes > kMaxSmemBytes || a->nstage < 1 || a->nstage > 4)
        return (int)cudaErrorInvalidValue;
    cudaError_t e = ensure_smem_attr(row_kernel<RMAX>, attr_mask, (size_t)a->smem_bytes);
    if (e != cudaSuccess) return (int)e;
    if (threads != last_threads || a->smem_bytes != last_smem) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, row_kernel<RMAX>, threads, (size_t)a->smem_bytes);
        if (e != cudaSuccess) return (int)e;
        last_threads = threads;
        last_smem = a->smem_bytes;
        last_occ = occ < 1 ? 1 : occ;
    }
    const int64_t ntiles = (a->ntf + a->tfpc - 1) / a->tfpc;
    int64_t grid = (int64_t)sm_count() * last_occ;
    if (a->grid > 0) grid = a->grid;
    if (grid < 1) grid = 1;
    if (grid > ntiles) grid = ntiles;
    return (int)launch_pdl(row_kernel<RMAX>, dim3((unsigned)grid), dim3(threads), (size_t)a->smem_bytes, st, *a);
}

template <int RMAX>
int launch_col_t(const ColArgs* a, cudaStream_t st)
{
    static unsigned long long attr_mask = 0;
    const int threads = a->ip.nthr * a->tfpc;
    if (threads <= 0 || threads > kernel_max_threads<RMAX>() || a->ncols <= 0) return (int)cudaErrorInvalidValue;
    const size_t smem = (size_t)a->nbuf * (size_t)a->ip.L * (size_t)a->tfp * sizeof(float2);
    if (smem > (size_t)kMaxSmemBytes) return (int)cudaErrorInvalidValue;
    cudaError_t e = ensure_smem_attr(col_kernel<RMAX>, attr_mask, smem);
    if (e != cudaSuccess) return (int)e;
    const int64_t grid = (a->ncols + a->tfpc - 1) / a->tfpc;
    if (grid > 0x7fffffff) return (int)cudaErrorInvalidValue;
    return (int)launch_pdl(col_kernel<RMAX>, dim3((unsigned)grid), dim3(threads), smem, st, *a);
}

template <class S, bool FC2R = false, bool FR2C = false>
int launch_codelet_t(const RowArgs* a, cudaStream_t st)
{
    static unsigned long long attr_mask = 0;
    static thread_local int last_threads = -1, last_smem = -1, last_occ = 1;
    const int threads = S::NTHR * a->ngroups;
    if (a->ip.L != S::L || a->ngroups < 1 || a->ngroups > 15 || threads > S::MAXT || a->ntf <= 0)
        return (int)cudaErrorInvalidValue;
    if (a->smem_bytes <= 0 || a->smem_bytes > kMaxSmemBytes || a->nstage < 1 || a->nstage > 4)
        return (int)cudaErrorInvalidValue;
    cudaError_t e = ensure_smem_attr(codelet_kernel<S, FC2R, FR2C>, attr_mask, (size_t)a->smem_bytes);
    if (e != cudaSuccess) return (int)e;
    if (threads != last_threads || a->smem_bytes != last_smem) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, codelet_kernel<S, FC2R, FR2C>, threads, (size_t)a->smem_bytes);
        if (e != cudaSuccess) return (int)e;
        last_threads = threads;
        last_smem = a->smem_bytes;
        last_occ = occ < 1 ? 1 : occ;
    }
    const int64_t nslots = (a->ntf + a->tfpc - 1) / a->tfpc;
    const int64_t ctas_needed = (nslots + a->ngroups - 1) / a->ngroups;
    int64_t grid = (int64_t)sm_count() * last_occ;
    if (a->grid > 0) grid = a->grid;
    if (grid < 1) grid = 1;
    if (grid > ctas_needed) grid = ctas_needed;
    return (int)launch_pdl(codelet_kernel<S, FC2R, FR2C>, dim3((unsigned)grid), dim3(threads), (size_t)a->smem_bytes, st, *a);
}

template <class S>
int launch_coltile_t(const ColArgs* a, cudaStream_t st)
{
    static unsigned long long attr_mask = 0;
    static thread_local int last_threads = -1, last_smem = -1, last_occ = 1;
    const int threads = S::NTHR * a->tfpc;
    if (a->ip.L != S::L || a->tfpc < 1 || threads > S::MAXT || a->ncols <= 0 || a->wsize <= 0)
        return (int)cudaErrorInvalidValue;
    if (a->smem_bytes <= 0 || a->smem_bytes > kMaxSmemBytes) return (int)cudaErrorInvalidValue;
    cudaError_t e = ensure_smem_attr(coltile_kernel<S>, attr_mask, (size_t)a->smem_bytes);
    if (e != cudaSuccess) return (int)e;
    if (threads != last_threads || a->smem_bytes != last_smem) {
        int occ = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, coltile_kernel<S>, threads, (size_t)a->smem_bytes);
        if (e != cudaSuccess) return (int)e;
        last_threads = threads;
        last_smem = a->smem_bytes;
        last_occ = occ < 1 ? 1 : occ;
    }
    const int64_t ntiles = (a->ncols + a->tfpc - 1) / a->tfpc;
    int64_t grid = (int64_t)sm_count() * last_occ;
    if (grid < 1) grid = 1;
    if (grid > ntiles) grid = ntiles;
    return (int)launch_pdl(coltile_kernel<S>, dim3((unsigned)grid), dim3(threads), (size_t)a->smem_bytes, st, *a);
}

#define GFFT_DECL_LAUNCH(ID, ...)                           \
    int launch_codelet_##ID(const RowArgs* a, cudaStream_t st); \
    int launch_coltile_##ID(const ColArgs* a, cudaStream_t st);
GFFT_CODELETS(GFFT_DECL_LAUNCH)
#undef GFFT_DECL_LAUNCH
int launch_row_r16(const RowArgs* a, cudaStream_t st);
int launch_row_r47(const RowArgs* a, cudaStream_t st);
int launch_col_r16(const ColArgs* a, cudaStream_t st);
int launch_col_r47(const ColArgs* a, cudaStream_t st);

}  // namespace gfft
