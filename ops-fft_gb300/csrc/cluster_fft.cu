// cluster_fft.cu - configuration lookup and mode dispatch of the
// thread-block-cluster transforms (kernels in cluster_fft.cuh, instantiated
// per mode in cluster_c2c.cu, cluster_r2c.cu and cluster_c2r.cu).
#include "cluster_fft.cuh"

using namespace gfft;

extern "C" {
int gfft_cluster_prepare_m0(int kid);
int gfft_cluster_prepare_m1(int kid);
int gfft_cluster_prepare_m2(int kid);
int gfft_cluster_launch_m0(const ClusterArgs* a, void* stream);
int gfft_cluster_launch_m1(const ClusterArgs* a, void* stream);
int gfft_cluster_launch_m2(const ClusterArgs* a, void* stream);
}

extern "C" int gfft_cluster_lookup(long long n, int want_c, int* csize, int* q, int* p, int* q0, int* p0,
                                   int* nt, int* smem_bytes)
{
#define GFFT_CL_LOOKUP(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)                                         \
    if (n == N && (want_c <= 0 || want_c == C)) {                                                     \
        if (csize) *csize = C;                                                                        \
        if (q) *q = Q;                                                                                \
        if (p) *p = P;                                                                                \
        if (q0) *q0 = Q0;                                                                             \
        if (p0) *p0 = P0;                                                                             \
        if (nt) *nt = NT;                                                                             \
        if (smem_bytes) *smem_bytes = GFFT_CL_SPEC(ID, N, C, Q, P, NT, MB, Q0, Q1, P0, P1)::SMEM;     \
        return ID;                                                                                    \
    }
    GFFT_CLUSTERS(GFFT_CL_LOOKUP)
#undef GFFT_CL_LOOKUP
    return -1;
}

extern "C" int gfft_cluster_prepare(int kid, int mode)
{
    switch (mode) {
    case IO_C2C: return gfft_cluster_prepare_m0(kid);
    case IO_R2C_EVEN: return gfft_cluster_prepare_m1(kid);
    case IO_C2R_EVEN: return gfft_cluster_prepare_m2(kid);
    default: return -(int)cudaErrorInvalidValue;
    }
}

extern "C" int gfft_launch_cluster(const ClusterArgs* a, void* stream)
{
    switch (a->io_mode) {
    case IO_C2C: return gfft_cluster_launch_m0(a, stream);
    case IO_R2C_EVEN: return gfft_cluster_launch_m1(a, stream);
    case IO_C2R_EVEN: return gfft_cluster_launch_m2(a, stream);
    default: return (int)cudaErrorInvalidValue;
    }
}
