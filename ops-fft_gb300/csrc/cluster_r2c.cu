// Cluster kernels, even real-to-complex (fused post-process) mode, for every configuration of
// cluster_list.h (see cluster_fft.cuh).
#include "cluster_fft.cuh"

namespace {
gfft::ClState g_state[GFFT_NUM_CLUSTER_CFGS];
}

extern "C" int gfft_cluster_prepare_m1(int kid) { return gfft::prepare_mode<1>(kid, g_state); }

extern "C" int gfft_cluster_launch_m1(const gfft::ClusterArgs* a, void* stream)
{
    return gfft::launch_mode<1>(a, static_cast<cudaStream_t>(stream));
}
