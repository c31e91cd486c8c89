// Cluster kernels, complex-to-complex mode, for every configuration of
// cluster_list.h (see cluster_fft.cuh).
#include "cluster_fft.cuh"

namespace {
gfft::ClState g_state[GFFT_NUM_CLUSTER_CFGS];
}

extern "C" int gfft_cluster_prepare_m0(int kid) { return gfft::prepare_mode<0>(kid, g_state); }

extern "C" int gfft_cluster_launch_m0(const gfft::ClusterArgs* a, void* stream)
{
    return gfft::launch_mode<0>(a, static_cast<cudaStream_t>(stream));
}
