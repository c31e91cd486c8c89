// pdl.cuh - programmatic dependent launch for the transform kernels.
//
// Every transform kernel is launched with programmatic stream serialisation
// allowed: the next kernel of the stream is launched as this one's CTAs
// exit (a CTA that exits counts as having signalled its dependents), so its
// CTAs take the SMs the drain frees and run their prologue while the last
// CTAs of this kernel finish.  A dependent kernel may only prepare before
// pdl_wait(): initialise barriers and load tables the plan owns (the
// twiddle blob is written at plan time, never by an exec).  pdl_wait()
// returns once every prerequisite grid has completed and its memory is
// visible, so every access to a caller's buffer or a workspace comes after
// it.  Without a programmatic dependency it is a no-op.
//
// Measured on GB300 (graphs of 20 launches): signalling dependents at kernel
// start instead (griddepcontrol.launch_dependents) made short launches
// slower (R2C N=1024 x 4096 10.5 -> 11.1 us, C2C 4096 x 256 on clusters
// 7.1 -> 8.2 us); letting the exits signal gives 9.6 and 7.0 us.
#pragma once
#include <cuda_runtime.h>

#include <cstdlib>

namespace gfft {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// OPS_FFT_PDL=0 launches without programmatic dependencies (read once).
inline bool pdl_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("OPS_FFT_PDL");
        return !(v && v[0] == '0');
    }();
    return on;
}

// cudaLaunchKernelEx with the programmatic-serialisation attribute (when
// enabled) after up to one extra attribute (e.g. a cluster shape).
template <class Kern, class Arg>
inline cudaError_t launch_pdl(Kern kernel, dim3 grid, dim3 block, size_t smem, cudaStream_t st, const Arg& arg,
                              const cudaLaunchAttribute* extra = nullptr)
{
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[2];
    unsigned n = 0;
    if (extra) attr[n++] = *extra;
    if (pdl_enabled()) {
        attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[n].val.programmaticStreamSerializationAllowed = 1;
        ++n;
    }
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = n ? attr : nullptr;
    cfg.numAttrs = n;
    return cudaLaunchKernelEx(&cfg, kernel, arg);
}

}  // namespace gfft
