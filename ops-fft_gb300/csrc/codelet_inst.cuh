// codelet_inst.cuh - one translation unit per codelet_list.h entry:
// a codelet_<id>.cu file holds GFFT_CODELET_TU(<id>), which instantiates
// that entry's row and column-tile kernels and their launchers only.
#pragma once
#include "codelet.cuh"
#include "codelet_list.h"
#include "launch_common.cuh"

namespace gfft {

template <int ID>
struct CodeletSpec;
#define GFFT_SPEC_OF(ID, MT, MB, L, NT, ...) \
    template <>                              \
    struct CodeletSpec<ID> {                 \
        using type = CSpec<MT, MB, L, NT, __VA_ARGS__>; \
    };
GFFT_CODELETS(GFFT_SPEC_OF)
#undef GFFT_SPEC_OF

// Lengths whose even-C2R launches use the instance with the pre-process fused
// into the first pass (a second kernel per length, so the plain instance's
// register allocation is unchanged).  Measured: C2R N=1024 12.7 -> 11.5 us
// (batch 4096); no gain for the 1500-point codelet (N=3000), which keeps
// the separate pre-process.
template <class S>
constexpr bool fuse_c2r()
{
    return S::L == 512 || S::L == 1024 || S::L == 2048;
}

// OPS_FFT_FUSE_R2C=0 keeps even-R2C launches on the plain instance (separate
// post-process after the last pass) instead of the fused one (read once).
inline bool fuse_r2c_enabled()
{
    static const bool on = [] {
        const char* v = std::getenv("OPS_FFT_FUSE_R2C");
        return !(v && v[0] == '0');
    }();
    return on;
}

}  // namespace gfft

#define GFFT_CODELET_TU(ID)                                                              \
    namespace gfft {                                                                     \
    int launch_codelet_##ID(const RowArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        using S_ = CodeletSpec<ID>::type;                                                \
        if constexpr (fuse_c2r<S_>())                                                    \
            if (a->io_mode == IO_C2R_EVEN) return launch_codelet_t<S_, true>(a, st);    \
        if constexpr (fuse_r2c_spec<S_>())                                               \
            if (a->io_mode == IO_R2C_EVEN && fuse_r2c_enabled())                        \
                return launch_codelet_t<S_, false, true>(a, st);                        \
        return launch_codelet_t<S_>(a, st);                                              \
    }                                                                                    \
    int launch_coltile_##ID(const ColArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        return launch_coltile_t<CodeletSpec<ID>::type>(a, st);                           \
    }                                                                                    \
    }
