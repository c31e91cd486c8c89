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

}  // namespace gfft

#define GFFT_CODELET_TU(ID)                                                              \
    namespace gfft {                                                                     \
    int launch_codelet_##ID(const RowArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        return launch_codelet_t<CodeletSpec<ID>::type>(a, st);                           \
    }                                                                                    \
    int launch_coltile_##ID(const ColArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        return launch_coltile_t<CodeletSpec<ID>::type>(a, st);                           \
    }                                                                                    \
    }
