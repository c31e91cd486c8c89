// Instantiates codelet 3 of codelet_list.h.
#include "codelet.cuh"
#include "codelet_list.h"
#include "launch_common.cuh"

namespace gfft {
#define GFFT_INST(ID, MT, MB, L, NT, ...)                                                        \
    int launch_codelet_##ID(const RowArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        return launch_codelet_t<CSpec<MT, MB, L, NT, __VA_ARGS__>>(a, st);                       \
    }                                                                                    \
    int launch_coltile_##ID(const ColArgs* a, cudaStream_t st)                           \
    {                                                                                    \
        return launch_coltile_t<CSpec<MT, MB, L, NT, __VA_ARGS__>>(a, st);                       \
    }
#define GFFT_PICK(ID, MT, MB, L, NT, ...) GFFT_PICK_##ID(ID, MT, MB, L, NT, __VA_ARGS__)
#define GFFT_PICK_3(ID, MT, MB, L, NT, ...) GFFT_INST(ID, MT, MB, L, NT, __VA_ARGS__)
#define GFFT_PICK_0(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_1(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_2(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_4(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_5(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_6(ID, MT, MB, L, NT, ...)
#define GFFT_PICK_7(ID, MT, MB, L, NT, ...)
GFFT_CODELETS(GFFT_PICK)
}  // namespace gfft
