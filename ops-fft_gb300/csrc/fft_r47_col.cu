// Instantiates the column Stockham kernel for radices up to 47.
#include "launch_common.cuh"

namespace gfft {
int launch_col_r47(const ColArgs* a, cudaStream_t st) { return launch_col_t<47>(a, st); }
}  // namespace gfft
