// Instantiates the row and column Stockham kernels for radices up to 47
// (one translation unit per instantiation so the build runs in parallel).
#include "launch_common.cuh"

namespace gfft {
int launch_row_r47(const RowArgs* a, cudaStream_t st) { return launch_row_t<47>(a, st); }
int launch_col_r47(const ColArgs* a, cudaStream_t st) { return launch_col_t<47>(a, st); }
}  // namespace gfft
