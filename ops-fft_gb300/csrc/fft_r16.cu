// Instantiates the row and column Stockham kernels for radices up to 16
// (one translation unit per instantiation so the build runs in parallel).
#include "launch_common.cuh"

namespace gfft {
int launch_row_r16(const RowArgs* a, cudaStream_t st) { return launch_row_t<16>(a, st); }
int launch_col_r16(const ColArgs* a, cudaStream_t st) { return launch_col_t<16>(a, st); }
}  // namespace gfft
