// Instantiates the row Stockham kernel for radices up to 47 (row and column
// instantiations sit in separate translation units so the build runs in
// parallel).
#include "launch_common.cuh"

namespace gfft {
int launch_row_r47(const RowArgs* a, cudaStream_t st) { return launch_row_t<47>(a, st); }
}  // namespace gfft
