// Instantiates codelet 10 of codelet_list.h.
#include "codelet_inst.cuh"

GFFT_CODELET_TU(10)
