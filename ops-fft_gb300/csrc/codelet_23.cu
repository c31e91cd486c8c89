// Instantiates codelet 23 of codelet_list.h.
#include "codelet_inst.cuh"

GFFT_CODELET_TU(23)
