// Instantiates codelet 21 of codelet_list.h.
#include "codelet_inst.cuh"

GFFT_CODELET_TU(21)
