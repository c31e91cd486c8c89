// Instantiates codelet 26 of codelet_list.h.
#include "codelet_inst.cuh"

GFFT_CODELET_TU(26)
