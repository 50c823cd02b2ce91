// Instantiates the fused pass kernels for pattern side(s): 2048.
#include "spe_sizes.cuh"
SPE_DEFINE_SIZE(2048)
