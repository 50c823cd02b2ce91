// Instantiates the fused pass kernels for pattern side(s): 1024.
#include "spe_sizes.cuh"
SPE_DEFINE_SIZE(1024)
