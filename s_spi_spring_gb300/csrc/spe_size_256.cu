// Instantiates the fused pass kernels for pattern side(s): 256.
#include "spe_sizes.cuh"
SPE_DEFINE_SIZE(256)
