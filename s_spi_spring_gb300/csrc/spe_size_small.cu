// Instantiates the fused pass kernels for pattern side(s): 16 32 64 128.
#include "spe_sizes.cuh"

SPE_DEFINE_SIZE(16)
SPE_DEFINE_SIZE(32)
SPE_DEFINE_SIZE(64)
SPE_DEFINE_SIZE(128)
