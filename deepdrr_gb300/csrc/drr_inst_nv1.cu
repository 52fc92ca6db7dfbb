// Forward-kernel instantiations for 1 volume(s).
#include "drr_launch.cuh"
DRR_INSTANTIATE_FORWARD(1)
