// Forward-kernel instantiations for 2 volume(s).
#include "drr_launch.cuh"
DRR_INSTANTIATE_FORWARD(2)
