// Forward-kernel instantiations for 3 volume(s).
#include "drr_launch.cuh"
DRR_INSTANTIATE_FORWARD(3)
