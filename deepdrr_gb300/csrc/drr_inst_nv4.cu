// Forward-kernel instantiations for 4 volume(s).
#include "drr_launch.cuh"
DRR_INSTANTIATE_FORWARD(4)
