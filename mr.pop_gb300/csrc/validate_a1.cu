// validate_a1.cu -- kernel instantiations and launchers for 1 arm(s).
#include "launch_impl.cuh"

MRPOP_DEFINE_ARM_LAUNCHERS(1)
