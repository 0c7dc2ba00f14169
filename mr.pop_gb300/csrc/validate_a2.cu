// validate_a2.cu -- kernel instantiations and launchers for 2 arm(s).
#include "launch_impl.cuh"

MRPOP_DEFINE_ARM_LAUNCHERS(2)
