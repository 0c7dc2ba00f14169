// validate_a4.cu -- kernel instantiations and launchers for 4 arm(s).
#include "launch_impl.cuh"

MRPOP_DEFINE_ARM_LAUNCHERS(4)
