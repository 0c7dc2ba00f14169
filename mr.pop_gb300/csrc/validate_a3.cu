// validate_a3.cu -- kernel instantiations and launchers for 3 arm(s).
#include "launch_impl.cuh"

MRPOP_DEFINE_ARM_LAUNCHERS(3)
