// validate_a5.cu -- kernel instantiations and launchers for 5 arm(s).
#include "launch_impl.cuh"

MRPOP_DEFINE_ARM_LAUNCHERS(5)
