// gpp_batched.cu -- persistent work-queue kernel for many states (in progress).
#include "gpp_kernels.h"
