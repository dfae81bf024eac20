// TEST INFRASTRUCTURE: the launch variables live in cuda_runtime.h of this directory.
#include "cuda_runtime.h"
