#include "_shim_math.h"
#include "_shim_quat.h"
