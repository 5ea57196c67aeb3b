#include "_shim_math.h"
