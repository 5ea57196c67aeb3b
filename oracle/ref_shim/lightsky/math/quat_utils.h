#include "_shim_quat.h"
