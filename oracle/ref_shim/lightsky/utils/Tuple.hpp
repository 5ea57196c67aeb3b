#include "_shim_utils.h"
