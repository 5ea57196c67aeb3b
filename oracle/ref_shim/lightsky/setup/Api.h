#include "_shim_setup.h"
