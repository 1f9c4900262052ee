#ifndef LCG_STUB_VRNA_utils
#define LCG_STUB_VRNA_utils
#include "data_structures.h"
#endif
