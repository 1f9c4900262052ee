#ifndef LCG_STUB_VRNA_params
#define LCG_STUB_VRNA_params
#include "data_structures.h"
#endif
