#ifndef LCG_STUB_VRNA_part_func
#define LCG_STUB_VRNA_part_func
#include "data_structures.h"
#endif
