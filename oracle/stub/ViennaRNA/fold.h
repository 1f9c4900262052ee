#ifndef LCG_STUB_VRNA_fold
#define LCG_STUB_VRNA_fold
#include "data_structures.h"
#endif
