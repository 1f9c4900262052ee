#ifndef LCG_STUB_VRNA_alifold
#define LCG_STUB_VRNA_alifold
#include "data_structures.h"
#endif
