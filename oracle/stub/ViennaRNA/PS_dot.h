#ifndef LCG_STUB_VRNA_PS_dot
#define LCG_STUB_VRNA_PS_dot
#include "data_structures.h"
#endif
