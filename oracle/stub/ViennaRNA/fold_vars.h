#ifndef LCG_STUB_VRNA_fold_vars
#define LCG_STUB_VRNA_fold_vars
#include "data_structures.h"
#endif
