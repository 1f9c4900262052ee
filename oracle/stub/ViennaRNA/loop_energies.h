#ifndef LCG_STUB_VRNA_loop_energies
#define LCG_STUB_VRNA_loop_energies
#include "data_structures.h"
#endif
