#ifndef LCG_STUB_VRNA_ENERGY_CONST_H
#define LCG_STUB_VRNA_ENERGY_CONST_H
/* minimal hairpin size used by the reference's base-pair filters */
#define TURN 3
#endif
