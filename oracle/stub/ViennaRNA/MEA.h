#ifndef LCG_STUB_VRNA_MEA_H
#define LCG_STUB_VRNA_MEA_H
#include "data_structures.h"
#ifdef __cplusplus
extern "C" {
#endif
float MEA(vrna_plist_t *p, char *structure, double gamma);
#ifdef __cplusplus
}
#endif
#endif
