/* Project-written minimal declarations so that the reference's own sources
 * compile without ViennaRNA. Folding is never called on the alignment path
 * (inputs are PP files with base-pair probabilities); every folding entry
 * point is an abort-on-call stub in ../ref_link_stubs.cc. */
#ifndef LCG_STUB_VRNA_DATA_STRUCTURES_H
#define LCG_STUB_VRNA_DATA_STRUCTURES_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct lcg_stub_md {
    int noLP;
    int max_bp_span;
    int dangles;
    int compute_bpp;
    int ribo;
    double cv_fact;
    double nc_fact;
    double temperature;
    double betaScale;
    int uniq_ML;
} vrna_md_t;
typedef struct vrna_md_t_dummy vrna_md_s;
typedef struct lcg_stub_plist { int i; int j; float p; int type; } vrna_plist_t;
typedef struct lcg_stub_fc vrna_fold_compound_t;
typedef struct lcg_stub_exp_param vrna_exp_param_t;
typedef struct lcg_stub_param vrna_param_t;
void vrna_md_set_default(vrna_md_t *md);
void vrna_md_copy(vrna_md_t *dst, const vrna_md_t *src);
#ifdef __cplusplus
}
#endif
#endif
