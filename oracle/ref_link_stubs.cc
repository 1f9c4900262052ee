// Test infrastructure only (oracle). Project-written link stubs so that the
// reference's own LocARNA sources link without ViennaRNA. Every folding entry
// point aborts: the alignment path reads base-pair probabilities from PP files
// and never folds (reference: src/LocARNA/rna_data.cc:45-69 only folds when the
// input carries no base-pair probabilities).
#include <cstdio>
#include <cstdlib>
#include <string>
#include "LocARNA/rna_ensemble.hh"
#include "LocARNA/multiple_alignment.hh"
#include "LocARNA/pfold_params.hh"

extern "C" {
void vrna_md_set_default(vrna_md_t *md) {
    md->noLP = 0; md->max_bp_span = -1; md->dangles = 2; md->compute_bpp = 1;
    md->ribo = 0; md->cv_fact = 1.0; md->nc_fact = 1.0; md->temperature = 37.0;
    md->betaScale = 1.0; md->uniq_ML = 0;
}
void vrna_md_copy(vrna_md_t *dst, const vrna_md_t *src) { *dst = *src; }
float MEA(vrna_plist_t *, char *, double) {
    std::fprintf(stderr, "oracle: MEA folding is unavailable (no ViennaRNA)\n");
    std::abort();
}
}

[[noreturn]] static void lcg_no_folding(const char *what) {
    std::fprintf(stderr, "oracle: folding unavailable (%s); give PP input\n", what);
    std::abort();
}

namespace LocARNA {
class RnaEnsembleImpl {};
RnaEnsemble::RnaEnsemble(const MultipleAlignment &, const PFoldParams &, bool, bool) { lcg_no_folding("RnaEnsemble"); }
RnaEnsemble::~RnaEnsemble() {}
bool RnaEnsemble::has_base_pair_probs() const { lcg_no_folding("has_base_pair_probs"); }
bool RnaEnsemble::has_stacking_probs() const { lcg_no_folding("has_stacking_probs"); }
bool RnaEnsemble::has_in_loop_probs() const { lcg_no_folding("has_in_loop_probs"); }
const MultipleAlignment &RnaEnsemble::multiple_alignment() const { lcg_no_folding("multiple_alignment"); }
double RnaEnsemble::arc_prob(size_type, size_type) const { lcg_no_folding("arc_prob"); }
double RnaEnsemble::arc_2_prob(size_type, size_type) const { lcg_no_folding("arc_2_prob"); }
double RnaEnsemble::arc_in_loop_prob(size_type, size_type, size_type, size_type) const { lcg_no_folding("arc_in_loop_prob"); }
double RnaEnsemble::arc_external_prob(size_type, size_type) const { lcg_no_folding("arc_external_prob"); }
double RnaEnsemble::unpaired_in_loop_prob(size_type, size_type, size_type) const { lcg_no_folding("unpaired_in_loop_prob"); }
double RnaEnsemble::unpaired_external_prob(size_type) const { lcg_no_folding("unpaired_external_prob"); }
std::string RnaEnsemble::min_free_energy_structure() const { lcg_no_folding("min_free_energy_structure"); }
double RnaEnsemble::min_free_energy() const { lcg_no_folding("min_free_energy"); }
}
