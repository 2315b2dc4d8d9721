// Batched ensemble (placeholder until the persistent kernel lands).
#include "mol_plan.h"

struct mol_batch { std::string err; };

extern "C" {
int mol_batch_create(const mol_problem_desc* const*, int32_t, mol_batch** out) { if (out) *out = nullptr; return MOL_ERR_UNSUPPORTED; }
int mol_batch_destroy(mol_batch* b) { delete b; return MOL_OK; }
const char* mol_batch_last_error(const mol_batch* b) { return b ? b->err.c_str() : "null batch"; }
int mol_batch_set_stream(mol_batch*, void*) { return MOL_ERR_UNSUPPORTED; }
int mol_batch_offsets(const mol_batch*, int64_t*) { return MOL_ERR_UNSUPPORTED; }
int mol_batch_step_ssprk33(mol_batch*, double*, const double*, double, int64_t) { return MOL_ERR_UNSUPPORTED; }
int mol_batch_step_ssprk33_f32state(mol_batch*, float*, const double*, double, int64_t) { return MOL_ERR_UNSUPPORTED; }
int mol_batch_tune(mol_batch*, int32_t, int32_t, int64_t) { return MOL_ERR_UNSUPPORTED; }
}
