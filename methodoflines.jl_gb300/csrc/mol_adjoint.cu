// Discrete adjoint (placeholder until the VJP kernels land).
#include "mol_plan.h"

extern "C" {
int mol_rhs_vjp(mol_plan* plan, const double*, const double*, const double*, double, double*, double*, double*) {
    return mol::set_err(plan, MOL_ERR_UNSUPPORTED, "vjp not built yet");
}
int mol_adjoint_ssprk33(mol_plan* plan, const double*, const double*, double, double, int64_t, int32_t, int32_t,
                        const double*, double*, double*, double*, double*, double*, int64_t*) {
    return mol::set_err(plan, MOL_ERR_UNSUPPORTED, "adjoint not built yet");
}
}
