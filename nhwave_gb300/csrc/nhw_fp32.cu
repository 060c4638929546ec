// nhw_fp32.cu -- FP32+IR form: 3-D state, fluxes and inner Krylov iterations in
// float; depth/eta/mask (2-D) fields, the Poisson operator for the residual and
// the refinement correction in double.
#include "ensemble.cuh"

namespace nhw {
SolverBase* make_solver_fp32(const nhw_params& p, int* status) { return make_solver_t<float>(p, status); }
int device_bytes_fp32(const nhw_params& p, size_t* bytes) { return device_bytes_t<float>(p, bytes); }
EnsembleBase* make_ensemble_fp32(SolverBase* const* members, int n, const nhw_ensemble_opts* o, int* status) {
  return make_ensemble_t<float>(members, n, o, status);
}
}  // namespace nhw
