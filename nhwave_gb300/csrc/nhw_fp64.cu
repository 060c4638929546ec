// nhw_fp64.cu -- plain FP64 form: every kernel instantiated for double.
// Built with --fmad=false so that products and sums round exactly as the
// reference's double build does (no fused multiply-add).
#include "ensemble.cuh"

namespace nhw {
SolverBase* make_solver_fp64(const nhw_params& p, int* status) { return make_solver_t<double>(p, status); }
int device_bytes_fp64(const nhw_params& p, size_t* bytes) { return device_bytes_t<double>(p, bytes); }
EnsembleBase* make_ensemble_fp64(SolverBase* const* members, int n, const nhw_ensemble_opts* o, int* status) {
  return make_ensemble_t<double>(members, n, o, status);
}
}  // namespace nhw
