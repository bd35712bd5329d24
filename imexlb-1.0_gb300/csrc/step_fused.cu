// Reference-rounding FP64 step kernel with the boundary copies folded in
// (boundary_fused.cuh): the default variant for rho0 == 1, variant 0 for
// other rho0, both lattices (compiled apart so that the build runs it in
// parallel with the other step-kernel files).
#include "exact_node.cuh"

namespace imx {

cudaError_t launch_step_fused(int dim, bool rho_one, unsigned grid, const DevGrid& g,
                              const DevCoef& c, const DevState& st, const double* fin,
                              double* fout, unsigned long long* monitor, cudaStream_t s) {
  const bool mon = monitor != nullptr;
#define L_(D, R, M, EM) k_step<D, R, M, EM, true><<<grid, kBlock, 0, s>>>(g, c, st, fin, fout, monitor)
  if (rho_one) {
    constexpr uint32_t E2 = Splits<2>::v[Splits<2>::kDefault], E3 = Splits<3>::v[Splits<3>::kDefault];
    if (dim == 2) { if (mon) L_(2, true, true, E2); else L_(2, true, false, E2); }
    else { if (mon) L_(3, true, true, E3); else L_(3, true, false, E3); }
  } else {
    if (dim == 2) { if (mon) L_(2, false, true, 0u); else L_(2, false, false, 0u); }
    else { if (mon) L_(3, false, true, 0u); else L_(3, false, false, 0u); }
  }
#undef L_
  return cudaGetLastError();
}

}  // namespace imx
