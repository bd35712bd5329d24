// Reference-rounding FP64 step kernel, D2Q9: the variants that run part of
// their FP64 additions and multiplications as integer emulation (compiled
// apart from kernels.cu so that the build runs them in parallel).
#include "exact_node.cuh"

namespace imx {

cudaError_t launch_step_split2(int split, unsigned grid, const DevGrid& g, const DevCoef& c,
                               const DevState& st, const double* fin, double* fout,
                               unsigned long long* monitor, cudaStream_t s) {
  return monitor ? launch_step_variant<2, true>(split, grid, g, c, st, fin, fout, monitor, s)
                 : launch_step_variant<2, false>(split, grid, g, c, st, fin, fout, monitor, s);
}

}  // namespace imx
