// FP64 instantiation of the multigrid-preconditioned CG (plain-FP64 path) and
// the FP64 operator used for refinement residuals.
#include "topo_mg_impl.cuh"

namespace topo {
template class MG<double>;

void p2_apply_f64(const P2Params<double>& p, const double* xi, const double* x, double* y, cudaStream_t s) {
  launch_p2_apply<double>(p, xi, x, y, s);
}
}  // namespace topo
