// FP64 instantiation of the multigrid-preconditioned CG (plain-FP64 path) and
// the operators of the refinement residuals (FP64, and pair-of-FP32).
#include "topo_mg_impl.cuh"

namespace topo {
template class MG<double>;

void p2_apply_f64(const P2Params<double>& p, const double* xi, const double* x, double* y, cudaStream_t s) {
  launch_p2_apply<double>(p, xi, x, y, s);
}

void p2_apply_dd(const P2Params<dd>& p, const double* x, double* y, cudaStream_t s) {
  launch_p2_apply_dd(p, x, y, s);
}

void p2_dd_prime() { (void)p2_march_bps<dd, kP2Apply>(); }
}  // namespace topo
