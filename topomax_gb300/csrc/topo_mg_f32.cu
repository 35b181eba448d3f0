// FP32 instantiation of the multigrid-preconditioned CG (inner solves of the
// mixed-precision path).
#include "topo_mg_impl.cuh"

namespace topo {
template class MG<float>;

void p2_apply_f32(const P2Params<float>& p, const float* xi, const float* x, float* y, cudaStream_t s) {
  launch_p2_apply<float>(p, xi, x, y, s);
}
}  // namespace topo
