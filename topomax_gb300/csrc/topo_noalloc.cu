// Sensitivity right-hand side for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: hosts that hand out device memory only
// through their own fixed pool, callers that run inside a fixed memory budget,
// and loops that must not pay an allocation's device-wide synchronisation
// (cudaMalloc and cudaFree can wait for all work on the device).  For them
// this entry point needs no context and allocates nothing: the per-triangle
// scratch lives in a fixed, file-scope device array that every GPU loading
// this library holds until the process exits.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>

#include "topomax_gb300.h"
#include "topo_sens.cuh"

namespace {

// 3 FP32 moments per triangle, at most TOPO_NOALLOC_MAX_TRIANGLES triangles
// (12 MiB).  Every call overwrites the entries it reads, so nothing needs to
// start at zero; the contents after a call are that call's moments.
__device__ __align__(256) float g_sens_scratch[3 * size_t(TOPO_NOALLOC_MAX_TRIANGLES)];

constexpr int kMaxDevices = 64;
// device address of g_sens_scratch per device (host code may not use the
// symbol itself: it names a host-side stand-in, not device memory)
std::atomic<float*> g_scratch_addr[kMaxDevices];

}  // namespace

extern "C" int topo_sensitivity_rhs_noalloc(const topo_grid_desc* grid, double young_modulus, double poisson_ratio,
                                            double penalization, double penal_min, const double* u,
                                            const double* xi, double* b, topo_stream_t stream) {
  using namespace topo;
  if (!grid || grid->nx < 1 || grid->ny < 1 || !(grid->width > 0) || !(grid->height > 0) || !u || !xi || !b)
    return TOPO_ERR_ARG;
  if (!(young_modulus > 0) || !(poisson_ratio < 0.5) || !std::isfinite(penalization) || !(penal_min > 0))
    return TOPO_ERR_ARG;
  const long long ntri = 2LL * grid->nx * grid->ny;
  if (ntri > TOPO_NOALLOC_MAX_TRIANGLES) return TOPO_ERR_ARG;  // scratch holds at most this many triangles
  // an error already pending on this thread belongs to an earlier call: leave it in
  // place for its owner and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return TOPO_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TOPO_ERR_CUDA;
  float* scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    // once per device, with that device current (the first call on a device
    // does this look-up: make it before any stream capture on that device).
    // The address is kept for the life of the process: after a cudaDeviceReset
    // the array may be reloaded elsewhere, so the entry point must not be used
    // across a reset.
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_sens_scratch) != cudaSuccess || !p) return TOPO_ERR_CUDA;
    scratch = static_cast<float*>(p);
    g_scratch_addr[dev].store(scratch, std::memory_order_release);
  }
  const int nx = grid->nx, ny = grid->ny;
  const double hx = grid->width / nx, hy = grid->height / ny;
  const double mu = young_modulus / (2 * (1 + poisson_ratio));
  const double lmbda = mu * poisson_ratio / (0.5 - poisson_ratio);
  const double area = 0.5 * hx * hy;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int sms = 148;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t nv = size_t(nx + 1) * (ny + 1);
  k_sens_tri<float><<<vec_grid(size_t(ntri), sms), kVecThreads, 0, s>>>(
      nx, ny, 1.0 / hx, 1.0 / hy, float(lmbda), float(mu), float(area), make_penal<float>(penalization, penal_min),
      u, xi, scratch);
  k_vertex_gather3<float><<<vec_grid(nv, sms), kVecThreads, 0, s>>>(nx, ny, scratch, b);
  // launch errors of this call only (nothing was pending before the launches)
  return cudaGetLastError() == cudaSuccess ? TOPO_OK : TOPO_ERR_CUDA;
}
