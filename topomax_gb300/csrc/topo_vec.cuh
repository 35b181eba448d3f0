// Element-wise vector kernels and deterministic grid reductions.
#pragma once

#include <cuda_runtime.h>
#include <type_traits>
#include "topo_common.cuh"

namespace topo {

constexpr int kVecThreads = 256;

inline int vec_grid(size_t n, int sms) {
  size_t b = (n + kVecThreads - 1) / kVecThreads;
  size_t cap = size_t(sms) * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return int(b);
}

#define TOPO_GRID_STRIDE(i, n) \
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)

template <class T>
__global__ void k_fill(T* x, T v, size_t n) { TOPO_PDL_ENTRY(); TOPO_GRID_STRIDE(i, n) x[i] = v; }

template <class TD, class TS>
__global__ void k_convert(TD* __restrict__ d, const TS* __restrict__ s, double scale, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) d[i] = TD(double(s[i]) * scale);
}

// y += a x
template <class T>
__global__ void k_axpy(T* __restrict__ y, T a, const T* __restrict__ x, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) y[i] += a * x[i];
}

// r = b - y
template <class T>
__global__ void k_sub(T* __restrict__ r, const T* __restrict__ b, const T* __restrict__ y, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) r[i] = b[i] - y[i];
}

template <class T>
__global__ void k_mul(T* __restrict__ y, const T* __restrict__ a, const T* __restrict__ x, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) y[i] = a[i] * x[i];
}

template <class T>
__global__ void k_scale(T* __restrict__ x, T a, size_t n) { TOPO_PDL_ENTRY(); TOPO_GRID_STRIDE(i, n) x[i] *= a; }

template <class T>
__global__ void k_inverse(T* __restrict__ y, const T* __restrict__ x, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) y[i] = T(1) / x[i];
}

// x /= sqrt(*nrm2) (nrm2 = x.x on the device; left unchanged when not positive)
template <class T>
__global__ void k_scale_unit(T* __restrict__ x, const double* __restrict__ nrm2, size_t n) { TOPO_PDL_ENTRY();
  __shared__ T a_s;
  if (threadIdx.x == 0) {
    const double q = *nrm2;
    a_s = (q > 0.0 && isfinite(q)) ? T(1.0 / sqrt(q)) : T(1);
  }
  __syncthreads();
  const T a = a_s;
  TOPO_GRID_STRIDE(i, n) x[i] *= a;
}

// ---------------------------------------------------------------------------
// reductions: per-block partial sums, the last block to finish adds the
// partials in block order (deterministic) and stores the result.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R warp_sum(R v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <class R>
__device__ __forceinline__ R block_sum(R v, R* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  if (lane == 0) sh[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : R(0);
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;  // valid in thread 0
}

// Finishes a reduction of NV values per block (1D or 2D grids).  Returns true
// in thread 0 of the last block, with the totals in tot[].  The in-block tree
// runs in R (float for FP32 data: FP64 arithmetic is scarce on this GPU), the
// per-block partials and their final combination in FP64.
template <int NV, class R>
__device__ bool finish_reduction(const R (&v)[NV], double* partials, unsigned* counter, double (&tot)[NV]) {
  __shared__ R shr[32];
  __shared__ double sh[32];
  __shared__ bool last;
  const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x, nb = gridDim.x * gridDim.y;
  for (int k = 0; k < NV; ++k) {
    const R s = block_sum(v[k], shr);
    if (threadIdx.x == 0) partials[size_t(bid) * NV + k] = double(s);
  }
  __threadfence();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == nb - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (unsigned b = threadIdx.x; b < nb; b += blockDim.x)
      s += ((volatile double*)partials)[size_t(b) * NV + k];
    // fixed-order combine: strided per-thread sums then a tree
    s = block_sum(s, sh);
    if (threadIdx.x == 0) tot[k] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
  return threadIdx.x == 0;
}

// out[0] = sum a_i b_i (or sum a_i^2 when b == nullptr)
template <class TA, class TB>
__global__ void k_dot(const TA* __restrict__ a, const TB* __restrict__ b, size_t n, double* partials,
                      unsigned* counter, double* out) { TOPO_PDL_ENTRY();
  // per-thread partial in the input precision (a handful of terms), then FP64
  using Acc = typename std::conditional<sizeof(TA) == 4 && sizeof(TB) == 4, float, double>::type;
  Acc acc = Acc(0);
  TOPO_GRID_STRIDE(i, n) acc += b ? Acc(a[i]) * Acc(b[i]) : Acc(a[i]) * Acc(a[i]);
  const Acc v[1] = {acc};
  double tot[1];
  if (finish_reduction<1>(v, partials, counter, tot)) out[0] = tot[0];
}

// two dots at once: out[0] = a.b, out[1] = c.d
template <class T>
__global__ void k_dot2(const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                       const T* __restrict__ d, size_t n, double* partials, unsigned* counter,
                       double* out) { TOPO_PDL_ENTRY();
  // per-thread partials in the input precision (a handful of terms), then FP64
  T p0 = T(0), p1 = T(0);
  TOPO_GRID_STRIDE(i, n) {
    p0 += a[i] * b[i];
    p1 += c[i] * d[i];
  }
  const T v[2] = {p0, p1};
  double tot[2];
  if (finish_reduction<2>(v, partials, counter, tot)) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// Multi-vector kernels with a compile-time vector count C (host code
// dispatches on the run-time count): out[k] = V_k . w and out[C] = w . w
constexpr int kMaxMulti = 16;
struct MultiCoef {
  double c[kMaxMulti];
};

template <class TV, class TW, int C>
__global__ void k_multidot(const TV* __restrict__ V, size_t stride, const TW* __restrict__ w, size_t n,
                           double* partials, unsigned* counter, double* out) { TOPO_PDL_ENTRY();
  double v[C + 1];
#pragma unroll
  for (int k = 0; k <= C; ++k) v[k] = 0.0;
  TOPO_GRID_STRIDE(i, n) {
    const double wi = double(w[i]);
#pragma unroll
    for (int k = 0; k < C; ++k) v[k] += double(V[size_t(k) * stride + i]) * wi;
    v[C] += wi * wi;
  }
  double tot[C + 1];
  if (finish_reduction<C + 1>(v, partials, counter, tot))
    for (int k = 0; k <= C; ++k) out[k] = tot[k];
}

// w -= sum_k c_k V_k
template <class TV, class TW, int C>
__global__ void k_sub_multi(TW* __restrict__ w, const TV* __restrict__ V, size_t stride, MultiCoef c, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) {
    double s = double(w[i]);
#pragma unroll
    for (int k = 0; k < C; ++k) s -= c.c[k] * double(V[size_t(k) * stride + i]);
    w[i] = TW(s);
  }
}

// x += sum_k c_k Z_k
template <class TZ, class TX, int C>
__global__ void k_add_multi(TX* __restrict__ x, const TZ* __restrict__ Z, size_t stride, MultiCoef c, size_t n) { TOPO_PDL_ENTRY();
  TOPO_GRID_STRIDE(i, n) {
    double s = double(x[i]);
#pragma unroll
    for (int k = 0; k < C; ++k) s += c.c[k] * double(Z[size_t(k) * stride + i]);
    x[i] = TX(s);
  }
}

// run-time count -> compile-time instance (1..9)
#define TOPO_DISPATCH_COUNT(count, F) \
  switch (count) {                    \
    case 1: F(1); break;              \
    case 2: F(2); break;              \
    case 3: F(3); break;              \
    case 4: F(4); break;              \
    case 5: F(5); break;              \
    case 6: F(6); break;              \
    case 7: F(7); break;              \
    case 8: F(8); break;              \
    default: F(9); break;             \
  }

}  // namespace topo
