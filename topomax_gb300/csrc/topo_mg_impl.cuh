// Kernels and host orchestration of the multigrid-preconditioned CG.
// Included by topo_mg_f32.cu / topo_mg_f64.cu, which instantiate MG<T>.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstring>

#include "topo_mg.h"
#include "topo_p1.cuh"
#include "topo_p2.cuh"
#include "topo_vec.cuh"

namespace topo {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(P2_THREADS)
    k_p2_apply(P2Params<T> P, const T* __restrict__ xi, const T* __restrict__ u, T* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& s = *reinterpret_cast<P2Smem<T>*>(smem_raw);
  P2Kern<T>::load(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, u, xi, s);
  __syncthreads();
  P2Kern<T>::compute(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, 0);
  __syncthreads();
  P2Kern<T>::gather(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, u, y, 0);
}

template <class T>
__global__ void __launch_bounds__(P2_THREADS)
    k_p2_diag(P2Params<T> P, const T* __restrict__ xi, T* __restrict__ d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& s = *reinterpret_cast<P2Smem<T>*>(smem_raw);
  P2Kern<T>::load(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, nullptr, xi, s);
  __syncthreads();
  P2Kern<T>::compute(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, 1);
  __syncthreads();
  P2Kern<T>::gather(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, nullptr, d, 1);
}

template <class T, int NC>
__global__ void k_p1_apply(P1Params<T, NC> P, const T* __restrict__ u, T* __restrict__ y) {
  const int NX = P.nx + 1, NY = P.ny + 1;
  const size_t nn = size_t(NX) * NY;
  TOPO_GRID_STRIDE(n, nn) P1Kern<T, NC>::node_apply(int(n % NX), int(n / NX), P, u, y);
}

template <class T, int NC>
__global__ void k_p1_diag(P1Params<T, NC> P, T* __restrict__ d) {
  const int NX = P.nx + 1, NY = P.ny + 1;
  const size_t nn = size_t(NX) * NY;
  TOPO_GRID_STRIDE(n, nn) P1Kern<T, NC>::node_diag(int(n % NX), int(n / NX), P, d);
}

template <class T, int NC>
__global__ void k_restrict(Transfer X, const T* __restrict__ rf, T* __restrict__ bc) {
  const size_t nn = size_t(X.NXc) * X.NYc;
  TOPO_GRID_STRIDE(n, nn) TransferKern<T, NC>::node_restrict(int(n % X.NXc), int(n / X.NXc), X, rf, bc);
}

template <class T, int NC>
__global__ void k_prolong_add(Transfer X, const T* __restrict__ xc, T* __restrict__ xf) {
  const size_t nn = size_t(X.NXf) * X.NYf;
  TOPO_GRID_STRIDE(n, nn) TransferKern<T, NC>::node_prolong_add(int(n % X.NXf), int(n / X.NXf), X, xc, xf);
}

// deterministic pseudo-random start vector for the power iteration
template <class T>
__global__ void k_power_start(T* x, size_t n) {
  TOPO_GRID_STRIDE(i, n) {
    unsigned h = unsigned(i) * 2654435761u + 0x9e3779b9u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    x[i] = T(0.5) + T(h & 0xffffu) / T(65536.0);
  }
}

// Dense inverse of the coarsest operator (n <= kCoarseMaxDofs), assembled from
// the FP64 coefficient masters, Gauss-Jordan in shared memory (SPD, no pivoting).
template <class T, int NC>
__global__ void k_coarse_inverse(int nx, int ny, Dir dir, ElemRefs R, const double* __restrict__ kK,
                                 const double* __restrict__ kM, T* __restrict__ inv, int* status) {
  __shared__ double A[kCoarseMaxDofs * kCoarseMaxDofs];
  __shared__ double f[kCoarseMaxDofs];
  __shared__ int bad;
  const int NX = nx + 1, NY = ny + 1, n = NX * NY * NC;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) A[i] = 0.0;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int cj = 0; cj < ny; ++cj)
      for (int ci = 0; ci < nx; ++ci)
        for (int o = 0; o < 2; ++o) {
          const size_t t = (size_t(cj) * nx + ci) * 2 + o;
          const double kk = kK[t];
          const double km = (NC == 1 && kM) ? kM[t] : 0.0;
          for (int k = 0; k < 3; ++k) {
            const int nk = (cj + p1_off_b(o, k)) * NX + ci + p1_off_a(o, k);
            for (int l = 0; l < 3; ++l) {
              const int nl = (cj + p1_off_b(o, l)) * NX + ci + p1_off_a(o, l);
              for (int c = 0; c < NC; ++c)
                for (int d = 0; d < NC; ++d) {
                  double v;
                  if (NC == 2) v = kk * R.K2[o][k * 2 + c][l * 2 + d];
                  else v = kk * R.K1[o][k][l] + km * R.M1[o][k][l];
                  A[(NC * nk + c) * n + NC * nl + d] += v;
                }
            }
          }
        }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i / n, c = i % n;
    const int nr = r / NC, nc = c / NC;
    const bool cr = is_clamped(dir, nr % NX, nr / NX), cc = is_clamped(dir, nc % NX, nc / NX);
    if (cr || cc) A[i] = (r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double p = A[k * n + k];
    if (!(p > 0.0) || !isfinite(p)) {
      if (threadIdx.x == 0) bad = 1;
      break;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) f[i] = A[i * n + k];
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += blockDim.x) A[k * n + j] = (j == k) ? 1.0 / p : A[k * n + j] / p;
    __syncthreads();
    for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
      const int i = idx / n, j = idx % n;
      if (i == k) continue;
      if (j == k) A[idx] = -f[i] / p;
      else A[idx] -= f[i] * A[k * n + j];
    }
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i / n, c = i % n;
    inv[i] = T(0.5 * (A[r * n + c] + A[c * n + r]));
  }
  if (threadIdx.x == 0) *status = bad;
}

template <class T>
__global__ void k_dense_matvec(const T* __restrict__ Ainv, const T* __restrict__ b, T* __restrict__ x, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T s = T(0);
    for (int j = 0; j < n; ++j) s += Ainv[size_t(i) * n + j] * b[j];
    x[i] = s;
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
template <class T>
inline void set_p2_smem_attr() {
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(k_p2_apply<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(P2Smem<T>)));
    cudaFuncSetAttribute(k_p2_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(P2Smem<T>)));
    done = true;
  }
}

template <class T>
inline void launch_p2_apply(const P2Params<T>& P, const T* xi, const T* x, T* y, cudaStream_t s) {
  set_p2_smem_attr<T>();
  dim3 g((P.nx + P2_TX - 1) / P2_TX, (P.ny + P2_TY - 1) / P2_TY);
  k_p2_apply<T><<<g, P2_THREADS, sizeof(P2Smem<T>), s>>>(P, xi, x, y);
}

template <class T, int NC>
inline P1Params<T, NC> make_p1(const LevelSpec& L, const ElemRefs& R, const T* kK, const T* kM) {
  P1Params<T, NC> P;
  std::memset(&P, 0, sizeof(P));
  P.nx = L.nx;
  P.ny = L.ny;
  P.dir = L.dir;
  for (int o = 0; o < 2; ++o) {
    for (int a = 0; a < 3 * NC; ++a)
      for (int b = 0; b < 3 * NC; ++b) P.K[o][a][b] = T(NC == 2 ? R.K2[o][a][b] : R.K1[o][a][b]);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) P.Mm[o][a][b] = T(R.M1[o][a][b]);
  }
  P.kK = kK;
  P.kM = kM;
  P.kK_c = T(0);
  P.kM_c = T(0);
  return P;
}

static inline Transfer make_transfer(const LevelSpec& f, const LevelSpec& c) {
  Transfer X;
  X.NXf = f.NX;
  X.NYf = f.NY;
  X.NXc = c.NX;
  X.NYc = c.NY;
  X.dirf = f.dir;
  X.dirc = c.dir;
  return X;
}

// ---------------------------------------------------------------------------
// MG<T>
// ---------------------------------------------------------------------------
template <class T>
void MG<T>::init(const std::vector<LevelSpec>& specs, const ElemRefs* refs, double lmbda, double mu,
                 Arena& arena, Reducer* red) {
  specs_ = specs;
  refs_ = refs;
  lmbda_ = lmbda;
  mu_ = mu;
  red_ = red;
  sms_ = red->sms;
  lv_.assign(specs.size(), Lev{});
  for (size_t l = 0; l < specs.size(); ++l) {
    const size_t n = specs[l].ndof();
    Lev& v = lv_[l];
    v.x = arena.alloc_n<T>(n);
    v.b = arena.alloc_n<T>(n);
    v.r = arena.alloc_n<T>(n);
    v.d = arena.alloc_n<T>(n);
    v.t = arena.alloc_n<T>(n);
    v.diag = arena.alloc_n<T>(n);
    v.dinv = arena.alloc_n<T>(n);
    if (!specs[l].p2) {
      v.kK = arena.alloc_n<T>(specs[l].ntri());
      if (specs[l].NC == 1) v.kM = arena.alloc_n<T>(specs[l].ntri());
    }
  }
  const size_t n0 = specs[0].ndof();
  for (int k = 0; k < kScratch; ++k) pcg_[k] = arena.alloc_n<T>(n0);
  const int nc = int(specs.back().ndof());
  cinv_ = arena.alloc_n<T>(size_t(nc) * nc);
  cstat_ = arena.alloc_n<int>(1);
}

template <class T>
void MG<T>::apply(int l, const T* x, T* y, cudaStream_t s, bool op) {
  const LevelSpec& L = specs_[l];
  if (L.p2) {
    launch_p2_apply<T>(op ? p2_op_ : p2_, xi_, x, y, s);
    return;
  }
  const int g = vec_grid(L.nn(), sms_);
  if (L.NC == 2) {
    auto P = make_p1<T, 2>(L, refs_[l], lv_[l].kK, nullptr);
    k_p1_apply<T, 2><<<g, kVecThreads, 0, s>>>(P, x, y);
  } else {
    auto P = make_p1<T, 1>(L, refs_[l], lv_[l].kK, lv_[l].kM);
    k_p1_apply<T, 1><<<g, kVecThreads, 0, s>>>(P, x, y);
  }
}

template <class T>
void MG<T>::diag_of(int l, T* d, cudaStream_t s) {
  const LevelSpec& L = specs_[l];
  if (L.p2) {
    set_p2_smem_attr<T>();
    dim3 g((L.nx + P2_TX - 1) / P2_TX, (L.ny + P2_TY - 1) / P2_TY);
    k_p2_diag<T><<<g, P2_THREADS, sizeof(P2Smem<T>), s>>>(p2_, xi_, d);
    return;
  }
  const int g = vec_grid(L.nn(), sms_);
  if (L.NC == 2) {
    auto P = make_p1<T, 2>(L, refs_[l], lv_[l].kK, nullptr);
    k_p1_diag<T, 2><<<g, kVecThreads, 0, s>>>(P, d);
  } else {
    auto P = make_p1<T, 1>(L, refs_[l], lv_[l].kK, lv_[l].kM);
    k_p1_diag<T, 1><<<g, kVecThreads, 0, s>>>(P, d);
  }
}

template <class T>
double MG<T>::dot(const T* a, const T* b, size_t n, cudaStream_t s) {
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(a, b, n, red_->partials, red_->counter, red_->out);
  cudaMemcpyAsync(red_->host, red_->out, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  return red_->host[0];
}

template <class T>
double MG<T>::estimate_lmax(int l, cudaStream_t s) {
  const size_t n = specs_[l].ndof();
  const int g = vec_grid(n, sms_);
  Lev& v = lv_[l];
  k_power_start<T><<<g, kVecThreads, 0, s>>>(v.x, n);
  for (int it = 0; it < power_iters; ++it) {
    apply(l, v.x, v.t, s);
    k_mul<T><<<g, kVecThreads, 0, s>>>(v.x, v.dinv, v.t, n);
    if (it % 4 == 3) {  // rescale to stay in range
      const double nrm = std::sqrt(dot(v.x, v.x, n, s));
      if (!(nrm > 0) || !std::isfinite(nrm)) return 4.0;
      k_scale<T><<<g, kVecThreads, 0, s>>>(v.x, T(1.0 / nrm), n);
    }
  }
  apply(l, v.x, v.t, s);
  const double num = dot(v.x, v.t, n, s);
  k_mul<T><<<g, kVecThreads, 0, s>>>(v.r, v.diag, v.x, n);
  const double den = dot(v.x, v.r, n, s);
  double lam = (den > 0) ? num / den : 4.0;
  if (!std::isfinite(lam) || lam <= 0) lam = 4.0;
  return lam;
}

template <class T>
int MG<T>::setup(cudaStream_t s) {
  const int L = levels();
  for (int l = 0; l < L; ++l) {
    const LevelSpec& S = specs_[l];
    Lev& v = lv_[l];
    if (!S.p2) {
      const int g = vec_grid(S.ntri(), sms_);
      k_convert<T, double><<<g, kVecThreads, 0, s>>>(v.kK, kK64_[l], 1.0, S.ntri());
      if (v.kM) k_convert<T, double><<<g, kVecThreads, 0, s>>>(v.kM, kM64_[l], 1.0, S.ntri());
    }
  }
  for (int l = 0; l < L; ++l) {
    const size_t n = specs_[l].ndof();
    const int g = vec_grid(n, sms_);
    diag_of(l, lv_[l].diag, s);
    k_convert<T, T><<<g, kVecThreads, 0, s>>>(lv_[l].dinv, lv_[l].diag, 1.0, n);
    k_recip<T><<<g, kVecThreads, 0, s>>>(lv_[l].dinv, n);
  }
  for (int l = 0; l + 1 < L; ++l) lv_[l].lmax = estimate_lmax(l, s);
  const LevelSpec& C = specs_[L - 1];
  if (C.NC == 2)
    k_coarse_inverse<T, 2><<<1, 256, 0, s>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], nullptr, cinv_, cstat_);
  else
    k_coarse_inverse<T, 1><<<1, 256, 0, s>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], kM64_[L - 1], cinv_,
                                             cstat_);
  int st = 0;
  cudaMemcpyAsync(&st, cstat_, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return -5;
  return st ? -2 : 0;
}

template <class T>
void MG<T>::smooth(int l, const T* b, T* x, bool xzero, cudaStream_t s) {
  Lev& v = lv_[l];
  const size_t n = specs_[l].ndof();
  const int g = vec_grid(n, sms_);
  const double hi = 1.1 * v.lmax, lo = cheb_lo_frac * v.lmax;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo);
  const double sigma = theta / delta;
  if (xzero) {
    cudaMemcpyAsync(v.r, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  } else {
    apply(l, x, v.t, s);
    k_sub<T><<<g, kVecThreads, 0, s>>>(v.r, b, v.t, n);
  }
  k_cheb_first<T><<<g, kVecThreads, 0, s>>>(v.r, v.dinv, v.d, x, T(1.0 / theta), xzero ? 1 : 0, n);
  double rho_old = 1.0 / sigma;
  for (int k = 1; k < cheb_degree; ++k) {
    apply(l, v.d, v.t, s);
    const double rho_new = 1.0 / (2.0 * sigma - rho_old);
    k_cheb_next<T><<<g, kVecThreads, 0, s>>>(v.r, v.t, v.dinv, v.d, x, T(rho_new * rho_old),
                                             T(2.0 * rho_new / delta), n);
    rho_old = rho_new;
  }
}

template <class T>
void MG<T>::restrict_to(int l, const T* rf, T* bc, cudaStream_t s) {
  const Transfer X = make_transfer(specs_[l], specs_[l + 1]);
  const int g = vec_grid(specs_[l + 1].nn(), sms_);
  if (specs_[l].NC == 2) k_restrict<T, 2><<<g, kVecThreads, 0, s>>>(X, rf, bc);
  else k_restrict<T, 1><<<g, kVecThreads, 0, s>>>(X, rf, bc);
}

template <class T>
void MG<T>::prolong_add(int l, const T* xc, T* xf, cudaStream_t s) {
  const Transfer X = make_transfer(specs_[l], specs_[l + 1]);
  const int g = vec_grid(specs_[l].nn(), sms_);
  if (specs_[l].NC == 2) k_prolong_add<T, 2><<<g, kVecThreads, 0, s>>>(X, xc, xf);
  else k_prolong_add<T, 1><<<g, kVecThreads, 0, s>>>(X, xc, xf);
}

template <class T>
void MG<T>::vcycle_level(int l, cudaStream_t s) {
  Lev& v = lv_[l];
  const int L = levels();
  if (l == L - 1) {
    const int n = int(specs_[l].ndof());
    k_dense_matvec<T><<<1, 256, 0, s>>>(cinv_, v.b, v.x, n);
    return;
  }
  const size_t n = specs_[l].ndof();
  const int g = vec_grid(n, sms_);
  smooth(l, v.b, v.x, true, s);
  apply(l, v.x, v.t, s);
  k_sub<T><<<g, kVecThreads, 0, s>>>(v.r, v.b, v.t, n);
  restrict_to(l, v.r, lv_[l + 1].b, s);
  vcycle_level(l + 1, s);
  prolong_add(l, lv_[l + 1].x, v.x, s);
  smooth(l, v.b, v.x, false, s);
}

template <class T>
void MG<T>::vcycle(const T* b, T* x, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  cudaMemcpyAsync(lv_[0].b, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  vcycle_level(0, s);
  cudaMemcpyAsync(x, lv_[0].x, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
}

template <class T>
int MG<T>::pcg(const T* b, T* x, bool x_nonzero, double rtol, int maxit, SolveStats& st, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  const int g = vec_grid(n, sms_);
  T* r = pcg_[0];
  T* z = pcg_[1];
  T* p = pcg_[2];
  T* q = pcg_[3];
  st = SolveStats{};
  const double bn = std::sqrt(dot(b, b, n, s));
  if (!std::isfinite(bn)) return -4;
  if (bn == 0.0) {
    k_fill<T><<<g, kVecThreads, 0, s>>>(x, T(0), n);
    return 0;
  }
  if (x_nonzero) {
    apply(0, x, q, s, true);
    k_sub<T><<<g, kVecThreads, 0, s>>>(r, b, q, n);
  } else {
    k_fill<T><<<g, kVecThreads, 0, s>>>(x, T(0), n);
    cudaMemcpyAsync(r, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  }
  double rn = std::sqrt(dot(r, r, n, s));
  st.relres = rn / bn;
  if (rn <= rtol * bn) return 0;
  vcycle(r, z, s);
  double rz = dot(r, z, n, s);
  cudaMemcpyAsync(p, z, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  for (int it = 1; it <= maxit; ++it) {
    apply(0, p, q, s, true);
    const double pq = dot(p, q, n, s);
    if (!std::isfinite(pq) || !std::isfinite(rz)) {
      st.iterations = it;
      return -4;
    }
    if (!(pq > 0.0) || !(rz > 0.0)) {
      // indefinite operator: continue with MINRES from the current iterate
      SolveStats ms;
      const int rc = minres(b, x, rtol, maxit - it, ms, s);
      st.iterations = it + ms.iterations;
      st.relres = ms.relres;
      st.minres = 1;
      return rc;
    }
    const double alpha = rz / pq;
    k_axpy<T><<<g, kVecThreads, 0, s>>>(x, T(alpha), p, n);
    k_axpy<T><<<g, kVecThreads, 0, s>>>(r, T(-alpha), q, n);
    rn = std::sqrt(dot(r, r, n, s));
    st.iterations = it;
    st.relres = rn / bn;
    if (!std::isfinite(rn)) return -4;
    if (rn <= rtol * bn) return 0;
    vcycle(r, z, s);
    const double rz_new = dot(r, z, n, s);
    const double beta = rz_new / rz;
    rz = rz_new;
    k_xpby<T><<<g, kVecThreads, 0, s>>>(p, z, T(beta), n);
  }
  return -2;
}

// Preconditioned MINRES (Paige & Saunders) with the SPD V-cycle as M, started
// from x.  The recurrence's residual estimate (in the M^-1 norm) steers the
// iteration; the true 2-norm residual is checked before returning.
template <class T>
int MG<T>::minres(const T* b, T* x, double rtol, int maxit, SolveStats& st, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  const int g = vec_grid(n, sms_);
  T* r1 = pcg_[0];
  T* r2 = pcg_[1];
  T* y = pcg_[2];
  T* v = pcg_[3];
  T* w = pcg_[5];
  T* w1 = pcg_[6];
  T* w2 = pcg_[7];
  T* t = pcg_[8];
  st = SolveStats{};
  const double bn = std::sqrt(dot(b, b, n, s));
  if (!std::isfinite(bn)) return -4;
  int total = 0;
  for (int restart = 0; restart < 4 && total < maxit; ++restart) {
    apply(0, x, t, s, true);
    k_sub<T><<<g, kVecThreads, 0, s>>>(r1, b, t, n);
    const double rn0 = std::sqrt(dot(r1, r1, n, s));
    st.relres = rn0 / bn;
    if (!std::isfinite(rn0)) return -4;
    if (rn0 <= rtol * bn) return 0;
    vcycle(r1, y, s);
    double beta1 = dot(r1, y, n, s);
    if (!(beta1 > 0.0)) return -2;
    beta1 = std::sqrt(beta1);
    cudaMemcpyAsync(r2, r1, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
    k_fill<T><<<g, kVecThreads, 0, s>>>(w, T(0), n);
    k_fill<T><<<g, kVecThreads, 0, s>>>(w2, T(0), n);
    double beta = beta1, oldb = 0.0, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
    // the M^-1-norm estimate is compared against the same ratio of the 2-norms
    const double target = rtol * bn / rn0;
    for (int it = 1; it <= maxit - total; ++it) {
      // v = y / beta ; y = A v - (beta/oldb) r1
      k_convert<T, T><<<g, kVecThreads, 0, s>>>(v, y, 1.0 / beta, n);
      apply(0, v, y, s, true);
      if (it >= 2) k_axpy<T><<<g, kVecThreads, 0, s>>>(y, T(-beta / oldb), r1, n);
      const double alpha = dot(v, y, n, s);
      k_axpy<T><<<g, kVecThreads, 0, s>>>(y, T(-alpha / beta), r2, n);
      std::swap(r1, r2);  // r1 <- r2, r2 <- y
      cudaMemcpyAsync(r2, y, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
      vcycle(r2, y, s);
      oldb = beta;
      const double bb = dot(r2, y, n, s);
      if (!std::isfinite(alpha) || !std::isfinite(bb)) return -4;
      if (!(bb > 0.0)) {
        total += it;
        break;
      }
      beta = std::sqrt(bb);
      const double oldeps = epsln;
      const double delta = cs * dbar + sn * alpha;
      const double gbar = sn * dbar - cs * alpha;
      epsln = sn * beta;
      dbar = -cs * beta;
      double gamma = std::sqrt(gbar * gbar + beta * beta);
      if (gamma < 1e-300) gamma = 1e-300;
      cs = gbar / gamma;
      sn = beta / gamma;
      const double phi = cs * phibar;
      phibar = sn * phibar;
      // w1 <- w2, w2 <- w, w = (v - oldeps w1 - delta w2) / gamma ; x += phi w
      std::swap(w1, w2);  // w1 <- old w2
      std::swap(w2, w);   // w2 <- old w ; w now holds the stale w1 (overwritten below)
      k_fill<T><<<g, kVecThreads, 0, s>>>(w, T(0), n);
      k_axpy<T><<<g, kVecThreads, 0, s>>>(w, T(1.0 / gamma), v, n);
      k_axpy<T><<<g, kVecThreads, 0, s>>>(w, T(-oldeps / gamma), w1, n);
      k_axpy<T><<<g, kVecThreads, 0, s>>>(w, T(-delta / gamma), w2, n);
      k_axpy<T><<<g, kVecThreads, 0, s>>>(x, T(phi), w, n);
      st.iterations = total + it;
      if (phibar / beta1 <= 0.5 * target) {
        total += it;
        break;
      }
      if (it == maxit - total) total = maxit;
    }
    st.minres = 1;
  }
  apply(0, x, t, s, true);
  k_sub<T><<<g, kVecThreads, 0, s>>>(r1, b, t, n);
  const double rn = std::sqrt(dot(r1, r1, n, s));
  st.relres = rn / bn;
  if (!std::isfinite(rn)) return -4;
  return rn <= rtol * bn ? 0 : -2;
}

}  // namespace topo
