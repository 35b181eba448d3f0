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
// Lattice kernels use a 2D grid: blockIdx.y is the row, x covers the columns.
constexpr int kRowThreads = 128;
#define kRowThreads_ 128
inline dim3 row_grid(int NX, int NY) { return dim3((NX + kRowThreads - 1) / kRowThreads, NY); }

// The tiled P2 kernel: load the operand tile, per-triangle element work,
// gather onto owned nodes with the mode's epilogue (apply, diagonal or one of
// the fused Chebyshev smoothing steps).
template <class T>
__global__ void __launch_bounds__(P2_THREADS)
    k_p2_tile(P2Params<T> P, const T* __restrict__ xi, P2Io<T> io) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  auto& s = *reinterpret_cast<P2Smem<T>*>(smem_raw);
  P2Kern<T>::load(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, io, xi, s);
  __syncthreads();
  P2Kern<T>::compute(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, io.mode == kP2Diag ? 1 : 0);
  __syncthreads();
  P2Kern<T>::gather(threadIdx.x, blockDim.x, blockIdx.x, blockIdx.y, P, s, io);
}

template <class T, int NC, int MODE>
__global__ void __launch_bounds__(kRowThreads_) k_p1_smooth(P1Params<T, NC> P, SmoothBufs<T> B) {
  const int a = blockIdx.x * kRowThreads_ + threadIdx.x, b = blockIdx.y;
  if (a > P.nx) return;
  if (MODE == kP2Pre) P1Smooth<T, NC>::pre(a, b, P, B);
  else if (MODE == kP2Res) P1Smooth<T, NC>::res(a, b, P, B);
  else if (MODE == kP2First) P1Smooth<T, NC>::first(a, b, P, B);
  else P1Smooth<T, NC>::post2(a, b, P, B);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads_) k_prolong_add(Transfer X, const T* __restrict__ xc, T* __restrict__ xf) {
  const int a = blockIdx.x * kRowThreads_ + threadIdx.x, b = blockIdx.y;
  if (a < X.NXf) TransferKern<T, NC>::node_prolong_add(a, b, X, xc, xf);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_p1_apply(P1Params<T, NC> P, const T* __restrict__ u, T* __restrict__ y) {
  const int a = blockIdx.x * kRowThreads + threadIdx.x, b = blockIdx.y;
  if (a <= P.nx) P1Kern<T, NC>::node_apply(a, b, P, u, y);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_p1_diag(P1Params<T, NC> P, T* __restrict__ d) {
  const int a = blockIdx.x * kRowThreads + threadIdx.x, b = blockIdx.y;
  if (a <= P.nx) P1Kern<T, NC>::node_diag(a, b, P, d);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_restrict(Transfer X, const T* __restrict__ rf, T* __restrict__ bc,
                                                          const T* __restrict__ tf) {
  const int I = blockIdx.x * kRowThreads + threadIdx.x, J = blockIdx.y;
  if (I < X.NXc) TransferKern<T, NC>::node_restrict(I, J, X, rf, bc, tf);
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
// coarse-level tail: the V-cycle over the smallest levels runs in one CTA with
// every work vector resident in shared memory (one launch for ~6 x levels
// phases; read-only data -- coefficients, D^-1, element matrices -- via L1)
// ---------------------------------------------------------------------------
constexpr int kTailThreads = 1024;
constexpr int kTailMaxLevels = 10;
constexpr int kTailMaxNodes = 4096;
constexpr size_t kTailSmemBudget = 160 * 1024;

template <class T, int NC>
struct TailLevel {
  P1Params<T, NC> P;
  Transfer X;  // to the next coarser level
  const T* dinv;
  const double* cheb;
  int NX, nn, off;  // off: first of this level's five shared vectors x, b, r, d, x2 (NC*nn each)
};

template <class T, int NC>
struct TailDesc {
  int nlev, smem_elems;
  const T* cinv;
  TailLevel<T, NC> lv[kTailMaxLevels];
};

template <class T, int NC>
__global__ void __launch_bounds__(kTailThreads)
    k_tail_vcycle(const TailDesc<T, NC>* __restrict__ D, const T* __restrict__ b_in, T* __restrict__ x_out) {
  extern __shared__ __align__(16) unsigned char tail_raw[];
  T* sm = reinterpret_cast<T*>(tail_raw);
  const int nlev = D->nlev;
  auto bufs = [&](int l) {
    const TailLevel<T, NC>& L = D->lv[l];
    const int m = NC * L.nn;
    T* base = sm + L.off;
    return SmoothBufs<T>{base + m, L.dinv, base, base + 4 * m, base + 2 * m, base + 3 * m, L.cheb};
  };
  {
    const int m = NC * D->lv[0].nn;
    T* b0 = sm + D->lv[0].off + m;
    for (int i = threadIdx.x; i < m; i += blockDim.x) b0[i] = b_in[i];
  }
  __syncthreads();
  for (int l = 0; l + 1 < nlev; ++l) {
    const TailLevel<T, NC>& L = D->lv[l];
    const SmoothBufs<T> B = bufs(l);
    for (int n = threadIdx.x; n < L.nn; n += blockDim.x) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::pre(a, b, L.P, B);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < L.nn; n += blockDim.x) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::res(a, b, L.P, B);
    }
    __syncthreads();
    const TailLevel<T, NC>& C = D->lv[l + 1];
    T* bc = sm + C.off + NC * C.nn;
    for (int n = threadIdx.x; n < C.nn; n += blockDim.x) {
      const int J = n / C.NX, I = n - J * C.NX;
      TransferKern<T, NC>::node_restrict(I, J, L.X, B.r, bc);
    }
    __syncthreads();
  }
  {
    const TailLevel<T, NC>& C = D->lv[nlev - 1];
    const int m = NC * C.nn;
    const T* bc = sm + C.off + m;
    T* xc = sm + C.off;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      T acc = T(0);
      for (int j = 0; j < m; ++j) acc += D->cinv[size_t(i) * m + j] * bc[j];
      xc[i] = acc;
    }
    __syncthreads();
  }
  for (int l = nlev - 2; l >= 0; --l) {
    const TailLevel<T, NC>& L = D->lv[l];
    const SmoothBufs<T> B = bufs(l);
    const T* xc = sm + D->lv[l + 1].off;
    for (int n = threadIdx.x; n < L.nn; n += blockDim.x) {
      const int b = n / L.NX, a = n - b * L.NX;
      TransferKern<T, NC>::node_prolong_add(a, b, L.X, xc, B.x);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < L.nn; n += blockDim.x) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::first(a, b, L.P, B);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < L.nn; n += blockDim.x) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::post2(a, b, L.P, B);
    }
    __syncthreads();
  }
  {
    const int m = NC * D->lv[0].nn;
    const T* x0 = sm + D->lv[0].off;
    for (int i = threadIdx.x; i < m; i += blockDim.x) x_out[i] = x0[i];
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
template <class T>
inline void set_p2_smem_attr() {
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(k_p2_tile<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(P2Smem<T>)));
    done = true;
  }
}

template <class T>
inline void launch_p2_tile(const P2Params<T>& P, const T* xi, const P2Io<T>& io, cudaStream_t s) {
  set_p2_smem_attr<T>();
  dim3 g((P.nx + P2_TX - 1) / P2_TX, (P.ny + P2_TY - 1) / P2_TY);
  k_p2_tile<T><<<g, P2_THREADS, sizeof(P2Smem<T>), s>>>(P, xi, io);
}

template <class T>
inline void launch_p2_apply(const P2Params<T>& P, const T* xi, const T* x, T* y, cudaStream_t s) {
  P2Io<T> io;
  std::memset(&io, 0, sizeof(io));
  io.mode = kP2Apply;
  io.u = x;
  io.y = y;
  launch_p2_tile<T>(P, xi, io, s);
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
// graph-resident CG scalars
// ---------------------------------------------------------------------------
// x += alpha p ; r -= alpha q with alpha = rz / pq read from device memory
template <class T>
__global__ void k_pcg_xr(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q,
                         const PcgDev* __restrict__ dv, size_t n) {
  const double pq = dv->pq;
  if (!(pq > 0.0) || !isfinite(pq)) return;
  const T alpha = T(dv->rz / pq);
  TOPO_GRID_STRIDE(i, n) {
    x[i] += alpha * p[i];
    r[i] -= alpha * q[i];
  }
}

// p = z + beta p
template <class T>
__global__ void k_pcg_p(T* __restrict__ p, const T* __restrict__ z, const PcgDev* __restrict__ dv, size_t n) {
  const T beta = T(dv->beta);
  TOPO_GRID_STRIDE(i, n) p[i] = z[i] + beta * p[i];
}

// after the prologue: decide whether the loop runs at all.  On entry dv->tol2
// holds rtol^2 and dv->maxit the iteration cap (both written by the host).
static __global__ void k_pcg_start(PcgDev* dv, cudaGraphConditionalHandle h, int use_cond) {
  const double bb = dv->bb, rr = dv->rr;
  dv->tol2 = dv->tol2 * bb;
  dv->it = 0;
  dv->relres = bb > 0 ? sqrt(rr / bb) : 0.0;
  int st = 1;
  if (!isfinite(bb) || !isfinite(rr) || !isfinite(dv->rz)) st = 4;
  else if (bb == 0.0) st = 5;
  else if (rr <= dv->tol2) st = 0;
  dv->status = st;
  if (use_cond) cudaGraphSetConditional(h, st == 1 ? 1u : 0u);
}

// end of one iteration: convergence / cap / breakdown test and beta
static __global__ void k_pcg_check(PcgDev* dv, cudaGraphConditionalHandle h, int use_cond) {
  dv->it += 1;
  const double pq = dv->pq, rr = dv->rr, rzn = dv->rz_new;
  dv->relres = sqrt(rr / dv->bb);
  int st = 1;
  if (!isfinite(pq) || !isfinite(rr) || !isfinite(rzn)) st = 4;
  else if (!(pq > 0.0) || !(dv->rz > 0.0)) st = 3;
  else if (rr <= dv->tol2) st = 0;
  else if (dv->it >= dv->maxit) st = 2;
  dv->beta = (st == 1) ? rzn / dv->rz : 0.0;
  dv->rz = rzn;
  dv->status = st;
  if (use_cond) cudaGraphSetConditional(h, st == 1 ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// MG<T>
// ---------------------------------------------------------------------------
template <class T>
MG<T>::~MG() {
  for (auto& g : graph_)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  for (auto c : cap_)
    if (c) cudaStreamDestroy(c);
  if (hdev_) cudaFreeHost(hdev_);
}

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
    if (l > 0) {
      v.x = arena.alloc_n<T>(n);
      v.b = arena.alloc_n<T>(n);
    }
    v.r = arena.alloc_n<T>(n);
    v.d = arena.alloc_n<T>(n);
    v.t = arena.alloc_n<T>(n);
    v.x2 = arena.alloc_n<T>(n);
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
  cheb_ = arena.alloc_n<double>(8 * specs.size());
  dev_ = arena.alloc_n<PcgDev>(1);
  if (!hdev_) cudaMallocHost(&hdev_, sizeof(PcgDev));
  for (auto& c : cap_)
    if (!c) cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking);
  set_p2_smem_attr<T>();
  graph_valid_ = false;
  build_tail(arena);
}

// Chooses the tail levels (smallest levels whose shared vectors fit the
// budget, never level 0) and uploads their descriptor.
template <class T>
void MG<T>::build_tail(Arena& arena) {
  tail_ = -1;
  tail_desc_ = nullptr;
  tail_smem_ = 0;
  const int L = levels();
  size_t bytes = 0;
  int first = L;
  for (int l = L - 1; l >= 1; --l) {
    const size_t add = 5 * specs_[l].ndof() * sizeof(T);
    if (specs_[l].nn() > size_t(kTailMaxNodes) || bytes + add > kTailSmemBudget || L - l > kTailMaxLevels) break;
    bytes += add;
    first = l;
  }
  if (first >= L - 1) return;  // fewer than two levels: nothing to gain
  auto build = [&](auto nc_tag) {
    constexpr int NC = decltype(nc_tag)::value;
    TailDesc<T, NC> h;
    std::memset(&h, 0, sizeof(h));
    h.nlev = L - first;
    h.cinv = cinv_;
    int off = 0;
    for (int k = 0; k < h.nlev; ++k) {
      const int l = first + k;
      TailLevel<T, NC>& d = h.lv[k];
      d.P = make_p1<T, NC>(specs_[l], refs_[l], lv_[l].kK, NC == 1 ? lv_[l].kM : nullptr);
      if (l + 1 < L) d.X = make_transfer(specs_[l], specs_[l + 1]);
      d.dinv = lv_[l].dinv;
      d.cheb = cheb_ + 8 * l;
      d.NX = specs_[l].NX;
      d.nn = int(specs_[l].nn());
      d.off = off;
      off += 5 * NC * d.nn;
    }
    h.smem_elems = off;
    void* p = arena.alloc(sizeof(h));
    if (!p) return;
    cudaMemcpy(p, &h, sizeof(h), cudaMemcpyHostToDevice);
    if (cudaFuncSetAttribute(k_tail_vcycle<T, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(size_t(off) * sizeof(T))) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    tail_desc_ = p;
    tail_smem_ = size_t(off) * sizeof(T);
    tail_ = first;
  };
  if (specs_[first].NC == 2) build(std::integral_constant<int, 2>{});
  else build(std::integral_constant<int, 1>{});
}

template <class T>
void MG<T>::apply(int l, const T* x, T* y, cudaStream_t s, bool op) {
  const LevelSpec& L = specs_[l];
  ++launches;
  if (L.p2) {
    launch_p2_apply<T>(op ? p2_op_ : p2_, xi_, x, y, s);
    return;
  }
  const dim3 g = row_grid(L.NX, L.NY);
  if (L.NC == 2) {
    auto P = make_p1<T, 2>(L, refs_[l], lv_[l].kK, nullptr);
    k_p1_apply<T, 2><<<g, kRowThreads, 0, s>>>(P, x, y);
  } else {
    auto P = make_p1<T, 1>(L, refs_[l], lv_[l].kK, lv_[l].kM);
    k_p1_apply<T, 1><<<g, kRowThreads, 0, s>>>(P, x, y);
  }
}

template <class T>
void MG<T>::diag_of(int l, T* d, cudaStream_t s) {
  const LevelSpec& L = specs_[l];
  ++launches;
  if (L.p2) {
    P2Io<T> io;
    std::memset(&io, 0, sizeof(io));
    io.mode = kP2Diag;
    io.y = d;
    launch_p2_tile<T>(p2_, xi_, io, s);
    return;
  }
  const dim3 g = row_grid(L.NX, L.NY);
  if (L.NC == 2) {
    auto P = make_p1<T, 2>(L, refs_[l], lv_[l].kK, nullptr);
    k_p1_diag<T, 2><<<g, kRowThreads, 0, s>>>(P, d);
  } else {
    auto P = make_p1<T, 1>(L, refs_[l], lv_[l].kK, lv_[l].kM);
    k_p1_diag<T, 1><<<g, kRowThreads, 0, s>>>(P, d);
  }
}

template <class T>
double MG<T>::dot(const T* a, const T* b, size_t n, cudaStream_t s) {
  ++launches;
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
  T* x = v.r;
  T* y = v.d;
  k_power_start<T><<<g, kVecThreads, 0, s>>>(x, n);
  for (int it = 0; it < power_iters; ++it) {
    apply(l, x, y, s);
    k_mul<T><<<g, kVecThreads, 0, s>>>(x, v.dinv, y, n);
    launches += 1;
    if (it % 4 == 3) {  // rescale to stay in range
      const double nrm = std::sqrt(dot(x, x, n, s));
      if (!(nrm > 0) || !std::isfinite(nrm)) return 4.0;
      k_scale<T><<<g, kVecThreads, 0, s>>>(x, T(1.0 / nrm), n);
      launches += 1;
    }
  }
  apply(l, x, y, s);
  const double num = dot(x, y, n, s);
  k_mul<T><<<g, kVecThreads, 0, s>>>(v.t, v.diag, x, n);
  launches += 2;
  const double den = dot(x, v.t, n, s);
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
      launches += v.kM ? 2 : 1;
    }
  }
  for (int l = 0; l < L; ++l) {
    const size_t n = specs_[l].ndof();
    const int g = vec_grid(n, sms_);
    diag_of(l, lv_[l].diag, s);
    k_convert<T, T><<<g, kVecThreads, 0, s>>>(lv_[l].dinv, lv_[l].diag, 1.0, n);
    k_recip<T><<<g, kVecThreads, 0, s>>>(lv_[l].dinv, n);
    launches += 2;
  }
  std::vector<double> cc(8 * L, 0.0);
  for (int l = 0; l + 1 < L; ++l) {
    const LevelSpec& S = specs_[l];
    if (!S.p2 && S.NC == 2) {
      lv_[l].lmax = p1_elasticity_bound(refs_[l]);
      lv_[l].bound = true;
    } else {
      lv_[l].lmax = estimate_lmax(l, s);
      lv_[l].bound = false;
    }
    const double hi = (lv_[l].bound ? 1.0 : 1.1) * lv_[l].lmax, lo = cheb_lo_frac * lv_[l].lmax;
    const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
    double* c = cc.data() + 8 * l;
    c[0] = 1.0 / theta;
    double rho_old = 1.0 / sigma;
    for (int k = 1; k < cheb_degree && k < 4; ++k) {
      const double rho_new = 1.0 / (2.0 * sigma - rho_old);
      c[2 * k - 1] = rho_new * rho_old;
      c[2 * k] = 2.0 * rho_new / delta;
      rho_old = rho_new;
    }
  }
  cudaMemcpyAsync(cheb_, cc.data(), cc.size() * sizeof(double), cudaMemcpyHostToDevice, s);
  const LevelSpec& C = specs_[L - 1];
  if (C.NC == 2)
    k_coarse_inverse<T, 2><<<1, 256, 0, s>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], nullptr, cinv_, cstat_);
  else
    k_coarse_inverse<T, 1><<<1, 256, 0, s>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], kM64_[L - 1], cinv_,
                                             cstat_);
  launches += 1;
  int st = 0;
  cudaMemcpyAsync(&st, cstat_, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return -5;
  return st ? -2 : 0;
}

// One V-cycle from level l down: fused degree-2 Chebyshev pre-smoothing from
// x = 0, residual restriction, coarse correction, fused post-smoothing.
template <class T>
void MG<T>::vcycle_level(int l, const T* b, T* x, cudaStream_t s) {
  Lev& v = lv_[l];
  const int L = levels();
  const LevelSpec& S = specs_[l];
  if (l == tail_ && tail_desc_) {
    if (S.NC == 2)
      k_tail_vcycle<T, 2><<<1, kTailThreads, tail_smem_, s>>>(static_cast<const TailDesc<T, 2>*>(tail_desc_), b, x);
    else
      k_tail_vcycle<T, 1><<<1, kTailThreads, tail_smem_, s>>>(static_cast<const TailDesc<T, 1>*>(tail_desc_), b, x);
    ++launches;
    return;
  }
  if (l == L - 1) {
    k_dense_matvec<T><<<1, 256, 0, s>>>(cinv_, b, x, int(S.ndof()));
    ++launches;
    return;
  }
  SmoothBufs<T> B{b, v.dinv, x, v.x2, v.r, v.d, cheb_ + 8 * l};
  const Transfer X = make_transfer(S, specs_[l + 1]);
  Lev& c = lv_[l + 1];
  const dim3 gf = row_grid(S.NX, S.NY), gc = row_grid(X.NXc, X.NYc);
  if (S.p2) {
    P2Io<T> io;
    std::memset(&io, 0, sizeof(io));
    io.B = B;
    io.u = x;
    io.mode = kP2Pre;
    launch_p2_tile<T>(p2_, xi_, io, s);
    io.mode = kP2Res;
    launch_p2_tile<T>(p2_, xi_, io, s);
    k_restrict<T, 2><<<gc, kRowThreads, 0, s>>>(X, v.r, c.b, nullptr);
    launches += 3;
    vcycle_level(l + 1, c.b, c.x, s);
    k_prolong_add<T, 2><<<gf, kRowThreads, 0, s>>>(X, c.x, x);
    io.mode = kP2First;
    launch_p2_tile<T>(p2_, xi_, io, s);
    io.mode = kP2Post2;
    launch_p2_tile<T>(p2_, xi_, io, s);
    launches += 3;
    return;
  }
  auto run = [&](auto nc_tag) {
    constexpr int NC = decltype(nc_tag)::value;
    const auto P = make_p1<T, NC>(S, refs_[l], v.kK, NC == 1 ? v.kM : nullptr);
    k_p1_smooth<T, NC, kP2Pre><<<gf, kRowThreads, 0, s>>>(P, B);
    k_p1_smooth<T, NC, kP2Res><<<gf, kRowThreads, 0, s>>>(P, B);
    k_restrict<T, NC><<<gc, kRowThreads, 0, s>>>(X, v.r, c.b, nullptr);
    launches += 3;
    vcycle_level(l + 1, c.b, c.x, s);
    k_prolong_add<T, NC><<<gf, kRowThreads, 0, s>>>(X, c.x, x);
    k_p1_smooth<T, NC, kP2First><<<gf, kRowThreads, 0, s>>>(P, B);
    k_p1_smooth<T, NC, kP2Post2><<<gf, kRowThreads, 0, s>>>(P, B);
    launches += 3;
  };
  if (S.NC == 2) run(std::integral_constant<int, 2>{});
  else run(std::integral_constant<int, 1>{});
}

template <class T>
void MG<T>::vcycle(const T* b, T* x, cudaStream_t s) {
  vcycle_level(0, b, x, s);
}

// Records the CG solve into a graph: a prologue (initial residual, first
// preconditioned direction, start test) followed by a WHILE conditional node
// whose body is one CG iteration; the body's last kernel decides whether the
// loop continues, so the solve runs without host round trips.  The loop is
// bounded by maxit (checked on the device).  Recording happens on two streams
// owned by this object (capture is not possible on the legacy default stream);
// every graph call is checked and nothing is launched unless all succeeded.
template <class T>
void MG<T>::pcg_prologue(bool warm, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  const int g = vec_grid(n, sms_);
  T *r = pcg_[0], *z = pcg_[1], *p = pcg_[2], *q = pcg_[3], *bi = pcg_[5], *xi = pcg_[6];
  if (warm) {
    apply(0, xi, q, s, true);
    k_sub<T><<<g, kVecThreads, 0, s>>>(r, bi, q, n);
  } else {
    k_fill<T><<<g, kVecThreads, 0, s>>>(xi, T(0), n);
    cudaMemcpyAsync(r, bi, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  }
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(bi, bi, n, red_->partials, red_->counter, &dev_->bb);
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(r, r, n, red_->partials, red_->counter, &dev_->rr);
  vcycle(r, z, s);
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(r, z, n, red_->partials, red_->counter, &dev_->rz);
  cudaMemcpyAsync(p, z, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  launches += 5;
}

template <class T>
void MG<T>::pcg_body(cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  const size_t n = specs_[0].ndof();
  const int g = vec_grid(n, sms_);
  T *r = pcg_[0], *z = pcg_[1], *p = pcg_[2], *q = pcg_[3], *xi = pcg_[6];
  apply(0, p, q, s, true);
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(p, q, n, red_->partials, red_->counter, &dev_->pq);
  k_pcg_xr<T><<<g, kVecThreads, 0, s>>>(xi, r, p, q, dev_, n);
  vcycle(r, z, s);
  k_dot2<T><<<red_->blocks, kVecThreads, 0, s>>>(r, r, r, z, n, red_->partials, red_->counter, &dev_->rr);
  k_pcg_check<<<1, 1, 0, s>>>(dev_, h, use_cond);
  k_pcg_p<T><<<g, kVecThreads, 0, s>>>(p, z, dev_, n);
  launches += 5;
}

// Records the CG solve into a graph: a prologue (initial residual, first
// preconditioned direction, start test) followed by a WHILE conditional node
// whose body is one CG iteration; the body's last kernel decides whether the
// loop continues, so the solve runs without host round trips.  The loop is
// bounded by maxit (checked on the device).  Recording happens on two streams
// owned by this object (capture is not possible on the legacy default stream);
// every graph call is checked and nothing is launched unless all succeeded.
template <class T>
int MG<T>::capture_pcg(bool warm) {
  cudaStream_t s = cap_[0], sb = cap_[1];
  if (!s || !sb) return -5;
  Graph& G = graph_[warm ? 1 : 0];
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  cudaGetLastError();
  const long long l0 = launches;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return -5;
  bool ok = true;
  cudaGraphNode_t wnode = nullptr;
  long long l1 = 0, l2 = 0;
  {
    pcg_prologue(warm, s);
    cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    ok &= cudaStreamGetCaptureInfo(s, &cst, nullptr, &cg, &deps, nullptr, &ndeps) == cudaSuccess;
    ok &= (cst == cudaStreamCaptureStatusActive) && cg != nullptr;
    cudaGraphConditionalHandle h = 0;
    if (ok) ok &= cudaGraphConditionalHandleCreate(&h, cg, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
      k_pcg_start<<<1, 1, 0, s>>>(dev_, h, 1);
      ok &= cudaStreamGetCaptureInfo(s, &cst, nullptr, &cg, &deps, nullptr, &ndeps) == cudaSuccess;
      ok &= (cst == cudaStreamCaptureStatusActive);
    }
    cudaGraphNodeParams cp = {};
    if (ok) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = h;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      ok &= cudaGraphAddNode(&wnode, cg, deps, nullptr, ndeps, &cp) == cudaSuccess;
      ok &= cp.conditional.phGraph_out != nullptr;
    }
    if (ok) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      l1 = launches;
      ok &= cudaStreamBeginCaptureToGraph(sb, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
            cudaSuccess;
      if (ok) {
        pcg_body(sb, h, 1);
        ok &= cudaStreamEndCapture(sb, &body) == cudaSuccess;
      }
      l2 = launches;
      if (ok) ok &= cudaStreamUpdateCaptureDependencies(s, &wnode, nullptr, 1, cudaStreamSetCaptureDependencies) ==
                    cudaSuccess;
    }
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(s, &graph);
  ok &= (ee == cudaSuccess) && graph != nullptr;
  if (ok) ok &= cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  ok &= cudaGetLastError() == cudaSuccess;
  launches = l0;  // recording is not execution
  if (!ok) {
    if (G.exec) cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
    return -5;
  }
  G.prologue_nodes = (l1 - l0) + 1;
  G.body_nodes = (l2 - l1);
  return 0;
}

// Runs the captured solve: inputs are copied into the graph's fixed buffers,
// rtol^2 and the iteration cap are written to the device scalars the start
// kernel reads, and the result and the scalars come back after one sync.
template <class T>
int MG<T>::graph_pcg(const T* b, T* x, bool warm, double rtol, int maxit, SolveStats& st, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  T* bi = pcg_[5];
  T* xi = pcg_[6];
  if (!graph_valid_) {
    for (auto& G : graph_)
      if (G.exec) {
        cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
      }
    graph_valid_ = true;
  }
  Graph& G = graph_[warm ? 1 : 0];
  if (use_graphs && !G.exec) {
    // the recording streams must not see work still queued on s
    if (cudaStreamSynchronize(s) != cudaSuccess) return -5;
    if (capture_pcg(warm) != 0) return -5;
  }
  hdev_->tol2 = rtol * rtol;
  hdev_->maxit = maxit;
  cudaMemcpyAsync(bi, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  if (warm) cudaMemcpyAsync(xi, x, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(&dev_->tol2, &hdev_->tol2, sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(&dev_->maxit, &hdev_->maxit, sizeof(int), cudaMemcpyHostToDevice, s);
  if (use_graphs) {
    cudaGraphLaunch(G.exec, s);
    launches += G.prologue_nodes;
  } else {
    // host-driven loop over the same kernels (one sync per iteration)
    pcg_prologue(warm, s);
    k_pcg_start<<<1, 1, 0, s>>>(dev_, 0, 0);
    ++launches;
    for (;;) {
      cudaMemcpyAsync(&hdev_->status, &dev_->status, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return -5;
      if (hdev_->status != 1) break;
      pcg_body(s, 0, 0);
    }
  }
  cudaMemcpyAsync(x, xi, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(hdev_, dev_, sizeof(PcgDev), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -5;
  st.iterations = hdev_->it;
  st.relres = hdev_->relres;
  if (use_graphs) launches += (long long)hdev_->it * G.body_nodes;
  switch (hdev_->status) {
    case 0: return 0;
    case 5:
      k_fill<T><<<vec_grid(n, sms_), kVecThreads, 0, s>>>(x, T(0), n);
      return 0;
    case 4: return -4;
    case 3: return -3;  // breakdown: caller falls back
    default: return -2;
  }
}

template <class T>
int MG<T>::pcg(const T* b, T* x, bool x_nonzero, double rtol, int maxit, SolveStats& st, cudaStream_t s) {
  st = SolveStats{};
  int rc = graph_pcg(b, x, x_nonzero, rtol, maxit, st, s);
  if (rc == -3) {
    // p.Ap <= 0: the operator is indefinite here; continue with MINRES from x
    SolveStats ms;
    rc = minres(b, x, rtol, std::max(1, maxit - st.iterations), ms, s);
    st.iterations += ms.iterations;
    st.relres = ms.relres;
    st.minres = 1;
  }
  return rc;
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
