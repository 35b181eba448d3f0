// Kernels and host orchestration of the multigrid-preconditioned CG.
// Included by topo_mg_f32.cu / topo_mg_f64.cu, which instantiate MG<T>.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <utility>

#include "topo_kclock.h"
#include "topo_mg.h"
#include "topo_p1.cuh"
#include "topo_p1march.cuh"
#include "topo_p2.cuh"
#include "topo_vec.cuh"

namespace topo {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// Lattice kernels use a 2D grid: blockIdx.y is the row, x covers the columns.
constexpr int kRowThreads = 128;
// P1 levels keep an assembled stencil up to a node count: elasticity levels
// up to 2^18 nodes (a larger one streams 112 B per node per pass, more than
// evaluating its element matrices on the fly costs), filter levels always
// (32 B per node).  TOPO_STENCIL_NODES overrides both limits.
inline size_t stencil_max_nodes(int NC) {
  if (const char* e = std::getenv("TOPO_STENCIL_NODES")) return size_t(std::strtoull(e, nullptr, 10));
  return NC == 2 ? (size_t(1) << 18) : (size_t(1) << 40);
}
#define kRowThreads_ 128
inline dim3 row_grid(int NX, int NY) { return dim3((NX + kRowThreads - 1) / kRowThreads, NY); }

// The column-march P2 kernel (see P2March): each warp marches over one
// segment of cell rows; operand, density and element results move between
// lanes by shuffles.
template <class T>
__device__ __forceinline__ T shfl_down1(T v) { return __shfl_down_sync(0xffffffffu, v, 1); }
template <class T>
__device__ __forceinline__ T shfl_up1(T v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ dd shfl_down1(dd v) { return dd(shfl_down1(v.hi), shfl_down1(v.lo)); }
__device__ __forceinline__ dd shfl_up1(dd v) { return dd(shfl_up1(v.hi), shfl_up1(v.lo)); }

// column 2 of rows R0..2 (operand) and of density rows from lane L+1
template <class T, int R0, bool OPERAND>
__device__ __forceinline__ void p2m_exchange_down(P2Lane<T>& L) {
  if (OPERAND) {
#pragma unroll
    for (int r = R0; r <= 2; ++r)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const T v = shfl_down1(L.U[r][0][c]);
        if (!L.edge) L.U[r][2][c] = v;
      }
  }
#pragma unroll
  for (int r = (R0 == 0 ? 0 : 1); r <= 1; ++r) {
    const T v = shfl_down1(L.X[r][0]);
    if (!L.edge) L.X[r][1] = v;
  }
}

// element results of column 2 to lane L+1's column 0
template <class T>
__device__ __forceinline__ void p2m_exchange_up(P2Lane<T>& L, int lane) {
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const T v = shfl_up1(L.A[r][2][c]);
      if (lane > 0) L.A[r][0][c] += v;
    }
}

// End of one CG iteration: convergence / cap / breakdown test and beta (run by
// one thread: the reduction's last block, or k_pcg_check).
__device__ inline void pcg_check_dev(PcgDev* dv, cudaGraphConditionalHandle h, int use_cond) {
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

// One warp's march over cell rows js .. je-1 (see P2March).  LEAN: the warp's
// region passed P2March::lean_region, so the phases make no per-node tests.
template <class T, int MODE, bool LEAN>
__device__ __forceinline__ void p2_march_run(const P2Params<T>& P, const T* __restrict__ xi, const P2Io<T>& io,
                                             int lane, int js, int je, T (&acc)[2]) {
  constexpr bool OPERAND = MODE != kP2Diag;
  P2Lane<T> L;
  P2March<T>::begin(P, L, int(blockIdx.x) * P2M_OWN - 1 + lane, lane == 31);
  const bool owner = lane > 0 && L.i <= P.nx;
  int j = js > 0 ? js - 1 : 0;
  P2March<T>::template load<0, LEAN>(P, io, xi, L, j);
  P2March<T>::template load_mass<LEAN>(P, L.K, L.i, j, L.M);
  p2m_exchange_down<T, 0, OPERAND>(L);
  P2Next<T> N;
  for (;;) {
    const bool more = j + 1 < je;
    if (more) P2March<T>::template prefetch<LEAN>(P, io, xi, L, j + 1, N);  // in flight during this step's arithmetic
    const bool fin = owner && j >= js;
    typename P2March<T>::Fin F;
    if (MODE != kP2Apply && MODE != kP2Diag && fin) P2March<T>::template fin_load<LEAN>(P, io, L, j, F);
    // the pair type keeps no prefetched mass matrices (registers): they are loaded here
    if constexpr (IsDD<T>::value) P2March<T>::template load_mass<LEAN>(P, L.K, L.i, j, L.M);
    P2March<T>::template compute<LEAN>(P, L, j, MODE);
    p2m_exchange_up<T>(L, lane);
    if (fin) P2March<T>::template finish<LEAN>(P, io, L, j, j == P.ny - 1 ? 3 : 2, F, acc);
    if (!more) break;
    ++j;
    P2March<T>::advance(L);
    P2March<T>::take(L, N);
    p2m_exchange_down<T, 1, OPERAND>(L);
  }
}

// resident blocks the register budget is sized for: FP32 4, pair-of-FP32 3, FP64 2
template <class T>
constexpr int p2_march_min_blocks() {
  return IsDD<T>::value ? 3 : sizeof(T) == 4 ? 4 : 2;
}

template <class T, int MODE>
__global__ void __launch_bounds__(P2M_THREADS, p2_march_min_blocks<T>())
    k_p2_march(P2Params<T> P, const T* __restrict__ xi, P2Io<T> io, int seg) {
  TOPO_PDL_ENTRY();
  io.mode = MODE;  // compile-time mode: the per-node switches fold
  P2March<T>::prepare(io);
  const int lane = threadIdx.x & 31;
  const int js = (blockIdx.y * P2M_WARPS + (threadIdx.x >> 5)) * seg;
  T acc[2] = {T(0), T(0)};  // fused CG reductions (P2Io::fuse)
  if (js < P.ny) {  // whole warp: warps past the last segment only join the reduction
    const int je = min(js + seg, P.ny);
    // warp-uniform: the same cell columns and rows for all lanes
    if constexpr (IsDD<T>::value) {
      // pair-of-FP32: issue-bound on a long element body; one copy of it (the masked
      // phases) keeps the code within reach of the instruction caches
      p2_march_run<T, MODE, false>(P, xi, io, lane, js, je, acc);
    } else if (P2March<T>::lean_region(P, int(blockIdx.x) * P2M_OWN - 1, js > 0 ? js - 1 : 0, je)) {
      p2_march_run<T, MODE, true>(P, xi, io, lane, js, je, acc);
    } else {
      p2_march_run<T, MODE, false>(P, xi, io, lane, js, je, acc);
    }
  }
  if constexpr ((MODE == kP2Apply || MODE == kP2Post2) && !IsDD<T>::value) {
    if (io.fuse != kFuseNone) {
      double tot[2];
      if (finish_reduction<2>(acc, io.partials, io.counter, tot)) {
        if (io.fuse == kFusePQ) {
          io.pcg->pq = tot[0];
        } else {
          io.pcg->rr = tot[0];
          io.pcg->rz_new = tot[1];
          pcg_check_dev(io.pcg, cudaGraphConditionalHandle(io.cond), io.use_cond);
        }
      }
    }
  }
}

// The column-march kernel of the large P1 levels (see P1March).
template <class T, int NC, int MODE>
__global__ void __launch_bounds__(P2M_THREADS) k_p1_march(P1Params<T, NC> P, P1Io<T> io, int seg) {
  TOPO_PDL_ENTRY();
  io.mode = MODE;
  P1March<T, NC>::prepare(io);
  const int lane = threadIdx.x & 31;
  const int js = (blockIdx.y * P2M_WARPS + (threadIdx.x >> 5)) * seg;
  if (js >= P.ny) return;  // whole warp
  const int je = min(js + seg, P.ny);
  P1Lane<T, NC> L;
  P1March<T, NC>::begin(L, int(blockIdx.x) * P2M_OWN - 1 + lane, lane == 31);
  const bool owner = lane > 0 && L.i <= P.nx;
  int j = js > 0 ? js - 1 : 0;
  auto down = [&](int r0) {
#pragma unroll
    for (int r = 0; r <= 1; ++r) {
      if (r < r0) continue;
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        const T v = shfl_down1(L.U[r][0][d]);
        if (!L.edge) L.U[r][1][d] = v;
      }
    }
  };
  P1March<T, NC>::template load<0>(P, io, L, j);
  P1March<T, NC>::load_coef(P, L.i, j, L.kk, L.km);
  down(0);
  P1Next<T, NC> N;
  for (;;) {
    const bool more = j + 1 < je;
    if (more) P1March<T, NC>::prefetch(P, io, L, j + 1, N);  // in flight during this step's arithmetic
    const bool fin = owner && j >= js;
    typename P1March<T, NC>::Fin F;
    if (MODE != kP2Apply && fin) P1March<T, NC>::fin_load(P, io, L.i, j, F);
    P1March<T, NC>::compute(P, L, j);
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int d = 0; d < NC; ++d) {
        const T v = shfl_up1(L.A[r][1][d]);
        if (lane > 0) L.A[r][0][d] += v;
      }
    if (fin) P1March<T, NC>::finish(P, io, L, j, j == P.ny - 1 ? 2 : 1, F);
    if (!more) break;
    ++j;
    P1March<T, NC>::advance(L);
    P1March<T, NC>::take(L, N);
    down(1);
  }
}

template <class T, int NC, int MODE, class PP>
__global__ void __launch_bounds__(kRowThreads_) k_p1_smooth(PP P, SmoothBufs<T> B) {
  TOPO_PDL_ENTRY();
  const int a = blockIdx.x * kRowThreads_ + threadIdx.x, b = blockIdx.y;
  if (a > P.nx) return;
  if (MODE == kP2Pre) P1Smooth<T, NC>::pre(a, b, P, B);
  else if (MODE == kP2Res) P1Smooth<T, NC>::res(a, b, P, B);
  else if (MODE == kP2First) P1Smooth<T, NC>::first(a, b, P, B);
  else P1Smooth<T, NC>::post2(a, b, P, B);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads_) k_prolong_add(Transfer X, const T* __restrict__ xc, T* __restrict__ xf) {
  TOPO_PDL_ENTRY();
  const int a = blockIdx.x * kRowThreads_ + threadIdx.x, b = blockIdx.y;
  if (a < X.NXf) TransferKern<T, NC>::node_prolong_add(a, b, X, xc, xf);
}

template <class T, int NC, class PP>
__global__ void __launch_bounds__(kRowThreads) k_p1_apply(PP P, const T* __restrict__ u, T* __restrict__ y) {
  TOPO_PDL_ENTRY();
  const int a = blockIdx.x * kRowThreads + threadIdx.x, b = blockIdx.y;
  if (a <= P.nx) p1_node_apply<T, NC>(a, b, P, u, y);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_p1_diag(P1Params<T, NC> P, T* __restrict__ d) {
  const int a = blockIdx.x * kRowThreads + threadIdx.x, b = blockIdx.y;
  if (a <= P.nx) P1Kern<T, NC>::node_diag(a, b, P, d);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_p1_stencil(P1Params<T, NC> P, T* __restrict__ st) {
  const int a = blockIdx.x * kRowThreads + threadIdx.x, b = blockIdx.y;
  if (a <= P.nx) p1_stencil_node<T, NC>(a, b, P, st + (size_t(b) * (P.nx + 1) + a) * StencilLayout<NC>::stride);
}

template <class T, int NC>
__global__ void __launch_bounds__(kRowThreads) k_restrict(Transfer X, const T* __restrict__ rf, T* __restrict__ bc,
                                                          const T* __restrict__ tf) {
  TOPO_PDL_ENTRY();
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
// the FP64 coefficient masters, Gauss-Jordan (SPD, no pivoting) by ONE warp:
// lane j owns column j in shared memory, so a step needs no block barrier and
// one reciprocal of the pivot.
template <class T, int NC>
__global__ void __launch_bounds__(32) k_coarse_inverse(int nx, int ny, Dir dir, ElemRefs R,
                                                       const double* __restrict__ kK, const double* __restrict__ kM,
                                                       T* __restrict__ inv, int* status) {
  __shared__ double A[kCoarseMaxDofs * kCoarseMaxDofs];
  const int NX = nx + 1, NY = ny + 1, n = NX * NY * NC;
  const int j = threadIdx.x;
  for (int i = j; i < n * n; i += 32) A[i] = 0.0;
  __syncwarp();
  if (j == 0) {
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
  __syncwarp();
  for (int i = j; i < n * n; i += 32) {
    const int r = i / n, c = i % n;
    const int nr = r / NC, nc = c / NC;
    const bool cr = is_clamped(dir, nr % NX, nr / NX), cc = is_clamped(dir, nc % NX, nc / NX);
    if (cr || cc) A[i] = (r == c) ? 1.0 : 0.0;
  }
  __syncwarp();
  int bad = 0;
  for (int k = 0; k < n; ++k) {
    const double p = A[k * n + k];
    if (!(p > 0.0) || !isfinite(p)) {  // the same value in every lane: a uniform exit
      bad = 1;
      break;
    }
    const double ip = 1.0 / p;
    double f[kCoarseMaxDofs];  // column k before this step
#pragma unroll
    for (int i = 0; i < kCoarseMaxDofs; ++i) f[i] = i < n ? A[i * n + k] : 0.0;
    __syncwarp();
    if (j < n) {
      if (j == k) {
#pragma unroll
        for (int i = 0; i < kCoarseMaxDofs; ++i)
          if (i < n) A[i * n + k] = (i == k) ? ip : -f[i] * ip;
      } else {
        const double c = A[k * n + j] * ip;
#pragma unroll
        for (int i = 0; i < kCoarseMaxDofs; ++i)
          if (i < n) A[i * n + j] = (i == k) ? c : A[i * n + j] - f[i] * c;
      }
    }
    __syncwarp();
  }
  for (int i = j; i < n * n; i += 32) {
    const int r = i / n, c = i % n;
    inv[i] = T(0.5 * (A[r * n + c] + A[c * n + r]));
  }
  if (j == 0) *status = bad;
}

template <class T>
__global__ void k_dense_matvec(const T* __restrict__ Ainv, const T* __restrict__ b, T* __restrict__ x, int n) {
  TOPO_PDL_ENTRY();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T s = T(0);
    for (int j = 0; j < n; ++j) s += Ainv[size_t(i) * n + j] * b[j];
    x[i] = s;
  }
}

// ---------------------------------------------------------------------------
// coarse-level tail: the V-cycle over the smallest levels runs in one CTA with
// every work vector, the stencils and D^-1 resident in shared memory (one
// launch instead of ~6 x levels; the phases touch no global memory)
// ---------------------------------------------------------------------------
constexpr int kTailThreads = 1024;
constexpr int kTailMaxLevels = 10;
constexpr size_t kTailSmemBudget = 196 * 1024;
constexpr int kTailTraceSlots = 64;  // [0, 62]: SM cycles per phase, [63]: launches

template <class T, int NC>
struct TailLevel {
  P1Stencil<T, NC> S;
  Transfer X;  // to the next coarser level
  const T* dinv;
  const T* cheb;
  int NX, nn, off;  // off: first of this level's five shared vectors x, b, r, d, x2 (NC*nn each)
  int soff, doff;   // shared copies of the stencil (stride*nn) and of dinv (NC*nn)
};

template <class T, int NC>
struct TailDesc {
  int nlev, smem_elems;
  const T* cinv;
  long long* trace;  // opt-in phase timing (null: off)
  TailLevel<T, NC> lv[kTailMaxLevels];
};

// Copies n values global -> shared with 16-byte accesses (both addresses 16-byte
// aligned), the remainder one by one: the tail's per-launch staging issues a few
// wide loads per thread instead of a long chain of scalar ones.
template <class T>
__device__ __forceinline__ void stage16(T* __restrict__ dst, const T* __restrict__ src, int n, int tid, int nt) {
  constexpr int V = 16 / sizeof(T);
  const int nv = n / V;
  const float4* s4 = reinterpret_cast<const float4*>(src);
  float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll 4
  for (int i = tid; i < nv; i += nt) d4[i] = s4[i];
  for (int i = nv * V + tid; i < n; i += nt) dst[i] = src[i];
}

template <class T, int NC>
__global__ void __launch_bounds__(kTailThreads)
    k_tail_vcycle(const TailDesc<T, NC>* __restrict__ D, const T* __restrict__ b_in, T* __restrict__ x_out) {
  TOPO_PDL_ENTRY();
  __shared__ TailLevel<T, NC> lv[kTailMaxLevels];
  __shared__ __align__(16) T cinv[kCoarseMaxDofs * kCoarseMaxDofs];
  extern __shared__ __align__(16) unsigned char tail_raw[];
  T* sm = reinterpret_cast<T*>(tail_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nlev = D->nlev;
  {
    const int* src = reinterpret_cast<const int*>(D->lv);
    int* dst = reinterpret_cast<int*>(lv);
    const int words = int(sizeof(TailLevel<T, NC>) / sizeof(int)) * nlev;
    for (int i = tid; i < words; i += nt) dst[i] = src[i];
  }
  __syncthreads();
  // (stencil and diagonal offsets are multiples of 16 bytes, every source a separate allocation)
  for (int l = 0; l < nlev; ++l) {
    const TailLevel<T, NC>& L = lv[l];
    stage16(sm + L.soff, L.S.s, StencilLayout<NC>::stride * L.nn, tid, nt);
    stage16(sm + L.doff, L.dinv, NC * L.nn, tid, nt);
  }
  {
    const int mc = NC * lv[nlev - 1].nn;
    stage16(cinv, D->cinv, mc * mc, tid, nt);
    const int m = NC * lv[0].nn;
    T* b0 = sm + lv[0].off + m;  // (inside the level's five vectors: not 16-byte aligned)
    for (int i = tid; i < m; i += nt) b0[i] = b_in[i];
  }
  __syncthreads();
  if (tid == 0)
    for (int l = 0; l < nlev; ++l) {
      lv[l].S.s = sm + lv[l].soff;
      lv[l].dinv = sm + lv[l].doff;
    }
  __syncthreads();
  // opt-in timing: SM cycles of every phase in execution order
  long long* const trace = tid == 0 ? D->trace : nullptr;
  long long t_prev = clock64();
  int slot = 1;
  auto mark = [&]() {
    __syncthreads();
    if (!trace) return;
    const long long t = clock64();
    if (slot < kTailTraceSlots - 1) trace[slot++] += t - t_prev;
    t_prev = t;
  };
  auto bufs = [&](int l) {
    const int m = NC * lv[l].nn;
    T* base = sm + lv[l].off;
    return SmoothBufs<T>{base + m, lv[l].dinv, base, base + 4 * m, base + 2 * m, base + 3 * m, lv[l].cheb};
  };
  for (int l = 0; l + 1 < nlev; ++l) {
    const TailLevel<T, NC>& L = lv[l];
    const SmoothBufs<T> B = bufs(l);
    for (int n = tid; n < L.nn; n += nt) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::pre(a, b, L.S, B);
    }
    mark();
    for (int n = tid; n < L.nn; n += nt) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::res(a, b, L.S, B);
    }
    mark();
    const TailLevel<T, NC>& C = lv[l + 1];
    T* bc = sm + C.off + NC * C.nn;
    for (int n = tid; n < C.nn; n += nt) {
      const int J = n / C.NX, I = n - J * C.NX;
      TransferKern<T, NC>::node_restrict(I, J, L.X, B.r, bc);
    }
    mark();
  }
  {  // coarsest level: dense inverse
    const TailLevel<T, NC>& C = lv[nlev - 1];
    const int m = NC * C.nn;
    const T* bc = sm + C.off + m;
    T* xc = sm + C.off;
    for (int i = tid; i < m; i += nt) {
      T acc = T(0);
#pragma unroll 8
      for (int j = 0; j < m; ++j) acc += cinv[i * m + j] * bc[j];
      xc[i] = acc;
    }
    mark();
  }
  for (int l = nlev - 2; l >= 0; --l) {
    const TailLevel<T, NC>& L = lv[l];
    const SmoothBufs<T> B = bufs(l);
    const T* xc = sm + lv[l + 1].off;
    for (int n = tid; n < L.nn; n += nt) {
      const int b = n / L.NX, a = n - b * L.NX;
      TransferKern<T, NC>::node_prolong_add(a, b, L.X, xc, B.x);
    }
    mark();
    for (int n = tid; n < L.nn; n += nt) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::first(a, b, L.S, B);
    }
    mark();
    for (int n = tid; n < L.nn; n += nt) {
      const int b = n / L.NX, a = n - b * L.NX;
      P1Smooth<T, NC>::post2(a, b, L.S, B);
      if (l == 0)
        for (int c = 0; c < NC; ++c) x_out[NC * n + c] = B.x[NC * n + c];
    }
    mark();
  }
  if (trace) trace[kTailTraceSlots - 1] += 1;
}

template <class T, int NC>
struct CoarseChebDesc {
  P1Stencil<T, NC> S;  // the level's stencil (global memory; staged into shared)
  const T* dinv;
  int NX, nn;
  CoarseCheb<T> C;
};

// The whole Chebyshev solve of a truncated hierarchy's last level in one CTA
// (scalar levels, at most coarse_cheb_npt<T>() nodes per thread).  A
// thread keeps its nodes' stencil rows, inverse diagonal, residual and
// iterate in registers; only the direction, which the neighbours read, goes
// through shared memory (two buffers, one barrier per step).  A neighbour
// outside the lattice has a zero coupling, so its index is only clamped into
// the array.  A step is ~30 instructions per node (the arithmetic of
// CoarseChebNode::step in the stencil's difference form).
// nodes per thread: what the registers of a 1024-thread block hold without spilling
template <class T>
constexpr int coarse_cheb_npt() {
  return sizeof(T) == 4 ? 3 : 2;
}

template <class T>
__global__ void __launch_bounds__(kTailThreads)
    k_coarse_cheb(const CoarseChebDesc<T, 1>* __restrict__ D, const T* __restrict__ b, T* __restrict__ x_out) {
  TOPO_PDL_ENTRY();
  constexpr int NP = coarse_cheb_npt<T>(), SW = StencilLayout<1>::stride;
  extern __shared__ __align__(16) unsigned char cc_raw[];
  T* d0 = reinterpret_cast<T*>(cc_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nn = D->nn, NX = D->NX;
  T* d1 = d0 + nn;
  const CoarseCheb<T>& C = D->C;  // read in place (uniform loads)
  const T* __restrict__ sg = D->S.s;
  T st[NP][7], dv[NP], r[NP], x[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const int n = tid + q * nt;
    const bool on = n < nn;
#pragma unroll
    for (int k = 0; k < 7; ++k) st[q][k] = on ? sg[size_t(n) * SW + k] : T(0);
    dv[q] = on ? D->dinv[n] : T(0);
    r[q] = on ? b[n] : T(0);
    x[q] = T(0);
    if (on) d0[n] = C.c0 * dv[q] * r[q];
  }
  __syncthreads();
  T* dc = d0;
  T* dn = d1;
  const int deg = C.deg;
  for (int k = 0; k + 1 < deg; ++k) {
    const T c1 = C.c1[k], c2 = C.c2[k];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const int n = tid + q * nt;
      if (n < nn) {
        const T dn0 = dc[n];
        T t = st[q][0] * dn0;
#pragma unroll
        for (int e = 1; e < 7; ++e) {
          const int m = min(max(n + st_da(e) + st_db(e) * NX, 0), nn - 1);
          t += st[q][e] * (dc[m] - dn0);
        }
        x[q] += dn0;
        r[q] -= t;
        dn[n] = c1 * dn0 + c2 * dv[q] * r[q];
      }
    }
    __syncthreads();
    T* tmp = dc;
    dc = dn;
    dn = tmp;
  }
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const int n = tid + q * nt;
    if (n < nn) x_out[n] = x[q] + dc[n];
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
inline int device_sms() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 1;
  }
  return cached[dev];
}

// Kernels of the solve chain are launched with programmatic stream
// serialization (they begin with TOPO_PDL_ENTRY): a launch overlaps the
// predecessor's drain instead of following its completion.  TOPO_PDL=0
// launches them plainly.
inline bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("TOPO_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <class... KP, class... A>
inline void launch_pdl(void (*k)(KP...), dim3 g, dim3 b, size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = g;
  cfg.blockDim = b;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

// resident blocks per SM of a march kernel at P2M_THREADS threads (its
// registers decide: the grid is sized to one wave of them)
template <class K>
inline int march_blocks_per_sm(K kernel) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, P2M_THREADS, 0) != cudaSuccess) {
    (void)cudaGetLastError();
    b = 0;
  }
  return b > 0 ? b : 1;
}

template <class T, int MODE>
inline int p2_march_bps() {
  static const int b = march_blocks_per_sm(k_p2_march<T, MODE>);
  return b;
}

template <class T, int NC, int MODE>
inline int p1_march_bps() {
  static const int b = march_blocks_per_sm(k_p1_march<T, NC, MODE>);
  return b;
}

// seg_force > 0: that segment length; else the tuned one for `family` (when tuned), else
// the one-wave rule
inline dim3 march_grid(int nx, int ny, int blocks_per_sm, int& seg, int family = -1, int seg_force = 0) {
  const int tuned = seg_force > 0 ? seg_force : (family >= 0 ? tuned_segment(family, nx, ny) : 0);
  seg = tuned > 0 ? std::min(tuned, ny) : p2_march_segment(nx, ny, device_sms(), blocks_per_sm);
  const int nseg = (ny + seg - 1) / seg;
  return dim3((nx + 1 + P2M_OWN - 1) / P2M_OWN, (nseg + P2M_WARPS - 1) / P2M_WARPS);
}

// occupancy queries happen outside any stream capture
template <class T>
inline void prime_march_occupancy() {
  (void)p2_march_bps<T, kP2Apply>();
  (void)p2_march_bps<T, kP2Diag>();
  (void)p2_march_bps<T, kP2Pre>();
  (void)p2_march_bps<T, kP2Res>();
  (void)p2_march_bps<T, kP2First>();
  (void)p2_march_bps<T, kP2Post2>();
  (void)p1_march_bps<T, 1, kP2Apply>();
  (void)p1_march_bps<T, 1, kP2Pre>();
  (void)p1_march_bps<T, 1, kP2Res>();
  (void)p1_march_bps<T, 1, kP2First>();
  (void)p1_march_bps<T, 1, kP2Post2>();
  (void)p1_march_bps<T, 2, kP2Apply>();
  (void)p1_march_bps<T, 2, kP2Pre>();
  (void)p1_march_bps<T, 2, kP2Res>();
  (void)p1_march_bps<T, 2, kP2First>();
  (void)p1_march_bps<T, 2, kP2Post2>();
}

// Kernel-clock names and algorithmic bytes of one launch (topo_kclock.h).  A mode
// reads and writes whole level vectors: `vecs` of them, each of n values.
inline const char* mode_name(int mode) {
  switch (mode) {
    case kP2Apply: return "Apply";
    case kP2Diag: return "Diag";
    case kP2Pre: return "Pre";
    case kP2Res: return "Res";
    case kP2First: return "First";
    default: return "Post2";
  }
}
template <class T>
inline const char* p2_family(int mode) {
  static const char* f32[6] = {"P2 march FP32 Apply", "P2 march FP32 Diag", "P2 march FP32 Pre",
                               "P2 march FP32 Res", "P2 march FP32 First", "P2 march FP32 Post2"};
  static const char* f64[6] = {"P2 march FP64 Apply", "P2 march FP64 Diag", "P2 march FP64 Pre",
                               "P2 march FP64 Res", "P2 march FP64 First", "P2 march FP64 Post2"};
  return (sizeof(T) == 4 ? f32 : f64)[mode];
}
// vectors of the level a smoothing or operator mode moves: operand(s) read, results written
// (P2: Pre reads b, D^-1 and writes x; First also writes w; Post2 reads d, w, D^-1 (+ b when
// it reduces r.r, r.z); P1 modes keep r between steps)
inline int mode_vectors(int mode, bool p2, bool fused_rz) {
  switch (mode) {
    case kP2Apply: return 2;
    case kP2Diag: return 1;
    case kP2Pre: return 3;
    case kP2Res: return 3;
    case kP2First: return 5;
    default: return p2 ? (fused_rz ? 5 : 4) : 5;
  }
}

template <class T, int MODE>
inline void launch_p2_mode(const P2Params<T>& P, const T* xi, const P2Io<T>& io, cudaStream_t s, int seg_force = 0) {
  int seg = 0;
  const dim3 g = march_grid(P.nx, P.ny, p2_march_bps<T, MODE>(), seg, march_family(true, sizeof(T), 2), seg_force);
  const double n = 2.0 * (2 * P.nx + 1) * (2 * P.ny + 1), nv = double(P.nx + 1) * (P.ny + 1);
  // the design (one value per vertex) plus, for First, the coarse correction (2 per vertex)
  const double bytes = (mode_vectors(MODE, true, io.fuse == kFuseRZ) * n + nv + (MODE == kP2First ? 2 * nv : 0)) *
                       sizeof(T);
  KClock kc(s, p2_family<T>(MODE), 0, bytes);
  launch_pdl(k_p2_march<T, MODE>, g, P2M_THREADS, 0, s, P, xi, io, seg);
}

template <class T>
inline void launch_p2_tile(const P2Params<T>& P, const T* xi, const P2Io<T>& io, cudaStream_t s) {
  switch (io.mode) {
    case kP2Apply: launch_p2_mode<T, kP2Apply>(P, xi, io, s); break;
    case kP2Diag: launch_p2_mode<T, kP2Diag>(P, xi, io, s); break;
    case kP2Pre: launch_p2_mode<T, kP2Pre>(P, xi, io, s); break;
    case kP2Res: launch_p2_mode<T, kP2Res>(P, xi, io, s); break;
    case kP2First: launch_p2_mode<T, kP2First>(P, xi, io, s); break;
    default: launch_p2_mode<T, kP2Post2>(P, xi, io, s); break;
  }
}

template <class T, int NC, int MODE>
inline void launch_p1_mode(const P1Params<T, NC>& P, const P1Io<T>& io, cudaStream_t s, int seg_force = 0) {
  int seg = 0;
  const dim3 g = march_grid(P.nx, P.ny, p1_march_bps<T, NC, MODE>(), seg, march_family(false, sizeof(T), NC), seg_force);
  static const char* fam[6] = {"P1 march Apply", "P1 march Diag", "P1 march Pre", "P1 march Res", "P1 march First",
                               "P1 march Post2"};
  const double n = double(NC) * (P.nx + 1) * (P.ny + 1), ntri = 2.0 * P.nx * P.ny;
  const double bytes = (mode_vectors(MODE, false, false) * n + ntri * ((P.kK ? 1 : 0) + (P.kM ? 1 : 0))) * sizeof(T);
  KClock kc(s, fam[MODE], 1, bytes);
  launch_pdl(k_p1_march<T, NC, MODE>, g, P2M_THREADS, 0, s, P, io, seg);
}

template <class T, int NC>
inline void launch_p1_march(const P1Params<T, NC>& P, const P1Io<T>& io, cudaStream_t s) {
  switch (io.mode) {
    case kP2Apply: launch_p1_mode<T, NC, kP2Apply>(P, io, s); break;
    case kP2Pre: launch_p1_mode<T, NC, kP2Pre>(P, io, s); break;
    case kP2Res: launch_p1_mode<T, NC, kP2Res>(P, io, s); break;
    case kP2First: launch_p1_mode<T, NC, kP2First>(P, io, s); break;
    default: launch_p1_mode<T, NC, kP2Post2>(P, io, s); break;
  }
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

// y = A x with the pair-of-FP32 operator: x, y FP64, P.rmass the mass matrices as
// (hi, lo) pairs (the design is not read)
inline void launch_p2_apply_dd(const P2Params<dd>& P, const double* x, double* y, cudaStream_t s) {
  P2Io<dd> io;
  std::memset(&io, 0, sizeof(io));
  io.mode = kP2Apply;
  io.u = reinterpret_cast<const dd*>(x);
  io.y = reinterpret_cast<dd*>(y);
  int seg = 0;
  const dim3 g = march_grid(P.nx, P.ny, p2_march_bps<dd, kP2Apply>(), seg);
  // x read and y written in FP64, the mass matrices (12 pairs per cell)
  const double n = 2.0 * (2 * P.nx + 1) * (2 * P.ny + 1), nc = double(P.nx) * P.ny;
  KClock kc(s, "P2 march pair-of-FP32 Apply", 0, 2.0 * n * 8.0 + 12.0 * nc * 8.0);
  launch_pdl(k_p2_march<dd, kP2Apply>, g, P2M_THREADS, 0, s, P, static_cast<const dd*>(nullptr), io, seg);
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
// (evaluated once per block: an FP64 division per thread is not free here)
// x in T or FP64 (TX = double: the product of two FP32 numbers is exact in FP64)
// r -= alpha q with alpha = rz / pq; block 0 records the alpha it applied
// (the solution update happens in k_pcg_p, which reads p anyway)
template <class T>
__global__ void k_pcg_r(T* __restrict__ r, const T* __restrict__ q, PcgDev* __restrict__ dv, size_t n) {
  TOPO_PDL_ENTRY();
  __shared__ T alpha_s;
  __shared__ bool ok_s;
  if (threadIdx.x == 0) {
    const double pq = dv->pq;
    ok_s = (pq > 0.0) && isfinite(pq);
    alpha_s = ok_s ? T(dv->rz / pq) : T(0);
    if (blockIdx.x == 0) dv->alpha = double(alpha_s);
  }
  __syncthreads();
  if (!ok_s) return;
  const T alpha = alpha_s;
  TOPO_GRID_STRIDE(i, n) r[i] -= alpha * q[i];
}

// x += alpha p (x in T or FP64: the product of two FP32 numbers is exact in
// FP64), then p = z + beta p
template <class T, class TX>
__global__ void k_pcg_p(T* __restrict__ p, const T* __restrict__ z, TX* __restrict__ x, const PcgDev* __restrict__ dv,
                        size_t n) {
  TOPO_PDL_ENTRY();
  __shared__ T beta_s, alpha_s;
  if (threadIdx.x == 0) {
    beta_s = T(dv->beta);
    alpha_s = T(dv->alpha);
  }
  __syncthreads();
  const T beta = beta_s, alpha = alpha_s;
  TOPO_GRID_STRIDE(i, n) {
    const T pi = p[i];
    x[i] += TX(alpha) * TX(pi);
    p[i] = z[i] + beta * pi;
  }
}

// after the prologue: decide whether the loop runs at all.  On entry dv->tol2
// holds rtol^2 and dv->maxit the iteration cap (both written by the host).
static __global__ void k_pcg_start(PcgDev* dv, cudaGraphConditionalHandle h, int use_cond) {
  TOPO_PDL_ENTRY();
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
  TOPO_PDL_ENTRY();
  pcg_check_dev(dv, h, use_cond);
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
  for (auto e : ev_)
    if (e) cudaEventDestroy(e);
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
  prime_march_occupancy<T>();
  if (const char* e = std::getenv("TOPO_POWER_WARM")) {  // warm-started power-iteration steps
    const int v = std::atoi(e);
    if (v >= 1 && v <= 50) power_iters_warm = v;
  }
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
      if (specs[l].nn() <= stencil_max_nodes(specs[l].NC))
        v.st = arena.alloc_n<T>(specs[l].nn() * (specs[l].NC == 2 ? StencilLayout<2>::stride : StencilLayout<1>::stride));
    }
  }
  const size_t n0 = specs[0].ndof();
  for (int k = 0; k < kScratch; ++k) pcg_[k] = arena.alloc_n<T>(n0);
  if (fp64_solution) xacc_ = arena.alloc_n<double>(n0);
  if (specs[0].p2) pw_ = arena.alloc_n<T>(n0);  // power-iteration vector kept between set-ups
  const int nc = int(specs.back().ndof());
  cinv_ = arena.alloc_n<T>(size_t(nc) * nc);
  cstat_ = arena.alloc_n<int>(1);
  cheb_ = arena.alloc_n<T>(8 * specs.size());
  dev_ = arena.alloc_n<PcgDev>(1);
  if (!hdev_) cudaMallocHost(&hdev_, sizeof(PcgDev));
  for (auto& c : cap_)
    if (!c) cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking);
  for (auto& e : ev_)
    if (!e) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  graph_valid_ = false;
  build_tail(arena);
  cc_buf_ = arena.alloc(sizeof(CoarseChebDesc<T, 1>));
  inner_buf_ = arena.alloc_n<T>(specs.size() * StencilLayout<1>::stride);
}

// Levels with a mass term (the filter), no clamped nodes and the same stencil
// row at every interior node (constant coefficients on the uniform lattice,
// checked on the rows themselves) read that row once instead of per node.
template <class T>
void MG<T>::detect_uniform_levels(cudaStream_t s) {
  const int L = levels();
  for (int l = 0; l < L; ++l) {
    const LevelSpec& S = specs_[l];
    Lev& v = lv_[l];
    v.inner = nullptr;
    if (S.p2 || S.NC != 1 || !v.st || !kM64_[l] || !inner_buf_) continue;
    const Dir& d = S.dir;
    if (d.x_lo || d.y_lo || d.npts || d.x_hi_from < S.NX || d.y_hi_from < S.NY || S.NX < 3 || S.NY < 3) continue;
    constexpr int SW = StencilLayout<1>::stride;
    std::vector<T> st(S.nn() * SW);
    if (cudaMemcpyAsync(st.data(), v.st, st.size() * sizeof(T), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    const T* ref = st.data() + (size_t(1) * S.NX + 1) * SW;
    bool same = true;
    for (int b = 1; same && b + 1 < S.NY; ++b)
      for (int a = 1; same && a + 1 < S.NX; ++a)
        same = std::memcmp(st.data() + (size_t(b) * S.NX + a) * SW, ref, SW * sizeof(T)) == 0;
    if (!same) continue;
    T* dst = inner_buf_ + size_t(l) * SW;
    // on s: the kernels that read the row run there (a pageable copy is staged before
    // the call returns, so `st` may go out of scope)
    if (cudaMemcpyAsync(dst, ref, SW * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    v.inner = dst;
  }
  graph_valid_ = false;
}

// Picks the truncation level (see CoarseCheb): the finest level l >= 1 with a
// scalar assembled stencil that fits one CTA's shared memory and whose Dinv A
// spectrum -- bounded element by element from the coefficient ratios kK/kM
// of the level's triangles -- needs at most coarse_cheb_max_degree steps for
// a residual reduction of 1e-2.  Levels past it are no longer visited.
template <class T>
void MG<T>::select_coarse_cheb(cudaStream_t s) {
  const int prev = cheb_coarse_;
  cheb_coarse_ = -1;
  cc_desc_ = nullptr;
  coarse_cheb_deg = 0;
  const int L = levels();
  for (int l = 1; use_coarse_cheb && cc_buf_ && l < L; ++l) {
    const LevelSpec& S = specs_[l];
    if (S.p2 || S.NC != 1 || !lv_[l].st || !kK64_[l] || !kM64_[l]) continue;
    const size_t smem = 2 * S.nn() * sizeof(T);  // the two direction buffers
    if (S.nn() > size_t(kTailThreads) * coarse_cheb_npt<T>() || smem > kTailSmemBudget) continue;
    const size_t nt = S.ntri();
    std::vector<double> kk(nt), km(nt);
    if (cudaMemcpyAsync(kk.data(), kK64_[l], nt * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(km.data(), kM64_[l], nt * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    double tmin = 1e300, tmax = 0.0;
    bool ok = nt > 0;
    for (size_t t = 0; t < nt && ok; ++t) {
      if (!(km[t] > 0.0) || !(kk[t] >= 0.0) || !std::isfinite(kk[t] / km[t])) ok = false;
      else {
        tmin = std::min(tmin, kk[t] / km[t]);
        tmax = std::max(tmax, kk[t] / km[t]);
      }
    }
    if (!ok) continue;
    double lo, hi;
    const int deg = coarse_cheb_plan(refs_[l], tmin, tmax, 1e-2, lo, hi);
    if (deg > coarse_cheb_max_degree || deg > kCoarseChebMax) continue;
    CoarseChebDesc<T, 1> h;
    std::memset(&h, 0, sizeof(h));
    h.S = P1Stencil<T, 1>{S.nx, S.ny, S.dir, lv_[l].st};
    h.dinv = lv_[l].dinv;
    h.NX = S.NX;
    h.nn = int(S.nn());
    double c0, c1[kCoarseChebMax], c2[kCoarseChebMax];
    coarse_cheb_coefficients(lo, hi, deg, c0, c1, c2);
    h.C.deg = deg;
    h.C.c0 = T(c0);
    for (int k = 0; k + 1 < deg; ++k) {
      h.C.c1[k] = T(c1[k]);
      h.C.c2[k] = T(c2[k]);
    }
    const int limit = int(kTailSmemBudget);
    if (cudaMemcpyAsync(cc_buf_, &h, sizeof(h), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaFuncSetAttribute(k_coarse_cheb<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    cheb_coarse_ = l;
    cc_desc_ = cc_buf_;
    cc_smem_ = smem;
    coarse_cheb_deg = deg;
    break;
  }
  if (cheb_coarse_ != prev) graph_valid_ = false;
}

// Chooses the tail levels (smallest levels whose shared vectors fit the
// budget, never level 0) and uploads their descriptor.
template <class T>
void MG<T>::build_tail(Arena& arena) {
  tail_ = -1;
  tail_desc_ = nullptr;
  tail_smem_ = 0;
  const int L = levels();
  const int stride = specs_[L - 1].NC == 2 ? StencilLayout<2>::stride : StencilLayout<1>::stride;
  size_t bytes = 0;
  int first = L;
  for (int l = L - 1; l >= 1; --l) {
    // five vectors, the inverse diagonal and the stencil
    const size_t add = (6 * specs_[l].ndof() + size_t(stride) * specs_[l].nn()) * sizeof(T);
    if (specs_[l].p2 || !lv_[l].st || bytes + add > kTailSmemBudget || L - l > kTailMaxLevels) break;
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
    constexpr int kAlign = 16 / int(sizeof(T));  // shared offsets in 16-byte units (stage16)
    auto align = [&](int o) { return (o + kAlign - 1) / kAlign * kAlign; };
    for (int k = 0; k < h.nlev; ++k) {
      const int l = first + k;
      TailLevel<T, NC>& d = h.lv[k];
      d.S = P1Stencil<T, NC>{specs_[l].nx, specs_[l].ny, specs_[l].dir, lv_[l].st};
      if (l + 1 < L) d.X = make_transfer(specs_[l], specs_[l + 1]);
      d.dinv = lv_[l].dinv;
      d.cheb = cheb_ + 8 * l;
      d.NX = specs_[l].NX;
      d.nn = int(specs_[l].nn());
      d.off = off;
      off += 5 * NC * d.nn;
    }
    for (int k = 0; k < h.nlev; ++k) {
      TailLevel<T, NC>& d = h.lv[k];
      d.soff = off = align(off);
      off += StencilLayout<NC>::stride * d.nn;
      d.doff = off = align(off);
      off += NC * d.nn;
    }
    h.smem_elems = off;
    h.trace = nullptr;
    if (profile_levels) {
      h.trace = static_cast<long long*>(arena.alloc(kTailTraceSlots * sizeof(long long)));
      if (h.trace) cudaMemset(h.trace, 0, kTailTraceSlots * sizeof(long long));
      tail_trace_ = h.trace;
    }
    void* p = arena.alloc(sizeof(h));
    if (!p) return;
    cudaMemcpy(p, &h, sizeof(h), cudaMemcpyHostToDevice);
    // the limit is a property of the kernel, shared by every context in the
    // process: always the budget, so that no context lowers another's
    const int static_bytes = int(sizeof(TailLevel<T, NC>) * kTailMaxLevels + sizeof(T) * kCoarseMaxDofs * kCoarseMaxDofs);
    const int limit = int(std::min<size_t>(kTailSmemBudget, size_t(227 * 1024 - static_bytes)));
    if (size_t(off) * sizeof(T) > size_t(limit) ||
        cudaFuncSetAttribute(k_tail_vcycle<T, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, limit) != cudaSuccess) {
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
  const Lev& v = lv_[l];
  // stencil operator: x read, y written, the stencil rows (unless one row is shared)
  const double abytes = 2.0 * L.ndof() * sizeof(T) +
                        (v.inner ? 0.0 : double((7 * L.NC * L.NC * sizeof(T) + 15) / 16 * 16) * L.nn());
  KClock kc(s, (v.st && stencils_ready_) ? "P1 stencil Apply" : "P1 march Apply (operator)", l,
            (v.st && stencils_ready_) ? abytes : 0.0);
  if (L.NC == 2) {
    if (v.st && stencils_ready_) {
      launch_pdl(k_p1_apply<T, 2, P1Stencil<T, 2>>, g, kRowThreads, 0, s, P1Stencil<T, 2>{L.nx, L.ny, L.dir, v.st, v.inner}, x, y);
    } else {
      P1Io<T> io;
      std::memset(&io, 0, sizeof(io));
      io.mode = kP2Apply;
      io.u = x;
      io.y = y;
      launch_p1_march<T, 2>(make_p1<T, 2>(L, refs_[l], v.kK, nullptr), io, s);
    }
  } else {
    if (v.st && stencils_ready_) {
      launch_pdl(k_p1_apply<T, 1, P1Stencil<T, 1>>, g, kRowThreads, 0, s, P1Stencil<T, 1>{L.nx, L.ny, L.dir, v.st, v.inner}, x, y);
    } else {
      P1Io<T> io;
      std::memset(&io, 0, sizeof(io));
      io.mode = kP2Apply;
      io.u = x;
      io.y = y;
      launch_p1_march<T, 1>(make_p1<T, 1>(L, refs_[l], v.kK, v.kM), io, s);
    }
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

// Power iteration for lambda_max(D^-1 A) on level l (Rayleigh quotient
// x'Ax / x'Dx).  On the state hierarchy's level 0 the iterate is kept between
// set-ups: consecutive designs differ little, so a warm start needs fewer
// steps.  Normalisation happens on the device; one host read at the end.
template <class T>
double MG<T>::estimate_lmax(int l, cudaStream_t s) {
  const size_t n = specs_[l].ndof();
  const int g = vec_grid(n, sms_);
  Lev& v = lv_[l];
  const bool keep = (l == 0 && pw_);
  T* x = keep ? pw_ : v.r;
  T* y = v.d;
  const bool warm = keep && pw_ready_;
  const int iters = warm ? power_iters_warm : power_iters;
  if (!warm) {
    k_power_start<T><<<g, kVecThreads, 0, s>>>(x, n);
    launches += 1;
  }
  for (int it = 0; it < iters; ++it) {
    apply(l, x, y, s);
    k_mul<T><<<g, kVecThreads, 0, s>>>(x, v.dinv, y, n);
    launches += 1;
    if (it % 4 == 3 || it + 1 == iters) {  // rescale to unit length (on the device)
      k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(x, x, n, red_->partials, red_->counter, red_->out);
      k_scale_unit<T><<<g, kVecThreads, 0, s>>>(x, red_->out, n);
      launches += 2;
    }
  }
  apply(l, x, y, s);
  k_mul<T><<<g, kVecThreads, 0, s>>>(v.t, v.diag, x, n);
  k_dot2<T><<<red_->blocks, kVecThreads, 0, s>>>(x, y, x, v.t, n, red_->partials, red_->counter, red_->out);
  launches += 2;
  cudaMemcpyAsync(red_->host, red_->out, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const double num = red_->host[0], den = red_->host[1];
  double lam = (den > 0) ? num / den : 4.0;
  const bool ok = std::isfinite(lam) && lam > 0;
  if (!ok) lam = 4.0;
  if (keep) pw_ready_ = ok;  // a failed estimate restarts from the fixed start vector
  return lam;
}

template <class T>
int MG<T>::setup(cudaStream_t s) {
  const int L = levels();
  auto t_last = std::chrono::steady_clock::now();
  auto mark = [&](const char* what) {  // trace_setup: synchronised phase times
    if (!trace_setup) return;
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[topo setup] %-22s %.3f ms\n", what, std::chrono::duration<double, std::milli>(now - t_last).count());
    t_last = now;
  };
  mark("(queued before)");
  // Three independent chains once the coefficient masters (written on s) are
  // ready: level 0's diagonal and eigenvalue estimate on s (the only user of
  // the shared reduction scratch); the P1 levels' coefficients, stencils and
  // diagonals on one owned stream; the coarsest inverse (one warp, long
  // latency) on the other.  s waits for both before it reads levels >= 1.
  cudaStream_t side = cap_[1], side2 = cap_[0];
  cudaEventRecord(ev_[0], s);
  cudaStreamWaitEvent(side, ev_[0], 0);
  cudaStreamWaitEvent(side2, ev_[0], 0);
  auto prep = [&](int l, cudaStream_t q) {
    const LevelSpec& S = specs_[l];
    Lev& v = lv_[l];
    if (!S.p2) {
      const int g = vec_grid(S.ntri(), sms_);
      k_convert<T, double><<<g, kVecThreads, 0, q>>>(v.kK, kK64_[l], 1.0, S.ntri());
      if (v.kM) k_convert<T, double><<<g, kVecThreads, 0, q>>>(v.kM, kM64_[l], 1.0, S.ntri());
      launches += v.kM ? 2 : 1;
      if (v.st) {
        const dim3 gr = row_grid(S.NX, S.NY);
        if (S.NC == 2) k_p1_stencil<T, 2><<<gr, kRowThreads, 0, q>>>(make_p1<T, 2>(S, refs_[l], v.kK, nullptr), v.st);
        else k_p1_stencil<T, 1><<<gr, kRowThreads, 0, q>>>(make_p1<T, 1>(S, refs_[l], v.kK, v.kM), v.st);
        launches += 1;
      }
    }
    stencils_ready_ = true;  // the operator of level l is chosen at launch time
    const size_t n = S.ndof();
    diag_of(l, v.diag, q);
    k_inverse<T><<<vec_grid(n, sms_), kVecThreads, 0, q>>>(v.dinv, v.diag, n);
    launches += 1;
  };
  const LevelSpec& C = specs_[L - 1];
  if (C.NC == 2)
    k_coarse_inverse<T, 2><<<1, 32, 0, side2>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], nullptr, cinv_, cstat_);
  else
    k_coarse_inverse<T, 1><<<1, 32, 0, side2>>>(C.nx, C.ny, C.dir, refs_[L - 1], kK64_[L - 1], kM64_[L - 1], cinv_,
                                                cstat_);
  launches += 1;
  cudaEventRecord(ev_[2], side2);
  for (int l = 1; l < L; ++l) prep(l, side);
  cudaEventRecord(ev_[1], side);
  prep(0, s);
  mark("level 0 diagonal");
  std::vector<double> cc(8 * L, 0.0);
  auto bounds = [&](int l) {
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
  };
  if (L > 1) bounds(0);
  mark("level 0 eigenvalue bound");
  cudaStreamWaitEvent(s, ev_[1], 0);
  if (!cc_selected_) {  // the coefficients of a hierarchy with a mass term do not change
    cudaStreamSynchronize(s);
    select_coarse_cheb(s);
    detect_uniform_levels(s);
    cc_selected_ = true;
  }
  for (int l = 1; l + 1 < L; ++l) bounds(l);
  mark("levels >= 1 (side stream)");
  // stored in the levels' precision: the kernels use them without conversion
  // (an FP64 load and convert per node costs FP64-pipe time on this GPU)
  cheb_host_.assign(cc.begin(), cc.end());
  cudaMemcpyAsync(cheb_, cheb_host_.data(), cheb_host_.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  cudaStreamWaitEvent(s, ev_[2], 0);
  int st = 0;
  cudaMemcpyAsync(&st, cstat_, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  mark("coarse inverse");
  if (e != cudaSuccess) return -5;
  if (st) return -2;
  tune_marches(s);
  return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -5;
}

// One V-cycle from level l down: fused degree-2 Chebyshev pre-smoothing from
// x = 0, residual restriction, coarse correction, fused post-smoothing.
template <class T>
void MG<T>::tail_profile(std::vector<long long>& cycles) const {
  cycles.clear();
  if (!tail_trace_) return;
  cycles.resize(kTailTraceSlots);
  cudaMemcpy(cycles.data(), tail_trace_, kTailTraceSlots * sizeof(long long), cudaMemcpyDeviceToHost);
}

template <class T>
void MG<T>::flush_level_profile() {
  if (prof_events_.empty()) return;
  cudaDeviceSynchronize();
  if (level_ms.size() < specs_.size()) {
    level_ms.assign(specs_.size(), 0.0);
    level_calls.assign(specs_.size(), 0);
  }
  for (auto& pe : prof_events_) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pe.second.first, pe.second.second);
    level_ms[pe.first] += ms;
    level_calls[pe.first] += 1;
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  prof_events_.clear();
}

template <class T>
void MG<T>::vcycle_level(int l, const T* b, T* x, cudaStream_t s) {
  if (profile_levels && !use_graphs) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    prof_depth_ += 1;
    vcycle_level_body(l, b, x, s);
    prof_depth_ -= 1;
    cudaEventRecord(e1, s);
    prof_events_.push_back({l, {e0, e1}});
    if (prof_events_.size() > 4096) flush_level_profile();
    return;
  }
  vcycle_level_body(l, b, x, s);
}

template <class T>
void MG<T>::vcycle_level_body(int l, const T* b, T* x, cudaStream_t s) {
  Lev& v = lv_[l];
  const int L = levels();
  const LevelSpec& S = specs_[l];
  if (l == cheb_coarse_ && cc_desc_) {
    KClock kc(s, "coarse Chebyshev (one CTA)", l, 0.0);
    launch_pdl(k_coarse_cheb<T>, 1, kTailThreads, cc_smem_, s, static_cast<const CoarseChebDesc<T, 1>*>(cc_desc_), b, x);
    ++launches;
    return;
  }
  if (l == tail_ && tail_desc_ && use_tail) {
    KClock kc(s, "tail V-cycle (one CTA)", l, 0.0);
    if (S.NC == 2)
      launch_pdl(k_tail_vcycle<T, 2>, 1, kTailThreads, tail_smem_, s, static_cast<const TailDesc<T, 2>*>(tail_desc_), b, x);
    else
      launch_pdl(k_tail_vcycle<T, 1>, 1, kTailThreads, tail_smem_, s, static_cast<const TailDesc<T, 1>*>(tail_desc_), b, x);
    ++launches;
    return;
  }
  if (l == L - 1) {
    launch_pdl(k_dense_matvec<T>, 1, 256, 0, s, static_cast<const T*>(cinv_), b, x, int(S.ndof()));
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
    {
      KClock kc(s, "restriction", l, 2.0 * (double(S.nn()) + double(X.NXc) * X.NYc) * sizeof(T));
      launch_pdl(k_restrict<T, 2>, gc, kRowThreads, 0, s, X, static_cast<const T*>(v.r), c.b, static_cast<const T*>(nullptr));
    }
    launches += 3;
    vcycle_level(l + 1, c.b, c.x, s);
    io.mode = kP2First;  // adds the prolonged coarse correction to its operand on the fly
    io.xc = c.x;
    launch_p2_tile<T>(p2_, xi_, io, s);
    io.mode = kP2Post2;
    if (l == 0 && fuse_rz_) {  // the CG's r.r, r.z and test (see pcg_body)
      io.fuse = kFuseRZ;
      io.partials = red_->partials;
      io.counter = red_->counter;
      io.pcg = dev_;
      io.cond = fuse_cond_;
      io.use_cond = fuse_use_cond_;
    }
    launch_p2_tile<T>(p2_, xi_, io, s);
    launches += 2;
    return;
  }
  // the level's operator: assembled stencil when there is one, else on the fly
  // algorithmic bytes of the transfers and of a smoothing step on a stencil level
  const double nf = double(S.nn()) * S.NC, ncrs = double(X.NXc) * X.NYc * S.NC;
  const double rbytes = (nf + ncrs) * sizeof(T), pbytes = (2 * nf + ncrs) * sizeof(T);
  auto sbytes = [&](int mode) {
    // the assembled stencil row of every node (7 NC x NC blocks, padded to 16 bytes), unless
    // the level shares one interior row
    const double row = double((7 * S.NC * S.NC * sizeof(T) + 15) / 16 * 16);
    return mode_vectors(mode, false, false) * nf * sizeof(T) + (v.inner ? 0.0 : row * double(S.nn()));
  };
  auto run = [&](auto nc_tag, const auto& P) {
    constexpr int NC = decltype(nc_tag)::value;
    using PP = std::decay_t<decltype(P)>;
    constexpr bool ST = std::is_same<PP, P1Stencil<T, NC>>::value;
    const char* fam_pre = ST ? "P1 stencil Pre" : "P1 node Pre";
    const char* fam_res = ST ? "P1 stencil Res" : "P1 node Res";
    const char* fam_first = ST ? "P1 stencil First" : "P1 node First";
    const char* fam_post = ST ? "P1 stencil Post2" : "P1 node Post2";
    { KClock kc(s, fam_pre, l, sbytes(kP2Pre)); launch_pdl(k_p1_smooth<T, NC, kP2Pre, PP>, gf, kRowThreads, 0, s, P, B); }
    { KClock kc(s, fam_res, l, sbytes(kP2Res)); launch_pdl(k_p1_smooth<T, NC, kP2Res, PP>, gf, kRowThreads, 0, s, P, B); }
    {
      KClock kc(s, "restriction", l, rbytes);
      launch_pdl(k_restrict<T, NC>, gc, kRowThreads, 0, s, X, static_cast<const T*>(v.r), c.b, static_cast<const T*>(nullptr));
    }
    launches += 3;
    vcycle_level(l + 1, c.b, c.x, s);
    { KClock kc(s, "prolongation", l, pbytes); launch_pdl(k_prolong_add<T, NC>, gf, kRowThreads, 0, s, X, static_cast<const T*>(c.x), x); }
    { KClock kc(s, fam_first, l, sbytes(kP2First)); launch_pdl(k_p1_smooth<T, NC, kP2First, PP>, gf, kRowThreads, 0, s, P, B); }
    { KClock kc(s, fam_post, l, sbytes(kP2Post2)); launch_pdl(k_p1_smooth<T, NC, kP2Post2, PP>, gf, kRowThreads, 0, s, P, B); }
    launches += 3;
  };
  // large levels without a stencil: the column march (element products per cell)
  auto run_march = [&](auto nc_tag, const auto& P) {
    constexpr int NC = decltype(nc_tag)::value;
    P1Io<T> io;
    std::memset(&io, 0, sizeof(io));
    io.B = B;
    io.u = x;
    io.mode = kP2Pre;
    launch_p1_march<T, NC>(P, io, s);
    io.mode = kP2Res;
    launch_p1_march<T, NC>(P, io, s);
    {
      KClock kc(s, "restriction", l, rbytes);
      launch_pdl(k_restrict<T, NC>, gc, kRowThreads, 0, s, X, static_cast<const T*>(v.r), c.b, static_cast<const T*>(nullptr));
    }
    launches += 3;
    vcycle_level(l + 1, c.b, c.x, s);
    { KClock kc(s, "prolongation", l, pbytes); launch_pdl(k_prolong_add<T, NC>, gf, kRowThreads, 0, s, X, static_cast<const T*>(c.x), x); }
    io.mode = kP2First;
    launch_p1_march<T, NC>(P, io, s);
    io.mode = kP2Post2;
    launch_p1_march<T, NC>(P, io, s);
    launches += 3;
  };
  using I2 = std::integral_constant<int, 2>;
  using I1 = std::integral_constant<int, 1>;
  const bool march = !v.st && use_p1_march;
  if (S.NC == 2) {
    if (v.st) run(I2{}, P1Stencil<T, 2>{S.nx, S.ny, S.dir, v.st, v.inner});
    else if (march) run_march(I2{}, make_p1<T, 2>(S, refs_[l], v.kK, nullptr));
    else run(I2{}, make_p1<T, 2>(S, refs_[l], v.kK, nullptr));
  } else {
    if (v.st) run(I1{}, P1Stencil<T, 1>{S.nx, S.ny, S.dir, v.st, v.inner});
    else if (march) run_march(I1{}, make_p1<T, 1>(S, refs_[l], v.kK, v.kM));
    else run(I1{}, make_p1<T, 1>(S, refs_[l], v.kK, v.kM));
  }
}

template <class T>
void MG<T>::vcycle(const T* b, T* x, cudaStream_t s) {
  vcycle_level(0, b, x, s);
}

// Autotuner of the column-march kernels' tile, the cell rows one warp marches:
// candidate segment lengths are timed on the Apply mode with CUDA events (R
// launches back to back per sample, best of two samples: the events resolve
// about 2 us) and the one-wave rule of p2_march_segment is kept unless a
// candidate is more than 5 % faster.  Once per kernel family and grid in the
// process, after set-up and before the first graph recording (graphs keep the
// segment they were recorded with).  Every segment length gives the same node
// values; only the grid, and with it the fused reductions' block partials, changes,
// so two processes may round a CG scalar differently (TOPO_AUTOTUNE=0 keeps the
// one-wave rule and with it bitwise reproducible runs).
template <class T>
void MG<T>::tune_marches(cudaStream_t s) {
  if (!autotune || !autotune_enabled()) return;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess) return;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return;
  }
  constexpr int R = 6;
  auto time_it = [&](const auto& launch) -> float {
    float best = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      launch();  // warm
      cudaEventRecord(e0, s);
      for (int k = 0; k < R; ++k) launch();
      cudaEventRecord(e1, s);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return 1e30f;
      best = std::min(best, ms / R);
    }
    return best;
  };
  // max_blocks > 0: a candidate whose grid exceeds it is skipped
  auto choose = [&](int family, int nx, int ny, int blocks_per_sm, size_t max_blocks, const auto& launch_with) {
    if (tuned_segment(family, nx, ny) > 0) return;
    // one tuner per key: a context set up concurrently for the same grid waits here and
    // then uses the same segment, so all contexts of a grid in the process agree
    std::lock_guard<std::recursive_mutex> lock(device_lock());
    if (tuned_segment(family, nx, ny) > 0) return;
    const int heur = p2_march_segment(nx, ny, device_sms(), blocks_per_sm);
    const float t_heur = time_it([&] { launch_with(heur); });
    int best = heur;
    float t_best = t_heur;
    for (int c : {1, 2, 3, 4, 6, 8, 12}) {
      if (c == heur || c > ny) continue;
      int sg = 0;
      const dim3 g = march_grid(nx, ny, blocks_per_sm, sg, -1, c);
      if (max_blocks && size_t(g.x) * g.y > max_blocks) continue;
      const float t = time_it([&] { launch_with(c); });
      if (t < t_best) {
        t_best = t;
        best = c;
      }
    }
    set_tuned_segment(family, nx, ny, t_best < 0.95f * t_heur ? best : heur);
  };
  const int L = levels();
  for (int l = 0; l < L; ++l) {
    const LevelSpec& S = specs_[l];
    Lev& v = lv_[l];
    if (l == tail_ && tail_desc_ && use_tail) break;  // the tail runs the rest
    if (l == cheb_coarse_ && cc_desc_) break;
    if (S.p2) {
      const size_t n = S.ndof();
      T *x = pcg_[8], *y = pcg_[9];
      cudaMemsetAsync(x, 0, n * sizeof(T), s);
      P2Io<T> io;
      std::memset(&io, 0, sizeof(io));
      io.mode = kP2Apply;
      io.u = x;
      io.y = y;
      // the fused CG reductions keep 2 partials per block in red_->blocks * 16 slots
      const size_t max_blocks = red_ ? size_t(red_->blocks) * 8 : 0;
      choose(march_family(true, sizeof(T), 2), S.nx, S.ny, p2_march_bps<T, kP2Apply>(), max_blocks,
             [&](int seg) { launch_p2_mode<T, kP2Apply>(p2_op_, xi_, io, s, seg); });
    } else if (!v.st && use_p1_march && l + 1 < L) {
      cudaMemsetAsync(v.x, 0, S.ndof() * sizeof(T), s);
      P1Io<T> io;
      std::memset(&io, 0, sizeof(io));
      io.mode = kP2Apply;
      io.u = v.x;
      io.y = v.t;
      if (S.NC == 2) {
        const auto P = make_p1<T, 2>(S, refs_[l], v.kK, nullptr);
        choose(march_family(false, sizeof(T), 2), S.nx, S.ny, p1_march_bps<T, 2, kP2Apply>(), 0,
               [&](int seg) { launch_p1_mode<T, 2, kP2Apply>(P, io, s, seg); });
      } else {
        const auto P = make_p1<T, 1>(S, refs_[l], v.kK, v.kM);
        choose(march_family(false, sizeof(T), 1), S.nx, S.ny, p1_march_bps<T, 1, kP2Apply>(), 0,
               [&](int seg) { launch_p1_mode<T, 1, kP2Apply>(P, io, s, seg); });
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
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
    // the FP64 solution starts exactly at the guess the residual belongs to
    if (xacc_) k_convert<double, T><<<g, kVecThreads, 0, s>>>(xacc_, xi, 1.0, n);
  } else {
    k_fill<T><<<g, kVecThreads, 0, s>>>(xi, T(0), n);
    if (xacc_) k_fill<double><<<g, kVecThreads, 0, s>>>(xacc_, 0.0, n);
    cudaMemcpyAsync(r, bi, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  }
  if (xacc_) launches += 1;
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(bi, bi, n, red_->partials, red_->counter, &dev_->bb);
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(r, r, n, red_->partials, red_->counter, &dev_->rr);
  vcycle(r, z, s);
  k_dot<T, T><<<red_->blocks, kVecThreads, 0, s>>>(r, z, n, red_->partials, red_->counter, &dev_->rz);
  cudaMemcpyAsync(p, z, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  launches += 5;
}

template <class T>
void MG<T>::pcg_xr(int g, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  T *r = pcg_[0], *q = pcg_[3];
  KClock kc(s, "CG r -= alpha q", 0, 3.0 * n * sizeof(T));
  launch_pdl(k_pcg_r<T>, g, kVecThreads, 0, s, r, static_cast<const T*>(q), dev_, n);
}

template <class T>
void MG<T>::pcg_p(int g, cudaStream_t s) {
  const size_t n = specs_[0].ndof();
  T *z = pcg_[1], *p = pcg_[2], *xi = pcg_[6];
  const PcgDev* dv = dev_;
  // p read and written, z read, x (FP64 when accumulated so) read and written
  KClock kc(s, "CG x += alpha p, p = z + beta p", 0, n * (3.0 * sizeof(T) + 2.0 * (xacc_ ? 8 : sizeof(T))));
  if (xacc_) launch_pdl(k_pcg_p<T, double>, g, kVecThreads, 0, s, p, static_cast<const T*>(z), xacc_, dv, n);
  else launch_pdl(k_pcg_p<T, T>, g, kVecThreads, 0, s, p, static_cast<const T*>(z), xi, dv, n);
}

template <class T>
void MG<T>::pcg_body(cudaStream_t s, cudaGraphConditionalHandle h, int use_cond) {
  const size_t n = specs_[0].ndof();
  const int g = vec_grid(n, sms_);
  T *r = pcg_[0], *z = pcg_[1], *p = pcg_[2], *q = pcg_[3];
  // both fused launches (operator and last post-smoothing) must fit the partial slots
  int seg = 0;
  const int fam = march_family(true, sizeof(T), 2);
  const dim3 ga = march_grid(specs_[0].nx, specs_[0].ny, p2_march_bps<T, kP2Apply>(), seg, fam);
  const dim3 gp = march_grid(specs_[0].nx, specs_[0].ny, p2_march_bps<T, kP2Post2>(), seg, fam);
  const size_t mblocks = std::max(size_t(ga.x) * ga.y, size_t(gp.x) * gp.y);
  if (specs_[0].p2 && mblocks * 2 <= size_t(red_->blocks) * 16) {
    // P2 level 0: p.q is reduced inside the operator launch, r.r / r.z and the
    // iteration's test inside the V-cycle's last post-smoothing launch
    P2Io<T> io;
    std::memset(&io, 0, sizeof(io));
    io.mode = kP2Apply;
    io.u = p;
    io.y = q;
    io.fuse = kFusePQ;
    io.partials = red_->partials;
    io.counter = red_->counter;
    io.pcg = dev_;
    launch_p2_tile<T>(p2_op_, xi_, io, s);
    pcg_xr(g, s);
    fuse_rz_ = true;
    fuse_cond_ = (unsigned long long)h;
    fuse_use_cond_ = use_cond;
    vcycle(r, z, s);
    fuse_rz_ = false;
    pcg_p(g, s);
    launches += 3;
    return;
  }
  apply(0, p, q, s, true);
  {
    KClock kc(s, "CG dot p.q", 0, 2.0 * n * sizeof(T));
    launch_pdl(k_dot<T, T>, red_->blocks, kVecThreads, 0, s, static_cast<const T*>(p), static_cast<const T*>(q), n,
               red_->partials, red_->counter, &dev_->pq);
  }
  pcg_xr(g, s);
  vcycle(r, z, s);
  {
    KClock kc(s, "CG dots r.r, r.z", 0, 2.0 * n * sizeof(T));
    launch_pdl(k_dot2<T>, red_->blocks, kVecThreads, 0, s, static_cast<const T*>(r), static_cast<const T*>(r),
               static_cast<const T*>(r), static_cast<const T*>(z), n, red_->partials, red_->counter, &dev_->rr);
  }
  launch_pdl(k_pcg_check, 1, 1, 0, s, dev_, h, use_cond);
  pcg_p(g, s);
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
  std::lock_guard<std::recursive_mutex> lock(device_lock());
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
int MG<T>::graph_pcg(const T* b, T* x, double* x64, bool warm, double rtol, int maxit, SolveStats& st,
                     cudaStream_t s) {
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
    if (capture_pcg(warm) != 0) {
      // a recording can fail when another thread's work synchronises the device
      // meanwhile (first use of a kernel, a free); this solve then runs the same
      // kernels from the host and the next one records again
      cudaGetLastError();
      ++capture_failures;
    }
  }
  const bool graphs = use_graphs && G.exec;
  hdev_->tol2 = rtol * rtol;
  hdev_->maxit = maxit;
  cudaMemcpyAsync(bi, b, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  if (warm) {
    if (x64) k_convert<T, double><<<vec_grid(n, sms_), kVecThreads, 0, s>>>(xi, x64, 1.0, n);
    else cudaMemcpyAsync(xi, x, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  }
  cudaMemcpyAsync(&dev_->tol2, &hdev_->tol2, sizeof(double), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(&dev_->maxit, &hdev_->maxit, sizeof(int), cudaMemcpyHostToDevice, s);
  if (graphs) {
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
  if (x64) cudaMemcpyAsync(x64, xacc_, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  else cudaMemcpyAsync(x, xi, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(hdev_, dev_, sizeof(PcgDev), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return -5;
  st.iterations = hdev_->it;
  st.relres = hdev_->relres;
  if (graphs) launches += (long long)hdev_->it * G.body_nodes;
  switch (hdev_->status) {
    case 0: return 0;
    case 5:
      if (x64) k_fill<double><<<vec_grid(n, sms_), kVecThreads, 0, s>>>(x64, 0.0, n);
      else k_fill<T><<<vec_grid(n, sms_), kVecThreads, 0, s>>>(x, T(0), n);
      return 0;
    case 4: return -4;
    case 3: return -3;  // breakdown: caller falls back
    default: return -2;
  }
}

template <class T>
int MG<T>::pcg(const T* b, T* x, bool x_nonzero, double rtol, int maxit, SolveStats& st, cudaStream_t s) {
  st = SolveStats{};
  int rc = graph_pcg(b, x, nullptr, x_nonzero, rtol, maxit, st, s);
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

template <class T>
int MG<T>::pcg_x64(const T* b, double* x64, bool x_nonzero, double rtol, int maxit, SolveStats& st,
                   cudaStream_t s) {
  st = SolveStats{};
  if (!xacc_) return -5;
  int rc = graph_pcg(b, nullptr, x64, x_nonzero, rtol, maxit, st, s);
  if (rc == -3) {
    // MINRES continues in T from the iterate rounded to T (pcg_[9]: neither
    // MINRES's work vectors nor the callers' scratch0(4))
    const size_t n = specs_[0].ndof();
    const int g = vec_grid(n, sms_);
    T* xt = pcg_[9];
    k_convert<T, double><<<g, kVecThreads, 0, s>>>(xt, x64, 1.0, n);
    SolveStats ms;
    rc = minres(b, xt, rtol, std::max(1, maxit - st.iterations), ms, s);
    k_convert<double, T><<<g, kVecThreads, 0, s>>>(x64, xt, 1.0, n);
    launches += 2;
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
