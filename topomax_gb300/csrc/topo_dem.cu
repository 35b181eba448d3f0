// Deep-energy-method strain energy on the structured quadrilateral mesh.
//
// Restates the FP32 arithmetic of DEM_src/objective_calculator.py:19-125
// (2x2 Gauss rule on bilinear cells, shape-derivative table, gradient
// accumulated node by node) and DEM_src/elasisity_problem.py:79-129
// (sigma:eps, SIMP r(rho), energy and objective/gradient), operation by
// operation: every per-cell float32 value (sigma:eps, r, r', the objective's
// per-cell gradient) is rounded exactly as the torch expressions round it
// (no contraction into FMAs).  The sums over cells run in FP64 with a
// deterministic grid reduction (the reference's torch.sum order is its own).
// The external work (traction and body-force integrals) is linear in u; the
// host passes it as per-node weights.  The backward kernel (d psi / d u) is
// node-centric: every node gathers the contributions of its <= 4 cells.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "topo_mg.h"
#include "topo_vec.cuh"
#include "topomax_gb300.h"

using namespace topo;

struct topo_dem_ctx {
  topo_dem_desc d{};
  double p = -1.0;
  bool penal_set = false;
  float* wext = nullptr;    // [nn][2] external work weights (device) or null
  float* mask = nullptr;    // [nn][2] Dirichlet mask (device) or null
  double* partials = nullptr;
  unsigned* counter = nullptr;
  int blocks = 0;
  int sms = 1;
  std::string err;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_check(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TOPO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return TOPO_OK;
  }
  ~topo_dem_ctx() {
    std::lock_guard<std::recursive_mutex> lock(device_lock());
    cudaFree(wext);
    cudaFree(mask);
    cudaFree(partials);
    cudaFree(counter);
  }
};

namespace {

constexpr int kDemThreads = 256;

// Per-launch constants (float32 as the reference rounds them).
struct DemK {
  int nx, ny;
  float D[4][4][2];  // [node][gauss point][x, y]
  float detJ, lam, two_mu;
  float m, onem;     // SIMP minimum 1e-6 and 1 - 1e-6 (float32)
  float p, pm1;      // exponent, exponent - 1
  int ip, ipm1;      // exponents 2 or 3 (torch evaluates x*x / x*x*x), else 0 (pow)
};

// rho ** q as torch's CPU kernel evaluates a float32 tensor to a scalar power
__device__ __forceinline__ float pow_torch(float x, int iq, float q) {
  if (iq == 2) return __fmul_rn(x, x);
  if (iq == 3) return __fmul_rn(__fmul_rn(x, x), x);
  if (iq == 1) return x;
  return powf(x, q);
}

// penalizer(rho) = m + rho**p * (1 - m)      (src/penalizers.py:36-40)
__device__ __forceinline__ float simp_r(const DemK& K, float rho) {
  return __fadd_rn(K.m, __fmul_rn(pow_torch(rho, K.ip, K.p), K.onem));
}
// penalizer.derivative(rho) = p * rho**(p-1) * (1 - m)   (src/penalizers.py:42-46)
__device__ __forceinline__ float simp_dr(const DemK& K, float rho) {
  return __fmul_rn(__fmul_rn(K.p, pow_torch(rho, K.ipm1, K.pm1)), K.onem);
}

// Corner displacements of cell (ix, iy), node order of get_gauss_points.
template <bool MASK>
__device__ __forceinline__ void load_cell(const DemK& K, const float* __restrict__ u, const float* __restrict__ mask,
                                          int ix, int iy, float (&U)[4][2]) {
  const int NY = K.ny + 1;
  const size_t n[4] = {size_t(ix) * NY + iy, size_t(ix) * NY + iy + 1, size_t(ix + 1) * NY + iy,
                       size_t(ix + 1) * NY + iy + 1};
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      float v = u[2 * n[i] + j];
      if (MASK) v = __fmul_rn(v, mask[2 * n[i] + j]);
      U[i][j] = v;
    }
}

// displacement gradient at Gauss point g: grad[j][k] = sum_i U[i][j] * D[i][g][k],
// accumulated over i in order (ObjectiveCalculator.get_grad_u)
__device__ __forceinline__ void grad_at(const DemK& K, const float (&U)[4][2], int g, float (&G)[2][2]) {
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float acc = __fmul_rn(U[0][j], K.D[0][g][k]);
#pragma unroll
      for (int i = 1; i < 4; ++i) acc = __fadd_rn(acc, __fmul_rn(U[i][j], K.D[i][g][k]));
      G[j][k] = acc;
    }
}

// sigma from the gradient (StrainEnergy.calculate_strain_energy); eps returned too
__device__ __forceinline__ void stress(const DemK& K, const float (&G)[2][2], float (&S)[2][2], float (&E)[2][2]) {
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int k = 0; k < 2; ++k) E[j][k] = __fmul_rn(0.5f, __fadd_rn(G[j][k], G[k][j]));
  const float ldiv = __fmul_rn(K.lam, __fadd_rn(G[0][0], G[1][1]));
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int k = 0; k < 2; ++k) S[j][k] = __fadd_rn(__fmul_rn(ldiv, j == k ? 1.0f : 0.0f), __fmul_rn(K.two_mu, E[j][k]));
}

// sum over the 4 Gauss points of sigma:eps (components summed (0,0),(0,1),(1,0),(1,1))
__device__ __forceinline__ float cell_strain_energy(const DemK& K, const float (&U)[4][2]) {
  float se = 0.0f;
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    float G[2][2], S[2][2], E[2][2];
    grad_at(K, U, g, G);
    stress(K, G, S, E);
    float s = __fmul_rn(S[0][0], E[0][0]);
    s = __fadd_rn(s, __fmul_rn(S[0][1], E[0][1]));
    s = __fadd_rn(s, __fmul_rn(S[1][0], E[1][0]));
    s = __fadd_rn(s, __fmul_rn(S[1][1], E[1][1]));
    se = g == 0 ? s : __fadd_rn(se, s);
  }
  return se;
}

enum DemMode { kDemEnergy = 0, kDemObjective = 1, kDemDensityGrad = 2 };

// One pass over the cells (and, for the energy, over the nodes for the external
// work).  kDemEnergy: out = 0.5 * sum r*SE*detJ - sum w.u ;  kDemObjective:
// out = sum r*(SE*detJ), cellv = -r' * (SE*detJ) ;  kDemDensityGrad:
// cellv = scale * 0.5 * r' * SE * detJ.
template <int MODE, bool MASK>
__global__ void __launch_bounds__(kDemThreads)
    k_dem_cells(DemK K, const float* __restrict__ u, const float* __restrict__ mask, const float* __restrict__ rho,
                const float* __restrict__ wext, const float* __restrict__ scale, float* __restrict__ cellv,
                double* partials, unsigned* counter, double* out) {
  const size_t ncell = size_t(K.nx) * K.ny;
  double acc = 0.0;
  const float sc = (MODE == kDemDensityGrad) ? *scale : 0.0f;
  for (size_t c = size_t(blockIdx.x) * blockDim.x + threadIdx.x; c < ncell; c += size_t(gridDim.x) * blockDim.x) {
    const int iy = int(c / K.nx), ix = int(c - size_t(iy) * K.nx);
    float U[4][2];
    load_cell<MASK>(K, u, mask, ix, iy, U);
    const float se = cell_strain_energy(K, U);
    const float rh = rho[c];
    if (MODE == kDemEnergy) {
      acc += double(__fmul_rn(__fmul_rn(simp_r(K, rh), se), K.detJ));
    } else if (MODE == kDemObjective) {
      const float sel = __fmul_rn(se, K.detJ);
      acc += double(__fmul_rn(simp_r(K, rh), sel));
      cellv[c] = __fmul_rn(-simp_dr(K, rh), sel);
    } else {
      cellv[c] = sc * 0.5f * simp_dr(K, rh) * se * K.detJ;
    }
  }
  if (MODE == kDemDensityGrad) return;
  double ext = 0.0;
  if (MODE == kDemEnergy && wext) {
    const size_t nn = size_t(K.nx + 1) * (K.ny + 1);
    for (size_t n = size_t(blockIdx.x) * blockDim.x + threadIdx.x; n < nn; n += size_t(gridDim.x) * blockDim.x)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float v = u[2 * n + j];
        if (MASK) v = __fmul_rn(v, mask[2 * n + j]);
        ext += double(wext[2 * n + j]) * double(v);
      }
  }
  const double v[2] = {acc, ext};
  double tot[2];
  if (finish_reduction<2>(v, partials, counter, tot))
    *out = (MODE == kDemEnergy) ? 0.5 * tot[0] - tot[1] : tot[0];
}

// d psi / d u at every node: sum over the node's cells of
// r * detJ * sum_g sum_k sigma_g[j][k] * D[i][g][k], minus the external
// weight, times *scale (and times the mask when u is the network output).
template <bool MASK>
__global__ void __launch_bounds__(kDemThreads)
    k_dem_du(DemK K, const float* __restrict__ u, const float* __restrict__ mask, const float* __restrict__ rho,
             const float* __restrict__ wext, const float* __restrict__ scale, float* __restrict__ du) {
  const int NX = K.nx + 1, NY = K.ny + 1;
  const size_t nn = size_t(NX) * NY;
  const float sc = *scale;
  for (size_t n = size_t(blockIdx.x) * blockDim.x + threadIdx.x; n < nn; n += size_t(gridDim.x) * blockDim.x) {
    const int ix = int(n / NY), iy = int(n - size_t(ix) * NY);
    float g0 = 0.0f, g1 = 0.0f;
#pragma unroll
    for (int dcx = -1; dcx <= 0; ++dcx)
#pragma unroll
      for (int dcy = -1; dcy <= 0; ++dcy) {
        const int cx = ix + dcx, cy = iy + dcy;
        if (cx < 0 || cx >= K.nx || cy < 0 || cy >= K.ny) continue;
        const int i = (iy - cy) + 2 * (ix - cx);  // local node index in the cell
        float U[4][2];
        load_cell<MASK>(K, u, mask, cx, cy, U);
        const float w = simp_r(K, rho[size_t(cy) * K.nx + cx]) * K.detJ;
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          float G[2][2], S[2][2], E[2][2];
          grad_at(K, U, g, G);
          stress(K, G, S, E);
          a0 += S[0][0] * K.D[i][g][0] + S[0][1] * K.D[i][g][1];
          a1 += S[1][0] * K.D[i][g][0] + S[1][1] * K.D[i][g][1];
        }
        g0 += w * a0;
        g1 += w * a1;
      }
    if (wext) {
      g0 -= wext[2 * n];
      g1 -= wext[2 * n + 1];
    }
    if (MASK) {
      g0 *= mask[2 * n];
      g1 *= mask[2 * n + 1];
    }
    du[2 * n] = sc * g0;
    du[2 * n + 1] = sc * g1;
  }
}

__global__ void k_dem_enforce(const float* __restrict__ uh, const float* __restrict__ mask, float* __restrict__ u,
                              size_t n2) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n2; i += size_t(gridDim.x) * blockDim.x)
    u[i] = __fmul_rn(uh[i], mask[i]);
}

DemK make_k(const topo_dem_ctx* C) {
  DemK K;
  K.nx = C->d.nx;
  K.ny = C->d.ny;
  for (int i = 0; i < 4; ++i)
    for (int g = 0; g < 4; ++g)
      for (int k = 0; k < 2; ++k) K.D[i][g][k] = C->d.dshape[i][g][k];
  K.detJ = C->d.detJ;
  K.lam = C->d.lame_lambda;
  K.two_mu = C->d.two_mu;
  K.m = float(1e-6);
  K.onem = float(1.0 - 1e-6);
  K.p = float(C->p);
  K.pm1 = float(C->p - 1.0);
  auto small = [](double q) { return (q == 1.0 || q == 2.0 || q == 3.0) ? int(q) : 0; };
  K.ip = small(C->p);
  K.ipm1 = small(C->p - 1.0);
  return K;
}

int grid_for(const topo_dem_ctx* C, size_t n) {
  const size_t b = (n + kDemThreads - 1) / kDemThreads;
  return int(b < size_t(C->blocks) ? (b > 0 ? b : 1) : size_t(C->blocks));
}

template <class F>
int guarded(topo_dem_ctx* C, F&& f) {
  if (!C) return TOPO_ERR_ARG;
  try {
    C->err.clear();
    return f();
  } catch (...) {
    return C->fail(TOPO_ERR_CUDA, "exception in the DEM kernels");
  }
}

int upload(topo_dem_ctx* C, float*& dst, const float* host) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  const size_t n = 2 * size_t(C->d.nx + 1) * (C->d.ny + 1);
  if (!host) {
    cudaFree(dst);
    dst = nullptr;
    return C->cuda_check("clear");
  }
  if (!dst && cudaMalloc(&dst, n * sizeof(float)) != cudaSuccess) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  if (cudaMemcpy(dst, host, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      settle_setup_stream() != cudaSuccess)
    return C->fail(TOPO_ERR_CUDA, "copy failed");
  return TOPO_OK;
}

// ---------------------------------------------------------------------------
// density filter (DEM_src/filter.py:8-31)
// ---------------------------------------------------------------------------
// W_ij = (radius - d_ij) / S_i for d_ij <= radius, d_ij the distance between the
// element points (np.linspace(0, W, Nx) x np.linspace(0, H, Ny), element i =
// iy*Nx + ix) and S_i the row sum.  Evaluated on the fly with the reference's
// rounding, term by term: d = sqrt(dx*dx + dy*dy), the row sum accumulated in
// ascending column order, each weight divided by it, products summed in column
// order (W x: the CSR product; W^T g: the CSC product, which accumulates the
// rows in ascending order into each output).  No FMA contraction.
struct DensGrid {
  int Nx, Ny, rx, ry;
  double W, H, radius, sx, sy;
};

__device__ __forceinline__ double dens_pt(int k, int n, double L, double step) {
  if (n <= 1) return 0.0;
  return k == n - 1 ? L : __dmul_rn(double(k), step);  // np.linspace: k * step, endpoint exact
}

// calls f(j, w_ij) for the neighbours j of element i in ascending order
template <class F>
__device__ __forceinline__ void dens_row(const DensGrid& G, int i, F&& f) {
  const int iy = i / G.Nx, ix = i - iy * G.Nx;
  const double xi = dens_pt(ix, G.Nx, G.W, G.sx), yi = dens_pt(iy, G.Ny, G.H, G.sy);
  const int y0 = max(0, iy - G.ry), y1 = min(G.Ny - 1, iy + G.ry);
  const int x0 = max(0, ix - G.rx), x1 = min(G.Nx - 1, ix + G.rx);
  for (int jy = y0; jy <= y1; ++jy) {
    const double dy = __dsub_rn(dens_pt(jy, G.Ny, G.H, G.sy), yi);
    const double dy2 = __dmul_rn(dy, dy);
    for (int jx = x0; jx <= x1; ++jx) {
      const double dx = __dsub_rn(dens_pt(jx, G.Nx, G.W, G.sx), xi);
      const double d = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), dy2));
      if (d <= G.radius) f(jy * G.Nx + jx, __dsub_rn(G.radius, d));
    }
  }
}

__global__ void k_dens_rowsum(DensGrid G, double* __restrict__ S, unsigned long long* __restrict__ nnz) {
  const int n = G.Nx * G.Ny;
  unsigned long long cnt = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    dens_row(G, i, [&](int, double w) {
      s = __dadd_rn(s, fabs(w));
      ++cnt;
    });
    S[i] = s;
  }
  if (cnt) atomicAdd(nnz, cnt);  // integer count: order-independent
}

template <bool TRANSPOSE>
__global__ void k_dens_apply(DensGrid G, const double* __restrict__ S, const double* __restrict__ x,
                             double* __restrict__ y) {
  const int n = G.Nx * G.Ny;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    if (!TRANSPOSE) {
      const double s = S[i];
      dens_row(G, i, [&](int j, double w) {
        const double wn = s != 0.0 ? __ddiv_rn(w, s) : w;
        acc = __dadd_rn(acc, __dmul_rn(wn, x[j]));
      });
    } else {  // the neighbours of i are the rows that hold column i (symmetric distances)
      dens_row(G, i, [&](int j, double w) {
        const double s = S[j];
        const double wn = s != 0.0 ? __ddiv_rn(w, s) : w;
        acc = __dadd_rn(acc, __dmul_rn(wn, x[j]));
      });
    }
    y[i] = acc;
  }
}

}  // namespace

struct topo_density_filter {
  DensGrid G;
  double* S = nullptr;
  int64_t nnz = 0;
};

extern "C" {

topo_density_filter* topo_density_filter_create(int Nx, int Ny, double width, double height, double radius,
                                                int* status) {
  auto fail = [&](int rc) -> topo_density_filter* {
    if (status) *status = rc;
    return nullptr;
  };
  if (Nx < 1 || Ny < 1 || !(width > 0) || !(height > 0) || !(radius >= 0) || !std::isfinite(radius) ||
      double(Nx) * Ny > 2.0e9)
    return fail(TOPO_ERR_ARG);
  auto* F = new topo_density_filter();
  DensGrid& G = F->G;
  G.Nx = Nx;
  G.Ny = Ny;
  G.W = width;
  G.H = height;
  G.radius = radius;
  G.sx = Nx > 1 ? width / double(Nx - 1) : 0.0;
  G.sy = Ny > 1 ? height / double(Ny - 1) : 0.0;
  // neighbour box: every point within radius, with one step of margin for rounding
  G.rx = Nx > 1 ? int(std::min<double>(Nx, std::floor(radius / G.sx) + 1.0)) : 0;
  G.ry = Ny > 1 ? int(std::min<double>(Ny, std::floor(radius / G.sy) + 1.0)) : 0;
  const size_t n = size_t(Nx) * Ny;
  unsigned long long* cnt = nullptr;
  if (cudaMalloc(&F->S, n * sizeof(double)) != cudaSuccess || cudaMalloc(&cnt, sizeof(*cnt)) != cudaSuccess) {
    cudaFree(F->S);
    cudaFree(cnt);
    delete F;
    cudaGetLastError();
    return fail(TOPO_ERR_CUDA);
  }
  cudaMemset(cnt, 0, sizeof(*cnt));
  const int blocks = int(std::min<size_t>((n + 255) / 256, 65535));
  k_dens_rowsum<<<blocks, 256>>>(G, F->S, cnt);
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(cnt);
  if (e != cudaSuccess) {
    cudaFree(F->S);
    delete F;
    cudaGetLastError();
    return fail(TOPO_ERR_CUDA);
  }
  F->nnz = int64_t(h);
  if (status) *status = TOPO_OK;
  return F;
}

void topo_density_filter_destroy(topo_density_filter* f) {
  if (!f) return;
  cudaFree(f->S);
  delete f;
}

int topo_density_filter_nnz(const topo_density_filter* f, int64_t* nnz) {
  if (!f || !nnz) return TOPO_ERR_ARG;
  *nnz = f->nnz;
  return TOPO_OK;
}

int topo_density_filter_apply(topo_density_filter* f, const double* x, double* y, int transpose,
                              topo_stream_t stream) {
  if (!f || !x || !y || x == y) return TOPO_ERR_ARG;
  const size_t n = size_t(f->G.Nx) * f->G.Ny;
  const int blocks = int(std::min<size_t>((n + 255) / 256, 65535));
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (transpose) k_dens_apply<true><<<blocks, 256, 0, s>>>(f->G, f->S, x, y);
  else k_dens_apply<false><<<blocks, 256, 0, s>>>(f->G, f->S, x, y);
  return cudaGetLastError() == cudaSuccess ? TOPO_OK : TOPO_ERR_CUDA;
}

topo_dem_ctx* topo_dem_create(const topo_dem_desc* desc, int* status) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  auto set = [&](int s) {
    if (status) *status = s;
  };
  if (!desc || desc->nx < 1 || desc->ny < 1 || !(desc->detJ > 0.0f)) {
    set(TOPO_ERR_ARG);
    return nullptr;
  }
  topo_dem_ctx* C = new topo_dem_ctx();
  C->d = *desc;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&C->sms, cudaDevAttrMultiProcessorCount, dev);
  if (C->sms < 1) C->sms = 1;
  C->blocks = C->sms * 8;
  if (cudaMalloc(&C->partials, size_t(C->blocks) * 2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&C->counter, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(C->counter, 0, sizeof(unsigned)) != cudaSuccess || settle_setup_stream() != cudaSuccess) {
    cudaGetLastError();
    delete C;
    set(TOPO_ERR_CUDA);
    return nullptr;
  }
  set(TOPO_OK);
  return C;
}

void topo_dem_destroy(topo_dem_ctx* ctx) { delete ctx; }

const char* topo_dem_last_error(const topo_dem_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int topo_dem_set_penalization(topo_dem_ctx* ctx, double p) {
  return guarded(ctx, [&]() {
    if (!std::isfinite(p)) return ctx->fail(TOPO_ERR_ARG, "invalid penalization");
    ctx->p = p;
    ctx->penal_set = true;
    return TOPO_OK;
  });
}

int topo_dem_set_external(topo_dem_ctx* ctx, const float* w) {
  return guarded(ctx, [&]() { return upload(ctx, ctx->wext, w); });
}

int topo_dem_set_mask(topo_dem_ctx* ctx, const float* m) {
  return guarded(ctx, [&]() { return upload(ctx, ctx->mask, m); });
}

int topo_dem_enforce(topo_dem_ctx* ctx, const float* u_hat, float* u, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!u_hat || !u) return ctx->fail(TOPO_ERR_ARG, "null array");
    if (!ctx->mask) return ctx->fail(TOPO_ERR_STATE, "no Dirichlet mask set");
    const size_t n2 = 2 * size_t(ctx->d.nx + 1) * (ctx->d.ny + 1);
    k_dem_enforce<<<grid_for(ctx, n2), kDemThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(u_hat, ctx->mask, u,
                                                                                                  n2);
    return ctx->cuda_check("enforce");
  });
}

int topo_dem_energy(topo_dem_ctx* ctx, const float* u, const float* density, int masked, double* energy,
                    topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!u || !density || !energy) return ctx->fail(TOPO_ERR_ARG, "null array");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (masked && !ctx->mask) return ctx->fail(TOPO_ERR_STATE, "no Dirichlet mask set");
    const DemK K = make_k(ctx);
    const size_t n = std::max(size_t(K.nx) * K.ny, size_t(K.nx + 1) * (K.ny + 1));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (masked)
      k_dem_cells<kDemEnergy, true><<<grid_for(ctx, n), kDemThreads, 0, s>>>(K, u, ctx->mask, density, ctx->wext,
                                                                             nullptr, nullptr, ctx->partials,
                                                                             ctx->counter, energy);
    else
      k_dem_cells<kDemEnergy, false><<<grid_for(ctx, n), kDemThreads, 0, s>>>(K, u, nullptr, density, ctx->wext,
                                                                              nullptr, nullptr, ctx->partials,
                                                                              ctx->counter, energy);
    return ctx->cuda_check("energy");
  });
}

int topo_dem_energy_backward(topo_dem_ctx* ctx, const float* u, const float* density, int masked, const float* scale,
                             float* du, float* ddensity, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!u || !density || !scale) return ctx->fail(TOPO_ERR_ARG, "null array");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (masked && !ctx->mask) return ctx->fail(TOPO_ERR_STATE, "no Dirichlet mask set");
    const DemK K = make_k(ctx);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t nc = size_t(K.nx) * K.ny, nn = size_t(K.nx + 1) * (K.ny + 1);
    if (ddensity) {
      if (masked)
        k_dem_cells<kDemDensityGrad, true><<<grid_for(ctx, nc), kDemThreads, 0, s>>>(
            K, u, ctx->mask, density, nullptr, scale, ddensity, nullptr, nullptr, nullptr);
      else
        k_dem_cells<kDemDensityGrad, false><<<grid_for(ctx, nc), kDemThreads, 0, s>>>(
            K, u, nullptr, density, nullptr, scale, ddensity, nullptr, nullptr, nullptr);
    }
    if (du) {
      if (masked)
        k_dem_du<true><<<grid_for(ctx, nn), kDemThreads, 0, s>>>(K, u, ctx->mask, density, ctx->wext, scale, du);
      else
        k_dem_du<false><<<grid_for(ctx, nn), kDemThreads, 0, s>>>(K, u, nullptr, density, ctx->wext, scale, du);
    }
    return ctx->cuda_check("energy backward");
  });
}

int topo_dem_objective_gradient(topo_dem_ctx* ctx, const float* u, const float* density, double* objective,
                                float* gradient, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!u || !density || !objective || !gradient) return ctx->fail(TOPO_ERR_ARG, "null array");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    const DemK K = make_k(ctx);
    const size_t nc = size_t(K.nx) * K.ny;
    k_dem_cells<kDemObjective, false><<<grid_for(ctx, nc), kDemThreads, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        K, u, nullptr, density, nullptr, nullptr, gradient, ctx->partials, ctx->counter, objective);
    return ctx->cuda_check("objective and gradient");
  });
}

}  // extern "C"
