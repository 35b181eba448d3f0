// C ABI of the Stokes-Brinkman fluid problem (FEM_src/fluid_problem.py:48-155):
// Taylor-Hood state solve, objective and CG1-projected gradient, FP64.
//
// State solve: the Dirichlet velocity rows (every side carries data: the flow
// profiles of BoundaryFlows or no slip) are eliminated, which leaves the
// symmetric saddle point [A B^T; B 0] (A = alpha-weighted P2 mass + vector
// Laplacian, B = -(div u, q)).  Its pressure is fixed up to a constant and the
// interpolated boundary data carry a small mass defect, so the continuity
// right-hand side is projected to zero sum and the pressure kept at zero sum
// (the reduced system's least-squares closure).  Flexible GMRES, right
// preconditioned with the block-diagonal
//   diag( P1-iso-P2 V-cycles of K + alpha M on the (2nx)x(2ny) lattice, one per component,
//         lumped-mass inverse + V-cycle of the 1/alpha-weighted P1 Laplacian )
// (a variable-coefficient Cahouet-Chabard Schur-complement approximation).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "topomax_gb300.h"
#include "topo_fluid.cuh"
#include "topo_mg_impl.cuh"
#include "topo_fluid_setup.h"
#include "topo_sens.cuh"
#include "topo_setup.h"

namespace topo {
extern template class MG<double>;
}  // namespace topo

using namespace topo;

namespace {

constexpr int kFluidRestart = 30;
constexpr double kLaplaceShift = 1e-3;  // mass shift of the pressure Laplacian (its constant mode)

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
__global__ void k_fluid_mass(int nx, int ny, const FluidTables* __restrict__ E, FluidPenal pen,
                             const double* __restrict__ rho, double* __restrict__ mass) {
  const size_t nt = size_t(2) * nx * ny;
  TOPO_GRID_STRIDE(t, nt) {
    double r[3];
    fluid_tri_rho(rho, nx, t, r);
    fluid_tri_mass(*E, pen, r, mass + t * kFluidMass);
  }
}

// x = [u (2 n2, interleaved) | p (nv)]
__global__ void k_fluid_tri(int nx, int ny, const FluidTables* __restrict__ E, const double* __restrict__ mass,
                            const double* __restrict__ x, double* __restrict__ out) {
  const size_t nt = size_t(2) * nx * ny;
  const size_t n2 = size_t(2 * nx + 1) * (2 * ny + 1);
  TOPO_GRID_STRIDE(t, nt) {
    size_t nd[6], vt[3];
    fluid_tri_nodes(nx, t, nd);
    fluid_tri_vertices(nx, t, vt);
    double ue[6][2], pe[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = x[2 * nd[k]];
      ue[k][1] = x[2 * nd[k] + 1];
    }
    for (int k = 0; k < 3; ++k) pe[k] = x[2 * n2 + vt[k]];
    fluid_tri_apply(*E, int(t & 1), mass + t * kFluidMass, ue, pe, out + t * kFluidOut);
  }
}

__global__ void k_fluid_gather(int nx, int ny, const double* __restrict__ tri_out, const double* __restrict__ x,
                               double* __restrict__ y, int clamp) {
  const int NX = 2 * nx + 1, NY = 2 * ny + 1, VX = nx + 1;
  const size_t n2 = size_t(NX) * NY, nv = size_t(nx + 1) * (ny + 1);
  TOPO_GRID_STRIDE(i, n2 + nv) {
    if (i < n2) {
      double v[2];
      fluid_gather_node(tri_out, nx, ny, int(i % NX), int(i / NX), clamp != 0, x, v);
      y[2 * i] = v[0];
      y[2 * i + 1] = v[1];
    } else {
      const size_t k = i - n2;
      y[2 * n2 + k] = fluid_gather_vertex(tri_out, nx, ny, int(k % VX), int(k / VX), kFluidOut, 12);
    }
  }
}

__global__ void k_fluid_objective(int nx, int ny, const FluidTables* __restrict__ E, FluidPenal pen, double mu,
                                  const double* __restrict__ rho, const double* __restrict__ u, double* partials,
                                  unsigned* counter, double* out) {
  const size_t nt = size_t(2) * nx * ny;
  double v[1] = {0.0};
  TOPO_GRID_STRIDE(t, nt) {
    size_t nd[6];
    fluid_tri_nodes(nx, t, nd);
    double ue[6][2], r[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = u[2 * nd[k]];
      ue[k][1] = u[2 * nd[k] + 1];
    }
    fluid_tri_rho(rho, nx, t, r);
    v[0] += fluid_tri_objective(*E, pen, mu, int(t & 1), r, ue);
  }
  double tot[1];
  if (finish_reduction<1>(v, partials, counter, tot)) out[0] = 0.5 * tot[0];
}

__global__ void k_fluid_grad_tri(int nx, int ny, const FluidTables* __restrict__ E, FluidPenal pen,
                                 const double* __restrict__ rho, const double* __restrict__ u,
                                 double* __restrict__ tri3) {
  const size_t nt = size_t(2) * nx * ny;
  TOPO_GRID_STRIDE(t, nt) {
    size_t nd[6];
    fluid_tri_nodes(nx, t, nd);
    double ue[6][2], r[3], o3[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = u[2 * nd[k]];
      ue[k][1] = u[2 * nd[k] + 1];
    }
    fluid_tri_rho(rho, nx, t, r);
    fluid_tri_gradient(*E, pen, r, ue, o3);
    tri3[3 * t] = o3[0];
    tri3[3 * t + 1] = o3[1];
    tri3[3 * t + 2] = o3[2];
  }
}

// rho at P2 node (a, b): the CG1 field interpolated linearly (vertex, edge midpoint
// or the cell's diagonal midpoint)
__device__ double fluid_rho_node(const double* rho, int nx, int a, int b) {
  const int VX = nx + 1;
  const int i0 = a >> 1, j0 = b >> 1;
  const int i1 = i0 + (a & 1), j1 = j0 + (b & 1);
  return 0.5 * (rho[size_t(j0) * VX + i0] + rho[size_t(j1) * VX + i1]);
}

// velocity preconditioner coefficients on the refined lattice: kM = alpha(rho) at each
// triangle's centroid (kK = 1)
__global__ void k_fluid_refined_alpha(int nx, int ny, FluidPenal pen, const double* __restrict__ rho,
                                      double* __restrict__ kM) {
  const int NXc = 2 * nx;  // cells of the refined lattice per row
  const size_t nt = size_t(2) * NXc * (2 * ny);
  TOPO_GRID_STRIDE(t, nt) {
    const int o = int(t & 1);
    const size_t cell = t >> 1;
    const int I = int(cell % NXc), J = int(cell / NXc);
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += fluid_rho_node(rho, nx, I + p1_off_a(o, k), J + p1_off_b(o, k));
    kM[t] = pen.a(s / 3.0);
  }
}

// pressure Laplacian coefficient kK = 1 / alpha(rho) at each base triangle's centroid
__global__ void k_fluid_inv_alpha(int nx, int ny, FluidPenal pen, const double* __restrict__ rho,
                                  double* __restrict__ kK) {
  const size_t nt = size_t(2) * nx * ny;
  TOPO_GRID_STRIDE(t, nt) {
    double r[3];
    fluid_tri_rho(rho, nx, t, r);
    kK[t] = 1.0 / pen.a((r[0] + r[1] + r[2]) / 3.0);
  }
}

__global__ void k_fluid_coarsen(const double* __restrict__ kf, int nxf, int nyf, double* __restrict__ kc, int nxc,
                                int nyc) {
  const size_t nt = size_t(2) * nxc * nyc;
  TOPO_GRID_STRIDE(t, nt) {
    const size_t cell = t >> 1;
    kc[t] = coarsen_kappa(kf, nxf, nyf, int(cell % nxc), int(cell / nxc), int(t & 1));
  }
}

// planar components of the interleaved velocity, zero on the boundary nodes
__global__ void k_fluid_split(int NX, int NY, const double* __restrict__ v, double* __restrict__ c0,
                              double* __restrict__ c1) {
  const size_t n = size_t(NX) * NY;
  TOPO_GRID_STRIDE(i, n) {
    const bool bd = fluid_boundary_node(int(i % NX), int(i / NX), NX, NY);
    c0[i] = bd ? 0.0 : v[2 * i];
    c1[i] = bd ? 0.0 : v[2 * i + 1];
  }
}

__global__ void k_fluid_merge(int NX, int NY, const double* __restrict__ c0, const double* __restrict__ c1,
                              double* __restrict__ v) {
  const size_t n = size_t(NX) * NY;
  TOPO_GRID_STRIDE(i, n) {
    const bool bd = fluid_boundary_node(int(i % NX), int(i / NX), NX, NY);
    v[2 * i] = bd ? 0.0 : c0[i];
    v[2 * i + 1] = bd ? 0.0 : c1[i];
  }
}

// y = x - sum(x)/n with the sum a device scalar (one reduction before); y may be x
__global__ void k_fluid_center(const double* x, double* y, size_t n, const double* __restrict__ sum) {
  const double m = *sum / double(n);
  TOPO_GRID_STRIDE(i, n) y[i] = x[i] - m;
}

// z = r / m_lumped + zl
__global__ void k_fluid_pcombine(const double* __restrict__ r, const double* __restrict__ ml,
                                 const double* __restrict__ zl, double* __restrict__ z, size_t n) {
  TOPO_GRID_STRIDE(i, n) z[i] = r[i] / ml[i] + zl[i];
}

// zero the boundary velocity rows: b[2i+c] = 0 at boundary nodes
__global__ void k_fluid_zero_boundary(int NX, int NY, double* __restrict__ v) {
  const size_t n = size_t(NX) * NY;
  TOPO_GRID_STRIDE(i, n) {
    if (fluid_boundary_node(int(i % NX), int(i / NX), NX, NY)) {
      v[2 * i] = 0.0;
      v[2 * i + 1] = 0.0;
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct topo_fluid_ctx {
  int nx = 0, ny = 0, sms = 148;
  double W = 0, H = 0, hx = 0, hy = 0, viscosity = 1.0;
  size_t n2 = 0, nv = 0, n = 0;  // P2 nodes, CG1 vertices, unknowns (2 n2 + nv)
  FluidPenal pen{};
  bool penal_set = false;
  long long launches = 0;
  std::string err;
  Arena arena;
  Reducer red;
  FluidTables host_tab{};
  FluidTables* tab = nullptr;  // device copy
  double* ub = nullptr;        // boundary data (interleaved, zero inside)
  double* mass = nullptr;      // [tri][21]
  double* tri_out = nullptr;   // [tri][16]
  double* tri3 = nullptr;      // [tri][3]
  double* ml = nullptr;        // lumped CG1 mass (vertex weights)
  double* ones = nullptr;      // nv ones (sums by a dot)
  double* rhs = nullptr;       // n
  double* x = nullptr;         // n (interior velocity | pressure)
  double* V = nullptr;         // (m + 1) n
  double* Z = nullptr;         // m n
  double* t = nullptr;         // n
  double* c0 = nullptr;        // planar velocity components (n2 each)
  double* c1 = nullptr;
  double* z0 = nullptr;
  double* z1 = nullptr;
  double* pt = nullptr;        // nv scratch
  double* pz = nullptr;
  double* gb = nullptr;        // gradient right-hand side (nv)
  // preconditioner hierarchies
  std::vector<LevelSpec> uspec, pspec;
  std::vector<ElemRefs> urefs, prefs;
  std::vector<double*> uK, uM, pK, pM;
  MG<double> mgu, mgp;
  topo_ctx* proj = nullptr;  // the CG1 projection (mass-matrix solve: a filter of radius 0)

  ~topo_fluid_ctx() {
    if (proj) topo_destroy(proj);
    if (red.host) cudaFreeHost(red.host);
  }
  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda_check(const char* where) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TOPO_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
    return TOPO_OK;
  }
  int grid(size_t m) const { return vec_grid(m, sms); }
  int NX() const { return 2 * nx + 1; }
  int NY() const { return 2 * ny + 1; }
  double* pp(double* v) const { return v + 2 * n2; }

  double dot(const double* a, const double* b, size_t m, cudaStream_t s) {
    k_dot<double, double><<<red.blocks, kVecThreads, 0, s>>>(a, b, m, red.partials, red.counter, red.out);
    ++launches;
    cudaMemcpyAsync(red.host, red.out, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return red.host[0];
  }
  // y = x - mean(x) on the pressure block (device-side mean)
  void center(const double* xp, double* yp, cudaStream_t s) {
    k_dot<double, double><<<red.blocks, kVecThreads, 0, s>>>(xp, ones, nv, red.partials, red.counter, red.out);
    k_fluid_center<<<grid(nv), kVecThreads, 0, s>>>(xp, yp, nv, red.out);
    launches += 2;
  }
  // y = A x: per-triangle rows, then the node / vertex gathers
  void apply(const double* xin, double* y, bool clamp, cudaStream_t s) {
    const size_t nt = size_t(2) * nx * ny;
    k_fluid_tri<<<grid(nt), kVecThreads, 0, s>>>(nx, ny, tab, mass, xin, tri_out);
    k_fluid_gather<<<grid(n2 + nv), kVecThreads, 0, s>>>(nx, ny, tri_out, xin, y, clamp ? 1 : 0);
    launches += 2;
  }
  // z = P r (block-diagonal preconditioner)
  void precond(const double* r, double* z, cudaStream_t s) {
    k_fluid_split<<<grid(n2), kVecThreads, 0, s>>>(NX(), NY(), r, c0, c1);
    mgu.vcycle(c0, z0, s);
    mgu.vcycle(c1, z1, s);
    k_fluid_merge<<<grid(n2), kVecThreads, 0, s>>>(NX(), NY(), z0, z1, z);
    const double* rp = r + 2 * n2;
    center(rp, pt, s);
    mgp.vcycle(pt, pz, s);
    k_fluid_pcombine<<<grid(nv), kVecThreads, 0, s>>>(rp, ml, pz, pp(z), nv);
    center(pp(z), pp(z), s);
    launches += 3;
  }
};

namespace {

int fluid_setup(topo_fluid_ctx* C, const double* rho, cudaStream_t s) {
  const size_t nt = size_t(2) * C->nx * C->ny;
  k_fluid_mass<<<C->grid(nt), kVecThreads, 0, s>>>(C->nx, C->ny, C->tab, C->pen, rho, C->mass);
  k_fluid_refined_alpha<<<C->grid(C->uspec[0].ntri()), kVecThreads, 0, s>>>(C->nx, C->ny, C->pen, rho, C->uM[0]);
  k_fluid_inv_alpha<<<C->grid(nt), kVecThreads, 0, s>>>(C->nx, C->ny, C->pen, rho, C->pK[0]);
  C->launches += 3;
  for (size_t l = 1; l < C->uspec.size(); ++l) {
    const LevelSpec &F = C->uspec[l - 1], &Cc = C->uspec[l];
    k_fluid_coarsen<<<C->grid(Cc.ntri()), kVecThreads, 0, s>>>(C->uM[l - 1], F.nx, F.ny, C->uM[l], Cc.nx, Cc.ny);
    ++C->launches;
  }
  for (size_t l = 1; l < C->pspec.size(); ++l) {
    const LevelSpec &F = C->pspec[l - 1], &Cc = C->pspec[l];
    k_fluid_coarsen<<<C->grid(Cc.ntri()), kVecThreads, 0, s>>>(C->pK[l - 1], F.nx, F.ny, C->pK[l], Cc.nx, Cc.ny);
    ++C->launches;
  }
  // both hierarchies' coefficients follow the design: choose their truncation and
  // uniform-row shortcuts again
  C->mgu.coefficients_changed();
  C->mgp.coefficients_changed();
  int st = C->mgu.setup(s);
  if (!st) st = C->mgp.setup(s);
  if (st == -5) return C->fail(TOPO_ERR_CUDA, "fluid preconditioner set-up: CUDA error");
  if (st) return C->fail(TOPO_ERR_NOT_CONVERGED, "fluid preconditioner set-up: coarse operator not positive definite");
  return C->cuda_check("fluid set-up");
}

// chunked classical Gram-Schmidt helpers over the Krylov basis (at most 8 vectors a launch)
void multidot(topo_fluid_ctx* C, int count, const double* w, double* h, double& ww, cudaStream_t s) {
  for (int i0 = 0; i0 < count; i0 += 8) {
    const int c = std::min(8, count - i0);
    const double* Vb = C->V + size_t(i0) * C->n;
#define TOPO_MD(K) \
  k_multidot<double, double, K><<<C->red.blocks, kVecThreads, 0, s>>>(Vb, C->n, w, C->n, C->red.partials, C->red.counter, C->red.out)
    TOPO_DISPATCH_COUNT(c, TOPO_MD)
#undef TOPO_MD
    ++C->launches;
    cudaMemcpyAsync(C->red.host, C->red.out, (c + 1) * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    for (int k = 0; k < c; ++k) h[i0 + k] = C->red.host[k];
    ww = C->red.host[c];
  }
}

void sub_multi(topo_fluid_ctx* C, int count, const double* h, double* w, cudaStream_t s) {
  for (int i0 = 0; i0 < count; i0 += 8) {
    const int c = std::min(8, count - i0);
    MultiCoef cf{};
    for (int k = 0; k < c; ++k) cf.c[k] = h[i0 + k];
    const double* Vb = C->V + size_t(i0) * C->n;
#define TOPO_SM(K) k_sub_multi<double, double, K><<<C->grid(C->n), kVecThreads, 0, s>>>(w, Vb, C->n, cf, C->n)
    TOPO_DISPATCH_COUNT(c, TOPO_SM)
#undef TOPO_SM
    ++C->launches;
  }
}

void add_multi(topo_fluid_ctx* C, int count, const double* y, double* x, cudaStream_t s) {
  for (int i0 = 0; i0 < count; i0 += 8) {
    const int c = std::min(8, count - i0);
    MultiCoef cf{};
    for (int k = 0; k < c; ++k) cf.c[k] = y[i0 + k];
    const double* Zb = C->Z + size_t(i0) * C->n;
#define TOPO_AM(K) k_add_multi<double, double, K><<<C->grid(C->n), kVecThreads, 0, s>>>(x, Zb, C->n, cf, C->n)
    TOPO_DISPATCH_COUNT(c, TOPO_AM)
#undef TOPO_AM
    ++C->launches;
  }
}

// Flexible GMRES(m), right preconditioned, on the clamped operator from x = 0;
// stops on the true residual |b - A x| <= rtol |b|.
int fluid_fgmres(topo_fluid_ctx* C, const double* b, double* x, double rtol, int maxit, int& iters, double& relres,
                 cudaStream_t s) {
  constexpr int m = kFluidRestart;
  const size_t n = C->n;
  const int g = C->grid(n);
  iters = 0;
  relres = 0.0;
  k_fill<double><<<g, kVecThreads, 0, s>>>(x, 0.0, n);
  ++C->launches;
  const double bn = std::sqrt(C->dot(b, b, n, s));
  if (!std::isfinite(bn)) return C->fail(TOPO_ERR_NAN, "non-finite right-hand side");
  if (bn == 0.0) return TOPO_OK;
  std::vector<double> H((m + 1) * m), cs(m), sn(m), gv(m + 1), h(m + 1), y(m);
  auto Hij = [&](int i, int j) -> double& { return H[size_t(i) * m + j]; };
  for (int cycle = 0;; ++cycle) {
    double* r = C->V;
    if (cycle == 0) {
      cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    } else {
      C->apply(x, C->t, true, s);
      k_sub<double><<<g, kVecThreads, 0, s>>>(r, b, C->t, n);
      ++C->launches;
    }
    const double beta = std::sqrt(C->dot(r, r, n, s));
    relres = beta / bn;
    if (!std::isfinite(beta)) return C->fail(TOPO_ERR_NAN, "non-finite residual in the fluid solve");
    if (beta <= rtol * bn) return TOPO_OK;
    if (iters >= maxit)
      return C->fail(TOPO_ERR_NOT_CONVERGED, "fluid state solve did not converge (relres %.3g after %d iterations)",
                     relres, iters);
    k_scale<double><<<g, kVecThreads, 0, s>>>(r, 1.0 / beta, n);
    ++C->launches;
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int k = 0;
    for (int j = 0; j < m && iters < maxit; ++j) {
      double* vj = C->V + size_t(j) * n;
      double* zj = C->Z + size_t(j) * n;
      double* w = C->V + size_t(j + 1) * n;
      C->precond(vj, zj, s);
      C->apply(zj, w, true, s);
      ++iters;
      // classical Gram-Schmidt, a second pass when the first cancelled more than half of w
      std::fill(h.begin(), h.end(), 0.0);
      double hn = 0.0;
      for (int pass = 0; pass < 2; ++pass) {
        std::vector<double> hp(j + 1);
        double ww = 0.0;
        multidot(C, j + 1, w, hp.data(), ww, s);
        double hh = 0.0;
        for (int i = 0; i <= j; ++i) {
          h[i] += hp[i];
          hh += hp[i] * hp[i];
        }
        sub_multi(C, j + 1, hp.data(), w, s);
        const double est = ww - hh;
        if (pass == 0 && est >= 0.5 * ww) {
          hn = std::sqrt(est);
          break;
        }
        if (pass == 1) hn = std::sqrt(C->dot(w, w, n, s));
      }
      if (!std::isfinite(hn)) return C->fail(TOPO_ERR_NAN, "non-finite Krylov vector in the fluid solve");
      for (int i = 0; i <= j; ++i) Hij(i, j) = h[i];
      Hij(j + 1, j) = hn;
      if (hn > 0) {
        k_scale<double><<<g, kVecThreads, 0, s>>>(w, 1.0 / hn, n);
        ++C->launches;
      }
      for (int i = 0; i < j; ++i) {
        const double t0 = cs[i] * Hij(i, j) + sn[i] * Hij(i + 1, j);
        Hij(i + 1, j) = -sn[i] * Hij(i, j) + cs[i] * Hij(i + 1, j);
        Hij(i, j) = t0;
      }
      const double den = std::hypot(Hij(j, j), Hij(j + 1, j));
      cs[j] = den > 0 ? Hij(j, j) / den : 1.0;
      sn[j] = den > 0 ? Hij(j + 1, j) / den : 0.0;
      Hij(j, j) = den;
      Hij(j + 1, j) = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      k = j + 1;
      if (std::fabs(gv[j + 1]) <= 0.5 * rtol * bn || hn == 0.0) break;
    }
    for (int i = k - 1; i >= 0; --i) {
      double acc = gv[i];
      for (int l = i + 1; l < k; ++l) acc -= Hij(i, l) * y[l];
      y[i] = Hij(i, i) != 0.0 ? acc / Hij(i, i) : 0.0;
    }
    add_multi(C, k, y.data(), x, s);
  }
}

template <class F>
int fguard(topo_fluid_ctx* C, F&& f) {
  if (!C) return TOPO_ERR_ARG;
  try {
    C->err.clear();
    return f();
  } catch (const std::exception& e) {
    return C->fail(TOPO_ERR_CUDA, "exception: %s", e.what());
  } catch (...) {
    return C->fail(TOPO_ERR_CUDA, "unknown exception");
  }
}

int fluid_init(topo_fluid_ctx* C, const topo_grid_desc* g, double viscosity, const topo_flow* flows, int nf) {
  if (!g || g->nx < 1 || g->ny < 1 || !(g->width > 0) || !(g->height > 0))
    return C->fail(TOPO_ERR_ARG, "invalid grid description");
  if (size_t(2 * g->nx + 1) * size_t(2 * g->ny + 1) > (size_t(1) << 28)) return C->fail(TOPO_ERR_ARG, "grid too large");
  if (!std::isfinite(viscosity)) return C->fail(TOPO_ERR_ARG, "invalid viscosity");
  if (nf < 0 || (nf > 0 && !flows)) return C->fail(TOPO_ERR_ARG, "invalid flow list");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return C->fail(TOPO_ERR_CUDA, "no CUDA device");
  cudaDeviceGetAttribute(&C->sms, cudaDevAttrMultiProcessorCount, dev);
  C->nx = g->nx;
  C->ny = g->ny;
  C->W = g->width;
  C->H = g->height;
  C->hx = g->width / g->nx;
  C->hy = g->height / g->ny;
  C->viscosity = viscosity;
  C->n2 = size_t(C->NX()) * C->NY();
  C->nv = size_t(C->nx + 1) * (C->ny + 1);
  C->n = 2 * C->n2 + C->nv;
  C->pen.amin = 2.5 / (100.0 * 100.0);  // src/penalizers.py:53-54
  C->pen.amax = 2.5 / (0.01 * 0.01);
  std::string msg;
  std::vector<double> ub;
  if (fluid_boundary_values(C->nx, C->ny, C->W, C->H, flows, nf, ub, msg)) return C->fail(TOPO_ERR_ARG, "%s", msg.c_str());
  fluid_tables(C->hx, C->hy, C->host_tab);
  C->red.init(C->arena, C->sms);
  const size_t nt = size_t(2) * C->nx * C->ny;
  C->tab = C->arena.alloc_n<FluidTables>(1);
  C->ub = C->arena.alloc_n<double>(2 * C->n2);
  C->mass = C->arena.alloc_n<double>(nt * kFluidMass);
  C->tri_out = C->arena.alloc_n<double>(nt * kFluidOut);
  C->tri3 = C->arena.alloc_n<double>(3 * nt);
  C->ml = C->arena.alloc_n<double>(C->nv);
  C->ones = C->arena.alloc_n<double>(C->nv);
  C->rhs = C->arena.alloc_n<double>(C->n);
  C->x = C->arena.alloc_n<double>(C->n);
  C->V = C->arena.alloc_n<double>(size_t(kFluidRestart + 1) * C->n);
  C->Z = C->arena.alloc_n<double>(size_t(kFluidRestart) * C->n);
  C->t = C->arena.alloc_n<double>(C->n);
  C->c0 = C->arena.alloc_n<double>(C->n2);
  C->c1 = C->arena.alloc_n<double>(C->n2);
  C->z0 = C->arena.alloc_n<double>(C->n2);
  C->z1 = C->arena.alloc_n<double>(C->n2);
  C->pt = C->arena.alloc_n<double>(C->nv);
  C->pz = C->arena.alloc_n<double>(C->nv);
  C->gb = C->arena.alloc_n<double>(C->nv);
  if (C->arena.failed()) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  const std::vector<double> w = vertex_weights(C->nx, C->ny, C->hx, C->hy);
  if (cudaMemcpy(C->tab, &C->host_tab, sizeof(FluidTables), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(C->ub, ub.data(), ub.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(C->ml, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    return C->cuda_check("fluid set-up copies");
  cudaStream_t s = 0;
  k_fill<double><<<C->grid(C->nv), kVecThreads, 0, s>>>(C->ones, 1.0, C->nv);
  // velocity hierarchy: P1 on the refined lattice, every side clamped
  Dir du = no_dir(C->NX(), C->NY());
  du.x_lo = 1;
  du.y_lo = 1;
  du.x_hi_from = C->NX() - 1;
  du.y_hi_from = C->NY() - 1;
  C->uspec = build_levels(false, 2 * C->nx, 2 * C->ny, 0.5 * C->hx, 0.5 * C->hy, du, 1);
  C->pspec = build_levels(false, C->nx, C->ny, C->hx, C->hy, no_dir(C->nx + 1, C->ny + 1), 1);
  auto hierarchy = [&](std::vector<LevelSpec>& spec, std::vector<ElemRefs>& refs, std::vector<double*>& kK,
                       std::vector<double*>& kM) {
    const int L = int(spec.size());
    refs.resize(L);
    kK.assign(L, nullptr);
    kM.assign(L, nullptr);
    for (int l = 0; l < L; ++l) {
      refs[l] = make_elem_refs(spec[l].hx, spec[l].hy, 0.0, 0.0);
      kK[l] = C->arena.alloc_n<double>(spec[l].ntri());
      kM[l] = C->arena.alloc_n<double>(spec[l].ntri());
    }
  };
  hierarchy(C->uspec, C->urefs, C->uK, C->uM);
  hierarchy(C->pspec, C->prefs, C->pK, C->pM);
  if (C->arena.failed()) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  // the design-independent coefficients: kK = 1 (velocity), kM = shift (pressure)
  for (size_t l = 0; l < C->uspec.size(); ++l)
    k_fill<double><<<C->grid(C->uspec[l].ntri()), kVecThreads, 0, s>>>(C->uK[l], 1.0, C->uspec[l].ntri());
  for (size_t l = 0; l < C->pspec.size(); ++l)
    k_fill<double><<<C->grid(C->pspec[l].ntri()), kVecThreads, 0, s>>>(C->pM[l], kLaplaceShift, C->pspec[l].ntri());
  for (auto* mg : {&C->mgu, &C->mgp}) {
    mg->use_graphs = false;  // only V-cycles are used, launched from the host
    mg->profile_levels = false;
  }
  C->mgu.init(C->uspec, C->urefs.data(), 0.0, 0.0, C->arena, &C->red);
  C->mgu.set_coefficients(std::vector<const double*>(C->uK.begin(), C->uK.end()),
                          std::vector<const double*>(C->uM.begin(), C->uM.end()));
  C->mgp.init(C->pspec, C->prefs.data(), 0.0, 0.0, C->arena, &C->red);
  C->mgp.set_coefficients(std::vector<const double*>(C->pK.begin(), C->pK.end()),
                          std::vector<const double*>(C->pM.begin(), C->pM.end()));
  if (C->arena.failed()) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  int st = 0;
  C->proj = topo_create_filter(g, 0.0, TOPO_PREC_FP64, &st);
  if (!C->proj) return C->fail(st ? st : TOPO_ERR_CUDA, "CG1 projection set-up failed");
  return C->cuda_check("fluid set-up");
}

}  // namespace

extern "C" {

topo_fluid_ctx* topo_fluid_create(const topo_grid_desc* grid, double viscosity, const topo_flow* flows, int n_flows,
                                  int* status) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  topo_fluid_ctx* C = nullptr;
  int rc = TOPO_OK;
  try {
    C = new topo_fluid_ctx();
    rc = fluid_init(C, grid, viscosity, flows, n_flows);
    if (!rc) {
      const cudaError_t e = settle_setup_stream();
      if (e != cudaSuccess) rc = C->fail(TOPO_ERR_CUDA, "set-up: %s", cudaGetErrorString(e));
    }
  } catch (...) {
    rc = TOPO_ERR_CUDA;
  }
  if (status) *status = rc;
  if (rc) {
    if (C) std::fprintf(stderr, "topo_fluid_create: %s\n", C->err.c_str());
    delete C;
    return nullptr;
  }
  return C;
}

void topo_fluid_destroy(topo_fluid_ctx* ctx) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  delete ctx;
}

const char* topo_fluid_last_error(const topo_fluid_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int topo_fluid_sizes(const topo_fluid_ctx* ctx, int64_t* n_vertices, int64_t* n_velocity) {
  if (!ctx) return TOPO_ERR_ARG;
  if (n_vertices) *n_vertices = int64_t(ctx->nv);
  if (n_velocity) *n_velocity = int64_t(2 * ctx->n2);
  return TOPO_OK;
}

int topo_fluid_set_penalization(topo_fluid_ctx* ctx, double q) {
  return fguard(ctx, [&]() {
    if (!std::isfinite(q) || !(q > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid penalization");
    ctx->pen.q = q;
    ctx->penal_set = true;
    return TOPO_OK;
  });
}

int topo_fluid_boundary_values(topo_fluid_ctx* ctx, double* u, topo_stream_t stream) {
  return fguard(ctx, [&]() {
    if (!u) return ctx->fail(TOPO_ERR_ARG, "null output");
    cudaMemcpyAsync(u, ctx->ub, 2 * ctx->n2 * sizeof(double), cudaMemcpyDeviceToDevice,
                    reinterpret_cast<cudaStream_t>(stream));
    return ctx->cuda_check("boundary values");
  });
}

int topo_fluid_apply(topo_fluid_ctx* ctx, const double* rho, const double* x, double* y, int clamp,
                     topo_stream_t stream) {
  return fguard(ctx, [&]() {
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!rho || !x || !y || x == y) return ctx->fail(TOPO_ERR_ARG, "invalid apply arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t nt = size_t(2) * ctx->nx * ctx->ny;
    k_fluid_mass<<<ctx->grid(nt), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, ctx->tab, ctx->pen, rho, ctx->mass);
    ++ctx->launches;
    ctx->apply(x, y, clamp != 0, s);
    return ctx->cuda_check("fluid apply");
  });
}

int topo_fluid_state_solve(topo_fluid_ctx* ctx, const double* rho, double* u, double* p, double rtol, int* iters,
                           topo_stream_t stream) {
  return fguard(ctx, [&]() {
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!rho || !u || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid state-solve arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    int rc = fluid_setup(ctx, rho, s);
    if (rc) return rc;
    // right-hand side: minus the unclamped operator on the boundary data, boundary rows
    // zero, continuity part projected to zero sum
    double* lift = ctx->t;
    cudaMemsetAsync(lift, 0, ctx->n * sizeof(double), s);
    cudaMemcpyAsync(lift, ctx->ub, 2 * ctx->n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    ctx->apply(lift, ctx->rhs, false, s);
    k_scale<double><<<ctx->grid(ctx->n), kVecThreads, 0, s>>>(ctx->rhs, -1.0, ctx->n);
    k_fluid_zero_boundary<<<ctx->grid(ctx->n2), kVecThreads, 0, s>>>(ctx->NX(), ctx->NY(), ctx->rhs);
    ctx->launches += 2;
    ctx->center(ctx->pp(ctx->rhs), ctx->pp(ctx->rhs), s);
    int it = 0;
    double rel = 0.0;
    rc = fluid_fgmres(ctx, ctx->rhs, ctx->x, rtol, 2000, it, rel, s);
    if (iters) *iters = it;
    if (rc) return rc;
    // u = interior solution + boundary data; p = the zero-sum pressure
    k_add_multi<double, double, 1><<<ctx->grid(2 * ctx->n2), kVecThreads, 0, s>>>(
        ctx->x, ctx->ub, 2 * ctx->n2, MultiCoef{{1.0}}, 2 * ctx->n2);
    cudaMemcpyAsync(u, ctx->x, 2 * ctx->n2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (p) cudaMemcpyAsync(p, ctx->pp(ctx->x), ctx->nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    ++ctx->launches;
    return ctx->cuda_check("fluid state solve");
  });
}

int topo_fluid_objective(topo_fluid_ctx* ctx, const double* rho, const double* u, double* objective,
                         topo_stream_t stream) {
  return fguard(ctx, [&]() {
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!rho || !u || !objective) return ctx->fail(TOPO_ERR_ARG, "invalid objective arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    k_fluid_objective<<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->nx, ctx->ny, ctx->tab, ctx->pen, ctx->viscosity,
                                                              rho, u, ctx->red.partials, ctx->red.counter, objective);
    ++ctx->launches;
    return ctx->cuda_check("fluid objective");
  });
}

int topo_fluid_gradient_rhs(topo_fluid_ctx* ctx, const double* rho, const double* u, double* b,
                            topo_stream_t stream) {
  return fguard(ctx, [&]() {
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!rho || !u || !b) return ctx->fail(TOPO_ERR_ARG, "invalid gradient arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t nt = size_t(2) * ctx->nx * ctx->ny;
    k_fluid_grad_tri<<<ctx->grid(nt), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, ctx->tab, ctx->pen, rho, u, ctx->tri3);
    k_vertex_gather3<double><<<ctx->grid(ctx->nv), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, ctx->tri3, b);
    ctx->launches += 2;
    return ctx->cuda_check("fluid gradient");
  });
}

int topo_fluid_gradient(topo_fluid_ctx* ctx, const double* rho, const double* u, double* g, double rtol, int* iters,
                        topo_stream_t stream) {
  int rc = topo_fluid_gradient_rhs(ctx, rho, u, ctx ? ctx->gb : nullptr, stream);
  if (rc) return rc;
  return fguard(ctx, [&]() {
    if (!g || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid gradient arguments");
    const int r = topo_filter_solve(ctx->proj, ctx->gb, g, rtol, iters, stream);
    if (r) return ctx->fail(r, "CG1 projection: %s", topo_last_error(ctx->proj));
    return TOPO_OK;
  });
}

int topo_fluid_launch_count(const topo_fluid_ctx* ctx, int64_t* launches) {
  if (!ctx || !launches) return TOPO_ERR_ARG;
  int64_t pl = 0;
  if (ctx->proj) topo_launch_count(ctx->proj, &pl);
  *launches = ctx->launches + ctx->mgu.launches + ctx->mgp.launches + pl;
  return TOPO_OK;
}

}  // extern "C"
