// C ABI of the topomax GB300 design loop: problem context, load assembly,
// iterative refinement, sensitivity and the entropic-mirror-descent update.
#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "topomax_gb300.h"
#include "topo_mg_impl.cuh"
#include "topo_setup.h"
#include "topo_sens.cuh"

namespace topo {
extern template class MG<float>;
extern template class MG<double>;
}  // namespace topo

using namespace topo;

namespace {

constexpr int kFilterMaxIt = 200;
constexpr int kStateMaxIt = 500;
constexpr int kMaxOuter = 30;

struct NewtonState {
  double c;
  double f, fp;
  int done, ok, iters, pad;
};

// Workspace of the flexible-GMRES refinement loop.
struct Fgmres {
  static constexpr int m = 8;  // restart length
  double* V = nullptr;         // (m+1) x n Krylov basis (FP64)
  double* Z = nullptr;         // m x n preconditioned directions (inner solutions, accumulated in FP64)
  double* t = nullptr;         // n
  void init(Arena& a, size_t n) {
    V = a.alloc_n<double>((m + 1) * n);
    Z = a.alloc_n<double>(m * n);
    t = a.alloc_n<double>(n);
  }
};

__device__ __forceinline__ double expit_d(double x) { return 1.0 / (1.0 + exp(-x)); }

// ---------------------------------------------------------------------------
// design-level kernels
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_cell_rmass(int nx, int ny, Penal<double> pen, const double* __restrict__ xi, T* __restrict__ out) {
  const size_t nc = size_t(nx) * ny;
  TOPO_GRID_STRIDE(c, nc) cell_rmass<T>(int(c % nx), int(c / nx), nx, ny, xi, pen, out);
}

// the FP32 operator's and its preconditioner's own r-weighted mass matrices, one
// pass (same arithmetic as their on-the-fly evaluation, so reading them instead
// changes no result)
__global__ void k_cell_rmass32(int nx, int ny, Penal<float> pen_op, Penal<float> pen_pc,
                               const float* __restrict__ xi, float* __restrict__ out_op,
                               float* __restrict__ out_pc) {
  const size_t nc = size_t(nx) * ny;
  TOPO_GRID_STRIDE(c, nc) cell_rmass_pair<float>(int(c % nx), int(c / nx), nx, xi, pen_op, pen_pc, out_op, out_pc);
}

// kappa of state level 1 and the residual operator's mass matrices (RM: FP64, or
// (hi, lo) pairs for the pair-of-FP32 operator), one pass
template <class RM>
__global__ void k_cell_rmass_kappa(int nx, int ny, Penal<double> pen, const double* __restrict__ xi,
                                   RM* __restrict__ rm, double* __restrict__ kK) {
  const size_t nc = size_t(nx) * ny;
  TOPO_GRID_STRIDE(c, nc) cell_rmass_kappa<double, RM>(int(c % nx), int(c / nx), nx, ny, xi, pen, rm, kK);
}

// The same one pass in pair-of-FP32 arithmetic (cell_rmass_kappa_dd) for an
// integer penalisation exponent: mass matrices as (hi, lo) pairs, kappa in FP64
__global__ void k_cell_rmass_kappa_dd(int nx, int ny, int ip, dd pmin, dd one_m_pmin,
                                      const double* __restrict__ xi, dd* __restrict__ rm,
                                      double* __restrict__ kK) {
  const size_t nc = size_t(nx) * ny;
  TOPO_GRID_STRIDE(c, nc) cell_rmass_kappa_dd(int(c % nx), int(c / nx), nx, xi, ip, pmin, one_m_pmin, rm, kK);
}

__global__ void k_coarsen_kappa(const double* __restrict__ kf, int nxf, int nyf, double* __restrict__ kc,
                                int nxc, int nyc) {
  const size_t nt = size_t(2) * nxc * nyc;
  TOPO_GRID_STRIDE(t, nt) {
    const int o = int(t & 1);
    const size_t cell = t >> 1;
    kc[t] = coarsen_kappa(kf, nxf, nyf, int(cell % nxc), int(cell / nxc), o);
  }
}

// half = psi_prev - alpha g, and ehalf = exp(-half) for the Newton evaluations
__global__ void k_emd_half(const double* __restrict__ psi_prev, const double* __restrict__ g, double alpha,
                           double* __restrict__ half, double* __restrict__ ehalf, size_t n) {
  TOPO_GRID_STRIDE(i, n) {
    const double h = psi_prev[i] - alpha * g[i];
    half[i] = h;
    ehalf[i] = exp(-h);
  }
}

// One Newton step of  F(c) = int expit(half + c) - volume = 0  (src/solver.py:149-186,
// scipy newton semantics: stop when |c_new - c| < tol).
// warm-start guess from a solution history x_0 (last), x_1, ...: y = sum_i c_i x_i (the
// polynomial extrapolation's weights, see topo_ctx::fwarm)
constexpr int kMaxExtrapolate = 4;
struct Extrapolation {
  const double* x[kMaxExtrapolate + 1];
  double c[kMaxExtrapolate + 1];
  int n;
};
__global__ void k_extrapolate(double* __restrict__ y, Extrapolation ex, size_t n) {
  TOPO_GRID_STRIDE(i, n) {
    double v = ex.c[0] * ex.x[0][i];
    for (int k = 1; k < ex.n; ++k) v += ex.c[k] * ex.x[k][i];
    y[i] = v;
  }
}

// expit(half + c) = 1 / (1 + exp(-half) exp(-c)): with exp(-half) evaluated once per
// projection (ehalf), an evaluation costs one exponential per thread instead of one
// per node (FP64 arithmetic is scarce on this GPU).  Where either factor is zero or
// infinite the product could be 0 * inf; those nodes take the direct formula.
__global__ void k_newton(const double* __restrict__ half, const double* __restrict__ ehalf,
                         const double* __restrict__ w, size_t n, double volume, double tol, int maxit,
                         double* partials, unsigned* counter, NewtonState* st) {
  if (st->done) return;
  const double c = st->c;
  const double q = exp(-c);
  const bool q_ok = q > 0.0 && q <= DBL_MAX;
  double v[2] = {0.0, 0.0};
  TOPO_GRID_STRIDE(i, n) {
    const double eh = ehalf[i];
    const double e = (q_ok && eh > 0.0 && eh <= DBL_MAX) ? 1.0 / (1.0 + eh * q) : expit_d(half[i] + c);
    v[0] += w[i] * e;
    v[1] += w[i] * (e * (1.0 - e));
  }
  double tot[2];
  if (finish_reduction<2>(v, partials, counter, tot)) {
    const double f = tot[0] - volume, fp = tot[1];
    st->f = f;
    st->fp = fp;
    st->iters += 1;
    if (f == 0.0) {
      st->done = 1;
      st->ok = 1;
    } else if (fp == 0.0 || !isfinite(f) || !isfinite(fp)) {
      st->done = 1;
      st->ok = 0;
    } else {
      const double p = c - f / fp;
      if (!isfinite(p)) {
        st->done = 1;
        st->ok = 0;
      } else if (fabs(p - c) < tol) {
        st->c = p;
        st->done = 1;
        st->ok = 1;
      } else {
        st->c = p;
        if (st->iters >= maxit) {
          st->done = 1;
          st->ok = 0;
        }
      }
    }
  }
}

__global__ void k_eval_volume(const double* __restrict__ half, const double* __restrict__ w, size_t n, double c,
                              double* partials, unsigned* counter, double* out) {
  double v[1] = {0.0};
  TOPO_GRID_STRIDE(i, n) v[0] += w[i] * expit_d(half[i] + c);
  double tot[1];
  if (finish_reduction<1>(v, partials, counter, tot)) out[0] = tot[0];
}

__global__ void k_emd_final(const double* __restrict__ half, const NewtonState* st, const double* cfix,
                            double* __restrict__ psi, size_t n) {
  const double c = cfix ? *cfix : st->c;
  TOPO_GRID_STRIDE(i, n) psi[i] = half[i] + c;
}

__global__ void k_emd_finish(const double* __restrict__ psi, const double* __restrict__ psi_prev,
                             const double* __restrict__ w, double* __restrict__ rho, size_t n, double* partials,
                             unsigned* counter, double* out) {
  double v[1] = {0.0};
  TOPO_GRID_STRIDE(i, n) {
    const double r = expit_d(psi[i]);
    if (rho) rho[i] = r;
    if (psi_prev) {
      const double d = r - expit_d(psi_prev[i]);
      v[0] += w[i] * d * d;
    }
  }
  if (!psi_prev) return;
  double tot[1];
  if (finish_reduction<1>(v, partials, counter, tot)) out[0] = tot[0];
}

}  // namespace

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct topo_ctx {
  int device = 0;
  int sms = 148;
  int precision = TOPO_PREC_MIXED;
  bool has_state = false;
  int nx = 0, ny = 0;
  double W = 0, H = 0, hx = 0, hy = 0;
  double E = 0, nu = 0, lmbda = 0, mu = 0, eps = 0, pmin = 1e-6;
  bool penal_set = false;
  double p = 0;
  long long launches = 0;          // kernels launched by the context itself
  bool state_ready = false;  // a state solve has set up the operator of a design
  Dir dir_p2{};
  Arena arena;
  Reducer red;
  std::string err;
  size_t nv = 0, nn2 = 0;
  double* vw = nullptr;
  double* load = nullptr;
  // state hierarchy
  std::vector<LevelSpec> sspec;
  std::vector<ElemRefs> srefs;
  std::vector<double*> skK;
  MG<float> smg32;
  MG<double> smg64;
  float* xi32 = nullptr;
  double* xi64 = nullptr;  // FP64 mode: the design copied to a fixed buffer (graphs keep their parameters)
  // per-triangle r-weighted mass matrices of the current design, [o][k][cell]
  double* rm_op64 = nullptr;  // true penalisation (residual operator): FP64, or (hi, lo) pairs when op_dd
  // mixed precision: the refinement residuals use the pair-of-FP32 operator
  // (TOPO_RESIDUAL_FP64=1: the FP64 one)
  bool op_dd = false;
  double* rm_pc64 = nullptr;  // clamped (FP64 preconditioner, FP64 mode)
  bool trace_solves = false;  // TOPO_TRACE_SOLVES=1: one line per refinement step and inner solve
  bool verify_residual = false;  // TOPO_VERIFY_RESIDUAL=1: confirm FGMRES convergence with a true residual
  // tightest relative tolerance of an FP32 inner solve (TOPO_INNER_FLOOR_STATE / _FILTER)
  double inner_floor_state = 1e-4, inner_floor_filter = 1e-5;
  // cap on the Krylov iterations of one solve (topo_set_iteration_limit; 0: the defaults)
  int iter_limit = 0;
  // lower end of the Chebyshev smoothing interval (fraction of lambda_max) per
  // hierarchy (TOPO_CHEB_LO_STATE / _FILTER): the high-contrast elasticity levels
  // converge best with a wide interval, the filter's with a narrower one
  double cheb_lo_state = 0.05, cheb_lo_filter = 0.2;
  double* fst64_stiff = nullptr;  // filter level-0 stencils (FP64): eps^2 K + M, and M
  double* fst64_mass = nullptr;
  float* rm_op32 = nullptr;   // FP32 copies for the mixed mode's FP32 operator and preconditioner
  float* rm_pc32 = nullptr;
  double* r64 = nullptr;
  double* y64 = nullptr;
  float* d32 = nullptr;
  // filter hierarchy
  std::vector<LevelSpec> fspec;
  std::vector<ElemRefs> frefs;
  std::vector<double*> fkK, fkM;
  MG<float> fmg32;
  MG<double> fmg64;
  double* fb64 = nullptr;
  // warm starts of the filter solves (topo_set_filter_warm_start): the last solution of
  // the design filter (channel 0, topo_filter_apply) and of the sensitivity filter
  // (channel 1, topo_sensitivity), each the next solve's initial guess on its channel
  bool filter_warm = false;
  // the filter solves of a mixed-precision context: FP32 multigrid CG inside FP64 FGMRES
  // (true) or FP64 multigrid CG (false, TOPO_FILTER_FP64=1); FP64 contexts always use FP64
  bool filter_mixed = false;
  // each channel's last solutions, newest first (kMaxExtrapolate + 1 buffers): the next
  // guess is their polynomial extrapolation over the design iterations,
  //   sum_i (-1)^i binom(order + 1, i + 1) x_i   (2 x1 - x2 for order 1)
  // (TOPO_EXTRAPOLATE: 0 keeps the last solution, 1 linear, ... 4; default 3)
  double* fwarm[2][kMaxExtrapolate + 1] = {};
  int fwarm_hist[2] = {0, 0};  // solutions held (0 .. kMaxExtrapolate + 1)
  int extrapolate = 3;
  double* fr64 = nullptr;
  double* fy64 = nullptr;
  float* fd32 = nullptr;
  Fgmres sgm, fgm;
  // sensitivity / design scratch
  void* sens_tri = nullptr;
  double* half = nullptr;
  double* ehalf = nullptr;  // exp(-half)
  NewtonState* nstate = nullptr;
  double* cfix = nullptr;

  ~topo_ctx() {
    if (std::getenv("TOPO_PROFILE")) {
      auto dump = [](const char* name, auto& mg) {
        mg.flush_level_profile();
        for (size_t l = 0; l < mg.level_ms.size(); ++l)
          if (mg.level_calls[l])
            std::fprintf(stderr, "[topo profile] %s level %zu (%dx%d nodes): %lld V-cycle visits, %.3f ms incl, %.2f us/visit\n",
                         name, l, mg.spec(int(l)).NX, mg.spec(int(l)).NY, mg.level_calls[l], mg.level_ms[l],
                         1e3 * mg.level_ms[l] / mg.level_calls[l]);
        std::vector<long long> cyc;
        mg.tail_profile(cyc);
        if (!cyc.empty() && cyc.back() > 0) {
          const int nl = mg.levels() - mg.tail_level();
          std::fprintf(stderr, "[topo profile] %s tail: levels %d.., %d levels, %lld launches; k-cycles per phase:",
                       name, mg.tail_level(), nl, cyc.back());
          int slot = 1;
          auto pr = [&](const char* what, int l) {
            std::fprintf(stderr, " %s%d=%.2f", what, l, 1e-3 * double(cyc[slot++]) / double(cyc.back()));
          };
          for (int l = 0; l + 1 < nl; ++l) { pr("pre", l); pr("res", l); pr("restr", l); }
          pr("coarse", nl - 1);
          for (int l = nl - 2; l >= 0; --l) { pr("prol", l); pr("first", l); pr("post", l); }
          std::fprintf(stderr, "\n");
        }
      };
      dump("state32", smg32);
      dump("state64", smg64);
      dump("filter32", fmg32);
      dump("filter64", fmg64);
    }
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
  int grid(size_t n) const { return vec_grid(n, sms); }
  // Krylov iteration cap of one solve: the context's limit if set, else the default
  int max_iterations(int dflt) const { return iter_limit > 0 ? iter_limit : dflt; }

  template <class T>
  P2Params<T> p2params(int clamp = 0, const T* rmass = nullptr) const {
    P2Params<T> P;
    std::memset(&P, 0, sizeof(P));
    P.nx = nx;
    P.ny = ny;
    P.ihx = T(1.0 / hx);
    P.ihy = T(1.0 / hy);
    const double area = 0.5 * hx * hy;
    P.lamT = T(lmbda * area);
    P.mu2T = T(2.0 * mu * area);
    P.pen = make_penal<T>(p, pmin, clamp);
    P.dir = dir_p2;
    P.rmass = rmass;
    return P;
  }

  double dot64(const double* a, const double* b, size_t n, cudaStream_t s) {
    k_dot<double, double><<<red.blocks, kVecThreads, 0, s>>>(a, b, n, red.partials, red.counter, red.out);
    cudaMemcpyAsync(red.host, red.out, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return red.host[0];
  }
};

namespace {


bool graphs_enabled() {
  const char* e = std::getenv("TOPO_GRAPHS");
  return !(e && e[0] == '0');
}
bool env_flag(const char* name, bool dflt) {
  const char* e = std::getenv(name);
  return e ? e[0] != '0' : dflt;
}

int init_common(topo_ctx* C, const topo_grid_desc* g, int precision) {
  C->trace_solves = env_flag("TOPO_TRACE_SOLVES", false);
  C->verify_residual = env_flag("TOPO_VERIFY_RESIDUAL", false);
  if (const char* e = std::getenv("TOPO_INNER_FLOOR_STATE"))
    C->inner_floor_state = std::max(1e-8, std::min(0.5, std::atof(e)));
  if (const char* e = std::getenv("TOPO_INNER_FLOOR_FILTER"))
    C->inner_floor_filter = std::max(1e-8, std::min(0.5, std::atof(e)));
  if (const char* e = std::getenv("TOPO_CHEB_LO_STATE")) C->cheb_lo_state = std::max(1e-3, std::min(0.9, std::atof(e)));
  if (const char* e = std::getenv("TOPO_CHEB_LO_FILTER")) C->cheb_lo_filter = std::max(1e-3, std::min(0.9, std::atof(e)));
  if (!g || g->nx < 1 || g->ny < 1 || !(g->width > 0) || !(g->height > 0))
    return C->fail(TOPO_ERR_ARG, "invalid grid description");
  if (precision != TOPO_PREC_FP64 && precision != TOPO_PREC_MIXED)
    return C->fail(TOPO_ERR_ARG, "unknown precision mode %d", precision);
  if (size_t(2 * g->nx + 1) * size_t(2 * g->ny + 1) > (size_t(1) << 31))
    return C->fail(TOPO_ERR_ARG, "grid too large");
  if (cudaGetDevice(&C->device) != cudaSuccess) return C->fail(TOPO_ERR_CUDA, "no CUDA device");
  cudaDeviceGetAttribute(&C->sms, cudaDevAttrMultiProcessorCount, C->device);
  C->precision = precision;
  C->nx = g->nx;
  C->ny = g->ny;
  C->W = g->width;
  C->H = g->height;
  C->hx = g->width / g->nx;
  C->hy = g->height / g->ny;
  C->nv = size_t(g->nx + 1) * (g->ny + 1);
  C->nn2 = size_t(2 * g->nx + 1) * (2 * g->ny + 1);
  C->red.init(C->arena, C->sms);
  const std::vector<double> w = vertex_weights(C->nx, C->ny, C->hx, C->hy);
  C->vw = C->arena.alloc_n<double>(C->nv);
  if (!C->vw) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  cudaMemcpy(C->vw, w.data(), C->nv * sizeof(double), cudaMemcpyHostToDevice);
  C->half = C->arena.alloc_n<double>(C->nv);
  C->ehalf = C->arena.alloc_n<double>(C->nv);
  C->nstate = C->arena.alloc_n<NewtonState>(1);
  C->cfix = C->arena.alloc_n<double>(1);
  return TOPO_OK;
}

int filter_stencils64(topo_ctx* C);

int init_filter(topo_ctx* C, double eps) {
  C->eps = eps;
  const Dir nd = no_dir(C->nx + 1, C->ny + 1);
  C->fspec = build_levels(false, C->nx, C->ny, C->hx, C->hy, nd, 1);
  const int L = int(C->fspec.size());
  C->frefs.resize(L);
  C->fkK.resize(L);
  C->fkM.resize(L);
  for (int l = 0; l < L; ++l) {
    C->frefs[l] = make_elem_refs(C->fspec[l].hx, C->fspec[l].hy, 0.0, 0.0);
    C->fkK[l] = C->arena.alloc_n<double>(C->fspec[l].ntri());
    C->fkM[l] = C->arena.alloc_n<double>(C->fspec[l].ntri());
  }
  cudaStream_t s = 0;
  k_fill<double><<<C->grid(C->fspec[0].ntri()), kVecThreads, 0, s>>>(C->fkK[0], eps * eps, C->fspec[0].ntri());
  k_fill<double><<<C->grid(C->fspec[0].ntri()), kVecThreads, 0, s>>>(C->fkM[0], 1.0, C->fspec[0].ntri());
  for (int l = 1; l < L; ++l) {
    const LevelSpec &F = C->fspec[l - 1], &Cc = C->fspec[l];
    k_coarsen_kappa<<<C->grid(Cc.ntri()), kVecThreads, 0, s>>>(C->fkK[l - 1], F.nx, F.ny, C->fkK[l], Cc.nx, Cc.ny);
    k_coarsen_kappa<<<C->grid(Cc.ntri()), kVecThreads, 0, s>>>(C->fkM[l - 1], F.nx, F.ny, C->fkM[l], Cc.nx, Cc.ny);
  }
  std::vector<const double*> kK(C->fkK.begin(), C->fkK.end()), kM(C->fkM.begin(), C->fkM.end());
  C->fb64 = C->arena.alloc_n<double>(C->nv);
  C->fr64 = C->arena.alloc_n<double>(C->nv);
  C->fy64 = C->arena.alloc_n<double>(C->nv);
  for (int k = 0; k < 2; ++k)
    for (int i = 0; i <= kMaxExtrapolate; ++i) C->fwarm[k][i] = C->arena.alloc_n<double>(C->nv);
  if (const char* e = std::getenv("TOPO_EXTRAPOLATE"))
    C->extrapolate = std::max(0, std::min(kMaxExtrapolate, std::atoi(e)));
  int st;
  C->filter_mixed = C->precision == TOPO_PREC_MIXED && !env_flag("TOPO_FILTER_FP64", false);
  if (C->filter_mixed) {
    C->fmg32.use_graphs = graphs_enabled();
    C->fmg32.fp64_solution = true;  // FGMRES directions keep the inner solutions in FP64
    C->fmg32.cheb_lo_frac = C->cheb_lo_filter;
    C->fmg32.use_tail = env_flag("TOPO_TAIL", true);
    C->fmg32.profile_levels = env_flag("TOPO_PROFILE", false);
    C->fmg32.init(C->fspec, C->frefs.data(), 0.0, 0.0, C->arena, &C->red);
    C->fmg32.set_coefficients(kK, kM);
    C->fd32 = C->arena.alloc_n<float>(C->nv);
    C->fgm.init(C->arena, C->nv);
    if (C->arena.failed()) return C->fail(TOPO_ERR_CUDA, "out of device memory");
    st = C->fmg32.setup(s);
  } else {
    C->fmg64.use_graphs = graphs_enabled();
    C->fmg64.cheb_lo_frac = C->cheb_lo_filter;
    C->fmg64.use_tail = env_flag("TOPO_TAIL", true);
    C->fmg64.profile_levels = env_flag("TOPO_PROFILE", false);
    C->fmg64.init(C->fspec, C->frefs.data(), 0.0, 0.0, C->arena, &C->red);
    C->fmg64.set_coefficients(kK, kM);
    if (C->arena.failed()) return C->fail(TOPO_ERR_CUDA, "out of device memory");
    st = C->fmg64.setup(s);
  }
  if (st) return C->fail(st == -5 ? TOPO_ERR_CUDA : TOPO_ERR_NOT_CONVERGED, "filter multigrid set-up failed (%d)", st);
  if (C->trace_solves) {
    const int lc = C->filter_mixed ? C->fmg32.coarse_cheb_level() : C->fmg64.coarse_cheb_level();
    const int dg = C->filter_mixed ? C->fmg32.coarse_cheb_deg : C->fmg64.coarse_cheb_deg;
    std::fprintf(stderr, "[topo setup] filter hierarchy: %zu levels, coarse Chebyshev at level %d (degree %d)\n",
                 C->fspec.size(), lc, dg);
  }
  if (int rc = filter_stencils64(C)) return rc;
  return C->cuda_check("filter set-up");
}

// FP64 filter operator y = (eps^2 K1 + M1) x  (or M1 x when stiff == 0)
// The filter's FP64 operators (eps^2 K + M, and M for the right-hand side) do
// not depend on the design: their 7-point stencils are assembled once.
void filter_apply64(topo_ctx* C, const double* x, double* y, bool stiff, cudaStream_t s) {
  const LevelSpec& F = C->fspec[0];
  const P1Stencil<double, 1> S{F.nx, F.ny, F.dir, stiff ? C->fst64_stiff : C->fst64_mass};
  k_p1_apply<double, 1><<<row_grid(C->nx + 1, C->ny + 1), kRowThreads, 0, s>>>(S, x, y);
}

int filter_stencils64(topo_ctx* C) {
  const LevelSpec& F = C->fspec[0];
  const size_t len = F.nn() * StencilLayout<1>::stride;
  C->fst64_stiff = C->arena.alloc_n<double>(len);
  C->fst64_mass = C->arena.alloc_n<double>(len);
  if (!C->fst64_stiff || !C->fst64_mass) return C->fail(TOPO_ERR_CUDA, "out of device memory");
  for (int stiff = 0; stiff < 2; ++stiff) {
    auto P = make_p1<double, 1>(F, C->frefs[0], nullptr, nullptr);
    P.kK_c = stiff ? C->eps * C->eps : 0.0;
    P.kM_c = 1.0;
    k_p1_stencil<double, 1><<<row_grid(F.NX, F.NY), kRowThreads>>>(P, stiff ? C->fst64_stiff : C->fst64_mass);
  }
  return C->cuda_check("filter stencils");
}

// FP32 multigrid Krylov solves inside an FP64 flexible GMRES (right
// preconditioning, restart Fgmres::m): every outer step computes the true FP64
// residual, the inner FP32 solve supplies the next search direction and the
// outer least-squares step fixes its length.  Converges like iterative
// refinement on well-conditioned problems and stays robust when the operator
// has a nearly singular or slightly negative mode that FP32 cannot resolve.
template <class Apply64>
int fgmres_ir(topo_ctx* C, MG<float>& mg, Apply64 apply64, const double* b, double* x, bool warm, size_t n,
              double rtol, Fgmres& W, int maxit, double inner_floor, SolveStats& st, cudaStream_t s) {
  constexpr int m = Fgmres::m;
  const int g = C->grid(n);
  st = SolveStats{};
  if (!warm) k_fill<double><<<g, kVecThreads, 0, s>>>(x, 0.0, n);
  const double bn = std::sqrt(C->dot64(b, b, n, s));
  if (!std::isfinite(bn)) return C->fail(TOPO_ERR_NAN, "non-finite right-hand side");
  if (bn == 0.0) {
    k_fill<double><<<g, kVecThreads, 0, s>>>(x, 0.0, n);
    return TOPO_OK;
  }
  float* r32 = mg.scratch0(4);
  double* hbuf = C->red.host;
  auto multidot = [&](int count, const double* w) {
#define TOPO_MD(K)                                                                                            \
  k_multidot<double, double, K><<<C->red.blocks, kVecThreads, 0, s>>>(W.V, n, w, n, C->red.partials, C->red.counter, \
                                                                     C->red.out)
    TOPO_DISPATCH_COUNT(count, TOPO_MD)
#undef TOPO_MD
    cudaMemcpyAsync(hbuf, C->red.out, (count + 1) * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
  };
  double prev = 0.0;
  bool capped = false;  // the context's iteration limit was reached
  for (int cycle = 0; cycle < kMaxOuter; ++cycle) {
    double* r = W.V;
    C->launches += 4;
    if (cycle == 0 && !warm) {
      cudaMemcpyAsync(r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, s);  // x = 0
    } else {
      apply64(x, W.t, s);
      k_sub<double><<<g, kVecThreads, 0, s>>>(r, b, W.t, n);
    }
    const double beta = std::sqrt(C->dot64(r, r, n, s));
    st.relres = beta / bn;
    if (C->trace_solves)
      std::fprintf(stderr, "[topo solve] fgmres cycle %d: |r|/|b| %.3e after %d inner iterations\n", cycle, beta / bn,
                   st.iterations);
    if (!std::isfinite(beta)) return C->fail(TOPO_ERR_NAN, "non-finite residual");
    if (beta <= rtol * bn) return TOPO_OK;
    if (cycle > 0 && beta > 0.9 * prev) break;  // stagnation at the FP64 residual floor
    prev = beta;
    k_scale<double><<<g, kVecThreads, 0, s>>>(r, 1.0 / beta, n);
    double H[m + 1][m] = {};
    double cs[m], sn[m], gv[m + 1] = {};
    gv[0] = beta;
    int k = 0;
    for (int j = 0; j < m; ++j) {
      st.outer += 1;
      C->launches += 6;
      double* vj = W.V + size_t(j) * n;
      double* zj = W.Z + size_t(j) * n;
      k_convert<float, double><<<g, kVecThreads, 0, s>>>(r32, vj, 1.0, n);
      // the inner solve aims at what is left of the target (|gv[j]| is the
      // current residual), but need not go much below what one refinement step
      // can use: the FP32 operator's arithmetic differs from the FP64
      // operator's by ~1e-5..1e-4 relative at smooth fields of high-contrast designs
      const double inner = std::min(0.1, std::max(inner_floor, 0.3 * rtol * bn / std::fabs(gv[j])));
      SolveStats is;
      const int rc = mg.pcg_x64(r32, zj, false, inner, maxit, is, s);
      st.iterations += is.iterations;
      if (C->trace_solves)
        std::fprintf(stderr, "[topo solve]   inner %d: tol %.1e, %d iterations, FP32 relres %.3e, rc %d\n", j, inner,
                     is.iterations, is.relres, rc);
      st.minres |= is.minres;
      if (C->iter_limit > 0 && st.iterations >= C->iter_limit) capped = true;
      if (rc == -4) return C->fail(TOPO_ERR_NAN, "non-finite value in the FP32 inner solve");
      if (rc == -5) return C->fail(TOPO_ERR_CUDA, "inner solve: CUDA graph recording or launch failed");
      double* w = W.V + size_t(j + 1) * n;
      apply64(zj, w, s);
      // classical Gram-Schmidt; a second pass only when the first one cancelled
      // more than half of w (Kahan's "twice is enough" test)
      double h[m + 1] = {};
      double hn = 0.0;
      for (int pass = 0; pass < 2; ++pass) {
        multidot(j + 1, w);
        MultiCoef cf{};
        double hh = 0.0;
        for (int i = 0; i <= j; ++i) {
          cf.c[i] = hbuf[i];
          h[i] += hbuf[i];
          hh += hbuf[i] * hbuf[i];
        }
        const double ww = hbuf[j + 1];
#define TOPO_SM(K) k_sub_multi<double, double, K><<<g, kVecThreads, 0, s>>>(w, W.V, n, cf, n)
        TOPO_DISPATCH_COUNT(j + 1, TOPO_SM)
#undef TOPO_SM
        const double est = ww - hh;
        if (pass == 0 && est >= 0.5 * ww) {
          hn = std::sqrt(est);
          break;
        }
        if (pass == 1) hn = std::sqrt(C->dot64(w, w, n, s));
      }
      if (!std::isfinite(hn)) return C->fail(TOPO_ERR_NAN, "non-finite Krylov vector");
      for (int i = 0; i <= j; ++i) H[i][j] = h[i];
      H[j + 1][j] = hn;
      if (hn > 0) k_scale<double><<<g, kVecThreads, 0, s>>>(w, 1.0 / hn, n);
      for (int i = 0; i < j; ++i) {  // previous rotations
        const double t0 = cs[i] * H[i][j] + sn[i] * H[i + 1][j];
        H[i + 1][j] = -sn[i] * H[i][j] + cs[i] * H[i + 1][j];
        H[i][j] = t0;
      }
      const double den = std::hypot(H[j][j], H[j + 1][j]);
      cs[j] = den > 0 ? H[j][j] / den : 1.0;
      sn[j] = den > 0 ? H[j + 1][j] / den : 0.0;
      H[j][j] = den;
      H[j + 1][j] = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      k = j + 1;
      if (std::fabs(gv[j + 1]) <= 0.5 * rtol * bn || hn == 0.0 || capped) break;
    }
    double y[m] = {};
    for (int i = k - 1; i >= 0; --i) {
      double acc = gv[i];
      for (int l = i + 1; l < k; ++l) acc -= H[i][l] * y[l];
      y[i] = (H[i][i] != 0.0) ? acc / H[i][i] : 0.0;
    }
    MultiCoef cf{};
    for (int i = 0; i < k; ++i) cf.c[i] = y[i];
#define TOPO_AM(K) k_add_multi<double, double, K><<<g, kVecThreads, 0, s>>>(x, W.Z, n, cf, n)
    TOPO_DISPATCH_COUNT(k, TOPO_AM)
#undef TOPO_AM
    // the least-squares residual is the FP64 residual of the updated x up to the
    // Arnoldi relation's rounding (~1e-11 relative here): accept it without
    // another operator apply unless asked to verify (TOPO_VERIFY_RESIDUAL=1)
    if (k > 0 && std::fabs(gv[k]) <= 0.5 * rtol * bn && !C->verify_residual) {
      st.relres = std::fabs(gv[k]) / bn;
      if (C->trace_solves)
        std::fprintf(stderr, "[topo solve] fgmres converged: estimated |r|/|b| %.3e after %d inner iterations\n",
                     st.relres, st.iterations);
      return TOPO_OK;
    }
    if (capped) break;
  }
  apply64(x, W.t, s);
  k_sub<double><<<g, kVecThreads, 0, s>>>(W.V, b, W.t, n);
  st.relres = std::sqrt(C->dot64(W.V, W.V, n, s)) / bn;
  if (st.relres <= rtol) return TOPO_OK;
  return C->fail(TOPO_ERR_NOT_CONVERGED, "refinement did not reach rtol %.3g (relres %.3g after %d inner iterations)",
                 rtol, st.relres, st.iterations);
}

// channel: 0 design filter, 1 sensitivity filter (warm-started from the channel's last
// solution when topo_set_filter_warm_start is on), -1 no warm start
int filter_solve_impl(topo_ctx* C, const double* b, double* xi, double rtol, int* iters, cudaStream_t s,
                      int channel = -1) {
  SolveStats st;
  int rc;
  const int hist = (C->filter_warm && channel >= 0) ? C->fwarm_hist[channel] : 0;
  const bool warm = hist > 0;
  if (warm) {
    const int order = std::min(C->extrapolate, hist - 1);
    if (order > 0) {
      Extrapolation ex{};
      ex.n = order + 1;
      double binom = 1.0;  // binom(order + 1, i + 1), built up term by term
      for (int i = 0; i <= order; ++i) {
        binom = binom * double(order + 1 - i) / double(i + 1);
        ex.x[i] = C->fwarm[channel][i];
        ex.c[i] = (i % 2 ? -1.0 : 1.0) * binom;
      }
      k_extrapolate<<<C->grid(C->nv), kVecThreads, 0, s>>>(xi, ex, C->nv);
      C->launches += 1;
    } else {
      cudaMemcpyAsync(xi, C->fwarm[channel][0], C->nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    }
  }
  if (channel >= 0) C->fwarm_hist[channel] = 0;  // until this solve succeeds
  if (C->filter_mixed) {
    auto ap = [C](const double* x, double* y, cudaStream_t ss) { filter_apply64(C, x, y, true, ss); };
    rc = fgmres_ir(C, C->fmg32, ap, b, xi, warm, C->nv, rtol, C->fgm, C->max_iterations(kFilterMaxIt),
                   C->inner_floor_filter, st, s);
  } else {
    rc = C->fmg64.pcg(b, xi, warm, rtol, C->max_iterations(kFilterMaxIt), st, s);
    if (rc == -4) rc = C->fail(TOPO_ERR_NAN, "non-finite value in the filter solve");
    else if (rc == -5) rc = C->fail(TOPO_ERR_CUDA, "filter solve: CUDA graph recording or launch failed");
    else if (rc) rc = C->fail(TOPO_ERR_NOT_CONVERGED, "filter CG did not converge (relres %.3g)", st.relres);
  }
  if (iters) *iters = st.iterations;
  if (rc) return rc;
  if (C->filter_warm && channel >= 0) {
    // shift the history by one (the oldest buffer takes this solution)
    double** h = C->fwarm[channel];
    double* oldest = h[kMaxExtrapolate];
    for (int i = kMaxExtrapolate; i > 0; --i) h[i] = h[i - 1];
    h[0] = oldest;
    cudaMemcpyAsync(h[0], xi, C->nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    C->fwarm_hist[channel] = std::min(kMaxExtrapolate + 1, hist + 1);
  }
  return C->cuda_check("filter solve");
}

int state_setup(topo_ctx* C, const double* xi, cudaStream_t s) {
  const int L = int(C->sspec.size());
  Penal<double> pen = make_penal<double>(C->p, C->pmin, 1);
  const size_t ncell = size_t(C->nx) * C->ny;
  const Penal<double> pen_op = make_penal<double>(C->p, C->pmin, 0);
  if (C->op_dd && pen_op.ip >= 1 && pen_op.ip <= 16)
    k_cell_rmass_kappa_dd<<<C->grid(ncell), kVecThreads, 0, s>>>(C->nx, C->ny, pen_op.ip, dd(C->pmin),
                                                                 dd(1.0 - C->pmin), xi,
                                                                 reinterpret_cast<dd*>(C->rm_op64), C->skK[1]);
  else if (C->op_dd)
    k_cell_rmass_kappa<dd><<<C->grid(ncell), kVecThreads, 0, s>>>(C->nx, C->ny, pen_op, xi,
                                                                  reinterpret_cast<dd*>(C->rm_op64), C->skK[1]);
  else
    k_cell_rmass_kappa<double><<<C->grid(ncell), kVecThreads, 0, s>>>(C->nx, C->ny, pen_op, xi, C->rm_op64,
                                                                      C->skK[1]);
  C->launches += 1 + (L - 2);
  for (int l = 2; l < L; ++l) {
    const LevelSpec &F = C->sspec[l - 1], &Cc = C->sspec[l];
    k_coarsen_kappa<<<C->grid(Cc.ntri()), kVecThreads, 0, s>>>(C->skK[l - 1], F.nx, F.ny, C->skK[l], Cc.nx, Cc.ny);
  }
  int st;
  if (C->trace_solves) {
    const auto t0 = std::chrono::steady_clock::now();
    cudaStreamSynchronize(s);
    std::fprintf(stderr, "[topo setup] kappa, FP64 mass (wait)  %.3f ms\n",
                 std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
  if (C->precision == TOPO_PREC_MIXED) {
    // the r-weighted mass matrices (12 values per cell) evaluated once per
    // design by the FP32 operator's own code and read by it afterwards instead
    // of seven r(xi) evaluations per triangle per apply (TOPO_RMASS32=0: on the fly)
    k_convert<float, double><<<C->grid(C->nv), kVecThreads, 0, s>>>(C->xi32, xi, 1.0, C->nv);
    if (C->rm_op32) {
      k_cell_rmass32<<<C->grid(ncell), kVecThreads, 0, s>>>(C->nx, C->ny, C->p2params<float>(0).pen,
                                                             C->p2params<float>(1).pen, C->xi32, C->rm_op32,
                                                             C->rm_pc32);
      C->launches += 1;
    }
    C->smg32.set_p2(C->p2params<float>(0, C->rm_op32), C->p2params<float>(1, C->rm_pc32), C->xi32);
    st = C->smg32.setup(s);
  } else {
    k_cell_rmass<double><<<C->grid(ncell), kVecThreads, 0, s>>>(C->nx, C->ny, pen, xi, C->rm_pc64);
    cudaMemcpyAsync(C->xi64, xi, C->nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
    C->smg64.set_p2(C->p2params<double>(0, C->rm_op64), C->p2params<double>(1, C->rm_pc64), C->xi64);
    st = C->smg64.setup(s);
  }
  if (st == -5) return C->fail(TOPO_ERR_CUDA, "state set-up: CUDA error");
  if (st) return C->fail(TOPO_ERR_NOT_CONVERGED, "state set-up: coarse operator not positive definite");
  return TOPO_OK;
}

// P2-lattice arrays are read and written two components at a time (16-byte
// accesses in FP64): their base must be 16-byte aligned (cudaMalloc and torch
// allocations are; a view at an odd element offset is not)
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <class F>
int guarded(topo_ctx* C, F&& f) {
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

}  // namespace

// ---------------------------------------------------------------------------
// exported entry points
// ---------------------------------------------------------------------------
extern "C" {

topo_ctx* topo_create(const topo_grid_desc* grid, const topo_material* mat, const topo_bc_desc* bc,
                      const topo_load_desc* load, int precision, int* status) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());  // set-up allocates and frees
  topo_ctx* C = nullptr;
  int rc = TOPO_OK;
  try {
    C = new topo_ctx();
    rc = init_common(C, grid, precision);
    if (!rc && !mat) rc = C->fail(TOPO_ERR_ARG, "material description missing");
    if (!rc) {
      if (!(mat->poisson_ratio < 0.5) || !(mat->young_modulus > 0) || !(mat->filter_radius >= 0))
        rc = C->fail(TOPO_ERR_ARG, "invalid material parameters");
    }
    if (!rc) {
      C->has_state = true;
      C->E = mat->young_modulus;
      C->nu = mat->poisson_ratio;
      C->mu = C->E / (2 * (1 + C->nu));                 // FEM_src/elasisity_problem.py:97-99
      C->lmbda = C->mu * C->nu / (0.5 - C->nu);
      C->pmin = mat->penal_min > 0 ? mat->penal_min : 1e-6;
      std::string msg;
      if (make_p2_dir(C->nx, C->ny, C->hx, C->hy, bc, C->dir_p2, msg)) rc = C->fail(TOPO_ERR_ARG, "%s", msg.c_str());
    }
    if (!rc && load) {
      if (load->n_tractions < 0 || (load->n_tractions > 0 && !load->tractions))
        rc = C->fail(TOPO_ERR_ARG, "invalid traction list");
      for (int k = 0; !rc && k < load->n_tractions; ++k) {
        const int sd = load->tractions[k].side;
        if (sd != TOPO_SIDE_LEFT && sd != TOPO_SIDE_RIGHT && sd != TOPO_SIDE_TOP && sd != TOPO_SIDE_BOTTOM)
          rc = C->fail(TOPO_ERR_ARG, "Malformed side: %d", sd);
      }
    }
    if (!rc) {
      std::vector<double> b;
      assemble_load(C->nx, C->ny, C->W, C->H, C->dir_p2, load, b);
      C->load = C->arena.alloc_n<double>(b.size());
      if (!C->load) rc = C->fail(TOPO_ERR_CUDA, "out of device memory");
      else cudaMemcpy(C->load, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (!rc) {
      C->sspec = build_levels(true, C->nx, C->ny, C->hx, C->hy, C->dir_p2, 2);
      const int L = int(C->sspec.size());
      C->srefs.resize(L);
      C->skK.assign(L, nullptr);
      for (int l = 0; l < L; ++l) {
        C->srefs[l] = make_elem_refs(C->sspec[l].hx, C->sspec[l].hy, C->lmbda, C->mu);
        if (l > 0) C->skK[l] = C->arena.alloc_n<double>(C->sspec[l].ntri());
      }
      std::vector<const double*> kK(C->skK.begin(), C->skK.end()), kM(L, nullptr);
      const size_t n = 2 * C->nn2;
      const size_t ncell = size_t(C->nx) * C->ny;
      C->rm_op64 = C->arena.alloc_n<double>(12 * ncell);
      if (precision == TOPO_PREC_FP64) C->rm_pc64 = C->arena.alloc_n<double>(12 * ncell);
      if (precision == TOPO_PREC_MIXED && env_flag("TOPO_RMASS32", true)) {
        C->rm_op32 = C->arena.alloc_n<float>(12 * ncell);
        C->rm_pc32 = C->arena.alloc_n<float>(12 * ncell);
      }
      C->r64 = C->arena.alloc_n<double>(n);
      C->y64 = C->arena.alloc_n<double>(n);
      if (precision == TOPO_PREC_MIXED) {
        C->op_dd = !env_flag("TOPO_RESIDUAL_FP64", false);
        if (C->op_dd) p2_dd_prime();
        C->smg32.use_graphs = graphs_enabled();
        C->smg32.fp64_solution = true;
        C->smg32.cheb_lo_frac = C->cheb_lo_state;
        C->smg32.trace_setup = C->trace_solves;
        C->smg32.use_tail = env_flag("TOPO_TAIL", true);
        C->smg32.profile_levels = env_flag("TOPO_PROFILE", false);
        C->smg32.init(C->sspec, C->srefs.data(), C->lmbda, C->mu, C->arena, &C->red);
        C->smg32.set_coefficients(kK, kM);
        C->xi32 = C->arena.alloc_n<float>(C->nv);
        C->d32 = C->arena.alloc_n<float>(n);
        C->sgm.init(C->arena, n);
        C->sens_tri = C->arena.alloc_n<float>(size_t(3) * C->sspec[0].ntri());
      } else {
        C->smg64.use_graphs = graphs_enabled();
        C->smg64.cheb_lo_frac = C->cheb_lo_state;
        C->smg64.use_tail = env_flag("TOPO_TAIL", true);
        C->smg64.profile_levels = env_flag("TOPO_PROFILE", false);
        C->smg64.init(C->sspec, C->srefs.data(), C->lmbda, C->mu, C->arena, &C->red);
        C->smg64.set_coefficients(kK, kM);
        C->xi64 = C->arena.alloc_n<double>(C->nv);
        C->sens_tri = C->arena.alloc_n<double>(size_t(3) * C->sspec[0].ntri());
      }
      if (C->arena.failed()) rc = C->fail(TOPO_ERR_CUDA, "out of device memory");
    }
    if (!rc) rc = init_filter(C, mat->filter_radius);
    if (!rc) {
      const cudaError_t e = settle_setup_stream();
      if (e != cudaSuccess) rc = C->fail(TOPO_ERR_CUDA, "set-up: %s", cudaGetErrorString(e));
    }
  } catch (...) {
    rc = TOPO_ERR_CUDA;
  }
  if (status) *status = rc;
  if (rc) {
    if (C && status) {
      // keep the message reachable through a failed create: print it
      std::fprintf(stderr, "topo_create: %s\n", C->err.c_str());
    }
    delete C;
    return nullptr;
  }
  return C;
}

topo_ctx* topo_create_filter(const topo_grid_desc* grid, double epsilon, int precision, int* status) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());  // set-up allocates and frees
  topo_ctx* C = nullptr;
  int rc = TOPO_OK;
  try {
    C = new topo_ctx();
    rc = init_common(C, grid, precision);
    if (!rc && !(epsilon >= 0)) rc = C->fail(TOPO_ERR_ARG, "invalid filter radius");
    if (!rc) rc = init_filter(C, epsilon);
    if (!rc) {
      const cudaError_t e = settle_setup_stream();
      if (e != cudaSuccess) rc = C->fail(TOPO_ERR_CUDA, "set-up: %s", cudaGetErrorString(e));
    }
  } catch (...) {
    rc = TOPO_ERR_CUDA;
  }
  if (status) *status = rc;
  if (rc) {
    if (C) std::fprintf(stderr, "topo_create_filter: %s\n", C->err.c_str());
    delete C;
    return nullptr;
  }
  return C;
}

void topo_destroy(topo_ctx* ctx) {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  delete ctx;
}

const char* topo_last_error(const topo_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int topo_sizes(const topo_ctx* ctx, int64_t* n_vertices, int64_t* n_dofs) {
  if (!ctx) return TOPO_ERR_ARG;
  if (n_vertices) *n_vertices = int64_t(ctx->nv);
  if (n_dofs) *n_dofs = int64_t(2 * ctx->nn2);
  return TOPO_OK;
}

int topo_set_filter_warm_start(topo_ctx* ctx, int enable) {
  return guarded(ctx, [&]() {
    ctx->filter_warm = enable != 0;
    ctx->fwarm_hist[0] = ctx->fwarm_hist[1] = 0;
    return TOPO_OK;
  });
}

int topo_set_iteration_limit(topo_ctx* ctx, int max_iterations) {
  return guarded(ctx, [&]() {
    if (max_iterations < 0) return ctx->fail(TOPO_ERR_ARG, "negative iteration limit");
    ctx->iter_limit = max_iterations;
    return TOPO_OK;
  });
}

int topo_set_penalization(topo_ctx* ctx, double p) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context has no penaliser");
    if (!std::isfinite(p)) return ctx->fail(TOPO_ERR_ARG, "non-finite penalisation");
    ctx->p = p;
    ctx->penal_set = true;
    return TOPO_OK;
  });
}

int topo_filter_apply(topo_ctx* ctx, const double* f, double* xi, double rtol, int* iters, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!f || !xi || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid filter arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    filter_apply64(ctx, f, ctx->fb64, false, s);
    ctx->launches += 1;
    return filter_solve_impl(ctx, ctx->fb64, xi, rtol, iters, s, 0);
  });
}

int topo_mass_apply(topo_ctx* ctx, const double* x, double* y, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!x || !y) return ctx->fail(TOPO_ERR_ARG, "invalid mass-apply arguments");
    filter_apply64(ctx, x, y, false, reinterpret_cast<cudaStream_t>(stream));
    ctx->launches += 1;
    return ctx->cuda_check("mass apply");
  });
}

int topo_filter_solve(topo_ctx* ctx, const double* b, double* xi, double rtol, int* iters, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!b || !xi || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid filter arguments");
    return filter_solve_impl(ctx, b, xi, rtol, iters, reinterpret_cast<cudaStream_t>(stream));
  });
}

int topo_state_solve(topo_ctx* ctx, const double* xi, double* u, double rtol, int flags, int* iters,
                     topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!xi || !u || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid state-solve arguments");
    if (!aligned16(u)) return ctx->fail(TOPO_ERR_ARG, "displacement array must be 16-byte aligned");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const auto t0 = std::chrono::steady_clock::now();
    int rc = state_setup(ctx, xi, s);
    if (rc) return rc;
    if (ctx->trace_solves) {
      cudaStreamSynchronize(s);
      std::fprintf(stderr, "[topo solve] state set-up %.3f ms\n",
                   std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    ctx->state_ready = true;
    const size_t n = 2 * ctx->nn2;
    const bool warm = (flags & TOPO_SOLVE_WARM) != 0;
    SolveStats st;
    if (ctx->precision == TOPO_PREC_MIXED) {
      if (ctx->op_dd) {
        const P2Params<dd> Pdd = ctx->p2params<dd>(0, reinterpret_cast<const dd*>(ctx->rm_op64));
        auto ap = [Pdd](const double* x, double* y, cudaStream_t ss) { p2_apply_dd(Pdd, x, y, ss); };
        rc = fgmres_ir(ctx, ctx->smg32, ap, ctx->load, u, warm, n, rtol, ctx->sgm,
                       ctx->max_iterations(kStateMaxIt), ctx->inner_floor_state, st, s);
      } else {
        const P2Params<double> P64 = ctx->p2params<double>(0, ctx->rm_op64);
        auto ap = [P64, xi](const double* x, double* y, cudaStream_t ss) { p2_apply_f64(P64, xi, x, y, ss); };
        rc = fgmres_ir(ctx, ctx->smg32, ap, ctx->load, u, warm, n, rtol, ctx->sgm,
                       ctx->max_iterations(kStateMaxIt), ctx->inner_floor_state, st, s);
      }
    } else {
      rc = ctx->smg64.pcg(ctx->load, u, warm, rtol, ctx->max_iterations(kStateMaxIt), st, s);
      if (rc == -4) rc = ctx->fail(TOPO_ERR_NAN, "non-finite value in the state solve");
      else if (rc == -5) rc = ctx->fail(TOPO_ERR_CUDA, "state solve: CUDA graph recording or launch failed");
      else if (rc) rc = ctx->fail(TOPO_ERR_NOT_CONVERGED, "state CG did not converge (relres %.3g)", st.relres);
    }
    if (iters) *iters = st.iterations;
    if (ctx->trace_solves) {
      cudaStreamSynchronize(s);
      std::fprintf(stderr, "[topo solve] state solve %.3f ms (set-up included), %d inner iterations, %d outer steps\n",
                   std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                   st.iterations, st.outer);
    }
    if (rc) return rc;
    return ctx->cuda_check("state solve");
  });
}

int topo_compliance(topo_ctx* ctx, const double* u, double* compliance, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!u || !compliance) return ctx->fail(TOPO_ERR_ARG, "invalid compliance arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    ctx->launches += 1;
    k_dot<double, double><<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->load, u, 2 * ctx->nn2, ctx->red.partials,
                                                                ctx->red.counter, compliance);
    return ctx->cuda_check("compliance");
  });
}

int topo_sensitivity_rhs(topo_ctx* ctx, const double* u, const double* xi, double* b, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!u || !xi || !b) return ctx->fail(TOPO_ERR_ARG, "invalid sensitivity arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t nt = size_t(2) * ctx->nx * ctx->ny;
    const double area = 0.5 * ctx->hx * ctx->hy;
    ctx->launches += 2;
    // both kernels: u (FP64) and the design read, the CG1 right-hand side written
    KClock kc(s, "sensitivity (moments + vertex gather)", 0, (2.0 * ctx->nn2 + 2.0 * ctx->nv) * 8.0);
    if (ctx->precision == TOPO_PREC_MIXED) {
      float* tri = static_cast<float*>(ctx->sens_tri);
      k_sens_tri<float><<<ctx->grid(nt / 2), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, 1.0 / ctx->hx, 1.0 / ctx->hy,
                                                               float(ctx->lmbda), float(ctx->mu), float(area),
                                                               make_penal<float>(ctx->p, ctx->pmin), u, xi, tri);
      k_vertex_gather3<float><<<ctx->grid(ctx->nv), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, tri, b);
    } else {
      double* tri = static_cast<double*>(ctx->sens_tri);
      k_sens_tri<double><<<ctx->grid(nt / 2), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, 1.0 / ctx->hx, 1.0 / ctx->hy,
                                                                ctx->lmbda, ctx->mu, area,
                                                                make_penal<double>(ctx->p, ctx->pmin), u, xi, tri);
      k_vertex_gather3<double><<<ctx->grid(ctx->nv), kVecThreads, 0, s>>>(ctx->nx, ctx->ny, tri, b);
    }
    return ctx->cuda_check("sensitivity");
  });
}

int topo_sensitivity(topo_ctx* ctx, const double* u, const double* xi, double* g, double rtol, int* iters,
                     topo_stream_t stream) {
  int rc = topo_sensitivity_rhs(ctx, u, xi, ctx ? ctx->fb64 : nullptr, stream);
  if (rc) return rc;
  return guarded(ctx, [&]() {
    if (!g || !(rtol > 0)) return ctx->fail(TOPO_ERR_ARG, "invalid sensitivity arguments");
    return filter_solve_impl(ctx, ctx->fb64, g, rtol, iters, reinterpret_cast<cudaStream_t>(stream), 1);
  });
}

int topo_emd_step(topo_ctx* ctx, const double* psi_prev, const double* g, double alpha, double volume, double* psi,
                  double* c_out, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!psi_prev || !g || !psi || !std::isfinite(alpha) || !std::isfinite(volume))
      return ctx->fail(TOPO_ERR_ARG, "invalid step arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const size_t n = ctx->nv;
    k_emd_half<<<ctx->grid(n), kVecThreads, 0, s>>>(psi_prev, g, alpha, ctx->half, ctx->ehalf, n);
    ctx->launches += 2;  // half step and the final update
    NewtonState init{};
    init.c = 0.0;
    cudaMemcpyAsync(ctx->nstate, &init, sizeof(init), cudaMemcpyHostToDevice, s);
    NewtonState hs{};
    const int maxit = 50;  // scipy.optimize.newton default
    for (int launched = 0; launched < maxit;) {
      const int chunk = std::min(8, maxit - launched);
      ctx->launches += chunk;
      for (int k = 0; k < chunk; ++k) {
        if (launched == 0 && k == 0) {
          // the clock times the first evaluation (later launches of a chunk may find Newton done)
          KClock kc(s, "Newton evaluation (volume and its derivative)", 0, 2.0 * n * 8.0);
          k_newton<<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->half, ctx->ehalf, ctx->vw, n, volume, 1e-12, maxit,
                                                            ctx->red.partials, ctx->red.counter, ctx->nstate);
        } else {
          k_newton<<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->half, ctx->ehalf, ctx->vw, n, volume, 1e-12, maxit,
                                                            ctx->red.partials, ctx->red.counter, ctx->nstate);
        }
      }
      launched += chunk;
      cudaMemcpyAsync(&hs, ctx->nstate, sizeof(hs), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return ctx->cuda_check("projection");
      if (hs.done) break;
    }
    double c = hs.c;
    if (!(hs.done && hs.ok)) {
      // bracketing fallback (src/utils.py:138-157): grow [-r, r] from 2 while r <= 2000
      auto F = [&](double cc) {
        ctx->launches += 1;
        k_eval_volume<<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->half, ctx->vw, n, cc, ctx->red.partials,
                                                                ctx->red.counter, ctx->red.out);
        cudaMemcpyAsync(ctx->red.host, ctx->red.out, sizeof(double), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        return ctx->red.host[0] - volume;
      };
      double r = 2.0, lo = 0, hi = 0, flo = 0, fhi = 0;
      bool found = false;
      while (r <= 2000.0) {
        flo = F(-r);
        fhi = F(r);
        if (std::isfinite(flo) && std::isfinite(fhi) && ((flo <= 0 && fhi >= 0) || (flo >= 0 && fhi <= 0))) {
          found = true;
          lo = -r;
          hi = r;
          break;
        }
        r *= 2;
      }
      // smart_brentq's error when no sign change is found up to the largest radius
      // (src/utils.py:147-151); the caller's design loop stops with this message
      if (!found) return ctx->fail(TOPO_ERR_PROJECTION, "f(-max_radius) and f(max_radius) must have different signs!");
      if (flo == 0) c = lo;
      else if (fhi == 0) c = hi;
      else {
        for (int it = 0; it < 200 && hi - lo > 2e-12; ++it) {
          const double mid = 0.5 * (lo + hi), fm = F(mid);
          if (fm == 0) { lo = hi = mid; break; }
          if ((fm < 0) == (flo < 0)) { lo = mid; flo = fm; }
          else hi = mid;
        }
        c = 0.5 * (lo + hi);
      }
      cudaMemcpyAsync(ctx->cfix, &c, sizeof(double), cudaMemcpyHostToDevice, s);
      k_emd_final<<<ctx->grid(n), kVecThreads, 0, s>>>(ctx->half, ctx->nstate, ctx->cfix, psi, n);
    } else {
      k_emd_final<<<ctx->grid(n), kVecThreads, 0, s>>>(ctx->half, ctx->nstate, nullptr, psi, n);
    }
    if (c_out) *c_out = c;
    return ctx->cuda_check("projection");
  });
}

int topo_emd_finish(topo_ctx* ctx, const double* psi, const double* psi_prev, double* rho, double* delta,
                    topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!psi) return ctx->fail(TOPO_ERR_ARG, "invalid arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    ctx->launches += 1;
    k_emd_finish<<<ctx->red.blocks, kVecThreads, 0, s>>>(psi, psi_prev, ctx->vw, rho, ctx->nv, ctx->red.partials,
                                                         ctx->red.counter, ctx->red.out);
    if (psi_prev && delta) {
      cudaMemcpyAsync(ctx->red.host, ctx->red.out, sizeof(double), cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      *delta = std::sqrt(ctx->red.host[0]);
    }
    return ctx->cuda_check("design update");
  });
}

int topo_integrate(topo_ctx* ctx, const double* f, double* out, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!f || !out) return ctx->fail(TOPO_ERR_ARG, "invalid integrate arguments");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    ctx->launches += 1;
    k_dot<double, double><<<ctx->red.blocks, kVecThreads, 0, s>>>(ctx->vw, f, ctx->nv, ctx->red.partials,
                                                                ctx->red.counter, out);
    return ctx->cuda_check("integrate");
  });
}

int topo_state_warm_start(topo_ctx* ctx, const double* const* history, int count, double* u,
                          topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!history || !u || count < 1 || count > kMaxExtrapolate + 1)
      return ctx->fail(TOPO_ERR_ARG, "invalid solution history");
    Extrapolation ex{};
    ex.n = count;
    double binom = 1.0;  // binom(count, i + 1), built up term by term (exact: small integers)
    for (int i = 0; i < count; ++i) {
      if (!history[i]) return ctx->fail(TOPO_ERR_ARG, "invalid solution history");
      binom = binom * double(count - i) / double(i + 1);
      ex.x[i] = history[i];
      ex.c[i] = (i % 2 ? -1.0 : 1.0) * binom;
    }
    const size_t n = 2 * ctx->nn2;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    k_extrapolate<<<ctx->grid(n), kVecThreads, 0, s>>>(u, ex, n);
    ctx->launches += 1;
    return ctx->cuda_check("state warm start");
  });
}

int topo_apply_state(topo_ctx* ctx, const double* xi, const double* u, double* y, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!xi || !u || !y) return ctx->fail(TOPO_ERR_ARG, "invalid apply arguments");
    if (!aligned16(u) || !aligned16(y)) return ctx->fail(TOPO_ERR_ARG, "displacement arrays must be 16-byte aligned");
    p2_apply_f64(ctx->p2params<double>(), xi, u, y, reinterpret_cast<cudaStream_t>(stream));
    ctx->launches += 1;
    return ctx->cuda_check("apply");
  });
}

int topo_time_operator(topo_ctx* ctx, double* ms, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state || !ms) return ctx->fail(TOPO_ERR_ARG, "invalid arguments");
    if (!ctx->penal_set) return ctx->fail(TOPO_ERR_STATE, "You must set penalization before calling penalizer");
    if (!ctx->state_ready) return ctx->fail(TOPO_ERR_STATE, "no state solve has set up the operator yet");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (ctx->precision == TOPO_PREC_MIXED) {
      float* x = ctx->smg32.scratch0(7);
      float* y = ctx->smg32.scratch0(8);
      cudaEventRecord(e0, s);
      p2_apply_f32(ctx->p2params<float>(0, ctx->rm_op32), ctx->xi32, x, y, s);
      cudaEventRecord(e1, s);
    } else {
      cudaEventRecord(e0, s);
      p2_apply_f64(ctx->p2params<double>(0, ctx->rm_op64), ctx->xi64, ctx->r64, ctx->y64, s);
      cudaEventRecord(e1, s);
    }
    ctx->launches += 1;
    cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t;
    return ctx->cuda_check("time operator");
  });
}

int topo_launch_count(const topo_ctx* ctx, int64_t* launches) {
  if (!ctx || !launches) return TOPO_ERR_ARG;
  *launches = ctx->launches + ctx->smg32.launches + ctx->smg64.launches + ctx->fmg32.launches + ctx->fmg64.launches;
  return TOPO_OK;
}

int topo_load_vector(topo_ctx* ctx, double* b, topo_stream_t stream) {
  return guarded(ctx, [&]() {
    if (!ctx->has_state) return ctx->fail(TOPO_ERR_STATE, "filter-only context");
    if (!b) return ctx->fail(TOPO_ERR_ARG, "null output");
    cudaMemcpyAsync(b, ctx->load, 2 * ctx->nn2 * sizeof(double), cudaMemcpyDeviceToDevice,
                    reinterpret_cast<cudaStream_t>(stream));
    return ctx->cuda_check("load vector");
  });
}

}  // extern "C"
