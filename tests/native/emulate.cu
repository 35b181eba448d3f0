// CPU emulation of the topomax_gb300 kernels, for the CPU test suite only.
//
// The device kernels are written as load / compute / gather phase functions
// (topo_p2.cuh, topo_p1.cuh) that are __host__ __device__.  This file runs
// those phases sequentially per tile on the host -- every thread of phase k
// before any thread of phase k+1, which is exactly the ordering the kernels'
// __syncthreads give -- so the tiling and index logic can be compared with
// the FP64 oracle without a GPU.  It is never linked into the product library.
#include <cstring>
#include <memory>
#include <type_traits>
#include <vector>

#include "topo_mg.h"
#include "topo_p1.cuh"
#include "topo_p2.cuh"
#include "topo_p1march.cuh"
#include "topo_setup.h"
#include "topo_fluid.cuh"
#include "topo_fluid_setup.h"

using namespace topo;

namespace {
constexpr int kDirInts = 5 + 2 * kMaxDirPoints;

Dir dir_from(const int* d) {
  Dir r;
  std::memset(&r, 0, sizeof(r));
  r.x_lo = d[0];
  r.y_lo = d[1];
  r.x_hi_from = d[2];
  r.y_hi_from = d[3];
  r.npts = d[4];
  for (int k = 0; k < 2 * kMaxDirPoints; ++k) r.pts[k] = d[5 + k];
  return r;
}

void dir_to(const Dir& r, int* d) {
  d[0] = r.x_lo;
  d[1] = r.y_lo;
  d[2] = r.x_hi_from;
  d[3] = r.y_hi_from;
  d[4] = r.npts;
  for (int k = 0; k < 2 * kMaxDirPoints; ++k) d[5 + k] = r.pts[k];
}

// Warps of the last emulated P2 march that took the lean phases.
static long lean_warps = 0;
// Segment length of the emulated P2 marches (0: the kernel's one-wave rule).
static int seg_override = 0;

// Runs the column-march P2 kernel on the CPU: the 32 lanes of a warp execute
// each phase in turn and the shuffles become copies between lane states.
template <class T>
void p2_run_io(const P2Params<T>& P, const T* xi, P2Io<T> io, int seg = 0) {
  P2March<T>::prepare(io);
  lean_warps = 0;
  if (seg <= 0) seg = seg_override > 0 ? std::min(seg_override, P.ny) : p2_march_segment(P.nx, P.ny, 4, 5);
  const int nxw = (P.nx + 1 + P2M_OWN - 1) / P2M_OWN;
  const bool operand = io.mode != kP2Diag;
  std::vector<P2Lane<T>> L(32);
  T acc[2] = {T(0), T(0)};
  auto down = [&](int r0) {
    for (int l = 0; l < 32; ++l) {
      const int src = l < 31 ? l + 1 : l;  // a shuffle from beyond the warp returns the own value
      if (L[l].edge) continue;
      if (operand)
        for (int r = r0; r <= 2; ++r)
          for (int c = 0; c < 2; ++c) L[l].U[r][2][c] = L[src].U[r][0][c];
      for (int r = (r0 == 0 ? 0 : 1); r <= 1; ++r) L[l].X[r][1] = L[src].X[r][0];
    }
  };
  auto up = [&]() {
    for (int l = 31; l >= 1; --l)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 2; ++c) L[l].A[r][0][c] += L[l - 1].A[r][2][c];
  };
  for (int w = 0; w < nxw; ++w)
    for (int js = 0; js < P.ny; js += seg) {
      const int je = std::min(js + seg, P.ny);
      for (int l = 0; l < 32; ++l) P2March<T>::begin(P, L[l], w * P2M_OWN - 1 + l, l == 31);
      int j = js > 0 ? js - 1 : 0;
      // the kernel's warp-uniform choice between the masked and the lean phases
      const bool lean = P2March<T>::lean_region(P, w * P2M_OWN - 1, j, je);
      lean_warps += lean;
      for (int l = 0; l < 32; ++l) {
        if (lean) {
          P2March<T>::template load<0, true>(P, io, xi, L[l], j);
          P2March<T>::template load_mass<true>(P, L[l].K, L[l].i, j, L[l].M);
        } else {
          P2March<T>::template load<0>(P, io, xi, L[l], j);
          P2March<T>::load_mass(P, L[l].K, L[l].i, j, L[l].M);
        }
      }
      down(0);
      std::vector<P2Next<T>> N(32);
      for (;;) {
        const bool more = j + 1 < je;
        if (more)
          for (int l = 0; l < 32; ++l) {
            if (lean) P2March<T>::template prefetch<true>(P, io, xi, L[l], j + 1, N[l]);
            else P2March<T>::prefetch(P, io, xi, L[l], j + 1, N[l]);
          }
        std::vector<typename P2March<T>::Fin> F(32);
        if (j >= js)
          for (int l = 1; l < 32; ++l)
            if (L[l].i <= P.nx) {
              if (lean) P2March<T>::template fin_load<true>(P, io, L[l], j, F[l]);
              else P2March<T>::fin_load(P, io, L[l], j, F[l]);
            }
        for (int l = 0; l < 32; ++l) {
          if constexpr (IsDD<T>::value) {  // the kernel's pair path loads the mass matrices here
            if (lean) P2March<T>::template load_mass<true>(P, L[l].K, L[l].i, j, L[l].M);
            else P2March<T>::load_mass(P, L[l].K, L[l].i, j, L[l].M);
          }
          if (lean) P2March<T>::template compute<true>(P, L[l], j, io.mode);
          else P2March<T>::compute(P, L[l], j, io.mode);
        }
        up();
        if (j >= js)
          for (int l = 1; l < 32; ++l)
            if (L[l].i <= P.nx) {
              if (lean) P2March<T>::template finish<true>(P, io, L[l], j, j == P.ny - 1 ? 3 : 2, F[l], acc);
              else P2March<T>::finish(P, io, L[l], j, j == P.ny - 1 ? 3 : 2, F[l], acc);
            }
        if (!more) break;
        ++j;
        for (int l = 0; l < 32; ++l) {
          P2March<T>::advance(L[l]);
          P2March<T>::take(L[l], N[l]);
        }
        down(1);
      }
    }
}

// Runs the P1 column-march kernel on the CPU (lanes in lockstep, shuffles as copies).
template <class T, int NC>
void p1_march_run(const P1Params<T, NC>& P, P1Io<T> io) {
  P1March<T, NC>::prepare(io);
  const int seg = p2_march_segment(P.nx, P.ny, 4, 5);
  const int nxw = (P.nx + 1 + P2M_OWN - 1) / P2M_OWN;
  std::vector<P1Lane<T, NC>> L(32);
  auto down = [&](int r0) {
    for (int l = 0; l < 31; ++l)
      if (!L[l].edge)
        for (int r = r0; r <= 1; ++r)
          for (int d = 0; d < NC; ++d) L[l].U[r][1][d] = L[l + 1].U[r][0][d];
  };
  for (int w = 0; w < nxw; ++w)
    for (int js = 0; js < P.ny; js += seg) {
      const int je = std::min(js + seg, P.ny);
      for (int l = 0; l < 32; ++l) P1March<T, NC>::begin(L[l], w * P2M_OWN - 1 + l, l == 31);
      int j = js > 0 ? js - 1 : 0;
      for (int l = 0; l < 32; ++l) {
        P1March<T, NC>::template load<0>(P, io, L[l], j);
        P1March<T, NC>::load_coef(P, L[l].i, j, L[l].kk, L[l].km);
      }
      down(0);
      std::vector<P1Next<T, NC>> N(32);
      for (;;) {
        const bool more = j + 1 < je;
        if (more)
          for (int l = 0; l < 32; ++l) P1March<T, NC>::prefetch(P, io, L[l], j + 1, N[l]);
        std::vector<typename P1March<T, NC>::Fin> F(32);
        if (j >= js && io.mode != kP2Apply)
          for (int l = 1; l < 32; ++l)
            if (L[l].i <= P.nx) P1March<T, NC>::fin_load(P, io, L[l].i, j, F[l]);
        for (int l = 0; l < 32; ++l) P1March<T, NC>::compute(P, L[l], j);
        for (int l = 31; l >= 1; --l)
          for (int r = 0; r < 2; ++r)
            for (int d = 0; d < NC; ++d) L[l].A[r][0][d] += L[l - 1].A[r][1][d];
        if (j >= js)
          for (int l = 1; l < 32; ++l)
            if (L[l].i <= P.nx) P1March<T, NC>::finish(P, io, L[l], j, j == P.ny - 1 ? 2 : 1, F[l]);
        if (!more) break;
        ++j;
        for (int l = 0; l < 32; ++l) {
          P1March<T, NC>::advance(L[l]);
          P1March<T, NC>::take(L[l], N[l]);
        }
        down(1);
      }
    }
}

template <class T>
void p2_run(const P2Params<T>& P, const T* xi, const T* u, T* y, int mode) {
  P2Io<T> io;
  std::memset(&io, 0, sizeof(io));
  io.mode = mode == 1 ? kP2Diag : kP2Apply;
  io.u = u;
  io.y = y;
  p2_run_io<T>(P, xi, io);
}

template <class T>
P2Params<T> p2params(int nx, int ny, double hx, double hy, double lam, double mu, double p, double pmin,
                     const int* dir) {
  P2Params<T> P;
  std::memset(&P, 0, sizeof(P));
  P.nx = nx;
  P.ny = ny;
  P.ihx = T(1.0 / hx);
  P.ihy = T(1.0 / hy);
  const double area = 0.5 * hx * hy;
  P.lamT = T(lam * area);
  P.mu2T = T(2.0 * mu * area);
  P.pen = make_penal<T>(p, pmin);
  P.dir = dir_from(dir);
  return P;
}
}  // namespace

extern "C" {

long emu_lean_warps() { return lean_warps; }
void emu_set_segment(int seg) { seg_override = seg; }

int emu_dir_ints() { return kDirInts; }

// y = K(xi) u (mode 0) or diag K(xi) (mode 1); prec 0 = FP64, 1 = FP32, 2 = pair-of-FP32 (mode 0)
int emu_p2_apply(int prec, int nx, int ny, double hx, double hy, double lam, double mu, double p, double pmin,
                 const int* dir, const double* xi, const double* u, double* y, int mode) {
  const size_t nv = size_t(nx + 1) * (ny + 1), nd = size_t(2) * (2 * nx + 1) * (2 * ny + 1);
  if (prec == 0) {
    auto P = p2params<double>(nx, ny, hx, hy, lam, mu, p, pmin, dir);
    p2_run<double>(P, xi, u, y, mode);
  } else if (prec == 2) {
    // pair-of-FP32 operator (Apply only): mass matrices precomputed in FP64 and split
    if (mode != 0 || !u) return -1;
    auto P = p2params<dd>(nx, ny, hx, hy, lam, mu, p, pmin, dir);
    // the library's set-up: pair-of-FP32 quadrature for an integer exponent, else FP64 split
    const Penal<double> pen = make_penal<double>(p, pmin, 0);
    std::vector<dd> rm(size_t(12) * nx * ny);
    std::vector<double> kK(size_t(2) * nx * ny);
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        if (pen.ip >= 1 && pen.ip <= 16)
          cell_rmass_kappa_dd(i, j, nx, xi, pen.ip, dd(pmin), dd(1.0 - pmin), rm.data(), kK.data());
        else
          cell_rmass_kappa<double, dd>(i, j, nx, ny, xi, pen, rm.data(), kK.data());
      }
    P.rmass = rm.data();
    p2_run<dd>(P, nullptr, reinterpret_cast<const dd*>(u), reinterpret_cast<dd*>(y), 0);
  } else {
    auto P = p2params<float>(nx, ny, hx, hy, lam, mu, p, pmin, dir);
    std::vector<float> xf(xi, xi + nv), uf(nd, 0.f), yf(nd, 0.f);
    if (u) for (size_t i = 0; i < nd; ++i) uf[i] = float(u[i]);
    p2_run<float>(P, xf.data(), uf.data(), yf.data(), mode);
    for (size_t i = 0; i < nd; ++i) y[i] = yf[i];
  }
  return 0;
}

int emu_p1_apply(int NC, int nx, int ny, double hx, double hy, double lam, double mu, const int* dir,
                 const double* kK, const double* kM, double kKc, double kMc, const double* u, double* y, int diag) {
  const ElemRefs R = make_elem_refs(hx, hy, lam, mu);
  const int NX = nx + 1, NY = ny + 1;
  auto fill = [&](auto& P) {
    P.nx = nx;
    P.ny = ny;
    P.dir = dir_from(dir);
    for (int o = 0; o < 2; ++o) {
      for (int a = 0; a < 3 * NC; ++a)
        for (int b = 0; b < 3 * NC; ++b) P.K[o][a][b] = NC == 2 ? R.K2[o][a][b] : R.K1[o][a][b];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) P.Mm[o][a][b] = R.M1[o][a][b];
    }
    P.kK = kK;
    P.kM = kM;
    P.kK_c = kKc;
    P.kM_c = kMc;
  };
  if (NC == 2) {
    P1Params<double, 2> P;
    std::memset(&P, 0, sizeof(P));
    fill(P);
    for (int b = 0; b < NY; ++b)
      for (int a = 0; a < NX; ++a)
        diag ? P1Kern<double, 2>::node_diag(a, b, P, y) : P1Kern<double, 2>::node_apply(a, b, P, u, y);
  } else {
    P1Params<double, 1> P;
    std::memset(&P, 0, sizeof(P));
    fill(P);
    for (int b = 0; b < NY; ++b)
      for (int a = 0; a < NX; ++a)
        diag ? P1Kern<double, 1>::node_diag(a, b, P, y) : P1Kern<double, 1>::node_apply(a, b, P, u, y);
  }
  return 0;
}

int emu_transfer(int NC, int NXf, int NYf, const int* dirf, int NXc, int NYc, const int* dirc, const double* in,
                 double* out, int prolong) {
  Transfer X;
  X.NXf = NXf;
  X.NYf = NYf;
  X.NXc = NXc;
  X.NYc = NYc;
  X.dirf = dir_from(dirf);
  X.dirc = dir_from(dirc);
  if (prolong) {
    for (int b = 0; b < NYf; ++b)
      for (int a = 0; a < NXf; ++a)
        NC == 2 ? TransferKern<double, 2>::node_prolong_add(a, b, X, in, out)
                : TransferKern<double, 1>::node_prolong_add(a, b, X, in, out);
  } else {
    for (int J = 0; J < NYc; ++J)
      for (int I = 0; I < NXc; ++I)
        NC == 2 ? TransferKern<double, 2>::node_restrict(I, J, X, in, out)
                : TransferKern<double, 1>::node_restrict(I, J, X, in, out);
  }
  return 0;
}

// fused smoothing steps (FP64).  bufs = {b, dinv, x, x2, r, d}; cheb = {c0, c1, c2};
// level given by p2 (P2 lattice of nx x ny cells) or P1 (NC comps on nx x ny cells);
// xc / dirc / NXc, NYc: the next coarser lattice (post1 source, resr target bc)
int emu_smooth(int p2, int NC, int mode, int nx, int ny, double hx, double hy, double lam, double mu, double p,
               double pmin, const int* dir, const double* xi, const double* kK, double* const* bufs,
               const double* cheb, int NXc, int NYc, const int* dirc, const double* xc, double* bc, int stencil,
               const double* kM) {
  SmoothBufs<double> B{bufs[0], bufs[1], bufs[2], bufs[3], bufs[4], bufs[5], cheb};
  Transfer X;
  X.NXf = p2 ? 2 * nx + 1 : nx + 1;
  X.NYf = p2 ? 2 * ny + 1 : ny + 1;
  X.NXc = NXc;
  X.NYc = NYc;
  X.dirf = dir_from(dir);
  X.dirc = dir_from(dirc);
  if (p2) {
    auto P = p2params<double>(nx, ny, hx, hy, lam, mu, p, pmin, dir);
    P2Io<double> io;
    std::memset(&io, 0, sizeof(io));
    io.mode = mode;
    io.u = bufs[2];
    io.B = B;
    io.xc = mode == kP2First ? xc : nullptr;  // optional fused prolongation
    p2_run_io<double>(P, xi, io);
    return 0;
  }
  const ElemRefs R = make_elem_refs(hx, hy, lam, mu);
  auto go = [&](auto& P, auto nc_tag) {
    constexpr int K = decltype(nc_tag)::value;
    P.nx = nx;
    P.ny = ny;
    P.dir = dir_from(dir);
    for (int o = 0; o < 2; ++o) {
      for (int a = 0; a < 3 * K; ++a)
        for (int b = 0; b < 3 * K; ++b) P.K[o][a][b] = K == 2 ? R.K2[o][a][b] : R.K1[o][a][b];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) P.Mm[o][a][b] = R.M1[o][a][b];
    }
    P.kK = kK;
    P.kM = K == 1 ? kM : nullptr;  // per-triangle mass coefficients (scalar levels), else 1
    P.kK_c = 0;
    P.kM_c = (K == 1 && !kM) ? 1.0 : 0.0;
    auto sweep = [&](const auto& Q) {
      for (int b = 0; b <= ny; ++b)
        for (int a = 0; a <= nx; ++a) {
          if (mode == kP2Pre) P1Smooth<double, K>::pre(a, b, Q, B);
          else if (mode == kP2Res) P1Smooth<double, K>::res(a, b, Q, B);
          else if (mode == kP2First) P1Smooth<double, K>::first(a, b, Q, B);
          else P1Smooth<double, K>::post2(a, b, Q, B);
        }
    };
    if (stencil == 2) {  // the column march
      P1Io<double> io;
      std::memset(&io, 0, sizeof(io));
      io.mode = mode;
      io.u = B.x;
      io.B = B;
      p1_march_run<double, K>(P, io);
    } else if (stencil) {
      // the assembled-stencil representation of the same level
      constexpr int SW = StencilLayout<K>::stride;
      std::vector<double> st(size_t(nx + 1) * (ny + 1) * SW);
      for (int b = 0; b <= ny; ++b)
        for (int a = 0; a <= nx; ++a) p1_stencil_node<double, K>(a, b, P, st.data() + (size_t(b) * (nx + 1) + a) * SW);
      sweep(P1Stencil<double, K>{nx, ny, P.dir, st.data()});
    } else {
      sweep(P);
    }
  };
  if (NC == 2) {
    P1Params<double, 2> P;
    std::memset(&P, 0, sizeof(P));
    go(P, std::integral_constant<int, 2>{});
  } else {
    P1Params<double, 1> P;
    std::memset(&P, 0, sizeof(P));
    go(P, std::integral_constant<int, 1>{});
  }
  return 0;
}

int emu_kappa(int nx, int ny, double p, double pmin, const double* xi, double* kK) {
  const Penal<double> pen = make_penal<double>(p, pmin);
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int o = 0; o < 2; ++o) {
        double xe[3];
        for (int k = 0; k < 3; ++k) xe[k] = xi[size_t(j + p1_off_b(o, k)) * (nx + 1) + i + p1_off_a(o, k)];
        kK[(size_t(j) * nx + i) * 2 + o] = tri_kappa(xe, pen);
      }
  return 0;
}

int emu_coarsen_kappa(const double* kf, int nxf, int nyf, double* kc, int nxc, int nyc) {
  for (int J = 0; J < nyc; ++J)
    for (int I = 0; I < nxc; ++I)
      for (int o = 0; o < 2; ++o) kc[(size_t(J) * nxc + I) * 2 + o] = coarsen_kappa(kf, nxf, nyf, I, J, o);
  return 0;
}

// per level: p2, nx, ny, NX, NY, NC, dir[kDirInts]
int emu_build_levels(int p2_top, int nx, int ny, double hx, double hy, const int* dir_top, int NC, int max_levels,
                     int* out) {
  const auto v = build_levels(p2_top != 0, nx, ny, hx, hy, dir_from(dir_top), NC);
  const int n = int(v.size());
  for (int l = 0; l < n && l < max_levels; ++l) {
    int* o = out + l * (6 + kDirInts);
    o[0] = v[l].p2;
    o[1] = v[l].nx;
    o[2] = v[l].ny;
    o[3] = v[l].NX;
    o[4] = v[l].NY;
    o[5] = v[l].NC;
    dir_to(v[l].dir, o + 6);
  }
  return n;
}

int emu_sensitivity(int prec, int nx, int ny, double hx, double hy, double lam, double mu, double p, double pmin,
                    const double* u, const double* xi, double* b) {
  const int NX = 2 * nx + 1, VX = nx + 1;
  const size_t nt = size_t(2) * nx * ny;
  std::vector<double> tri(3 * nt);
  const double area = 0.5 * hx * hy;
  for (size_t t = 0; t < nt; ++t) {
    const int o = int(t & 1);
    const size_t cell = t >> 1;
    const int i = int(cell % nx), j = int(cell / nx);
    double ue[6][2];
    for (int k = 0; k < 6; ++k) {
      const size_t n = size_t(2 * j + p2_off_b(o, k)) * NX + 2 * i + p2_off_a(o, k);
      ue[k][0] = u[2 * n];
      ue[k][1] = u[2 * n + 1];
    }
    if (prec == 0) {
      double xe[3], c[3];
      for (int k = 0; k < 3; ++k) xe[k] = xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)];
      const auto pen = make_penal<double>(p, pmin);
      if (o == 0) tri_sensitivity<0, double, double>(ue, xe, 1.0 / hx, 1.0 / hy, lam, mu, area, pen, c);
      else tri_sensitivity<1, double, double>(ue, xe, 1.0 / hx, 1.0 / hy, lam, mu, area, pen, c);
      for (int k = 0; k < 3; ++k) tri[3 * t + k] = c[k];
    } else {
      float xe[3], c[3];
      for (int k = 0; k < 3; ++k) xe[k] = float(xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)]);
      const auto pen = make_penal<float>(p, pmin);
      // the kernel's difference form: u - u_A from the values' (hi, lo) splits in FP32,
      // gradients and quadrature in FP32
      float ud[6][2];
      for (int k = 0; k < 6; ++k)
        for (int d = 0; d < 2; ++d) {
          const dd a = dd_from_double(ue[k][d]), b = dd_from_double(ue[0][d]);
          ud[k][d] = k == 0 ? 0.0f : (a.hi - b.hi) + (a.lo - b.lo);
        }
      if (o == 0)
        tri_sensitivity<0, float, float>(ud, xe, float(1.0 / hx), float(1.0 / hy), float(lam), float(mu), float(area),
                                         pen, c);
      else
        tri_sensitivity<1, float, float>(ud, xe, float(1.0 / hx), float(1.0 / hy), float(lam), float(mu), float(area),
                                         pen, c);
      for (int k = 0; k < 3; ++k) tri[3 * t + k] = c[k];
    }
  }
  const size_t nv = size_t(nx + 1) * (ny + 1);
  for (size_t v = 0; v < nv; ++v) {
    const int a = int(v % VX), bb = int(v / VX);
    double s = 0.0;
    for (int e = 0; e < 6; ++e) {
      int dci, dcj, o, loc;
      p1_incidence(e, dci, dcj, o, loc);
      const int ci = a + dci, cj = bb + dcj;
      if (ci < 0 || ci >= nx || cj < 0 || cj >= ny) continue;
      s += tri[3 * ((size_t(cj) * nx + ci) * 2 + o) + loc];
    }
    b[v] = s;
  }
  return 0;
}

int emu_make_dir(int nx, int ny, double hx, double hy, int sides, int npts, const double* pts, int* out) {
  topo_bc_desc bc{sides, npts, pts};
  Dir d;
  std::string msg;
  if (make_p2_dir(nx, ny, hx, hy, &bc, d, msg)) return 1;
  dir_to(d, out);
  return 0;
}

// tr: 5 doubles per traction (side, center, length, vx, vy)
int emu_load(int nx, int ny, double W, double H, const int* dir, int has_bf, double cx, double cy, double r,
             double fx, double fy, int ntr, const double* tr, double* b) {
  std::vector<topo_traction> T(ntr);
  for (int k = 0; k < ntr; ++k) T[k] = topo_traction{int(tr[5 * k]), tr[5 * k + 1], tr[5 * k + 2], tr[5 * k + 3], tr[5 * k + 4]};
  topo_load_desc L{has_bf, cx, cy, r, fx, fy, ntr, T.data()};
  std::vector<double> v;
  assemble_load(nx, ny, W, H, dir_from(dir), &L, v);
  std::memcpy(b, v.data(), v.size() * sizeof(double));
  return 0;
}

int emu_vertex_weights(int nx, int ny, double hx, double hy, double* w) {
  const auto v = vertex_weights(nx, ny, hx, hy);
  std::memcpy(w, v.data(), v.size() * sizeof(double));
  return 0;
}

// Coarse Chebyshev solve of the scalar level eps2 K + M (assembled stencil, no
// clamping) from x = 0: the node phases of k_coarse_cheb run sequentially.
// info: [lo, hi, degree] of the plan for the level's coefficient ratio eps2.
int emu_coarse_cheb(int nx, int ny, double hx, double hy, double eps2, int deg_force, const double* b, double* x,
                    double* info) {
  const ElemRefs R = make_elem_refs(hx, hy, 0.0, 0.0);
  const int NX = nx + 1, NY = ny + 1, nn = NX * NY;
  P1Params<double, 1> P;
  std::memset(&P, 0, sizeof(P));
  P.nx = nx;
  P.ny = ny;
  std::memset(&P.dir, 0, sizeof(P.dir));  // no clamped nodes
  P.dir.x_hi_from = NX;
  P.dir.y_hi_from = NY;
  for (int o = 0; o < 2; ++o)
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) {
        P.K[o][a][c] = R.K1[o][a][c];
        P.Mm[o][a][c] = R.M1[o][a][c];
      }
  P.kK_c = eps2;
  P.kM_c = 1.0;
  constexpr int SW = StencilLayout<1>::stride;
  std::vector<double> st(size_t(nn) * SW), dinv(nn);
  for (int bb = 0; bb < NY; ++bb)
    for (int a = 0; a < NX; ++a) p1_stencil_node<double, 1>(a, bb, P, st.data() + (size_t(bb) * NX + a) * SW);
  for (int n = 0; n < nn; ++n) {  // diagonal = row sum - couplings (difference form)
    double d = st[size_t(n) * SW];
    for (int k = 1; k < 7; ++k) d -= st[size_t(n) * SW + k];
    dinv[n] = 1.0 / d;
  }
  double lo, hi;
  int deg = coarse_cheb_plan(R, eps2, eps2, 1e-2, lo, hi);
  info[0] = lo;
  info[1] = hi;
  info[2] = deg;
  if (deg_force > 0) deg = deg_force;
  if (deg > kCoarseChebMax) return 1;
  CoarseCheb<double> C;
  std::memset(&C, 0, sizeof(C));
  double c0, c1[kCoarseChebMax], c2[kCoarseChebMax];
  coarse_cheb_coefficients(lo, hi, deg, c0, c1, c2);
  C.deg = deg;
  C.c0 = c0;
  for (int k = 0; k + 1 < deg; ++k) {
    C.c1[k] = c1[k];
    C.c2[k] = c2[k];
  }
  const P1Stencil<double, 1> S{nx, ny, P.dir, st.data()};
  std::vector<double> r(nn), xv(nn), d0(nn), d1(nn);
  for (int n = 0; n < nn; ++n) CoarseChebNode<double, 1>::init(size_t(n), C, b, dinv.data(), r.data(), xv.data(), d0.data());
  double* dc = d0.data();
  double* dn = d1.data();
  for (int k = 0; k + 1 < deg; ++k) {
    for (int n = 0; n < nn; ++n)
      CoarseChebNode<double, 1>::step(n % NX, n / NX, k, S, C, dinv.data(), dc, r.data(), xv.data(), dn);
    std::swap(dc, dn);
  }
  for (int n = 0; n < nn; ++n) CoarseChebNode<double, 1>::finish(size_t(n), dc, xv.data(), x);
  return 0;
}

// ---- Stokes-Brinkman fluid: the kernels' triangle phases and gathers, run per
// triangle / node in the kernels' order
int emu_fluid_tables_doubles() { return int(sizeof(FluidTables) / sizeof(double)); }

void emu_fluid_tables(double hx, double hy, double* out) {
  FluidTables E;
  fluid_tables(hx, hy, E);
  std::memcpy(out, &E, sizeof(E));
}

// flows [nf][4] = side, center, length, rate
int emu_fluid_bc(int nx, int ny, double W, double H, int nf, const double* flows, double* ub) {
  std::vector<topo_flow> F(nf);
  for (int f = 0; f < nf; ++f) {
    F[f].side = int(flows[4 * f]);
    F[f].center = flows[4 * f + 1];
    F[f].length = flows[4 * f + 2];
    F[f].rate = flows[4 * f + 3];
  }
  std::vector<double> v;
  std::string msg;
  if (fluid_boundary_values(nx, ny, W, H, F.data(), nf, v, msg)) return 1;
  std::memcpy(ub, v.data(), v.size() * sizeof(double));
  return 0;
}

static FluidPenal emu_fluid_penal(double q) {
  FluidPenal pen;
  pen.q = q;
  pen.amin = 2.5 / (100.0 * 100.0);
  pen.amax = 2.5 / (0.01 * 0.01);
  return pen;
}

double emu_fluid_alpha(double q, double rho, int derivative) {
  const FluidPenal pen = emu_fluid_penal(q);
  return derivative ? pen.da(rho) : pen.a(rho);
}

void emu_fluid_apply(int nx, int ny, double W, double H, double q, const double* rho, const double* x, double* y,
                     int clamp) {
  FluidTables E;
  fluid_tables(W / nx, H / ny, E);
  const FluidPenal pen = emu_fluid_penal(q);
  const size_t nt = size_t(2) * nx * ny, n2 = size_t(2 * nx + 1) * (2 * ny + 1), nv = size_t(nx + 1) * (ny + 1);
  std::vector<double> mass(nt * kFluidMass), out(nt * kFluidOut);
  for (size_t t = 0; t < nt; ++t) {
    double r[3];
    fluid_tri_rho(rho, nx, t, r);
    fluid_tri_mass(E, pen, r, mass.data() + t * kFluidMass);
  }
  for (size_t t = 0; t < nt; ++t) {
    size_t nd[6], vt[3];
    fluid_tri_nodes(nx, t, nd);
    fluid_tri_vertices(nx, t, vt);
    double ue[6][2], pe[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = x[2 * nd[k]];
      ue[k][1] = x[2 * nd[k] + 1];
    }
    for (int k = 0; k < 3; ++k) pe[k] = x[2 * n2 + vt[k]];
    fluid_tri_apply(E, int(t & 1), mass.data() + t * kFluidMass, ue, pe, out.data() + t * kFluidOut);
  }
  const int NX = 2 * nx + 1;
  for (size_t i = 0; i < n2; ++i) {
    double v[2];
    fluid_gather_node(out.data(), nx, ny, int(i % NX), int(i / NX), clamp != 0, x, v);
    y[2 * i] = v[0];
    y[2 * i + 1] = v[1];
  }
  for (size_t k = 0; k < nv; ++k)
    y[2 * n2 + k] = fluid_gather_vertex(out.data(), nx, ny, int(k % (nx + 1)), int(k / (nx + 1)), kFluidOut, 12);
}

double emu_fluid_objective(int nx, int ny, double W, double H, double q, double mu, const double* rho,
                           const double* u) {
  FluidTables E;
  fluid_tables(W / nx, H / ny, E);
  const FluidPenal pen = emu_fluid_penal(q);
  double s = 0.0;
  for (size_t t = 0; t < size_t(2) * nx * ny; ++t) {
    size_t nd[6];
    fluid_tri_nodes(nx, t, nd);
    double ue[6][2], r[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = u[2 * nd[k]];
      ue[k][1] = u[2 * nd[k] + 1];
    }
    fluid_tri_rho(rho, nx, t, r);
    s += fluid_tri_objective(E, pen, mu, int(t & 1), r, ue);
  }
  return 0.5 * s;
}

void emu_fluid_gradient_rhs(int nx, int ny, double W, double H, double q, const double* rho, const double* u,
                            double* b) {
  FluidTables E;
  fluid_tables(W / nx, H / ny, E);
  const FluidPenal pen = emu_fluid_penal(q);
  const size_t nt = size_t(2) * nx * ny;
  std::vector<double> tri3(3 * nt);
  for (size_t t = 0; t < nt; ++t) {
    size_t nd[6];
    fluid_tri_nodes(nx, t, nd);
    double ue[6][2], r[3], o3[3];
    for (int k = 0; k < 6; ++k) {
      ue[k][0] = u[2 * nd[k]];
      ue[k][1] = u[2 * nd[k] + 1];
    }
    fluid_tri_rho(rho, nx, t, r);
    fluid_tri_gradient(E, pen, r, ue, o3);
    for (int k = 0; k < 3; ++k) tri3[3 * t + k] = o3[k];
  }
  for (size_t v = 0; v < size_t(nx + 1) * (ny + 1); ++v)
    b[v] = fluid_gather_vertex(tri3.data(), nx, ny, int(v % (nx + 1)), int(v / (nx + 1)), 3, 0);
}

// incident (triangle, local node) pairs of P2 node (a, b); returns the count
int emu_p2_node_incidence(int a, int b, int nx, int ny, long long* tri, int* loc) {
  size_t t[6];
  int l[6];
  const int n = p2_node_incidence(a, b, nx, ny, t, l);
  for (int e = 0; e < n; ++e) {
    tri[e] = (long long)t[e];
    loc[e] = l[e];
  }
  return n;
}

}  // extern "C"
