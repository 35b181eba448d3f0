// Host-side set-up of the Stokes-Brinkman problem: quadrature rules, element
// tables and the Dirichlet data of the flow profiles.  Header-only so the test
// emulator can check it against the FP64 oracle on the CPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "topomax_gb300.h"
#include "topo_fluid.cuh"
#include "topo_setup.h"

namespace topo {

// ---------------------------------------------------------------------------
// quadrature and element tables (host)
// ---------------------------------------------------------------------------

// Jacobi polynomial P_n^(a,b)(x) and its derivative, by the three-term recurrence
inline void jacobi_eval(int n, double a, double b, double x, double& p, double& dp) {
  double p0 = 1.0, p1 = 0.5 * (a - b + (a + b + 2.0) * x);
  if (n == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k) {
    const double c = 2.0 * k + a + b;
    const double a1 = 2.0 * k * (k + a + b) * (c - 2.0);
    const double a2 = (c - 1.0) * (c * (c - 2.0) * x + a * a - b * b);
    const double a3 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * c;
    const double p2 = (a2 * p1 - a3 * p0) / a1;
    p0 = p1;
    p1 = p2;
  }
  p = p1;  // P_n, p0 = P_(n-1)
  const double c = 2.0 * n + a + b;
  dp = (n * (a - b - c * x) * p1 + 2.0 * (n + a) * (n + b) * p0) / (c * (1.0 - x * x));
}

// Gauss-Jacobi rule for the weight (1-x)^a (1+x)^b on [-1, 1]: Newton on P_n with
// the roots already found divided out; ascending nodes.
inline void gauss_jacobi(int n, double a, double b, double* x, double* w) {
  for (int k = 0; k < n; ++k) {
    double z = std::cos(M_PI * (k + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      jacobi_eval(n, a, b, z, p, dp);
      double s = 0.0;
      for (int j = 0; j < k; ++j) s += 1.0 / (z - x[j]);
      const double dz = p / (dp - s * p);
      z -= dz;
      if (std::fabs(dz) <= 1e-16 * std::max(1.0, std::fabs(z))) break;
    }
    x[k] = z;
  }
  std::sort(x, x + n);
  const double cst = std::exp(std::lgamma(n + a + 1.0) + std::lgamma(n + b + 1.0) - std::lgamma(n + a + b + 1.0) -
                              std::lgamma(n + 1.0)) *
                     std::pow(2.0, a + b + 1.0);
  for (int k = 0; k < n; ++k) {
    double p, dp;
    jacobi_eval(n, a, b, x[k], p, dp);
    w[k] = cst / ((1.0 - x[k] * x[k]) * dp * dp);
  }
}

// The 12-point Strang-Fix rule (degree 6) as barycentric points and weights summing to 1.
inline void fluid_rule6(double (&lam)[kFluidQ6][3], double (&w)[kFluidQ6]) {
  int q = 0;
  auto orbit3 = [&](double a, double wt) {
    const double b = 1.0 - 2.0 * a;
    const double pts[3][3] = {{b, a, a}, {a, b, a}, {a, a, b}};
    for (auto& p : pts) {
      for (int k = 0; k < 3; ++k) lam[q][k] = p[k];
      w[q++] = wt;
    }
  };
  auto orbit6 = [&](double a, double b, double wt) {
    const double c = 1.0 - a - b;
    const double pts[6][3] = {{a, b, c}, {a, c, b}, {b, a, c}, {b, c, a}, {c, a, b}, {c, b, a}};
    for (auto& p : pts) {
      for (int k = 0; k < 3; ++k) lam[q][k] = p[k];
      w[q++] = wt;
    }
  };
  orbit3(0.063089014491502, 0.050844906370207);
  orbit3(0.249286745170910, 0.116786275726379);
  orbit6(0.053145049844816, 0.310352451033785, 0.082851075618374);
}

// The collapsed Gauss-Jacobi rule with 4 x 4 points (degree 7): Gauss-Legendre in
// one direction, Gauss-Jacobi with weight (1 - eta) in the collapsed one.
inline void fluid_rule7(double (&lam)[kFluidQ7][3], double (&w)[kFluidQ7]) {
  double x[4], wx[4], y[4], wy[4];
  gauss_jacobi(4, 0.0, 0.0, x, wx);
  gauss_jacobi(4, 1.0, 0.0, y, wy);
  int q = 0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const double s = 0.25 * (1.0 + x[i]) * (1.0 - y[j]);
      const double t = 0.5 * (1.0 + y[j]);
      lam[q][0] = 1.0 - s - t;
      lam[q][1] = s;
      lam[q][2] = t;
      w[q++] = 0.25 * wx[i] * wy[j];
    }
}


// Element tables of the lattice with spacing (hx, hy); the geometry of both
// orientations as in the CG1/P2 lattice conventions of topo_common.cuh.
inline void fluid_tables(double hx, double hy, FluidTables& E) {
  std::memset(&E, 0, sizeof(E));
  fluid_rule6(E.lam6, E.w6);
  fluid_rule7(E.lam7, E.w7);
  for (int q = 0; q < kFluidQ6; ++q) {
    const double l[3] = {E.lam6[q][0], E.lam6[q][1], E.lam6[q][2]};
    p2_values(l, E.N6[q]);
  }
  for (int q = 0; q < kFluidQ7; ++q) {
    const double l[3] = {E.lam7[q][0], E.lam7[q][1], E.lam7[q][2]};
    p2_values(l, E.N7[q]);
  }
  for (int o = 0; o < 2; ++o) {
    const double P[3][2] = {{0.0, 0.0}, {o == 0 ? hx : 0.0, o == 0 ? 0.0 : hy}, {hx, hy}};
    const double a2 = (P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[2][0] - P[0][0]) * (P[1][1] - P[0][1]);
    const double G[3][2] = {{(P[1][1] - P[2][1]) / a2, (P[2][0] - P[1][0]) / a2},
                            {(P[2][1] - P[0][1]) / a2, (P[0][0] - P[2][0]) / a2},
                            {(P[0][1] - P[1][1]) / a2, (P[1][0] - P[0][0]) / a2}};
    E.area = 0.5 * std::fabs(a2);
    for (int q = 0; q < kFluidQ6; ++q) {
      const double* l = E.lam6[q];
      for (int c = 0; c < 2; ++c) {
        E.dN6[o][q][0][c] = (4 * l[0] - 1) * G[0][c];
        E.dN6[o][q][1][c] = (4 * l[1] - 1) * G[1][c];
        E.dN6[o][q][2][c] = (4 * l[2] - 1) * G[2][c];
        E.dN6[o][q][3][c] = 4 * (l[1] * G[2][c] + l[2] * G[1][c]);
        E.dN6[o][q][4][c] = 4 * (l[0] * G[2][c] + l[2] * G[0][c]);
        E.dN6[o][q][5][c] = 4 * (l[0] * G[1][c] + l[1] * G[0][c]);
      }
    }
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double s = 0.0;
        for (int q = 0; q < kFluidQ6; ++q)
          s += E.w6[q] * (E.dN6[o][q][i][0] * E.dN6[o][q][j][0] + E.dN6[o][q][i][1] * E.dN6[o][q][j][1]);
        E.lap[o][i][j] = E.area * s;
      }
    for (int i = 0; i < 6; ++i)
      for (int c = 0; c < 2; ++c)
        for (int k = 0; k < 3; ++k) {
          double s = 0.0;
          for (int q = 0; q < kFluidQ6; ++q) s += E.w6[q] * E.N6[q][i] * G[k][c];
          E.grad[o][i][c][k] = E.area * s;
        }
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 6; ++j)
        for (int c = 0; c < 2; ++c) {
          double s = 0.0;
          for (int q = 0; q < kFluidQ6; ++q) s += E.w6[q] * E.lam6[q][k] * E.dN6[o][q][j][c];
          E.div[o][k][j][c] = E.area * s;
        }
  }
}

// BoundaryFlows.eval (FEM_src/fluid_problem.py:12-45) at the P2 nodes: the flow
// profiles on the flow sides (exact coordinate tests, as eval makes them), then
// the no-slip sides set to zero (their DirichletBC is applied last,
// FEM_src/fluid_problem.py:126-150).  Every boundary node is a Dirichlet node.
inline int fluid_boundary_values(int nx, int ny, double W, double H, const topo_flow* flows, int nf,
                          std::vector<double>& ub, std::string& msg) {
  const int NX = 2 * nx + 1, NY = 2 * ny + 1;
  ub.assign(size_t(2) * NX * NY, 0.0);
  int flow_sides = 0;
  for (int f = 0; f < nf; ++f) {
    const int sd = flows[f].side;
    if (sd != TOPO_SIDE_LEFT && sd != TOPO_SIDE_RIGHT && sd != TOPO_SIDE_TOP && sd != TOPO_SIDE_BOTTOM) {
      msg = "Malformed side: " + std::to_string(sd);
      return 1;
    }
    if (!(flows[f].length > 0) || !std::isfinite(flows[f].center) || !std::isfinite(flows[f].rate)) {
      msg = "invalid flow description";
      return 1;
    }
    flow_sides |= sd;
  }
  std::vector<double> X2, Y2;
  lattice_coords(W, nx, X2);
  lattice_coords(H, ny, Y2);
  auto profile = [](double pos, double center, double length, double rate) {
    const double t = pos - center;
    if (-length / 2 < t && t < length / 2) {
      const double s = 2 * t / length;
      return rate * (1 - s * s);
    }
    return 0.0;
  };
  auto side_of = [&](int a, int b) {
    int s = 0;
    if (a == 0) s |= TOPO_SIDE_LEFT;
    if (a == NX - 1) s |= TOPO_SIDE_RIGHT;
    if (b == 0) s |= TOPO_SIDE_BOTTOM;
    if (b == NY - 1) s |= TOPO_SIDE_TOP;
    return s;
  };
  for (int b = 0; b < NY; ++b)
    for (int a = 0; a < NX; ++a) {
      const int s = side_of(a, b);
      if (!(s & flow_sides)) continue;
      const double x = X2[a], y = Y2[b];
      double v0 = 0.0, v1 = 0.0;
      for (int f = 0; f < nf; ++f) {
        const topo_flow& F = flows[f];
        if (F.side == TOPO_SIDE_LEFT) {
          if (x == 0.0) v0 += profile(y, F.center, F.length, F.rate);
        } else if (F.side == TOPO_SIDE_RIGHT) {
          if (x == W) v0 -= profile(y, F.center, F.length, F.rate);
        } else if (F.side == TOPO_SIDE_TOP) {
          if (y == H) v1 -= profile(x, F.center, F.length, F.rate);
        } else {
          if (y == 0) v1 += profile(x, F.center, F.length, F.rate);
        }
      }
      const size_t n = size_t(b) * NX + a;
      ub[2 * n] = v0;
      ub[2 * n + 1] = v1;
    }
  const int no_slip = 15 & ~flow_sides;
  for (int b = 0; b < NY; ++b)
    for (int a = 0; a < NX; ++a)
      if (side_of(a, b) & no_slip) {
        const size_t n = size_t(b) * NX + a;
        ub[2 * n] = 0.0;
        ub[2 * n + 1] = 0.0;
      }
  return 0;
}

}  // namespace topo
