// Stokes-Brinkman state on the P2-P1 (Taylor-Hood) lattice: element tables,
// node incidence and the per-triangle phases of the operator, the objective
// and the gradient's right-hand side.
//
// Follows FEM_src/fluid_problem.py:48-155 and src/penalizers.py:49-67:
//   a((u,p),(v,q)) = (alpha(rho) u, v) + (grad u, grad v) + (grad p, v) + (div u, q),
//   alpha(rho) = a_max + (a_min - a_max) rho (1 + q) / (rho + q),
//   objective 1/2 int alpha(rho) |u|^2 + mu |grad u|^2 dx,
//   gradient  = L2 projection onto CG1 of 1/2 alpha'(rho) |u|^2.
// The form compiler integrates the state form and the objective with a degree-6
// rule (Strang-Fix, 12 points) and the projection's right-hand side with the
// collapsed Gauss-Jacobi 4 x 4 rule (degree 7); the same rules are used here.
//
// Everything here compiles for host and device: the test emulator runs the
// triangle phases and the incidence gathers on the CPU against the oracle.
#pragma once

#include <cmath>
#include <cstddef>

#include "topo_common.cuh"

namespace topo {

constexpr int kFluidQ6 = 12;
constexpr int kFluidQ7 = 16;
constexpr int kFluidMass = 21;   // upper triangle of the 6 x 6 alpha-weighted P2 mass matrix
constexpr int kFluidOut = 16;    // per-triangle output: 12 velocity rows, 3 pressure rows, pad

// alpha(rho) and alpha'(rho) in the reference's operation order
struct FluidPenal {
  double q = 0.0, amin = 0.0, amax = 0.0;
  TOPO_HD double a(double rho) const { return amax + (amin - amax) * rho * (1 + q) / (rho + q); }
  TOPO_HD double da(double rho) const {
    const double s = rho + q;
    return (amin - amax) * q * (1 + q) / (s * s);
  }
};

// Element tables shared by every triangle of the lattice (both orientations
// have the same area; gradients differ).  Built once per context on the host.
struct FluidTables {
  double area;
  double lam6[kFluidQ6][3], w6[kFluidQ6];
  double lam7[kFluidQ7][3], w7[kFluidQ7];
  double N6[kFluidQ6][6], N7[kFluidQ7][6];
  double dN6[2][kFluidQ6][6][2];  // physical basis gradients at the degree-6 points
  double lap[2][6][6];            // int grad N_i . grad N_j
  double grad[2][6][2][3];        // int N_i d_c lambda_k    (velocity row (i,c), pressure vertex k)
  double div[2][3][6][2];         // int lambda_k d_c N_j    (pressure row k, velocity column (j,c))
};

TOPO_HD int fluid_mass_index(int i, int j) {  // i <= j
  return i * 6 - (i * (i - 1)) / 2 + (j - i);
}

// P2 basis [A, B, C, mid(BC), mid(AC), mid(AB)] at barycentric point l
TOPO_HD void p2_values(const double (&l)[3], double (&N)[6]) {
  N[0] = l[0] * (2 * l[0] - 1);
  N[1] = l[1] * (2 * l[1] - 1);
  N[2] = l[2] * (2 * l[2] - 1);
  N[3] = 4 * l[1] * l[2];
  N[4] = 4 * l[0] * l[2];
  N[5] = 4 * l[0] * l[1];
}

// Triangles incident to P2 node (a, b) of the (2nx+1) x (2ny+1) lattice, with
// the node's local index in each; a fixed order (cell row, cell column,
// orientation).  Returns the count (at most 6).
TOPO_HD int p2_node_incidence(int a, int b, int nx, int ny, size_t (&tri)[6], int (&loc)[6]) {
  int n = 0;
  for (int j = b / 2 - 1; j <= b / 2; ++j) {
    if (j < 0 || j >= ny || b - 2 * j > 2) continue;
    for (int i = a / 2 - 1; i <= a / 2; ++i) {
      if (i < 0 || i >= nx || a - 2 * i > 2) continue;
      for (int o = 0; o < 2; ++o)
        for (int k = 0; k < 6; ++k)
          if (p2_off_a(o, k) == a - 2 * i && p2_off_b(o, k) == b - 2 * j) {
            tri[n] = (size_t(j) * nx + i) * 2 + o;
            loc[n] = k;
            ++n;
          }
    }
  }
  return n;
}

TOPO_HD bool fluid_boundary_node(int a, int b, int NX, int NY) {
  return a == 0 || b == 0 || a == NX - 1 || b == NY - 1;
}

// rho at the three vertices of triangle t (cell-major, orientation t & 1)
TOPO_HD void fluid_tri_rho(const double* rho, int nx, size_t t, double (&r)[3]) {
  const int o = int(t & 1);
  const size_t cell = t >> 1;
  const int i = int(cell % nx), j = int(cell / nx);
  for (int k = 0; k < 3; ++k) r[k] = rho[size_t(j + p1_off_b(o, k)) * (nx + 1) + i + p1_off_a(o, k)];
}

TOPO_HD void fluid_tri_nodes(int nx, size_t t, size_t (&n)[6]) {
  const int o = int(t & 1);
  const size_t cell = t >> 1;
  const int i = int(cell % nx), j = int(cell / nx);
  const int NX = 2 * nx + 1;
  for (int k = 0; k < 6; ++k) n[k] = size_t(2 * j + p2_off_b(o, k)) * NX + 2 * i + p2_off_a(o, k);
}

TOPO_HD void fluid_tri_vertices(int nx, size_t t, size_t (&v)[3]) {
  const int o = int(t & 1);
  const size_t cell = t >> 1;
  const int i = int(cell % nx), j = int(cell / nx);
  for (int k = 0; k < 3; ++k) v[k] = size_t(j + p1_off_b(o, k)) * (nx + 1) + i + p1_off_a(o, k);
}

// The alpha-weighted P2 mass matrix of triangle t (upper triangle, kFluidMass values):
// area * sum_q w_q alpha(rho_q) N_i(q) N_j(q), rho_q interpolated from the vertices.
TOPO_HD void fluid_tri_mass(const FluidTables& E, const FluidPenal& pen, const double (&r)[3], double* m) {
  double aw[kFluidQ6];
  for (int q = 0; q < kFluidQ6; ++q) {
    const double rq = r[0] * E.lam6[q][0] + r[1] * E.lam6[q][1] + r[2] * E.lam6[q][2];
    aw[q] = pen.a(rq) * E.w6[q];
  }
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j) {
      double s = 0.0;
      for (int q = 0; q < kFluidQ6; ++q) s += aw[q] * E.N6[q][i] * E.N6[q][j];
      m[fluid_mass_index(i, j)] = E.area * s;
    }
}

// Local rows of the symmetric saddle-point operator on triangle t:
//   out[2i+c] = sum_j (M_ij + K_ij) u_(j,c) + sum_k G_(i,c),k p_k   (momentum)
//   out[12+k] = - sum_(j,c) D_k,(j,c) u_(j,c)                       (continuity, B = -D)
// The sign of the continuity rows makes the assembled operator symmetric on
// velocities that vanish on the boundary ((grad p, v) = -(p, div v) there).
TOPO_HD void fluid_tri_apply(const FluidTables& E, int o, const double* m, const double (&ue)[6][2],
                             const double (&pe)[3], double* out) {
  for (int i = 0; i < 6; ++i)
    for (int c = 0; c < 2; ++c) {
      double s = 0.0;
      for (int j = 0; j < 6; ++j) {
        const double mij = i <= j ? m[fluid_mass_index(i, j)] : m[fluid_mass_index(j, i)];
        s += (mij + E.lap[o][i][j]) * ue[j][c];
      }
      for (int k = 0; k < 3; ++k) s += E.grad[o][i][c][k] * pe[k];
      out[2 * i + c] = s;
    }
  for (int k = 0; k < 3; ++k) {
    double s = 0.0;
    for (int j = 0; j < 6; ++j) s += E.div[o][k][j][0] * ue[j][0] + E.div[o][k][j][1] * ue[j][1];
    out[12 + k] = -s;
  }
  out[15] = 0.0;
}

// Objective integrand of triangle t: area * sum_q w_q (alpha |u|^2 + mu |grad u|^2)
TOPO_HD double fluid_tri_objective(const FluidTables& E, const FluidPenal& pen, double mu, int o,
                                   const double (&r)[3], const double (&ue)[6][2]) {
  double s = 0.0;
  for (int q = 0; q < kFluidQ6; ++q) {
    const double rq = r[0] * E.lam6[q][0] + r[1] * E.lam6[q][1] + r[2] * E.lam6[q][2];
    double u0 = 0.0, u1 = 0.0, g00 = 0.0, g01 = 0.0, g10 = 0.0, g11 = 0.0;
    for (int k = 0; k < 6; ++k) {
      u0 += E.N6[q][k] * ue[k][0];
      u1 += E.N6[q][k] * ue[k][1];
      g00 += E.dN6[o][q][k][0] * ue[k][0];
      g01 += E.dN6[o][q][k][1] * ue[k][0];
      g10 += E.dN6[o][q][k][0] * ue[k][1];
      g11 += E.dN6[o][q][k][1] * ue[k][1];
    }
    const double f = pen.a(rq) * (u0 * u0 + u1 * u1) + mu * (g00 * g00 + g01 * g01 + g10 * g10 + g11 * g11);
    s += f * E.w6[q];
  }
  return E.area * s;
}

// Gradient right-hand side of triangle t: out[k] = int 1/2 alpha'(rho) |u|^2 lambda_k
// with the degree-7 rule.
TOPO_HD void fluid_tri_gradient(const FluidTables& E, const FluidPenal& pen, const double (&r)[3],
                                const double (&ue)[6][2], double (&out)[3]) {
  out[0] = out[1] = out[2] = 0.0;
  for (int q = 0; q < kFluidQ7; ++q) {
    const double rq = r[0] * E.lam7[q][0] + r[1] * E.lam7[q][1] + r[2] * E.lam7[q][2];
    double u0 = 0.0, u1 = 0.0;
    for (int k = 0; k < 6; ++k) {
      u0 += E.N7[q][k] * ue[k][0];
      u1 += E.N7[q][k] * ue[k][1];
    }
    const double f = 0.5 * pen.da(rq) * (u0 * u0 + u1 * u1) * E.w7[q] * E.area;
    for (int k = 0; k < 3; ++k) out[k] += f * E.lam7[q][k];
  }
}

// Gathers of the per-triangle rows (kFluidOut values per triangle) onto the
// P2 nodes and the CG1 vertices.  Velocity node rows: with clamp, boundary
// nodes return x itself (identity rows; the Krylov vectors are zero there).
TOPO_HD void fluid_gather_node(const double* tri_out, int nx, int ny, int a, int b, bool clamp, const double* x,
                               double (&y)[2]) {
  const int NX = 2 * nx + 1, NY = 2 * ny + 1;
  const size_t node = size_t(b) * NX + a;
  if (clamp && fluid_boundary_node(a, b, NX, NY)) {
    y[0] = x[2 * node];
    y[1] = x[2 * node + 1];
    return;
  }
  size_t tri[6];
  int loc[6];
  const int n = p2_node_incidence(a, b, nx, ny, tri, loc);
  double s0 = 0.0, s1 = 0.0;
  for (int e = 0; e < n; ++e) {
    s0 += tri_out[tri[e] * kFluidOut + 2 * loc[e]];
    s1 += tri_out[tri[e] * kFluidOut + 2 * loc[e] + 1];
  }
  y[0] = s0;
  y[1] = s1;
}

TOPO_HD double fluid_gather_vertex(const double* tri_out, int nx, int ny, int a, int b, int stride, int offset) {
  // CG1 vertex (a, b): the six incidences of the right-diagonal lattice
  const int inc[6][4] = {{-1, -1, 0, 2}, {-1, -1, 1, 2}, {0, -1, 1, 1}, {-1, 0, 0, 1}, {0, 0, 0, 0}, {0, 0, 1, 0}};
  double s = 0.0;
  for (int e = 0; e < 6; ++e) {
    const int ci = a + inc[e][0], cj = b + inc[e][1];
    if (ci < 0 || ci >= nx || cj < 0 || cj >= ny) continue;
    const size_t t = (size_t(cj) * nx + ci) * 2 + inc[e][2];
    s += tri_out[t * stride + offset + inc[e][3]];
  }
  return s;
}

}  // namespace topo
