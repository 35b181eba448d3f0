// Host-side set-up of a design problem: clamped-node description, lumped
// CG1 weights and the pre-assembled load vector.  Header-only so the test
// emulator can check it against the FP64 oracle on the CPU.
#pragma once

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "topomax_gb300.h"
#include "topo_common.cuh"

namespace topo {

constexpr double kDolfinEps = 3e-16;  // DOLFIN_EPS of df.between / df.near

inline Dir no_dir(int NX, int NY) {
  Dir d;
  std::memset(&d, 0, sizeof(d));
  d.x_hi_from = NX;
  d.y_hi_from = NY;
  return d;
}

// Clamped P2 nodes: whole sides (topological DirichletBC on the facets marked by
// SidesDomain, FEM_src/domains.py:18-38 -- vertex and edge nodes of the side)
// plus optional clamped vertices.  Returns non-zero with a message on bad input.
inline int make_p2_dir(int nx, int ny, double hx, double hy, const topo_bc_desc* bc, Dir& d, std::string& msg) {
  const int NX = 2 * nx + 1, NY = 2 * ny + 1;
  d = no_dir(NX, NY);
  const int sides = bc ? bc->fixed_sides : 0;
  if (sides & ~15) {
    msg = "Malformed side mask";
    return 1;
  }
  d.x_lo = (sides & TOPO_SIDE_LEFT) ? 1 : 0;
  d.y_lo = (sides & TOPO_SIDE_BOTTOM) ? 1 : 0;
  if (sides & TOPO_SIDE_RIGHT) d.x_hi_from = NX - 1;
  if (sides & TOPO_SIDE_TOP) d.y_hi_from = NY - 1;
  if (bc && bc->n_fixed_points > 0) {
    if (bc->n_fixed_points > kMaxDirPoints || !bc->fixed_points) {
      msg = "too many fixed points";
      return 1;
    }
    for (int k = 0; k < bc->n_fixed_points; ++k) {
      const int i = int(std::lround(bc->fixed_points[2 * k] / hx));
      const int j = int(std::lround(bc->fixed_points[2 * k + 1] / hy));
      if (i < 0 || i > nx || j < 0 || j > ny) {
        msg = "fixed point outside the domain";
        return 1;
      }
      d.pts[2 * d.npts] = 2 * i;
      d.pts[2 * d.npts + 1] = 2 * j;
      ++d.npts;
    }
  }
  return 0;
}

// int phi_i dx of every CG1 basis function: sum of |T|/3 over incident triangles
// (the weights FEMSolver.integrate's assemble(f*dx) applies, FEM_src/solver.py:81-84).
inline std::vector<double> vertex_weights(int nx, int ny, double hx, double hy) {
  std::vector<double> w(size_t(nx + 1) * (ny + 1), 0.0);
  const double a3 = 0.5 * hx * hy / 3.0;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i)
      for (int o = 0; o < 2; ++o)
        for (int k = 0; k < 3; ++k) w[size_t(j + p1_off_b(o, k)) * (nx + 1) + i + p1_off_a(o, k)] += a3;
  return w;
}

// Vertex coordinates as dolfin's RectangleMesh computes them (x_i = a + i*(b-a)/nx),
// P2 edge nodes at 0.5*x_a + 0.5*x_b (the dof points of an interpolated expression).
inline void lattice_coords(double W, int nx, std::vector<double>& X2) {
  const double ab = W / nx;
  X2.assign(2 * nx + 1, 0.0);
  for (int i = 0; i <= nx; ++i) X2[2 * i] = 0.0 + i * ab;
  for (int i = 0; i < nx; ++i) X2[2 * i + 1] = 0.5 * X2[2 * i] + 0.5 * X2[2 * i + 2];
}

// TractionExpression.eval (FEM_src/elasisity_problem.py:39-73)
inline void traction_at(const topo_load_desc* L, double W, double H, double x, double y, double& vx, double& vy) {
  vx = vy = 0.0;
  for (int k = 0; k < L->n_tractions; ++k) {
    const topo_traction& t = L->tractions[k];
    const double lo = t.center - t.length / 2, hi = t.center + t.length / 2;
    bool hit = false;
    switch (t.side) {
      case TOPO_SIDE_LEFT: hit = (x == 0.0) && lo - kDolfinEps <= y && y <= hi + kDolfinEps; break;
      case TOPO_SIDE_RIGHT: hit = (x == W) && lo - kDolfinEps <= y && y <= hi + kDolfinEps; break;
      case TOPO_SIDE_TOP: hit = (y == H) && lo - kDolfinEps <= x && x <= hi + kDolfinEps; break;
      case TOPO_SIDE_BOTTOM: hit = (y == 0.0) && lo - kDolfinEps <= x && x <= hi + kDolfinEps; break;
      default: break;
    }
    if (hit) {
      vx += t.value_x;
      vy += t.value_y;
    }
  }
}

// Pre-assembled load vector L = (f, v) dx + (t, v) ds with the body-force indicator
// (BodyForce.eval, FEM_src/elasisity_problem.py:20-36) and the traction interpolated
// at P2 nodes and integrated exactly; clamped dofs zero.
inline void assemble_load(int nx, int ny, double W, double H, const Dir& dir, const topo_load_desc* L,
                          std::vector<double>& b) {
  const int NX = 2 * nx + 1, NY = 2 * ny + 1;
  const double hx = W / nx, hy = H / ny;
  b.assign(size_t(2) * NX * NY, 0.0);
  std::vector<double> X2, Y2;
  lattice_coords(W, nx, X2);
  lattice_coords(H, ny, Y2);
  if (L && L->has_body_force) {
    std::vector<unsigned char> in(size_t(NX) * NY, 0);
    bool any = false;
    for (int bb = 0; bb < NY; ++bb)
      for (int a = 0; a < NX; ++a) {
        const double dx = X2[a] - L->center_x, dy = Y2[bb] - L->center_y;
        if (std::sqrt(dx * dx + dy * dy) < L->radius) {
          in[size_t(bb) * NX + a] = 1;
          any = true;
        }
      }
    if (any) {
      // P2 mass matrix, local order (A,B,C,mid(BC),mid(AC),mid(AB)), times 180/|T|
      const double Mr[6][6] = {{6, -1, -1, -4, 0, 0}, {-1, 6, -1, 0, -4, 0}, {-1, -1, 6, 0, 0, -4},
                               {-4, 0, 0, 32, 16, 16}, {0, -4, 0, 16, 32, 16}, {0, 0, -4, 16, 16, 32}};
      const double sc = 0.5 * hx * hy / 180.0;
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i)
          for (int o = 0; o < 2; ++o) {
            size_t nodes[6];
            bool hit = false;
            for (int k = 0; k < 6; ++k) {
              nodes[k] = size_t(2 * j + p2_off_b(o, k)) * NX + 2 * i + p2_off_a(o, k);
              hit |= in[nodes[k]] != 0;
            }
            if (!hit) continue;
            for (int m = 0; m < 6; ++m) {
              double s = 0.0;
              for (int k = 0; k < 6; ++k) s += Mr[m][k] * (in[nodes[k]] ? 1.0 : 0.0);
              b[2 * nodes[m]] += sc * s * L->value_x;
              b[2 * nodes[m] + 1] += sc * s * L->value_y;
            }
          }
    }
  }
  if (L && L->n_tractions > 0) {
    const double Mf[3][3] = {{4, 2, -1}, {2, 16, 2}, {-1, 2, 4}};
    auto facet = [&](const size_t (&nodes)[3], const double (&xs)[3], const double (&ys)[3], double h) {
      double tv[3][2];
      bool any = false;
      for (int k = 0; k < 3; ++k) {
        traction_at(L, W, H, xs[k], ys[k], tv[k][0], tv[k][1]);
        any |= (tv[k][0] != 0.0 || tv[k][1] != 0.0);
      }
      if (!any) return;
      for (int m = 0; m < 3; ++m)
        for (int c = 0; c < 2; ++c) {
          double s = 0.0;
          for (int k = 0; k < 3; ++k) s += Mf[m][k] * tv[k][c];
          b[2 * nodes[m] + c] += h / 30.0 * s;
        }
    };
    for (int i = 0; i < nx; ++i)
      for (int bb : {0, NY - 1}) {
        const size_t nodes[3] = {size_t(bb) * NX + 2 * i, size_t(bb) * NX + 2 * i + 1, size_t(bb) * NX + 2 * i + 2};
        const double xs[3] = {X2[2 * i], X2[2 * i + 1], X2[2 * i + 2]};
        const double ys[3] = {Y2[bb], Y2[bb], Y2[bb]};
        facet(nodes, xs, ys, hx);
      }
    for (int j = 0; j < ny; ++j)
      for (int a : {0, NX - 1}) {
        const size_t nodes[3] = {size_t(2 * j) * NX + a, size_t(2 * j + 1) * NX + a, size_t(2 * j + 2) * NX + a};
        const double xs[3] = {X2[a], X2[a], X2[a]};
        const double ys[3] = {Y2[2 * j], Y2[2 * j + 1], Y2[2 * j + 2]};
        facet(nodes, xs, ys, hy);
      }
  }
  for (int bb = 0; bb < NY; ++bb)
    for (int a = 0; a < NX; ++a)
      if (is_clamped(dir, a, bb)) {
        b[2 * (size_t(bb) * NX + a)] = 0.0;
        b[2 * (size_t(bb) * NX + a) + 1] = 0.0;
      }
}

}  // namespace topo
