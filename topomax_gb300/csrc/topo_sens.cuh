// Sensitivity right-hand side kernels: per-triangle moments into a scratch
// array, then a gather onto the CG1 vertices (deterministic, no atomics).
#pragma once

#include "topo_p1.cuh"
#include "topo_p2.cuh"
#include "topo_vec.cuh"

namespace topo {

// out[3t+k] = int_T s phi_k for every triangle t (FEM_src/elasisity_problem.py:146-149)
template <class TQ>
__global__ void k_sens_tri(int nx, int ny, double ihx, double ihy, TQ lam, TQ mu, TQ area, Penal<TQ> pen,
                           const double* __restrict__ u, const double* __restrict__ xi, TQ* __restrict__ out) {
  const size_t nt = size_t(2) * nx * ny;
  const int VX = nx + 1, NX = 2 * nx + 1;
  TOPO_GRID_STRIDE(t, nt) {
    const int o = int(t & 1);
    const size_t cell = t >> 1;
    const int i = int(cell % nx), j = int(cell / nx);
    double ue[6][2];
    for (int k = 0; k < 6; ++k) {
      const size_t n = size_t(2 * j + p2_off_b(o, k)) * NX + 2 * i + p2_off_a(o, k);
      ue[k][0] = u[2 * n];
      ue[k][1] = u[2 * n + 1];
    }
    TQ xe[3];
    for (int k = 0; k < 3; ++k) xe[k] = TQ(xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)]);
    TQ c[3];
    if constexpr (sizeof(TQ) == 4) {
      // difference form: the gradient ignores a translation, so the node values enter as
      // u - u_A, subtracted in FP64 (exact for a smooth field) and rounded to FP32, where
      // the gradients and the quadrature run (FP64 arithmetic is scarce on this GPU)
      TQ ud[6][2];
      for (int k = 0; k < 6; ++k)
        for (int d = 0; d < 2; ++d) ud[k][d] = k == 0 ? TQ(0) : TQ(ue[k][d] - ue[0][d]);
      if (o == 0) tri_sensitivity<0, TQ, TQ>(ud, xe, TQ(ihx), TQ(ihy), lam, mu, area, pen, c);
      else tri_sensitivity<1, TQ, TQ>(ud, xe, TQ(ihx), TQ(ihy), lam, mu, area, pen, c);
    } else {
      if (o == 0) tri_sensitivity<0, double, TQ>(ue, xe, ihx, ihy, lam, mu, area, pen, c);
      else tri_sensitivity<1, double, TQ>(ue, xe, ihx, ihy, lam, mu, area, pen, c);
    }
    out[3 * t] = c[0];
    out[3 * t + 1] = c[1];
    out[3 * t + 2] = c[2];
  }
}

template <class TQ>
__global__ void k_vertex_gather3(int nx, int ny, const TQ* __restrict__ tri3, double* __restrict__ b) {
  const int VX = nx + 1;
  const size_t nv = size_t(nx + 1) * (ny + 1);
  TOPO_GRID_STRIDE(v, nv) {
    const int a = int(v % VX), bb = int(v / VX);
    double s = 0.0;
    for (int e = 0; e < 6; ++e) {
      int dci, dcj, o, loc;
      p1_incidence(e, dci, dcj, o, loc);
      const int ci = a + dci, cj = bb + dcj;
      if (ci < 0 || ci >= nx || cj < 0 || cj >= ny) continue;
      const size_t t = (size_t(cj) * nx + ci) * 2 + o;
      s += double(tri3[3 * t + loc]);
    }
    b[v] = s;
  }
}


}  // namespace topo
