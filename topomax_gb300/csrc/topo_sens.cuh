// Sensitivity right-hand side kernels: per-triangle moments into a scratch
// array, then a gather onto the CG1 vertices (deterministic, no atomics).
#pragma once

#include "topo_p1.cuh"
#include "topo_p2.cuh"
#include "topo_vec.cuh"

namespace topo {

// moments of triangle O of a cell from the cell's node values U (3x3 nodes) and
// vertex densities X (2x2), in the node orders of P2Off / P1Off
template <int O, class TG, class TQ>
__device__ __forceinline__ void sens_cell_tri(const TG (&U)[3][3][2], const TQ (&X)[2][2], TG ihx, TG ihy, TQ lam,
                                              TQ mu, TQ area, const Penal<TQ>& pen, TQ (&c)[3]) {
  TG ue[6][2];
#define TOPO_UE(K)                                      \
  ue[K][0] = U[P2Off<O, K>::b][P2Off<O, K>::a][0];      \
  ue[K][1] = U[P2Off<O, K>::b][P2Off<O, K>::a][1];
  TOPO_UE(0) TOPO_UE(1) TOPO_UE(2) TOPO_UE(3) TOPO_UE(4) TOPO_UE(5)
#undef TOPO_UE
  const TQ xe[3] = {X[P1Off<O, 0>::b][P1Off<O, 0>::a], X[P1Off<O, 1>::b][P1Off<O, 1>::a],
                    X[P1Off<O, 2>::b][P1Off<O, 2>::a]};
  tri_sensitivity<O, TG, TQ>(ue, xe, ihx, ihy, lam, mu, area, pen, c);
}

// out[3t+k] = int_T s phi_k for every triangle t (FEM_src/elasisity_problem.py:146-149).
// One thread per cell: the cell's 3x3 P2 nodes and 2x2 vertices are loaded once
// and both triangles are evaluated with compile-time node offsets, so the lanes
// of a warp run the same instructions (a thread per triangle would alternate
// orientations within the warp and run both code paths).  Output t = 2 cell + o:
// six consecutive values per cell.
template <class TQ>
__global__ void k_sens_tri(int nx, int ny, double ihx, double ihy, TQ lam, TQ mu, TQ area, Penal<TQ> pen,
                           const double* __restrict__ u, const double* __restrict__ xi, TQ* __restrict__ out) {
  const size_t ncell = size_t(nx) * ny;
  const int VX = nx + 1, NX = 2 * nx + 1;
  TOPO_GRID_STRIDE(cell, ncell) {
    const int i = int(cell % nx), j = int(cell / nx);
    double un[3][3][2];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t n = size_t(2 * j + r) * NX + 2 * i + c;
        un[r][c][0] = u[2 * n];
        un[r][c][1] = u[2 * n + 1];
      }
    TQ xv[2][2];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const double x = xi[size_t(j + r) * VX + i + c];
        if constexpr (sizeof(TQ) == 4) xv[r][c] = float_from_double(x);  // (integer pipe)
        else xv[r][c] = TQ(x);
      }
    TQ c0[3], c1[3];
    if constexpr (sizeof(TQ) == 4) {
      // difference form: the gradient ignores a translation, so the node values enter as
      // u - u_A (vertex A = node (0,0) of both triangles), rounded to FP32, where the
      // gradients and the quadrature run.  The difference is taken on the FP32 pipe from
      // the values' (hi, lo) splits (FP64 arithmetic is scarce on this GPU): hi - hi is
      // exact for nearby values, and lo - lo carries the rest, so the float result is
      // within a rounding or two of the FP64 difference rounded to FP32.
      dd us[3][3][2];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 2; ++d) us[r][c][d] = dd_from_double(un[r][c][d]);
      TQ ud[3][3][2];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 2; ++d)
            ud[r][c][d] = (r | c) ? ddop::add(ddop::sub(us[r][c][d].hi, us[0][0][d].hi),
                                              ddop::sub(us[r][c][d].lo, us[0][0][d].lo))
                                  : TQ(0);
      sens_cell_tri<0>(ud, xv, TQ(ihx), TQ(ihy), lam, mu, area, pen, c0);
      sens_cell_tri<1>(ud, xv, TQ(ihx), TQ(ihy), lam, mu, area, pen, c1);
    } else {
      sens_cell_tri<0>(un, xv, ihx, ihy, lam, mu, area, pen, c0);
      sens_cell_tri<1>(un, xv, ihx, ihy, lam, mu, area, pen, c1);
    }
    TQ* o = out + 6 * cell;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      o[k] = c0[k];
      o[3 + k] = c1[k];
    }
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
