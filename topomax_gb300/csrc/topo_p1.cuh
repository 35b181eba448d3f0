// P1 lattice operators: the coarse levels of the elasticity multigrid
// hierarchy (NC = 2) and every level of the Helmholtz filter (NC = 1,
// FEM_src/filter.py:15-41: a = eps^2 (grad u, grad v) + (u, v)).
//
// A level's operator is  sum_T kK_T Kref_o + kM_T Mref_o  with per-triangle
// coefficients.  The first P1 level under the P2 operator uses
// kK_T = (1/|T|) int_T r(xi) (exact Galerkin projection of the P2 form onto
// P1), coarser levels average the four child triangles (exact Galerkin for
// nested P1 spaces; children outside the domain of an odd-sized level count
// as zero).
#pragma once

#include "topo_common.cuh"

namespace topo {

template <class T, int NC>
struct P1Params {
  int nx, ny;  // cells of this level
  Dir dir;
  T K[2][3 * NC][3 * NC];  // unit-coefficient element stiffness per orientation
  T Mm[2][3][3];           // unit-coefficient element mass (used when NC == 1)
  const T* kK;             // per-triangle coefficients (null: kK_c)
  const T* kM;             // per-triangle mass coefficients (null: kM_c)
  T kK_c, kM_c;
};

// The six (cell offset, orientation, local vertex) incidences of vertex (a,b).
TOPO_HD void p1_incidence(int e, int& dci, int& dcj, int& o, int& loc) {
  const int t[6][4] = {{-1, -1, 0, 2}, {-1, -1, 1, 2}, {0, -1, 1, 1},
                       {-1, 0, 0, 1},  {0, 0, 0, 0},   {0, 0, 1, 0}};
  dci = t[e][0]; dcj = t[e][1]; o = t[e][2]; loc = t[e][3];
}

template <class T, int NC>
struct P1Kern {
  TOPO_HD static void node_apply(int a, int b, const P1Params<T, NC>& P, const T* u, T* y) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    if (is_clamped(P.dir, a, b)) {
      for (int c = 0; c < NC; ++c) y[NC * n + c] = u[NC * n + c];
      return;
    }
    T acc[NC];
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    for (int e = 0; e < 6; ++e) {
      int dci, dcj, o, loc;
      p1_incidence(e, dci, dcj, o, loc);
      const int ci = a + dci, cj = b + dcj;
      if (ci < 0 || ci >= P.nx || cj < 0 || cj >= P.ny) continue;
      const size_t t = (size_t(cj) * P.nx + ci) * 2 + o;
      const T kk = P.kK ? P.kK[t] : P.kK_c;
      const T km = (NC == 1) ? (P.kM ? P.kM[t] : P.kM_c) : T(0);
      for (int l = 0; l < 3; ++l) {
        const int al = ci + p1_off_a(o, l), bl = cj + p1_off_b(o, l);
        if (is_clamped(P.dir, al, bl)) continue;
        const size_t m = size_t(bl) * NX + al;
        T ul[NC];
        for (int d = 0; d < NC; ++d) ul[d] = u[NC * m + d];
        for (int c = 0; c < NC; ++c) {
          T s = T(0);
          for (int d = 0; d < NC; ++d) s += P.K[o][loc * NC + c][l * NC + d] * ul[d];
          acc[c] += kk * s;
          if (NC == 1) acc[c] += km * P.Mm[o][loc][l] * ul[c];
        }
      }
    }
    for (int c = 0; c < NC; ++c) y[NC * n + c] = acc[c];
  }

  TOPO_HD static void node_diag(int a, int b, const P1Params<T, NC>& P, T* d) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    if (is_clamped(P.dir, a, b)) {
      for (int c = 0; c < NC; ++c) d[NC * n + c] = T(1);
      return;
    }
    T acc[NC];
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    for (int e = 0; e < 6; ++e) {
      int dci, dcj, o, loc;
      p1_incidence(e, dci, dcj, o, loc);
      const int ci = a + dci, cj = b + dcj;
      if (ci < 0 || ci >= P.nx || cj < 0 || cj >= P.ny) continue;
      const size_t t = (size_t(cj) * P.nx + ci) * 2 + o;
      const T kk = P.kK ? P.kK[t] : P.kK_c;
      const T km = (NC == 1) ? (P.kM ? P.kM[t] : P.kM_c) : T(0);
      for (int c = 0; c < NC; ++c) {
        acc[c] += kk * P.K[o][loc * NC + c][loc * NC + c];
        if (NC == 1) acc[c] += km * P.Mm[o][loc][loc];
      }
    }
    for (int c = 0; c < NC; ++c) d[NC * n + c] = acc[c];
  }
};

// Coarse coefficient of coarse triangle (I,J,o): mean of its four children
// on the fine level (fine cells beyond nxf x nyf contribute zero).
template <class T>
TOPO_HD T coarsen_kappa(const T* kf, int nxf, int nyf, int I, int J, int o) {
  // children (dci, dcj, orientation)
  const int ch[2][4][3] = {{{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 0}},
                           {{0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 1, 1}}};
  T s = T(0);
  for (int k = 0; k < 4; ++k) {
    const int i = 2 * I + ch[o][k][0], j = 2 * J + ch[o][k][1];
    if (i < nxf && j < nyf) s += kf[(size_t(j) * nxf + i) * 2 + ch[o][k][2]];
  }
  return T(0.25) * s;
}

// Lattice transfers between a fine lattice (NXf x NYf) and the coarse lattice
// (NXc x NYc) whose node (I,J) sits on fine node (2I,2J).  Used for P2 -> P1
// on the same mesh and for P1(h) -> P1(2h): in both cases the coarse hat
// function is 1 at (2I,2J) and 1/2 at the midpoints of the coarse edges out of
// (I,J): (2I+-1,2J), (2I,2J+-1), (2I+1,2J+1), (2I-1,2J-1).
struct Transfer {
  int NXf, NYf, NXc, NYc;
  Dir dirf, dirc;
};

template <class T, int NC>
struct TransferKern {
  // b_c = P^T r_f
  TOPO_HD static void node_restrict(int I, int J, const Transfer& X, const T* rf, T* bc) {
    const size_t nc = size_t(J) * X.NXc + I;
    if (is_clamped(X.dirc, I, J)) {
      for (int c = 0; c < NC; ++c) bc[NC * nc + c] = T(0);
      return;
    }
    const int a = 2 * I, b = 2 * J;
    const int nb[6][2] = {{a - 1, b}, {a + 1, b}, {a, b - 1}, {a, b + 1}, {a + 1, b + 1}, {a - 1, b - 1}};
    for (int c = 0; c < NC; ++c) {
      T s = T(0);
      if (a < X.NXf && b < X.NYf) s = rf[NC * (size_t(b) * X.NXf + a) + c];
      T h = T(0);
      for (int k = 0; k < 6; ++k) {
        const int aa = nb[k][0], bb = nb[k][1];
        if (aa >= 0 && aa < X.NXf && bb >= 0 && bb < X.NYf)
          h += rf[NC * (size_t(bb) * X.NXf + aa) + c];
      }
      bc[NC * nc + c] = s + T(0.5) * h;
    }
  }

  // x_f += P x_c
  TOPO_HD static void node_prolong_add(int a, int b, const Transfer& X, const T* xc, T* xf) {
    if (is_clamped(X.dirf, a, b)) return;
    const size_t nf = size_t(b) * X.NXf + a;
    const int pa = a & 1, pb = b & 1;
    const int I0 = (a - pa) >> 1, J0 = (b - pb) >> 1;  // floor(a/2), floor(b/2)
    for (int c = 0; c < NC; ++c) {
      T v;
      const T x00 = xc[NC * (size_t(J0) * X.NXc + I0) + c];
      if (!pa && !pb) v = x00;
      else if (pa && !pb) v = T(0.5) * (x00 + xc[NC * (size_t(J0) * X.NXc + I0 + 1) + c]);
      else if (!pa && pb) v = T(0.5) * (x00 + xc[NC * (size_t(J0 + 1) * X.NXc + I0) + c]);
      else v = T(0.5) * (x00 + xc[NC * (size_t(J0 + 1) * X.NXc + I0 + 1) + c]);
      xf[NC * nf + c] += v;
    }
  }
};

}  // namespace topo
