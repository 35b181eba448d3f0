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

#include <cmath>

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
// Packed five bits per incidence e (at bit 5 e): dci + 1, dcj + 1, o, loc (two bits):
//   e = 0..5: (-1,-1,0,2) (-1,-1,1,2) (0,-1,1,1) (-1,0,0,1) (0,0,0,0) (0,0,1,0)
TOPO_HD constexpr unsigned p1_incidence_bits(int e) { return (0xe353690u >> (5 * e)) & 31u; }
TOPO_HD void p1_incidence(int e, int& dci, int& dcj, int& o, int& loc) {
  const unsigned f = p1_incidence_bits(e);
  dci = int(f & 1u) - 1;
  dcj = int((f >> 1) & 1u) - 1;
  o = int((f >> 2) & 1u);
  loc = int(f >> 3);
}

// Input of a node apply read directly from an array.
template <class T, int NC>
struct FetchArray {
  const T* u;
  TOPO_HD void operator()(size_t m, int, int, T (&v)[NC]) const {
    for (int d = 0; d < NC; ++d) v[d] = u[NC * m + d];
  }
};

template <class T, int NC>
struct P1Kern {
  // contribution of incidence (dci, dcj, O, LOC) of vertex (a,b) to y; chk
  // enables the clamped-neighbour test (only needed near clamped nodes)
  template <int DCI, int DCJ, int O, int LOC, class F>
  TOPO_HD static void inc(int a, int b, const P1Params<T, NC>& P, const F& fetch, bool chk, T (&acc)[NC]) {
    const int ci = a + DCI, cj = b + DCJ;
    if (ci < 0 || ci >= P.nx || cj < 0 || cj >= P.ny) return;
    const int NX = P.nx + 1;
    const size_t t = (size_t(cj) * P.nx + ci) * 2 + O;
    const T kk = P.kK ? P.kK[t] : P.kK_c;
    T km = T(0);
    if constexpr (NC == 1) km = P.kM ? P.kM[t] : P.kM_c;
#define TOPO_P1_NB(L)                                                                     \
  {                                                                                       \
    const int al = ci + P1Off<O, L>::a, bl = cj + P1Off<O, L>::b;                         \
    if (!(chk && is_clamped(P.dir, al, bl))) {                                            \
      T ul[NC];                                                                           \
      fetch(size_t(bl) * NX + al, al, bl, ul);                                            \
      for (int c = 0; c < NC; ++c) {                                                      \
        T sacc = T(0);                                                                    \
        for (int d = 0; d < NC; ++d) sacc += P.K[O][LOC * NC + c][L * NC + d] * ul[d];    \
        acc[c] += kk * sacc;                                                              \
        if constexpr (NC == 1) acc[c] += km * P.Mm[O][LOC][L] * ul[c];                    \
      }                                                                                   \
    }                                                                                     \
  }
    TOPO_P1_NB(0) TOPO_P1_NB(1) TOPO_P1_NB(2)
#undef TOPO_P1_NB
  }

  TOPO_HD static bool near_clamped(const Dir& d, int a, int b) {
    return d.npts > 0 || (d.x_lo && a <= 1) || (d.y_lo && b <= 1) || a + 1 >= d.x_hi_from || b + 1 >= d.y_hi_from;
  }

  // t = (A u)(a,b) with u read through fetch; returns false for a clamped node
  // (identity row: the caller uses u itself)
  template <class F>
  TOPO_HD static bool node_eval(int a, int b, const P1Params<T, NC>& P, const F& fetch, T (&acc)[NC]) {
    const bool chk = near_clamped(P.dir, a, b);
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    if (chk && is_clamped(P.dir, a, b)) return false;
    // the six incidences (cell offset, orientation, local vertex) of vertex (a,b)
    inc<-1, -1, 0, 2>(a, b, P, fetch, chk, acc);
    inc<-1, -1, 1, 2>(a, b, P, fetch, chk, acc);
    inc<0, -1, 1, 1>(a, b, P, fetch, chk, acc);
    inc<-1, 0, 0, 1>(a, b, P, fetch, chk, acc);
    inc<0, 0, 0, 0>(a, b, P, fetch, chk, acc);
    inc<0, 0, 1, 0>(a, b, P, fetch, chk, acc);
    return true;
  }

  TOPO_HD static void node_apply(int a, int b, const P1Params<T, NC>& P, const T* u, T* y) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    T acc[NC];
    if (!node_eval(a, b, P, FetchArray<T, NC>{u}, acc))
      for (int c = 0; c < NC; ++c) acc[c] = u[NC * n + c];
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
  // children k = 0..3 of coarse triangle o: (dci, dcj, orientation) as bits 0, 1, 2
  // of the 3-bit field 4 o + k:  o = 0: (0,0,0) (1,0,0) (1,0,1) (1,1,0);
  //                              o = 1: (0,0,1) (0,1,1) (0,1,0) (1,1,1)
  T s = T(0);
  for (int k = 0; k < 4; ++k) {
    const unsigned c = (0xeb4748u >> (3 * (4 * o + k))) & 7u;
    const int i = 2 * I + int(c & 1u), j = 2 * J + int((c >> 1) & 1u);
    if (i < nxf && j < nyf) s += kf[(size_t(j) * nxf + i) * 2 + int(c >> 2)];
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
  // b_c = P^T r_f, with r_f = bf - tf when tf is given (the fine residual)
  TOPO_HD static void node_restrict(int I, int J, const Transfer& X, const T* rf, T* bc, const T* tf = nullptr) {
    const size_t nc = size_t(J) * X.NXc + I;
    if (is_clamped(X.dirc, I, J)) {
      for (int c = 0; c < NC; ++c) bc[NC * nc + c] = T(0);
      return;
    }
    const int a = 2 * I, b = 2 * J;
    const int nb[6][2] = {{a - 1, b}, {a + 1, b}, {a, b - 1}, {a, b + 1}, {a + 1, b + 1}, {a - 1, b - 1}};
    for (int c = 0; c < NC; ++c) {
      T s = T(0);
      if (a < X.NXf && b < X.NYf) {
        const size_t m = NC * (size_t(b) * X.NXf + a) + c;
        s = tf ? rf[m] - tf[m] : rf[m];
      }
      T h = T(0);
      for (int k = 0; k < 6; ++k) {
        const int aa = nb[k][0], bb = nb[k][1];
        if (aa >= 0 && aa < X.NXf && bb >= 0 && bb < X.NYf) {
          const size_t m = NC * (size_t(bb) * X.NXf + aa) + c;
          h += tf ? rf[m] - tf[m] : rf[m];
        }
      }
      bc[NC * nc + c] = s + T(0.5) * h;
    }
  }

  // (P x_c) at fine node (a,b) (0 at clamped fine nodes)
  TOPO_HD static void prolong_value(int a, int b, const Transfer& X, const T* xc, T (&v)[NC]) {
    if (is_clamped(X.dirf, a, b)) {
      for (int c = 0; c < NC; ++c) v[c] = T(0);
      return;
    }
    const int pa = a & 1, pb = b & 1;
    const int I0 = (a - pa) >> 1, J0 = (b - pb) >> 1;
    for (int c = 0; c < NC; ++c) {
      const T x00 = xc[NC * (size_t(J0) * X.NXc + I0) + c];
      if (!pa && !pb) v[c] = x00;
      else if (pa && !pb) v[c] = T(0.5) * (x00 + xc[NC * (size_t(J0) * X.NXc + I0 + 1) + c]);
      else if (!pa && pb) v[c] = T(0.5) * (x00 + xc[NC * (size_t(J0 + 1) * X.NXc + I0) + c]);
      else v[c] = T(0.5) * (x00 + xc[NC * (size_t(J0 + 1) * X.NXc + I0 + 1) + c]);
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

namespace topo {

// ---------------------------------------------------------------------------
// assembled 7-point stencil of a P1 level
// ---------------------------------------------------------------------------
// On the right-diagonal triangulation node (a,b) couples to itself and to
// (a+-1,b), (a,b+-1), (a+1,b+1), (a-1,b-1).  For the small levels the NC x NC
// coupling blocks are assembled once per coefficient update, so that a node
// evaluation is seven independent block products instead of a chain through
// six incidences' element matrices, coefficients and clamping tests (the
// smallest levels are bound by that chain's latency, not by bandwidth).
// Columns of clamped nodes are zero; a clamped node's own row is the
// identity (its evaluation reports "clamped" as P1Kern does).  Block 0 is
// stored as the row sum (difference form, see p1_stencil_node).
template <int NC>
struct StencilLayout {
  static constexpr int stride = NC == 2 ? 28 : 8;  // values per node: 7 blocks, padded to 16 bytes
};
TOPO_HD constexpr int st_da(int k) { return k == 1 ? 1 : k == 2 ? -1 : k == 5 ? 1 : k == 6 ? -1 : 0; }
TOPO_HD constexpr int st_db(int k) { return k == 3 ? 1 : k == 4 ? -1 : k == 5 ? 1 : k == 6 ? -1 : 0; }
// block of offset (da, db): 0 self, 1 E, 2 W, 3 N, 4 S, 5 NE, 6 SW
TOPO_HD constexpr int st_block(int da, int db) {
  if (da == 0) return db == 0 ? 0 : db == 1 ? 3 : 4;
  if (db == 0) return da == 1 ? 1 : 2;
  return da == 1 ? 5 : 6;
}

template <class T, int NC>
struct P1Stencil {
  int nx, ny;  // cells of this level
  Dir dir;
  const T* s;  // node n, block k, row c, column d at s[n*stride + k*NC*NC + c*NC + d]; block 0: row sum
  // optional: the one stencil row shared by every interior node (a level with
  // constant coefficients and no clamped nodes, e.g. the filter): interior
  // nodes read it instead of their own row (null: every node reads its row)
  const T* inner = nullptr;
};

// Stencil row of node (a,b) assembled from the level's coefficients (the
// same incidences and clamping rules as P1Kern::node_eval), in difference
// form: block 0 holds the row sum S_0 = sum_k A_(n,k) (accumulated in FP64),
// blocks 1..6 the neighbour couplings, and
//     (A u)_n = S_0 u_n + sum_(k>=1) A_(n,k) (u_k - u_n).
// The row sum of an elasticity or filter row is small against its entries
// (zero for rigid translations, the mass for the filter), so summing rounded
// entries at run time would lose the smooth modes' accuracy in FP32.
template <class T, int NC>
TOPO_HD void p1_stencil_node(int a, int b, const P1Params<T, NC>& P, T* out) {
  constexpr int SB = NC * NC;
  T blk[7 * SB];
  double rs[SB];
  for (int i = 0; i < 7 * SB; ++i) blk[i] = T(0);
  for (int i = 0; i < SB; ++i) rs[i] = 0.0;
  for (int i = 7 * SB; i < StencilLayout<NC>::stride; ++i) out[i] = T(0);
  if (is_clamped(P.dir, a, b)) {
    for (int c = 0; c < NC; ++c) rs[c * NC + c] = 1.0;
  } else {
    const bool chk = P1Kern<T, NC>::near_clamped(P.dir, a, b);
    // fully unrolled on the GPU: every block index is then a constant and the
    // row stays in registers
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int e = 0; e < 6; ++e) {
      int dci, dcj, o, loc;
      p1_incidence(e, dci, dcj, o, loc);
      const int ci = a + dci, cj = b + dcj;
      if (ci < 0 || ci >= P.nx || cj < 0 || cj >= P.ny) continue;
      const size_t t = (size_t(cj) * P.nx + ci) * 2 + o;
      const double kk = P.kK ? double(P.kK[t]) : double(P.kK_c);
      const double km = (NC == 1) ? (P.kM ? double(P.kM[t]) : double(P.kM_c)) : 0.0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
      for (int L = 0; L < 3; ++L) {
        const int da = dci + p1_off_a(o, L), db = dcj + p1_off_b(o, L);
        if (chk && is_clamped(P.dir, a + da, b + db)) continue;
        T* bk = blk + st_block(da, db) * SB;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int c = 0; c < NC; ++c)
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
          for (int d = 0; d < NC; ++d) {
            double v = kk * double(P.K[o][loc * NC + c][L * NC + d]);
            if (NC == 1) v += km * double(P.Mm[o][loc][L]);
            bk[c * NC + d] += T(v);
            rs[c * NC + d] += v;
          }
      }
    }
  }
  for (int i = 0; i < SB; ++i) blk[i] = T(rs[i]);
  for (int i = 0; i < 7 * SB; ++i) out[i] = blk[i];
}

template <class T, int NC>
struct P1StencilKern {
  template <class F>
  TOPO_HD static bool node_eval(int a, int b, const P1Stencil<T, NC>& P, const F& fetch, T (&acc)[NC]) {
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
    if (!surely_free(P.dir, a, b) && is_clamped(P.dir, a, b)) return false;
    const int NX = P.nx + 1, NY = P.ny + 1;
    const size_t n = size_t(b) * NX + a;
    const bool interior = P.inner && a > 0 && b > 0 && a < NX - 1 && b < NY - 1;
    const T* sn = interior ? P.inner : P.s + n * StencilLayout<NC>::stride;
    T un[NC];
    fetch(n, a, b, un);
    for (int c = 0; c < NC; ++c)
      for (int d = 0; d < NC; ++d) acc[c] += sn[c * NC + d] * un[d];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int k = 1; k < 7; ++k) {
      const int al = a + st_da(k), bl = b + st_db(k);
      if (al < 0 || al >= NX || bl < 0 || bl >= NY) continue;
      T ul[NC];
      fetch(size_t(bl) * NX + al, al, bl, ul);
      for (int c = 0; c < NC; ++c)
        for (int d = 0; d < NC; ++d) acc[c] += sn[k * NC * NC + c * NC + d] * (ul[d] - un[d]);
    }
    return true;
  }
};

// node evaluation through either representation of a level
template <class T, int NC, class F>
TOPO_HD bool p1_node_eval(int a, int b, const P1Params<T, NC>& P, const F& f, T (&acc)[NC]) {
  return P1Kern<T, NC>::node_eval(a, b, P, f, acc);
}
template <class T, int NC, class F>
TOPO_HD bool p1_node_eval(int a, int b, const P1Stencil<T, NC>& P, const F& f, T (&acc)[NC]) {
  return P1StencilKern<T, NC>::node_eval(a, b, P, f, acc);
}

// y = A u at node (a,b) (clamped rows: identity)
template <class T, int NC, class PP>
TOPO_HD void p1_node_apply(int a, int b, const PP& P, const T* u, T* y) {
  const size_t n = size_t(b) * (P.nx + 1) + a;
  T acc[NC];
  if (!p1_node_eval<T, NC>(a, b, P, FetchArray<T, NC>{u}, acc))
    for (int c = 0; c < NC; ++c) acc[c] = u[NC * n + c];
  for (int c = 0; c < NC; ++c) y[NC * n + c] = acc[c];
}

// ---------------------------------------------------------------------------
// fused degree-2 Chebyshev smoothing steps of one P1 level (node-centric)
// ---------------------------------------------------------------------------
// Buffers of one level for the fused V-cycle.
template <class T>
struct SmoothBufs {
  const T* b;      // right-hand side
  const T* dinv;   // inverse diagonal
  T* x;            // solution (pre-smoothed, then final)
  T* x2;           // intermediate solution of post-smoothing
  T* r;            // residual
  T* d;            // Chebyshev direction
  const T* cheb;   // c0 = 1/theta, c1, c2 of the second step (in the level's precision)
};

// PRE input: first step from x = 0, d0 = c0 Dinv b, computed per node
template <class T, int NC>
struct FetchPre {
  const T* b;
  const T* dinv;
  T c0;
  TOPO_HD void operator()(size_t m, int, int, T (&v)[NC]) const {
    for (int d = 0; d < NC; ++d) v[d] = c0 * dinv[NC * m + d] * b[NC * m + d];
  }
};

template <class T, int NC>
struct P1Smooth {
  // PRE: x = d0 + d1 with d0 = c0 Dinv b, r1 = b - A d0, d1 = c1 d0 + c2 Dinv r1
  template <class PP>
  TOPO_HD static void pre(int a, int b, const PP& P, const SmoothBufs<T>& B) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    const T c0 = B.cheb[0], c1 = B.cheb[1], c2 = B.cheb[2];
    const FetchPre<T, NC> f{B.b, B.dinv, c0};
    T t[NC], u[NC];
    f(n, a, b, u);
    if (!p1_node_eval<T, NC>(a, b, P, f, t))
      for (int c = 0; c < NC; ++c) t[c] = u[c];
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      const T r1 = B.b[i] - t[c];
      B.x[i] = u[c] + c1 * u[c] + c2 * B.dinv[i] * r1;
    }
  }
  // RES: r = b - A x
  template <class PP>
  TOPO_HD static void res(int a, int b, const PP& P, const SmoothBufs<T>& B) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    T t[NC];
    if (!p1_node_eval<T, NC>(a, b, P, FetchArray<T, NC>{B.x}, t))
      for (int c = 0; c < NC; ++c) t[c] = B.x[NC * n + c];
    for (int c = 0; c < NC; ++c) B.r[NC * n + c] = B.b[NC * n + c] - t[c];
  }
  // FIRST (after the coarse correction was added to x):
  // r0 = b - A x ; d0 = c0 Dinv r0 ; x2 = x + d0 (writes r, d, x2)
  template <class PP>
  TOPO_HD static void first(int a, int b, const PP& P, const SmoothBufs<T>& B) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    const T c0 = B.cheb[0];
    T t[NC];
    if (!p1_node_eval<T, NC>(a, b, P, FetchArray<T, NC>{B.x}, t))
      for (int c = 0; c < NC; ++c) t[c] = B.x[NC * n + c];
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      const T r0 = B.b[i] - t[c];
      const T d0 = c0 * B.dinv[i] * r0;
      B.r[i] = r0;
      B.d[i] = d0;
      B.x2[i] = B.x[i] + d0;
    }
  }
  // POST2: r1 = r0 - A d0 ; d1 = c1 d0 + c2 Dinv r1 ; x = x2 + d1
  template <class PP>
  TOPO_HD static void post2(int a, int b, const PP& P, const SmoothBufs<T>& B) {
    const int NX = P.nx + 1;
    const size_t n = size_t(b) * NX + a;
    const T c1 = B.cheb[1], c2 = B.cheb[2];
    const FetchArray<T, NC> f{B.d};
    T t[NC];
    if (!p1_node_eval<T, NC>(a, b, P, f, t))
      for (int c = 0; c < NC; ++c) t[c] = B.d[NC * n + c];
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      const T r1 = B.r[i] - t[c];
      B.x[i] = B.x2[i] + c1 * B.d[i] + c2 * B.dinv[i] * r1;
    }
  }
};

// ---------------------------------------------------------------------------
// Chebyshev iteration as the coarse solver of a truncated hierarchy
// ---------------------------------------------------------------------------
// Where a level's operator is well conditioned in the Jacobi metric (the
// filter's eps^2 K + M once the mesh width passes eps: mass-dominated), the
// V-cycle stops there and solves it with a fixed-degree Chebyshev iteration
// from x = 0 (Saad, Iterative Methods for Sparse Linear Systems, Alg. 12.1):
//   d_0 = c0 Dinv b ;  x_(k+1) = x_k + d_k ;  r_(k+1) = r_k - A d_k ;
//   d_(k+1) = c1_k d_k + c2_k Dinv r_(k+1)
// The result is p(Dinv A) Dinv b for a fixed polynomial p: a symmetric positive
// definite preconditioner when [lo, hi] holds the spectrum of Dinv A.
constexpr int kCoarseChebMax = 16;

template <class T>
struct CoarseCheb {
  int deg;                  // polynomial degree (deg - 1 operator applications)
  T c0;                     // 1 / theta
  T c1[kCoarseChebMax], c2[kCoarseChebMax];
};

// host: the coefficients for the interval [lo, hi]
inline void coarse_cheb_coefficients(double lo, double hi, int deg, double& c0, double* c1, double* c2) {
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  c0 = 1.0 / theta;
  double rho = 1.0 / sigma;
  for (int k = 1; k < deg; ++k) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    c1[k - 1] = rn * rho;
    c2[k - 1] = 2.0 * rn / delta;
    rho = rn;
  }
}

template <class T, int NC>
struct CoarseChebNode {
  // r = b, x = 0, d = c0 Dinv b
  TOPO_HD static void init(size_t n, const CoarseCheb<T>& C, const T* b, const T* dinv, T* r, T* x, T* d) {
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      r[i] = b[i];
      x[i] = T(0);
      d[i] = C.c0 * dinv[i] * b[i];
    }
  }
  // step k: x += d ; r -= A d ; dn = c1_k d + c2_k Dinv r   (reads d around the node)
  template <class PP>
  TOPO_HD static void step(int a, int b, int k, const PP& P, const CoarseCheb<T>& C, const T* dinv, const T* d, T* r,
                           T* x, T* dn) {
    const size_t n = size_t(b) * (P.nx + 1) + a;
    T t[NC];
    if (!p1_node_eval<T, NC>(a, b, P, FetchArray<T, NC>{d}, t))
      for (int c = 0; c < NC; ++c) t[c] = d[NC * n + c];
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      x[i] += d[i];
      const T rn = r[i] - t[c];
      r[i] = rn;
      dn[i] = C.c1[k] * d[i] + C.c2[k] * dinv[i] * rn;
    }
  }
  TOPO_HD static void finish(size_t n, const T* d, const T* x, T* out) {
    for (int c = 0; c < NC; ++c) out[NC * n + c] = x[NC * n + c] + d[NC * n + c];
  }
};

}  // namespace topo
