// Column-march kernel phases for the large P1 levels (the same scheme as the
// P2 march, see P2March): a warp covers 32 consecutive cell columns
// i = i0-1 .. i0+30 and marches upward through a segment of cell rows.  At
// step j lane L works on cell (i0-1+L, j): it holds the operand at the cell's
// 2x2 nodes (i+c, j+r) and the element results there.  Column 1 of a lane is
// column 0 of the next lane (operand down by a shuffle, results up), row 1 of
// a step is row 0 of the next (registers).  After a step the lane holds the
// complete sum at its node (i, j) and finishes it (apply or a fused smoothing
// step, the formulas of P1Smooth).  Per cell: two element products
// y = kK Kref u (+ kM Mref u), against ~six incidences per node walked by the
// node-centric kernel.
#pragma once

#include "topo_p1.cuh"
#include "topo_p2.cuh"

namespace topo {

template <class T>
struct P1Io {
  int mode;         // P2Mode: kP2Apply, kP2Pre, kP2Res, kP2First, kP2Post2
  const T* u;       // Apply / Res / First operand (x)
  T* y;             // Apply output
  SmoothBufs<T> B;  // smoothing modes
  T cf[3];          // B.cheb[0..2], copied in by P1March::prepare (registers, not re-read)
};

template <class T, int NC>
struct P1Lane {
  int i;            // cell column
  bool edge;        // last lane of the warp: loads its column 1 itself
  T U[2][2][NC];    // operand at nodes (i+c, j+r), zero outside the lattice (raw at clamped nodes)
  T A[2][2][NC];    // element results at the same nodes
  T kk[2], km[2];   // the cell's triangle coefficients
};

// The loads of the next step, issued before the current step's arithmetic.
template <class T, int NC>
struct P1Next {
  T U[2][NC];       // operand row 1 of the next step (column 1 on the edge lane)
  T kk[2], km[2];
};

template <class T, int NC>
struct P1March {
  // once per launch, before any phase: the smoothing coefficients by value
  TOPO_HD static void prepare(P1Io<T>& io) {
    const bool smooth = io.mode == kP2Pre || io.mode == kP2First || io.mode == kP2Post2;
    for (int k = 0; k < 3; ++k) io.cf[k] = (smooth && io.B.cheb) ? io.B.cheb[k] : T(0);
  }

  TOPO_HD static void operand(const P1Io<T>& io, size_t n, T (&v)[NC]) {
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      switch (io.mode) {
        case kP2Pre: v[c] = io.cf[0] * io.B.dinv[i] * io.B.b[i]; break;
        case kP2Post2: v[c] = io.B.d[i]; break;
        default: v[c] = io.u[i];
      }
    }
  }

  // operand at node (a,b), zero outside the lattice.  At a clamped node it is the
  // raw operand: the element phase zeroes it (tri) and the finish phase uses it as the
  // identity row's value without loading it again.
  TOPO_HD static void fetch(const P1Params<T, NC>& P, const P1Io<T>& io, int a, int b, T (&v)[NC]) {
    for (int c = 0; c < NC; ++c) v[c] = T(0);
    if (a >= 0 && a <= P.nx && b >= 0 && b <= P.ny) operand(io, size_t(b) * (P.nx + 1) + a, v);
  }

  TOPO_HD static bool clamped(const P1Params<T, NC>& P, int a, int b) {
    return !surely_free(P.dir, a, b) && is_clamped(P.dir, a, b);
  }

  template <int R0>
  TOPO_HD static void load(const P1Params<T, NC>& P, const P1Io<T>& io, P1Lane<T, NC>& L, int j) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = R0; r <= 1; ++r) {
      fetch(P, io, L.i, j + r, L.U[r][0]);
      if (L.edge) fetch(P, io, L.i + 1, j + r, L.U[r][1]);
    }
  }

  // coefficients of cell (i, j) (zero outside the mesh)
  TOPO_HD static void load_coef(const P1Params<T, NC>& P, int i, int j, T (&kk)[2], T (&km)[2]) {
    const bool in = i >= 0 && i < P.nx && j >= 0 && j < P.ny;
    for (int o = 0; o < 2; ++o) {
      const size_t t = in ? (size_t(j) * P.nx + i) * 2 + o : 0;
      kk[o] = in ? (P.kK ? P.kK[t] : P.kK_c) : T(0);
      km[o] = (in && NC == 1) ? (P.kM ? P.kM[t] : P.kM_c) : T(0);
    }
  }

  TOPO_HD static void prefetch(const P1Params<T, NC>& P, const P1Io<T>& io, const P1Lane<T, NC>& L, int j,
                               P1Next<T, NC>& N) {
    fetch(P, io, L.i, j + 1, N.U[0]);
    if (L.edge) fetch(P, io, L.i + 1, j + 1, N.U[1]);
    load_coef(P, L.i, j, N.kk, N.km);
  }

  // after advance(): the prefetched loads become row 1 of the step
  TOPO_HD static void take(P1Lane<T, NC>& L, const P1Next<T, NC>& N) {
    for (int c = 0; c < 2; ++c)
      for (int d = 0; d < NC; ++d) L.U[1][c][d] = N.U[c][d];
    for (int o = 0; o < 2; ++o) {
      L.kk[o] = N.kk[o];
      L.km[o] = N.km[o];
    }
  }

  // Z: the cell's clamped nodes (their operand enters the element product as zero)
  template <int O>
  TOPO_HD static void tri(const P1Params<T, NC>& P, P1Lane<T, NC>& L, const bool (&Z)[2][2]) {
    const T kk = L.kk[O];
    const T km = L.km[O];
    T u[3][NC];
#define TOPO_LD(LV)                                                                          \
  for (int d = 0; d < NC; ++d)                                                               \
    u[LV][d] = Z[P1Off<O, LV>::b][P1Off<O, LV>::a] ? T(0) : L.U[P1Off<O, LV>::b][P1Off<O, LV>::a][d];
    TOPO_LD(0) TOPO_LD(1) TOPO_LD(2)
#undef TOPO_LD
#define TOPO_ST(LV)                                                                 \
  for (int c = 0; c < NC; ++c) {                                                    \
    T s = T(0);                                                                     \
    for (int l = 0; l < 3; ++l)                                                     \
      for (int d = 0; d < NC; ++d) s += P.K[O][LV * NC + c][l * NC + d] * u[l][d];  \
    T y = kk * s;                                                                   \
    if constexpr (NC == 1) {                                                        \
      T m = T(0);                                                                   \
      for (int l = 0; l < 3; ++l) m += P.Mm[O][LV][l] * u[l][0];                    \
      y += km * m;                                                                  \
    }                                                                               \
    L.A[P1Off<O, LV>::b][P1Off<O, LV>::a][c] += y;                                  \
  }
    TOPO_ST(0) TOPO_ST(1) TOPO_ST(2)
#undef TOPO_ST
  }

  TOPO_HD static void compute(const P1Params<T, NC>& P, P1Lane<T, NC>& L, int j) {
    if (L.i < 0 || L.i >= P.nx || j < 0 || j >= P.ny) return;
    bool Z[2][2];
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c) Z[r][c] = clamped(P, L.i + c, j + r);
    tri<0>(P, L, Z);
    tri<1>(P, L, Z);
  }

  // The finish phase's per-node vectors of the lane's row-0 node at step j,
  // loaded before the step's arithmetic so that it hides their latency:
  //   Pre, First: b, Dinv   Res: b   Post2: r, x2, Dinv
  struct Fin {
    T v[3][NC];
  };
  TOPO_HD static void fin_load(const P1Params<T, NC>& P, const P1Io<T>& io, int a, int b, Fin& F) {
    const size_t n = size_t(b) * (P.nx + 1) + a;
    const SmoothBufs<T>& B = io.B;
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      switch (io.mode) {
        case kP2Pre:
        case kP2First:
          F.v[0][c] = B.b[i];
          F.v[1][c] = B.dinv[i];
          break;
        case kP2Res: F.v[0][c] = B.b[i]; break;
        case kP2Post2:
          F.v[0][c] = B.r[i];
          F.v[1][c] = B.x2[i];
          F.v[2][c] = B.dinv[i];
          break;
        default: break;
      }
    }
  }

  // finish node (a,b) with the complete sum t (clamped rows act as identity rows);
  // F: the node's finish vectors (fin_load)
  TOPO_HD static void finish_node(const P1Params<T, NC>& P, const P1Io<T>& io, int a, int b, const T (&sum)[NC],
                                  const T (&u)[NC], const Fin& F) {
    const size_t n = size_t(b) * (P.nx + 1) + a;
    const bool cl = clamped(P, a, b);
    T un[NC], t[NC];
    for (int c = 0; c < NC; ++c) {
      un[c] = u[c];  // the operand as fetched: raw at a clamped node
      t[c] = cl ? un[c] : sum[c];
    }
    const SmoothBufs<T>& B = io.B;
    for (int c = 0; c < NC; ++c) {
      const size_t i = NC * n + c;
      switch (io.mode) {
        case kP2Apply: io.y[i] = t[c]; break;
        case kP2Pre: {
          const T r1 = F.v[0][c] - t[c];
          B.x[i] = un[c] + io.cf[1] * un[c] + io.cf[2] * F.v[1][c] * r1;
          break;
        }
        case kP2Res: B.r[i] = F.v[0][c] - t[c]; break;
        case kP2First: {
          const T r0 = F.v[0][c] - t[c];
          const T d0 = io.cf[0] * F.v[1][c] * r0;
          B.r[i] = r0;
          B.d[i] = d0;
          B.x2[i] = un[c] + d0;
          break;
        }
        default: {  // kP2Post2
          const T r1 = F.v[0][c] - t[c];
          B.x[i] = F.v[1][c] + io.cf[1] * un[c] + io.cf[2] * F.v[2][c] * r1;
        }
      }
    }
  }

  // finish the lane's node of row 0 (F: its preloaded vectors) and, on the
  // last cell row, of row 1
  TOPO_HD static void finish(const P1Params<T, NC>& P, const P1Io<T>& io, const P1Lane<T, NC>& L, int j, int nrows,
                             const Fin& F) {
    finish_node(P, io, L.i, j, L.A[0][0], L.U[0][0], F);
    if (nrows > 1 && j + 1 <= P.ny) {
      Fin F1;
      fin_load(P, io, L.i, j + 1, F1);
      finish_node(P, io, L.i, j + 1, L.A[1][0], L.U[1][0], F1);
    }
  }

  // row 1 becomes row 0 of the next step
  TOPO_HD static void advance(P1Lane<T, NC>& L) {
    for (int c = 0; c < 2; ++c)
      for (int d = 0; d < NC; ++d) {
        L.U[0][c][d] = L.U[1][c][d];
        L.A[0][c][d] = c == 0 ? L.A[1][c][d] : T(0);  // column 1 went to the next lane
        L.A[1][c][d] = T(0);
      }
  }

  TOPO_HD static void begin(P1Lane<T, NC>& L, int i, bool edge) {
    L.i = i;
    L.edge = edge;
    for (int r = 0; r < 2; ++r)
      for (int c = 0; c < 2; ++c)
        for (int d = 0; d < NC; ++d) L.U[r][c][d] = L.A[r][c][d] = T(0);
    L.kk[0] = L.kk[1] = L.km[0] = L.km[1] = T(0);
  }
};

}  // namespace topo
