// Matrix-free vector-P2 SIMP elasticity operator on the structured lattice.
//
// Restates the bilinear form of FEM_src/elasisity_problem.py:104-132,
//   a(u,v) = (r(xi) [lambda div(u) I + 2 mu eps(u)], eps(v)) dx,
// integrated with the 7-point degree-5 rule.  Per triangle the displacement
// gradient is linear, so with vertex values G_k of grad(u) and the
// r-weighted mass matrix M_kl = sum_q w_q r(xi_q) lam_qk lam_ql the quadrature
// sum becomes   y_(m,c) = sum_k (S_k gradN_m(v_k))_c,   S_k = sum_l M_kl sigma(G_l),
// which is algebraically identical to the quadrature of the assembled form.
//
// The kernels are split into load / compute / gather phases (separated by
// __syncthreads on the GPU) so the test emulator can run the same phases on
// the CPU.
#pragma once

#include "topo_common.cuh"
#include "topo_dd.cuh"
#include "topo_p1.cuh"

namespace topo {

// The two displacement components of a node (and the smoothing vectors' pair
// at a node) are adjacent: one 8-byte (FP32) or 16-byte (FP64) access.  With the
// pair-of-FP32 type (dd) the vectors are FP64 in memory: a load keeps the double's
// bits (dd_pack_double; the element phase takes differences in FP64 and splits
// them), a store rounds hi + lo to a double.
template <class T>
TOPO_HD void ld2(const T* p, T (&v)[2]) {
  if constexpr (IsDD<T>::value) {
    const double* q = reinterpret_cast<const double*>(p);
#if defined(__CUDA_ARCH__)
    const double2 t = *reinterpret_cast<const double2*>(q);
    v[0] = dd_pack_double(t.x);
    v[1] = dd_pack_double(t.y);
#else
    v[0] = dd_pack_double(q[0]);
    v[1] = dd_pack_double(q[1]);
#endif
  } else {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 4) {
      const float2 t = *reinterpret_cast<const float2*>(p);
      v[0] = t.x;
      v[1] = t.y;
    } else {
      const double2 t = *reinterpret_cast<const double2*>(p);
      v[0] = t.x;
      v[1] = t.y;
    }
#else
    v[0] = p[0];
    v[1] = p[1];
#endif
  }
}

template <class T>
TOPO_HD void st2(T* p, T a, T b) {
  if constexpr (IsDD<T>::value) {
    double* q = reinterpret_cast<double*>(p);
#if defined(__CUDA_ARCH__)
    *reinterpret_cast<double2*>(q) = make_double2(dd_to_double(a), dd_to_double(b));
#else
    q[0] = dd_to_double(a);
    q[1] = dd_to_double(b);
#endif
  } else {
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 4) *reinterpret_cast<float2*>(p) = make_float2(a, b);
    else *reinterpret_cast<double2*>(p) = make_double2(a, b);
#else
    p[0] = a;
    p[1] = b;
#endif
  }
}

template <class T>
struct P2Params {
  int nx, ny;     // cells
  T ihx, ihy;     // 1/hx, 1/hy
  T lamT, mu2T;   // lambda*|T|, 2*mu*|T|
  Penal<T> pen;
  Dir dir;        // on the (2nx+1)x(2ny+1) node lattice
  // optional precomputed r-weighted mass matrices, 12 consecutive values per
  // cell (cell = j*nx + i): [o][k], k over [00,11,22,01,02,12] (null: evaluate
  // r(xi) on the fly).  48 B (FP32) / 96 B (FP64) per cell: 16-byte vector loads.
  const T* rmass;
};

// r-weighted P1 mass matrix of one triangle, packed [00,11,22,01,02,12].
template <class T>
TOPO_HD void tri_rmass(const T (&xi)[3], const Penal<T>& pen, T (&M)[6]) {
  for (int k = 0; k < 6; ++k) M[k] = T(0);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int q = 0; q < Rule7::n; ++q) {
    const T l0 = T(Rule7::lam(q, 0)), l1 = T(Rule7::lam(q, 1)), l2 = T(Rule7::lam(q, 2));
    const T x = l0 * xi[0] + l1 * xi[1] + l2 * xi[2];
    const T wr = T(Rule7::w(q)) * pen.r(x);
    M[0] += wr * (l0 * l0);
    M[1] += wr * (l1 * l1);
    M[2] += wr * (l2 * l2);
    M[3] += wr * (l0 * l1);
    M[4] += wr * (l0 * l2);
    M[5] += wr * (l1 * l2);
  }
}

// tri_rmass for two penalisations of the same design in one pass (the FP32
// operator's and its preconditioner's, which differ only in the clamp): each
// matrix with exactly the arithmetic of tri_rmass.
template <class T>
TOPO_HD void tri_rmass_pair(const T (&xi)[3], const Penal<T>& pa, const Penal<T>& pb, T (&Ma)[6], T (&Mb)[6]) {
  for (int k = 0; k < 6; ++k) Ma[k] = Mb[k] = T(0);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int q = 0; q < Rule7::n; ++q) {
    const T l0 = T(Rule7::lam(q, 0)), l1 = T(Rule7::lam(q, 1)), l2 = T(Rule7::lam(q, 2));
    const T x = l0 * xi[0] + l1 * xi[1] + l2 * xi[2];
    const T wa = T(Rule7::w(q)) * pa.r(x), wb = T(Rule7::w(q)) * pb.r(x);
    Ma[0] += wa * (l0 * l0);
    Ma[1] += wa * (l1 * l1);
    Ma[2] += wa * (l2 * l2);
    Ma[3] += wa * (l0 * l1);
    Ma[4] += wa * (l0 * l2);
    Ma[5] += wa * (l1 * l2);
    Mb[0] += wb * (l0 * l0);
    Mb[1] += wb * (l1 * l1);
    Mb[2] += wb * (l2 * l2);
    Mb[3] += wb * (l0 * l1);
    Mb[4] += wb * (l0 * l2);
    Mb[5] += wb * (l1 * l2);
  }
}

// S * g_I for symmetric S = (xx, yy, xy); g in units of (ihx, ihy).
template <int O, int I, class T>
TOPO_HD void sg(const T (&s)[3], T ihx, T ihy, T& ox, T& oy) {
  if constexpr (O == 0) {
    if constexpr (I == 0) { ox = -s[0] * ihx; oy = -s[2] * ihx; }
    else if constexpr (I == 1) { ox = s[0] * ihx - s[2] * ihy; oy = s[2] * ihx - s[1] * ihy; }
    else { ox = s[2] * ihy; oy = s[1] * ihy; }
  } else {
    if constexpr (I == 0) { ox = -s[2] * ihy; oy = -s[1] * ihy; }
    else if constexpr (I == 1) { ox = s[2] * ihy - s[0] * ihx; oy = s[1] * ihy - s[2] * ihx; }
    else { ox = s[0] * ihx; oy = s[2] * ihx; }
  }
}

// Vertex gradients G[k] = grad(u)(v_k) = [[ux_x, ux_y],[uy_x, uy_y]] of the P2
// field with local node values u (order A,B,C,mid(BC),mid(AC),mid(AB)).
template <int O, class T, class TU>
TOPO_HD void p2_vertex_grads(const TU (&u)[6][2], T ihx, T ihy, T (&G)[3][2][2]) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int c = 0; c < 2; ++c) {
    // W[k][i]: coefficient of g_i in grad(u)(v_k), component c
    const TU w00 = mul_small<3>(u[0][c]), w01 = mul_small<4>(u[5][c]) - u[1][c], w02 = mul_small<4>(u[4][c]) - u[2][c];
    const TU w10 = mul_small<4>(u[5][c]) - u[0][c], w11 = mul_small<3>(u[1][c]), w12 = mul_small<4>(u[3][c]) - u[2][c];
    const TU w20 = mul_small<4>(u[4][c]) - u[0][c], w21 = mul_small<4>(u[3][c]) - u[1][c], w22 = mul_small<3>(u[2][c]);
    if constexpr (O == 0) {
      G[0][c][0] = T(w01 - w00) * ihx; G[0][c][1] = T(w02 - w01) * ihy;
      G[1][c][0] = T(w11 - w10) * ihx; G[1][c][1] = T(w12 - w11) * ihy;
      G[2][c][0] = T(w21 - w20) * ihx; G[2][c][1] = T(w22 - w21) * ihy;
    } else {
      G[0][c][0] = T(w02 - w01) * ihx; G[0][c][1] = T(w01 - w00) * ihy;
      G[1][c][0] = T(w12 - w11) * ihx; G[1][c][1] = T(w11 - w10) * ihy;
      G[2][c][0] = T(w22 - w21) * ihx; G[2][c][1] = T(w21 - w20) * ihy;
    }
  }
}

// y = K_T u for one triangle of orientation O with r-weighted mass matrix M.
template <int O, class T>
TOPO_HD void tri_apply_m(const T (&u)[6][2], const T (&M)[6], const P2Params<T>& P, T (&y)[6][2]) {
  T G[3][2][2];
  p2_vertex_grads<O>(u, P.ihx, P.ihy, G);
  const T muT = half_of(P.mu2T);
  T sig[3][3];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int k = 0; k < 3; ++k) {
    const T exx = G[k][0][0], eyy = G[k][1][1];
    const T tr = exx + eyy;
    sig[k][0] = P.lamT * tr + P.mu2T * exx;
    sig[k][1] = P.lamT * tr + P.mu2T * eyy;
    sig[k][2] = muT * (G[k][0][1] + G[k][1][0]);
  }
  T S[3][3];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int c = 0; c < 3; ++c) {
    S[0][c] = dot3(M[0], sig[0][c], M[3], sig[1][c], M[4], sig[2][c]);
    S[1][c] = dot3(M[3], sig[0][c], M[1], sig[1][c], M[5], sig[2][c]);
    S[2][c] = dot3(M[4], sig[0][c], M[5], sig[1][c], M[2], sig[2][c]);
  }
  // vertex nodes: (4 S_i - sum S) g_i
  T Q[3][3];
  for (int c = 0; c < 3; ++c) {
    const T tot = S[0][c] + S[1][c] + S[2][c];
    Q[0][c] = mul_small<4>(S[0][c]) - tot;
    Q[1][c] = mul_small<4>(S[1][c]) - tot;
    Q[2][c] = mul_small<4>(S[2][c]) - tot;
  }
  sg<O, 0>(Q[0], P.ihx, P.ihy, y[0][0], y[0][1]);
  sg<O, 1>(Q[1], P.ihx, P.ihy, y[1][0], y[1][1]);
  sg<O, 2>(Q[2], P.ihx, P.ihy, y[2][0], y[2][1]);
  // edge nodes: 4 (S_i g_j + S_j g_i)
  T ax, ay, bx, by;
  sg<O, 2>(S[1], P.ihx, P.ihy, ax, ay);
  sg<O, 1>(S[2], P.ihx, P.ihy, bx, by);
  y[3][0] = mul_small<4>(ax + bx); y[3][1] = mul_small<4>(ay + by);
  sg<O, 2>(S[0], P.ihx, P.ihy, ax, ay);
  sg<O, 0>(S[2], P.ihx, P.ihy, bx, by);
  y[4][0] = mul_small<4>(ax + bx); y[4][1] = mul_small<4>(ay + by);
  sg<O, 1>(S[0], P.ihx, P.ihy, ax, ay);
  sg<O, 0>(S[1], P.ihx, P.ihy, bx, by);
  y[5][0] = mul_small<4>(ax + bx); y[5][1] = mul_small<4>(ay + by);
}

// y = K_T u for one triangle of orientation O.
template <int O, class T>
TOPO_HD void tri_apply(const T (&u)[6][2], const T (&xi)[3], const P2Params<T>& P, T (&y)[6][2]) {
  T M[6];
  tri_rmass(xi, P.pen, M);
  tri_apply_m<O>(u, M, P, y);
}

// Diagonal of K_T for one triangle.
template <class T>
TOPO_HD void tri_diag(int o, const T (&xi)[3], const P2Params<T>& P, T (&d)[6][2]) {
  T M[6];
  tri_rmass(xi, P.pen, M);
  const int gxs_[2][3] = {{-1, 1, 0}, {0, -1, 1}};
  const int gys_[2][3] = {{0, -1, 1}, {-1, 1, 0}};
  const T lmT = P.lamT + P.mu2T, muT = T(0.5) * P.mu2T;
  for (int m = 0; m < 6; ++m) {
    T vx[3], vy[3];
    for (int k = 0; k < 3; ++k) {
      int cx, cy;  // gradient of N_m at vertex k in units of (ihx, ihy)
      if (m < 3) {
        const int f = (k == m) ? 3 : -1;
        cx = f * gxs_[o][m];
        cy = f * gys_[o][m];
      } else {
        const int i = (m == 3) ? 1 : 0, j = (m == 5) ? 1 : 2;  // edge (i,j)
        cx = 0; cy = 0;
        if (k == i) { cx += 4 * gxs_[o][j]; cy += 4 * gys_[o][j]; }
        if (k == j) { cx += 4 * gxs_[o][i]; cy += 4 * gys_[o][i]; }
      }
      vx[k] = T(cx) * P.ihx;
      vy[k] = T(cy) * P.ihy;
    }
    const T qx = M[0] * vx[0] * vx[0] + M[1] * vx[1] * vx[1] + M[2] * vx[2] * vx[2] +
                 T(2) * (M[3] * vx[0] * vx[1] + M[4] * vx[0] * vx[2] + M[5] * vx[1] * vx[2]);
    const T qy = M[0] * vy[0] * vy[0] + M[1] * vy[1] * vy[1] + M[2] * vy[2] * vy[2] +
                 T(2) * (M[3] * vy[0] * vy[1] + M[4] * vy[0] * vy[2] + M[5] * vy[1] * vy[2]);
    d[m][0] = lmT * qx + muT * qy;
    d[m][1] = lmT * qy + muT * qx;
  }
}

// ---------------------------------------------------------------------------
// column-march kernel phases
// ---------------------------------------------------------------------------
// One warp covers 32 consecutive cell columns i = i0-1 .. i0+30 and marches
// upward through a segment of cell rows.  At step j, lane L works on cell
// (i0-1+L, j): it holds the operand at the cell's 3x3 nodes (2i+c, 2j+r),
// the density at its 2x2 vertices and the element results at the same nodes.
//  * column 2 of a lane is column 0 of the next lane: operand and density
//    come down from lane L+1 by a shuffle (the last lane loads its own);
//  * row 2 of a step is row 0 of the next step: kept in registers;
//  * element results of column 2 go up to lane L+1, which adds them to its
//    column 0; results of row 2 are carried to the next step.
// After a step a lane therefore holds the complete sums at its nodes of rows
// 0,1 and columns 0,1 and finishes them (apply, diagonal or a smoothing
// update).  Lane 0 only feeds lane 1 (its own nodes belong to the previous
// warp), and the first step of a segment recomputes the cell row below it
// (whose results only complete row 0).  No shared memory, no block barriers:
// the nodes move through registers once per launch.
constexpr int P2M_OWN = 31;                   // owned cell columns per warp
constexpr int P2M_WARPS = 4;                  // warps per block, one row segment each
constexpr int P2M_THREADS = 32 * P2M_WARPS;

// What one launch of the P2 kernel computes.
enum P2Mode { kP2Apply = 0, kP2Diag = 1, kP2Pre = 2, kP2Res = 3, kP2First = 4, kP2Post2 = 5 };

struct PcgDev;

// Reductions of the state CG fused into a P2 launch (P2Io::fuse):
enum P2Fuse {
  kFuseNone = 0,
  kFusePQ = 1,    // apply q = A p: p.q -> PcgDev::pq
  kFuseRZ = 2,    // last post-smoothing step of the V-cycle (z = B.x, r = B.b):
                  // r.r, r.z -> PcgDev::rr, rz_new, then the iteration's test
};

template <class T>
struct P2Io {
  int mode;
  const T* u;          // kP2Apply / kP2Res / kP2First input (x)
  T* y;                // kP2Apply / kP2Diag output
  SmoothBufs<T> B;     // smoothing modes (see P1Smooth for the formulas)
  const T* xc;         // kP2First: coarse correction on the P1 vertex lattice, added to the
                       // operand x at free nodes on the fly (the prolongation, not stored)
  int fuse;            // P2Fuse
  double* partials;    // per-block partial sums (2 per block)
  unsigned* counter;   // last-block counter
  PcgDev* pcg;         // CG scalars
  unsigned long long cond;  // graph conditional handle of the CG loop
  int use_cond;
  T cf[3];             // B.cheb[0..2], copied in by P2March::prepare (registers, not re-read)
};

// Which of a lane's cells and nodes exist and which nodes are clamped.  A lane
// keeps its columns for the whole march, so this is set once (P2March::begin);
// the node rows of every step lie inside the lattice (2j + r <= 2 ny), so only
// their clamps vary, and those are the same for the whole warp.
struct P2Mask {
  bool cell;      // cell column i inside the mesh
  bool col[3];    // node columns 2i, 2i+1, 2i+2 inside the lattice
  bool ccl[3];    // ... on a clamped left or right side
  bool vcol[2];   // vertex columns i, i+1 inside the lattice
  bool pts;       // clamped points exist: tested node by node
};

template <class T>
struct P2Lane {
  int i;          // cell column
  bool edge;      // last lane of the warp: loads its column 2 itself
  P2Mask K;       // the lane's cells and node columns
  T U[3][3][2];   // operand at nodes (2i+c, 2j+r) (raw at clamped nodes, zero outside the lattice)
  T X[2][2];      // density at vertices (i+c, j+r)
  T A[3][3][2];   // element results at the same nodes
  T M[12];        // r-weighted mass matrices of the cell (when precomputed), [o][k]
};

// The loads of the next step, issued before the current step's arithmetic so
// that their latency hides behind it.
template <class T>
struct P2Next {
  T U[2][3][2];   // operand rows 1, 2 of the next step
  T X[2];         // density row 1 of the next step
  T M[12];        // mass matrices of the next cell
};

template <class T>
struct P2March {
  // once per launch, before any phase: the smoothing coefficients by value
  TOPO_HD static void prepare(P2Io<T>& io) {
    const bool smooth = io.mode == kP2Pre || io.mode == kP2First || io.mode == kP2Post2;
    for (int k = 0; k < 3; ++k) io.cf[k] = (smooth && io.B.cheb) ? io.B.cheb[k] : T(0);
  }

  // operand of the apply at node n for the launch's mode
  TOPO_HD static void operand(const P2Io<T>& io, size_t n, T (&v)[2]) {
    switch (io.mode) {
      case kP2Pre: {
        const T c0 = io.cf[0];
        T dv[2], bv[2];
        ld2(io.B.dinv + 2 * n, dv);
        ld2(io.B.b + 2 * n, bv);
        v[0] = c0 * dv[0] * bv[0];
        v[1] = c0 * dv[1] * bv[1];
        break;
      }
      case kP2Post2:
        ld2(io.B.d + 2 * n, v);
        break;
      default:
        ld2(io.u + 2 * n, v);
    }
  }

  // P1 -> P2 prolongation of the coarse correction at node (a,b): the coarse
  // hat functions are 1 at vertex (a/2, b/2) and 1/2 at the edge midpoints
  TOPO_HD static void prolong(const P2Params<T>& P, const T* xc, int a, int b, T (&v)[2]) {
    const int NXc = P.nx + 1;
    const int pa = a & 1, pb = b & 1, I0 = a >> 1, J0 = b >> 1;
    const size_t m0 = size_t(J0) * NXc + I0;
    T x0[2];
    ld2(xc + 2 * m0, x0);
    if (pa | pb) {
      const size_t m1 = size_t(J0 + pb) * NXc + I0 + pa;
      T x1[2];
      ld2(xc + 2 * m1, x1);
      v[0] += T(0.5) * (x0[0] + x1[0]);
      v[1] += T(0.5) * (x0[1] + x1[1]);
    } else {
      v[0] += x0[0];
      v[1] += x0[1];
    }
  }

  // Whether a warp's whole march runs on the lean path: every cell it touches
  // (columns i0 .. i0+31, rows j0 .. je-1) lies inside the mesh, its nodes stay
  // below the top node row, and none of its nodes is clamped.  The lean phases
  // then make no per-node tests.  (Indices are 32-bit on both paths: a lattice
  // holds far fewer than 2^31 values.)
  TOPO_HD static bool lean_region(const P2Params<T>& P, int i0, int j0, int je) {
    const int a_lo = 2 * i0, a_hi = 2 * (i0 + 31) + 2, b_lo = 2 * j0, b_hi = 2 * je;
    const Dir& d = P.dir;
    return i0 >= 0 && i0 + 31 < P.nx && j0 >= 0 && je < P.ny && d.npts == 0 && !(d.x_lo && a_lo == 0) &&
           a_hi < d.x_hi_from && !(d.y_lo && b_lo == 0) && b_hi < d.y_hi_from;
  }

  // node row b on a clamped bottom or top side (the same for every lane)
  TOPO_HD static bool row_clamped(const P2Params<T>& P, int b) {
    return (P.dir.y_lo && b == 0) || b >= P.dir.y_hi_from;
  }

  // node (a, b) = (2i + c, b) of the lane with mask K is clamped (an identity row)
  TOPO_HD static bool clamped(const P2Params<T>& P, const P2Mask& K, int c, int a, int b) {
    return K.ccl[c] || row_clamped(P, b) || (K.pts && is_clamped(P.dir, a, b));
  }

  // Operand at node (a, b) = (2i + c, b) of the lane, zero outside the lattice.
  // At a clamped node it is the raw operand (without the First mode's coarse
  // correction): the element phase zeroes it (tri), and the finish phase uses it
  // as the identity row's value without loading it again.  LEAN: the node is
  // known to be inside and free.
  template <bool LEAN = false>
  TOPO_HD static void fetch(const P2Params<T>& P, const P2Io<T>& io, const P2Mask& K, int c, int a, int b,
                            T (&v)[2]) {
    const int NX = 2 * P.nx + 1;
    if (!LEAN && !K.col[c]) {
      v[0] = v[1] = T(0);
      return;
    }
    operand(io, unsigned(b) * unsigned(NX) + unsigned(a), v);
    if (io.mode == kP2First && io.xc && (LEAN || !clamped(P, K, c, a, b))) prolong(P, io.xc, a, b, v);
  }

  // density at vertex (i + c, j) of the lane (rows j <= ny always)
  template <bool LEAN = false>
  TOPO_HD static T density(const P2Params<T>& P, const T* xi, const P2Mask& K, int c, int i, int j) {
    if constexpr (IsDD<T>::value) return T(0);  // the pair-of-FP32 operator reads precomputed mass matrices
    if (!LEAN && !K.vcol[c]) return T(0);
    return xi[unsigned(j) * unsigned(P.nx + 1) + unsigned(i + c)];
  }

  // loads of step j: operand rows R0..2 and density rows (R0 == 0 ? 0 : 1)..1,
  // columns 0 (and, on the edge lane, the last column)
  template <int R0, bool LEAN = false>
  TOPO_HD static void load(const P2Params<T>& P, const P2Io<T>& io, const T* xi, P2Lane<T>& L, int j) {
    if (io.mode != kP2Diag) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
      for (int r = R0; r <= 2; ++r) {
        const int b = 2 * j + r;
        fetch<LEAN>(P, io, L.K, 0, 2 * L.i, b, L.U[r][0]);
        fetch<LEAN>(P, io, L.K, 1, 2 * L.i + 1, b, L.U[r][1]);
        if (L.edge) fetch<LEAN>(P, io, L.K, 2, 2 * L.i + 2, b, L.U[r][2]);
      }
    }
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = (R0 == 0 ? 0 : 1); r <= 1; ++r) {
      L.X[r][0] = density<LEAN>(P, xi, L.K, 0, L.i, j + r);
      if (L.edge) L.X[r][1] = density<LEAN>(P, xi, L.K, 1, L.i, j + r);
    }
  }

  // Z: the step's clamped nodes (their operand enters the element as zero)
  template <int O, bool LEAN = false>
  TOPO_HD static void tri(const P2Params<T>& P, P2Lane<T>& L, const bool (&Z)[3][3], int mode) {
    const T xe[3] = {L.X[P1Off<O, 0>::b][P1Off<O, 0>::a], L.X[P1Off<O, 1>::b][P1Off<O, 1>::a],
                     L.X[P1Off<O, 2>::b][P1Off<O, 2>::a]};
    T y[6][2];
    if constexpr (IsDD<T>::value) mode = kP2Apply;  // Apply only (precomputed mass matrices)
    if (mode == kP2Diag) {
      if constexpr (!IsDD<T>::value) tri_diag(O, xe, P, y);
    } else {
      T ue[6][2];
#define TOPO_LD(K)                                                                                      \
  ue[K][0] = (!LEAN && Z[P2Off<O, K>::b][P2Off<O, K>::a]) ? T(0) : L.U[P2Off<O, K>::b][P2Off<O, K>::a][0]; \
  ue[K][1] = (!LEAN && Z[P2Off<O, K>::b][P2Off<O, K>::a]) ? T(0) : L.U[P2Off<O, K>::b][P2Off<O, K>::a][1];
      TOPO_LD(0) TOPO_LD(1) TOPO_LD(2) TOPO_LD(3) TOPO_LD(4) TOPO_LD(5)
#undef TOPO_LD
      // difference form: the element operator annihilates translations, so
      // K_T u = K_T (u - u_A); the differences of a smooth field are exact
      // (Sterbenz) and small, which keeps the products' rounding relative to
      // the local variation of u instead of to |u|.  At a solved displacement
      // of a high-contrast design this takes the FP32 operator's disagreement
      // with the FP64 one from ~1e-2 to ~1e-4 of |K u|.
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
      for (int c = 0; c < 2; ++c) {
        if constexpr (IsDD<T>::value) {  // operand packed as doubles: FP64 differences, then split
          const double ua = dd_unpack_double(ue[0][c]);
          for (int k = 1; k < 6; ++k) ue[k][c] = dd_from_double(dd_unpack_double(ue[k][c]) - ua);
        } else {
          const T ua = ue[0][c];
          for (int k = 1; k < 6; ++k) ue[k][c] -= ua;
        }
        ue[0][c] = T(0);
      }
      if (IsDD<T>::value || P.rmass) {
        T M[6];
        for (int k = 0; k < 6; ++k) M[k] = L.M[O * 6 + k];
        tri_apply_m<O>(ue, M, P, y);
      } else {
        if constexpr (!IsDD<T>::value) tri_apply<O>(ue, xe, P, y);
      }
    }
#define TOPO_ST(K)                                             \
  L.A[P2Off<O, K>::b][P2Off<O, K>::a][0] += y[K][0];           \
  L.A[P2Off<O, K>::b][P2Off<O, K>::a][1] += y[K][1];
    TOPO_ST(0) TOPO_ST(1) TOPO_ST(2) TOPO_ST(3) TOPO_ST(4) TOPO_ST(5)
#undef TOPO_ST
  }

  // mass matrices of the lane's cell (i, j) (zero outside the mesh; 0 <= j < ny always)
  template <bool LEAN = false>
  TOPO_HD static void load_mass(const P2Params<T>& P, const P2Mask& K, int i, int j, T (&M)[12]) {
    if (!P.rmass) return;
    if (!LEAN && !K.cell) {
      for (int k = 0; k < 12; ++k) M[k] = T(0);
      return;
    }
    const T* src = P.rmass + (unsigned(j) * unsigned(P.nx) + unsigned(i)) * 12u;
#if defined(__CUDA_ARCH__)
    if constexpr (IsDD<T>::value) {  // (hi, lo) pairs: two per 16-byte load
      const float4* q = reinterpret_cast<const float4*>(src);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const float4 t = q[k];
        M[2 * k] = dd(t.x, t.y);
        M[2 * k + 1] = dd(t.z, t.w);
      }
    } else if constexpr (sizeof(T) == 4) {
      const float4* q = reinterpret_cast<const float4*>(src);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float4 t = q[k];
        M[4 * k] = t.x;
        M[4 * k + 1] = t.y;
        M[4 * k + 2] = t.z;
        M[4 * k + 3] = t.w;
      }
    } else {
      const double2* q = reinterpret_cast<const double2*>(src);
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const double2 t = q[k];
        M[2 * k] = t.x;
        M[2 * k + 1] = t.y;
      }
    }
#else
    for (int k = 0; k < 12; ++k) M[k] = src[k];
#endif
  }

  // the loads of step j (operand rows 1, 2, density row 1, mass matrices)
  template <bool LEAN = false>
  TOPO_HD static void prefetch(const P2Params<T>& P, const P2Io<T>& io, const T* xi, const P2Lane<T>& L, int j,
                               P2Next<T>& N) {
    if (io.mode != kP2Diag) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
      for (int r = 1; r <= 2; ++r) {
        const int b = 2 * j + r;
        fetch<LEAN>(P, io, L.K, 0, 2 * L.i, b, N.U[r - 1][0]);
        fetch<LEAN>(P, io, L.K, 1, 2 * L.i + 1, b, N.U[r - 1][1]);
        if (L.edge) fetch<LEAN>(P, io, L.K, 2, 2 * L.i + 2, b, N.U[r - 1][2]);
      }
    }
    N.X[0] = density<LEAN>(P, xi, L.K, 0, L.i, j + 1);
    if (L.edge) N.X[1] = density<LEAN>(P, xi, L.K, 1, L.i, j + 1);
    if constexpr (!IsDD<T>::value) load_mass<LEAN>(P, L.K, L.i, j, N.M);  // (dd: loaded at compute time)
  }

  // after advance(): the prefetched loads become rows 1, 2 of the step
  TOPO_HD static void take(P2Lane<T>& L, const P2Next<T>& N) {
    for (int r = 1; r <= 2; ++r)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 2; ++d) L.U[r][c][d] = N.U[r - 1][c][d];
    L.X[1][0] = N.X[0];
    L.X[1][1] = N.X[1];
    if constexpr (!IsDD<T>::value)
      for (int k = 0; k < 12; ++k) L.M[k] = N.M[k];
  }

  // element results of cell (L.i, j), both triangles (0 <= j < ny always)
  template <bool LEAN = false>
  TOPO_HD static void compute(const P2Params<T>& P, P2Lane<T>& L, int j, int mode) {
    if (!LEAN && !L.K.cell) return;
    bool Z[3][3] = {};
    if (!LEAN)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Z[r][c] = clamped(P, L.K, c, 2 * L.i + c, 2 * j + r);
    tri<0, LEAN>(P, L, Z, mode);
    tri<1, LEAN>(P, L, Z, mode);
  }

  // finish node (a,b) with the complete sum r (clamped rows act as identity rows)
  // The finish phase's per-node vectors of step j (rows 0, 1 of the lane's
  // nodes), loaded before the step's arithmetic so that it hides their latency:
  //   Pre, First: b, Dinv   Res: b   Post2: w, Dinv (+ b for the fused r.r, r.z)
  struct Fin {
    T v[4][3][2];
  };
  template <bool LEAN = false>
  TOPO_HD static void fin_load(const P2Params<T>& P, const P2Io<T>& io, const P2Lane<T>& L, int j, Fin& F) {
    const int NX = 2 * P.nx + 1;
    const SmoothBufs<T>& B = io.B;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int q = 0; q < 4; ++q) {
      const int a = 2 * L.i + (q & 1), b = 2 * j + (q >> 1);  // b < NY always
      if (!LEAN && !L.K.col[q & 1]) continue;
      const size_t i = size_t(2u * (unsigned(b) * unsigned(NX) + unsigned(a)));
      switch (io.mode) {
        case kP2Pre:
        case kP2First:
          ld2(B.b + i, F.v[q][0]);
          ld2(B.dinv + i, F.v[q][1]);
          break;
        case kP2Res: ld2(B.b + i, F.v[q][0]); break;
        case kP2Post2:
          ld2(B.x2 + i, F.v[q][0]);
          ld2(B.dinv + i, F.v[q][1]);
          if (io.fuse == kFuseRZ) ld2(B.b + i, F.v[q][2]);
          break;
        default: break;
      }
    }
  }
  // the same vectors for one node (row 2 of the last cell row)
  TOPO_HD static void fin_load_node(const P2Io<T>& io, size_t i, T (&v)[3][2]) {
    const SmoothBufs<T>& B = io.B;
    switch (io.mode) {
      case kP2Pre:
      case kP2First:
        ld2(B.b + i, v[0]);
        ld2(B.dinv + i, v[1]);
        break;
      case kP2Res: ld2(B.b + i, v[0]); break;
      case kP2Post2:
        ld2(B.x2 + i, v[0]);
        ld2(B.dinv + i, v[1]);
        if (io.fuse == kFuseRZ) ld2(B.b + i, v[2]);
        break;
      default: break;
    }
  }

  // v: the node's finish vectors (Fin); cl: the node is clamped (an identity row);
  // u: the node's operand as fetched (raw at a clamped node)
  TOPO_HD static void finish_node(const P2Params<T>& P, const P2Io<T>& io, int a, int b, bool cl, const T (&sum)[2],
                                  const T (&u)[2], const T (&v)[3][2], T (&acc)[2]) {
    const int NX = 2 * P.nx + 1;
    const size_t n = size_t(unsigned(b) * unsigned(NX) + unsigned(a)), i = 2 * n;
    if (io.mode == kP2Diag) {
      st2(io.y + i, cl ? T(1) : sum[0], cl ? T(1) : sum[1]);
      return;
    }
    const T un[2] = {u[0], u[1]};
    T r[2] = {sum[0], sum[1]};
    if (cl) {
      if constexpr (!IsDD<T>::value) {  // (dd: the operand is packed as doubles; Apply stores it)
        r[0] = un[0];
        r[1] = un[1];
      }
    }
    const SmoothBufs<T>& B = io.B;
    const T c0 = io.cf[0], c1 = io.cf[1], c2 = io.cf[2];
    switch (io.mode) {
      case kP2Apply:
        if constexpr (IsDD<T>::value) {
          if (cl) {  // identity row: the operand's double itself
            double* q = reinterpret_cast<double*>(io.y + i);
            q[0] = dd_unpack_double(un[0]);
            q[1] = dd_unpack_double(un[1]);
            break;
          }
        }
        st2(io.y + i, r[0], r[1]);
        if (io.fuse == kFusePQ) {
          acc[0] += un[0] * r[0];
          acc[0] += un[1] * r[1];
        }
        break;
      case kP2Pre: {
        const T(&bv)[2] = v[0];
        const T(&dv)[2] = v[1];
        const T r0 = bv[0] - r[0], r1 = bv[1] - r[1];
        st2(B.x + i, un[0] + c1 * un[0] + c2 * dv[0] * r0, un[1] + c1 * un[1] + c2 * dv[1] * r1);
        break;
      }
      case kP2Res: {
        const T(&bv)[2] = v[0];
        st2(B.r + i, bv[0] - r[0], bv[1] - r[1]);
        break;
      }
      case kP2First: {
        // d0 = c0 Dinv r0 and w = x + d0 + c2 Dinv r0 (into x2): the second
        // step then needs only w, Dinv and A d0 (x = w + c1 d0 - c2 Dinv A d0)
        const T(&bv)[2] = v[0];
        const T(&dv)[2] = v[1];
        const T r0 = bv[0] - r[0], r1 = bv[1] - r[1];
        const T d0 = c0 * dv[0] * r0, d1 = c0 * dv[1] * r1;
        st2(B.d + i, d0, d1);
        st2(B.x2 + i, un[0] + d0 + c2 * dv[0] * r0, un[1] + d1 + c2 * dv[1] * r1);
        break;
      }
      default: {  // kP2Post2
        const T(&wv)[2] = v[0];
        const T(&dv)[2] = v[1];
        const T z0 = wv[0] + c1 * un[0] - c2 * dv[0] * r[0];
        const T z1 = wv[1] + c1 * un[1] - c2 * dv[1] * r[1];
        st2(B.x + i, z0, z1);
        if (io.fuse == kFuseRZ) {
          const T(&bv)[2] = v[2];
          acc[0] += bv[0] * bv[0];
          acc[1] += bv[0] * z0;
          acc[0] += bv[1] * bv[1];
          acc[1] += bv[1] * z1;
        }
      }
    }
  }

  // finish the lane's nodes of rows 0 .. nrows-1 (nrows = 3 on the last cell row)
  // acc: the lane's partial sums of the fused reductions, in the operator's
  // precision (a few dozen terms; blocks combine them in FP64)
  // (LEAN: nrows is 2 and every node is inside and free)
  template <bool LEAN = false>
  TOPO_HD static void finish(const P2Params<T>& P, const P2Io<T>& io, const P2Lane<T>& L, int j, int nrows,
                             const Fin& F, T (&acc)[2]) {
    const int NX = 2 * P.nx + 1;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < (LEAN ? 2 : 3); ++r) {
      if (!LEAN && r >= nrows) continue;  // 2j + r < NY for r < nrows
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
      for (int c = 0; c < 2; ++c) {
        const int a = 2 * L.i + c, b = 2 * j + r;
        if (!LEAN && !L.K.col[c]) continue;
        const bool cl = !LEAN && clamped(P, L.K, c, a, b);
        if (r < 2) {
          finish_node(P, io, a, b, cl, L.A[r][c], L.U[r][c], F.v[2 * r + c], acc);
        } else {  // row 2: only on the last cell row
          T v[3][2] = {};
          fin_load_node(io, 2 * (size_t(b) * NX + a), v);
          finish_node(P, io, a, b, cl, L.A[r][c], L.U[r][c], v, acc);
        }
      }
    }
  }

  // row 2 becomes row 0 of the next step
  TOPO_HD static void advance(P2Lane<T>& L) {
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 2; ++d) {
        L.U[0][c][d] = L.U[2][c][d];
        L.A[0][c][d] = c < 2 ? L.A[2][c][d] : T(0);  // column 2 went to the next lane
        L.A[1][c][d] = T(0);
        L.A[2][c][d] = T(0);
      }
    L.X[0][0] = L.X[1][0];
    L.X[0][1] = L.X[1][1];
  }

  TOPO_HD static void begin(const P2Params<T>& P, P2Lane<T>& L, int i, bool edge) {
    L.i = i;
    L.edge = edge;
    const int NX = 2 * P.nx + 1;
    const Dir& d = P.dir;
    L.K.cell = i >= 0 && i < P.nx;
    for (int c = 0; c < 3; ++c) {
      const int a = 2 * i + c;
      L.K.col[c] = a >= 0 && a < NX;
      L.K.ccl[c] = (d.x_lo && a == 0) || a >= d.x_hi_from;
    }
    for (int c = 0; c < 2; ++c) L.K.vcol[c] = i + c >= 0 && i + c <= P.nx;
    L.K.pts = d.npts > 0;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 2; ++d) L.U[r][c][d] = L.A[r][c][d] = T(0);
    L.X[0][0] = L.X[0][1] = L.X[1][0] = L.X[1][1] = T(0);
    for (int k = 0; k < 12; ++k) L.M[k] = T(0);
  }
};

// Cell rows per warp segment.  A block holds P2M_WARPS consecutive segments of
// one warp column, so the grid is (warp columns) x ceil(segments / P2M_WARPS)
// blocks.  The segment is the shortest whose grid still fits in ONE wave of
// `blocks_per_sm` resident blocks on each of `sms` SMs (a second, partial wave
// costs a whole segment's latency for a few blocks), and at least 4 rows so
// that the recomputed row below a segment stays a bounded share.  A lattice
// too wide for one wave gets whole-height segments.
inline int p2_march_segment(int nx, int ny, int sms, int blocks_per_sm) {
  if (ny <= 1) return 1;
  const long gx = (nx + 1 + P2M_OWN - 1) / P2M_OWN;
  const long cap = long(sms > 0 ? sms : 1) * (blocks_per_sm > 0 ? blocks_per_sm : 1);
  const long gy = cap / gx;  // block rows of one wave
  long seg = ny;
  if (gy >= 1) {
    const long nseg = gy * P2M_WARPS;  // ceil(ny / seg) <= nseg  =>  at most gy block rows
    seg = (ny + nseg - 1) / nseg;
  }
  if (seg < 4) seg = 4;
  if (seg > ny) seg = ny;
  return int(seg);
}

// ---------------------------------------------------------------------------
// per-triangle kernels (no tiling)
// ---------------------------------------------------------------------------

// r-weighted mass matrices of every triangle, layout [o][k][cell] (P2Params::rmass)
template <class T, class TC>
TOPO_HD void cell_rmass(int i, int j, int nx, int ny, const TC* xi, const Penal<TC>& pen, T* out) {
  const size_t c = size_t(j) * nx + i;
  const int VX = nx + 1;
  for (int o = 0; o < 2; ++o) {
    TC xe[3];
    for (int k = 0; k < 3; ++k) xe[k] = xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)];
    TC M[6];
    tri_rmass(xe, pen, M);
    for (int k = 0; k < 6; ++k) out[c * 12 + o * 6 + k] = T(M[k]);
  }
}

// cell_rmass for two penalisations in one pass (tri_rmass_pair)
template <class T>
TOPO_HD void cell_rmass_pair(int i, int j, int nx, const T* xi, const Penal<T>& pa, const Penal<T>& pb, T* outa,
                             T* outb) {
  const size_t c = size_t(j) * nx + i;
  const int VX = nx + 1;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int o = 0; o < 2; ++o) {
    T xe[3];
    for (int k = 0; k < 3; ++k) xe[k] = xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)];
    T Ma[6], Mb[6];
    tri_rmass_pair(xe, pa, pb, Ma, Mb);
    for (int k = 0; k < 6; ++k) {
      outa[c * 12 + o * 6 + k] = Ma[k];
      outb[c * 12 + o * 6 + k] = Mb[k];
    }
  }
}

// Both per-design FP64 coefficient sets of a cell in one pass over the
// quadrature points: the r-weighted mass matrices of the operator (r as given)
// and kappa_T of the P1 levels (r clamped at pmin, the preconditioner's
// coefficient).  Same arithmetic, term by term, as cell_rmass and tri_kappa.
// RM: the mass matrices' storage type (T, or dd pairs for the pair-of-FP32 operator)
template <class T, class RM = T>
TOPO_HD void cell_rmass_kappa(int i, int j, int nx, int ny, const T* xi, const Penal<T>& pen, RM* rm, T* kK) {
  const size_t c = size_t(j) * nx + i;
  const int VX = nx + 1;
  for (int o = 0; o < 2; ++o) {
    T xe[3];
    for (int k = 0; k < 3; ++k) xe[k] = xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)];
    T M[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
    T kap = T(0);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int q = 0; q < Rule7::n; ++q) {
      const T l0 = T(Rule7::lam(q, 0)), l1 = T(Rule7::lam(q, 1)), l2 = T(Rule7::lam(q, 2));
      const T x = l0 * xe[0] + l1 * xe[1] + l2 * xe[2];
      const T r = pen.r(x);
      const T wr = T(Rule7::w(q)) * r;
      M[0] += wr * (l0 * l0);
      M[1] += wr * (l1 * l1);
      M[2] += wr * (l2 * l2);
      M[3] += wr * (l0 * l1);
      M[4] += wr * (l0 * l2);
      M[5] += wr * (l1 * l2);
      kap += T(Rule7::w(q)) * (r >= pen.pmin ? r : pen.pmin);
    }
    for (int k = 0; k < 6; ++k) {
      if constexpr (IsDD<RM>::value) rm[c * 12 + o * 6 + k] = dd_from_double(M[k]);
      else rm[c * 12 + o * 6 + k] = M[k];
    }
    kK[c * 2 + o] = kap;
  }
}

// cell_rmass_kappa in pair-of-FP32 arithmetic (FP32 pipe; FP64 arithmetic is scarce
// on this GPU) for an integer penalisation exponent ip (1..16), r = pmin + xi^p
// (1 - pmin): the same 7-point quadrature, with the constants' products formed in
// FP64 at compile time.  Mass matrices as (hi, lo) pairs, kappa rounded to FP64.
TOPO_HD bool dd_ge(dd a, dd b) { return a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo); }

TOPO_HD void cell_rmass_kappa_dd(int i, int j, int nx, const double* xi, int ip, dd pmin, dd one_m_pmin, dd* rm,
                                 double* kK) {
  const size_t c = size_t(j) * nx + i;
  const int VX = nx + 1;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int o = 0; o < 2; ++o) {
    dd xe[3];
    for (int k = 0; k < 3; ++k) xe[k] = dd_from_double(xi[size_t(j + p1_off_b(o, k)) * VX + i + p1_off_a(o, k)]);
    dd M[6] = {dd(0), dd(0), dd(0), dd(0), dd(0), dd(0)};
    dd kap = dd(0);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int q = 0; q < Rule7::n; ++q) {
      const double l0 = Rule7::lam(q, 0), l1 = Rule7::lam(q, 1), l2 = Rule7::lam(q, 2), w = Rule7::w(q);
      const dd x = dd(l0) * xe[0] + dd(l1) * xe[1] + dd(l2) * xe[2];
      dd xp = x;
      for (int k = 1; k < ip; ++k) xp = xp * x;
      const dd r = pmin + xp * one_m_pmin;
      M[0] += r * dd(w * l0 * l0);
      M[1] += r * dd(w * l1 * l1);
      M[2] += r * dd(w * l2 * l2);
      M[3] += r * dd(w * l0 * l1);
      M[4] += r * dd(w * l0 * l2);
      M[5] += r * dd(w * l1 * l2);
      kap += dd(w) * (dd_ge(r, pmin) ? r : pmin);
    }
    for (int k = 0; k < 6; ++k) rm[c * 12 + o * 6 + k] = M[k];
    kK[c * 2 + o] = dd_to_double(kap);
  }
}

// kappa_T = (1/|T|) int_T r(xi) with the 7-point rule: the Galerkin P1
// coefficient of the P2 operator (P1 strains are constant per triangle).
template <class T>
TOPO_HD T tri_kappa(const T (&xi)[3], const Penal<T>& pen) {
  T s = T(0);
  for (int q = 0; q < Rule7::n; ++q) {
    const T x = T(Rule7::lam(q, 0)) * xi[0] + T(Rule7::lam(q, 1)) * xi[1] + T(Rule7::lam(q, 2)) * xi[2];
    s += T(Rule7::w(q)) * pen.r(x);
  }
  return s;
}

// Sensitivity moments c_k = int_T s phi_k, s = -r'(xi)(lambda div(u)^2 + 2 mu eps:eps)
// (FEM_src/elasisity_problem.py:146-149) with the 12-point rule.  The vertex
// gradients are formed in TG from the nodal values (this carries the
// cancellation), the quadrature runs in TQ.
template <int O, class TG, class TQ>
TOPO_HD void tri_sensitivity(const TG (&u)[6][2], const TQ (&xi)[3], TG ihx, TG ihy, TQ lam,
                             TQ mu, TQ area, const Penal<TQ>& pen, TQ (&c)[3]) {
  TG Gd[3][2][2];
  p2_vertex_grads<O>(u, ihx, ihy, Gd);
  TQ G[3][2][2];
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) G[k][a][b] = TQ(Gd[k][a][b]);
  c[0] = c[1] = c[2] = TQ(0);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int q = 0; q < Rule12::n; ++q) {
    const TQ l0 = TQ(Rule12::lam(q, 0)), l1 = TQ(Rule12::lam(q, 1)), l2 = TQ(Rule12::lam(q, 2));
    const TQ gxx = l0 * G[0][0][0] + l1 * G[1][0][0] + l2 * G[2][0][0];
    const TQ gxy = l0 * G[0][0][1] + l1 * G[1][0][1] + l2 * G[2][0][1];
    const TQ gyx = l0 * G[0][1][0] + l1 * G[1][1][0] + l2 * G[2][1][0];
    const TQ gyy = l0 * G[0][1][1] + l1 * G[1][1][1] + l2 * G[2][1][1];
    const TQ dv = gxx + gyy;
    const TQ exy = TQ(0.5) * (gxy + gyx);
    const TQ ee = gxx * gxx + gyy * gyy + TQ(2) * exy * exy;
    const TQ x = l0 * xi[0] + l1 * xi[1] + l2 * xi[2];
    const TQ sq = -pen.dr(x) * (lam * dv * dv + TQ(2) * mu * ee) * (TQ(Rule12::w(q)) * area);
    c[0] += sq * l0;
    c[1] += sq * l1;
    c[2] += sq * l2;
  }
}

}  // namespace topo
