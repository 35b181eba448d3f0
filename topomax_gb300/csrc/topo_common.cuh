// Shared definitions for the topomax GB300 kernels.
//
// Lattice conventions (fixed across every kernel and the C ABI):
//   * the domain [0,W]x[0,H] is split into nx x ny squares, square (i,j) into
//     the triangles T0 = (v0,v1,v3) and T1 = (v0,v2,v3) (v0 bottom-left,
//     v3 top-right) -- dolfin's RectangleMesh "right" diagonal
//     (FEM_src/solver.py:38-49 builds that mesh);
//   * CG1 vertex (i,j) has index j*(nx+1)+i;
//   * P2 nodes form the (2nx+1)x(2ny+1) half-spacing lattice, node (a,b) has
//     index b*(2nx+1)+a and its displacement components sit at 2*idx+c.
//
// Everything in this header compiles for host and device so the tile logic
// of the kernels can be exercised on the CPU by the test emulator.
#pragma once

#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define TOPO_HD __host__ __device__ __forceinline__
#else
#define TOPO_HD inline
#endif

// Programmatic dependent launch.  Kernels of the solve chain start with
// TOPO_PDL_ENTRY(): they wait for their predecessor's results (a no-op when
// launched without the programmatic attribute), then allow their own
// successor to be scheduled; the successor launches once every block of this
// grid has passed that point and overlaps its launch with this grid's drain.
#if defined(__CUDA_ARCH__)
#define TOPO_PDL_ENTRY()                                 \
  do {                                                   \
    asm volatile("griddepcontrol.wait;" ::: "memory");   \
    asm volatile("griddepcontrol.launch_dependents;" :::); \
  } while (0)
#else
#define TOPO_PDL_ENTRY() ((void)0)
#endif

namespace topo {

constexpr int kMaxDirPoints = 32;

// Dirichlet description of one lattice level.  Node (a,b) of an NX x NY
// lattice is clamped iff (x_lo && a==0) || a>=x_hi_from || (y_lo && b==0) ||
// b>=y_hi_from || (a,b) is one of the listed points.
struct Dir {
  int x_lo, y_lo;
  int x_hi_from, y_hi_from;
  int npts;
  int pts[2 * kMaxDirPoints];
};

TOPO_HD bool is_clamped(const Dir& d, int a, int b) {
  if ((d.x_lo && a == 0) || a >= d.x_hi_from || (d.y_lo && b == 0) || b >= d.y_hi_from)
    return true;
  for (int k = 0; k < d.npts; ++k)
    if (d.pts[2 * k] == a && d.pts[2 * k + 1] == b) return true;
  return false;
}

// Quick rejection: true when (a,b) is at least one node away from every
// clamped column/row and no clamped points exist (then is_clamped is false).
TOPO_HD bool surely_free(const Dir& d, int a, int b) {
  return d.npts == 0 && !(d.x_lo && a == 0) && !(d.y_lo && b == 0) && a < d.x_hi_from && b < d.y_hi_from;
}

TOPO_HD float topo_pow(float x, float p) { return powf(x, p); }
TOPO_HD double topo_pow(double x, double p) { return pow(x, p); }

// x^p, by products when p is a small positive integer (ip > 0): branch-free
// for ip <= 4 (the penalties of every design), a loop above.
template <class T>
TOPO_HD T pow_p(T x, int ip, T p) {
  if (ip > 0 && ip <= 4) {
    const T x2 = x * x;
    const T lo = ip == 1 ? x : x2;
    const T hi = ip == 4 ? x2 : x;
    return ip <= 2 ? lo : x2 * hi;
  }
  if (ip > 4) {
    T r = x;
    for (int k = 1; k < ip; ++k) r *= x;
    return r;
  }
  if (ip == 0) return T(1);
  return topo_pow(x, p);
}

// SIMP penalisation (src/penalizers.py:29-46): r(x) = m + x^p (1-m).
template <class T>
struct Penal {
  T pmin;  // m
  T p;     // exponent
  int ip;  // p as a positive integer, or -1
  T pm1;   // p-1
  int ipm1;
  int clamp;  // 1: r is clamped below at pmin (the SPD preconditioner's coefficient)

  TOPO_HD T r(T x) const {
    const T v = pmin + pow_p(x, ip, p) * (T(1) - pmin);
    return (clamp && !(v >= pmin)) ? pmin : v;
  }
  TOPO_HD T dr(T x) const { return p * pow_p(x, ipm1, pm1) * (T(1) - pmin); }
};

// clamp: the multigrid preconditioner uses max(r, m) so that it stays SPD even
// where the filtered density undershoots below zero (then r(xi) < 0 at some
// quadrature points and the true operator can be indefinite).
template <class T>
TOPO_HD Penal<T> make_penal(double p, double pmin, int clamp = 0) {
  Penal<T> q;
  q.clamp = clamp;
  q.pmin = T(pmin);
  q.p = T(p);
  q.pm1 = T(p - 1.0);
  double rp = std::floor(p + 0.5);
  q.ip = (rp == p && p >= 1.0 && p <= 16.0) ? int(rp) : -1;
  double rq = std::floor(p - 1.0 + 0.5);
  q.ipm1 = (rq == p - 1.0 && p - 1.0 >= 0.0 && p - 1.0 <= 16.0) ? int(rq) : -1;
  return q;
}

// Radon's 7-point rule, exact to degree 5: the rule the state form's total
// degree (r(xi) cubic in a CG1 xi, times two P2 strains) selects.  Points in
// barycentric coordinates (centroid, then two orbits (b,a,a)), weights sum 1.
struct Rule7 {
  static constexpr int n = 7;
  static constexpr double a1 = 0.1012865073234563388009874;
  static constexpr double b1 = 0.7974269853530873223980253;
  static constexpr double a2 = 0.4701420641051150897704412;
  static constexpr double b2 = 0.0597158717897698204591176;
  static constexpr double w0 = 0.225;
  static constexpr double w1 = 0.1259391805448271525956839;
  static constexpr double w2 = 0.1323941527885061807376494;
  TOPO_HD static double lam(int q, int k) {
    if (q == 0) return 1.0 / 3.0;
    if (q <= 3) return (q - 1 == k) ? b1 : a1;
    return (q - 4 == k) ? b2 : a2;
  }
  TOPO_HD static double w(int q) { return q == 0 ? w0 : (q <= 3 ? w1 : w2); }
};

// Strang & Fix (Dunavant) 12-point rule, exact to degree 6: the rule the
// gradient right-hand side's degree (r'(xi) * strain^2 * CG1 test) selects.
struct Rule12 {
  static constexpr int n = 12;
  TOPO_HD static double lam(int q, int k) {
    const double a1 = 0.063089014491502, b1 = 1.0 - 2.0 * 0.063089014491502;
    const double a2 = 0.249286745170910, b2 = 1.0 - 2.0 * 0.249286745170910;
    const double c0 = 0.053145049844816, c1 = 0.310352451033785;
    const double c2 = 1.0 - 0.053145049844816 - 0.310352451033785;
    if (q < 3) return (q == k) ? b1 : a1;
    if (q < 6) return (q - 3 == k) ? b2 : a2;
    // six permutations of (c0, c1, c2)
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    const double c[3] = {c0, c1, c2};
    return c[perm[q - 6][k]];
  }
  TOPO_HD static double w(int q) {
    return q < 3 ? 0.050844906370207 : (q < 6 ? 0.116786275726379 : 0.082851075618374);
  }
};

// Gradients of the barycentric coordinates, in units of 1/hx, 1/hy.
// orientation 0 (v0,v1,v3): g0=(-1,0) g1=(1,-1) g2=(0,1)
// orientation 1 (v0,v2,v3): g0=(0,-1) g1=(-1,1) g2=(1,0)
template <int O, int I>
TOPO_HD constexpr int gxs() {
  return O == 0 ? (I == 0 ? -1 : (I == 1 ? 1 : 0)) : (I == 0 ? 0 : (I == 1 ? -1 : 1));
}
template <int O, int I>
TOPO_HD constexpr int gys() {
  return O == 0 ? (I == 0 ? 0 : (I == 1 ? -1 : 1)) : (I == 0 ? -1 : (I == 1 ? 1 : 0));
}

// Compile-time local offsets (used in the kernels' inner loops so no table is
// indexed at run time).
template <int O, int K>
struct P2Off {
  static constexpr int a = O == 0 ? (K == 0 ? 0 : K == 1 ? 2 : K == 2 ? 2 : K == 3 ? 2 : 1)
                                  : (K == 0 ? 0 : K == 1 ? 0 : K == 2 ? 2 : K == 3 ? 1 : K == 4 ? 1 : 0);
  static constexpr int b = O == 0 ? (K == 0 ? 0 : K == 1 ? 0 : K == 2 ? 2 : K == 3 ? 1 : K == 4 ? 1 : 0)
                                  : (K == 0 ? 0 : K == 1 ? 2 : K == 2 ? 2 : K == 3 ? 2 : 1);
};
template <int O, int K>
struct P1Off {
  static constexpr int a = O == 0 ? (K == 0 ? 0 : 1) : (K == 2 ? 1 : 0);
  static constexpr int b = O == 0 ? (K == 2 ? 1 : 0) : (K == 0 ? 0 : 1);
};

// Local P2 node offsets (da,db) inside a square, order [A,B,C,mid(BC),mid(AC),mid(AB)].
// The tables are packed two bits per entry, entry (o, k) at bit 2 (6 o + k) (P1:
// 2 (3 o + k)), so that a run-time orientation costs a shift instead of a table
// built in local memory.
TOPO_HD constexpr int p2_off_a(int o, int k) { return int((0x1605a8u >> (2 * (6 * o + k))) & 3u); }
TOPO_HD constexpr int p2_off_b(int o, int k) { return int((0x5a8160u >> (2 * (6 * o + k))) & 3u); }
// Local P1 vertex offsets, order [A,B,C].
TOPO_HD constexpr int p1_off_a(int o, int k) { return int((0x414u >> (2 * (3 * o + k))) & 3u); }
TOPO_HD constexpr int p1_off_b(int o, int k) { return int((0x510u >> (2 * (3 * o + k))) & 3u); }

}  // namespace topo
