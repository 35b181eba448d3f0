// Precision-independent parts of the multigrid set-up.
#include <algorithm>
#include <cmath>
#include <cstring>

#include <mutex>

#include "topo_mg.h"

namespace topo {

std::recursive_mutex& device_lock() {
  static std::recursive_mutex m;
  return m;
}

Arena::~Arena() {
  std::lock_guard<std::recursive_mutex> lock(device_lock());
  for (void* p : ptrs_) cudaFree(p);
}

void* Arena::alloc(size_t bytes) {
  void* p = nullptr;
  const size_t b = std::max<size_t>(bytes, 16);
  if (cudaMalloc(&p, b) != cudaSuccess) {
    failed_ = true;
    return nullptr;
  }
  cudaMemset(p, 0, b);
  ptrs_.push_back(p);
  bytes_ += b;
  return p;
}

static void add_point(Dir& d, int a, int b, int NX, int NY) {
  if (a < 0 || b < 0 || a >= NX || b >= NY) return;
  for (int k = 0; k < d.npts; ++k)
    if (d.pts[2 * k] == a && d.pts[2 * k + 1] == b) return;
  if (d.npts < kMaxDirPoints) {
    d.pts[2 * d.npts] = a;
    d.pts[2 * d.npts + 1] = b;
    ++d.npts;
  }
}

// Coarse node I is clamped when its hat function is non-zero at a clamped
// fine node (fine columns 2I-1..2I+1), so the coarse space stays inside the
// fine space of functions vanishing on the clamped nodes.
Dir coarsen_dir(const Dir& f, int NXf, int NYf, int NXc, int NYc) {
  Dir c;
  std::memset(&c, 0, sizeof(c));
  c.x_lo = f.x_lo;
  c.y_lo = f.y_lo;
  c.x_hi_from = (f.x_hi_from >= NXf) ? NXc : f.x_hi_from / 2;
  c.y_hi_from = (f.y_hi_from >= NYf) ? NYc : f.y_hi_from / 2;
  for (int k = 0; k < f.npts; ++k) {
    const int a = f.pts[2 * k], b = f.pts[2 * k + 1];
    const int pa = a & 1, pb = b & 1;
    if (!pa && !pb) {
      add_point(c, a / 2, b / 2, NXc, NYc);
    } else if (pa && !pb) {
      add_point(c, (a - 1) / 2, b / 2, NXc, NYc);
      add_point(c, (a + 1) / 2, b / 2, NXc, NYc);
    } else if (!pa && pb) {
      add_point(c, a / 2, (b - 1) / 2, NXc, NYc);
      add_point(c, a / 2, (b + 1) / 2, NXc, NYc);
    } else {
      add_point(c, (a - 1) / 2, (b - 1) / 2, NXc, NYc);
      add_point(c, (a + 1) / 2, (b + 1) / 2, NXc, NYc);
    }
  }
  return c;
}

std::vector<LevelSpec> build_levels(bool p2_top, int nx, int ny, double hx, double hy, const Dir& top, int NC) {
  std::vector<LevelSpec> v;
  LevelSpec L;
  if (p2_top) {
    L.p2 = true;
    L.nx = nx;
    L.ny = ny;
    L.NX = 2 * nx + 1;
    L.NY = 2 * ny + 1;
    L.NC = 2;
    L.hx = hx;
    L.hy = hy;
    L.dir = top;
    v.push_back(L);
    LevelSpec P;
    P.p2 = false;
    P.nx = nx;
    P.ny = ny;
    P.NX = nx + 1;
    P.NY = ny + 1;
    P.NC = 2;
    P.hx = hx;
    P.hy = hy;
    P.dir = coarsen_dir(top, L.NX, L.NY, P.NX, P.NY);
    v.push_back(P);
  } else {
    L.p2 = false;
    L.nx = nx;
    L.ny = ny;
    L.NX = nx + 1;
    L.NY = ny + 1;
    L.NC = NC;
    L.hx = hx;
    L.hy = hy;
    L.dir = top;
    v.push_back(L);
  }
  while (v.back().ndof() > size_t(kCoarseMaxDofs) && (v.back().nx > 1 || v.back().ny > 1)) {
    const LevelSpec& F = v.back();
    LevelSpec C;
    C.p2 = false;
    C.nx = (F.nx + 1) / 2;
    C.ny = (F.ny + 1) / 2;
    C.NX = C.nx + 1;
    C.NY = C.ny + 1;
    C.NC = F.NC;
    C.hx = 2 * F.hx;
    C.hy = 2 * F.hy;
    C.dir = coarsen_dir(F.dir, F.NX, F.NY, C.NX, C.NY);
    v.push_back(C);
  }
  return v;
}

ElemRefs make_elem_refs(double hx, double hy, double lmbda, double mu) {
  ElemRefs R;
  std::memset(&R, 0, sizeof(R));
  const double area = 0.5 * hx * hy;
  // barycentric gradients, orientation 0: (v0,v1,v3), 1: (v0,v2,v3)
  const double G[2][3][2] = {{{-1 / hx, 0}, {1 / hx, -1 / hy}, {0, 1 / hy}},
                             {{0, -1 / hy}, {-1 / hx, 1 / hy}, {1 / hx, 0}}};
  for (int o = 0; o < 2; ++o) {
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) {
        const double gg = G[o][k][0] * G[o][l][0] + G[o][k][1] * G[o][l][1];
        R.K1[o][k][l] = area * gg;
        R.M1[o][k][l] = area / 12.0 * (k == l ? 2.0 : 1.0);
        for (int c = 0; c < 2; ++c)
          for (int d = 0; d < 2; ++d) {
            // K[(k,c),(l,d)] = lam dc(lk) dd(ll) + mu dcd grad lk.grad ll + mu dc(ll) dd(lk)
            double v = lmbda * G[o][k][c] * G[o][l][d] + mu * G[o][l][c] * G[o][k][d];
            if (c == d) v += mu * gg;
            R.K2[o][2 * k + c][2 * l + d] = area * v;
          }
      }
  }
  return R;
}

// Eigenvalue range of the symmetric n x n matrix A (cyclic Jacobi rotations).
static void sym_eig_range(std::vector<double> A, int n, double& lo, double& hi) {
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += A[p * n + q] * A[p * n + q];
    if (off < 1e-30) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A[p * n + q];
        if (std::fabs(apq) < 1e-300) continue;
        const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < n; ++k) {  // columns p, q
          const double akp = A[k * n + p], akq = A[k * n + q];
          A[k * n + p] = c * akp - sn * akq;
          A[k * n + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p, q
          const double apk = A[p * n + k], aqk = A[q * n + k];
          A[p * n + k] = c * apk - sn * aqk;
          A[q * n + k] = sn * apk + c * aqk;
        }
      }
  }
  lo = hi = A[0];
  for (int k = 1; k < n; ++k) {
    lo = std::min(lo, A[k * n + k]);
    hi = std::max(hi, A[k * n + k]);
  }
}

static double sym_eig_max(const std::vector<double>& A, int n) {
  double lo, hi;
  sym_eig_range(A, n, lo, hi);
  return hi;
}

// max over orientations of lambda_max(D_e^-1 K_e) for the unit-coefficient P1
// elasticity element: since lambda_max(D^-1 A) <= max_e lambda_max(D_e^-1 A_e)
// and a per-triangle coefficient cancels in D_e^-1 A_e, this bounds every P1
// elasticity level whatever its coefficients.
double p1_elasticity_bound(const ElemRefs& R) {
  double m = 1.0;
  for (int o = 0; o < 2; ++o) {
    std::vector<double> A(36);
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) A[i * 6 + j] = R.K2[o][i][j] / std::sqrt(R.K2[o][i][i] * R.K2[o][j][j]);
    m = std::max(m, sym_eig_max(A, 6));
  }
  return m;
}

// Range of the element eigenvalues of D_e^-1 (t K_e + M_e) over both triangle
// orientations (P1, Jacobi-scaled): bounds the spectrum of Dinv A of any
// operator assembled from such elements with coefficient ratio t.
void p1_helmholtz_bounds(const ElemRefs& R, double t, double& lo, double& hi) {
  lo = 1e300;
  hi = 0.0;
  for (int o = 0; o < 2; ++o) {
    double E[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) E[i][j] = t * R.K1[o][i][j] + R.M1[o][i][j];
    std::vector<double> A(9);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) A[i * 3 + j] = E[i][j] / std::sqrt(E[i][i] * E[j][j]);
    double l, h;
    sym_eig_range(A, 3, l, h);
    lo = std::min(lo, l);
    hi = std::max(hi, h);
  }
}

int coarse_cheb_plan(const ElemRefs& R, double tmin, double tmax, double tol, double& lo, double& hi) {
  lo = 1e300;
  hi = 0.0;
  // the element bounds at ratios spread over [tmin, tmax], with margins
  for (int k = 0; k <= 8; ++k) {
    const double t = tmin > 0 ? tmin * std::pow(tmax / tmin, k / 8.0) : tmin + (tmax - tmin) * k / 8.0;
    double a, b;
    p1_helmholtz_bounds(R, t, a, b);
    lo = std::min(lo, a);
    hi = std::max(hi, b);
  }
  lo = std::min(0.9 * lo, 1.0);  // clamped rows are identity rows (eigenvalue 1)
  hi = std::max(1.05 * hi, 1.0);
  const double kap = hi / lo, q = (std::sqrt(kap) - 1.0) / (std::sqrt(kap) + 1.0);
  if (!(q > 0.0)) return 1;
  const int d = int(std::ceil(std::log(0.5 * tol) / std::log(q)));
  return d < 1 ? 1 : d;
}

void Reducer::init(Arena& a, int nsms) {
  sms = nsms;
  blocks = nsms * 8;
  partials = a.alloc_n<double>(size_t(blocks) * 16);
  counter = a.alloc_n<unsigned>(1);
  out = a.alloc_n<double>(16);
  cudaMallocHost(&host, 16 * sizeof(double));
}

}  // namespace topo
