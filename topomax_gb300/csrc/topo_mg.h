// Geometric multigrid-preconditioned CG on the structured lattice.
//
// Level 0 is either the matrix-free P2 elasticity operator (state solve) or
// a P1 operator (Helmholtz filter).  Every coarser level is a P1 operator with
// per-triangle coefficients (see topo_p1.cuh); the coarsest level (at most
// kCoarseMaxDofs unknowns) is solved with a dense inverse formed on the GPU.
// Smoothing: Chebyshev polynomials in D^-1 A with eigenvalue bounds from a
// power iteration at set-up.
#pragma once

#include <cuda_runtime.h>
#include <cstring>
#include <string>
#include <mutex>
#include <vector>

#include "topo_common.cuh"
#include "topo_p2.cuh"

namespace topo {

constexpr int kCoarseMaxDofs = 32;

// Device memory owner: everything allocated here is freed with the arena.
class Arena {
 public:
  Arena() = default;
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  ~Arena();
  void* alloc(size_t bytes);
  template <class T>
  T* alloc_n(size_t n) { return static_cast<T*>(alloc(n * sizeof(T))); }
  size_t bytes() const { return bytes_; }
  bool failed() const { return failed_; }

 private:
  std::vector<void*> ptrs_;
  size_t bytes_ = 0;
  bool failed_ = false;
};

// Serialises, across the threads of a process, what must not overlap another
// thread's CUDA-graph recording: device memory release (cudaFree synchronises
// the whole device, which would invalidate a recording in progress), context
// set-up and the recordings themselves.
std::recursive_mutex& device_lock();

// Context set-up writes device memory on the default stream: Arena::alloc zeroes
// with cudaMemset, host tables go up with pageable cudaMemcpy (which may return
// before its DMA lands), and set-up kernels launch without a stream.  A caller's
// stream created non-blocking (every torch stream is) is not ordered after that
// work, so a context is handed out only after the default stream has drained.
inline cudaError_t settle_setup_stream() { return cudaStreamSynchronize(0); }

struct LevelSpec {
  bool p2 = false;  // P2 elasticity level (only level 0 of the state hierarchy)
  int nx = 0, ny = 0;
  int NX = 0, NY = 0, NC = 1;
  double hx = 0, hy = 0;
  Dir dir{};
  size_t nn() const { return size_t(NX) * NY; }
  size_t ndof() const { return nn() * NC; }
  size_t ntri() const { return size_t(2) * nx * ny; }
};

Dir coarsen_dir(const Dir& f, int NXf, int NYf, int NXc, int NYc);
std::vector<LevelSpec> build_levels(bool p2_top, int nx, int ny, double hx, double hy,
                                    const Dir& top, int NC);

// Unit-coefficient P1 element matrices of one level.
struct ElemRefs {
  double K2[2][6][6];  // elasticity (lambda, mu given)
  double K1[2][3][3];  // Laplacian
  double M1[2][3][3];  // mass
};
ElemRefs make_elem_refs(double hx, double hy, double lmbda, double mu);
double p1_elasticity_bound(const ElemRefs& R);
void p1_helmholtz_bounds(const ElemRefs& R, double t, double& lo, double& hi);
// Interval [lo, hi] holding the spectrum of Dinv A for P1 levels assembled from
// t K_e + M_e with t in [tmin, tmax], and the Chebyshev degree reaching a
// residual reduction tol on it.
int coarse_cheb_plan(const ElemRefs& R, double tmin, double tmax, double tol, double& lo, double& hi);

// Reduction scratch shared by one stream.
struct Reducer {
  double* partials = nullptr;  // [blocks * 16]
  unsigned* counter = nullptr;
  double* out = nullptr;       // device scalars [16]
  double* host = nullptr;      // pinned mirror [16]
  int sms = 148;
  int blocks = 0;
  void init(Arena& a, int sms);
};

// Device-resident scalars of one preconditioned-CG solve (read back once at the end).
struct PcgDev {
  double bb, rz, pq, beta, tol2, relres;
  double rr, rz_new;  // adjacent: one two-value reduction writes both
  double alpha;       // the iteration's step as applied to r (rounded to the CG's precision; 0 on breakdown)
  int it, maxit, status, pad;  // status: 0 converged, 1 running, 2 iteration cap, 3 breakdown, 4 non-finite, 5 zero rhs
};

struct SolveStats {
  int iterations = 0;       // inner Krylov iterations (sum)
  int minres = 0;           // 1 if the MINRES fallback ran
  int outer = 0;            // refinement steps
  double relres = 0.0;      // final relative residual (in the solve's precision)
  int status = 0;
};

template <class T>
class MG {
 public:
  // coefficient masters (double, per P1 level; index by level) are owned by
  // the caller and must outlive the MG object.
  void init(const std::vector<LevelSpec>& specs, const ElemRefs* refs, double lmbda, double mu,
            Arena& arena, Reducer* red);
  // level-0 P2 parameters: the Krylov operator (true penalisation) and the
  // preconditioner's operator (penalisation clamped at its minimum, SPD);
  // xi points to the design in precision T
  void set_p2(const P2Params<T>& op, const P2Params<T>& pc, const T* xi) {
    // kernel parameters are baked into the captured solve graphs
    if (std::memcmp(&op, &p2_op_, sizeof(op)) || std::memcmp(&pc, &p2_, sizeof(pc)) || xi != xi_)
      graph_valid_ = false;
    p2_op_ = op;
    p2_ = pc;
    xi_ = xi;
  }
  MG() = default;
  MG(const MG&) = delete;
  MG& operator=(const MG&) = delete;
  ~MG();
  // kK/kM masters per level (entries for P2 level ignored; nullptr allowed)
  void set_coefficients(const std::vector<const double*>& kK, const std::vector<const double*>& kM) {
    kK64_ = kK;
    kM64_ = kM;
  }
  // constant mass coefficient on level 0 when it is P1 (filter)
  int setup(cudaStream_t s);  // diagonals, eigen bounds, coarse inverse
  // The coarse-Chebyshev truncation and the shared interior stencil rows are
  // chosen from the coefficients at the first setup() (a filter's never
  // change); a caller whose scalar coefficients change between setups calls
  // this first so that the next setup() chooses them again.
  void coefficients_changed() { cc_selected_ = false; }
  // y = A_l x; on level 0, op selects the Krylov operator instead of the
  // preconditioner's (they differ only where the penalisation is clamped)
  void apply(int l, const T* x, T* y, cudaStream_t s, bool op = false);
  void vcycle(const T* b, T* x, cudaStream_t s);
  // Krylov solve on level 0, multigrid-preconditioned: CG, restarted as MINRES
  // from the current iterate if CG meets p.Ap <= 0 (an indefinite operator).
  // Solves A x = b to ||r|| <= rtol ||b|| (x used as initial guess when x_nonzero).
  // Returns 0, -2 (iteration cap) or -4 (non-finite).
  int pcg(const T* b, T* x, bool x_nonzero, double rtol, int maxit, SolveStats& st, cudaStream_t s);
  // As pcg, with the solution accumulated and returned in FP64 (requires
  // fp64_solution): x64 is the initial guess when x_nonzero (rounded to T) and
  // receives the result.  Returns -5 when the object was set up without it.
  int pcg_x64(const T* b, double* x64, bool x_nonzero, double rtol, int maxit, SolveStats& st, cudaStream_t s);
  int minres(const T* b, T* x, double rtol, int maxit, SolveStats& st, cudaStream_t s);
  const LevelSpec& spec(int l) const { return specs_[l]; }
  int levels() const { return int(specs_.size()); }
  double lmax(int l) const { return lv_[l].lmax; }
  // device scratch vectors of level 0 (n dofs), free for callers between solves
  T* scratch0(int k) { return pcg_[k]; }
  static constexpr int kScratch = 10;
  // Accumulate the CG solution in FP64 (x += alpha p with the exact product).
  // With T = float the solution's own FP32 rounding limits its residual: on a
  // high-contrast design |A fl32(u) - f| / |f| is ~1e-2 at the exact u, while
  // the FP32 operator arithmetic alone is consistent to ~1e-4.  Set before init().
  bool fp64_solution = false;

  int cheb_degree = 2;  // the fused smoothing kernels implement degree 2
  double cheb_lo_frac = 0.1;   // smoothing interval [lo_frac, 1.1] * lambda_max
  int power_iters = 10;
  int power_iters_warm = 4;  // level 0 of a P2 hierarchy, started from the previous set-up's vector
  // kernels launched by this object since construction (graph nodes counted per execution)
  long long launches = 0;
  // record the CG loop as a CUDA graph with a device-side WHILE node (default);
  // false runs the same kernels from a host loop
  bool use_graphs = true;
  bool use_tail = true;      // run the smallest levels in the one-CTA shared-memory kernel
  // stop the V-cycle at the first P1 level whose Jacobi-scaled operator is well
  // conditioned enough for a short Chebyshev solve (scalar mass+stiffness levels)
  bool use_coarse_cheb = true;
  int coarse_cheb_max_degree = 16;
  int coarse_cheb_level() const { return cheb_coarse_; }
  int coarse_cheb_deg = 0;
  bool use_p1_march = true;  // large P1 levels: column march (false: node-centric kernels)
  long long capture_failures = 0;  // recordings that failed (those solves ran host-driven)
  // opt-in level timing (host-driven mode only): inclusive ms per level, summed
  bool profile_levels = false;
  bool trace_setup = false;  // print synchronised set-up phase times to stderr
  std::vector<double> level_ms;
  std::vector<long long> level_calls;
  void flush_level_profile();
  // tail phase timing (profile_levels only): SM cycles summed per phase in
  // execution order, last entry = launches; empty without a tail
  void tail_profile(std::vector<long long>& cycles) const;
  int tail_level() const { return tail_; }
  // tune the segment length of this hierarchy's march kernels (level 0 if P2, the P1
  // levels without a stencil) once per family and grid; needs set-up data in place
  bool autotune = true;

 private:
  struct Lev {
    T *x = nullptr, *b = nullptr, *r = nullptr, *d = nullptr, *t = nullptr, *x2 = nullptr;
    T* diag = nullptr;
    T* dinv = nullptr;
    T* kK = nullptr;
    T* kM = nullptr;
    T* st = nullptr;  // assembled stencil (levels up to stencil_max_nodes(NC) nodes)
    T* inner = nullptr;  // the shared interior stencil row (uniform levels; see P1Stencil::inner)
    double lmax = 1.0;
    bool bound = false;  // lmax is a guaranteed upper bound (no safety factor)
  };
  void vcycle_level(int l, const T* b, T* x, cudaStream_t s);
  void tune_marches(cudaStream_t s);
  void vcycle_level_body(int l, const T* b, T* x, cudaStream_t s);
  int prof_depth_ = 0;
  int capture_pcg(bool warm);
  void pcg_prologue(bool warm, cudaStream_t s);
  void pcg_body(cudaStream_t s, cudaGraphConditionalHandle h, int use_cond);
  // x (precision T) or x64 (FP64 solution mode) is the initial guess / result
  int graph_pcg(const T* b, T* x, double* x64, bool warm, double rtol, int maxit, SolveStats& st, cudaStream_t s);
  void pcg_xr(int g, cudaStream_t s);  // r -= alpha q (alpha recorded for pcg_p)
  void pcg_p(int g, cudaStream_t s);   // x += alpha p, p = z + beta p
  double dot(const T* a, const T* b, size_t n, cudaStream_t s);  // synchronising
  void diag_of(int l, T* d, cudaStream_t s);
  double estimate_lmax(int l, cudaStream_t s);

  std::vector<LevelSpec> specs_;
  std::vector<Lev> lv_;
  const ElemRefs* refs_ = nullptr;
  std::vector<const double*> kK64_, kM64_;
  double lmbda_ = 0, mu_ = 0;
  P2Params<T> p2_{};     // preconditioner operator (clamped penalisation)
  P2Params<T> p2_op_{};  // Krylov operator
  const T* xi_ = nullptr;
  T* cinv_ = nullptr;  // dense coarsest inverse
  int* cstat_ = nullptr;
  T* cheb_ = nullptr;  // Chebyshev coefficients, 8 per level (device, level precision)
  std::vector<T> cheb_host_;
  PcgDev* dev_ = nullptr;   // device scalars of the graph solve
  PcgDev* hdev_ = nullptr;  // pinned mirror
  cudaStream_t cap_[2] = {nullptr, nullptr};  // owned streams: graph recording, concurrent set-up
  cudaEvent_t ev_[3] = {nullptr, nullptr, nullptr};  // set-up fork/join
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    long long prologue_nodes = 0, body_nodes = 0;
  } graph_[2];
  bool graph_valid_ = false;
  void build_tail(Arena& arena);
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_events_;
  // truncated hierarchy: the V-cycle stops at level cheb_coarse_ and solves it
  // with a fixed-degree Chebyshev iteration in one CTA (CoarseChebDesc, device)
  int cheb_coarse_ = -1;
  void* cc_desc_ = nullptr;
  size_t cc_smem_ = 0;
  void select_coarse_cheb(cudaStream_t s);
  void detect_uniform_levels(cudaStream_t s);  // sets Lev::inner where every interior row is the same
  void* cc_buf_ = nullptr;
  T* inner_buf_ = nullptr;  // per level: one stencil row (detect_uniform_levels)
  bool cc_selected_ = false;
  int tail_ = -1;              // first level run by the one-CTA shared-memory tail kernel
  void* tail_desc_ = nullptr;  // TailDesc<T, NC> (device)
  size_t tail_smem_ = 0;
  long long* tail_trace_ = nullptr;
  // set by pcg_body around its V-cycle: the level-0 post-smoothing launch also
  // reduces r.r, r.z and runs the iteration's test
  bool stencils_ready_ = false;  // set once setup() has assembled the stencils
  bool fuse_rz_ = false;
  unsigned long long fuse_cond_ = 0;
  int fuse_use_cond_ = 0;

  T* pcg_[kScratch] = {};
  double* xacc_ = nullptr;  // FP64 solution of the CG loop (fp64_solution)
  T* pw_ = nullptr;         // level-0 power-iteration vector (P2 hierarchies)
  bool pw_ready_ = false;
  Reducer* red_ = nullptr;
  int sms_ = 148;
};

// Segment lengths of the column-march kernels chosen by the autotuner
// (MG::setup, once per kernel family and grid in a process): 0 when not tuned
// (the one-wave rule of p2_march_segment applies).  TOPO_AUTOTUNE=0 turns the
// tuner off.
int tuned_segment(int family, int nx, int ny);
void set_tuned_segment(int family, int nx, int ny, int seg);
bool autotune_enabled();
// march kernel family of the segment table: P2 or P1 march, precision, components
constexpr int march_family(bool p2, int value_bytes, int nc) { return (p2 ? 0 : 8) + (value_bytes == 8 ? 4 : 0) + nc; }

// y = A x for the FP64 P2 operator (used for refinement residuals)
void p2_apply_f64(const P2Params<double>& p, const double* xi, const double* x, double* y,
                  cudaStream_t s);
void p2_apply_f32(const P2Params<float>& p, const float* xi, const float* x, float* y,
                  cudaStream_t s);
// y = A x with pair-of-FP32 arithmetic (x, y FP64; p.rmass: per-cell mass matrices as
// (hi, lo) pairs), and its one-time occupancy query (outside any stream capture)
void p2_apply_dd(const P2Params<dd>& p, const double* x, double* y, cudaStream_t s);
void p2_dd_prime();

}  // namespace topo
