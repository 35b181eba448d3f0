/*
 * topomax_gb300 -- C ABI of the GB300 (sm_103a) elasticity design loop.
 *
 * One context holds one structured design problem on one GPU: the CG1 design
 * space on the (nx+1) x (ny+1) vertex lattice, the vector-P2 displacement
 * space on the (2nx+1) x (2ny+1) node lattice, the Helmholtz filter, the
 * SIMP elasticity operator, the load vector and the clamped nodes.
 *
 * Conventions
 *   - every array argument is a DEVICE pointer owned by the caller, FP64;
 *   - CG1 vectors: vertex (i,j) at index j*(nx+1)+i;
 *   - P2 displacement: node (a,b) at index b*(2nx+1)+a, component c at
 *     2*index+c;
 *   - calls are stream-ordered on the stream passed in; a call returns after
 *     its work is enqueued, except where a host decision needs a device value
 *     (iterative solves and the projection synchronise the stream);
 *   - return 0 on success, a negative TOPO_ERR_* code otherwise; the message
 *     of the last failure is available from topo_last_error();
 *   - a context is not thread-safe: use one host thread and one stream per
 *     context;
 *   - the create functions finish their device set-up before they return, so
 *     the first call may use any stream, blocking or not.
 *
 * Each entry point names the reference interface (Emilinya/topomax) it
 * replaces.
 */
#ifndef TOPOMAX_GB300_H
#define TOPOMAX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* topo_stream_t; /* == cudaStream_t */
typedef struct topo_ctx topo_ctx;

#define TOPO_OK 0
#define TOPO_ERR_ARG (-1)           /* invalid argument / size */
#define TOPO_ERR_NOT_CONVERGED (-2) /* iterative solve hit its iteration cap */
#define TOPO_ERR_TIMEOUT (-3)       /* bounded device wait gave up */
#define TOPO_ERR_NAN (-4)           /* non-finite value met */
#define TOPO_ERR_CUDA (-5)          /* CUDA runtime error */
#define TOPO_ERR_STATE (-6)         /* call order violated (e.g. no penalisation set) */
#define TOPO_ERR_PROJECTION (-7)    /* volume projection failed to bracket/converge */

/* sides, FEM_src/domains.py:18-38 / designs/definitions.py:22-46 */
#define TOPO_SIDE_LEFT 1
#define TOPO_SIDE_RIGHT 2
#define TOPO_SIDE_TOP 4
#define TOPO_SIDE_BOTTOM 8

/* arithmetic of the iterative solves */
#define TOPO_PREC_FP64 0  /* FP64 multigrid-preconditioned CG */
#define TOPO_PREC_MIXED 1 /* FP32 multigrid-preconditioned CG inside FP64 iterative refinement */

/* flags of the solve calls */
#define TOPO_SOLVE_WARM 1 /* use the output array's contents as the initial guess */

typedef struct {
  double width, height; /* domain [0,width] x [0,height] */
  int nx, ny;           /* squares along x and y (each split in two triangles) */
} topo_grid_desc;

typedef struct {
  double young_modulus, poisson_ratio; /* designs/definitions.py:169-200 */
  double filter_radius;                /* Helmholtz filter epsilon */
  double penal_min;                    /* SIMP minimum m (src/penalizers.py:34: 1e-6) */
} topo_material;

typedef struct {
  int fixed_sides;          /* OR of TOPO_SIDE_*: zero displacement on whole sides */
  int n_fixed_points;       /* extension: clamped mesh vertices */
  const double* fixed_points; /* host array of (x, y) pairs, snapped to the nearest vertex */
} topo_bc_desc;

typedef struct {
  int side; /* TOPO_SIDE_* */
  double center, length, value_x, value_y;
} topo_traction;

typedef struct {
  int has_body_force; /* circular body force, FEM_src/elasisity_problem.py:20-36 */
  double center_x, center_y, radius, value_x, value_y;
  int n_tractions;                /* FEM_src/elasisity_problem.py:39-73 */
  const topo_traction* tractions; /* host array */
} topo_load_desc;

/* Problem set-up: mesh (FEM_src/solver.py:38-49), spaces (FEM_src/elasisity_problem.py:194-196),
 * clamped sides (FEM_src/elasisity_problem.py:171-192), the pre-assembled load vector
 * (FEM_src/pde_solver.py:102-104) and the filter operator (FEM_src/filter.py:15-38).
 * Replaces ElasticityProblem.__init__ (FEM_src/elasisity_problem.py:79-102). */
topo_ctx* topo_create(const topo_grid_desc* grid, const topo_material* mat, const topo_bc_desc* bc,
                      const topo_load_desc* load, int precision, int* status);

/* Filter-only context: replaces HelmholtzFilter.__init__ (FEM_src/filter.py:15-38). */
topo_ctx* topo_create_filter(const topo_grid_desc* grid, double epsilon, int precision, int* status);

void topo_destroy(topo_ctx* ctx);

/* Message of the last failed call on this context ("" if none). */
const char* topo_last_error(const topo_ctx* ctx);

/* Sizes: CG1 vertices and P2 displacement dofs. */
int topo_sizes(const topo_ctx* ctx, int64_t* n_vertices, int64_t* n_dofs);

/* Replaces Problem.set_penalization (src/problem.py:13, src/penalizers.py:14-20). */
int topo_set_penalization(topo_ctx* ctx, double p);

/* Warm starts of the filter solves (enable = 1; off by default, 0 turns them off and forgets the
 * stored solutions): topo_filter_apply starts from the solution of the previous
 * topo_filter_apply on this context, topo_sensitivity from the previous topo_sensitivity's
 * (extrapolated over the design iterations once more solutions exist: 2 x1 - x2 from two,
 * 3 x1 - 3 x2 + x3 from three, 4 x1 - 6 x2 + 4 x3 - x4 from four; environment
 * TOPO_EXTRAPOLATE at context creation: 0 keeps x1, 1 linear ... 4 quartic, 3 cubic the
 * default); a failed solve is not reused.  Between design iterations both right-hand sides change little,
 * so a solve to the same rtol takes fewer iterations.  No counterpart in the reference, whose
 * HelmholtzFilter (FEM_src/filter.py:40-41) factorises and solves directly. */
int topo_set_filter_warm_start(topo_ctx* ctx, int enable);

/* Cap on the Krylov iterations of one filter or state solve (0 restores the defaults: 200
 * for the filter, 500 for the state; in mixed precision the cap counts the FP32 inner
 * iterations over all refinement steps of the solve).  A solve that reaches the cap
 * without meeting its tolerance returns TOPO_ERR_NOT_CONVERGED.  No counterpart in the
 * reference, whose SmartMumpsSolver (FEM_src/pde_solver.py:106-133) is a direct solver. */
int topo_set_iteration_limit(topo_ctx* ctx, int max_iterations);

/* xi = A_f^-1 M1 f for a CG1 field f: replaces HelmholtzFilter.apply
 * (FEM_src/filter.py:40-41).  iters receives the inner CG iterations (may be NULL). */
int topo_filter_apply(topo_ctx* ctx, const double* f, double* xi, double rtol, int* iters,
                      topo_stream_t stream);

/* xi = A_f^-1 b for an assembled CG1 right-hand side b (the filter of a UFL expression,
 * FEM_src/pde_solver.py:121-131 with l_arg an expression). */
int topo_filter_solve(topo_ctx* ctx, const double* b, double* xi, double rtol, int* iters,
                      topo_stream_t stream);

/* u = K(xi)^-1 f: replaces ElasticityProblem.forward / SmartMumpsSolver.solve
 * (FEM_src/elasisity_problem.py:168-169, FEM_src/pde_solver.py:106-133).
 * flags: TOPO_SOLVE_WARM uses u as the initial guess.  u must be 16-byte aligned
 * (TOPO_ERR_ARG otherwise): the kernels access a node's two components at once. */
int topo_state_solve(topo_ctx* ctx, const double* xi, double* u, double rtol, int flags, int* iters,
                     topo_stream_t stream);

/* *compliance = int u.f dx + int u.t ds  (FEM_src/elasisity_problem.py:161-166). */
int topo_compliance(topo_ctx* ctx, const double* u, double* compliance, topo_stream_t stream);

/* b_i = int -r'(xi)(lambda div(u)^2 + 2 mu eps(u):eps(u)) phi_i dx: the right-hand side that
 * ElasticityProblem.calculate_objective_gradient filters (FEM_src/elasisity_problem.py:134-150). */
int topo_sensitivity_rhs(topo_ctx* ctx, const double* u, const double* xi, double* b,
                         topo_stream_t stream);

/* g = A_f^-1 b_s: replaces ElasticityProblem.calculate_objective_gradient
 * (FEM_src/elasisity_problem.py:134-150). */
int topo_sensitivity(topo_ctx* ctx, const double* u, const double* xi, double* g, double rtol,
                     int* iters, topo_stream_t stream);

/* psi = project(psi_prev - alpha g, volume): replaces Solver.step / Solver.project
 * (src/solver.py:149-194; Newton from c=0 with tol 1e-12, bracketing fallback as
 * src/utils.py:138-157).  *c receives the multiplier (host pointer, may be NULL). */
int topo_emd_step(topo_ctx* ctx, const double* psi_prev, const double* g, double alpha, double volume,
                  double* psi, double* c, topo_stream_t stream);

/* rho = expit(psi) and *delta = sqrt(int (rho - expit(psi_prev))^2): the design update and
 * convergence measure of Solver.solve (src/solver.py:262, 284-286).  psi_prev may be NULL
 * (then *delta is not written); delta is a host pointer. */
int topo_emd_finish(topo_ctx* ctx, const double* psi, const double* psi_prev, double* rho,
                    double* delta, topo_stream_t stream);

/* *out = int f dx for a CG1 field: replaces FEMSolver.integrate (FEM_src/solver.py:81-84). */
int topo_integrate(topo_ctx* ctx, const double* f, double* out, topo_stream_t stream);

/* Starting point of a warm-started state solve from the last `count` solutions
 * (history[0] the newest, 1 <= count <= 5), in one pass:
 *   u = sum_i (-1)^i binom(count, i + 1) history[i],
 * the polynomial extrapolation of degree count - 1 over the design iterations (count 1
 * copies history[0]).  The reference solves each state directly
 * (FEM_src/elasisity_problem.py:168-169); this only supplies the iterative solve's
 * first iterate (topo_state_solve with TOPO_SOLVE_WARM).  u and every history entry
 * hold n_dofs doubles (topo_sizes); history is a host array of device pointers. */
int topo_state_warm_start(topo_ctx* ctx, const double* const* history, int count, double* u,
                          topo_stream_t stream);

/* y = K(xi) u in FP64 with clamped rows/columns as identity (test hook: the operator of
 * FEM_src/elasisity_problem.py:104-132 after bc.apply).  u and y 16-byte aligned. */
int topo_apply_state(topo_ctx* ctx, const double* xi, const double* u, double* y, topo_stream_t stream);

/* Measurement hook (no counterpart in the reference): *ms = duration of ONE launch of the
 * state operator y = K(xi) x on the design of the last topo_state_solve, timed with CUDA events
 * on `stream` -- the FP32 matrix-free kernel for a TOPO_PREC_MIXED context, the FP64 one
 * otherwise.  Synchronises the stream. */
int topo_time_operator(topo_ctx* ctx, double* ms, topo_stream_t stream);

/* Measurement hook (no counterpart in the reference): kernels this context has launched so far
 * (kernels executed inside CUDA graphs are counted per execution). */
int topo_launch_count(const topo_ctx* ctx, int64_t* launches);

/* Measurement hook (no counterpart in the reference), process-wide and off by default:
 * enable = 1 clears the totals and starts the kernel clock, 0 stops it.  While it runs, the
 * solver's main kernels launched from the host (contexts created with TOPO_GRAPHS=0; launches
 * on a capturing stream are never timed) are each bracketed by CUDA events and summed per
 * family and level with their algorithmic bytes.  Not thread-safe: one measuring thread. */
int topo_kernel_clock(int enable);

/* Writes the kernel clock's totals as text, one line per family and level:
 * "family<TAB>level<TAB>launches<TAB>milliseconds<TAB>algorithmic bytes<LF>", into buf when len
 * is large enough (waits for the timed launches).  Returns the length needed including the
 * terminating NUL, or TOPO_ERR_CUDA. */
int64_t topo_kernel_clock_report(char* buf, int64_t len);

/* Measurement hook (no counterpart in the reference): the tiles the march-kernel autotuner
 * chose in this process (cell rows per warp segment), as text, one line per kernel family and
 * grid: "family<TAB>nx<TAB>ny<TAB>segment<LF>", into buf when len is large enough.  Returns the
 * length needed including the terminating NUL. */
int64_t topo_march_tiles_report(char* buf, int64_t len);

/* y = M1 x with M1 the consistent CG1 mass matrix (the assembled (x, v) form, as the filter's
 * right-hand side FEM_src/filter.py:30-37 assembles it), FP64.  No counterpart as a function in
 * the reference: the Euclidean gradient of the compliance with respect to the nodal design is
 * M1 g, g the CG1 Riesz representative topo_sensitivity returns
 * (FEM_src/elasisity_problem.py:134-150). */
int topo_mass_apply(topo_ctx* ctx, const double* x, double* y, topo_stream_t stream);

/* Copy of the pre-assembled load vector (2*n_p2 entries, clamped dofs zero). */
int topo_load_vector(topo_ctx* ctx, double* b, topo_stream_t stream);

/* Largest mesh (in triangles, 2*nx*ny) topo_sensitivity_rhs_noalloc accepts. */
#define TOPO_NOALLOC_MAX_TRIANGLES (1 << 20)

/* topo_sensitivity_rhs without a context and without any device allocation -- it has no
 * counterpart in the reference.  For callers that cannot call cudaMalloc (hosts that only hand
 * out device memory from their own fixed pool, callers inside a fixed memory budget, loops that
 * must not pay an allocation's device-wide synchronisation):
 * the per-triangle scratch is a fixed 12 MiB device array inside this library, held by every
 * GPU that loads it until the process exits.  Computes b exactly as topo_sensitivity_rhs on a
 * TOPO_PREC_MIXED context of the same grid and material (FP64 inputs/outputs, FP32 quadrature).
 * Returns TOPO_ERR_ARG when 2*nx*ny > TOPO_NOALLOC_MAX_TRIANGLES.  The first call on a device
 * looks up the array's device address (make it before any stream capture on that device).
 * Every call shares the one array: calls whose work overlaps on the GPU (different streams,
 * threads or processes sharing the context) race and must be serialised by the caller.
 * The status covers this call's launch errors; a CUDA error already pending on the calling
 * thread is left in place and the call returns TOPO_ERR_CUDA without launching.  The device
 * address is looked up once per process: do not use the entry point across a cudaDeviceReset. */
int topo_sensitivity_rhs_noalloc(const topo_grid_desc* grid, double young_modulus, double poisson_ratio,
                                 double penalization, double penal_min, const double* u, const double* xi,
                                 double* b, topo_stream_t stream);

/* ---------------------------------------------------------------------------------------
 * Deep-energy-method (DEM) strain energy on the structured quadrilateral mesh
 * ---------------------------------------------------------------------------------------
 * The energy functional of DEM_src/elasisity_problem.py:79-129 (StrainEnergy) evaluated with
 * the 2x2 Gauss rule of DEM_src/objective_calculator.py:19-125 (ObjectiveCalculator), the
 * Dirichlet mask of DEM_src/dirichlet_enforcer.py:14-56 (ElasticityEnforcer) and the external
 * work of DEM_src/integrator.py:44-99 (boundary_integral, circular_integral), which is linear
 * in u and is passed in as per-node weights (the host precomputes them from the traction
 * intervals and the circle-cell areas of DEM_src/domains.py).
 * Layouts (the reference's): u float32 [(nx+1)*(ny+1)][2] with node (ix, iy) at
 * ix*(ny+1)+iy (DEM_src/utils.py:34-45 flatten order); density float32 [ny][nx] (cell (ix, iy)
 * at iy*nx+ix).  All arrays are device pointers unless stated otherwise. */
typedef struct topo_dem_ctx topo_dem_ctx;

typedef struct {
  int nx, ny;                /* cells in x and y (Mesh.Nx, Mesh.Ny) */
  float dshape[4][4][2];     /* Jinv * dN_i at Gauss point g: [node i][point g][x or y], nodes in the
                                order (ix,iy), (ix,iy+1), (ix+1,iy), (ix+1,iy+1) of
                                ObjectiveCalculator.get_gauss_points; float32 as torch rounds them */
  float detJ;                /* dx*dy/4 */
  float lame_lambda;         /* StrainEnergy.lame_lda, float32 */
  float two_mu;              /* 2 * StrainEnergy.lame_mu, float32 */
} topo_dem_desc;

/* Replaces StrainEnergy.__init__ / ObjectiveCalculator.__init__ (DEM_src/elasisity_problem.py:
 * 63-77, DEM_src/objective_calculator.py:19-23). */
topo_dem_ctx* topo_dem_create(const topo_dem_desc* desc, int* status);
void topo_dem_destroy(topo_dem_ctx* ctx);
const char* topo_dem_last_error(const topo_dem_ctx* ctx);

/* ObjectiveCalculator.set_penalization (DEM_src/objective_calculator.py:25-26). */
int topo_dem_set_penalization(topo_dem_ctx* ctx, double p);

/* External work weights: host float32 [(nx+1)*(ny+1)][2]; the external energy is
 * sum_n w[n][0]*u[n][0] + w[n][1]*u[n][1] (calculate_traction_integral +
 * calculate_body_force_integral, DEM_src/elasisity_problem.py:31-60).  NULL clears them. */
int topo_dem_set_external(topo_dem_ctx* ctx, const float* weights_host);

/* Dirichlet mask: host float32 [(nx+1)*(ny+1)][2] (ElasticityEnforcer.zero_enforcer).  NULL
 * clears it. */
int topo_dem_set_mask(topo_dem_ctx* ctx, const float* mask_host);

/* ElasticityEnforcer.__call__ (DEM_src/dirichlet_enforcer.py:55-56): u = u_hat * mask. */
int topo_dem_enforce(topo_dem_ctx* ctx, const float* u_hat, float* u, topo_stream_t stream);

/* StrainEnergy.calculate_energy (DEM_src/elasisity_problem.py:97-118):
 * psi = 0.5 * sum_cells r(rho) SE detJ - external work, SE = sum over the 4 Gauss points of
 * sigma:eps.  With masked != 0, u is the network output u_hat and the mask is applied on the
 * fly (the enforcer fused into the energy).  energy: device double scalar. */
int topo_dem_energy(topo_dem_ctx* ctx, const float* u, const float* density, int masked, double* energy,
                    topo_stream_t stream);

/* Gradient of topo_dem_energy times the device float scalar *scale: du float32 [nn][2]
 * (d psi / d u, or d psi / d u_hat when masked) and/or ddensity float32 [ny][nx]
 * (0.5 r'(rho) SE detJ); either may be NULL.  No counterpart in the reference (torch autograd
 * of calculate_energy there). */
int topo_dem_energy_backward(topo_dem_ctx* ctx, const float* u, const float* density, int masked,
                             const float* scale, float* du, float* ddensity, topo_stream_t stream);

/* StrainEnergy.calculate_objective_and_gradient (DEM_src/elasisity_problem.py:120-129):
 * objective = sum r(rho) SE detJ (device double scalar), gradient = -r'(rho) SE detJ
 * (device float32 [ny][nx]). */
int topo_dem_objective_gradient(topo_dem_ctx* ctx, const float* u, const float* density, double* objective,
                                float* gradient, topo_stream_t stream);

/* ---- DEM density filter: replaces create_density_filter (DEM_src/filter.py:8-31) and
 * its two uses, W @ rho and W.T @ g (DEM_src/elasisity_problem.py:148, 162, 171). ------
 * W_ij = (radius - d_ij) / S_i for element points i, j (np.linspace(0, width, Nx) x
 * np.linspace(0, height, Ny), element i = iy*Nx + ix) within radius, S_i the row sum;
 * evaluated on the fly in FP64 with the reference's order of operations (bit-identical
 * to the scipy/sklearn product).  create computes the row sums (synchronises). */
typedef struct topo_density_filter topo_density_filter;
topo_density_filter* topo_density_filter_create(int Nx, int Ny, double width, double height, double radius,
                                                int* status);
void topo_density_filter_destroy(topo_density_filter* f);
/* number of stored entries of the reference's sparse W (entries with d_ij <= radius) */
int topo_density_filter_nnz(const topo_density_filter* f, int64_t* nnz);
/* y = W x (transpose = 0) or y = W^T x (transpose = 1); device FP64 [Nx*Ny], x != y */
int topo_density_filter_apply(topo_density_filter* f, const double* x, double* y, int transpose,
                              topo_stream_t stream);

/* ---------------------------------------------------------------------------------------
 * Stokes-Brinkman fluid problem (Taylor-Hood P2 velocity / P1 pressure), FP64
 * ---------------------------------------------------------------------------------------
 * Replaces FluidProblem (FEM_src/fluid_problem.py:48-155) with the FluidPenalizer of
 * src/penalizers.py:49-67: forward (:168-169), calculate_objective (:152-166) and
 * calculate_objective_gradient (:134-150).  Velocities are interleaved [(2nx+1)(2ny+1)][2]
 * on the P2 lattice, pressures and designs are CG1 [(nx+1)(ny+1)], all device FP64.  Every
 * side is a Dirichlet side: the flow profiles of BoundaryFlows (:12-45) on the flow sides,
 * no slip (applied last) on the others.  The pressure is returned with zero sum: the state
 * system is singular in the pressure constant and, with the interpolated profiles, slightly
 * inconsistent; the continuity right-hand side is projected to zero sum. */
typedef struct {
  int side;      /* TOPO_SIDE_* */
  double center; /* profile centre along the side */
  double length; /* profile width */
  double rate;   /* peak velocity (rate * (1 - (2 t / length)^2)) */
} topo_flow;

typedef struct topo_fluid_ctx topo_fluid_ctx;
topo_fluid_ctx* topo_fluid_create(const topo_grid_desc* grid, double viscosity, const topo_flow* flows, int n_flows,
                                  int* status);
void topo_fluid_destroy(topo_fluid_ctx* ctx);
const char* topo_fluid_last_error(const topo_fluid_ctx* ctx);
int topo_fluid_sizes(const topo_fluid_ctx* ctx, int64_t* n_vertices, int64_t* n_velocity);
/* FluidPenalizer.set_penalization (src/penalizers.py:9-14): q > 0 */
int topo_fluid_set_penalization(topo_fluid_ctx* ctx, double q);
/* the Dirichlet data (zero at interior nodes) into u [2 n2] */
int topo_fluid_boundary_values(topo_fluid_ctx* ctx, double* u, topo_stream_t stream);
/* y = A x for x = [u (2 n2) | p (nv)] (n = 2 n2 + nv), A the state operator with the
 * continuity rows negated (symmetric on velocities vanishing on the boundary); clamp = 1
 * makes the boundary velocity rows identity rows.  x != y. */
int topo_fluid_apply(topo_fluid_ctx* ctx, const double* rho, const double* x, double* y, int clamp,
                     topo_stream_t stream);
/* forward: velocity u [2 n2] (boundary data included) and pressure p [nv] (may be null),
 * flexible GMRES to |r| <= rtol |b| on the reduced system; synchronises */
int topo_fluid_state_solve(topo_fluid_ctx* ctx, const double* rho, double* u, double* p, double rtol, int* iters,
                           topo_stream_t stream);
/* 1/2 int alpha(rho) |u|^2 + viscosity |grad u|^2 dx into a device double */
int topo_fluid_objective(topo_fluid_ctx* ctx, const double* rho, const double* u, double* objective,
                         topo_stream_t stream);
/* b_k = int 1/2 alpha'(rho) |u|^2 phi_k (the projection's right-hand side, degree-7 rule) */
int topo_fluid_gradient_rhs(topo_fluid_ctx* ctx, const double* rho, const double* u, double* b,
                            topo_stream_t stream);
/* g = M1^-1 b: the CG1 L2 projection of 1/2 alpha'(rho) |u|^2 (df.project); synchronises */
int topo_fluid_gradient(topo_fluid_ctx* ctx, const double* rho, const double* u, double* g, double rtol,
                        int* iters, topo_stream_t stream);
int topo_fluid_launch_count(const topo_fluid_ctx* ctx, int64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* TOPOMAX_GB300_H */
