/*
 * nnpp_gb300.h -- C ABI of the GB300 (sm_103a) nonlocal Nernst-Planck-Poisson hot path.
 *
 * The library replaces, for one GPU, the reference's
 *   - neighbourhood build   build_clouds_hash(...)          src/helpers/grid.h:43-204
 *   - bond-sum residuals    utils::Residuals(...) F1..F4,F11  src/helpers/utils.h:29-842
 *   - potential operator    utils::NewtonMatrices(...) K11   src/helpers/utils.h:1794-1848
 *     and its solve         Eigen::GMRES on K11              src/main.cpp:764-779
 *   - step / front update   time loop of main()              src/main.cpp:547-1025
 * behind plain C entry points: host pointers and sizes only, no C++ or torch types.
 *
 * Layout conventions (the reference's Eigen containers, column-major):
 *   nodes   : double[3*N]   x[0..N-1], y[0..N-1], z[0..N-1]      (Eigen::MatrixXd N x 3)
 *   clouds  : int[N*max]    entry (i, j) at j*N + i, -1 padded     (Eigen::MatrixXi N x max)
 *   fields  : double[(S+1)*N] species k at k*N, the potential at S*N
 *             (U1..U4 and U11 of the reference, S = 4)
 *   phase   : int[N]        1 solid, 0 liquid                       (nodePhase)
 *
 * Error behaviour: every call returns an nnpp_status; no C++ exception crosses the ABI.
 * NNPP_ERR_CAPACITY is the reference's std::runtime_error("Not enough room to store
 * clouds") of grid.h:187-189.  nnpp_last_error() returns a message for the calling thread.
 *
 * Threading: a handle owns one CUDA stream and its device memory.  A handle is not
 * thread-safe; distinct handles are.  All entry points are synchronous with respect to the
 * host buffers they take.
 */
#ifndef NNPP_GB300_H
#define NNPP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NNPP_NSPECIES 4
#define NNPP_ABI_VERSION 1

typedef enum nnpp_status {
  NNPP_OK = 0,
  NNPP_ERR_INVALID = 1,          /* bad argument (null pointer, size, parameter) */
  NNPP_ERR_CAPACITY = 2,         /* neighbour list longer than max_node_no (grid.h:187-189) */
  NNPP_ERR_NONFINITE = 3,        /* a NaN/Inf appeared in the state */
  NNPP_ERR_CG_NO_CONVERGE = 4,   /* potential solve hit its iteration cap (strict mode) */
  NNPP_ERR_CUDA = 5,             /* CUDA runtime error, or no GPU */
  NNPP_ERR_UNSUPPORTED = 6,      /* valid for the reference, outside this library's scope */
  NNPP_ERR_STATE = 7,            /* call order violated (e.g. step before neighbour build) */
  NNPP_ERR_NOMEM = 8             /* device or host allocation failed */
} nnpp_status;

typedef enum nnpp_precision {
  NNPP_FP64 = 0,    /* plain FP64: FP64 bond sums, FP64 Jacobi-CG for the potential */
  NNPP_MIXED = 1    /* FP32 bond sums (compensated), FP32 inner CG + FP64 refinement */
} nnpp_precision;

typedef enum nnpp_preconditioner {
  NNPP_PRECOND_JACOBI = 0,     /* z = D^-1 r (the reference's diagonal scaling)            */
  NNPP_PRECOND_TWO_LEVEL = 1   /* z = D^-1 r + P A_c^-1 P^T r, aggregates of bin blocks     */
} nnpp_preconditioner;

/* Device-side checks (nnpp_set_checks), for debugging and for tests of the failure paths. */
typedef enum nnpp_check {
  NNPP_CHECK_BOUNDS = 1,       /* the halo-staged CG operator (operator 8) checks every quad,
                                  row and neighbour code against its array before using it;
                                  a violation is skipped and reported as NNPP_ERR_CUDA */
  NNPP_CHECK_WAIT_PROBE = 2    /* test of the bounded-wait path: after each tile's copies have
                                  landed, operator 8 also waits, bounded, on a barrier that
                                  nothing completes; the call then returns NNPP_ERR_CUDA (its
                                  results are invalid; nnpp_reset makes the handle usable) */
} nnpp_check;

typedef enum nnpp_order_mode {
  NNPP_ORDER_REFERENCE = 0,  /* within-cell order of std::sort as in grid.h:90 (bit-exact) */
  NNPP_ORDER_CANONICAL = 1   /* within-cell order by node index (stable counting sort)   */
} nnpp_order_mode;

/*
 * Model parameters: the subset of utils::parameter (utils.h:2186-2485) that the hot path
 * reads, for S = 4 transported species and the potential.  Species 0 follows the Mg2+
 * branch of Residuals (utils.h:72-178: solid-solid bonds kept, BV factor on mixed bonds);
 * species 1..3 follow the generic branch (utils.h:181-257: solid-solid bonds skipped).
 */
typedef struct nnpp_params {
  double dt, dx, dy, dz;          /* time step, lattice spacing (data2[2..5])            */
  double delta;                   /* horizon (data2[6])                                  */
  double CSolid, CSat;            /* normalising and saturation concentration (data2[7,8]) */
  double F, R, T;                 /* Faraday, gas constant, temperature (data2[49,48,47]) */
  double vol_red;                 /* BV = 10^(-vol_red*(1-voln1rel)) on mixed Mg bonds (data2[50]) */
  double z[NNPP_NSPECIES];        /* charges          (datac_k[0]) */
  double D_solid[NNPP_NSPECIES];  /* D_kSolid         (datac_k[1]) */
  double D_liquid[NNPP_NSPECIES]; /* D_kLiquid        (datac_k[2]) */
  double s1[NNPP_NSPECIES];       /* s_k1 diffusion kernel exponent (datac_k[3]) */
  double s2[NNPP_NSPECIES];       /* s_k2 migration kernel exponent (datac_k[4]) */
  double K1[NNPP_NSPECIES];       /* K_kprop1         (datac_k[5]) */
  double K2[NNPP_NSPECIES];       /* K_kprop2         (datac_k[6]) */
  double sigma;                   /* sigma1           (datac11[1]) */
  double s_phi;                   /* s111             (datac11[2]) */
  double K_phi;                   /* K11prop1         (datac11[3]) */
  double k_diss;                  /* dissolution rate of the Mg source on solid interface nodes */
  double switch_width;            /* 0: hard dissolution switch; w>0: sigmoid((c-CSat/CSolid)/w) */
  double c_floor;                 /* positivity clamp, 1e-8/CSolid in main.cpp:805-837 */
  int    sub_step_no;             /* volume (voln1rel) update period, 8 in main.cpp:39 */
  int    reserved;
} nnpp_params;

/* Per-run diagnostics, all accumulated in FP64 on the device. */
typedef struct nnpp_diag {
  int64_t steps_done;
  int64_t solid_count;            /* main.cpp:914-922 */
  double  voln1rel;               /* main.cpp:944-949 */
  double  vol0rel;                /* main.cpp:474-480 */
  double  mass[NNPP_NSPECIES];    /* sum_i c_k,i * dV, global ion-mass balance */
  double  mg_mass_lost;           /* dV * sum_i (c_0,i(t=0) - c_0,i(t)) */
  double  dissolved_total;        /* dV * dt * sum over steps of the dissolution source */
  int64_t cg_iterations_total;    /* inner CG iterations over the run */
  int64_t cg_solves;              /* potential solves over the run */
  int64_t cg_not_converged;       /* solves that hit the iteration cap */
  double  last_rel_residual;      /* FP64 ||b - A phi|| / ||b|| of the last solve */
  int64_t outer_iterations_total; /* FP64 refinement sweeps (mixed) */
} nnpp_diag;

typedef struct nnpp_handle nnpp_handle;

/* ---- library ------------------------------------------------------------------------- */

/* Thread-local message of the last failing call ("" if none). */
const char* nnpp_last_error(void);
/* NNPP_ABI_VERSION. */
int nnpp_abi_version(void);
/* Number of CUDA devices visible (0 on a machine without a GPU); never fails. */
int nnpp_device_count(void);
/* Device on which the calling thread's next nnpp_create allocates (cudaSetDevice). */
nnpp_status nnpp_set_device(int device);

/* Fill nnpp_params from the reference's positional control vectors: data2 (51 values,
 * utils.h:2343-2395), datac1..datac4 (7 values each, utils.h:2397-2423) and datac11
 * (4 values, utils.h:2480-2483).  k_diss and switch_width have no counterpart in the
 * reference's data files.  Replaces utils::parameter::set_double. */
nnpp_status nnpp_params_from_reference(const double* data2, const double* datac1,
                                       const double* datac2, const double* datac3,
                                       const double* datac4, const double* datac11,
                                       double k_diss, double switch_width, nnpp_params* out);

/* ---- neighbourhood build (grid.h:43-204) --------------------------------------------- */

/* Stateless drop-in for build_clouds_hash(max_node_no, r, dx, dy, dz, nodes, clouds,
 * cloud_lengths, max_cloud_length) (grid.h:43-44): the hash, index, corner and scan steps
 * run on the GPU.  clouds (N*max_node_no, column-major, -1 padded, self at column 0) and
 * cloud_lengths (N, self included) may each be NULL.  order_mode selects the within-cell
 * order (NNPP_ORDER_REFERENCE reproduces the reference bit for bit). */
nnpp_status nnpp_build_clouds_hash(int max_node_no, double r, double dx, double dy, double dz,
                                   int n_nodes, const double* nodes_colmajor, int order_mode,
                                   int* clouds_colmajor, int* cloud_lengths,
                                   int* max_cloud_length);

/* No counterpart in the reference.  For callers that cannot allocate device memory (a host
 * framework that owns every device allocation, a real-time loop that must not touch the
 * allocator, an application already at its memory cap): the canonical-order build
 * (NNPP_ORDER_CANONICAL) into caller-owned DEVICE buffers -- d_nodes_colmajor (3*N
 * doubles), d_clouds_colmajor (N*max_node_no ints, written -1 padded with self at column
 * 0) and d_cloud_lengths (N ints) -- on `stream` (a cudaStream_t; NULL for the legacy
 * default stream).  It calls no cudaMalloc/cudaFree: every temporary lives in one
 * fixed-size device array (about 6.3 MB) that each GPU loading this library holds until
 * the process exits.  N is limited to 262,144 nodes and the hash grid over the nodes'
 * bounding box (cells of dx x dy x dz) to 262,144 cells; larger inputs return
 * NNPP_ERR_INVALID.  Every call looks up that array's device address on the current device
 * (cudaGetSymbolAddress).  Calls share the array: calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.  The call
 * synchronises `stream` three times to read the bounding box, the grid size and the
 * capacity flag back to the host. */
nnpp_status nnpp_build_clouds_hash_noalloc(int max_node_no, double r, double dx, double dy,
                                           double dz, int n_nodes, const double* d_nodes_colmajor,
                                           int* d_clouds_colmajor, int* d_cloud_lengths,
                                           int* max_cloud_length, void* stream);

/* ---- the complete ten-species residual (utils.h:29-842) -------------------------------- */

/* The reference's complete residual, utils::Residuals (utils.h:29-842): the ten species
 * with their reactions (utils.h:162-174, 241-253, 321-330, 396-401, 466-476, 541-547,
 * 612-618, 683-690, including the interface's Butler-Volmer H+ source) and the potential, in
 * FP64.  Inputs as the reference holds them: nodes N x 3 column-major, clouds N x max_node_no
 * column-major (self in column 0, as build_clouds_hash fills them) with cloud_lengths,
 * U_n1 and U_n 11*N (fields 1..10 then the potential, field-major), phase N (1 solid), the
 * volume ratio voln1rel, and the parameter arrays of the reference's data files: data2 (51
 * values, the .data2 file), datac (10 x 7, the .datac1..datac10 files one after another) and
 * datac11 (4).  Writes F: 11*N (F1..F11).  (The reference's U^{n0} arguments are not read by
 * utils.h:29-842 and are not taken.)  Copies in and out of the device inside the call. */
nnpp_status nnpp_residuals_full(int n_nodes, const double* nodes_colmajor, const int* clouds_colmajor,
                                int max_node_no, const int* cloud_lengths, const double* U_n1,
                                const double* U_n, const int* phase, double voln1rel,
                                const double* data2, const double* datac, const double* datac11,
                                double* F);

/* The same on device arrays (clouds with N rows and at least the longest length in columns;
 * every index checked by the caller), launched on the given CUDA stream (NULL: the legacy
 * default stream); returns after the launch. */
nnpp_status nnpp_residuals_full_device(int n_nodes, const double* d_nodes, const int* d_clouds,
                                       const int* d_lengths, const double* d_U_n1,
                                       const double* d_U_n, const int* d_phase, double voln1rel,
                                       const double* data2, const double* datac,
                                       const double* datac11, double* d_F, void* stream);

/* ---- the complete model's implicit step (main.cpp:640-922) ------------------------------ */

/* The reference's time step with its complete model: ten species and the potential, backward
 * Euler with the tangents of utils::NewtonMatrices (utils.h:846-1849) at U^n and modified
 * Newton iterations on utils::Residuals (utils.h:29-842), each correction by Eigen's left-
 * Jacobi GMRES(30) (GMRES.h:56-203), the Dirichlet rows of main.cpp:676-712, the clamp of
 * main.cpp:805-837, the flip of main.cpp:914-922 and the relative volume every 8 steps
 * (main.cpp:944-949).  FP64 on the GPU in the reference's node order.  Created from the
 * reference's arrays: nodes N x 3 and clouds N x max_node_no column-major (self in column 0,
 * as build_clouds_hash fills them) with cloud_lengths, bctypes (N), bcvalues (11*N, the
 * .bc1..bc11 files field-major), data2 (51), datac (10 x 7), datac11 (4).  The bond weights are
 * beta dV / xi^3: every kernel exponent s must be 0 (NNPP_ERR_UNSUPPORTED otherwise). */
typedef struct nnpp_chem nnpp_chem;
nnpp_status nnpp_chem_create(nnpp_chem** out, int n_nodes, const double* nodes_colmajor,
                             const int* clouds_colmajor, int max_node_no, const int* cloud_lengths,
                             const int* bctypes, const double* bcvalues, const double* data2,
                             const double* datac, const double* datac11);
/* The state U (11*N: U1..U10 divided by CSolid, then the potential) and phases (1 solid);
 * voln1rel the relative volume for BV; vol0rel the run's initial volume (<= 0: formed from this
 * state as main.cpp:472-480 does at t = 0).  Steps are counted from here. */
nnpp_status nnpp_chem_set_state(nnpp_chem* c, const double* U, const int* phase, double voln1rel,
                                double vol0rel);
/* n_steps implicit steps; the Newton and GMRES iterations summed over them (may be NULL). */
nnpp_status nnpp_chem_step(nnpp_chem* c, int n_steps, int64_t* newton_iterations,
                           int64_t* krylov_iterations);
/* The state after the steps (any pointer may be NULL). */
nnpp_status nnpp_chem_get_state(nnpp_chem* c, double* U, int* phase, double* voln1rel);
void nnpp_chem_destroy(nnpp_chem* c);

/* ---- implant mask (main.cpp:316-325, 422-457) ------------------------------------------- */

/* The phase of every node from the implant's point cloud, as the reference sets it up when
 * it starts from a surface-mesh implant (BunnyConditions): counts[i] is the number of points
 * within r of node i -- inside the FP64 box node +- r (libkdtree++'s find_within_range) and
 * at Euclidean distance sqrt(x*x + y*y + z*z) <= r, kd_tree_interface.h:156-252 -- and
 * phase[i] = 1 (solid) where counts[i] > 0, else 0.  The reference calls it with
 * r = 3 * 0.4 * dx * (1 + 1e-5).  nodes and points are column-major (x[], y[], z[]) host
 * arrays; counts and phase may each be NULL.  NNPP_ERR_CAPACITY where a count exceeds
 * max_node_no (the reference's runtime_error of kd_tree_interface.h:213-216; the outputs are
 * still written). */
nnpp_status nnpp_implant_mask(int n_nodes, const double* nodes_colmajor, int n_points,
                              const double* points_colmajor, double r, int max_node_no,
                              int* counts, int* phase);

/* ---- simulation handle ---------------------------------------------------------------- */

/* Create a handle for N nodes.  bcvalues/icvalues hold (S+1)*N doubles in the reference's
 * file units: boundary values of the species are divided by CSolid (main.cpp:560-620,
 * 676-712), the potential's is not; initial values are used as given (main.cpp:398-409).
 * A node is Dirichlet for field f when bctypes[i] == 0 and bcvalues[f*N+i] != -1
 * (main.cpp:676-712).  phase0 may be NULL: then phase = (ic_Mg > 0 + 1e-5) as in
 * main.cpp:411-420. */
nnpp_status nnpp_create(nnpp_handle** out, const nnpp_params* p, int n_nodes,
                        const double* nodes_colmajor, const int* bctypes,
                        const double* bcvalues, const double* icvalues, const int* phase0);
nnpp_status nnpp_destroy(nnpp_handle* h);

/* Build the neighbour lists for this handle (main.cpp:304-305 calls the reference with
 * r = delta*(1+1e-5) and cells of 10*dx).  The optional outputs are as in
 * nnpp_build_clouds_hash. */
nnpp_status nnpp_build_neighbours(nnpp_handle* h, int max_node_no, double r, double cx,
                                  double cy, double cz, int order_mode, int* clouds_colmajor,
                                  int* cloud_lengths, int* max_cloud_length);

/* Neighbour lists in CSR form, reference order, self excluded: row_ptr[N+1], cols[nnz].
 * Call with cols == NULL to get nnz in *nnz_out first. */
nnpp_status nnpp_get_neighbours_csr(nnpp_handle* h, int* row_ptr, int* cols, int64_t* nnz_out);

/* Advance n_steps explicit steps on the device.  Each step: solve the potential from the
 * current concentrations (FP64 tolerance tol, relative 2-norm), then advance c, apply the
 * Dirichlet values and the positivity clamp, flip saturated solid nodes, update the
 * diagnostics.  The step sequence is captured once into a CUDA graph per precision. */
nnpp_status nnpp_forward(nnpp_handle* h, int n_steps, int precision);

/* The reference's own time integration (main.cpp:640-922) for n_steps steps from the
 * handle's state, in FP64: backward Euler with one tangent per step (utils::NewtonMatrices,
 * utils.h:844-1849) and modified Newton iterations -- the residual of utils::Residuals at the
 * iterate with the migration on the previous step's potential, Dirichlet rows U - bc, every
 * field's correction from K_f dU_f = -F_f by GMRES(30) with the diagonal preconditioner to
 * EPS = 1e-5 (Eigen::GMRES as main.cpp:714-779 calls it: initial guess the right-hand side,
 * at most MAX_ITER = 200 iterations), the positivity clamp, until the update norms change by
 * less than EPS (main.cpp:847-895) -- then the phase flip.  The five fields' Krylov solves run
 * together on the GPU (one pass over the bonds serves all five).  newton_iterations and
 * krylov_iterations (GMRES iterations summed over fields and steps) may be NULL.  The state,
 * flip steps and diagnostics continue as after nnpp_forward; the step is the reference's, so
 * it is stable at time steps far above the explicit limit. */
nnpp_status nnpp_forward_implicit(nnpp_handle* h, int n_steps, int64_t* newton_iterations,
                                  int64_t* krylov_iterations);

/* Return to the initial state of nnpp_build_neighbours (initial values, phase0, zeroed
 * counters and diagnostics, no flipped node), keeping the lists, solver settings and tuning.
 * The reference starts each run from its .icvalues files (main.cpp:398-420). */
nnpp_status nnpp_reset(nnpp_handle* h);

/* Replace the model parameters of a handle (diffusivities, rate constant, time step,
 * charges, constants) without rebuilding its neighbour lists, e.g. between the iterations of
 * a calibration loop.  The geometry fields (dx, dy, dz, delta, the kernel exponents) and
 * CSolid must equal the handle's, since the bond weights and the scaled Dirichlet values
 * depend on them (NNPP_ERR_INVALID otherwise).
 * Discards a recorded forward_ckpt run.  The reference fixes its utils::parameter object
 * once per run (main.cpp:224-230, from the .data2/.datac* files); this entry point lets one
 * handle serve many parameter sets. */
nnpp_status nnpp_set_params(nnpp_handle* h, const nnpp_params* p);

/* Solver settings: relative tolerance of the potential (default 1e-10), iteration cap of
 * the CG (default 2000), strict != 0 turns a capped solve into NNPP_ERR_CG_NO_CONVERGE. */
nnpp_status nnpp_set_solver(nnpp_handle* h, double tol, int max_iter, int strict);

/* Mixed-precision refinement of the potential solve (no counterpart in the reference, which
 * solves in FP64): each FP32 inner CG sweep reduces its residual by inner_rel (default 1e-4;
 * the last sweep stops at what the tolerance needs), at most max_outer sweeps (default 30). */
nnpp_status nnpp_set_refinement(nnpp_handle* h, double inner_rel, int max_outer);

/* Initial guess of each potential solve.  history 0: the previous potential (the
 * reference's warm start, main.cpp:764-779); 1 or 2: linear extrapolation 2 phi^n -
 * phi^{n-1}; 3..6 (default 6): the combination of the last `history` potentials and their
 * divided differences that minimises the energy-norm error (a Galerkin projection onto the
 * history, using the stored images A phi = b - r of earlier solves; no extra operator
 * application).  Only the iteration count depends on it: every solve still runs to the
 * solver tolerance.  Discards a recorded forward_ckpt run. */
nnpp_status nnpp_set_warm_start(nnpp_handle* h, int history);

/* Preconditioner of the potential CG (both precisions).  NNPP_PRECOND_TWO_LEVEL (the
 * default) adds to the Jacobi scaling a coarse space of aggregates of f x f x f hash bins (at
 * most 3000 aggregates): the Galerkin coarse operator P^T A P of the phases, inverted on the
 * GPU and applied as one dense product per iteration.  The mixed-precision inner CG of a
 * single-instance run is deflated by that space while the coarse operator matches the
 * phases, and adds the coarse correction to the Jacobi scaling otherwise (as the FP64 path
 * and ensembles do).  It is rebuilt when
 * the state is replaced (nnpp_set_state, nnpp_reset) and, when refresh_every > 0 (default
 * 64), after every refresh_every steps counted from then if a phase has changed; backward
 * replays the rebuilds of forward_ckpt.  In an ensemble every member applies its own
 * coarse correction (block diagonal).
 * Only the iteration count depends on it: every solve still runs to the solver tolerance.
 * A change discards a recorded forward_ckpt run.  The reference's solve of K11 is
 * diagonally preconditioned (Eigen::GMRES with DiagonalPreconditioner, main.cpp:764-766,
 * solved at main.cpp:779). */
nnpp_status nnpp_set_preconditioner(nnpp_handle* h, int kind, int refresh_every);
/* Current preconditioner, its number of coarse unknowns (0 for Jacobi), refresh period and
 * the number of coarse inverses computed so far; any pointer may be NULL. */
nnpp_status nnpp_get_preconditioner(nnpp_handle* h, int* kind, int* coarse_unknowns, int* refresh_every,
                                    int64_t* rebuilds);

/* Device-side checks of the handle's kernels: a combination of nnpp_check flags (0: none,
 * the default).  Runs with checks launch the checked build of the kernels that have one.  No
 * counterpart in the reference (whose only failure path is grid.h:187-189). */
nnpp_status nnpp_set_checks(nnpp_handle* h, int flags);

/* Rebuild statistics of the two-level preconditioner's coarse inverse: inverses computed
 * since the handle was built, of which warm-started (Newton-Schulz from the previous
 * inverse); rebuilds triggered by phase changes during runs and their summed duration in
 * milliseconds (host clock, the stream drained before and after: the time a run spends on
 * them); the Newton-Schulz steps of the last rebuild.  Any pointer may be NULL.  No
 * counterpart in the reference (measurement). */
nnpp_status nnpp_get_coarse_stats(nnpp_handle* h, int64_t* rebuilds, int64_t* warm_rebuilds,
                                  int64_t* run_rebuilds, double* run_rebuild_ms,
                                  int* last_ns_steps);

/* Copy the state to host buffers (user node order).  c: S*N, phi: N, phase: N; any may be
 * NULL. */
nnpp_status nnpp_get_state(nnpp_handle* h, double* c, double* phi, int* phase);
/* Overwrite the state from host buffers (user node order); phase may be NULL.  As after the
 * reference's restart from file (main.cpp:527-533), the relative volume voln1rel and the
 * interface factor BV are recomputed for the new state against the initial state's vol0rel;
 * the step counter and the initial Mg mass are kept. */
nnpp_status nnpp_set_state(nnpp_handle* h, const double* c, const double* phi,
                           const int* phase);
nnpp_status nnpp_get_diagnostics(nnpp_handle* h, nnpp_diag* out);
/* Per-node step of the last flip (-1 if never flipped), user order; N ints. */
nnpp_status nnpp_get_flip_steps(nnpp_handle* h, int* flip_step);

/* Host-buffer step, the call a host-side time loop makes: upload c (S*N) and phase (N),
 * run one step with the handle's potential (and its warm-start history) as the initial
 * guess of the potential solve, download c, phi and phase.  in and out buffers may alias. */
nnpp_status nnpp_step_host(nnpp_handle* h, int precision, const double* c_in,
                           const int* phase_in, double* c_out, double* phi_out,
                           int* phase_out);

/* Drop-in for utils::Residuals restricted to F1..F4 and F11 (utils.h:29-842) with
 * U^{n+1} = U^n: F[k*N+i] = sum_KRk1 + sum_KRk2 - R_k for the species, F[S*N+i] the
 * potential residual of utils.h:798-841 (0 on nodes without liquid-liquid bonds), with
 * R_k the dissolution source of species 0 (0 for the others).  c: S*N, phi: N, phase: N,
 * F: (S+1)*N, all user order.  voln1rel enters the BV factor. */
nnpp_status nnpp_residuals(nnpp_handle* h, int precision, const double* c, const double* phi,
                           const int* phase, double voln1rel, double* F);

/* Solve the potential for the given concentrations and phase (user order) into phi
 * (in: warm start, out: solution).  Returns the iteration count and FP64 relative
 * residual. */
nnpp_status nnpp_solve_potential(nnpp_handle* h, int precision, const double* c,
                                 const int* phase, double* phi, int* iterations,
                                 double* rel_residual);

/* ---- measurement (no counterpart in the reference) ------------------------------------ */

/* nnpp_forward, timed with CUDA events recorded on the handle's stream around the graph
 * launches (graphs are built before the first event). */
nnpp_status nnpp_forward_timed(nnpp_handle* h, int n_steps, int precision, double* ms);

/* Average duration of one launch of a single step kernel on the current state, CUDA-event
 * timed on the handle's stream over `reps` launches after 3 warm-up launches; the state is
 * restored afterwards.  kernel_id: 0 transport (bond sums), 1 CG matrix-vector product,
 * 2 FP64 refinement residual, 3 CG vector update; for one instance with the two-level
 * preconditioner the three kernels of 3 one by one: 4 restriction (with the additive form's
 * update), 5 coarse product, 6 z and the dots. */
nnpp_status nnpp_time_kernel(nnpp_handle* h, int kernel_id, int precision, int reps,
                             double* ms_per_launch);

/* The execution configuration of the handle's kernels: bins per tile, lanes per node of the
 * FP64 tile kernels, and the FP32 CG operator's variant: 0 / 3 gathers from L1/L2 (batches
 * of 16 bond columns; 0 keeps the next batch's stream in flight), 1 operator and slice windows streamed by bulk copies into shared
 * memory, 2 / 4 slice windows copied into shared memory by asynchronous copies (batches of
 * 8 / 16), 5 / 6 / 7 the variants 4 / 3 / 2 with bulk L2 prefetches of the operator stream
 * a few batches ahead, 8 the tile's halo (positions and the CG vector) staged in shared
 * memory, rows and columns restricted to the nodes without a Dirichlet value of the
 * potential, 2-byte neighbour codes streamed and the bond weights recomputed from the
 * positions.  Chosen by the autotuner on the first run (0 / -1 before); nnpp_set_tuning pins
 * a configuration instead (bins in {2,4,8,16}, lanes in {4,8,16}, operator 0..8;
 * NNPP_ERR_UNSUPPORTED when a tile halo, a slice window or a tile's code block does not fit,
 * or, for operator 8, the kernel exponent s is not 0 or the tiles are longer than 8 bins). */
nnpp_status nnpp_get_tuning(nnpp_handle* h, int* bins_per_tile, int* lanes_per_node,
                            int* cg_operator);
nnpp_status nnpp_set_tuning(nnpp_handle* h, int bins_per_tile, int lanes_per_node,
                            int cg_operator);

/* The FP32 transport's form (no counterpart in the reference): 0 (the default, the faster on
 * a GB300) gathers the bonds' neighbour records from L1/L2; 1 stages each tile's halo
 * records in shared memory by bulk copies and gathers them there.  Both compute the same
 * sums in the same order (the same states bit for bit).  NNPP_ERR_UNSUPPORTED for 1 when a
 * tile halo exceeds a CTA's shared memory. */
nnpp_status nnpp_set_transport_variant(nnpp_handle* h, int variant);

/* ---- differentiation ------------------------------------------------------------------ */

/* Forward half of a forward/backward pair: from the handle's current state run n_steps
 * steps, sampling the cumulative Mg mass loss dV*sum_i(c_0,i(0) - c_0,i(t)) every
 * sample_every steps into mass_curve[n_steps/sample_every] (FP64), keeping a state
 * checkpoint every ckpt_every steps for the backward pass.  The handle's state is left at
 * the final step. */
nnpp_status nnpp_forward_ckpt(nnpp_handle* h, int n_steps, int precision, int ckpt_every,
                              int sample_every, double* mass_curve);

/* Storage of the recorded forward run.  0 (default): automatic, every step's FP64
 * snapshot (64 bytes per node and step) when they fit a quarter of the free device memory,
 * else as 1; 1: a state checkpoint every ckpt_every steps plus every step's solved potential
 * (8 bytes per node and step) when those fit a quarter of the free memory: backward
 * recomputes each segment's bond sums and updates from its checkpoint without re-solving the
 * potential (else as 3); 2: every step's snapshot, NNPP_ERR_NOMEM when they do not fit;
 * 3: checkpoints only, backward recomputes each segment's whole steps (the least memory).
 * The gradients do not depend on the mode (bit for bit).  Discards a recorded run. */
nnpp_status nnpp_set_adjoint_store(nnpp_handle* h, int mode);

/* Backward half: given dL/d(mass_curve) (same length), run the adjoint of the explicit step
 * backwards (recomputing each checkpoint segment when the run was recorded with
 * checkpoints), returning dL/dD_liquid[k] (the solid diffusivity D_solid[k] scales with
 * D_liquid[k]) and dL/dk_diss.  The handle's state is restored to the end of the forward
 * run. */
nnpp_status nnpp_backward(nnpp_handle* h, const double* dL_dmass, double* grad_D,
                          double* grad_k);

/* Relative tolerance of backward's adjoint potential solves (no counterpart in the
 * reference, which has no adjoint).  0 (default): a mixed-precision run solves to
 * max(tol, 1e-8) and an FP64 run to tol, tol being the forward's (nnpp_set_solver); the
 * mixed gradient's own error (FP32 adjoint bond sums, ~5e-7 relative on the calibration
 * workload) is far above what a 1e-8 adjoint solve adds (~2e-12).  The recomputed forward
 * steps always use the forward's tolerance. */
nnpp_status nnpp_set_adjoint_solver(nnpp_handle* h, double tol);

/* The last nnpp_backward's adjoint potential solves: their inner CG iterations, count and
 * refinement sweeps (any pointer may be NULL; the handle's diagnostics are those of the
 * forward run), and, when iterations_per_step is not NULL, each step's inner iterations
 * (n_steps of the recorded run, indexed by step). */
nnpp_status nnpp_get_adjoint_stats(nnpp_handle* h, int64_t* cg_iterations, int64_t* solves,
                                   int64_t* sweeps, int* iterations_per_step);

/* ---- ensembles -------------------------------------------------------------------------- */

typedef struct nnpp_ensemble nnpp_ensemble;

/* Group handles (each already built, on one device) into batched launches: each step of
 * every member -- of any size, with its own parameters, time step and solver iteration
 * count -- runs in one CUDA graph whose kernels walk work lists of tiles and node chunks
 * over all members (persistent grids); a member whose potential solve has converged drops
 * out of the loop while the others continue.  The bins per tile and lanes per node come
 * from the library's autotuner on the first run.  The members keep their own state and
 * can still be used alone; a handle may belong to one ensemble at a time. */
nnpp_status nnpp_ensemble_create(nnpp_ensemble** out, nnpp_handle* const* members, int n);
nnpp_status nnpp_ensemble_forward(nnpp_ensemble* e, int n_steps, int precision);
/* nnpp_ensemble_forward timed with CUDA events on the ensemble's stream (milliseconds). */
nnpp_status nnpp_ensemble_forward_timed(nnpp_ensemble* e, int n_steps, int precision,
                                        double* ms);
/* The autotuned configuration: bins per tile and lanes per node. */
nnpp_status nnpp_ensemble_tuning(nnpp_ensemble* e, int* bins_per_tile, int* lanes_per_node);
nnpp_status nnpp_ensemble_destroy(nnpp_ensemble* e);

/* ---- synthetic inputs --------------------------------------------------------------------- */

/* Deterministic synthetic workloads in the reference's input layout (no input data of the
 * reference's paper case is available).  kind: 0 lattice with a central solid block,
 * 1 jittered lattice with a perturbed solid sphere, 2 jittered permuted lattice with a
 * screw-shaped implant, 3 jittered lattice with a solid cylinder and an 8-node Dirichlet
 * shell, 4 ensemble member (seeded inclusion, diffusivities and rate).  n_side nodes per
 * axis.  nnpp_synth_count returns N. */
int64_t nnpp_synth_count(int kind, int n_side);
nnpp_status nnpp_synth_fill(int kind, int n_side, uint64_t seed, double* nodes_colmajor,
                            int* bctypes, double* bcvalues, double* icvalues, int* phase0,
                            nnpp_params* params);

#ifdef __cplusplus
}
#endif

#endif /* NNPP_GB300_H */
