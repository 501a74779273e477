/*
 * musg.h -- C ABI of the GB300-native µSpectre Newton-CG homogenization path.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes.  Every
 * function returns MUSG_OK (0) or an error code; the message of the last error of
 * the calling thread is available through musg_last_error().  Arrays passed in or
 * out are HOST memory in the reference's layouts unless the name says "_device":
 *
 *   - a strain/stress field ("vector" of nb_dof = nb_pixels*D*D doubles) is
 *     pixel-major (AoS); pixel p, tensor entry A(i,j) sits at p*D*D + i + D*j
 *     (Eigen column-major per pixel), pixels row-major with the last index fastest
 *     (src/common/ccoord_operations.hh:151-192 of the reference);
 *   - a tangent field holds D^4 doubles per pixel at (i+D*j) + D*D*(k+D*l)
 *     (src/common/T4_map_proxy.hh:84-105);
 *   - an FFT workspace holds nb_hermitian*nb_components complex values as
 *     interleaved (re, im) doubles, AoS, the last axis halved to n/2+1
 *     (src/fft/fftw_engine.cc:65-77).
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef MUSG_H
#define MUSG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; the C++ layer maps them back onto the reference exception types */
#define MUSG_OK 0
#define MUSG_ERR_RUNTIME 1     /* std::runtime_error                                */
#define MUSG_ERR_PROJECTION 2  /* ProjectionError (src/fft/projection_base.hh)      */
#define MUSG_ERR_SOLVER 3      /* SolverError (src/solver/solver_common.hh:80-83)   */
#define MUSG_ERR_CONVERGENCE 4 /* ConvergenceError (solver_common.hh:86-88)         */
#define MUSG_ERR_SHAPE 5       /* size/shape mismatch (std::runtime_error upstream) */
#define MUSG_ERR_CUDA 6        /* CUDA runtime failure                              */
#define MUSG_ERR_MEMORY 7      /* device allocation failed                          */
#define MUSG_ERR_ARGUMENT 8    /* invalid argument / handle                         */
#define MUSG_ERR_NONFINITE 9   /* NaN/Inf met by a device kernel                    */

/* Formulation (src/common/common.hh:149-153) */
#define MUSG_FINITE_STRAIN 0
#define MUSG_SMALL_STRAIN 1

/* cell / projection creation flags */
#define MUSG_FLAG_ALLOW_EVEN 1 /* lift the odd-grid guard: Ghat = 0 at Nyquist k-points */

/* precision of the inner CG solve */
#define MUSG_PRECISION_FP64 0  /* everything in FP64 (the reference method)          */
#define MUSG_PRECISION_MIXED 1 /* FP32 CG/FFT/projection/tangent, FP64 Newton level   */

/* material laws */
#define MUSG_LAW_LE1 1  /* MaterialLinearElastic1:  params (E, nu)               */
#define MUSG_LAW_LE2 2  /* MaterialLinearElastic2:  params (E, nu); per pixel D*D eigenstrain */
#define MUSG_LAW_LE3 3  /* MaterialLinearElastic3:  per pixel (E, nu), full C   */
#define MUSG_LAW_LE4 4  /* MaterialLinearElastic4:  per pixel (E, nu) -> (lambda, mu) */
#define MUSG_LAW_HEP1 5 /* MaterialHyperElastoPlastic1: params (E, nu, tau_y0, H[, mode]);
                           mode 0 the reference (projector logm, j-independent Kirchhoff->PK1
                           tangent), 1 spectral logm, 2 spectral logm with the consistent
                           tangent dP/dF and eps_p.cur = eps_p.old + dgamma (extensions) */
#define MUSG_LAW_GENERIC 6 /* MaterialLinearElasticGeneric: params the Voigt stiffness,
                              vsize x vsize row-major (vsize 3 in 2-D, 6 in 3-D) */

/* projection kinds */
#define MUSG_PROJ_SMALL_STRAIN 0       /* ProjectionSmallStrain       */
#define MUSG_PROJ_FINITE_STRAIN_FAST 1 /* ProjectionFiniteStrainFast  */
#define MUSG_PROJ_FINITE_STRAIN 2      /* ProjectionFiniteStrain      */

typedef struct musg_cell musg_cell;
typedef struct musg_solver musg_solver;
typedef struct musg_fft musg_fft;
typedef struct musg_projection musg_projection;
typedef struct musg_batch musg_batch;

/* OptimizeResult (src/solver/solver_common.hh:50-67) without its two field arrays,
 * which musg_newton_cg writes into caller buffers. */
typedef struct musg_result_info {
  int success;           /* OptimizeResult::success                    */
  int status;            /* OptimizeResult::status                     */
  unsigned nb_it;        /* Newton iterations of this load step        */
  unsigned nb_fev;       /* cumulative CG iterations (solver counter)  */
  char message[64];      /* OptimizeResult::message                    */
  double hom_stress[9];  /* pixel mean of the stress after the load step, D*D column-major
                            (no counterpart: the reference's callers average
                            OptimizeResult::stress themselves, solvers.cc:197) */
} musg_result_info;

/* -------------------------------------------------------------- library */
const char *musg_last_error(void);
int musg_version(void);
/* number of visible CUDA devices (0 without a GPU; never fails on a CPU host) */
int musg_device_count(int *count);
/* device used by the objects the calling thread creates afterwards (one process per
 * GPU; no counterpart in the reference, whose ranks are MPI processes) */
int musg_set_device(int device);
/* self-test of the bounded waits of the TMA-fed passes (no counterpart in the
 * reference): one block waits on an mbarrier that nothing completes, gives up after
 * limit_ms, and sets the device fault word; the host reads it the way it does after
 * every FP32 CG solve, clears it, and reports *timed_out = 1.  The device stays usable. */
int musg_selftest_wait_timeout(double limit_ms, int *timed_out);

/* -------------------------------------------------------------- cell
 * make_cell<D,D>(res, lengths, form) (src/cell/cell_factory.hh:93-105) and
 * CellBase<D,D> (src/cell/cell_base.hh:241-526).  The projection is chosen by the
 * formulation as upstream (cell_factory.hh:59-86): finite strain ->
 * ProjectionFiniteStrainFast, small strain -> ProjectionSmallStrain; both reject
 * even resolutions unless MUSG_FLAG_ALLOW_EVEN is given. */
int musg_cell_create(int dim, const int *resolutions, const double *lengths,
                     int formulation, int flags, musg_cell **out);
int musg_cell_destroy(musg_cell *cell);
/* Cell::get_nb_dof (cell_base.hh:115) and Cell::size (cell_base.hh:118) */
int musg_cell_sizes(musg_cell *cell, long long *nb_dof, long long *nb_pixels);
/* runs the cell's kernels on this CUDA stream (default: a stream the cell owns) */
int musg_cell_set_stream(musg_cell *cell, void *cuda_stream);
/* MaterialMuSpectre<...>::make(cell, name, params...) (material_muSpectre_base.hh:228-237) */
int musg_material_create(musg_cell *cell, int law, const char *name,
                         const double *params, int nb_params, int *material);
/* add_pixel for many pixels at once (material_base.cc / LE2-4 .cc add_pixel):
 * pixel indices are row-major linear indices; per_pixel holds stride values per
 * pixel (LE2: D*D eigenstrain column-major; LE3/LE4: Young, Poisson), else NULL. */
int musg_material_add_pixels(musg_cell *cell, int material,
                             const long long *pixels, long long count,
                             const double *per_pixel, int stride);
/* MaterialBase::size */
int musg_material_size(musg_cell *cell, int material, long long *count);
/* CellBase::initialise (cell_base.cc:445-454): material coverage check, device
 * upload of the microstructure, FFT plans.  Called implicitly by the first
 * evaluation. plan_flags follows FFT_PlanFlags (estimate=0, measure=1, patient=2). */
int musg_cell_initialise(musg_cell *cell, int plan_flags);
/* launch shapes of the spectral passes (threads per block, shared-memory target
 * per block) for FP64 then FP32, passes last-axis / middle-axis / Green: 6 entries
 * each.  FFT_PlanFlags measure/patient at initialise times candidates on the cell's
 * grid (the FFTW_MEASURE analogue); no counterpart in the reference. */
int musg_cell_tuning(musg_cell *cell, int *threads, long long *bytes);
/* CellBase::set_uniform_strain (cell_base.cc:110-112); strain is D*D column-major */
int musg_cell_set_uniform_strain(musg_cell *cell, const double *strain);
/* Cell::get_strain_vector / get_stress_vector (cell_base.cc:96-106): copies */
int musg_cell_get_strain(musg_cell *cell, double *out);
int musg_cell_set_strain(musg_cell *cell, const double *in);
int musg_cell_get_stress(musg_cell *cell, double *out);
/* Cell::evaluate_stress_tangent (cell_base.cc:129-146); either output may be NULL */
int musg_cell_evaluate_stress_tangent(musg_cell *cell, double *stress_out,
                                      double *tangent_out);
/* Cell::apply_projection (cell_base.cc:202-208): in place on a host vector */
int musg_cell_apply_projection(musg_cell *cell, double *vec);
/* homogenised stress: the pixel mean of the cell's stress field (D*D doubles,
 * column-major), the metric quantity; the reference forms it on the host from
 * OptimizeResult::stress (the idiom of solvers.cc:197).  Reduced on the device in a
 * fixed order, so it is identical for a cell however it was solved. */
int musg_cell_homogenised_stress(musg_cell *cell, double *out);
/* Cell::evaluate_projected_directional_stiffness (cell_base.cc:150-192) */
int musg_cell_directional_stiffness(musg_cell *cell, const double *dF, double *dP);
/* G(K:dF) through the kernels of one CG iteration (the operator SolverCG applies) in
 * the given precision (MUSG_PRECISION_FP64 or _MIXED = FP32 operator).  No reference
 * counterpart: it exposes the operator of the mixed-precision path for checking.
 * Needs an evaluated tangent; host arrays as in musg_cell_directional_stiffness. */
int musg_cell_cg_operator(musg_cell *cell, int precision, const double *dF, double *dP);
/* Cell::save_history_variables (cell_base.cc:458-462) */
int musg_cell_save_history_variables(musg_cell *cell);
/* CellBase::get_globalised_internal_real_array (cell_base.cc:370-436): the internal
 * field `name` of the materials that have it, zero at the other pixels; host array
 * of nb_components values per pixel (pixel-major).  Names as in the reference:
 * "Eigenstrain" (LE2), "local stiffness tensor" (LE3), "local first Lame constant",
 * "local second Lame constant(shear modulus)" (LE4), and the HEP1 state fields
 * "cumulated plastic flow εₚ, sub_field index k", "Previous placement gradient Fᵗ,
 * sub_field index k", "Previous left Cauchy-Green deformation bₑᵗ, sub_field index k"
 * (k = 0, 1; the current one alternates with save_history_variables).  out = NULL
 * returns nb_components only. */
int musg_cell_get_internal(musg_cell *cell, const char *name, double *out, long long capacity,
                           int *nb_components);
/* checkpoint / resume of a cell's device state at a load-step boundary (no
 * counterpart in the reference): strain and stress fields and the elasto-plastic
 * state with its current/old index, as one host image.  Loading needs a cell of the
 * same grid, formulation and material kinds (built the same way); its tangent is
 * re-evaluated by the next solve. */
int musg_cell_checkpoint_size(musg_cell *cell, unsigned long long *bytes);
int musg_cell_checkpoint_save(musg_cell *cell, void *buf, unsigned long long bytes);
int musg_cell_checkpoint_load(musg_cell *cell, const void *buf, unsigned long long bytes);

/* -------------------------------------------------------------- solvers
 * SolverCG(cell, tol, maxiter, verbose) (src/solver/solver_cg.hh:51-106) with the
 * vectors resident on the device; precision selects the plain FP64 method or the
 * mixed FP32-inner / FP64-outer variant. */
int musg_solver_cg_create(musg_cell *cell, double tol, unsigned maxiter,
                          int verbose, int precision, musg_solver **out);
int musg_solver_destroy(musg_solver *solver);
/* MUSG_PRECISION_MIXED only (no counterpart in the reference): the FP32 inner
 * solve stops at max(tol, inner_tol), default 1e-2 (the forcing term of an inexact
 * Newton method), and newton_cg refines in FP64 */
int musg_solver_set_inner_tol(musg_solver *solver, double inner_tol);
/* MUSG_PRECISION_MIXED only (no counterpart in the reference; on by default): newton_cg
 * projects the first residual G(-P) of a load step in FP64 and every later one as
 * G(rhs_prev - (P - P_prev)) in FP32, the previous residual minus the stress change
 * since (one FP64 projection per load step instead of one per Newton iteration).
 * enable = 0 projects every residual in FP64. */
int musg_solver_set_incremental_residual(musg_solver *solver, int enable);
/* newton_cg with a backtracking line search (no counterpart in the reference; off by
 * default): every Newton increment dF is applied as F0 + lam dF with lam = 1, 1/2, ...
 * until the norm of the projected residual G(-P) falls below (1 - 1e-4 lam) of the
 * current one, or lam = 1/1024; the convergence test still measures |dF|, and a load
 * step takes at most min(maxiter, 100) Newton iterations.  It lets the consistent
 * elasto-plastic tangent (HEP1 mode 2) converge on heterogeneous cells. */
int musg_solver_set_line_search(musg_solver *solver, int enable);
/* Cancellation of a running solve (no counterpart in the reference): flag points to
 * a host int that another thread may set; while it is nonzero, SolverCG::solve,
 * newton_cg and de_geus stop at their next check (after each replay of 16 CG
 * iterations, before each Newton iteration) with MUSG_ERR_RUNTIME "cancelled while
 * running".  NULL removes the flag; the int must outlive the solves that read it. */
int musg_solver_set_stop_flag(musg_solver *solver, const int *flag);
/* SolverBase::get_counter / reset_counter / has_converged (solver_base.hh:62-109) */
int musg_solver_get_counter(musg_solver *solver, unsigned *counter);
int musg_solver_reset_counter(musg_solver *solver);
int musg_solver_has_converged(musg_solver *solver, int *converged);
/* SolverCG::solve (solver_cg.cc:54-110): x_out = A^-1 rhs */
int musg_solver_solve(musg_solver *solver, const double *rhs, double *x_out);

/* newton_cg(cell, load_steps, solver, newton_tol, equil_tol, verbose)
 * (src/solver/solvers.cc:44-217).  load_steps: nb_steps D*D column-major
 * matrices.  grads / stresses (may be NULL) receive nb_steps*nb_dof doubles. */
int musg_newton_cg(musg_cell *cell, const double *load_steps, int nb_steps,
                   musg_solver *solver, double newton_tol, double equil_tol,
                   int verbose, musg_result_info *infos, double *grads,
                   double *stresses);

/* de_geus(cell, load_steps, solver, newton_tol, equil_tol, verbose)
 * (src/solver/solvers.cc:220-408): per load step, the first Newton iteration solves
 * for the response to the macroscopic increment at the previous equilibrium
 * (rhs = -G(K:DF)); arguments and outputs as musg_newton_cg. */
int musg_de_geus(musg_cell *cell, const double *load_steps, int nb_steps,
                 musg_solver *solver, double newton_tol, double equil_tol,
                 int verbose, musg_result_info *infos, double *grads,
                 double *stresses);

/* -------------------------------------------------------------- batches
 * Many cells (RVEs, or right-hand sides on copies of one microstructure) solved
 * together: newton_cg's Newton steps run in lockstep per cell and every CG iteration
 * is one launch per pass for all cells (replayed from one CUDA graph).  No
 * counterpart in the reference, which solves one cell at a time.  Cells of one grid
 * run the solo solve's kernels (results equal those of musg_newton_cg on each cell
 * alone, bit for bit); cells of different grids (same dimension, formulation and
 * material-law kind) run grouped launches of the generic pass kernels, each cell
 * owning a range of blocks and its own plans (results equal to the solo ones within
 * rounding).  load_steps: nb_cells x nb_steps D*D column-major matrices; infos:
 * nb_cells x nb_steps records; stresses (may be NULL): for each cell in turn,
 * nb_steps x its nb_dof.  A cell whose CG fails is reported (success 0, the
 * ConvergenceError message) and leaves the batch. */
int musg_batch_create(musg_cell **cells, int nb_cells, double tol, unsigned maxiter,
                      int precision, musg_batch **out);
int musg_batch_destroy(musg_batch *batch);
int musg_batch_set_inner_tol(musg_batch *batch, double inner_tol);
/* musg_solver_set_stop_flag for a batch: checked after each graph replay and before
 * each lockstep Newton iteration; the whole batch stops */
int musg_batch_set_stop_flag(musg_batch *batch, const int *flag);
int musg_batch_newton_cg(musg_batch *batch, const double *load_steps, int nb_steps,
                         double newton_tol, double equil_tol, musg_result_info *infos,
                         double *stresses);

/* ---------------------------------------------------------- serving
 * A continuous-batching request server (no counterpart in the reference, which
 * solves one cell per process).  Requests are admitted while their estimated device
 * footprint (musg_request_bytes) fits the HBM budget next to the requests already
 * running; waiting requests of the same kind (dimension, formulation, material-law
 * kind, number of load steps; grids within a factor 8 in pixels) are taken together
 * and solved as one batch (musg_batch_*: one launch per CG pass, grouped over
 * different grids).  Each lane is a host thread with its own CUDA stream, so admitted
 * work overlaps on the device; a request's fields and plastic state stay on the
 * device for all its load steps and return to the budget when it completes.  A
 * request batched with requests of its own grid gets the kernels of its solo solve in
 * the same order (the same result bit for bit); batched with other grids it runs the
 * generic pass kernels (the same result within rounding). */
typedef struct musg_server musg_server;

/* one request; the server copies everything at submission */
typedef struct musg_request {
  int dim;                    /* 2 or 3                                              */
  int resolutions[3];
  double lengths[3];
  int formulation;            /* MUSG_FINITE_STRAIN / MUSG_SMALL_STRAIN               */
  int flags;                  /* MUSG_FLAG_*                                          */
  int nb_materials;           /* <= 256                                               */
  const int *laws;            /* nb_materials MUSG_LAW_*                              */
  const double *params;       /* nb_materials x 5: the law's parameters (E, nu[, tau_y0, H, logm mode]) */
  const unsigned char *phase; /* material index of every pixel (row-major)            */
  const double *per_pixel;    /* LE3/LE4: (E, nu); LE2: D*D eigenstrain (column-major); NULL if unused */
  int per_pixel_stride;       /* doubles per pixel in per_pixel                        */
  int nb_steps;
  const double *load_steps;   /* nb_steps D*D column-major macroscopic increments     */
} musg_request;

typedef struct musg_server_result {
  long long id;
  int success;                /* every load step converged                           */
  int nb_steps_done;
  unsigned nb_it;             /* Newton iterations of the last load step             */
  unsigned nb_fev;            /* CG iterations of the last load step                 */
  double stress[9];           /* homogenised stress after the last step (column-major), at
                                 the returned strain (elasto-plastic: the last evaluation) */
  double latency_s;           /* completion - submission                             */
  double service_s;           /* completion - admission (0 if never admitted)        */
  int batched_with;           /* requests of the batch it was solved in              */
  char message[64];
} musg_server_result;

typedef struct musg_server_stats {
  long long submitted, completed, batches;
  unsigned long long budget, in_use, peak_in_use;
  long long queued;  /* submitted, not yet admitted */
} musg_server_stats;

/* device bytes a request holds while it runs (fields, spectra, tangent data, CG
 * vectors, state), for the precision it runs in */
int musg_request_bytes(const musg_request *req, int precision, unsigned long long *bytes);
/* lanes = 0 starts no thread and touches no GPU: musg_server_admit / _release then
 * step the admission by hand (host-side checks of the policy) */
int musg_server_create(unsigned long long hbm_budget, int lanes, int max_batch, int precision,
                       double tol, unsigned maxiter, double newton_tol, musg_server **out);
int musg_server_submit(musg_server *srv, const musg_request *req, long long *id);
/* no more submissions; lanes finish the queue and exit */
int musg_server_close(musg_server *srv);
/* drops the requests still waiting for admission: each completes at once, unsolved,
 * with the message "cancelled before admission" (a deadline on a stream); running
 * groups finish.  *cancelled (may be NULL) receives their number. */
int musg_server_cancel_waiting(musg_server *srv, long long *cancelled);
/* asks every running group to stop: each ends at its next check (after a replay of 16
 * CG iterations, before a Newton iteration) and completes, unsolved, with the message
 * "cancelled while running".  *groups (may be NULL) receives the number signalled. */
int musg_server_cancel_running(musg_server *srv, long long *groups);
/* result of request id, waiting at most timeout_s seconds (MUSG_ERR_RUNTIME when it
 * is not done by then); a result can be fetched once */
int musg_server_wait(musg_server *srv, long long id, double timeout_s, musg_server_result *out);
int musg_server_get_stats(musg_server *srv, musg_server_stats *out);
/* closes the server and joins its lanes */
int musg_server_destroy(musg_server *srv);
/* the admission step of a lane: the oldest waiting request that fits the budget next
 * to the running ones and the waiting requests of its kind that fit too, at most cap
 * (a request with the consistent elasto-plastic tangent, solved with the line search,
 * is taken alone); their ids, count and bytes (now counted as in use).  A request
 * larger than the whole budget is refused by musg_server_submit (MUSG_ERR_MEMORY). */
int musg_server_admit(musg_server *srv, long long *ids, int cap, int *count, unsigned long long *bytes);
/* returns bytes of a finished group to the budget */
int musg_server_release(musg_server *srv, unsigned long long bytes);

/* ---------------------------------------------------------- instrumentation
 * (no counterpart in the reference, which has no device)
 * musg_launch_count: kernels launched by the library in this process, CUDA graph
 *   replays counted per kernel node.
 * musg_solver_profile: mean duration (ms, CUDA events on the cell's stream) of each
 *   kernel of one CG iteration over `iterations` eager iterations started from the
 *   cell's last projected residual; ms_out needs 8 entries; kernel names by
 *   musg_solver_kernel_name.  Needs an evaluated tangent (after newton_cg). */
int musg_launch_count(unsigned long long *count);
/* measured FP64 FMA throughput of the current device in TFLOP/s (a probe kernel of
 * independent fused multiply-add chains on every SM, best of three timed launches):
 * the bound of the FP64 passes, whose arithmetic intensity is about 1 flop/byte */
int musg_probe_fp64_fma(double *tflops);
int musg_solver_profile(musg_solver *solver, int iterations, double *ms_out, int *nb_kernels);
const char *musg_solver_kernel_name(musg_solver *solver, int k);

/* -------------------------------------------------------------- FFT engine
 * FFTEngineBase<D> / FFTWEngine<D> (src/fft/fft_engine_base.hh:75-148,
 * fftw_engine.cc:53-158): unnormalised r2c / c2r over nb_components interleaved
 * components.  normalisation() is 1/nb_pixels. */
int musg_fft_create(int dim, const int *resolutions, int nb_components, musg_fft **out);
int musg_fft_destroy(musg_fft *fft);
int musg_fft_forward(musg_fft *fft, const double *in, double *out_complex);
int musg_fft_inverse(musg_fft *fft, const double *in_complex, double *out);

/* -------------------------------------------------------------- projections
 * ProjectionSmallStrain / ProjectionFiniteStrainFast / ProjectionFiniteStrain
 * (src/fft/projection_*.cc; ProjectionBase projection_base.hh:99-161) */
int musg_projection_create(int dim, const int *resolutions, const double *lengths,
                           int kind, int flags, musg_projection **out);
int musg_projection_destroy(musg_projection *proj);
int musg_projection_apply(musg_projection *proj, double *vec);
/* Allocation-free variant of musg_projection_apply, for callers that cannot
 * allocate device memory (a caller-owned pool or arena that forbids cudaMalloc,
 * allocation-free real-time loops).  No counterpart in the reference.  in_device /
 * out_device are caller DEVICE buffers of nb_dof doubles in the reference layout
 * (may be the same buffer); the work is enqueued on cuda_stream and the call
 * returns before it finishes.  All temporaries live in one 64 MiB file-scope device
 * array that every GPU loading the library holds until exit; grids that do not fit
 * are rejected with MUSG_ERR_ARGUMENT.  The first call on a device looks the
 * array's address up, so make it before any stream capture; under CUDA's lazy
 * module loading it is also the point where the 64 MiB may be committed, so a
 * caller that hands the rest of the device to a pool makes one call first (or sets
 * CUDA_MODULE_LOADING=EAGER).  Calls share the array: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int musg_projection_apply_noalloc(int dim, const int *resolutions, const double *lengths,
                                  int kind, int flags, const double *in_device,
                                  double *out_device, void *cuda_stream);
/* get_operator(): rows x nb_hermitian doubles, column-major as the reference
 * stores Ghat (rows = D^4 for small/full finite strain, D for the fast variant);
 * out may be NULL to query rows/cols */
int musg_projection_get_operator(musg_projection *proj, double *out,
                                 long long *rows, long long *cols);

#ifdef __cplusplus
}
#endif
#endif /* MUSG_H */
