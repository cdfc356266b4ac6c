/*
 * collops.h -- C ABI of the GB300 (sm_103a) collision-operator library.
 *
 * Drop-in for the hot-loop hooks of CollisionOperators.jl: each entry point
 * replaces one Julia routine that solver.jl reaches through COLLISION_FN,
 * COLLMETRIC_FN, L2PROJ_FN, COMPG_FN or LOGGRAD_FN (solver.jl:30-34), plus the
 * CPU stages between them (quadrature, mass solve) and the whole implicit step.
 *
 * Conventions
 *  - Marker arrays are the reference's Julia Matrix{Float64} N x 2 in
 *    column-major order: v[0..N-1] = v1, v[N..2N-1] = v2. G, g, dot_v likewise;
 *    A is N x 3 (A11, A12, A22 columns). w is a length-N vector.
 *  - Coefficient vectors (f_coeffs, r, L) have length n_dofs =
 *    (n_el1 + 2)(n_el2 + 2), index i1 + i2*(n_el1 + 2) (first dimension fastest,
 *    MantisWrappers.jl:136 and projection_gpu.jl:66, 0-based here).
 *  - Plain entry points take HOST pointers; the library copies in and out on
 *    its own stream and returns after the result is on the host. The *_dev
 *    variants take device pointers and leave results in device memory.
 *  - Every entry point returns an int status: CO_OK or a CO_ERR_* code. The
 *    library never falls back to a CPU path.
 *  - One context per mesh and device; calls on a context must not overlap
 *    (the reference never calls a hook concurrently).
 */
#ifndef COLLOPS_H
#define COLLOPS_H
#ifdef __cplusplus
extern "C" {
#endif

#define CO_ABI_VERSION 1

#define CO_OK 0
#define CO_ERR_ARG 1          /* bad argument (NULL, N < 0, sizes)             */
#define CO_ERR_CUDA 2         /* a CUDA runtime call failed                    */
#define CO_ERR_UNSUPPORTED 3  /* e.g. P_DEG != 2 (enable_gpu! keeps the CPU)   */
#define CO_ERR_NONFINITE 4    /* NaN/Inf in the inputs or in a residual        */
#define CO_ERR_TIMEOUT 5      /* a bounded device-side wait gave up            */
#define CO_ERR_NOMEM 6        /* device allocation failed                      */
#define CO_ERR_NODEVICE 7     /* no CUDA device visible                        */
#define CO_ERR_SIZE 8         /* N beyond the fixed scratch of co_collision_noalloc */

/* context flags */
#define CO_FLAG_LOGSQ 1u      /* use_logsq (Parameters.jl:63; functions.jl:9)  */
#define CO_FLAG_FP32_PAIR 2u  /* gpu_fp32 (Parameters.jl:133): co_collision
                                 runs the mixed FP32 pair sum                  */
#define CO_FLAG_ONESIDED 4u   /* evaluate every ordered pair (no Newton's-third-
                                 law symmetric kernels); for comparison runs   */

/* model */
#define CO_MODEL_LANDAU 0
#define CO_MODEL_LB 1

/* precision of the implicit solve */
#define CO_PREC_FP64 0        /* plain FP64 form                                */
#define CO_PREC_MIXED 1       /* FP32 pair maps, FP64 exit Picard map           */
#define CO_PREC_MIXED_DS 2    /* FP32 pair maps, then double-single pair maps
                                 (FP32 head+tail arithmetic, ~44 bits) for the
                                 FP64 stage; a single map at this precision is
                                 a double-single map                            */

typedef struct co_ctx co_ctx;

/* Solver options: the SimParameters fields step_anderson! reads
 * (Parameters.jl:50-106, solver.jl:305-312), plus the precision form. */
typedef struct {
    int model;               /* CO_MODEL_LANDAU / CO_MODEL_LB (collision_model) */
    double nu;               /* LB collision frequency                          */
    int use_gonzalez;
    int use_anderson;
    int exit_picard_step;
    int m;                   /* Anderson depth, 1..8                            */
    int max_iter;
    double tol;
    double abs_floor;
    int stag_window;
    double stag_rel_tol;
    int damp_decay_start;
    double damp_decay_factor;
    double restart_factor;   /* <= 0 means Inf                                  */
    double damping;
    double reg_factor;
    int precision;           /* CO_PREC_FP64, CO_PREC_MIXED or CO_PREC_MIXED_DS */
    double mixed_floor;      /* mixed form: absolute residual floor of the FP32
                                phase; <= 0 selects the default                 */
} co_opts;

/* Library version (CO_ABI_VERSION). */
int co_version(void);
/* Human-readable status text. */
const char *co_strerror(int status);

/* Workspace creation: replaces build_workspace (MantisWrappers.jl:90-158) for
 * the device side -- breakpoints, P_DEG=2 C1 B-spline tables, 1D mass-matrix
 * inverses, N_QUAD Gauss-Legendre rule. p_deg != 2 -> CO_ERR_UNSUPPORTED (the
 * reference keeps the CPU projection then, main.jl:396-404). */
int co_ctx_create(const double *bp1, int nb1, const double *bp2, int nb2,
                  int p_deg, int n_quad, unsigned flags, int device, co_ctx **out);
int co_ctx_destroy(co_ctx *ctx);
/* n_dofs of the context's space. */
int co_ctx_n_dofs(const co_ctx *ctx, int *n_dofs);

/* COLLISION_FN: compute_collision! (functions.jl:205-237),
 * compute_collision_gpu! / compute_collision_gpu32! (collision_gpu.jl:233-280). */
int co_collision(co_ctx *ctx, const double *v, const double *w, const double *G,
                 double *dot_v, int N);

/* COLLMETRIC_FN: compute_collision_metric! (functions.jl:249-290),
 * compute_collision_metric_gpu! (collision_gpu.jl:377-402). A is N x 3. */
int co_collision_metric(co_ctx *ctx, const double *v, const double *w,
                        const double *G, double *dot_v, double *A, int N);

/* L2PROJ_FN: l2_project! (functions.jl:121-134), l2_project_gpu!
 * (projection_gpu.jl:213-226); includes the mass solve, deterministic. */
int co_l2_project(co_ctx *ctx, const double *v, const double *w,
                  double *f_coeffs, int N);

/* COMPG_FN: compute_G! (functions.jl:182-202), compute_G_gpu!
 * (projection_gpu.jl:228-246). */
int co_grad_L(co_ctx *ctx, const double *v, const double *L, double *G, int N);

/* LOGGRAD_FN: eval_loggrad_at_particles! (functions.jl:37-64),
 * eval_loggrad_gpu! (projection_gpu.jl:251-269). */
int co_loggrad(co_ctx *ctx, const double *v, const double *f_coeffs, double *g,
               int N);

/* compute_r! (functions.jl:158-179): CPU-only in the reference. */
int co_compute_r(co_ctx *ctx, const double *f_coeffs, double *r);

/* compute_entropy (functions.jl:137-155): CPU-only in the reference. */
int co_entropy(co_ctx *ctx, const double *f_coeffs, double *S);

/* ldiv!(out, ws.M_lu, rhs) (solver.jl:67; projection_gpu.jl:224). */
int co_mass_solve(co_ctx *ctx, const double *rhs, double *out);

/* picard_map! (solver.jl:176-227), Landau or LB per opts->model. */
int co_picard_map(co_ctx *ctx, const co_opts *opts, double *v_out,
                  const double *v_in, const double *v0, const double *w, int N,
                  double S0, double dt);

/* step_anderson! (solver.jl:300-423) entirely on the device; v1 is the initial
 * guess in and the solution out. Outputs mirror its return tuple
 * (iterations, residual, n_restarts, initial residual). */
int co_step_anderson(co_ctx *ctx, const co_opts *opts, double *v1,
                     const double *v0, const double *w, int N, double S0,
                     double dt, int *iters, double *res, int *n_restarts,
                     double *r0);

/* Same with device pointers (inputs resident in HBM). */
int co_step_anderson_dev(co_ctx *ctx, const co_opts *opts, double *v1,
                         const double *v0, const double *w, int N, double S0,
                         double dt, int *iters, double *res, int *n_restarts,
                         double *r0);

/* Options of step_defect! (solver.jl:569-576) beyond co_opts: the inner
 * tolerance factor eta, the inner-map cap and the outer stagnation window
 * (SimParameters dc_eta, dc_max_inner, dc_stag_window; Parameters.jl:89-91),
 * and, for CO_PREC_MIXED, the FP32-stage stall ratio: FP32 outer maps run
 * while each outer residual is below fp32_stall times the previous one
 * (<= 0 selects 0.5), then FP64 outer maps take over. */
typedef struct {
    double eta;
    int max_inner;
    int stag_window;
    double fp32_stall;
    int metric64;   /* 1: the frozen metric A comes from the FP64 F+A pair kernel
                       (COLLMETRIC_FN, the reference's path); 0: F from the
                       Newton's-third-law kernel and A from an FP32 kernel (A
                       only shapes the inner model, not the fixed point)      */
    int outer_m;    /* 0: the reference's outer iteration v_{k+1} = D(v_k), D the
                       inner solution; 1..8: Anderson mixing of depth outer_m
                       over the outer iterates (D's fixed points are G's, and
                       the stopping rule stays on ||G(v) - v||). The window
                       restarts when the precision stage changes and when the
                       outer residual exceeds twice its best.                  */
    int precond;    /* 0: the reference's inner iteration (Anderson on the frozen
                       map); 1: Anderson on u + P^{-1} (Phi(u) - u) with the
                       per-marker 2x2 block P = I + dt A (H/2 - (lambda/w) I),
                       H the Hessian of L at v_mid -- a Newton step for each
                       marker's locally stiff part; 2: the same with M = H/2
                       (no lambda/w term). The inner stopping test and the
                       fixed points are unchanged.                            */
    double metric_freeze; /* with metric64 = 0: the FP32 metric A is rebuilt at
                       outer map k only while ||r_{k-1}|| >= metric_freeze *
                       ||r_1|| (A only shapes the inner model, so near the
                       fixed point the last A serves); 0 rebuilds it at every
                       outer map, as the reference does                       */
    int fp32_window; /* mixed forms: 0 leaves the FP32 outer maps as soon as one
                       map cuts the residual by less than fp32_stall; W > 0
                       once W maps in a row brought no new best residual cut
                       by fp32_stall                                          */
    int cap_refresh; /* with metric64 = 0: 1 rebuilds the FP32 metric at the
                       outer map after an inner solve that hit max_inner, even
                       past metric_freeze; 0 (the reference) does not         */
    int cap_abort;   /* K > 0: leave through the stagnation exit (best
                       iterate) once K FP64-stage outer maps in a row ended in
                       an inner solve that hit max_inner without a new best
                       outer residual; 0 (the reference) waits for the
                       stagnation window                                      */
} co_defect_opts;

/* step_defect! (solver.jl:569-634): defect correction around a frozen
 * metric, Landau only. opts->m, damping, tol, abs_floor, max_iter (outer cap),
 * stag_rel_tol, use_gonzalez and precision apply. Outputs mirror its return
 * tuple (outer_iterations, residual, inner_iterations, initial_residual). */
int co_step_defect(co_ctx *ctx, const co_opts *opts, const co_defect_opts *dopts,
                   double *v1, const double *v0, const double *w, int N, double S0,
                   double dt, int *outer, double *res, int *inner, double *r0);
int co_step_defect_dev(co_ctx *ctx, const co_opts *opts, const co_defect_opts *dopts,
                       double *v1, const double *v0, const double *w, int N, double S0,
                       double dt, int *outer, double *res, int *inner, double *r0);

/* Options of step_newton! (solver.jl:460-486) beyond co_opts: the GMRES basis
 * size, the absolute finite-difference step of the Jacobian-vector products and
 * the cap of the Eisenstat-Walker forcing term (SimParameters nk_krylov_max,
 * nk_fd_h, nk_eta_max; Parameters.jl:92-103). */
typedef struct {
    int krylov_max;      /* 1..200 Arnoldi vectors (2N doubles each, in HBM) */
    double fd_h;         /* > 0, e.g. 1e-6 for FP64 maps                   */
    double eta_max;      /* in (0, 1), e.g. 0.9                              */
} co_newton_opts;

/* step_newton! (solver.jl:460-486) with newton_krylov! and gmres!
 * (newton_krylov.jl:74-303) on the device: inexact Newton on F(v) = v - G(v),
 * matrix-free GMRES (modified Gram-Schmidt), Armijo backtracking; the maps run
 * in FP64, or in double-single pair sums for CO_PREC_MIXED_DS. opts->max_iter
 * caps the map evaluations; tol and abs_floor set the target and
 * exit_picard_step the exit update, as in the reference. Outputs mirror its
 * return tuple (evaluations, ||F||, Newton steps, ||F_0||) plus the status of
 * newton_krylov! (0 converged, 1 stalled, 2 budget). v1: guess in, solution out. */
int co_step_newton(co_ctx *ctx, const co_opts *opts, const co_newton_opts *nopts,
                   double *v1, const double *v0, const double *w, int N, double S0,
                   double dt, int *evals, double *res, int *n_newton, double *r0,
                   int *status);
int co_step_newton_dev(co_ctx *ctx, const co_opts *opts, const co_newton_opts *nopts,
                       double *v1, const double *v0, const double *w, int N, double S0,
                       double dt, int *evals, double *res, int *n_newton, double *r0,
                       int *status);

/* Explicit Euler predictor of the time loop (main.jl:233-245):
 * v1 = v + dt * vdot(v) with the model's right-hand side. */
int co_predictor(co_ctx *ctx, const co_opts *opts, double *v1, const double *v,
                 const double *w, int N, double dt);
int co_predictor_dev(co_ctx *ctx, const co_opts *opts, double *v1,
                     const double *v, const double *w, int N, double dt);

/* Post-step diagnostics of the time loop (main.jl:298-307): out6 (host) =
 * {entropy S of the projection of v, energy 1/2 sum w |v|^2, momentum P1, P2,
 * ||f_s - f_p||_2 with f_p the element-constant histogram density
 * (compute_fs_minus_fp_l2, functions.jl:315-347), the negative-part L1 norm of
 * f_s (compute_negative_part_l1, :300-313)}; Gauss grid of N_QUAD points per
 * direction. co_diagnostics takes host arrays, co_diagnostics_dev device ones. */
int co_diagnostics(co_ctx *ctx, const double *v, const double *w, int N, double *out6);
int co_diagnostics_dev(co_ctx *ctx, const double *v, const double *w, int N, double *out6);

/* Entropy of the projection of markers v (f_s(v) -> S), device pointers:
 * the S0 of the next step (main.jl:228, :298-300). */
int co_entropy_of_markers_dev(co_ctx *ctx, const double *v, const double *w,
                              int N, double *S);

/* COLLISION_FN for callers that cannot allocate device memory (no
 * counterpart in the reference). Some hosts own every byte of device memory
 * themselves -- a Julia process whose CUDA.jl pool manages the GPU, or an
 * application that must not allocate between time steps -- and cannot create
 * a co_ctx, which allocates. This entry point allocates nothing: v, w, G and
 * dot_v are DEVICE pointers in the reference's layout, (lo1, hi1) x (lo2, hi2)
 * is the domain (bp1[1], bp1[end]) x (bp2[1], bp2[end]), and its scratch is a
 * fixed 4 MiB __device__ array that every GPU loading the library keeps until
 * exit. N must be <= 32768 (else CO_ERR_SIZE). The first call on a device sets
 * up the array's address and should come before any stream capture. All calls
 * share the array: calls whose kernels overlap on the GPU race and must be
 * serialised by the caller. The inputs are first checked for NaN/Inf on the
 * GPU; the call waits for that check on `stream` (a cudaStream_t, NULL for the
 * default stream) and returns CO_ERR_NONFINITE, with dot_v untouched, if one
 * is found. The pair sum is then enqueued on `stream` and not synchronised.
 * FP64, one-sided pair loop. */
int co_collision_noalloc(const double *v, const double *w, const double *G,
                         double *dot_v, int N, double lo1, double hi1, double lo2,
                         double hi2, void *stream);

/* ---- batched form: many independent ensembles in one engine ----
 * (no counterpart in the reference, which runs one ensemble per process) */
typedef struct co_batch co_batch;
typedef struct {
    const double *bp1;   /* breakpoints of this instance's mesh */
    int nb1;
    const double *bp2;
    int nb2;
    int model;           /* CO_MODEL_LANDAU or CO_MODEL_LB */
    double nu;           /* LB collision frequency          */
    int N;               /* markers of this instance        */
} co_batch_instance;
int co_batch_create(const co_batch_instance *inst, int n, int n_quad, unsigned flags,
                    int device, co_batch **out);
int co_batch_destroy(co_batch *batch);
/* Autotune the batched pair kernel (tile width, tile-pair chunk, persistent
 * grid) by timing candidates on the current packed operands; the first
 * co_batch_step_dev does this by itself. */
int co_batch_tune(co_batch *batch, int *warps, int *chunk, int *grid, double *best_ms);
/* One implicit step (step_anderson!, FP64) of every instance. Concatenated
 * device arrays: instance i occupies v[2*off_i, 2*off_i + 2*N_i) (its own
 * N_i x 2 column-major block, off_i = sum of the N_j before it) and
 * w[off_i, off_i + N_i). S0[i], iters[i], res[i] are per instance (host).
 * use_graph != 0 captures one iteration of all instances as a CUDA graph and
 * replays it until every instance has exited. */
int co_batch_step_dev(co_batch *batch, const co_opts *opts, double *v1, const double *v0,
                      const double *w, const double *S0, double dt, int use_graph,
                      int *iters, double *res);
int co_batch_predictor_dev(co_batch *batch, const co_opts *opts, double *v1,
                           const double *v, const double *w, double dt);
int co_batch_entropy_dev(co_batch *batch, const double *v, const double *w, double *S);
int co_batch_launch_count(const co_batch *batch, unsigned long long *launches);

/* ---- learned warm start: a small MLP trained by this library's kernels ----
 * (the reference planned an NN warm start, Parameters.jl:108-117, but its
 * warmstart_nn.jl is not in the tree). Network n_in -> 64 -> 64 -> 64 -> n_out
 * with GELU, BF16 weights, FP32 accumulation; MSE loss; Adam. X, T, Y are
 * DEVICE row-major float arrays (B x n_in, B x n_out). */
typedef struct co_mlp co_mlp;
int co_mlp_create(int n_in, int n_out, unsigned seed, int device, co_mlp **out);
int co_mlp_destroy(co_mlp *mlp);
int co_mlp_num_params(const co_mlp *mlp, int *P);
/* FP32 master parameters (host arrays of P floats); the BF16 copy follows. */
int co_mlp_set_params(co_mlp *mlp, const float *host);
int co_mlp_get_params(const co_mlp *mlp, float *host);
int co_mlp_forward(co_mlp *mlp, const float *X, int B, float *Y, void *stream);
/* gradient of the loss w.r.t. every parameter (host array of P) and the loss */
int co_mlp_gradients(co_mlp *mlp, const float *X, const float *T, int B, float *grad,
                     float *loss);
int co_mlp_train_step(co_mlp *mlp, const float *X, const float *T, int B, float lr,
                      float *loss);
/* Per-marker features of the warm start at the start of a step (device
 * pointers): runs the explicit predictor, writing v_pred, and fills X (N x 15,
 * row-major FP32): vdot1, vdot2 (predictor velocity), G1, G2 (entropy
 * gradient), grad f_s / f_s (clamped as LOGGRAD_FN), log max(f_s, 1e-30), the
 * Hessian of L (H11, H12, H22), the FP32 pair metric A (A11, A12, A22; H and A
 * are 0 for LB), and the predictor's first residual (G(v_pred) - v_pred) / dt;
 * res_pred (may be NULL) receives ||G(v_pred) - v_pred||. The mixed forms run
 * the predictor and the residual map on the FP32 pair sum. S0 is the entropy of
 * v's projection (for the Gonzalez correction of the residual map). */
int co_warmstart_features_dev(co_ctx *ctx, const co_opts *opts, const double *v,
                              const double *w, int N, double S0, double dt, double *v_pred,
                              float *X, double *res_pred);
/* v1 = v_pred + dt^2 (Y * scale + shift) per component (device pointers). */
int co_warmstart_apply_dev(co_ctx *ctx, const double *v_pred, const float *Y, int N,
                           double dt, const double *scale2, const double *shift2,
                           double *v1);
/* ||G(v_in) - v_in|| of one Picard map (device pointers): FP64 pair sum for
 * CO_PREC_FP64, the FP32 pair sum for the mixed forms (a first-residual
 * comparison at the warm-start level). */
int co_picard_residual_dev(co_ctx *ctx, const co_opts *opts, const double *v_in,
                           const double *v0, const double *w, int N, double S0, double dt,
                           double *res);

/* Feature and output normalisation of the network, applied by co_mlp_forward
 * (inference only; training kernels take the data as given): inputs become
 * (x - x_mean) / x_std, outputs y * y_std + y_mean. Host arrays of n_in, n_in,
 * n_out, n_out values; x_mean = NULL removes the normalisation. */
int co_mlp_set_normalization(co_mlp *mlp, const double *x_mean, const double *x_std,
                             const double *y_mean, const double *y_std);

/* Record of one co_step_learned time step. */
typedef struct {
    int outer;            /* outer maps (defect) or iterations (Anderson), all attempts */
    int inner;            /* inner maps of the defect correction, all attempts          */
    double res;           /* residual of the kept solve (its best, if it stagnated)     */
    double r0;            /* initial residual of the kept solve                         */
    int converged;        /* the kept solve met max(tol ||v||, abs_floor)               */
    int exit;             /* 1 converged, 2 stagnation exit (solver.jl:357-367),
                             3 iteration cap (solver.jl:419-422)                        */
    int start;            /* start of the kept solve: 0 explicit predictor, 1 learned
                             proposal, 2 previous-step state                            */
    int attempts;         /* 2 when a non-converged solve was repeated from the next start */
    double r_start[3];    /* first residuals ||G(x) - x|| of the three starts (predictor,
                             learned, previous state; learned = +inf without a network) */
    double S_new;         /* entropy of the new state's projection: the next step's S0  */
} co_step_info;

/* One whole time step of the reference's loop (main.jl:233-271: predictor,
 * network correction nn_warmstart_correct! at :252-254, implicit solve) on the
 * device. Starts: the explicit predictor, the learned proposal v_pred + dt^2 *
 * mlp(features) (mlp carries its normalisation; NULL: no proposal) and the
 * previous-step state v. The solve (dopts != NULL: step_defect!, else
 * step_anderson!, in opts->precision) starts from the candidate with the
 * smallest first residual of the unmodified map (FP32 pair maps in the mixed
 * forms); with retry != 0 a solve that does not converge is repeated once from
 * the next candidate and the smaller residual is kept. v_new receives the new
 * markers, info the record. co_step_learned takes HOST arrays (copies in and
 * out inside the call); co_step_learned_dev device arrays. */
int co_step_learned(co_ctx *ctx, const co_opts *opts, const co_defect_opts *dopts,
                    co_mlp *mlp, int retry, double *v_new, const double *v,
                    const double *w, int N, double S0, double dt, co_step_info *info);
int co_step_learned_dev(co_ctx *ctx, const co_opts *opts, const co_defect_opts *dopts,
                        co_mlp *mlp, int retry, double *v_new, const double *v,
                        const double *w, int N, double S0, double dt, co_step_info *info);

/* Limits of the context's bounded device-side waits (no counterpart in the
 * reference, whose GPU code never waits on the device). The LB drift kernel
 * reduces its moments across the grid through a barrier that polls at most
 * `spins` times (about 64 ns each; <= 0 selects the default of 2^22) and then
 * gives up: the kernel finishes and the call returns CO_ERR_TIMEOUT, leaving
 * the context usable. `phantom_blocks` (0 in normal use) adds arrivals the
 * barrier waits for; a failure-path test sets 1, so that the barrier cannot
 * complete and the timeout path runs without any fault. */
int co_ctx_set_wait_limit(co_ctx *ctx, int spins, int phantom_blocks);

/* Number of kernels this context has launched so far. */
int co_launch_count(const co_ctx *ctx, unsigned long long *launches);

/* ---- measurement (no counterpart in the reference: its timing is host-side
 * wall time, main.jl:227, :295; scripts/check_metric_gpu.jl:39-42) ---- */

/* The context's CUDA stream (a cudaStream_t), for callers that time work
 * with their own events on the launching stream. */
int co_ctx_stream(const co_ctx *ctx, void **stream);

/* Per-kernel timing of the pair sums with CUDA events recorded around each
 * launch on the context's stream. */
typedef struct {
    double pair64_ms;                    /* summed event time, FP64 pair kernels */
    unsigned long long pair64_launches;
    double pair64_pairs;                 /* sum over launches of M (M - 1)      */
    double pair32_ms;                    /* same for the mixed FP32 kernel       */
    unsigned long long pair32_launches;
    double pair32_pairs;
    unsigned long long maps64, maps32;   /* Picard maps by pair precision       */
    double pairds_ms;                    /* double-single pair kernels           */
    unsigned long long pairds_launches;
    double pairds_pairs;
    unsigned long long mapsds;
} co_profile_t;
/* enable != 0 starts (and zeroes) the counters; 0 stops them. */
int co_profile(co_ctx *ctx, int enable);
int co_profile_read(co_ctx *ctx, co_profile_t *out);

/* Sustained FMA throughput of this GPU in FLOP/s (2 per FMA), measured by a
 * register-resident FFMA (fp64 = 0) or DFMA (fp64 = 1) chain kernel. */
int co_measure_fma_peak(int device, int fp64, double *flops_per_s);

#ifdef __cplusplus
}
#endif
#endif
