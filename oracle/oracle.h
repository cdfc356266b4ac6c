/*
 * oracle.h -- CPU FP64 restatement of the CollisionOperators.jl per-iteration
 * right-hand side. TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check
 * and the CPU-baseline leg of bench.py call this; the shipped library never does.
 *
 * Parity status: partially pinned. The reference is Julia (no julia binary here)
 * and its FEM layer is the un-vendored Mantis.jl 0.6.0, so no reference output
 * can be produced on this machine. The oracle is pinned by the reference's own
 * known-answer tests (test/integration/main_helpers.jl:13-61: momentum/energy,
 * compute_moments, LB drift conservation) and by exact identities of the method
 * (pair-sum conservation, L2-projection moment reproduction, the entropy chain
 * rule, the Gonzalez identity, mass-matrix row sums, Gaussian entropy
 * normalisation). Everything else is a line-by-line restatement of the cited
 * reference loops.
 *
 * Layout follows the reference (Julia column-major N x 2): v[0..N-1] = v1,
 * v[N..2N-1] = v2. Coefficient vectors are indexed i1 + i2*nd1 (0-based).
 */
#ifndef COLLOPS_ORACLE_H
#define COLLOPS_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_mesh om_mesh;

/* Workspace analogue (MantisWrappers.jl:90-158): breakpoints, P=2 C1 clamped
 * B-spline space, 3x3 GL mass matrix (banded Cholesky in place of sparse LU),
 * nquad x nquad GL rule for r and S. */
om_mesh *om_create(const double *bp1, int nb1, const double *bp2, int nb2,
                   int nquad, int use_logsq);
void om_destroy(om_mesh *m);
int om_n_dofs(const om_mesh *m);
int om_nd1(const om_mesh *m);

/* Dense 2D mass matrix (n_dofs x n_dofs, row-major) for small meshes (tests). */
void om_mass_matrix_dense(const om_mesh *m, double *out);
/* Extraction table of dimension d (1 or 2): n_el x 3 x 3, C[e][k][j]. */
void om_extraction(const om_mesh *m, int dim, double *out);
/* GL nodes/weights on [0,1] used for r and S. */
void om_quadrature(const om_mesh *m, double *x, double *w);

/* Mass-solve variant used by every later call: 0 = 2D banded Cholesky of the
 * assembled matrix (default); 1 = the tensor-product solve M^{-1} = M2^{-1} (x)
 * M1^{-1} with banded Cholesky factors of the 1D matrices. Both are correct FP64
 * solves; comparing results of the two measures how far FP64 round-off of the
 * solve alone moves a downstream quantity. */
void om_set_mass_solver(om_mesh *m, int kind);
/* ldiv!(out, M_lu, rhs)  (solver.jl:67) */
void om_mass_solve(const om_mesh *m, const double *rhs, double *out);
/* l2_project!  (functions.jl:121-134) */
void om_l2_project(const om_mesh *m, const double *v, const double *w, int N,
                   double *f_out);
/* scatter part of l2_project! only (rhs b, before the mass solve) */
void om_l2_rhs(const om_mesh *m, const double *v, const double *w, int N,
               double *b_out);
/* compute_r!  (functions.jl:158-179) */
void om_compute_r(const om_mesh *m, const double *f, double *r_out);
/* compute_entropy  (functions.jl:137-155) */
double om_entropy(const om_mesh *m, const double *f);
/* compute_G!  (functions.jl:182-202) */
void om_compute_G(const om_mesh *m, const double *v, int N, const double *L,
                  double *G_out);
/* eval_loggrad_at_particles!  (functions.jl:37-64) */
void om_loggrad(const om_mesh *m, const double *v, int N, const double *f,
                double *g_out);
/* value of f_s at one point (0 outside the domain) */
double om_eval_field(const om_mesh *m, const double *c, double x1, double x2);

/* compute_collision!  (functions.jl:205-237); nthreads<=0: all cores */
void om_collision(const om_mesh *m, const double *v, const double *w,
                  const double *G, int N, double *dot_v, int nthreads);
/* the same pair loop restricted to target rows rows[0..nrows-1]; writes
 * dot_v_rows[r] and dot_v_rows[nrows + r] (sampled CPU baseline) */
void om_collision_rows(const om_mesh *m, const double *v, const double *w,
                       const double *G, int N, const int *rows, int nrows,
                       double *dot_v_rows, int nthreads);
/* compute_collision_metric!  (functions.jl:249-290); A is N x 3 */
void om_collision_metric(const om_mesh *m, const double *v, const double *w,
                         const double *G, int N, double *dot_v, double *A,
                         int nthreads);

/* compute_moments (functions.jl:68-83): out = n, U1, U2, Q */
void om_moments(const double *v, const double *w, int N, double *out4);
/* compute_drift_multipliers (functions.jl:91-107): out = A1, A2, B */
void om_drift_multipliers(const double *v, const double *w, const double *g,
                          int N, double n, double U1, double U2, double Q,
                          double *out3);
/* compute_LB_velocity! (functions.jl:110-116) */
void om_lb_velocity(double *dot_v, const double *v, const double *g, int N,
                    double A1, double A2, double B, double nu);

/* Solver options mirroring SimParameters (Parameters.jl:50-106). */
typedef struct {
    int model;             /* 0 = :landau, 1 = :lb */
    double nu;
    int use_gonzalez;
    int use_anderson;
    int exit_picard_step;
    int m;                 /* Anderson depth */
    int max_iter;
    double tol;
    double abs_floor;
    int stag_window;
    double stag_rel_tol;
    int damp_decay_start;
    double damp_decay_factor;
    double restart_factor; /* <= 0 means Inf */
    double damping;
    double reg_factor;
    int nthreads;
} om_opts;

/* picard_map!  (solver.jl:176-227). Returns via v_out. */
void om_picard_map(const om_mesh *m, const om_opts *o, double *v_out,
                   const double *v_in, const double *v0, const double *w,
                   int N, double S0, double dt);
/* Post-step diagnostics (main.jl:298-307): out6 = S, energy, momentum (2),
 * ||f_s - f_p||_2 (histogram density), integral of max(-f_s, 0). */
void om_diagnostics(const om_mesh *m, const double *v, const double *w, int N, double *out6);
/* step_anderson!  (solver.jl:300-423). v1: initial guess in, solution out.
 * out4 = iterations, residual, n_restarts, initial residual. */
void om_step_anderson(const om_mesh *m, const om_opts *o, double *v1,
                      const double *v0, const double *w, int N, double S0,
                      double dt, double *out4);
/* Explicit Euler predictor of the time loop (main.jl:233-245):
 * v1 = v + dt * vdot(v); f_coeffs = l2 projection of v. */
void om_predictor(const om_mesh *m, const om_opts *o, double *v1,
                  const double *v, const double *w, int N, double dt);
/* Hessian (d11, d12, d22) of the spline field with coefficients Lv at markers
 * v (3N out: H11, H12, H22; 0 outside the domain). */
void om_hessian_L(const om_mesh *m, const double *v, int N, const double *Lv, double *H);
/* step_defect! (solver.jl:569-634); outer_m > 0 adds Anderson mixing of the
 * outer iterates and precond = 1 the block-Newton preconditioner of the inner
 * iteration (0, 0 = the reference's algorithm). v1: guess in, solution out.
 * out4 = outer iterations, residual, inner iterations, initial residual. */
void om_step_defect(const om_mesh *m, const om_opts *o, double eta, int max_inner,
                    int stag_window, int outer_m, int precond, double *v1, const double *v0,
                    const double *w, int N, double S0, double dt, double *out4);

/* step_newton! (solver.jl:460-486) with newton_krylov! and gmres!
 * (newton_krylov.jl:74-303): inexact Newton with matrix-free GMRES of at most
 * krylov_max vectors, forward-difference products with the absolute step fd_h,
 * Eisenstat-Walker forcing capped at eta_max, Armijo backtracking; o->max_iter
 * caps the map evaluations. out5 = evaluations, ||F||, Newton steps, ||F_0||,
 * status (0 converged, 1 stalled, 2 budget). */
void om_step_newton(const om_mesh *m, const om_opts *o, int krylov_max, double fd_h,
                    double eta_max, double *v1, const double *v0, const double *w, int N,
                    double S0, double dt, double *out5);

#ifdef __cplusplus
}
#endif
#endif
