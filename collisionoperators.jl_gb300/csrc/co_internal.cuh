// co_internal.cuh -- shared declarations of the collops GB300 library.
//
// One context (co_ctx) per (mesh, device): it owns the mesh tables in HBM, the
// marker-sized device buffers (reallocated only when N grows), one CUDA stream,
// and the device-side solver state. All kernels are hand-written for sm_103a;
// the host side only sequences launches and copies.
//
// Device data layout (all FP64 unless noted):
//   markers  SoA, Julia column-major N x 2: x[0..N) = v1, x[N..2N) = v2
//   sorted   in-domain markers in (cell, index) order: sx1, sx2, sw, perm, scell
//   coeffs   n_dofs vectors indexed i1 + i2*nd1 (first dimension fastest)
//   packed   pair-sum operands in sorted order: px = {v1,v2} (double2),
//            pg = {G1,G2} (double2), pw (double); FP32 copies for the mixed form
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/collops.h"

#define CO_CHUNK 1024        // markers per sort chunk (one block of 1024 threads)
#define CO_RED_THREADS 256   // threads of the reduction-producing kernels
#define CO_TICKETS 8         // arrival counters per context (ctx.tickets)
#define CO_TICKET_FROZEN 2   // k_frozen_map's counter (0, 1: k_cellcount per set)
#define CO_TICKET_LAMBDA 3   // k_grad_L's counter when it forms lambda
#define CO_TICKET_WINDOW 4   // k_anderson_cols's counter when it solves the window
#define CO_MAX_M 8           // Anderson depth limit of the device solver
#define CO_FS_FLOOR 1e-30    // functions.jl:23
#define CO_G_MAX 100.0       // functions.jl:31

// Device-side solver state, mirrored from step_anderson!'s locals
// (solver.jl:320-332) and read back by the host each iteration.
struct co_solver_state {
    int k;               // current iteration (1-based)
    int history, slot;   // Anderson window (solver.jl:320-321)
    int n_restart;
    int k64;             // defect correction: FP64 outer maps so far
    int finished;        // batch engine: the exit copy of this instance is done
    int done;            // 0 running, 1 converged, 2 stagnated, 3 max_iter
    int path;            // 0 damped Picard, 1 Anderson, for the current k
    int improved;        // nrm_r < nrm_best at the current k
    int error;           // device-detected error (non-finite residual, timeout)
    double nrm_r0, nrm_r, nrm_v, nrm_best, nrm_best_window, damp, res_out;
    double best32;       // defect correction: best FP32-stage outer residual
    int kbest32;         // and the outer map that reached it
    double ATA[CO_MAX_M * CO_MAX_M];
    double gamma[CO_MAX_M];
    double lambda;       // Gonzalez correction of the current map
    double S1;           // entropy of v_in's projection
    double lb[8];        // LB: n, U1, U2, Q, Sg1, Sg2, P  (+ spare)
    double ab[3];        // LB multipliers A1, A2, B
};

struct co_bufs {
    int cap;             // marker capacity
    int nchunk_cap;
    // per-marker (original order)
    double *vmid, *dv, *G, *dS, *Gv, *r, *rp, *Gp, *vbest, *v1, *v0, *w, *vin, *dotv;
    int *cell, *inv;
    double *xi;          // 2N: xi1, xi2
    // sorted in-domain markers
    int *perm, *scell;
    double *sw, *sphi;   // sphi: 6 per marker (phi1[3], phi2[3])
    // packed pair operands
    double2 *px, *pg;
    double *pw;
    float4 *pf_x;        // {x1h, x2h, x1l, x2l}
    float4 *pf_g;        // {g1h, g2h, g1l, g2l}
    float *pf_w, *pf_wl; // weight head / tail
    double *pdot;        // packed vdot (2 x cap)
    double *pA;          // packed metric A (3 x cap)
    double *part;        // slice partials of the pair kernels
    size_t part_cap;
    // sort scratch
    int *hist, *hoff, *count, *cstart;
    // reductions
    double *red;         // block partials (sized for the largest grid)
    int red_cap;
    // Anderson window
    double *dF, *dG;     // 2N x m each
    int m_cap;
    // defect correction (allocated on first use)
    double *Gk, *Phi, *Adef;
    // Anderson mixing of the defect correction's outer iterates (allocated on
    // first use): vk, u, r, rp, Gp (2 cap each) then dF, dG (2 cap x aa_m each)
    double *aa;
    int aa_m;
    // block-Newton preconditioner of the inner iteration (allocated on first
    // use): Psi, z (2 cap each) and the Hessian of L (3 cap)
    double *pc;
};

// Buffers of one counting sort + projection (co_spline.cu). Set 0 is the
// context's primary set (mb.cell ... mb.sphi, bS, b, y); set 1 (ctx.gs) holds
// the second marker set of the Gonzalez chain -- v_in, whose entropy S(v_in)
// is needed beside the v_mid projection -- sorted and projected in the same
// launches as set 0 (blockIdx.y selects the set).
struct co_sortset {
    int *cell, *inv, *perm, *scell, *hist, *hoff, *count, *cstart;
    double *xi, *sw, *sphi, *bS, *b, *y;
};

// The Gonzalez lambda formed by the last block of k_grad_L (st == nullptr: not)
struct co_lambda_job {
    co_solver_state *st;
    double S0;
    int gonzalez;
    const double *Ep;   // element entropy partials of v_in (S1 = their sum), or nullptr: st->S1
    int n_el;
    unsigned *ticket;
};

struct co_ctx {
    int device;
    cudaStream_t stream;
    unsigned flags;
    int n1, n2, nd1, nd2, n_dofs, n_el, nq;
    double lo1, hi1, lo2, hi2;
    // mesh tables
    double *bp1, *bp2;       // breakpoints
    double *C1, *C2;         // extraction [n][9]
    double *Tq1, *Tq2;       // basis at quad nodes: [n][3][nq]
    double *ih1, *ih2;       // reciprocal cell widths 1 / (bp[i+1] - bp[i])
    double *P1, *P2;         // cell-local basis C^T B in monomial form: [n][3][4] =
                             // (alpha, beta, gamma, 2 gamma), p = alpha + beta x + gamma x^2
    double *qw;              // quad weights [nq]
    double *Minv1, *Minv2;   // inverse 1D mass matrices (nd x nd, symmetric)
    // coefficient-sized buffers
    double *bS;              // cell sums [n_el][9]
    double *b, *y, *f, *fin, *rr, *L;  // n_dofs each
    double *E;               // element-local r contributions [n_el][9]
    double *Ep;              // element entropy partials [n_el]
    co_sortset gs;           // sort/projection set 1 (Gonzalez v_in), allocated on use
    int gs_cap;              // marker capacity of gs (0: not allocated)
    // arrival counters of the kernels whose last block finishes the launch's work
    // (k_cellcount: one per marker set; k_frozen_map: slot CO_TICKET_FROZEN); each
    // last block resets its counter, so launches and graph replays reuse them
    unsigned *tickets;
    co_bufs mb;
    co_solver_state *st;     // device state
    co_solver_state *st2;    // inner-solve state of the defect correction
    co_solver_state *st3;    // outer Anderson window of the defect correction
    co_solver_state *st_host;  // pinned mirror
    double *hstage;          // pinned host staging (grows)
    size_t hstage_cap;
    int pair_split_fp64, pair_split_fp32;  // split factors of the plain kernels (0 = auto)
    int pair_symmetric;      // 1: Newton's-third-law kernels (default), 0: one-sided
    int nsm;
    // launch counter (kernels of this library launched through the context)
    unsigned long long launches;
    // pair-kernel profiling (co_prof.cu)
    struct co_prof *prof;
    unsigned long long maps64, maps32, mapsds;
    // batch membership (co_batch): marker count and whether the instance has a pair sum
    int batch_N, batch_landau;
    int lb_two_pass;          // LB drift in two launches (capturable) instead of cooperative
    // bounded grid barrier of the cooperative LB kernel: polls before it gives
    // up with CO_ERR_TIMEOUT, and phantom blocks it waits for on top of the
    // grid (0 in normal use; a test sets 1 so that the barrier cannot complete)
    int barrier_spins, barrier_phantom;
    struct co_step_bufs *sb;  // buffers of co_step_learned (co_step.cu), allocated on first use
    struct co_nk_bufs *nk;    // buffers of the Newton-Krylov solve (co_newton.cu), on first use
};

// ------------------------------------------------------------- helpers
#define CO_CK(call)                                                   \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return CO_ERR_CUDA;                    \
    } while (0)

static inline int co_cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// ------------------------------------------------------------- spline stage
// (co_spline.cu)
int co_ensure_capacity(co_ctx *c, int N, int m);
int co_sort_markers(co_ctx *c, const double *x, int N);       // locate + stable cell sort
// v_mid = (v0 + v_in)/2 and dv = v_in - v0 into mb.vmid/mb.dv, v_mid sorted into
// set 0 and, with two != 0, v_in sorted into set 1, in the same launches
int co_sort_mid(co_ctx *c, const double *vin, const double *v0, int N, int two);
// co_project_sorted for set 0 -> f0 and (two != 0) set 1 -> f1
int co_project_two(co_ctx *c, double *f0, double *f1, int two);
// r-local of f (-> dof vector r) and, with fS != nullptr, the entropy partials of
// fS (-> Ep), in one quadrature launch
int co_r_and_entropy_dev(co_ctx *c, const double *f, double *r, const double *fS);
// L = M^{-1} r(f) (quadrature, dof gather and mass solve in three launches) and,
// with fS != nullptr, the entropy partials of fS (-> Ep) in the quadrature launch
int co_r_solve_dev(co_ctx *c, const double *f, double *L, const double *fS);
// co_grad_L_dev with dS and the Gonzalez partials, and lambda into ctx->st (the
// last block of the launch): S1 from Ep (element entropy partials) or st->S1
int co_grad_L_lambda_dev(co_ctx *c, const double *x, int N, const double *L, double *G,
                         const double *w, double *dS, const double *dv, double *red,
                         double S0, int gonzalez, const double *Ep);
void co_sortset_free(co_ctx *c);
int co_project_sorted(co_ctx *c, double *f_out);               // scatter + dof gather + mass solve
int co_mass_solve_dev(co_ctx *c, const double *rhs, double *out);
int co_compute_r_dev(co_ctx *c, const double *f, double *r);
int co_entropy_parts_dev(co_ctx *c, const double *f);          // fills c->Ep
int co_entropy_finalize_dev(co_ctx *c, double *S_dev);         // sums Ep -> *S_dev
int co_grad_L_dev(co_ctx *c, const double *x, int N, const double *L, double *G,
                  const double *w, double *dS, const double *dv, double *red);
int co_loggrad_dev(co_ctx *c, const double *x, int N, const double *f, double *g,
                   const double *w, const double *dv, double *red);
int co_hess_L_dev(co_ctx *c, int N, double *H);
int co_diagnostics_impl(co_ctx *c, const double *x, int N, double *out6);
#define CO_WS_NFEAT 15   // warm-start features per marker
int co_features_dev(co_ctx *c, int N, const double *H, const double *A, float *X);
int co_features_res_dev(co_ctx *c, int N, const double *r, double dt, float *X);

// ------------------------------------------------------------- pair stage
// (co_pair.cu)
int co_pair_fp64(co_ctx *c, int M, int with_metric);   // packed -> pdot (and pA)
int co_pair_fp32(co_ctx *c, int M);                    // packed FP32 -> pdot
int co_pair_ds(co_ctx *c, int M);                      // packed FP32 head/tail -> pdot,
                                                       // double-single arithmetic
int co_pack_landau(co_ctx *c, int N, int Mub, int precision, int gonzalez);
int co_pack_plain(co_ctx *c, int N, int Mub, int precision, const double *x, const double *G);
int co_unpack_A(co_ctx *c, int N, double *A);
int co_metric32(co_ctx *c, int Mub);   // FP32 metric A (3 x ld in pA) from pf_x/pf_w
int co_predictor_buffers(co_ctx *c, const co_opts *o, int precision, const double *v, int N,
                         double dt, double *out);
void co_ctx_destroy_detached(co_ctx *c);   // free a context whose stream/state it does not own
int co_step_defect_buffers(co_ctx *c, const co_opts *o, const co_defect_opts *dopt, int N,
                           double S0, double dt, int *outer, double *res, int *inner, double *r0);
void co_step_free(co_ctx *c);           // co_step.cu
void co_newton_free(co_ctx *c);         // co_newton.cu
int co_step_newton_buffers(co_ctx *c, const co_opts *o, const co_newton_opts *nko, int N,
                           double S0, double dt, int *evals, double *res, int *n_newton,
                           double *r0, int *status);
#define CO_PREC_BOTH 3                  // pack both FP64 and FP32 operands (internal)
// packed-operand sets a precision needs: 1 = FP64 arrays, 2 = FP32 head/tail arrays
static inline int co_pack_mode(int precision) {
    return precision == CO_PREC_FP64 ? 1 : precision == CO_PREC_BOTH ? 3 : 2;
}
int co_unpack_update(co_ctx *c, int N, double dt, double *Gv, const double *v0,
                     const double *v1, double *r, double *red);

// ------------------------------------------------------------- batch
// work description of one instance for the batched pair kernel
struct co_bwork {
    const double2 *px, *pg;
    const double *pw;
    double *gpart, *apart, *pdot;
    size_t ld;
    const co_solver_state *st;
    int nt, H, nchunk, blk0;
};
int co_batch_work_table(co_ctx *const *ctxs, const co_solver_state *const *states, int n,
                        int W, int KC, co_bwork *tab, int *max_pos);
int co_pair64_batch(cudaStream_t s, const co_bwork *d_tab, int n, int total, int W, int KC,
                    int grid, unsigned *d_counter, int max_pos);

// ------------------------------------------------------------- profiling
// (co_prof.cu) -- event pairs around pair-kernel launches, collected after
// stream synchronisation
void co_prof_begin(co_ctx *c, int fp64);
void co_prof_end(co_ctx *c);
void co_prof_collect(co_ctx *c);
void co_prof_free(co_ctx *c);

// ------------------------------------------------------------- solver stage
// (co_solver.cu)
int co_picard_map_dev(co_ctx *c, const co_opts *o, int precision, double *Gv,
                      const double *vin, const double *v0, const double *w, int N,
                      double S0, double dt, int want_resid);
int co_lb_fused(co_ctx *c, int N, double nu, double dt, double *Gv, const double *v0,
                const double *vmid, const double *w, double *g, const double *dv,
                int gonzalez, const double *v1, double *r);
