// co_solver.cu -- Picard map orchestration, Gonzalez correction, the fused LB
// drift, and step_anderson! entirely on the device.
//
// Picard map (solver.jl:176-227), Landau:
//   [Gonzalez] sort(v_in) -> project -> f_in -> S1 (element quadrature)
//   v_mid, dv -> sort(v_mid) -> project -> f -> r -> L = M^{-1} r
//   -> grad L at v_mid (+ dS = -w G, + dv.dS and |dv|^2 block partials)
//   -> lambda (one block, fixed order) -> pack G_eff -> pair sum -> unpack,
//   Gv = v0 + dt vdot (+ Anderson residual partials)
// LB: the same projection; the clamped log-gradient gather; then one
//   cooperative kernel applies lambda, forms the seven moments, solves the
//   3x3 system redundantly in every block and writes the drift and Gv.
//
// The Anderson control (solver.jl:334-417) runs in one-block kernels that own
// the device state; the host only launches the fixed kernel sequence of an
// iteration and reads the `done` word.
//
// Also here:
//   - step_defect! (solver.jl:569-634) with the staged precision of the mixed
//     forms, and the optional outer Anderson mixing, inner preconditioner and
//     metric freeze;
//   - the explicit predictor (main.jl:233-245);
//   - the batch engine (many ensembles, one persistent pair launch per
//     iteration, graph replay over the live instances);
//   - the warm-start entry points (features, proposal, first residual).
#include <math.h>

#include "co_internal.cuh"
#include "co_reduce.cuh"

#include <stdio.h>
#include <stdlib.h>

#include <vector>

// COLLOPS_VERBOSE=1 prints the solver's progress to stderr, one line per
// iteration, as the reference's `verbose = true` does (solver.jl:420, :613-627)
static int co_verbose() {
    static int v = -1;
    if (v < 0) {
        const char *e = getenv("COLLOPS_VERBOSE");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v;
}
static const char *prec_name(int p) {
    return p == CO_PREC_MIXED ? "fp32" : p == CO_PREC_MIXED_DS ? "ds" : "fp64";
}

#define CO_RED_COMPS 16
#define CO_BARRIER_SPINS (1 << 22)

// ---------------------------------------------------------------- lambda

__global__ void __launch_bounds__(256)
k_lambda(const double *__restrict__ red, int nred, co_solver_state *st, double S0,
         int gonzalez, const double *__restrict__ Ep, int n_el) {
    __shared__ double sh[32];
    // with Ep: S1 = S(v_in) from the element entropy partials first (the sum
    // k_sum_to forms, in the same order)
    double S1 = Ep ? co_sum_partials(Ep, n_el, 1, 0, sh) : 0.0;
    double dot = co_sum_partials(red, nred, 2, 0, sh);
    double n2 = co_sum_partials(red, nred, 2, 1, sh);
    if (threadIdx.x == 0) {
        if (Ep) st->S1 = S1;
        else S1 = st->S1;
        double lam = 0.0;
        if (gonzalez) lam = n2 > 1e-30 ? (S1 - S0 - dot) / n2 : 0.0;
        st->lambda = lam;
    }
}

// ---------------------------------------------------------------- LB fused

// Grid barrier for a cooperative launch (all blocks co-resident). The wait is
// bounded: after max_spins polls (CO_BARRIER_SPINS unless a test lowers it)
// the block records a timeout in *err and continues, so the kernel always
// terminates. nblocks is the number of arrivals the barrier waits for: the
// grid size, or more when a test asks for a barrier that cannot complete.
__device__ __forceinline__ void grid_barrier(unsigned *counter, unsigned nblocks, int *err,
                                             int max_spins) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned old = atomicAdd(counter, 1u);
        unsigned target = (old / nblocks + 1u) * nblocks;
        int spins = 0;
        while (*((volatile unsigned *)counter) < target) {
            if (++spins > max_spins) {
                atomicExch(err, 1);
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
}

__device__ void lu3_solve(double *M, double *b) {
    // LU with partial pivoting (Julia's `\` on the 3x3 system, functions.jl:103-105)
    int piv[3];
    for (int k = 0; k < 3; k++) {
        int p = k;
        double mx = fabs(M[k * 3 + k]);
        for (int i = k + 1; i < 3; i++)
            if (fabs(M[i * 3 + k]) > mx) { mx = fabs(M[i * 3 + k]); p = i; }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < 3; j++) { double t = M[k * 3 + j]; M[k * 3 + j] = M[p * 3 + j]; M[p * 3 + j] = t; }
        for (int i = k + 1; i < 3; i++) {
            M[i * 3 + k] /= M[k * 3 + k];
            for (int j = k + 1; j < 3; j++) M[i * 3 + j] -= M[i * 3 + k] * M[k * 3 + j];
        }
    }
    for (int k = 0; k < 3; k++) if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
    for (int i = 0; i < 3; i++) for (int j = 0; j < i; j++) b[i] -= M[i * 3 + j] * b[j];
    for (int i = 2; i >= 0; i--) {
        for (int j = i + 1; j < 3; j++) b[i] -= M[i * 3 + j] * b[j];
        b[i] /= M[i * 3 + i];
    }
}

// LB drift with exact momentum/energy multipliers (functions.jl:68-116,
// solver.jl:205-221), Gonzalez lambda applied first (solver.jl:204-209).
__global__ void __launch_bounds__(CO_RED_THREADS)
k_lb_fused(int N, const double *__restrict__ vmid, const double *__restrict__ w,
           double *__restrict__ g, const double *__restrict__ dv, int use_lambda, double nu,
           double dt, const double *__restrict__ v0, double *__restrict__ Gv,
           const double *__restrict__ v1, double *__restrict__ r, double *__restrict__ red7,
           double *__restrict__ red2, co_solver_state *st, unsigned *bar, int *err,
           unsigned bar_blocks, int bar_spins) {
    __shared__ double sh[32];
    __shared__ double sol[3];
    const double lam = use_lambda ? st->lambda : 0.0;
    double m[7] = {0, 0, 0, 0, 0, 0, 0};
    const int stride = gridDim.x * blockDim.x;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += stride) {
        double wa = w[a], x = vmid[a], y = vmid[N + a];
        double g1 = g[a], g2 = g[N + a];
        if (use_lambda) {
            double iw = 1.0 / wa;
            g1 -= lam * dv[a] * iw;
            g2 -= lam * dv[N + a] * iw;
            g[a] = g1;
            g[N + a] = g2;
        }
        m[0] += wa;
        m[1] += wa * x;
        m[2] += wa * y;
        m[3] += wa * (x * x + y * y);
        m[4] += wa * g1;
        m[5] += wa * g2;
        m[6] += wa * (x * g1 + y * g2);
    }
    for (int k = 0; k < 7; k++) {
        double s = co_block_sum(m[k], sh);
        if (threadIdx.x == 0) red7[blockIdx.x * 8 + k] = s;
    }
    grid_barrier(bar, bar_blocks, err, bar_spins);
    if (threadIdx.x == 0 && *((volatile int *)err)) st->error = CO_ERR_TIMEOUT;
    // every block reduces the partials in the same fixed order
    double tot[7];
    for (int k = 0; k < 7; k++) tot[k] = co_sum_partials(red7, gridDim.x, 8, k, sh);
    if (threadIdx.x == 0) {
        double M[9] = {tot[0], 0.0, tot[1], 0.0, tot[0], tot[2], tot[1], tot[2], tot[3]};
        double b[3] = {-tot[4], -tot[5], -tot[6]};
        lu3_solve(M, b);
        sol[0] = b[0]; sol[1] = b[1]; sol[2] = b[2];
        if (blockIdx.x == 0) {
            for (int k = 0; k < 7; k++) st->lb[k] = tot[k];
            st->ab[0] = b[0]; st->ab[1] = b[1]; st->ab[2] = b[2];
        }
    }
    __syncthreads();
    const double A1 = sol[0], A2 = sol[1], B = sol[2];
    double sr = 0.0, sv = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += stride) {
        double x = vmid[a], y = vmid[N + a];
        double q1 = -nu * (g[a] + A1 + B * x);
        double q2 = -nu * (g[N + a] + A2 + B * y);
        double o1 = v0[a] + dt * q1, o2 = v0[N + a] + dt * q2;
        Gv[a] = o1;
        Gv[N + a] = o2;
        if (r) {
            double x1 = v1[a], x2 = v1[N + a];
            double r1 = o1 - x1, r2 = o2 - x2;
            r[a] = r1;
            r[N + a] = r2;
            sr += r1 * r1 + r2 * r2;
            sv += x1 * x1 + x2 * x2;
        }
    }
    if (r) {
        double s1 = co_block_sum(sr, sh);
        double s2 = co_block_sum(sv, sh);
        if (threadIdx.x == 0) {
            red2[blockIdx.x * 2 + 0] = s1;
            red2[blockIdx.x * 2 + 1] = s2;
        }
    }
}

// The same LB drift in two launches without a grid barrier (for CUDA-graph
// capture in the batch engine): pass 1 applies lambda and writes the block
// partials of the seven moments; pass 2 reduces them redundantly in every
// block in the same fixed order, solves the 3x3 system and writes the drift.
__global__ void __launch_bounds__(CO_RED_THREADS)
k_lb_part(int N, const double *__restrict__ vmid, const double *__restrict__ w,
          double *__restrict__ g, const double *__restrict__ dv, int use_lambda,
          const co_solver_state *st, double *__restrict__ red7) {
    __shared__ double sh[32];
    const double lam = use_lambda ? st->lambda : 0.0;
    double m[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        double wa = w[a], x = vmid[a], y = vmid[N + a];
        double g1 = g[a], g2 = g[N + a];
        if (use_lambda) {
            double iw = 1.0 / wa;
            g1 -= lam * dv[a] * iw;
            g2 -= lam * dv[N + a] * iw;
            g[a] = g1;
            g[N + a] = g2;
        }
        m[0] += wa;
        m[1] += wa * x;
        m[2] += wa * y;
        m[3] += wa * (x * x + y * y);
        m[4] += wa * g1;
        m[5] += wa * g2;
        m[6] += wa * (x * g1 + y * g2);
    }
    for (int k = 0; k < 7; k++) {
        double s = co_block_sum(m[k], sh);
        if (threadIdx.x == 0) red7[blockIdx.x * 8 + k] = s;
    }
}

__global__ void __launch_bounds__(CO_RED_THREADS)
k_lb_apply(int N, int nred7, const double *__restrict__ red7, const double *__restrict__ vmid,
           const double *__restrict__ g, double nu, double dt, const double *__restrict__ v0,
           double *__restrict__ Gv, const double *__restrict__ v1, double *__restrict__ r,
           double *__restrict__ red2, co_solver_state *st) {
    __shared__ double sh[32];
    __shared__ double sol[3];
    double tot[7];
    for (int k = 0; k < 7; k++) tot[k] = co_sum_partials(red7, nred7, 8, k, sh);
    if (threadIdx.x == 0) {
        double M[9] = {tot[0], 0.0, tot[1], 0.0, tot[0], tot[2], tot[1], tot[2], tot[3]};
        double b[3] = {-tot[4], -tot[5], -tot[6]};
        lu3_solve(M, b);
        sol[0] = b[0]; sol[1] = b[1]; sol[2] = b[2];
        if (blockIdx.x == 0) {
            for (int k = 0; k < 7; k++) st->lb[k] = tot[k];
            st->ab[0] = b[0]; st->ab[1] = b[1]; st->ab[2] = b[2];
        }
    }
    __syncthreads();
    const double A1 = sol[0], A2 = sol[1], B = sol[2];
    double sr = 0.0, sv = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        double x = vmid[a], y = vmid[N + a];
        double q1 = -nu * (g[a] + A1 + B * x);
        double q2 = -nu * (g[N + a] + A2 + B * y);
        double o1 = v0[a] + dt * q1, o2 = v0[N + a] + dt * q2;
        Gv[a] = o1;
        Gv[N + a] = o2;
        if (r) {
            double x1 = v1[a], x2 = v1[N + a];
            double r1 = o1 - x1, r2 = o2 - x2;
            r[a] = r1;
            r[N + a] = r2;
            sr += r1 * r1 + r2 * r2;
            sv += x1 * x1 + x2 * x2;
        }
    }
    if (r) {
        double s1 = co_block_sum(sr, sh);
        double s2 = co_block_sum(sv, sh);
        if (threadIdx.x == 0) {
            red2[blockIdx.x * 2 + 0] = s1;
            red2[blockIdx.x * 2 + 1] = s2;
        }
    }
}

// ---------------------------------------------------------------- Anderson

struct co_dev_opts {
    int use_anderson, exit_picard_step, m, max_iter, stag_window, damp_decay_start;
    double tol, abs_floor, stag_rel_tol, damp_decay_factor, restart_factor, damping, reg_factor;
};

__global__ void k_state_reset(co_solver_state *st) {
    if (threadIdx.x == 0) {
        st->k = 0;
        st->history = 0;
        st->slot = 0;
        st->n_restart = 0;
        st->k64 = 0;
        st->finished = 0;
        st->done = 0;
        st->path = 0;
        st->improved = 0;
        st->error = 0;
        st->nrm_r0 = 0.0;
        st->nrm_r = 0.0;
        st->nrm_best = INFINITY;
        st->nrm_best_window = INFINITY;
        st->res_out = 0.0;
        st->best32 = INFINITY;
        st->kbest32 = 0;
    }
}

// residual norms and the exit / restart / damping decisions of iteration k
// (solver.jl:339-391)
__global__ void __launch_bounds__(256)
k_ctrl1(const double *__restrict__ red, int nred, co_solver_state *st, co_dev_opts o) {
    __shared__ double sh[32];
    if (st->done) return;
    double r2 = co_sum_partials(red, nred, 2, 0, sh);
    double v2 = co_sum_partials(red, nred, 2, 1, sh);
    if (threadIdx.x != 0) return;
    if (st->error) {
        st->done = 4;
        return;
    }
    int k = st->k + 1;
    st->k = k;
    double nrm_r = sqrt(r2), nrm_v = sqrt(v2);
    st->nrm_r = nrm_r;
    st->nrm_v = nrm_v;
    if (!isfinite(nrm_r)) {
        st->error = CO_ERR_NONFINITE;
        st->done = 4;
        st->res_out = nrm_r;
        return;
    }
    if (k == 1) st->nrm_r0 = nrm_r;
    st->improved = 0;
    if (nrm_r < st->nrm_best) {
        st->nrm_best = nrm_r;
        st->improved = 1;
    }
    double eff_tol = fmax(o.tol * (nrm_v + 1e-30), o.abs_floor);
    if (nrm_r < eff_tol) {
        st->done = 1;
        st->res_out = nrm_r;
        return;
    }
    if (k > o.stag_window && k % o.stag_window == 0) {
        double rel = (st->nrm_best_window - st->nrm_best) / (st->nrm_best_window + 1e-30);
        if (rel < o.stag_rel_tol) {
            st->done = 2;
            st->res_out = st->nrm_best;
            return;
        }
        st->nrm_best_window = st->nrm_best;
    }
    int just_restarted = 0;
    double rf = o.restart_factor > 0 ? o.restart_factor : INFINITY;
    if (k > 1 && nrm_r > rf * st->nrm_best) {
        st->history = 0;
        st->slot = 0;
        st->n_restart += 1;
        just_restarted = 1;
    }
    st->damp = k > o.damp_decay_start ? o.damping * o.damp_decay_factor : o.damping;
    if (k == 1 || just_restarted || !o.use_anderson) {
        st->path = 0;
    } else {
        st->path = 1;
        st->slot = st->slot % o.m + 1;
        st->history = st->history + 1 < o.m ? st->history + 1 : o.m;
    }
    if (k == o.max_iter) {
        // the host stops after this iteration; k_finish returns v_best
        st->res_out = st->nrm_best;
    }
}

__device__ void anderson_solve_body(const double *__restrict__ red, int nred,
                                    co_solver_state *st, const co_dev_opts &o);

// The iterate update after the control of iteration k, one launch for both
// branches: the damped Picard branch (path 0, solver.jl:384; the former
// k_plain_update) or the new window column (solver.jl:393-394) with its dot
// products with the window and with r (path 1; block partials laid out
// [block][2*CO_MAX_M], solved by the launch's last block); in both, the best-iterate copy
// (solver.jl:343-346) when the residual improved.
__global__ void __launch_bounds__(CO_RED_THREADS)
k_anderson_cols(int n2, co_solver_state *st, int exit_picard, double *__restrict__ v1,
                const double *__restrict__ r, double *__restrict__ rp,
                const double *__restrict__ Gv, double *__restrict__ Gp,
                double *__restrict__ dF, double *__restrict__ dG, size_t ldF,
                double *__restrict__ vbest, double *__restrict__ red, co_dev_opts o,
                unsigned *ticket) {
    if (st->done) return;
    const int improved = st->improved;
    if (st->path != 1) {
        const double damp = st->damp;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
            double x = v1[i], g = Gv[i];
            if (improved) vbest[i] = exit_picard ? g : x;
            v1[i] = damp * g + (1 - damp) * x;
            rp[i] = r[i];
            Gp[i] = g;
        }
        return;
    }
    const int slot = st->slot - 1, hist = st->history;
    // the window loops run to CO_MAX_M, unrolled with a guard, so that pa, pb
    // stay in registers (a runtime bound would put them in local memory)
    double pa[CO_MAX_M], pb[CO_MAX_M];
#pragma unroll
    for (int j = 0; j < CO_MAX_M; j++) pa[j] = pb[j] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        double ri = r[i], gi = Gv[i];
        if (improved) vbest[i] = exit_picard ? gi : v1[i];
        double F = ri - rp[i];
        double Gd = gi - Gp[i];
        dF[(size_t)slot * ldF + i] = F;
        dG[(size_t)slot * ldF + i] = Gd;
        rp[i] = ri;
        Gp[i] = gi;
#pragma unroll
        for (int j = 0; j < CO_MAX_M; j++) {
            if (j < hist) {
                double fj = j == slot ? F : dF[(size_t)j * ldF + i];
                pa[j] += F * fj;
                pb[j] += fj * ri;
            }
        }
    }
    // all 2*CO_MAX_M block sums at once: a recursive-halving warp reduction
    // (16 FP64 adds per lane instead of 5 per value, which matters at GB300's
    // FP64 rate), then warp partials summed in warp order by one thread per
    // value (fixed order, one barrier)
    static_assert(CO_MAX_M == 8, "k_anderson_cols reduces 2 x 8 values per lane");
    __shared__ double wsum[CO_RED_THREADS / 32][2 * CO_MAX_M];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double v[2 * CO_MAX_M];
#pragma unroll
    for (int j = 0; j < CO_MAX_M; j++) {
        v[j] = pa[j];
        v[CO_MAX_M + j] = pb[j];
    }
    const double sj = co_warp_sum16(v, lane);   // value (lane >> 1)
    if ((lane & 1) == 0) wsum[warp][lane >> 1] = sj;
    __syncthreads();
    const int t = threadIdx.x;
    if (t < 2 * CO_MAX_M && (t % CO_MAX_M) < hist) {
        double s = 0.0;
        for (int w = 0; w < nw; w++) s += wsum[w][t];
        red[(size_t)blockIdx.x * 2 * CO_MAX_M + t] = s;
    }
    // the last block to finish solves for the mixing coefficients
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x == 0) *ticket = 0u;
    anderson_solve_body(red, gridDim.x, st, o);
}

// normal equations with Tikhonov shift, gamma = ATA \ ATr (solver.jl:396-409),
// from the nred block partials of the new Gram row and of A^T r; run by the last
// block (256 threads) of k_anderson_cols, which wrote the partials
__device__ void anderson_solve_body(const double *__restrict__ red, int nred,
                                    co_solver_state *st, const co_dev_opts &o) {
    __shared__ double dots[2 * CO_MAX_M];
    const int slot = st->slot - 1, h = st->history;
    // the 2h sums over the nred block partials: one warp per value, lanes stride
    // the partials in order, then a shuffle tree (fixed order)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int c = warp; c < 2 * h; c += nw) {
            const int col = c < h ? c : CO_MAX_M + (c - h);
            double s = co_strided_sum_cg(red, lane, nred, 32, 2 * CO_MAX_M, col, 0.0);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) dots[col] = s;
        }
    }
    // the cached Gram matrix through shared memory, with the new row and column
    __shared__ double sA[CO_MAX_M * CO_MAX_M];
    for (int t = threadIdx.x; t < CO_MAX_M * CO_MAX_M; t += blockDim.x) sA[t] = st->ATA[t];
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    if (lane == 0)
        for (int j = 0; j < h; j++) {
            sA[slot * CO_MAX_M + j] = dots[j];
            sA[j * CO_MAX_M + slot] = dots[j];
            st->ATA[slot * CO_MAX_M + j] = dots[j];
            st->ATA[j * CO_MAX_M + slot] = dots[j];
        }
    __syncwarp();
    // LU with partial pivoting on the leading h x h block, by one warp: lane r
    // holds row r of A and b[r]. Each element sees the operations of the
    // sequential algorithm in the same order (pivot: the first row of largest
    // |A[i][k]|; L stored below the diagonal; b permuted as the rows; forward
    // substitution in ascending j, back substitution in ascending j per row),
    // but the rows of one elimination step and the forward updates run on
    // different lanes, so the chain is ~h steps long instead of ~h^3 / 3.
    double a[CO_MAX_M];
#pragma unroll
    for (int j = 0; j < CO_MAX_M; j++)
        a[j] = (lane < h && j < h) ? sA[lane * CO_MAX_M + j] : 0.0;
    double bb = lane < h ? dots[CO_MAX_M + lane] : 0.0;
    double dm = 0.0;
    for (int j = 0; j < h; j++) dm += sA[j * CO_MAX_M + j];
    dm /= h;
    const double l2 = o.reg_factor * dm + 1e-30;
#pragma unroll
    for (int j = 0; j < CO_MAX_M; j++)
        if (j == lane && lane < h) a[j] += l2;
    for (int k = 0; k < h; k++) {
        double akk = 0.0;   // this lane's A[lane][k]
#pragma unroll
        for (int j = 0; j < CO_MAX_M; j++)
            if (j == k) akk = a[j];
        const bool cand = lane >= k && lane < h;
        double mx = cand ? fabs(akk) : -1.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        const unsigned ball = __ballot_sync(0xffffffffu, cand && fabs(akk) == mx);
        const int p = ball ? __ffs(ball) - 1 : k;
        if (p != k) {   // swap rows k and p (and b)
            const int src = lane == k ? p : (lane == p ? k : lane);
#pragma unroll
            for (int j = 0; j < CO_MAX_M; j++) a[j] = __shfl_sync(0xffffffffu, a[j], src);
            bb = __shfl_sync(0xffffffffu, bb, src);
        }
        double rk[CO_MAX_M];   // pivot row
#pragma unroll
        for (int j = 0; j < CO_MAX_M; j++) rk[j] = __shfl_sync(0xffffffffu, a[j], k);
        if (lane > k && lane < h) {
            double f = 0.0;
#pragma unroll
            for (int j = 0; j < CO_MAX_M; j++)
                if (j == k) {
                    a[j] /= rk[j];
                    f = a[j];
                }
#pragma unroll
            for (int j = 0; j < CO_MAX_M; j++)
                if (j > k && j < h) a[j] -= f * rk[j];
        }
    }
    // forward substitution with the unit lower factor
    for (int j = 0; j + 1 < h; j++) {
        const double bj = __shfl_sync(0xffffffffu, bb, j);
        double aij = 0.0;
#pragma unroll
        for (int t = 0; t < CO_MAX_M; t++)
            if (t == j) aij = a[t];
        if (lane > j && lane < h) bb -= aij * bj;
    }
    // back substitution, row by row from the last
    for (int i = h - 1; i >= 0; i--) {
        for (int j = i + 1; j < h; j++) {
            const double bj = __shfl_sync(0xffffffffu, bb, j);
            double aij = 0.0;
#pragma unroll
            for (int t = 0; t < CO_MAX_M; t++)
                if (t == j) aij = a[t];
            if (lane == i) bb -= aij * bj;
        }
        double aii = 1.0;
#pragma unroll
        for (int t = 0; t < CO_MAX_M; t++)
            if (t == i) aii = a[t];
        if (lane == i) bb /= aii;
    }
    if (lane < h) st->gamma[lane] = bb;
}

// v1 = damp (Gv - dG gamma) + (1 - damp) v_old (solver.jl:410-412)
__global__ void k_anderson_update(int n2, co_solver_state *st, double *__restrict__ v1,
                                  const double *__restrict__ Gv, const double *__restrict__ dG,
                                  size_t ldF) {
    if (st->done || st->path != 1) return;
    const int h = st->history;
    const double damp = st->damp;
    double gam[CO_MAX_M];
#pragma unroll
    for (int j = 0; j < CO_MAX_M; j++) gam[j] = j < h ? st->gamma[j] : 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        double s = Gv[i];
#pragma unroll
        for (int j = 0; j < CO_MAX_M; j++)
            if (j < h) s += -1.0 * dG[(size_t)j * ldF + i] * gam[j];
        v1[i] = damp * s + (1 - damp) * v1[i];
    }
}

// exit copies (solver.jl:351, :361, :420)
__global__ void k_finish(int n2, co_solver_state *st, int exit_picard, double *__restrict__ v1,
                         const double *__restrict__ Gv, const double *__restrict__ vbest) {
    int done = st->done, improved = st->improved;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        if (done == 1) {
            if (exit_picard) v1[i] = Gv[i];
        } else if (done == 2) {
            v1[i] = improved ? (exit_picard ? Gv[i] : v1[i]) : vbest[i];
        } else if (done == 0 || done == 3) {
            v1[i] = vbest[i];
        }
    }
}

__global__ void k_set_done(co_solver_state *st, int v) {
    if (threadIdx.x == 0 && st->done == 0) st->done = v;
}

// ---------------------------------------------------------------- host

static int ew_grid(co_ctx *c, long long n) {
    int g = co_cdiv(n, 256);
    int cap = 8 * c->nsm;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

static int red_blocks(co_ctx *c, int N) {
    int g = co_cdiv(N, CO_RED_THREADS);
    if (g > c->mb.red_cap) g = c->mb.red_cap;
    return g < 1 ? 1 : g;
}

// Grid of k_anderson_cols: two blocks per SM, each thread striding over several
// elements, so the per-thread partial dot products cover several elements
// before the (FP64) warp reduction
static int window_blocks(co_ctx *c, int n2) {
    int g = red_blocks(c, n2);
    return g > 2 * c->nsm ? 2 * c->nsm : g;
}

int co_lb_fused(co_ctx *c, int N, double nu, double dt, double *Gv, const double *v0,
                const double *vmid, const double *w, double *g, const double *dv,
                int gonzalez, const double *v1, double *r) {
    static int max_blocks_per_sm = -1;
    if (max_blocks_per_sm < 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_blocks_per_sm, k_lb_fused,
                                                          CO_RED_THREADS, 0) != cudaSuccess)
            return CO_ERR_CUDA;
    }
    int grid = red_blocks(c, N);
    int cap = max_blocks_per_sm * c->nsm;
    if (grid > cap) grid = cap;
    if (grid > c->mb.red_cap / 2) grid = c->mb.red_cap / 2;
    if (grid < 1) grid = 1;
    unsigned *bar = (unsigned *)(c->mb.red + (size_t)c->mb.red_cap * CO_RED_COMPS);
    int *err = (int *)(bar + 4);
    CO_CK(cudaMemsetAsync(bar, 0, 32, c->stream));
    double *red7 = c->mb.red + (size_t)c->mb.red_cap * 8;  // disjoint from red2 (first 2*grid)
    double *red2 = c->mb.red;
    int use_lambda = gonzalez;
    unsigned bar_blocks = (unsigned)(grid + (c->barrier_phantom > 0 ? c->barrier_phantom : 0));
    int bar_spins = c->barrier_spins > 0 ? c->barrier_spins : CO_BARRIER_SPINS;
    void *args[] = {&N, &vmid, &w, &g, &dv, &use_lambda, &nu, &dt, &v0, &Gv, &v1, &r,
                    &red7, &red2, &c->st, &bar, &err, &bar_blocks, &bar_spins};
    CO_CK(cudaLaunchCooperativeKernel((void *)k_lb_fused, grid, CO_RED_THREADS, args, 0,
                                      c->stream));
    c->launches++;
    return CO_OK;
}

// landau_geff! (solver.jl:86-113) after the v_mid projection: r, L = M^{-1} r,
// grad L at v_mid with dS = -w G and the Gonzalez partials, then lambda.
// With gonzalez, the quadrature launch also takes the entropy partials of
// v_in's projection (c->fin), summed into st->S1 before lambda needs it.
static int landau_tail(co_ctx *c, int gonzalez, int N, double S0, int nred) {
    int rc;
    co_bufs &b = c->mb;
    if ((rc = co_r_solve_dev(c, c->f, c->L, gonzalez ? c->fin : nullptr))) return rc;
    // grad L with dS and the Gonzalez partials; its last block forms lambda
    if (N > 0)
        return co_grad_L_lambda_dev(c, b.vmid, N, c->L, b.G, b.w, b.dS, b.dv, b.red, S0,
                                    gonzalez, gonzalez ? c->Ep : nullptr);
    k_lambda<<<1, 256, 0, c->stream>>>(b.red, 0, c->st, S0, gonzalez,
                                       gonzalez ? c->Ep : nullptr, c->n_el);
    c->launches++;
    (void)nred;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// v_mid, dv and the projection of v_mid (set 0 -> c->f) and, with gonzalez, of
// v_in (set 1 -> c->fin, for S(v_in)), in shared launches
static int project_mid(co_ctx *c, int gonzalez, const double *vin, const double *v0, int N) {
    int rc;
    if ((rc = co_sort_mid(c, vin, v0, N, gonzalez))) return rc;
    return co_project_two(c, c->f, c->fin, gonzalez);
}

// full landau_geff! at v_in: leaves dS, dv, lambda (st) and the sorted v_mid
static int landau_geff_dev(co_ctx *c, int gonzalez, const double *vin, const double *v0, int N,
                           double S0) {
    int rc;
    if ((rc = project_mid(c, gonzalez, vin, v0, N))) return rc;
    return landau_tail(c, gonzalez, N, S0, red_blocks(c, N));
}

// One Picard map on device buffers. vin/v0/w device pointers (w must be
// c->mb.w). If r != nullptr, r = Gv - vin with residual partials in mb.red.
static int picard_map_impl(co_ctx *c, int model, int gonzalez, double nu, int precision,
                           double *Gv, const double *vin, const double *v0, int N, double S0,
                           double dt, double *r, int *nred_out) {
    int rc;
    co_bufs &b = c->mb;
    int nred = red_blocks(c, N);
    if ((rc = project_mid(c, gonzalez, vin, v0, N))) return rc;
    if (model == CO_MODEL_LB) {
        if (gonzalez && (rc = co_entropy_parts_dev(c, c->fin))) return rc;
        if ((rc = co_loggrad_dev(c, b.vmid, N, c->f, b.G, b.w, b.dv, b.red))) return rc;
        k_lambda<<<1, 256, 0, c->stream>>>(b.red, nred, c->st, S0, gonzalez,
                                           gonzalez ? c->Ep : nullptr, c->n_el);
        c->launches++;
        CO_CK(cudaGetLastError());
        if (c->lb_two_pass) {
            int g1 = nred;  // grid of both passes
            double *red7 = b.red + (size_t)b.red_cap * 8;
            k_lb_part<<<g1, CO_RED_THREADS, 0, c->stream>>>(N, b.vmid, b.w, b.G, b.dv, gonzalez,
                                                           c->st, red7);
            k_lb_apply<<<g1, CO_RED_THREADS, 0, c->stream>>>(N, g1, red7, b.vmid, b.G, nu, dt, v0,
                                                            Gv, vin, r, b.red, c->st);
            c->launches += 2;
            CO_CK(cudaGetLastError());
            if (nred_out) *nred_out = g1;
            return CO_OK;
        }
        if ((rc = co_lb_fused(c, N, nu, dt, Gv, v0, b.vmid, b.w, b.G, b.dv, gonzalez, vin, r)))
            return rc;
        // residual partials of the fused kernel use its own grid size
        int max_bps = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&max_bps, k_lb_fused, CO_RED_THREADS, 0);
        int grid = red_blocks(c, N);
        if (grid > max_bps * c->nsm) grid = max_bps * c->nsm;
        if (grid > c->mb.red_cap / 2) grid = c->mb.red_cap / 2;
        if (grid < 1) grid = 1;
        nred = grid;
    } else {
        if ((rc = landau_tail(c, gonzalez, N, S0, nred))) return rc;
        if ((rc = co_pack_landau(c, N, N, precision, gonzalez))) return rc;
        if (precision == CO_PREC_MIXED) {
            rc = co_pair_fp32(c, N);
            c->maps32++;
        } else if (precision == CO_PREC_MIXED_DS) {
            rc = co_pair_ds(c, N);
            c->mapsds++;
        } else {
            rc = co_pair_fp64(c, N, 0);
            c->maps64++;
        }
        if (rc) return rc;
        if ((rc = co_unpack_update(c, N, dt, Gv, v0, vin, r, r ? b.red : nullptr))) return rc;
    }
    if (nred_out) *nred_out = nred;
    return CO_OK;
}

int co_picard_map_dev(co_ctx *c, const co_opts *o, int precision, double *Gv,
                      const double *vin, const double *v0, const double *w, int N, double S0,
                      double dt, int want_resid) {
    (void)w;
    return picard_map_impl(c, o->model, o->use_gonzalez, o->nu, precision, Gv, vin, v0, N, S0,
                           dt, want_resid ? c->mb.r : nullptr, nullptr);
}

static co_dev_opts dev_opts(const co_opts *o, double floor_extra) {
    co_dev_opts d;
    d.use_anderson = o->use_anderson;
    d.exit_picard_step = o->exit_picard_step;
    d.m = o->m;
    d.max_iter = o->max_iter;
    d.stag_window = o->stag_window;
    d.damp_decay_start = o->damp_decay_start;
    d.tol = o->tol;
    d.abs_floor = fmax(o->abs_floor, floor_extra);
    d.stag_rel_tol = o->stag_rel_tol;
    d.damp_decay_factor = o->damp_decay_factor;
    d.restart_factor = o->restart_factor;
    d.damping = o->damping;
    d.reg_factor = o->reg_factor;
    return d;
}

// The Anderson loop on device buffers mb.v1 (in/out), mb.v0, mb.w.
// precision selects the pair kernel of the maps.
static int anderson_loop(co_ctx *c, const co_opts *o, int precision, int N, double S0, double dt,
                         co_dev_opts d, int max_iter, int *iters_out) {
    int rc;
    co_bufs &b = c->mb;
    int n2 = 2 * N;
    size_t ldF = 2 * (size_t)b.cap;
    int eg = ew_grid(c, n2);
    k_state_reset<<<1, 32, 0, c->stream>>>(c->st);
    c->launches++;
    int k;
    for (k = 1; k <= max_iter; k++) {
        int nred = 0;
        if ((rc = picard_map_impl(c, o->model, o->use_gonzalez, o->nu, precision, b.Gv, b.v1,
                                  b.v0, N, S0, dt, b.r, &nred)))
            return rc;
        k_ctrl1<<<1, 256, 0, c->stream>>>(b.red, nred, c->st, d);
        const int ng = window_blocks(c, n2);
        k_anderson_cols<<<ng, CO_RED_THREADS, 0, c->stream>>>(n2, c->st, o->exit_picard_step, b.v1,
                                                              b.r, b.rp, b.Gv, b.Gp, b.dF, b.dG,
                                                              ldF, b.vbest, b.red, d,
                                                              c->tickets + CO_TICKET_WINDOW);
        c->launches += 2;
        if (o->use_anderson) {
            k_anderson_update<<<eg, 256, 0, c->stream>>>(n2, c->st, b.v1, b.Gv, b.dG, ldF);
            c->launches += 1;
        }
        CO_CK(cudaGetLastError());
        CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                              c->stream));
        CO_CK(cudaStreamSynchronize(c->stream));
        co_prof_collect(c);
        if (co_verbose())
            fprintf(stderr, "    anderson[%s] k=%d  |r|=%.6e  |v|=%.6e%s\n", prec_name(precision), k,
                    c->st_host->nrm_r, c->st_host->nrm_v,
                    c->st_host->done == 1 ? "  [converged]"
                    : c->st_host->done == 2 ? "  [stagnated]" : "");
        if (c->st_host->done) break;
    }
    if (k > max_iter) {
        k_set_done<<<1, 32, 0, c->stream>>>(c->st, 3);
        c->launches++;
    }
    k_finish<<<eg, 256, 0, c->stream>>>(n2, c->st, o->exit_picard_step, b.v1, b.Gv, b.vbest);
    c->launches++;
    CO_CK(cudaGetLastError());
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    if (iters_out) *iters_out = k > max_iter ? max_iter : k;
    if (c->st_host->error) return c->st_host->error;
    return CO_OK;
}

// step_anderson! on device buffers: mb.v1 (guess in, solution out), mb.v0, mb.w
int co_step_anderson_buffers(co_ctx *c, const co_opts *o, int N, double S0, double dt,
                             int *iters, double *res, int *nrs, double *r0) {
    int rc;
    if (o->m < 1 || o->m > CO_MAX_M) return CO_ERR_ARG;
    if ((rc = co_ensure_capacity(c, N, o->m))) return rc;
    if (N == 0) {
        if (iters) *iters = 0;
        if (res) *res = 0;
        if (nrs) *nrs = 0;
        if (r0) *r0 = 0;
        return CO_OK;
    }
    int it = 0;
    if (o->precision == CO_PREC_MIXED || o->precision == CO_PREC_MIXED_DS) {
        // phase 1: Anderson on the FP32-pair map, floored at mixed_floor
        double fl = o->mixed_floor > 0 ? o->mixed_floor : 0.0;
        co_dev_opts d = dev_opts(o, fl);
        if ((rc = anderson_loop(c, o, CO_PREC_MIXED, N, S0, dt, d, o->max_iter, &it))) return rc;
        double r0_32 = c->st_host->nrm_r0;
        int nrs32 = c->st_host->n_restart;
        // phase 2: Anderson on the FP64 (or double-single) map from the phase-1
        // iterate, to the full tolerance; its exit map is the exit_picard_step
        const int prec2 = o->precision == CO_PREC_MIXED_DS ? CO_PREC_MIXED_DS : CO_PREC_FP64;
        const int left = o->max_iter - it > 1 ? o->max_iter - it : 1;
        int it2 = 0;
        co_dev_opts d2 = dev_opts(o, 0.0);
        if ((rc = anderson_loop(c, o, prec2, N, S0, dt, d2, left, &it2))) return rc;
        if (iters) *iters = it + (c->st_host->done == 0 || c->st_host->done == 3 ? left
                                                                                 : c->st_host->k);
        if (res) *res = c->st_host->res_out;
        if (nrs) *nrs = nrs32 + c->st_host->n_restart;
        if (r0) *r0 = r0_32;
        return CO_OK;
    }
    co_dev_opts d = dev_opts(o, 0.0);
    if ((rc = anderson_loop(c, o, CO_PREC_FP64, N, S0, dt, d, o->max_iter, &it))) return rc;
    if (iters) *iters = c->st_host->done == 0 || c->st_host->done == 3 ? o->max_iter : c->st_host->k;
    if (res) *res = c->st_host->res_out;
    if (nrs) *nrs = c->st_host->n_restart;
    if (r0) *r0 = c->st_host->nrm_r0;
    return CO_OK;
}

// Explicit predictor (main.jl:233-245) on device: out = v + dt vdot(v)
int co_predictor_buffers(co_ctx *c, const co_opts *o, int precision, const double *v, int N,
                         double dt, double *out) {
    int rc;
    co_bufs &b = c->mb;
    if ((rc = co_ensure_capacity(c, N, 1))) return rc;
    if (N == 0) return CO_OK;
    if ((rc = co_sort_markers(c, v, N))) return rc;
    if ((rc = co_project_sorted(c, c->f))) return rc;
    if (o->model == CO_MODEL_LB) {
        if ((rc = co_loggrad_dev(c, v, N, c->f, b.G, b.w, nullptr, nullptr))) return rc;
        if ((rc = co_lb_fused(c, N, o->nu, dt, out, v, v, b.w, b.G, nullptr, 0, nullptr, nullptr)))
            return rc;
    } else {
        if ((rc = co_compute_r_dev(c, c->f, c->rr))) return rc;
        if ((rc = co_mass_solve_dev(c, c->rr, c->L))) return rc;
        if ((rc = co_grad_L_dev(c, v, N, c->L, b.G, nullptr, nullptr, nullptr, nullptr))) return rc;
        // the predictor is an initial guess: the mixed forms take the FP32 pair sum
        const int pprec = precision == CO_PREC_FP64 ? CO_PREC_FP64 : CO_PREC_MIXED;
        if ((rc = co_pack_plain(c, N, N, pprec, v, b.G))) return rc;
        rc = pprec == CO_PREC_MIXED ? co_pair_fp32(c, N) : co_pair_fp64(c, N, 0);
        if (rc) return rc;
        if ((rc = co_unpack_update(c, N, dt, out, v, nullptr, nullptr, nullptr))) return rc;
    }
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// ================================================================ defect correction
//
// step_defect! (solver.jl:569-634) with _anderson_inner! (solver.jl:492-526).
// Outer iteration k: G_eff(v_k) and the full Picard map G(v_k) with the pair
// sum -- FP64 in the plain form; in the mixed form FP32 until the FP32 outer
// residual stalls, then FP64 -- plus the frozen metric A_k (FP32 kernel, it only
// shapes the inner model). Inner: Anderson on
//     Phi_k(u) = G(v_k) - dt A_k (G_eff(u) - G_eff(v_k))
// to max(eta ||G(v_k) - v_k||, abs_floor/2); each Phi_k needs the O(N)
// projection chain but no pair sum. The exit returns G(v) from a pair sum, so
// momentum and energy are conserved as in step_anderson!.

// G_eff = -(dS + lambda dv)/w in marker order (solver.jl:107-111)
__global__ void k_geff_store(int N, const double *__restrict__ dS, const double *__restrict__ dv,
                             const double *__restrict__ w, const co_solver_state *st, int use_lambda,
                             double *__restrict__ Gk) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    double lam = use_lambda ? st->lambda : 0.0;
    double iw = 1.0 / w[a];
    Gk[a] = -(dS[a] + lam * dv[a]) * iw;
    Gk[N + a] = -(dS[N + a] + lam * dv[N + a]) * iw;
}

// frozen_map! (solver.jl:585-595): Phi = Gv - dt A (G_eff(u) - Gk), r = Phi - u
__device__ void ctrl_inner_body(const double *__restrict__ red, int nred, co_solver_state *si,
                                const co_solver_state *so, int m, double damping,
                                cudaGraphConditionalHandle hnd, int use_cond, int cap,
                                double *sh);

__global__ void __launch_bounds__(CO_RED_THREADS)
k_frozen_map(int N, const double *__restrict__ Gv, const double *__restrict__ A,
             const double *__restrict__ Gk, const double *__restrict__ dS,
             const double *__restrict__ dv, const double *__restrict__ w,
             const co_solver_state *st, int use_lambda, double dt, const double *__restrict__ u,
             double *__restrict__ Phi, double *__restrict__ r, double *__restrict__ red,
             co_solver_state *si, int m, double damping, cudaGraphConditionalHandle hnd,
             int use_cond, int cap, unsigned *ticket) {
    __shared__ double sh[32];
    double lam = use_lambda ? st->lambda : 0.0;
    double sr = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        double iw = 1.0 / w[a];
        double d1 = -(dS[a] + lam * dv[a]) * iw - Gk[a];
        double d2 = -(dS[N + a] + lam * dv[N + a]) * iw - Gk[N + a];
        double A11 = A[a], A12 = A[N + a], A22 = A[2 * (size_t)N + a];
        double p1 = Gv[a] - dt * (A11 * d1 + A12 * d2);
        double p2 = Gv[N + a] - dt * (A12 * d1 + A22 * d2);
        Phi[a] = p1;
        Phi[N + a] = p2;
        double r1 = p1 - u[a], r2 = p2 - u[N + a];
        r[a] = r1;
        r[N + a] = r2;
        sr += r1 * r1 + r2 * r2;
    }
    double s = co_block_sum(sr, sh);
    if (threadIdx.x == 0) {
        red[blockIdx.x * 2 + 0] = s;
        red[blockIdx.x * 2 + 1] = 0.0;
    }
    // the last block to finish runs the inner control on all blocks' partials
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x == 0) *ticket = 0u;
    ctrl_inner_body(red, gridDim.x, si, st, m, damping, hnd, use_cond, cap, sh);
}

// Block-Newton preconditioner of the inner iteration (co_defect_opts.precond):
// per marker, R(u) = Phi(u) - u has the local Jacobian -(I + dt A M), with
// M = H/2 - (lambda/w) I (G_eff = G(v_mid) - lambda dv/w, v_mid = (u + v0)/2, H
// the Hessian of L at v_mid). z = (I + dt A M)^{-1} r (plain r where
// |det| < 0.1) and Psi = u + z, the map Anderson then iterates. use_lambda:
// 1 with the lambda/w term (Gonzalez on, precond = 1), else M = H/2.
__global__ void k_precond(int N, const double *__restrict__ A, const double *__restrict__ H,
                          const double *__restrict__ w, const co_solver_state *st, int use_lambda,
                          double dt, const double *__restrict__ u, const double *__restrict__ r,
                          double *__restrict__ z, double *__restrict__ Psi) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    double lam = use_lambda == 1 ? st->lambda : 0.0;
    double iw = 1.0 / w[a];
    double A11 = A[a], A12 = A[N + a], A22 = A[2 * (size_t)N + a];
    double M11 = 0.5 * H[a] - lam * iw, M12 = 0.5 * H[N + a];
    double M22 = 0.5 * H[2 * (size_t)N + a] - lam * iw;
    double P11 = 1.0 + dt * (A11 * M11 + A12 * M12);
    double P12 = dt * (A11 * M12 + A12 * M22);
    double P21 = dt * (A12 * M11 + A22 * M12);
    double P22 = 1.0 + dt * (A12 * M12 + A22 * M22);
    double det = P11 * P22 - P12 * P21;
    double r1 = r[a], r2 = r[N + a], z1 = r1, z2 = r2;
    if (fabs(det) >= 0.1) {
        z1 = (P22 * r1 - P12 * r2) / det;
        z2 = (P11 * r2 - P21 * r1) / det;
    }
    z[a] = z1;
    z[N + a] = z2;
    Psi[a] = u[a] + z1;
    Psi[N + a] = u[N + a] + z2;
}

struct co_defect_dev {
    double tol, abs_floor, eta, stag_rel_tol, fp32_stall;
    int stag_window, fp32_window;
};

// outer decisions (solver.jl:603-626). stage: 1 = FP32 outer map, 0 = FP64.
// st->path <- next stage; st->res_out <- inner tolerance.
__global__ void __launch_bounds__(256)
k_ctrl_outer(const double *__restrict__ red, int nred, co_solver_state *st, co_defect_dev o,
             int stage) {
    __shared__ double sh[32];
    if (st->done) return;
    double r2 = co_sum_partials(red, nred, 2, 0, sh);
    double v2 = co_sum_partials(red, nred, 2, 1, sh);
    if (threadIdx.x != 0) return;
    if (st->error) {
        st->done = 4;
        return;
    }
    int k = st->k + 1;
    st->k = k;
    double nrm = sqrt(r2), nv = sqrt(v2);
    st->nrm_v = nv;
    if (!isfinite(nrm)) {
        st->error = CO_ERR_NONFINITE;
        st->done = 4;
        return;
    }
    st->improved = 0;
    if (stage == 1) {
        // FP32 outer maps: stop them at the FP32 noise floor, where the FP64
        // stage takes over. fp32_window = 0: as soon as a map cuts the residual
        // by less than fp32_stall; fp32_window = W > 0: once W maps in a row
        // brought no new best cut by fp32_stall (robust to the non-monotone
        // residuals of the outer Anderson mixing)
        double prev = st->nrm_r;
        st->nrm_r = nrm;
        if (k == 1) st->nrm_r0 = nrm;
        bool stall;
        if (o.fp32_window > 0) {
            if (nrm < o.fp32_stall * st->best32) {
                st->best32 = nrm;
                st->kbest32 = k;
            }
            stall = k - st->kbest32 >= o.fp32_window;
        } else {
            stall = k > 1 && nrm > o.fp32_stall * prev;
        }
        if (stall || nrm < fmax(o.tol * (nv + 1e-30), o.abs_floor))
            st->path = 0;
        else
            st->path = 1;
        st->res_out = fmax(o.eta * nrm, 0.5 * o.abs_floor);
        return;
    }
    st->nrm_r = nrm;
    if (st->k64 == 0) {  // first FP64 outer map: the stopping rule starts here
        st->nrm_best = INFINITY;
        st->nrm_best_window = INFINITY;
        if (k == 1) st->nrm_r0 = nrm;
    }
    st->k64 += 1;
    int k64 = st->k64;
    if (nrm < st->nrm_best) {
        st->nrm_best = nrm;
        st->improved = 1;
    }
    if (nrm < fmax(o.tol * (nv + 1e-30), o.abs_floor)) {
        st->done = 1;
        st->res_out = nrm;
        return;
    }
    if (k64 > o.stag_window && k64 % o.stag_window == 0) {
        if ((st->nrm_best_window - st->nrm_best) / (st->nrm_best_window + 1e-30) < o.stag_rel_tol) {
            st->done = 2;
            st->res_out = st->nrm_best;
            return;
        }
        st->nrm_best_window = st->nrm_best;
    }
    st->path = 0;
    st->res_out = fmax(o.eta * nrm, 0.5 * o.abs_floor);
}

// vbest <- Gv when the outer residual improved
__global__ void k_defect_best(int n2, const co_solver_state *st, const double *__restrict__ Gv,
                              double *__restrict__ vbest) {
    if (!st->improved) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x)
        vbest[i] = Gv[i];
}

// inner Anderson control (solver.jl:497-521): tolerance from the outer state
// Inner-iteration control (after the frozen map's residual): the residual
// norm, the exit test against the outer stage's tolerance, and the Anderson
// window bookkeeping; inside the device-side inner loop also the loop
// condition. Run by the last block of k_frozen_map, whose partials it sums.
__device__ void ctrl_inner_body(const double *__restrict__ red, int nred, co_solver_state *si,
                                const co_solver_state *so, int m, double damping,
                                cudaGraphConditionalHandle hnd, int use_cond, int cap,
                                double *sh) {
    if (si->done) {
        if (use_cond && threadIdx.x == 0) cudaGraphSetConditional(hnd, 0u);
        return;
    }
    double r2 = co_block_sum(co_strided_sum_cg(red, threadIdx.x, nred, blockDim.x, 2, 0, 0.0), sh);
    if (threadIdx.x != 0) return;
    int k = si->k + 1;
    si->k = k;
    double nrm = sqrt(r2);
    si->nrm_r = nrm;
    si->improved = 0;
    if (!isfinite(nrm)) {
        si->error = CO_ERR_NONFINITE;
        si->done = 4;
    } else if (nrm < so->res_out) {
        si->done = 1;
    } else {
        si->damp = damping;
        if (k == 1) {
            si->path = 0;
        } else {
            si->path = 1;
            si->slot = si->slot % m + 1;
            si->history = si->history + 1 < m ? si->history + 1 : m;
        }
    }
    // inside the device-side inner loop: repeat the body while the inner solve
    // has not exited and fewer than cap iterations ran
    if (use_cond)
        cudaGraphSetConditional(hnd, (!si->done && !si->error && k < cap) ? 1u : 0u);
}

// Anderson mixing of the outer iterates (co_defect_opts.outer_m > 0): the
// outer step v_k -> u_k = D(v_k) (the inner solution) is a fixed-point map
// whose fixed points are those of the Picard map; its slow modes (the part of
// the Jacobian the frozen metric misses) are removed by mixing over the last
// outer_m pairs (v_j, u_j). Window control: restart on the first call, when the
// host flags a change of the pair precision, and when the current outer
// residual is above twice the best since the last restart; otherwise the next
// window slot. Undamped (damp = 1): path 0 takes u_k itself.
__global__ void k_ctrl_aa(co_solver_state *sa, const co_solver_state *so, int m, int restart) {
    if (threadIdx.x != 0 || so->done) return;
    const double nr = so->nrm_r;
    int k = sa->k + 1;
    sa->improved = 0;
    sa->damp = 1.0;
    if (k == 1 || restart || nr > 2.0 * sa->nrm_best) {
        if (k > 1) sa->n_restart += 1;
        sa->k = 1;
        sa->history = 0;
        sa->slot = 0;
        sa->path = 0;
        sa->nrm_best = nr;
        return;
    }
    sa->k = k;
    if (nr < sa->nrm_best) sa->nrm_best = nr;
    sa->path = 1;
    sa->slot = sa->slot % m + 1;
    sa->history = sa->history + 1 < m ? sa->history + 1 : m;
}

// u <- D(v_k) (in v1), r <- u - v_k
__global__ void k_aa_resid(int n2, const co_solver_state *so, const double *__restrict__ v1,
                           const double *__restrict__ vk, double *__restrict__ u,
                           double *__restrict__ r) {
    if (so->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        double x = v1[i];
        u[i] = x;
        r[i] = x - vk[i];
    }
}

__global__ void k_copy_if_done(int n2, const co_solver_state *st, int want, double *__restrict__ dst,
                               const double *__restrict__ src) {
    if (st->done != want) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

static bool co_inner_host_loop() {
    const char *e = getenv("COLLOPS_INNER_LOOP");
    return e && strcmp(e, "host") == 0;
}

int co_step_defect_buffers(co_ctx *c, const co_opts *o, const co_defect_opts *dopt, int N,
                           double S0, double dt, int *outer, double *res, int *inner,
                           double *r0) {
    int rc;
    if (o->m < 1 || o->m > CO_MAX_M) return CO_ERR_ARG;
    if ((rc = co_ensure_capacity(c, N, o->m))) return rc;
    if (N == 0) {
        if (outer) *outer = 0;
        if (res) *res = 0;
        if (inner) *inner = 0;
        if (r0) *r0 = 0;
        return CO_OK;
    }
    if (!c->st2 && cudaMalloc(&c->st2, sizeof(co_solver_state)) != cudaSuccess) return CO_ERR_NOMEM;
    co_bufs &b = c->mb;
    if (!b.Gk && cudaMalloc(&b.Gk, 2 * sizeof(double) * b.cap) != cudaSuccess) return CO_ERR_NOMEM;
    if (!b.Phi && cudaMalloc(&b.Phi, 2 * sizeof(double) * b.cap) != cudaSuccess) return CO_ERR_NOMEM;
    if (!b.Adef && cudaMalloc(&b.Adef, 3 * sizeof(double) * b.cap) != cudaSuccess) return CO_ERR_NOMEM;
    const int mo = dopt->outer_m;
    if (mo < 0 || mo > CO_MAX_M) return CO_ERR_ARG;
    const size_t ld2 = 2 * (size_t)b.cap;
    if (mo > 0) {
        if (!c->st3 && cudaMalloc(&c->st3, sizeof(co_solver_state)) != cudaSuccess)
            return CO_ERR_NOMEM;
        if (b.aa && b.aa_m < mo) {
            cudaFree(b.aa);
            b.aa = nullptr;
        }
        if (!b.aa) {
            if (cudaMalloc(&b.aa, sizeof(double) * ld2 * (5 + 2 * (size_t)mo)) != cudaSuccess)
                return CO_ERR_NOMEM;
            b.aa_m = mo;
        }
    }
    const int pcon = dopt->precond;
    if (pcon < 0 || pcon > 2) return CO_ERR_ARG;
    if (pcon && !b.pc && cudaMalloc(&b.pc, 7 * sizeof(double) * b.cap) != cudaSuccess)
        return CO_ERR_NOMEM;
    double *pc_Psi = b.pc, *pc_z = b.pc ? b.pc + ld2 : nullptr,
           *pc_H = b.pc ? b.pc + 2 * ld2 : nullptr;
    double *aa_vk = b.aa, *aa_u = b.aa + ld2, *aa_r = b.aa + 2 * ld2, *aa_rp = b.aa + 3 * ld2,
           *aa_Gp = b.aa + 4 * ld2, *aa_dF = b.aa + 5 * ld2,
           *aa_dG = b.aa + (5 + (size_t)b.aa_m) * ld2;
    const int n2 = 2 * N;
    const size_t ldF = 2 * (size_t)b.cap;
    const int eg = ew_grid(c, n2);
    const int nred = red_blocks(c, N);
    const int gz = o->use_gonzalez;
    co_defect_dev d;
    d.tol = o->tol;
    d.abs_floor = o->abs_floor;
    d.eta = dopt->eta;
    d.stag_rel_tol = o->stag_rel_tol;
    d.stag_window = dopt->stag_window;
    d.fp32_stall = dopt->fp32_stall > 0 ? dopt->fp32_stall : 0.5;
    d.fp32_window = dopt->fp32_window;
    if (d.fp32_window < 0) return CO_ERR_ARG;
    co_dev_opts di = dev_opts(o, 0.0);
    int stage = o->precision != CO_PREC_FP64 ? 1 : 0;
    const int ds = o->precision == CO_PREC_MIXED_DS;  // FP64 stage in double-single
    int max_outer = o->max_iter;
    int total_inner = 0;
    k_state_reset<<<1, 32, 0, c->stream>>>(c->st);
    c->launches++;
    if (mo > 0) {
        k_state_reset<<<1, 32, 0, c->stream>>>(c->st3);
        c->launches++;
    }
    // one inner iteration: G_eff at u, the frozen-metric map Phi(u) and its
    // residual, the Anderson control and update of u (= v1, in place)
    auto inner_iteration = [&](cudaGraphConditionalHandle hnd, int use_cond) -> int {
        int rc;
        if ((rc = landau_geff_dev(c, gz, b.v1, b.v0, N, S0))) return rc;
        // the frozen map, and in its last block the inner control (residual
        // norm, exit test, window bookkeeping, loop condition)
        k_frozen_map<<<nred, CO_RED_THREADS, 0, c->stream>>>(
            N, b.Gv, b.Adef, b.Gk, b.dS, b.dv, b.w, c->st, gz, dt, b.v1, b.Phi, b.r, b.red,
            c->st2, o->m, o->damping, hnd, use_cond, dopt->max_inner,
            c->tickets + CO_TICKET_FROZEN);
        // the map Anderson iterates and its residual: Phi, r -- or, with the
        // preconditioner, Psi = u + P^{-1} r and P^{-1} r
        double *mapv = b.Phi, *res = b.r;
        if (pcon) {
            if ((rc = co_hess_L_dev(c, N, pc_H))) return rc;
            k_precond<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, b.Adef, pc_H, b.w, c->st,
                                                              gz && pcon == 1, dt, b.v1, b.r,
                                                              pc_z, pc_Psi);
            c->launches++;
            mapv = pc_Psi;
            res = pc_z;
        }
        int ng = window_blocks(c, n2);
        k_anderson_cols<<<ng, CO_RED_THREADS, 0, c->stream>>>(n2, c->st2, 0, b.v1, res, b.rp,
                                                              mapv, b.Gp, b.dF, b.dG, ldF,
                                                              b.vbest, b.red, di,
                                                              c->tickets + CO_TICKET_WINDOW);
        k_anderson_update<<<eg, 256, 0, c->stream>>>(n2, c->st2, b.v1, mapv, b.dG, ldF);
        c->launches += 3;
        CO_CK(cudaGetLastError());
        return CO_OK;
    };
    // The inner loop runs on the device: inner_iteration is captured once per
    // call as the body of a conditional WHILE node, and the inner control (the
    // last block of k_frozen_map) ends it when the inner solve exits or
    // max_inner iterations ran. The host launches
    // one graph and waits once per outer iteration instead of once per inner
    // iteration (COLLOPS_INNER_LOOP=host restores the host-driven loop; both
    // run the same kernels on the same data and give identical results).
    const bool host_loop = co_inner_host_loop();
    struct inner_graph {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t e = nullptr;
        unsigned long long body_launches = 0;
        ~inner_graph() {
            if (e) cudaGraphExecDestroy(e);
            if (g) cudaGraphDestroy(g);
        }
    } ig;
    auto capture_inner = [&]() -> int {
        CO_CK(cudaGraphCreate(&ig.g, 0));
        cudaGraphConditionalHandle hnd;
        CO_CK(cudaGraphConditionalHandleCreate(&hnd, ig.g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = hnd;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        CO_CK(cudaGraphAddNode(&node, ig.g, nullptr, nullptr, 0, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        CO_CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
        const unsigned long long l0 = c->launches;
        int r = inner_iteration(hnd, 1);
        ig.body_launches = c->launches - l0;
        cudaError_t ce = cudaStreamEndCapture(c->stream, &body);
        if (r) return r;
        if (ce != cudaSuccess) return CO_ERR_CUDA;
        if (cudaGraphInstantiate(&ig.e, ig.g, 0) != cudaSuccess) return CO_ERR_CUDA;
        return CO_OK;
    };
    int aa_stage = -1;   // pair precision of the outer map the window was built on
    double first_outer = 0.0, prev_outer = 0.0;   // outer residuals (metric_freeze)
    // capped inner solves (co_defect_opts.cap_refresh / cap_abort): whether the
    // last inner solve hit max_inner, how many FP64-stage outer maps in a row
    // ended in a capped inner solve without a new best outer residual, and that best
    bool last_capped = false;
    int capped_run = 0;
    double best_outer64 = INFINITY;
    int k;
    for (k = 1; k <= max_outer; k++) {
        // ---- outer: G_eff(v_k), F (+ A), G(v_k), residual
        if ((rc = landau_geff_dev(c, gz, b.v1, b.v0, N, S0))) return rc;
        k_geff_store<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, b.dS, b.dv, b.w, c->st, gz, b.Gk);
        c->launches++;
        const int m64 = dopt->metric64 && stage == 0 && !ds;
        int prec_pack = (stage == 1 || ds) ? CO_PREC_MIXED : (m64 ? CO_PREC_FP64 : CO_PREC_BOTH);
        if ((rc = co_pack_landau(c, N, N, prec_pack, gz))) return rc;
        if (stage == 1) {
            rc = co_pair_fp32(c, N);
            c->maps32++;
        } else if (ds) {
            rc = co_pair_ds(c, N);
            c->mapsds++;
        } else {
            rc = co_pair_fp64(c, N, m64);   // with_metric: F and A in one FP64 pass
            c->maps64++;
        }
        if (rc) return rc;
        if ((rc = co_unpack_update(c, N, dt, b.Gv, b.v0, b.v1, b.r, b.red))) return rc;
        // the FP32 metric is rebuilt while the previous outer residual is above
        // metric_freeze x the first (always at k = 1)
        const bool new_A = m64 || k == 1 || !(dopt->metric_freeze > 0.0) ||
                           (dopt->cap_refresh && last_capped) ||
                           prev_outer >= dopt->metric_freeze * first_outer;
        if (!m64 && new_A)
            if ((rc = co_metric32(c, N))) return rc;
        if (new_A)
            if ((rc = co_unpack_A(c, N, b.Adef))) return rc;
        k_ctrl_outer<<<1, 256, 0, c->stream>>>(b.red, nred, c->st, d, stage);
        k_defect_best<<<eg, 256, 0, c->stream>>>(n2, c->st, b.Gv, b.vbest);
        c->launches += 2;
        CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                              c->stream));
        CO_CK(cudaStreamSynchronize(c->stream));
        co_prof_collect(c);
        if (c->st_host->error) return c->st_host->error;
        if (c->st_host->done) break;
        int next_stage = stage == 1 ? c->st_host->path : 0;
        const double outer_nrm = c->st_host->nrm_r;
        if (k == 1) first_outer = outer_nrm;
        prev_outer = outer_nrm;
        if (mo > 0)
            CO_CK(cudaMemcpyAsync(aa_vk, b.v1, n2 * sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->stream));
        // ---- inner: Anderson on the frozen-metric map (u = v1 in place)
        k_state_reset<<<1, 32, 0, c->stream>>>(c->st2);
        c->launches++;
        int j;   // inner iterations run (max_inner + 1: the cap was reached)
        if (host_loop) {
            for (j = 1; j <= dopt->max_inner; j++) {
                if ((rc = inner_iteration(0, 0))) return rc;
                CO_CK(cudaMemcpyAsync(c->st_host, c->st2, sizeof(co_solver_state),
                                      cudaMemcpyDeviceToHost, c->stream));
                CO_CK(cudaStreamSynchronize(c->stream));
                if (c->st_host->error) return c->st_host->error;
                if (c->st_host->done) break;
            }
        } else if (dopt->max_inner < 1) {
            j = 1;
        } else {
            if (!ig.e && (rc = capture_inner())) return rc;
            CO_CK(cudaGraphLaunch(ig.e, c->stream));
            CO_CK(cudaMemcpyAsync(c->st_host, c->st2, sizeof(co_solver_state),
                                  cudaMemcpyDeviceToHost, c->stream));
            CO_CK(cudaStreamSynchronize(c->stream));
            if (c->st_host->error) return c->st_host->error;
            const int ran = c->st_host->k;   // the inner control counts every iteration
            c->launches += (unsigned long long)(ran > 1 ? ran - 1 : 0) * ig.body_launches;
            j = c->st_host->done ? ran : dopt->max_inner + 1;
        }
        total_inner += j > dopt->max_inner ? dopt->max_inner : j;
        last_capped = j > dopt->max_inner;
        if (stage == 0) {
            const bool better = outer_nrm < best_outer64;
            if (better) best_outer64 = outer_nrm;
            capped_run = (last_capped && !better) ? capped_run + 1 : 0;
        }
        if (co_verbose())
            fprintf(stderr, "    outer k=%d [%s]  |r|=%.6e  inner +%d%s\n", k,
                    stage == 1 ? "fp32" : ds ? "ds" : "fp64", outer_nrm,
                    j > dopt->max_inner ? dopt->max_inner : j,
                    j > dopt->max_inner ? " (cap)" : "");
        // converged inner solve: u <- Phi(u) (solver.jl:501-503)
        k_copy_if_done<<<eg, 256, 0, c->stream>>>(n2, c->st2, 1, b.v1, b.Phi);
        c->launches++;
        if (mo > 0) {
            // v_{k+1} from the window of outer pairs (v_j, D(v_j))
            k_ctrl_aa<<<1, 32, 0, c->stream>>>(c->st3, c->st, mo, stage != aa_stage);
            aa_stage = stage;
            k_aa_resid<<<eg, 256, 0, c->stream>>>(n2, c->st, b.v1, aa_vk, aa_u, aa_r);
            int ng = window_blocks(c, n2);
            k_anderson_cols<<<ng, CO_RED_THREADS, 0, c->stream>>>(n2, c->st3, 0, aa_vk, aa_r,
                                                                  aa_rp, aa_u, aa_Gp, aa_dF,
                                                                  aa_dG, ld2, b.vbest, b.red, di,
                                                                  c->tickets + CO_TICKET_WINDOW);
            k_anderson_update<<<eg, 256, 0, c->stream>>>(n2, c->st3, aa_vk, aa_u, aa_dG, ld2);
            c->launches += 4;
            CO_CK(cudaMemcpyAsync(b.v1, aa_vk, n2 * sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->stream));
        }
        stage = next_stage;
        // cap_abort: the FP64-stage outer iteration has stopped improving while
        // its inner solves no longer converge; leave through the stagnation exit
        // (best iterate) at once instead of after the stagnation window
        if (dopt->cap_abort > 0 && capped_run >= dopt->cap_abort) {
            k_set_done<<<1, 32, 0, c->stream>>>(c->st, 2);
            c->launches++;
            c->st_host->done = 2;
            break;
        }
    }
    if (co_verbose())
        fprintf(stderr, "    outer k=%d  |r|=%.6e  [%s]\n", k > max_outer ? max_outer : k,
                c->st_host->nrm_r,
                c->st_host->done == 1 ? "converged" : c->st_host->done == 2 ? "stagnated" : "cap");
    if (k > max_outer) {
        k_set_done<<<1, 32, 0, c->stream>>>(c->st, 3);
        c->launches++;
    }
    // exit: converged -> G(v); stagnated / cap -> best G(v) (solver.jl:611, :617, :631)
    k_copy_if_done<<<eg, 256, 0, c->stream>>>(n2, c->st, 1, b.v1, b.Gv);
    k_copy_if_done<<<eg, 256, 0, c->stream>>>(n2, c->st, 2, b.v1, b.vbest);
    k_copy_if_done<<<eg, 256, 0, c->stream>>>(n2, c->st, 3, b.v1, b.vbest);
    c->launches += 3;
    CO_CK(cudaGetLastError());
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    if (c->st_host->error) return c->st_host->error;
    if (outer) *outer = k > max_outer ? max_outer : k;
    if (res) *res = c->st_host->done == 1 ? c->st_host->nrm_r : c->st_host->nrm_best;
    if (inner) *inner = total_inner;
    if (r0) *r0 = c->st_host->nrm_r0;
    return CO_OK;
}

// ================================================================ batch engine
//
// Many independent ensembles (Landau or LB, different N and meshes) advance
// together: one context per instance, all on one stream; per Picard iteration
// every instance's O(N) stage, ONE persistent launch of the batched symmetric
// FP64 pair kernel for all Landau instances, and every instance's Anderson
// control. The iteration is captured once per time step as a CUDA graph and
// replayed until every instance has exited; converged instances are skipped by
// the pair kernel and their state no longer changes. Tile width, chunk size and
// grid size of the pair kernel are chosen by timing candidates on the batch's
// own data (co_batch_tune).

struct co_batch {
    int device;
    cudaStream_t stream;
    int n;
    std::vector<co_ctx *> ctx;
    std::vector<int> N, model;
    std::vector<double> nu;
    std::vector<size_t> off;          // marker offset of each instance in concatenated arrays
    co_solver_state *st_all;          // device, n states
    int *d_loop;                      // device: [0] iterations of the current device loop,
                                      // [1..] the live instances it covers
    co_solver_state *st_host;         // pinned
    co_bwork *d_tab;
    std::vector<co_bwork> tab;
    unsigned *d_counter;
    int total, max_pos;
    std::vector<int> live;            // instances still iterating (table and graph cover these)
    // the O(N) stages of different instances are independent: an iteration forks
    // them over aux streams (joined around the batched pair launch)
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> ev_join1, ev_join2;
    cudaEvent_t ev_fork1, ev_fork2;
    int W, KC, grid, tuned;
    double tune_ms;
    int nsm;
};

__global__ void k_finish_once(int n2, co_solver_state *st, int exit_picard, double *__restrict__ v1,
                              const double *__restrict__ Gv, const double *__restrict__ vbest) {
    if (!st->done || st->finished) return;
    int done = st->done, improved = st->improved;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        if (done == 1) {
            if (exit_picard) v1[i] = Gv[i];
        } else if (done == 2) {
            v1[i] = improved ? (exit_picard ? Gv[i] : v1[i]) : vbest[i];
        } else if (done == 3) {
            v1[i] = vbest[i];
        }
    }
}

__global__ void k_mark_finished(co_solver_state *st) {
    if (threadIdx.x == 0 && st->done) st->finished = 1;
}

// work table of the batched pair kernel over the live instances (B->live)
static int batch_rebuild_table(co_batch *B) {
    const int n = (int)B->live.size();
    if (n == 0) {
        B->total = 0;
        return CO_OK;
    }
    std::vector<co_ctx *> cs(n);
    std::vector<const co_solver_state *> sts(n);
    for (int j = 0; j < n; j++) {
        cs[j] = B->ctx[B->live[j]];
        sts[j] = B->st_all + B->live[j];
    }
    B->tab.resize(n + 1);
    int mp = 0;
    int total = co_batch_work_table(cs.data(), sts.data(), n, B->W, B->KC, B->tab.data(), &mp);
    if (total < 0) return -total;
    B->tab[n] = B->tab[n - 1];
    B->tab[n].blk0 = total;  // sentinel
    B->total = total;
    B->max_pos = mp;
    CO_CK(cudaMemcpyAsync(B->d_tab, B->tab.data(), sizeof(co_bwork) * (n + 1),
                          cudaMemcpyHostToDevice, B->stream));
    CO_CK(cudaStreamSynchronize(B->stream));
    return CO_OK;
}

extern "C" int co_batch_create(const co_batch_instance *inst, int n, int n_quad, unsigned flags,
                               int device, co_batch **out) {
    if (!out || !inst || n < 1) return CO_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CO_ERR_NODEVICE;
    if (device < 0 || device >= ndev) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(device));
    co_batch *B = new co_batch();
    B->device = device;
    B->n = n;
    B->W = 4;
    B->KC = 8;
    B->tuned = 0;
    B->tune_ms = 0;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    B->nsm = prop.multiProcessorCount;
    B->grid = 4 * B->nsm;
    int rc = CO_OK;
    if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete B;
        return CO_ERR_CUDA;
    }
    B->ev_fork1 = B->ev_fork2 = nullptr;
    {
        const int n_aux = n < 8 ? n : 8;
        bool ok = cudaEventCreateWithFlags(&B->ev_fork1, cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&B->ev_fork2, cudaEventDisableTiming) == cudaSuccess;
        for (int j = 0; ok && j < n_aux; j++) {
            cudaStream_t st;
            cudaEvent_t e1, e2;
            ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
            if (ok) B->aux.push_back(st);
            ok = ok && cudaEventCreateWithFlags(&e1, cudaEventDisableTiming) == cudaSuccess;
            if (ok) B->ev_join1.push_back(e1);
            ok = ok && cudaEventCreateWithFlags(&e2, cudaEventDisableTiming) == cudaSuccess;
            if (ok) B->ev_join2.push_back(e2);
        }
        if (!ok) {
            co_batch_destroy(B);
            return CO_ERR_CUDA;
        }
    }
    if (cudaMalloc(&B->st_all, sizeof(co_solver_state) * n) != cudaSuccess ||
        cudaMallocHost(&B->st_host, sizeof(co_solver_state) * n) != cudaSuccess ||
        cudaMalloc(&B->d_tab, sizeof(co_bwork) * (n + 1)) != cudaSuccess ||
        cudaMalloc(&B->d_counter, 64) != cudaSuccess ||
        cudaMalloc(&B->d_loop, sizeof(int) * (n + 1)) != cudaSuccess) {
        co_batch_destroy(B);
        return CO_ERR_NOMEM;
    }
    cudaMemset(B->st_all, 0, sizeof(co_solver_state) * n);
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        const co_batch_instance &d = inst[i];
        if (d.N < 0 || (d.model != CO_MODEL_LANDAU && d.model != CO_MODEL_LB)) {
            co_batch_destroy(B);
            return CO_ERR_ARG;
        }
        co_ctx *c = nullptr;
        rc = co_ctx_create(d.bp1, d.nb1, d.bp2, d.nb2, 2, n_quad, flags, device, &c);
        if (rc) {
            co_batch_destroy(B);
            return rc;
        }
        // join the batch: shared stream and state array
        cudaStreamDestroy(c->stream);
        c->stream = B->stream;
        cudaFree(c->st);
        c->st = B->st_all + i;
        c->lb_two_pass = 1;
        c->batch_N = d.N;
        c->batch_landau = d.model == CO_MODEL_LANDAU;
        B->ctx.push_back(c);
        B->N.push_back(d.N);
        B->model.push_back(d.model);
        B->nu.push_back(d.nu);
        B->off.push_back(off);
        off += (size_t)d.N;
        if ((rc = co_ensure_capacity(c, d.N, CO_MAX_M))) {
            co_batch_destroy(B);
            return rc;
        }
    }
    for (int i = 0; i < n; i++)
        if (B->N[i] > 0) B->live.push_back(i);
    if ((rc = batch_rebuild_table(B))) {
        co_batch_destroy(B);
        return rc;
    }
    *out = B;
    return CO_OK;
}

extern "C" int co_batch_destroy(co_batch *B) {
    if (!B) return CO_ERR_ARG;
    cudaSetDevice(B->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    for (co_ctx *c : B->ctx) {
        c->st = nullptr;           // owned by the batch
        c->stream = nullptr;       // shared
        co_ctx_destroy_detached(c);
    }
    if (B->st_all) cudaFree(B->st_all);
    if (B->d_loop) cudaFree(B->d_loop);
    if (B->st_host) cudaFreeHost(B->st_host);
    if (B->d_tab) cudaFree(B->d_tab);
    if (B->d_counter) cudaFree(B->d_counter);
    for (cudaStream_t st : B->aux) cudaStreamDestroy(st);
    for (cudaEvent_t e : B->ev_join1) cudaEventDestroy(e);
    for (cudaEvent_t e : B->ev_join2) cudaEventDestroy(e);
    if (B->ev_fork1) cudaEventDestroy(B->ev_fork1);
    if (B->ev_fork2) cudaEventDestroy(B->ev_fork2);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
    return CO_OK;
}

// everything of one iteration up to the pair sum (Landau) or the whole map (LB)
static int batch_pre(co_batch *B, int i, const co_opts *o, double S0i, double dt, int *nred) {
    co_ctx *c = B->ctx[i];
    co_bufs &b = c->mb;
    int N = B->N[i], rc;
    if (N == 0) return CO_OK;
    if (B->model[i] == CO_MODEL_LB)
        return picard_map_impl(c, CO_MODEL_LB, o->use_gonzalez, B->nu[i], CO_PREC_FP64, b.Gv, b.v1,
                               b.v0, N, S0i, dt, b.r, nred);
    *nred = red_blocks(c, N);
    if ((rc = landau_geff_dev(c, o->use_gonzalez, b.v1, b.v0, N, S0i))) return rc;
    return co_pack_landau(c, N, N, CO_PREC_FP64, o->use_gonzalez);
}

// fork: every aux stream waits for the main stream's work so far
static int batch_fork(co_batch *B, cudaEvent_t ev) {
    CO_CK(cudaEventRecord(ev, B->stream));
    for (cudaStream_t st : B->aux) CO_CK(cudaStreamWaitEvent(st, ev, 0));
    return CO_OK;
}
// join: the main stream waits for every aux stream
static int batch_join(co_batch *B, std::vector<cudaEvent_t> &ev) {
    for (size_t j = 0; j < B->aux.size(); j++) {
        CO_CK(cudaEventRecord(ev[j], B->aux[j]));
        CO_CK(cudaStreamWaitEvent(B->stream, ev[j], 0));
    }
    return CO_OK;
}

// one Picard iteration of the live instances: their O(N) stages (instance j of
// the live set on aux stream j mod K), one batched pair-sum launch on the main
// stream, their Anderson updates (aux streams again)
static int batch_iteration_impl(co_batch *B, const co_opts *o, const double *S0, double dt,
                                const co_dev_opts &d) {
    int rc;
    std::vector<int> nred(B->n, 1);
    const size_t K = B->aux.size();
    if ((rc = batch_fork(B, B->ev_fork1))) return rc;
    for (size_t j = 0; j < B->live.size(); j++) {
        const int i = B->live[j];
        B->ctx[i]->stream = B->aux[j % K];
        if ((rc = batch_pre(B, i, o, S0[i], dt, &nred[i]))) return rc;
    }
    if ((rc = batch_join(B, B->ev_join1))) return rc;
    if ((rc = co_pair64_batch(B->stream, B->d_tab, (int)B->live.size(), B->total, B->W, B->KC,
                              B->grid, B->d_counter, B->max_pos)))
        return rc;
    if ((rc = batch_fork(B, B->ev_fork2))) return rc;
    for (int i : B->live) {
        co_ctx *c = B->ctx[i];
        co_bufs &b = c->mb;
        int N = B->N[i];
        if (N == 0) continue;
        if (B->model[i] == CO_MODEL_LANDAU)
            if ((rc = co_unpack_update(c, N, dt, b.Gv, b.v0, b.v1, b.r, b.red))) return rc;
        int n2 = 2 * N, eg = ew_grid(c, n2);
        size_t ldF = 2 * (size_t)b.cap;
        cudaStream_t cs = c->stream;
        k_ctrl1<<<1, 256, 0, cs>>>(b.red, nred[i], c->st, d);
        int ng = window_blocks(c, n2);
        k_anderson_cols<<<ng, CO_RED_THREADS, 0, cs>>>(n2, c->st, o->exit_picard_step, b.v1, b.r,
                                                       b.rp, b.Gv, b.Gp, b.dF, b.dG, ldF, b.vbest,
                                                       b.red, d, c->tickets + CO_TICKET_WINDOW);
        k_anderson_update<<<eg, 256, 0, cs>>>(n2, c->st, b.v1, b.Gv, b.dG, ldF);
        k_finish_once<<<eg, 256, 0, cs>>>(n2, c->st, o->exit_picard_step, b.v1, b.Gv, b.vbest);
        k_mark_finished<<<1, 32, 0, cs>>>(c->st);
        c->launches += 5;
    }
    if ((rc = batch_join(B, B->ev_join2))) return rc;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// Condition of the device-side iteration loop of the batch engine: one more
// iteration while every instance the loop covers is still running and the
// loop has done fewer than `cap` iterations. The loop ends on the device as
// soon as any instance finishes, so the host only wakes to shrink the live set.
__global__ void k_batch_continue(cudaGraphConditionalHandle h, const co_solver_state *st_all,
                                 int *loop, int nlive, int cap) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int k = ++loop[0];
    unsigned go = k < cap ? 1u : 0u;
    for (int j = 0; j < nlive && go; j++) {
        const co_solver_state &st = st_all[loop[1 + j]];
        if (st.finished || st.error) go = 0u;
    }
    cudaGraphSetConditional(h, go);
}

static int batch_iteration(co_batch *B, const co_opts *o, const double *S0, double dt,
                           const co_dev_opts &d) {
    int rc = batch_iteration_impl(B, o, S0, dt, d);
    for (co_ctx *c : B->ctx) c->stream = B->stream;   // every context back on the main stream
    return rc;
}

extern "C" int co_batch_tune(co_batch *B, int *W, int *KC, int *grid, double *best_ms) {
    if (!B) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(B->device));
    B->live.clear();   // the tuner times the pair sum of every instance
    for (int i = 0; i < B->n; i++)
        if (B->N[i] > 0) B->live.push_back(i);
    // candidates: tile width, chunk of tile pairs, persistent blocks per SM
    const int Ws[] = {4, 8};
    const int KCs[] = {4, 16};
    const int mults[] = {2, 8};
    cudaEvent_t e0, e1;
    CO_CK(cudaEventCreate(&e0));
    CO_CK(cudaEventCreate(&e1));
    double best = 1e30;
    int bW = B->W, bK = B->KC, bG = B->grid;
    for (int w : Ws)
        for (int kc : KCs)
            for (int m : mults) {
                B->W = w;
                B->KC = kc;
                B->grid = m * B->nsm;
                int rc = batch_rebuild_table(B);
                if (rc) return rc;
                CO_CK(cudaEventRecord(e0, B->stream));
                rc = co_pair64_batch(B->stream, B->d_tab, (int)B->live.size(), B->total, B->W,
                                     B->KC, B->grid, B->d_counter, B->max_pos);
                if (rc) return rc;
                CO_CK(cudaEventRecord(e1, B->stream));
                CO_CK(cudaEventSynchronize(e1));
                float ms = 0.f;
                CO_CK(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best) {
                    best = ms;
                    bW = w;
                    bK = kc;
                    bG = B->grid;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->W = bW;
    B->KC = bK;
    B->grid = bG;
    B->tuned = 1;
    B->tune_ms = best;
    int rc = batch_rebuild_table(B);
    if (rc) return rc;
    if (W) *W = bW;
    if (KC) *KC = bK;
    if (grid) *grid = bG;
    if (best_ms) *best_ms = best;
    return CO_OK;
}

// concatenated device arrays: instance i's markers are v_all[2*off_i .. 2*off_i + 2*N_i)
// (its own N x 2 column-major block) and w_all[off_i .. off_i + N_i)
extern "C" int co_batch_step_dev(co_batch *B, const co_opts *o, double *v1_all,
                                 const double *v0_all, const double *w_all, const double *S0,
                                 double dt, int use_graph, int *iters, double *res) {
    if (!B || !o || !v1_all || !v0_all || !w_all || !S0) return CO_ERR_ARG;
    if (o->m < 1 || o->m > CO_MAX_M || o->precision != CO_PREC_FP64) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(B->device));
    int rc;
    for (int i = 0; i < B->n; i++) {
        co_ctx *c = B->ctx[i];
        size_t n2 = 2 * (size_t)B->N[i] * sizeof(double);
        CO_CK(cudaMemcpyAsync(c->mb.v1, v1_all + 2 * B->off[i], n2, cudaMemcpyDeviceToDevice,
                              B->stream));
        CO_CK(cudaMemcpyAsync(c->mb.v0, v0_all + 2 * B->off[i], n2, cudaMemcpyDeviceToDevice,
                              B->stream));
        CO_CK(cudaMemcpyAsync(c->mb.w, w_all + B->off[i], (size_t)B->N[i] * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
        k_state_reset<<<1, 32, 0, B->stream>>>(c->st);
    }
    co_dev_opts d = dev_opts(o, 0.0);
    B->live.clear();
    for (int i = 0; i < B->n; i++)
        if (B->N[i] > 0) B->live.push_back(i);
    if (!B->tuned) {
        // pack every instance once at the initial guess, then time the candidates
        std::vector<int> nred(B->n);
        for (int i = 0; i < B->n; i++)
            if (B->model[i] == CO_MODEL_LANDAU)
                if ((rc = batch_pre(B, i, o, S0[i], dt, &nred[i]))) return rc;
        if ((rc = co_batch_tune(B, nullptr, nullptr, nullptr, nullptr))) return rc;
    } else if ((rc = batch_rebuild_table(B))) {
        return rc;
    }
    // The iteration of the live instances as a CUDA graph whose body repeats on
    // the device (a conditional WHILE node; k_batch_continue decides) until an
    // instance finishes or the cap is reached. The host then reads the states
    // once, drops finished instances from the live set and re-captures, so
    // finished instances cost nothing per iteration and the host waits once per
    // change of the live set, not once per iteration.
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    auto capture = [&](int cap) -> int {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        CO_CK(cudaStreamSynchronize(B->stream));
        std::vector<int> hl(1 + B->live.size(), 0);
        for (size_t j = 0; j < B->live.size(); j++) hl[1 + j] = B->live[j];
        CO_CK(cudaMemcpy(B->d_loop, hl.data(), sizeof(int) * hl.size(), cudaMemcpyHostToDevice));
        CO_CK(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle hnd;
        CO_CK(cudaGraphConditionalHandleCreate(&hnd, graph, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = hnd;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        CO_CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        CO_CK(cudaStreamBeginCaptureToGraph(B->stream, body, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeThreadLocal));
        int r = batch_iteration(B, o, S0, dt, d);
        if (!r) {
            k_batch_continue<<<1, 32, 0, B->stream>>>(hnd, B->st_all, B->d_loop,
                                                      (int)B->live.size(), cap);
            if (cudaGetLastError() != cudaSuccess) r = CO_ERR_CUDA;
        }
        cudaError_t ce = cudaStreamEndCapture(B->stream, &body);
        if (r) return r;
        if (ce != cudaSuccess) return CO_ERR_CUDA;
        if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) return CO_ERR_CUDA;
        return CO_OK;
    };
    if (use_graph && (rc = capture(o->max_iter))) {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    int k = 0;           // iterations done
    while (k < o->max_iter) {
        int ran = 1;
        if (use_graph) {
            if (cudaMemsetAsync(B->d_loop, 0, sizeof(int), B->stream) != cudaSuccess ||
                cudaGraphLaunch(exec, B->stream) != cudaSuccess ||
                cudaMemcpyAsync(&ran, B->d_loop, sizeof(int), cudaMemcpyDeviceToHost,
                                B->stream) != cudaSuccess) {
                rc = CO_ERR_CUDA;
                break;
            }
        } else if ((rc = batch_iteration(B, o, S0, dt, d))) {
            break;
        }
        if (cudaMemcpyAsync(B->st_host, B->st_all, sizeof(co_solver_state) * B->n,
                            cudaMemcpyDeviceToHost, B->stream) != cudaSuccess ||
            cudaStreamSynchronize(B->stream) != cudaSuccess) {
            rc = CO_ERR_CUDA;
            break;
        }
        k += ran;
        std::vector<int> still;
        for (int i : B->live) {
            if (B->st_host[i].error) rc = B->st_host[i].error;
            if (!B->st_host[i].finished) still.push_back(i);
        }
        if (rc || still.empty() || k >= o->max_iter) break;
        if (still.size() < B->live.size()) {
            B->live.swap(still);
            if ((rc = batch_rebuild_table(B))) break;
            if (use_graph && (rc = capture(o->max_iter - k))) break;
        }
    }
    if (k >= o->max_iter) k = o->max_iter + 1;   // the cap: best iterates below
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
    // instances still running hit the iteration cap: best iterate (solver.jl:419-422)
    for (int i = 0; i < B->n; i++) {
        co_ctx *c = B->ctx[i];
        int N = B->N[i];
        if (N == 0) continue;
        int n2 = 2 * N, eg = ew_grid(c, n2);
        k_set_done<<<1, 32, 0, B->stream>>>(c->st, 3);
        k_finish_once<<<eg, 256, 0, B->stream>>>(n2, c->st, o->exit_picard_step, c->mb.v1,
                                                 c->mb.Gv, c->mb.vbest);
        k_mark_finished<<<1, 32, 0, B->stream>>>(c->st);
        CO_CK(cudaMemcpyAsync(v1_all + 2 * B->off[i], c->mb.v1, 2 * (size_t)N * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
    }
    CO_CK(cudaMemcpyAsync(B->st_host, B->st_all, sizeof(co_solver_state) * B->n,
                          cudaMemcpyDeviceToHost, B->stream));
    CO_CK(cudaStreamSynchronize(B->stream));
    for (int i = 0; i < B->n; i++) {
        const co_solver_state &s = B->st_host[i];
        if (iters) iters[i] = (s.done == 3) ? (k > o->max_iter ? o->max_iter : s.k) : s.k;
        if (res) res[i] = s.res_out;
    }
    return CO_OK;
}

// batch predictor and entropies (per instance, on the batch stream)
extern "C" int co_batch_predictor_dev(co_batch *B, const co_opts *o, double *v1_all,
                                      const double *v_all, const double *w_all, double dt) {
    if (!B || !o || !v1_all || !v_all || !w_all) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(B->device));
    int rc;
    for (int i = 0; i < B->n; i++) {
        co_ctx *c = B->ctx[i];
        int N = B->N[i];
        if (N == 0) continue;
        co_opts oi = *o;
        oi.model = B->model[i];
        oi.nu = B->nu[i];
        CO_CK(cudaMemcpyAsync(c->mb.v0, v_all + 2 * B->off[i], 2 * (size_t)N * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
        CO_CK(cudaMemcpyAsync(c->mb.w, w_all + B->off[i], (size_t)N * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
        if ((rc = co_predictor_buffers(c, &oi, CO_PREC_FP64, c->mb.v0, N, dt, c->mb.v1))) return rc;
        CO_CK(cudaMemcpyAsync(v1_all + 2 * B->off[i], c->mb.v1, 2 * (size_t)N * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
    }
    CO_CK(cudaStreamSynchronize(B->stream));
    return CO_OK;
}

extern "C" int co_batch_entropy_dev(co_batch *B, const double *v_all, const double *w_all,
                                    double *S) {
    if (!B || !v_all || !w_all || !S) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(B->device));
    int rc;
    for (int i = 0; i < B->n; i++) {
        co_ctx *c = B->ctx[i];
        int N = B->N[i];
        CO_CK(cudaMemcpyAsync(c->mb.w, w_all + B->off[i], (size_t)N * sizeof(double),
                              cudaMemcpyDeviceToDevice, B->stream));
        if ((rc = co_sort_markers(c, v_all + 2 * B->off[i], N))) return rc;
        if ((rc = co_project_sorted(c, c->f))) return rc;
        if ((rc = co_entropy_parts_dev(c, c->f))) return rc;
        if ((rc = co_entropy_finalize_dev(c, c->y))) return rc;
        CO_CK(cudaMemcpyAsync(S + i, c->y, sizeof(double), cudaMemcpyDeviceToHost, B->stream));
    }
    CO_CK(cudaStreamSynchronize(B->stream));
    return CO_OK;
}

extern "C" int co_batch_launch_count(const co_batch *B, unsigned long long *l) {
    if (!B || !l) return CO_ERR_ARG;
    unsigned long long s = 0;
    for (co_ctx *c : B->ctx) s += c->launches;
    *l = s;
    return CO_OK;
}

// ================================================================ warm start

__global__ void k_dotv_from(int n2, const double *__restrict__ v1, const double *__restrict__ v0,
                            double inv_dt, double *__restrict__ dotv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n2) dotv[i] = (v1[i] - v0[i]) * inv_dt;
}

__global__ void k_ws_apply(int N, const double *__restrict__ vp, const float *__restrict__ Y,
                           double dt2, double s0, double s1, double h0, double h1,
                           double *__restrict__ v1) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    v1[a] = vp[a] + dt2 * ((double)Y[2 * (size_t)a] * s0 + h0);
    v1[N + a] = vp[N + a] + dt2 * ((double)Y[2 * (size_t)a + 1] * s1 + h1);
}

// The warm start compares first residuals (order 1 against tol ~1e-10): the
// mixed forms take them on the FP32 pair map.
static int ws_prec(int precision) {
    return precision == CO_PREC_FP64 ? CO_PREC_FP64 : CO_PREC_MIXED;
}

extern "C" int co_warmstart_features_dev(co_ctx *c, const co_opts *o, const double *v,
                                         const double *w, int N, double S0, double dt,
                                         double *v_pred, float *X, double *res_pred) {
    if (!c || !o || N < 0 || (N > 0 && (!v || !w || !v_pred || !X))) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(c->device));
    int rc;
    if ((rc = co_ensure_capacity(c, N, 1))) return rc;
    if (res_pred) *res_pred = 0.0;
    if (N == 0) return CO_OK;
    co_bufs &b = c->mb;
    if (!b.pc && cudaMalloc(&b.pc, 7 * sizeof(double) * b.cap) != cudaSuccess) return CO_ERR_NOMEM;
    if (!b.Adef && cudaMalloc(&b.Adef, 3 * sizeof(double) * b.cap) != cudaSuccess)
        return CO_ERR_NOMEM;
    double *H = b.pc + 4 * (size_t)b.cap;   // 3N: the Hessian of L at v
    CO_CK(cudaMemcpyAsync(b.v0, v, 2 * (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    const int pp = ws_prec(o->precision);
    if ((rc = co_predictor_buffers(c, o, pp, b.v0, N, dt, b.v1))) return rc;
    if (o->model == CO_MODEL_LB) {
        // dotv of the LB predictor: (v1 - v)/dt is what Gv holds; use it directly
        k_dotv_from<<<co_cdiv(2LL * N, 256), 256, 0, c->stream>>>(2 * N, b.v1, b.v0, 1.0 / dt,
                                                                  b.dotv);
        c->launches++;
        // no entropy potential L in the LB map: no Hessian and no pair metric
        CO_CK(cudaMemsetAsync(H, 0, 3 * (size_t)N * sizeof(double), c->stream));
        CO_CK(cudaMemsetAsync(b.Adef, 0, 3 * (size_t)N * sizeof(double), c->stream));
    } else {
        // the local stiffness factors at v (v's sort, L and G are still current):
        // the Hessian of L and the FP32 pair metric A
        if ((rc = co_hess_L_dev(c, N, H))) return rc;
        if ((rc = co_pack_plain(c, N, N, CO_PREC_MIXED, b.v0, b.G))) return rc;
        if ((rc = co_metric32(c, N))) return rc;
        if ((rc = co_unpack_A(c, N, b.Adef))) return rc;
    }
    if ((rc = co_features_dev(c, N, H, b.Adef, X))) return rc;
    // the predictor's first residual r = G(v_pred) - v_pred, per marker and its norm
    int nred = 0;
    if ((rc = picard_map_impl(c, o->model, o->use_gonzalez, o->nu, pp, b.Gv, b.v1, b.v0, N, S0, dt,
                              b.r, &nred)))
        return rc;
    if ((rc = co_features_res_dev(c, N, b.r, dt, X))) return rc;
    co_dev_opts d = dev_opts(o, 0.0);
    k_state_reset<<<1, 32, 0, c->stream>>>(c->st);
    k_ctrl1<<<1, 256, 0, c->stream>>>(b.red, nred, c->st, d);
    c->launches += 2;
    CO_CK(cudaMemcpyAsync(v_pred, b.v1, 2 * (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    if (res_pred) *res_pred = c->st_host->nrm_r;
    return c->st_host->error ? c->st_host->error : CO_OK;
}

extern "C" int co_warmstart_apply_dev(co_ctx *c, const double *v_pred, const float *Y, int N,
                                      double dt, const double *scale2, const double *shift2,
                                      double *v1) {
    if (!c || N < 0 || (N > 0 && (!v_pred || !Y || !v1 || !scale2 || !shift2))) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(c->device));
    if (N == 0) return CO_OK;
    k_ws_apply<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, v_pred, Y, dt * dt, scale2[0], scale2[1],
                                                       shift2[0], shift2[1], v1);
    c->launches++;
    CO_CK(cudaGetLastError());
    CO_CK(cudaStreamSynchronize(c->stream));
    return CO_OK;
}

extern "C" int co_picard_residual_dev(co_ctx *c, const co_opts *o, const double *v_in,
                                      const double *v0, const double *w, int N, double S0,
                                      double dt, double *res) {
    if (!c || !o || !res || N < 0 || (N > 0 && (!v_in || !v0 || !w))) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(c->device));
    int rc;
    if ((rc = co_ensure_capacity(c, N, 1))) return rc;
    *res = 0.0;
    if (N == 0) return CO_OK;
    co_bufs &b = c->mb;
    size_t n2 = 2 * (size_t)N * sizeof(double);
    CO_CK(cudaMemcpyAsync(b.vin, v_in, n2, cudaMemcpyDeviceToDevice, c->stream));
    CO_CK(cudaMemcpyAsync(b.v0, v0, n2, cudaMemcpyDeviceToDevice, c->stream));
    CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    int nred = 0;
    if ((rc = picard_map_impl(c, o->model, o->use_gonzalez, o->nu, ws_prec(o->precision), b.Gv,
                              b.vin, b.v0, N, S0, dt, b.r, &nred)))
        return rc;
    co_dev_opts d = dev_opts(o, 0.0);
    k_state_reset<<<1, 32, 0, c->stream>>>(c->st);
    k_ctrl1<<<1, 256, 0, c->stream>>>(b.red, nred, c->st, d);
    c->launches += 2;
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    *res = c->st_host->nrm_r;
    return c->st_host->error ? c->st_host->error : CO_OK;
}
