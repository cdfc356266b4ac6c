// co_step.cu -- one whole time step of the headline form behind one call.
//
// The reference's time loop (main.jl:233-271) runs the explicit predictor, an
// optional network correction of it (nn_warmstart_correct!, main.jl:252-254)
// and the implicit solver (step_anderson! or step_defect!, main.jl:256-271).
// co_step_learned does all of that on the device:
//
//   1. features of the step and the explicit predictor v_pred with its first
//      residual ||G(v_pred) - v_pred|| (co_warmstart_features_dev);
//   2. the network (normalisation folded into k_mlp_forward) and the learned
//      proposal v_learn = v_pred + dt^2 delta with its first residual;
//   3. the previous-step state v itself as a third start: G(v) is v_pred, so
//      its first residual is ||v_pred - v||, with no extra map;
//   4. the implicit solve from the start with the smallest first residual, the
//      unmodified fixed-point map judging convergence;
//   5. if that solve stagnates (or hits its cap), one more solve from the next
//      start, keeping the result with the smaller residual;
//   6. the entropy of the new state's projection, the next step's S0.
//
// The host only sequences launches and reads scalars (first residuals, the
// solver state); marker data stays on the device.
#include <math.h>

#include "co_internal.cuh"
#include "co_reduce.cuh"

int co_step_anderson_buffers(co_ctx *c, const co_opts *o, int N, double S0, double dt,
                             int *iters, double *res, int *nrs, double *r0);

#define CO_STEP_RED 256   // blocks of the norm reduction

struct co_step_bufs {
    int cap;
    float *X, *Y;            // features (N x 15) and network output (N x 2)
    double *vp, *vl, *keep;  // predictor, learned proposal, kept result (2N each)
    double *hv, *hw;         // staging of host inputs (2N, N)
    double *red;             // CO_STEP_RED partials + 1 result
};

void co_step_free(co_ctx *c) {
    co_step_bufs *s = c->sb;
    if (!s) return;
    void *p[] = {s->X, s->Y, s->vp, s->vl, s->keep, s->hv, s->hw, s->red};
    for (void *q : p)
        if (q) cudaFree(q);
    free(s);
    c->sb = nullptr;
}

static int step_ensure(co_ctx *c, int N) {
    if (!c->sb) {
        c->sb = (co_step_bufs *)calloc(1, sizeof(co_step_bufs));
        if (!c->sb) return CO_ERR_NOMEM;
    }
    co_step_bufs *s = c->sb;
    if (N <= s->cap && s->red) return CO_OK;
    int cap = N > s->cap ? N : s->cap;
    if (cap < 1) cap = 1;
    void *p[] = {s->X, s->Y, s->vp, s->vl, s->keep, s->hv, s->hw, s->red};
    for (void *q : p)
        if (q) cudaFree(q);
    memset(s, 0, sizeof(*s));
    const size_t n2 = 2 * (size_t)cap * sizeof(double);
    if (cudaMalloc(&s->X, sizeof(float) * CO_WS_NFEAT * (size_t)cap) != cudaSuccess ||
        cudaMalloc(&s->Y, sizeof(float) * 2 * (size_t)cap) != cudaSuccess ||
        cudaMalloc(&s->vp, n2) != cudaSuccess || cudaMalloc(&s->vl, n2) != cudaSuccess ||
        cudaMalloc(&s->keep, n2) != cudaSuccess || cudaMalloc(&s->hv, n2) != cudaSuccess ||
        cudaMalloc(&s->hw, sizeof(double) * (size_t)cap) != cudaSuccess ||
        cudaMalloc(&s->red, sizeof(double) * (CO_STEP_RED + 1)) != cudaSuccess)
        return CO_ERR_NOMEM;
    s->cap = cap;
    return CO_OK;
}

// ||a - b||^2 over n entries: block partials, then one block sums them in order
__global__ void __launch_bounds__(256)
k_diff_sq(int n, const double *__restrict__ a, const double *__restrict__ b,
          double *__restrict__ red) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = a[i] - b[i];
        s = fma(d, d, s);
    }
    s = co_block_sum(s, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_red_final(int nb, double *__restrict__ red) {
    __shared__ double sh[32];
    double s = co_sum_partials(red, nb, 1, 0, sh);
    if (threadIdx.x == 0) red[CO_STEP_RED] = s;
}

__global__ void k_apply_delta(int N, const double *__restrict__ vp, const float *__restrict__ Y,
                              double dt2, double *__restrict__ v1) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    v1[a] = vp[a] + dt2 * (double)Y[2 * (size_t)a];
    v1[N + a] = vp[N + a] + dt2 * (double)Y[2 * (size_t)a + 1];
}

static int diff_norm(co_ctx *c, int n, const double *a, const double *b, double *out) {
    co_step_bufs *s = c->sb;
    int g = co_cdiv(n, 256);
    if (g > CO_STEP_RED) g = CO_STEP_RED;
    if (g < 1) g = 1;
    k_diff_sq<<<g, 256, 0, c->stream>>>(n, a, b, s->red);
    k_red_final<<<1, 256, 0, c->stream>>>(g, s->red);
    c->launches += 2;
    CO_CK(cudaGetLastError());
    double h = 0.0;
    CO_CK(cudaMemcpyAsync(&h, s->red + CO_STEP_RED, sizeof(double), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    *out = sqrt(h);
    return CO_OK;
}

// the implicit solve from the start in mb.v1 (mb.v0 = v, mb.w = w)
static int solve_once(co_ctx *c, const co_opts *o, const co_defect_opts *d, int N, double S0,
                      double dt, int *outer, int *inner, double *res, double *r0, int *exit) {
    int rc;
    int it = 0, in = 0, nrs = 0;
    if (d)
        rc = co_step_defect_buffers(c, o, d, N, S0, dt, &it, res, &in, r0);
    else
        rc = co_step_anderson_buffers(c, o, N, S0, dt, &it, res, &nrs, r0);
    if (rc) return rc;
    *outer = it;
    *inner = in;
    *exit = c->st_host->done;
    return CO_OK;
}

static int step_learned_impl(co_ctx *c, const co_opts *o, const co_defect_opts *d, co_mlp *mlp,
                             int retry, double *v_new, const double *v, const double *w, int N,
                             double S0, double dt, co_step_info *info) {
    int rc;
    co_step_info I;
    memset(&I, 0, sizeof(I));
    if ((rc = co_ensure_capacity(c, N, o->m))) return rc;
    if ((rc = step_ensure(c, N))) return rc;
    co_step_bufs *s = c->sb;
    co_bufs &b = c->mb;
    const size_t n2 = 2 * (size_t)N * sizeof(double);
    // 1. features, predictor and its first residual
    double r_pred = 0.0;
    if ((rc = co_warmstart_features_dev(c, o, v, w, N, S0, dt, s->vp, s->X, &r_pred))) return rc;
    // 3. the previous-step state: G(v) = v_pred
    double r_prev = 0.0;
    if ((rc = diff_norm(c, 2 * N, s->vp, v, &r_prev))) return rc;
    // 2. the learned proposal
    double r_learn = INFINITY;
    if (mlp) {
        if ((rc = co_mlp_forward(mlp, s->X, N, s->Y, (void *)c->stream))) return rc;
        k_apply_delta<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, s->vp, s->Y, dt * dt, s->vl);
        c->launches += 2;
        CO_CK(cudaGetLastError());
        if ((rc = co_picard_residual_dev(c, o, s->vl, v, w, N, S0, dt, &r_learn))) return rc;
        if (!isfinite(r_learn)) r_learn = INFINITY;
    }
    I.r_start[0] = r_pred;
    I.r_start[1] = r_learn;
    I.r_start[2] = r_prev;
    // candidates ordered by first residual (ties keep predictor, learned, previous)
    int order[3] = {0, 1, 2};
    for (int i = 1; i < 3; i++)
        for (int j = i; j > 0 && I.r_start[order[j]] < I.r_start[order[j - 1]]; j--) {
            int t = order[j];
            order[j] = order[j - 1];
            order[j - 1] = t;
        }
    const double *src[3] = {s->vp, s->vl, v};
    int cand[3], nc = 0;
    for (int i = 0; i < 3; i++)
        if (order[i] != 1 || mlp) cand[nc++] = order[i];
    // 4. solve from the best start
    CO_CK(cudaMemcpyAsync(b.v0, v, n2, cudaMemcpyDeviceToDevice, c->stream));
    CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    CO_CK(cudaMemcpyAsync(b.v1, src[cand[0]], n2, cudaMemcpyDeviceToDevice, c->stream));
    int outer = 0, inner = 0, ex = 0;
    double res = 0.0, r0 = 0.0;
    if ((rc = solve_once(c, o, d, N, S0, dt, &outer, &inner, &res, &r0, &ex))) return rc;
    I.outer = outer;
    I.inner = inner;
    I.res = res;
    I.r0 = r0;
    I.exit = ex;
    I.start = cand[0];
    I.attempts = 1;
    // 5. a stagnated (or capped) solve is repeated once from the next start
    if (ex != 1 && retry && nc > 1) {
        CO_CK(cudaMemcpyAsync(s->keep, b.v1, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.v1, src[cand[1]], n2, cudaMemcpyDeviceToDevice, c->stream));
        int outer2 = 0, inner2 = 0, ex2 = 0;
        double res2 = 0.0, r02 = 0.0;
        if ((rc = solve_once(c, o, d, N, S0, dt, &outer2, &inner2, &res2, &r02, &ex2))) return rc;
        I.outer += outer2;
        I.inner += inner2;
        I.attempts = 2;
        if (ex2 == 1 || res2 < res) {
            I.res = res2;
            I.r0 = r02;
            I.exit = ex2;
            I.start = cand[1];
        } else {
            CO_CK(cudaMemcpyAsync(b.v1, s->keep, n2, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    I.converged = I.exit == 1;
    // 6. the new state and its entropy
    CO_CK(cudaMemcpyAsync(v_new, b.v1, n2, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = co_sort_markers(c, b.v1, N))) return rc;
    if ((rc = co_project_sorted(c, c->f))) return rc;
    if ((rc = co_entropy_parts_dev(c, c->f))) return rc;
    if ((rc = co_entropy_finalize_dev(c, c->y))) return rc;
    CO_CK(cudaMemcpyAsync(&I.S_new, c->y, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CO_CK(cudaGetLastError());
    CO_CK(cudaStreamSynchronize(c->stream));
    if (info) *info = I;
    return CO_OK;
}

static int check_step_args(co_ctx *c, const co_opts *o, const co_defect_opts *d, int N,
                           const void *v_new, const void *v, const void *w) {
    if (!c || !o || N < 1 || !v_new || !v || !w) return CO_ERR_ARG;
    if (o->model != CO_MODEL_LANDAU && o->model != CO_MODEL_LB) return CO_ERR_ARG;
    if (o->m < 1 || o->m > CO_MAX_M || o->max_iter < 1 || o->stag_window < 1) return CO_ERR_ARG;
    if (o->precision < CO_PREC_FP64 || o->precision > CO_PREC_MIXED_DS) return CO_ERR_ARG;
    if (o->model == CO_MODEL_LB && o->precision != CO_PREC_FP64) return CO_ERR_ARG;
    if (d && (o->model != CO_MODEL_LANDAU || d->max_inner < 1 || d->stag_window < 1 ||
              !(d->eta > 0) || d->cap_abort < 0))
        return CO_ERR_ARG;
    return CO_OK;
}

extern "C" int co_step_learned_dev(co_ctx *c, const co_opts *o, const co_defect_opts *d,
                                   co_mlp *mlp, int retry, double *v_new, const double *v,
                                   const double *w, int N, double S0, double dt,
                                   co_step_info *info) {
    int rc = check_step_args(c, o, d, N, v_new, v, w);
    if (rc) return rc;
    CO_CK(cudaSetDevice(c->device));
    return step_learned_impl(c, o, d, mlp, retry, v_new, v, w, N, S0, dt, info);
}

extern "C" int co_step_learned(co_ctx *c, const co_opts *o, const co_defect_opts *d, co_mlp *mlp,
                               int retry, double *v_new, const double *v, const double *w, int N,
                               double S0, double dt, co_step_info *info) {
    int rc = check_step_args(c, o, d, N, v_new, v, w);
    if (rc) return rc;
    for (size_t i = 0; i < 2 * (size_t)N; i++)
        if (!isfinite(v[i])) return CO_ERR_NONFINITE;
    for (int i = 0; i < N; i++)
        if (!isfinite(w[i])) return CO_ERR_NONFINITE;
    if (!isfinite(S0) || !isfinite(dt)) return CO_ERR_NONFINITE;
    CO_CK(cudaSetDevice(c->device));
    if ((rc = co_ensure_capacity(c, N, o->m))) return rc;
    if ((rc = step_ensure(c, N))) return rc;
    co_step_bufs *s = c->sb;
    const size_t n2 = 2 * (size_t)N * sizeof(double);
    CO_CK(cudaMemcpyAsync(s->hv, v, n2, cudaMemcpyHostToDevice, c->stream));
    CO_CK(cudaMemcpyAsync(s->hw, w, (size_t)N * sizeof(double), cudaMemcpyHostToDevice,
                          c->stream));
    // the new state lands in s->keep (free once the solves are done), then on the host
    if ((rc = step_learned_impl(c, o, d, mlp, retry, s->keep, s->hv, s->hw, N, S0, dt, info)))
        return rc;
    CO_CK(cudaMemcpyAsync(v_new, s->keep, n2, cudaMemcpyDeviceToHost, c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    return CO_OK;
}
