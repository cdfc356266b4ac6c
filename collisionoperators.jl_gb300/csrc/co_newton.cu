// co_newton.cu -- step_newton! (solver.jl:460-486) on the device: inexact
// Jacobian-free Newton-Krylov on F(v) = v - G(v), G the Picard map, after
// newton_krylov! and gmres! (newton_krylov.jl:74-303).
//
//   - GMRES: unrestarted, at most krylov_max Arnoldi vectors of length 2N in
//     HBM, modified Gram-Schmidt. Each projection coefficient is reduced on
//     the device (fixed-order block partials, then one block) and consumed by
//     the next kernel from device memory, so the host reads back only one
//     Hessenberg column per Arnoldi step; the Givens rotations, the rotated
//     right-hand side and the back substitution are a few scalars on the host.
//   - Products J u = (F(x + h u) - F(x)) / h with h = fd_h / ||u||: one Picard
//     map each, in the precision of the solve (FP64, or double-single pair sums
//     for CO_PREC_MIXED_DS).
//   - Eisenstat-Walker forcing (choice 2, safeguarded, capped at eta_max),
//     Armijo backtracking (8 halvings), the best iterate kept for a stalled or
//     budget exit, and the exit Picard update v - F(v) = G(v).
#include <math.h>
#include <string.h>

#include <vector>

#include "co_internal.cuh"
#include "co_reduce.cuh"

#define NK_RED 256   // blocks of the vector reductions

struct co_nk_bufs {
    int cap, mem;
    double *V;                                   // (mem + 1) x ld Arnoldi basis
    double *F, *Ft, *xt, *xp, *Fp, *d, *xb, *Fb, *wv;
    double *red;                                 // NK_RED partials
    double *scal;                                // device scalars: [0..mem] column, [mem+1] result
    double *z;                                   // mem coefficients of the final combination
};

void co_newton_free(co_ctx *c) {
    co_nk_bufs *s = c->nk;
    if (!s) return;
    void *p[] = {s->V, s->F, s->Ft, s->xt, s->xp, s->Fp, s->d, s->xb, s->Fb, s->wv, s->red,
                 s->scal, s->z};
    for (void *q : p)
        if (q) cudaFree(q);
    free(s);
    c->nk = nullptr;
}

static int nk_ensure(co_ctx *c, int N, int mem) {
    if (!c->nk) {
        c->nk = (co_nk_bufs *)calloc(1, sizeof(co_nk_bufs));
        if (!c->nk) return CO_ERR_NOMEM;
    }
    co_nk_bufs *s = c->nk;
    if (N <= s->cap && mem <= s->mem && s->V) return CO_OK;
    int cap = N > s->cap ? N : s->cap;
    int m = mem > s->mem ? mem : s->mem;
    co_newton_free(c);
    c->nk = (co_nk_bufs *)calloc(1, sizeof(co_nk_bufs));
    if (!c->nk) return CO_ERR_NOMEM;
    s = c->nk;
    const size_t n2 = 2 * (size_t)cap * sizeof(double);
    double **v[] = {&s->F, &s->Ft, &s->xt, &s->xp, &s->Fp, &s->d, &s->xb, &s->Fb, &s->wv};
    for (double **p : v)
        if (cudaMalloc(p, n2) != cudaSuccess) return CO_ERR_NOMEM;
    if (cudaMalloc(&s->V, n2 * (size_t)(m + 1)) != cudaSuccess ||
        cudaMalloc(&s->red, sizeof(double) * NK_RED) != cudaSuccess ||
        cudaMalloc(&s->scal, sizeof(double) * (m + 2)) != cudaSuccess ||
        cudaMalloc(&s->z, sizeof(double) * (m + 1)) != cudaSuccess)
        return CO_ERR_NOMEM;
    s->cap = cap;
    s->mem = m;
    return CO_OK;
}

// ---------------------------------------------------------------- kernels

// block partials of a . b (b == nullptr: a . a)
__global__ void __launch_bounds__(256)
k_nk_dot(int n, const double *__restrict__ a, const double *__restrict__ b,
         double *__restrict__ red) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double x = a[i];
        s = fma(x, b ? b[i] : x, s);
    }
    s = co_block_sum(s, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = s;
}

// out = sum of the partials in block order (sqrt for a norm)
__global__ void __launch_bounds__(256)
k_nk_final(int nb, const double *__restrict__ red, int take_sqrt, double *__restrict__ out) {
    __shared__ double sh[32];
    double s = co_sum_partials(red, nb, 1, 0, sh);
    if (threadIdx.x == 0) *out = take_sqrt ? sqrt(s) : s;
}

// y = x + a * u, with a = scale * (*ap) when ap is given
__global__ void k_nk_axpy(int n, double *y, const double *x, double a,
                          const double *__restrict__ ap, double scale,
                          const double *__restrict__ u) {
    const double al = ap ? scale * *ap : a;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = fma(al, u[i], x[i]);
}

// y = a * u
__global__ void k_nk_scale(int n, double *__restrict__ y, double a, const double *__restrict__ u) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = a * u[i];
}

// F = x - Gv
__global__ void k_nk_resid(int n, const double *__restrict__ x, const double *__restrict__ Gv,
                           double *__restrict__ F) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        F[i] = x[i] - Gv[i];
}

// w = (Fp - F) * inv_h
__global__ void k_nk_fd(int n, const double *__restrict__ Fp, const double *__restrict__ F,
                        double inv_h, double *__restrict__ w) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = (Fp[i] - F[i]) * inv_h;
}

// x = sum_i z[i] V[i] (fixed order)
__global__ void k_nk_combine(int n, int k, const double *__restrict__ V, size_t ld,
                             const double *__restrict__ z, double *__restrict__ x) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < k; i++) s = fma(z[i], V[(size_t)i * ld + j], s);
        x[j] = s;
    }
}

// ---------------------------------------------------------------- host side

struct nk_run {
    co_ctx *c;
    const co_opts *o;
    int prec, N, n, grid;
    double S0, dt;
    const double *v0;
    int evals;
};

static int nk_reduce(nk_run &r, const double *a, const double *b, int take_sqrt, double *dst) {
    co_nk_bufs *s = r.c->nk;
    int g = co_cdiv(r.n, 256);
    if (g > NK_RED) g = NK_RED;
    k_nk_dot<<<g, 256, 0, r.c->stream>>>(r.n, a, b, s->red);
    k_nk_final<<<1, 256, 0, r.c->stream>>>(g, s->red, take_sqrt, dst);
    r.c->launches += 2;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

static int nk_read(nk_run &r, const double *src, double *host, int count) {
    CO_CK(cudaMemcpyAsync(host, src, sizeof(double) * count, cudaMemcpyDeviceToHost,
                          r.c->stream));
    CO_CK(cudaStreamSynchronize(r.c->stream));
    return CO_OK;
}

// F = x - G(x) and ||F|| (residual! of step_newton!, solver.jl:465-472)
static int nk_residual(nk_run &r, double *F, const double *x, double *nrm) {
    co_ctx *c = r.c;
    int rc = co_picard_map_dev(c, r.o, r.prec, c->mb.Gv, x, r.v0, c->mb.w, r.N, r.S0, r.dt, 0);
    if (rc) return rc;
    k_nk_resid<<<r.grid, 256, 0, c->stream>>>(r.n, x, c->mb.Gv, F);
    c->launches++;
    r.evals++;
    if ((rc = nk_reduce(r, F, nullptr, 1, c->nk->scal + c->nk->mem + 1))) return rc;
    if ((rc = nk_read(r, c->nk->scal + c->nk->mem + 1, nrm, 1))) return rc;
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    CO_CK(cudaStreamSynchronize(c->stream));
    if (c->st_host->error) return c->st_host->error;
    if (!isfinite(*nrm)) return CO_ERR_NONFINITE;
    return CO_OK;
}

// _sym_givens (newton_krylov.jl:37-58)
static void sym_givens(double a, double b, double *cc, double *ss, double *rho) {
    if (b == 0.0) {
        *cc = (a > 0) - (a < 0) + (a == 0.0);
        *ss = 0.0;
        *rho = fabs(a);
    } else if (a == 0.0) {
        *cc = 0.0;
        *ss = (b > 0) - (b < 0);
        *rho = fabs(b);
    } else if (fabs(b) > fabs(a)) {
        double t = a / b;
        *ss = ((b > 0) - (b < 0)) / sqrt(1.0 + t * t);
        *cc = *ss * t;
        *rho = b / *ss;
    } else {
        double t = b / a;
        *cc = ((a > 0) - (a < 0)) / sqrt(1.0 + t * t);
        *ss = *cc * t;
        *rho = a / *cc;
    }
}

// gmres! (newton_krylov.jl:74-130): solve J d = F(x) from d = 0; F(x) in nk->F
static int nk_gmres(nk_run &r, const double *x, double Fnorm, double rtol, int itmax,
                    double fd_h, int *k_out) {
    co_ctx *c = r.c;
    co_nk_bufs *s = c->nk;
    const int mem = s->mem, n = r.n;
    const size_t ld = 2 * (size_t)s->cap;
    const int kmax = itmax < mem ? itmax : mem;
    int rc;
    CO_CK(cudaMemsetAsync(s->d, 0, sizeof(double) * n, c->stream));
    *k_out = 0;
    if (Fnorm == 0.0) return CO_OK;
    const double beta = Fnorm, eps = rtol * beta, btol = pow(2.220446049250313e-16, 0.75);
    std::vector<double> R((size_t)mem * mem, 0.0), cs(mem, 0.0), sn(mem, 0.0), z(mem + 1, 0.0);
    std::vector<double> col(mem + 2, 0.0);
    z[0] = beta;
    // V_1 = F / beta
    k_nk_scale<<<r.grid, 256, 0, c->stream>>>(n, s->V, 1.0 / beta, s->F);
    c->launches++;
    int k = 0;
    while (k < kmax) {
        k++;
        double *u = s->V + (size_t)(k - 1) * ld;
        double unrm = 0.0;
        if ((rc = nk_reduce(r, u, nullptr, 1, s->scal + mem + 1))) return rc;
        if ((rc = nk_read(r, s->scal + mem + 1, &unrm, 1))) return rc;
        const double h = fd_h / unrm;
        k_nk_axpy<<<r.grid, 256, 0, c->stream>>>(n, s->xp, x, h, nullptr, 0.0, u);
        c->launches++;
        double dummy;
        if ((rc = nk_residual(r, s->Fp, s->xp, &dummy))) return rc;
        k_nk_fd<<<r.grid, 256, 0, c->stream>>>(n, s->Fp, s->F, 1.0 / h, s->wv);
        c->launches++;
        // modified Gram-Schmidt: each coefficient stays on the device until read back
        for (int i = 0; i < k; i++) {
            const double *vi = s->V + (size_t)i * ld;
            if ((rc = nk_reduce(r, vi, s->wv, 0, s->scal + i))) return rc;
            k_nk_axpy<<<r.grid, 256, 0, c->stream>>>(n, s->wv, s->wv, 0.0, s->scal + i, -1.0, vi);
            c->launches++;
        }
        if ((rc = nk_reduce(r, s->wv, nullptr, 1, s->scal + k))) return rc;
        if ((rc = nk_read(r, s->scal, col.data(), k + 1))) return rc;
        for (int i = 0; i < k; i++) R[(size_t)i * mem + (k - 1)] = col[i];
        const double hnext = col[k];
        for (int i = 0; i < k - 1; i++) {
            double a = R[(size_t)i * mem + (k - 1)], bb = R[(size_t)(i + 1) * mem + (k - 1)];
            double tmp = cs[i] * a + sn[i] * bb;
            R[(size_t)(i + 1) * mem + (k - 1)] = sn[i] * a - cs[i] * bb;
            R[(size_t)i * mem + (k - 1)] = tmp;
        }
        double rho;
        sym_givens(R[(size_t)(k - 1) * mem + (k - 1)], hnext, &cs[k - 1], &sn[k - 1], &rho);
        R[(size_t)(k - 1) * mem + (k - 1)] = rho;
        z[k] = sn[k - 1] * z[k - 1];
        z[k - 1] = cs[k - 1] * z[k - 1];
        if (fabs(z[k]) <= eps || hnext <= btol) break;
        if (k < kmax) {
            k_nk_scale<<<r.grid, 256, 0, c->stream>>>(n, s->V + (size_t)k * ld, 1.0 / hnext,
                                                      s->wv);
            c->launches++;
        }
    }
    for (int i = k - 1; i >= 0; i--) {
        double acc = z[i];
        for (int j = i + 1; j < k; j++) acc -= R[(size_t)i * mem + j] * z[j];
        z[i] = fabs(R[(size_t)i * mem + i]) <= btol ? 0.0 : acc / R[(size_t)i * mem + i];
    }
    CO_CK(cudaMemcpyAsync(s->z, z.data(), sizeof(double) * k, cudaMemcpyHostToDevice, c->stream));
    k_nk_combine<<<r.grid, 256, 0, c->stream>>>(n, k, s->V, ld, s->z, s->d);
    c->launches++;
    CO_CK(cudaGetLastError());
    CO_CK(cudaStreamSynchronize(c->stream));   // z (host) stays alive until the copy is done
    *k_out = k;
    return CO_OK;
}

// newton_krylov! (newton_krylov.jl:207-303) + step_newton! (solver.jl:460-486)
// on mb.v1 (guess in, solution out), mb.v0, mb.w
int co_step_newton_buffers(co_ctx *c, const co_opts *o, const co_newton_opts *nko, int N,
                           double S0, double dt, int *evals, double *res, int *n_newton,
                           double *r0, int *status) {
    int rc;
    if ((rc = co_ensure_capacity(c, N, 1))) return rc;
    if (N == 0) {
        if (evals) *evals = 0;
        if (res) *res = 0.0;
        if (n_newton) *n_newton = 0;
        if (r0) *r0 = 0.0;
        if (status) *status = 0;
        return CO_OK;
    }
    if ((rc = nk_ensure(c, N, nko->krylov_max))) return rc;
    co_nk_bufs *s = c->nk;
    co_bufs &b = c->mb;
    nk_run r;
    r.c = c;
    r.o = o;
    r.prec = o->precision == CO_PREC_MIXED_DS ? CO_PREC_MIXED_DS : CO_PREC_FP64;
    r.N = N;
    r.n = 2 * N;
    r.grid = co_cdiv(r.n, 256) < 8 * c->nsm ? co_cdiv(r.n, 256) : 8 * c->nsm;
    r.S0 = S0;
    r.dt = dt;
    r.v0 = b.v0;
    r.evals = 0;
    const int n = r.n;
    const size_t nb = sizeof(double) * n;
    double *x = b.v1;
    CO_CK(cudaMemsetAsync(&c->st->error, 0, sizeof(int), c->stream));
    // tolerance taken once at the predictor (solver.jl:474)
    double xn = 0.0;
    if ((rc = nk_reduce(r, x, nullptr, 1, s->scal + s->mem + 1))) return rc;
    if ((rc = nk_read(r, s->scal + s->mem + 1, &xn, 1))) return rc;
    const double tol = fmax(o->tol * (xn + 1e-30), o->abs_floor);
    double rnorm = 0.0;
    if ((rc = nk_residual(r, s->F, x, &rnorm))) return rc;
    const double rnorm0 = rnorm;
    double rbest = rnorm, eta = nko->eta_max, rprev = rnorm;
    CO_CK(cudaMemcpyAsync(s->xb, x, nb, cudaMemcpyDeviceToDevice, c->stream));
    CO_CK(cudaMemcpyAsync(s->Fb, s->F, nb, cudaMemcpyDeviceToDevice, c->stream));
    int nn = 0, st = 2;   // 0 converged, 1 stalled, 2 budget
    const double gamma = 0.9, armijo = 1e-4;
    for (;;) {
        if (rnorm < tol) {
            st = 0;
            break;
        }
        const int budget = o->max_iter - r.evals;
        if (budget < 2) break;
        if (nn > 0) {
            double ew = gamma * (rnorm / rprev) * (rnorm / rprev);
            const double safe = gamma * eta * eta;
            if (safe > 0.1) ew = fmax(ew, safe);
            eta = fmin(fmax(ew, 0.5 * tol / rnorm), nko->eta_max);
        }
        const int itmax = nko->krylov_max < budget - 1 ? nko->krylov_max : budget - 1;
        int kl = 0;
        if ((rc = nk_gmres(r, x, rnorm, eta, itmax, nko->fd_h, &kl))) return rc;
        nn++;
        double lam = 1.0, rt = INFINITY;
        int accepted = 0;
        for (int bt = 0; bt <= 8; bt++) {
            k_nk_axpy<<<r.grid, 256, 0, c->stream>>>(n, s->xt, x, -lam, nullptr, 0.0, s->d);
            c->launches++;
            if ((rc = nk_residual(r, s->Ft, s->xt, &rt))) return rc;
            if (rt <= (1.0 - armijo * lam * (1.0 - eta)) * rnorm) {
                accepted = 1;
                break;
            }
            if (r.evals >= o->max_iter) break;
            lam /= 2.0;
        }
        if (rt < rbest) {
            rbest = rt;
            CO_CK(cudaMemcpyAsync(s->xb, s->xt, nb, cudaMemcpyDeviceToDevice, c->stream));
            CO_CK(cudaMemcpyAsync(s->Fb, s->Ft, nb, cudaMemcpyDeviceToDevice, c->stream));
        }
        if (!accepted) {
            st = r.evals >= o->max_iter ? 2 : 1;
            break;
        }
        CO_CK(cudaMemcpyAsync(x, s->xt, nb, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(s->F, s->Ft, nb, cudaMemcpyDeviceToDevice, c->stream));
        rprev = rnorm;
        rnorm = rt;
    }
    if (st != 0 && rbest < rnorm) {
        CO_CK(cudaMemcpyAsync(x, s->xb, nb, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(s->F, s->Fb, nb, cudaMemcpyDeviceToDevice, c->stream));
        rnorm = rbest;
    }
    if (o->exit_picard_step) {   // v1 -= F: the Picard update G(v) (solver.jl:480)
        k_nk_axpy<<<r.grid, 256, 0, c->stream>>>(n, x, x, -1.0, nullptr, 0.0, s->F);
        c->launches++;
    }
    CO_CK(cudaGetLastError());
    CO_CK(cudaStreamSynchronize(c->stream));
    if (evals) *evals = r.evals;
    if (res) *res = rnorm;
    if (n_newton) *n_newton = nn;
    if (r0) *r0 = rnorm0;
    if (status) *status = st;
    return CO_OK;
}
