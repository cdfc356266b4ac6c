// co_abi.cu -- the extern "C" entry points declared in include/collops.h.
//
// Context creation does the Workspace set-up of MantisWrappers.jl:90-158 for
// the device: Gauss-Legendre rule, Bezier extraction of the clamped C1
// quadratic B-spline space, basis tables at the quadrature nodes, and the 1D
// mass matrices M1, M2 (3-point rule per element, exact for the degree-4
// integrand) whose inverses realise M^{-1} = M1^{-1} (x) M2^{-1}.
//
// The hook entry points copy the caller's host arrays into the context's
// device buffers, run the device stage, and copy the result back; the *_dev
// variants skip the copies.
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "co_internal.cuh"

int co_spline_configure(co_ctx *c);
int co_step_anderson_buffers(co_ctx *c, const co_opts *o, int N, double S0, double dt,
                             int *iters, double *res, int *nrs, double *r0);

#define CO_RED_CAP 1024
#define CO_RED_COMPS 16

// ---------------------------------------------------------------- host FEM

// Gauss-Legendre nodes/weights on [0,1] (weights sum to 1), ascending.
static void gl01(int n, double *x, double *w) {
    for (int i = 0; i < n; i++) {
        double z = cos(M_PI * (n - i - 0.25) / (n + 0.5));  // ascending guess
        for (int it = 0; it < 200; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p0 = 1.0; p1 = z; }
            double dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-17) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; k++) {
            double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        double dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = 0.5 * (1.0 + z);
        w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Bezier extraction of element e: phi_j = sum_k C[k*3+j] B_k, with the
// neighbour widths of the clamped C1 quadratic knot vector.
static void extraction(const std::vector<double> &bp, std::vector<double> &C) {
    int n = (int)bp.size() - 1;
    C.assign(9 * (size_t)n, 0.0);
    for (int e = 0; e < n; e++) {
        double h = bp[e + 1] - bp[e];
        double hl = e > 0 ? bp[e] - bp[e - 1] : 0.0;
        double hr = e < n - 1 ? bp[e + 2] - bp[e + 1] : 0.0;
        double *c = &C[9 * (size_t)e];
        c[0] = h / (hl + h);   // B0 -> phi0
        c[1] = hl / (hl + h);  // B0 -> phi1
        c[4] = 1.0;            // B1 -> phi1
        c[7] = hr / (h + hr);  // B2 -> phi1
        c[8] = h / (h + hr);   // B2 -> phi2
    }
}

static void bern2h(double xi, double *B) {
    double om = 1.0 - xi;
    B[0] = om * om;
    B[1] = 2.0 * xi * om;
    B[2] = xi * xi;
}

static void phi_at(const double *c, double xi, double *phi) {
    double B[3];
    bern2h(xi, B);
    for (int j = 0; j < 3; j++) phi[j] = c[j] * B[0] + c[3 + j] * B[1] + c[6 + j] * B[2];
}

// dense 1D mass matrix, exact with the 3-point rule
static void mass1d(const std::vector<double> &bp, const std::vector<double> &C,
                   std::vector<double> &M) {
    int n = (int)bp.size() - 1, nd = n + 2;
    M.assign((size_t)nd * nd, 0.0);
    double gx[3], gw[3];
    gl01(3, gx, gw);
    for (int e = 0; e < n; e++) {
        double h = bp[e + 1] - bp[e];
        for (int q = 0; q < 3; q++) {
            double phi[3];
            phi_at(&C[9 * (size_t)e], gx[q], phi);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) M[(size_t)(e + a) * nd + (e + b)] += phi[a] * phi[b] * gw[q] * h;
        }
    }
}

// inverse of an SPD matrix through Cholesky (nd is small: n_el + 2)
static int spd_inverse(std::vector<double> A, int n, std::vector<double> &inv) {
    std::vector<double> L((size_t)n * n, 0.0);
    for (int j = 0; j < n; j++) {
        double s = A[(size_t)j * n + j];
        for (int k = 0; k < j; k++) s -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
        if (!(s > 0)) return CO_ERR_ARG;
        L[(size_t)j * n + j] = sqrt(s);
        for (int i = j + 1; i < n; i++) {
            double t = A[(size_t)i * n + j];
            for (int k = 0; k < j; k++) t -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            L[(size_t)i * n + j] = t / L[(size_t)j * n + j];
        }
    }
    inv.assign((size_t)n * n, 0.0);
    std::vector<double> col(n);
    for (int c = 0; c < n; c++) {
        for (int i = 0; i < n; i++) {  // L y = e_c
            double s = i == c ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * col[k];
            col[i] = s / L[(size_t)i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {  // L^T x = y
            double s = col[i];
            for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * col[k];
            col[i] = s / L[(size_t)i * n + i];
        }
        for (int i = 0; i < n; i++) inv[(size_t)i * n + c] = col[i];
    }
    // symmetrise (round-off)
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double s = 0.5 * (inv[(size_t)i * n + j] + inv[(size_t)j * n + i]);
            inv[(size_t)i * n + j] = inv[(size_t)j * n + i] = s;
        }
    return CO_OK;
}

template <typename T>
static int upload(T **dst, const std::vector<T> &src) {
    if (cudaMalloc((void **)dst, src.size() * sizeof(T)) != cudaSuccess) return CO_ERR_NOMEM;
    if (cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return CO_ERR_CUDA;
    return CO_OK;
}

// ---------------------------------------------------------------- lifecycle

extern "C" int co_version(void) { return CO_ABI_VERSION; }

extern "C" const char *co_strerror(int s) {
    switch (s) {
        case CO_OK: return "ok";
        case CO_ERR_ARG: return "invalid argument";
        case CO_ERR_CUDA: return "CUDA runtime error";
        case CO_ERR_UNSUPPORTED: return "unsupported configuration (P_DEG must be 2)";
        case CO_ERR_NONFINITE: return "non-finite value in inputs or residual";
        case CO_ERR_TIMEOUT: return "device-side wait timed out";
        case CO_ERR_NOMEM: return "device allocation failed";
        case CO_ERR_NODEVICE: return "no CUDA device";
        case CO_ERR_SIZE: return "N exceeds the 32768-marker limit of co_collision_noalloc";
        default: return "unknown status";
    }
}

static void free_ctx(co_ctx *c) {
    if (!c) return;
    void *ptrs[] = {c->bp1, c->bp2, c->C1, c->C2, c->Tq1, c->Tq2, c->ih1, c->ih2, c->P1, c->P2,
                    c->qw, c->Minv1, c->Minv2,
                    c->bS, c->b, c->y, c->f, c->fin, c->rr, c->L, c->E, c->Ep, c->st,
                    c->mb.vmid, c->mb.dv, c->mb.G, c->mb.dS, c->mb.Gv, c->mb.r, c->mb.rp,
                    c->mb.Gp, c->mb.vbest, c->mb.v1, c->mb.v0, c->mb.w, c->mb.vin, c->mb.dotv,
                    c->mb.cell, c->mb.inv, c->mb.xi, c->mb.perm, c->mb.scell, c->mb.sw,
                    c->mb.sphi, c->mb.px, c->mb.pg, c->mb.pw, c->mb.pf_x, c->mb.pf_g, c->mb.pf_w, c->mb.pf_wl,
                    c->mb.pdot, c->mb.pA, c->mb.part, c->mb.hist, c->mb.hoff, c->mb.count,
                    c->mb.cstart, c->mb.red, c->mb.dF, c->mb.dG, c->mb.Gk, c->mb.Phi,
                    c->mb.Adef, c->mb.aa, c->mb.pc, c->st2, c->st3, c->tickets};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    co_step_free(c);
    co_newton_free(c);
    co_sortset_free(c);
    co_prof_free(c);
    if (c->st_host) cudaFreeHost(c->st_host);
    if (c->stream) cudaStreamDestroy(c->stream);
    free(c);
}

extern "C" int co_ctx_create(const double *bp1, int nb1, const double *bp2, int nb2, int p_deg,
                             int n_quad, unsigned flags, int device, co_ctx **out) {
    if (!out) return CO_ERR_ARG;
    *out = nullptr;
    // nb1 - 1 <= 4096 cells per dimension: the fused dof-gather + mass kernel
    // holds one column of nb1 + 1 dofs in shared memory
    if (!bp1 || !bp2 || nb1 < 2 || nb2 < 2 || nb1 > 4097 || nb2 > 4097 || n_quad < 1 ||
        n_quad > 8)
        return CO_ERR_ARG;
    if (p_deg != 2) return CO_ERR_UNSUPPORTED;
    for (int i = 0; i + 1 < nb1; i++)
        if (!(bp1[i + 1] > bp1[i])) return CO_ERR_ARG;
    for (int i = 0; i + 1 < nb2; i++)
        if (!(bp2[i + 1] > bp2[i])) return CO_ERR_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CO_ERR_NODEVICE;
    if (device < 0 || device >= ndev) return CO_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return CO_ERR_CUDA;
    co_ctx *c = (co_ctx *)calloc(1, sizeof(co_ctx));
    c->device = device;
    c->flags = flags;
    c->n1 = nb1 - 1;
    c->n2 = nb2 - 1;
    c->nd1 = c->n1 + 2;
    c->nd2 = c->n2 + 2;
    c->n_dofs = c->nd1 * c->nd2;
    c->n_el = c->n1 * c->n2;
    c->nq = n_quad;
    c->pair_symmetric = (flags & CO_FLAG_ONESIDED) ? 0 : 1;
    c->lo1 = bp1[0];
    c->hi1 = bp1[c->n1];
    c->lo2 = bp2[0];
    c->hi2 = bp2[c->n2];
    int rc = CO_OK;
#define TRY(x)                 \
    do {                       \
        if ((rc = (x))) {      \
            free_ctx(c);       \
            return rc;         \
        }                      \
    } while (0)
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        free_ctx(c);
        return CO_ERR_CUDA;
    }
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, device);
    c->nsm = prop.multiProcessorCount;

    std::vector<double> B1(bp1, bp1 + nb1), B2(bp2, bp2 + nb2), C1, C2, M1, M2, I1, I2;
    extraction(B1, C1);
    extraction(B2, C2);
    std::vector<double> qx(n_quad), qw(n_quad);
    gl01(n_quad, qx.data(), qw.data());
    std::vector<double> T1((size_t)c->n1 * 3 * n_quad), T2((size_t)c->n2 * 3 * n_quad);
    for (int e = 0; e < c->n1; e++)
        for (int q = 0; q < n_quad; q++) {
            double phi[3];
            phi_at(&C1[9 * (size_t)e], qx[q], phi);
            for (int a = 0; a < 3; a++) T1[((size_t)e * 3 + a) * n_quad + q] = phi[a];
        }
    for (int e = 0; e < c->n2; e++)
        for (int q = 0; q < n_quad; q++) {
            double phi[3];
            phi_at(&C2[9 * (size_t)e], qx[q], phi);
            for (int a = 0; a < 3; a++) T2[((size_t)e * 3 + a) * n_quad + q] = phi[a];
        }
    // per-cell tables of the marker kernels (locate, sort, grad L): the
    // reciprocal widths, and each cell-local basis function
    // p_j(x) = sum_k C[k][j] B_k(x) with B = ((1-x)^2, 2x(1-x), x^2) rewritten
    // as alpha + beta x + gamma x^2, so that p and dp/dx cost 3 FMAs on the
    // device instead of the Bernstein values plus the 3x3 extraction product
    auto cell_tables = [](const std::vector<double> &B, const std::vector<double> &C, int n,
                          std::vector<double> &ih, std::vector<double> &P) {
        ih.resize(n);
        P.resize((size_t)n * 12);
        for (int e = 0; e < n; e++) {
            ih[e] = 1.0 / (B[e + 1] - B[e]);
            for (int j = 0; j < 3; j++) {
                const double c0 = C[9 * (size_t)e + j], c1 = C[9 * (size_t)e + 3 + j],
                             c2 = C[9 * (size_t)e + 6 + j];
                const double gam = (c0 - 2.0 * c1) + c2;
                P[12 * (size_t)e + 4 * j + 0] = c0;
                P[12 * (size_t)e + 4 * j + 1] = 2.0 * (c1 - c0);
                P[12 * (size_t)e + 4 * j + 2] = gam;
                P[12 * (size_t)e + 4 * j + 3] = 2.0 * gam;
            }
        }
    };
    std::vector<double> IH1, IH2, P1, P2;
    cell_tables(B1, C1, c->n1, IH1, P1);
    cell_tables(B2, C2, c->n2, IH2, P2);
    TRY(upload(&c->ih1, IH1));
    TRY(upload(&c->ih2, IH2));
    TRY(upload(&c->P1, P1));
    TRY(upload(&c->P2, P2));
    mass1d(B1, C1, M1);
    mass1d(B2, C2, M2);
    TRY(spd_inverse(M1, c->nd1, I1));
    TRY(spd_inverse(M2, c->nd2, I2));
    TRY(upload(&c->bp1, B1));
    TRY(upload(&c->bp2, B2));
    TRY(upload(&c->C1, C1));
    TRY(upload(&c->C2, C2));
    TRY(upload(&c->Tq1, T1));
    TRY(upload(&c->Tq2, T2));
    TRY(upload(&c->qw, qw));
    TRY(upload(&c->Minv1, I1));
    TRY(upload(&c->Minv2, I2));
    double **cv[] = {&c->b, &c->y, &c->f, &c->fin, &c->rr, &c->L};
    for (double **p : cv)
        if (cudaMalloc(p, sizeof(double) * c->n_dofs) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->bS, sizeof(double) * 9 * c->n_el) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->E, sizeof(double) * 9 * c->n_el) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->Ep, sizeof(double) * c->n_el) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->mb.count, sizeof(int) * c->n_el) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->mb.cstart, sizeof(int) * (c->n_el + 1)) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    c->mb.red_cap = CO_RED_CAP;
    if (cudaMalloc(&c->mb.red, sizeof(double) * CO_RED_CAP * CO_RED_COMPS + 64) != cudaSuccess)
        { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->st, sizeof(co_solver_state)) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    if (cudaMalloc(&c->tickets, sizeof(unsigned) * CO_TICKETS) != cudaSuccess ||
        cudaMemset(c->tickets, 0, sizeof(unsigned) * CO_TICKETS) != cudaSuccess) {
        free_ctx(c);
        return CO_ERR_NOMEM;
    }
    if (cudaMallocHost(&c->st_host, sizeof(co_solver_state)) != cudaSuccess) { free_ctx(c); return CO_ERR_NOMEM; };
    memset(c->st_host, 0, sizeof(co_solver_state));
    if (cudaMemset(c->st, 0, sizeof(co_solver_state)) != cudaSuccess) { free_ctx(c); return CO_ERR_CUDA; };
    TRY(co_spline_configure(c));
    TRY(co_ensure_capacity(c, 1024, 1));
#undef TRY
    *out = c;
    return CO_OK;
}

void co_ctx_destroy_detached(co_ctx *c) {
    if (c) free_ctx(c);
}

extern "C" int co_ctx_destroy(co_ctx *c) {
    if (!c) return CO_ERR_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_ctx(c);
    return CO_OK;
}

extern "C" int co_ctx_n_dofs(const co_ctx *c, int *n) {
    if (!c || !n) return CO_ERR_ARG;
    *n = c->n_dofs;
    return CO_OK;
}

extern "C" int co_ctx_set_wait_limit(co_ctx *c, int spins, int phantom_blocks) {
    if (!c || phantom_blocks < 0) return CO_ERR_ARG;
    c->barrier_spins = spins > 0 ? spins : 0;
    c->barrier_phantom = phantom_blocks;
    return CO_OK;
}

extern "C" int co_launch_count(const co_ctx *c, unsigned long long *l) {
    if (!c || !l) return CO_ERR_ARG;
    *l = c->launches;
    return CO_OK;
}

// ---------------------------------------------------------------- helpers

static int h2d(co_ctx *c, double *dst, const double *src, size_t n) {
    if (n == 0) return CO_OK;
    CO_CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return CO_OK;
}
static int d2h(co_ctx *c, double *dst, const double *src, size_t n) {
    if (n == 0) return CO_OK;
    CO_CK(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    return CO_OK;
}
static int finish(co_ctx *c) {
    CO_CK(cudaGetLastError());
    CO_CK(cudaStreamSynchronize(c->stream));
    return CO_OK;
}

static int all_finite(const double *x, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!isfinite(x[i])) return 0;
    return 1;
}

#define ENTER(c)                                  \
    do {                                          \
        if (!(c)) return CO_ERR_ARG;              \
        if (cudaSetDevice((c)->device) != cudaSuccess) return CO_ERR_CUDA; \
    } while (0)

#define RC(x)                \
    do {                     \
        int rc_ = (x);       \
        if (rc_) return rc_; \
    } while (0)

static int check_opts(const co_opts *o) {
    if (!o) return CO_ERR_ARG;
    if (o->model != CO_MODEL_LANDAU && o->model != CO_MODEL_LB) return CO_ERR_ARG;
    if (o->m < 1 || o->m > CO_MAX_M || o->max_iter < 1 || o->stag_window < 1) return CO_ERR_ARG;
    if (o->precision < CO_PREC_FP64 || o->precision > CO_PREC_MIXED_DS) return CO_ERR_ARG;
    if (o->model == CO_MODEL_LB && o->precision != CO_PREC_FP64) return CO_ERR_ARG;
    return CO_OK;
}

// ---------------------------------------------------------------- hooks

static int collision_common(co_ctx *c, const double *v, const double *w, const double *G,
                            double *dot_v, int N) {
    ENTER(c);
    if (N < 0 || (N > 0 && (!v || !w || !G || !dot_v))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v, 2 * (size_t)N) || !all_finite(w, N) || !all_finite(G, 2 * (size_t)N))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    int prec = (c->flags & CO_FLAG_FP32_PAIR) ? CO_PREC_MIXED : CO_PREC_FP64;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, b.G, G, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_sort_markers(c, b.vmid, N));
    RC(co_pack_plain(c, N, N, prec, b.vmid, b.G));
    RC(prec == CO_PREC_MIXED ? co_pair_fp32(c, N) : co_pair_fp64(c, N, 0));
    RC(co_unpack_update(c, N, 0.0, nullptr, nullptr, nullptr, nullptr, nullptr));
    RC(d2h(c, dot_v, b.dotv, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_collision(co_ctx *c, const double *v, const double *w, const double *G,
                            double *dot_v, int N) {
    return collision_common(c, v, w, G, dot_v, N);
}

extern "C" int co_collision_metric(co_ctx *c, const double *v, const double *w, const double *G,
                                   double *dot_v, double *A, int N) {
    ENTER(c);
    if (N < 0 || (N > 0 && (!v || !w || !G || !dot_v || !A))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v, 2 * (size_t)N) || !all_finite(w, N) || !all_finite(G, 2 * (size_t)N))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 2));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, b.G, G, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_sort_markers(c, b.vmid, N));
    RC(co_pack_plain(c, N, N, CO_PREC_FP64, b.vmid, b.G));
    RC(co_pair_fp64(c, N, 1));
    RC(co_unpack_update(c, N, 0.0, nullptr, nullptr, nullptr, nullptr, nullptr));
    RC(d2h(c, dot_v, b.dotv, 2 * (size_t)N));
    // A (N x 3) unpacked into the Anderson window buffer (>= 2 x 2N doubles)
    RC(co_unpack_A(c, N, b.dF));
    RC(d2h(c, A, b.dF, 3 * (size_t)N));
    return finish(c);
}

extern "C" int co_l2_project(co_ctx *c, const double *v, const double *w, double *f, int N) {
    ENTER(c);
    if (N < 0 || !f || (N > 0 && (!v || !w))) return CO_ERR_ARG;
    if (N > 0 && (!all_finite(v, 2 * (size_t)N) || !all_finite(w, N))) return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_sort_markers(c, b.vmid, N));
    RC(co_project_sorted(c, c->f));
    RC(d2h(c, f, c->f, c->n_dofs));
    return finish(c);
}

extern "C" int co_grad_L(co_ctx *c, const double *v, const double *L, double *G, int N) {
    ENTER(c);
    if (N < 0 || !L || (N > 0 && (!v || !G))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v, 2 * (size_t)N) || !all_finite(L, c->n_dofs)) return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, c->L, L, c->n_dofs));
    RC(co_sort_markers(c, b.vmid, N));
    RC(co_grad_L_dev(c, b.vmid, N, c->L, b.G, nullptr, nullptr, nullptr, nullptr));
    RC(d2h(c, G, b.G, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_loggrad(co_ctx *c, const double *v, const double *f, double *g, int N) {
    ENTER(c);
    if (N < 0 || !f || (N > 0 && (!v || !g))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v, 2 * (size_t)N) || !all_finite(f, c->n_dofs)) return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, c->f, f, c->n_dofs));
    RC(co_sort_markers(c, b.vmid, N));
    RC(co_loggrad_dev(c, b.vmid, N, c->f, b.G, nullptr, nullptr, nullptr));
    RC(d2h(c, g, b.G, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_compute_r(co_ctx *c, const double *f, double *r) {
    ENTER(c);
    if (!f || !r) return CO_ERR_ARG;
    if (!all_finite(f, c->n_dofs)) return CO_ERR_NONFINITE;
    RC(h2d(c, c->f, f, c->n_dofs));
    RC(co_compute_r_dev(c, c->f, c->rr));
    RC(d2h(c, r, c->rr, c->n_dofs));
    return finish(c);
}

extern "C" int co_entropy(co_ctx *c, const double *f, double *S) {
    ENTER(c);
    if (!f || !S) return CO_ERR_ARG;
    if (!all_finite(f, c->n_dofs)) return CO_ERR_NONFINITE;
    RC(h2d(c, c->f, f, c->n_dofs));
    RC(co_entropy_parts_dev(c, c->f));
    RC(co_entropy_finalize_dev(c, c->y));
    RC(d2h(c, S, c->y, 1));
    return finish(c);
}

extern "C" int co_mass_solve(co_ctx *c, const double *rhs, double *out) {
    ENTER(c);
    if (!rhs || !out) return CO_ERR_ARG;
    if (!all_finite(rhs, c->n_dofs)) return CO_ERR_NONFINITE;
    RC(h2d(c, c->b, rhs, c->n_dofs));
    RC(co_mass_solve_dev(c, c->b, c->f));
    RC(d2h(c, out, c->f, c->n_dofs));
    return finish(c);
}

extern "C" int co_picard_map(co_ctx *c, const co_opts *o, double *v_out, const double *v_in,
                             const double *v0, const double *w, int N, double S0, double dt) {
    ENTER(c);
    RC(check_opts(o));
    if (N < 0 || (N > 0 && (!v_out || !v_in || !v0 || !w))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v_in, 2 * (size_t)N) || !all_finite(v0, 2 * (size_t)N) || !all_finite(w, N))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vin, v_in, 2 * (size_t)N));
    RC(h2d(c, b.v0, v0, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    CO_CK(cudaMemsetAsync(&c->st->error, 0, sizeof(int), c->stream));
    RC(co_picard_map_dev(c, o, o->precision, b.Gv, b.vin, b.v0, b.w, N, S0, dt, 0));
    RC(d2h(c, v_out, b.Gv, 2 * (size_t)N));
    CO_CK(cudaMemcpyAsync(c->st_host, c->st, sizeof(co_solver_state), cudaMemcpyDeviceToHost,
                          c->stream));
    RC(finish(c));
    return c->st_host->error ? c->st_host->error : CO_OK;
}

extern "C" int co_step_anderson(co_ctx *c, const co_opts *o, double *v1, const double *v0,
                                const double *w, int N, double S0, double dt, int *iters,
                                double *res, int *nrs, double *r0) {
    ENTER(c);
    RC(check_opts(o));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    if (N > 0 && (!all_finite(v1, 2 * (size_t)N) || !all_finite(v0, 2 * (size_t)N) ||
                  !all_finite(w, N)))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, o->m));
    co_bufs &b = c->mb;
    RC(h2d(c, b.v1, v1, 2 * (size_t)N));
    RC(h2d(c, b.v0, v0, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_step_anderson_buffers(c, o, N, S0, dt, iters, res, nrs, r0));
    RC(d2h(c, v1, b.v1, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_step_anderson_dev(co_ctx *c, const co_opts *o, double *v1, const double *v0,
                                    const double *w, int N, double S0, double dt, int *iters,
                                    double *res, int *nrs, double *r0) {
    ENTER(c);
    RC(check_opts(o));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    RC(co_ensure_capacity(c, N, o->m));
    co_bufs &b = c->mb;
    size_t n2 = 2 * (size_t)N * sizeof(double);
    if (N > 0) {
        CO_CK(cudaMemcpyAsync(b.v1, v1, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.v0, v0, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
    }
    RC(co_step_anderson_buffers(c, o, N, S0, dt, iters, res, nrs, r0));
    if (N > 0) CO_CK(cudaMemcpyAsync(v1, b.v1, n2, cudaMemcpyDeviceToDevice, c->stream));
    return finish(c);
}

extern "C" int co_predictor(co_ctx *c, const co_opts *o, double *v1, const double *v,
                            const double *w, int N, double dt) {
    ENTER(c);
    RC(check_opts(o));
    if (N < 0 || (N > 0 && (!v1 || !v || !w))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    if (!all_finite(v, 2 * (size_t)N) || !all_finite(w, N)) return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.v0, v, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_predictor_buffers(c, o, o->precision, b.v0, N, dt, b.v1));
    RC(d2h(c, v1, b.v1, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_predictor_dev(co_ctx *c, const co_opts *o, double *v1, const double *v,
                                const double *w, int N, double dt) {
    ENTER(c);
    RC(check_opts(o));
    if (N < 0 || (N > 0 && (!v1 || !v || !w))) return CO_ERR_ARG;
    if (N == 0) return CO_OK;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    CO_CK(cudaMemcpyAsync(b.v0, v, 2 * (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    RC(co_predictor_buffers(c, o, o->precision, b.v0, N, dt, b.v1));
    CO_CK(cudaMemcpyAsync(v1, b.v1, 2 * (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                          c->stream));
    return finish(c);
}

extern "C" int co_entropy_of_markers_dev(co_ctx *c, const double *v, const double *w, int N,
                                         double *S) {
    ENTER(c);
    if (N < 0 || !S || (N > 0 && (!v || !w))) return CO_ERR_ARG;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    if (N > 0)
        CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
    RC(co_sort_markers(c, v, N));
    RC(co_project_sorted(c, c->f));
    RC(co_entropy_parts_dev(c, c->f));
    RC(co_entropy_finalize_dev(c, c->y));
    RC(d2h(c, S, c->y, 1));
    return finish(c);
}

// post-step diagnostics (main.jl:298-307): out6 = {S, energy, P1, P2,
// ||f_s - f_p||_2, negative-part L1}
extern "C" int co_diagnostics_dev(co_ctx *c, const double *v, const double *w, int N,
                                  double *out6) {
    ENTER(c);
    if (N < 0 || !out6 || (N > 0 && (!v || !w))) return CO_ERR_ARG;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    if (N > 0)
        CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
    RC(co_diagnostics_impl(c, v, N, c->y));
    RC(d2h(c, out6, c->y, 6));
    return finish(c);
}

extern "C" int co_diagnostics(co_ctx *c, const double *v, const double *w, int N,
                              double *out6) {
    ENTER(c);
    if (N < 0 || !out6 || (N > 0 && (!v || !w))) return CO_ERR_ARG;
    if (N > 0 && (!all_finite(v, 2 * (size_t)N) || !all_finite(w, N))) return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.vmid, v, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_diagnostics_impl(c, b.vmid, N, c->y));
    RC(d2h(c, out6, c->y, 6));
    return finish(c);
}

static int check_newton(const co_opts *o, const co_newton_opts *k) {
    int rc = check_opts(o);
    if (rc) return rc;
    if (!k || k->krylov_max < 1 || k->krylov_max > 200 || !(k->fd_h > 0) ||
        !(k->eta_max > 0 && k->eta_max < 1))
        return CO_ERR_ARG;
    return CO_OK;
}

extern "C" int co_step_newton(co_ctx *c, const co_opts *o, const co_newton_opts *k, double *v1,
                              const double *v0, const double *w, int N, double S0, double dt,
                              int *evals, double *res, int *n_newton, double *r0, int *status) {
    ENTER(c);
    RC(check_newton(o, k));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    if (N > 0 && (!all_finite(v1, 2 * (size_t)N) || !all_finite(v0, 2 * (size_t)N) ||
                  !all_finite(w, N)))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    RC(h2d(c, b.v1, v1, 2 * (size_t)N));
    RC(h2d(c, b.v0, v0, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_step_newton_buffers(c, o, k, N, S0, dt, evals, res, n_newton, r0, status));
    RC(d2h(c, v1, b.v1, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_step_newton_dev(co_ctx *c, const co_opts *o, const co_newton_opts *k,
                                  double *v1, const double *v0, const double *w, int N, double S0,
                                  double dt, int *evals, double *res, int *n_newton, double *r0,
                                  int *status) {
    ENTER(c);
    RC(check_newton(o, k));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    RC(co_ensure_capacity(c, N, 1));
    co_bufs &b = c->mb;
    size_t n2 = 2 * (size_t)N * sizeof(double);
    if (N > 0) {
        CO_CK(cudaMemcpyAsync(b.v1, v1, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.v0, v0, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
    }
    RC(co_step_newton_buffers(c, o, k, N, S0, dt, evals, res, n_newton, r0, status));
    if (N > 0) CO_CK(cudaMemcpyAsync(v1, b.v1, n2, cudaMemcpyDeviceToDevice, c->stream));
    return finish(c);
}

static int check_defect(const co_opts *o, const co_defect_opts *d) {
    int rc = check_opts(o);
    if (rc) return rc;
    if (!d || o->model != CO_MODEL_LANDAU || d->max_inner < 1 || d->stag_window < 1 ||
        !(d->eta > 0) || d->cap_abort < 0)
        return CO_ERR_ARG;
    return CO_OK;
}

extern "C" int co_step_defect(co_ctx *c, const co_opts *o, const co_defect_opts *d, double *v1,
                              const double *v0, const double *w, int N, double S0, double dt,
                              int *outer, double *res, int *inner, double *r0) {
    ENTER(c);
    RC(check_defect(o, d));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    if (N > 0 && (!all_finite(v1, 2 * (size_t)N) || !all_finite(v0, 2 * (size_t)N) ||
                  !all_finite(w, N)))
        return CO_ERR_NONFINITE;
    RC(co_ensure_capacity(c, N, o->m));
    co_bufs &b = c->mb;
    RC(h2d(c, b.v1, v1, 2 * (size_t)N));
    RC(h2d(c, b.v0, v0, 2 * (size_t)N));
    RC(h2d(c, b.w, w, N));
    RC(co_step_defect_buffers(c, o, d, N, S0, dt, outer, res, inner, r0));
    RC(d2h(c, v1, b.v1, 2 * (size_t)N));
    return finish(c);
}

extern "C" int co_step_defect_dev(co_ctx *c, const co_opts *o, const co_defect_opts *d,
                                  double *v1, const double *v0, const double *w, int N, double S0,
                                  double dt, int *outer, double *res, int *inner, double *r0) {
    ENTER(c);
    RC(check_defect(o, d));
    if (N < 0 || (N > 0 && (!v1 || !v0 || !w))) return CO_ERR_ARG;
    RC(co_ensure_capacity(c, N, o->m));
    co_bufs &b = c->mb;
    size_t n2 = 2 * (size_t)N * sizeof(double);
    if (N > 0) {
        CO_CK(cudaMemcpyAsync(b.v1, v1, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.v0, v0, n2, cudaMemcpyDeviceToDevice, c->stream));
        CO_CK(cudaMemcpyAsync(b.w, w, (size_t)N * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
    }
    RC(co_step_defect_buffers(c, o, d, N, S0, dt, outer, res, inner, r0));
    if (N > 0) CO_CK(cudaMemcpyAsync(v1, b.v1, n2, cudaMemcpyDeviceToDevice, c->stream));
    return finish(c);
}
