/*
 * oracle.c -- CPU FP64 restatement of the CollisionOperators.jl hot path.
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); the shipped
 * library never links or calls it. Parity status: partially pinned -- see
 * oracle.h for what pins it.
 *
 * Each function restates one reference routine in the same loop order and with
 * the same guards and clamps; citations are file:line in the reference tree.
 * The Mantis.jl pieces (B-spline space, extraction, Gauss-Legendre rule, mass
 * matrix) are restated from the mathematics:
 *   - clamped quadratic knot vector on the breakpoints, single interior knots
 *     (regularity 1): n_dofs_1d = n_el + 2, element e carries basis e, e+1, e+2;
 *   - Bezier extraction of that space (knot insertion for quadratics);
 *   - Gauss-Legendre nodes mapped to [0,1], weights summing to 1, times the
 *     element area;
 *   - the mass matrix assembled element by element with the 3x3 rule, then
 *     factorised (banded Cholesky instead of sparse LU; same solution up to
 *     round-off).
 * Compile with -ffp-contract=off: Julia does not fuse a*b+c unless asked to.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FS_FLOOR 1e-30 /* functions.jl:23 */
#define G_MAX 100.0    /* functions.jl:31 */

struct om_mesh {
    int n1, n2;          /* elements per dimension */
    double *bp1, *bp2;   /* n+1 breakpoints each */
    int nd1, nd2, n_dofs, n_el;
    double *C1, *C2;     /* extraction [n][3][3]: phi_j = sum_k C[k][j] B_k */
    int nq;
    double qx[32], qw[32];
    int bw;              /* half bandwidth of the 2D mass matrix */
    double *Lb;          /* banded Cholesky factor, row i: cols i-bw..i */
    int use_logsq;
    int mass_kind;       /* 0: 2D banded Cholesky (default); 1: tensor-product
                            solve with the 1D factors below                      */
    double *L1, *L2;     /* banded Cholesky factors of the 1D mass matrices,
                            row i: cols i-2..i (5-diagonal matrices)            */
    double *I1, *I2;     /* dense inverses of the 1D mass matrices (kind 2)    */
};

/* ---------------------------------------------------------------- quadrature */

/* Gauss-Legendre rule on [0,1] (weights sum to 1) by Newton on P_n. */
static void gauss_legendre01(int n, double *x, double *w) {
    for (int i = 0; i < n; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5));
        double pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            pp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / pp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            pp = n * (z * p1 - p0) / (z * z - 1.0);
        }
        /* ascending order on [0,1] */
        x[i] = 0.5 * (1.0 + z);
        w[i] = 1.0 / ((1.0 - z * z) * pp * pp);
    }
    /* sort ascending (cos gives descending z) */
    for (int i = 0; i < n / 2; i++) {
        double t = x[i]; x[i] = x[n - 1 - i]; x[n - 1 - i] = t;
        t = w[i]; w[i] = w[n - 1 - i]; w[n - 1 - i] = t;
    }
}

/* ------------------------------------------------------------------- basis */

/* Bezier extraction of the clamped C1 quadratic B-spline space on breakpoints
 * bp[0..n]: element e with neighbour widths hl (left), h, hr (right), hl = 0 at
 * the first element and hr = 0 at the last. */
static void build_extraction(const double *bp, int n, double *C) {
    for (int e = 0; e < n; e++) {
        double h = bp[e + 1] - bp[e];
        double hl = e > 0 ? bp[e] - bp[e - 1] : 0.0;
        double hr = e < n - 1 ? bp[e + 2] - bp[e + 1] : 0.0;
        double *c = C + 9 * e; /* c[k*3 + j] */
        memset(c, 0, 9 * sizeof(double));
        c[0 * 3 + 0] = h / (hl + h);
        c[0 * 3 + 1] = hl / (hl + h);
        c[1 * 3 + 1] = 1.0;
        c[2 * 3 + 1] = hr / (h + hr);
        c[2 * 3 + 2] = h / (h + hr);
    }
}

/* _bernstein_eval! for p = 2 (MantisWrappers.jl:201-216), same expression
 * order: binomial(p,i) * xi^i * (1-xi)^(p-i) and p*(left - right). */
static void bern2(double xi, double *B, double *dB) {
    double om = 1.0 - xi;
    B[0] = 1.0 * 1.0 * (om * om);
    B[1] = 2.0 * xi * om;
    B[2] = 1.0 * (xi * xi) * 1.0;
    if (dB) {
        dB[0] = 2.0 * (0.0 - 1.0 * 1.0 * om);
        dB[1] = 2.0 * (1.0 * 1.0 * om - 1.0 * xi * 1.0);
        dB[2] = 2.0 * (1.0 * xi * 1.0 - 0.0);
    }
}

/* mul!(phi, transpose(C), B) */
static void extract3(const double *c, const double *B, double *phi) {
    for (int j = 0; j < 3; j++)
        phi[j] = c[0 * 3 + j] * B[0] + c[1 * 3 + j] * B[1] + c[2 * 3 + j] * B[2];
}

/* searchsortedlast(bp, x) - 1 for bp[0] < x < bp[n] */
static int search_last(const double *bp, int n, double x) {
    int lo = 0, hi = n; /* bp[lo] <= x < bp[hi] */
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (bp[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

typedef struct {
    int i, j;          /* element indices (0-based) */
    double xi1, xi2, h1, h2;
} loc_t;

/* locate_particle (MantisWrappers.jl:168-179) */
static int locate(const om_mesh *m, double v1, double v2, loc_t *L) {
    if (v1 <= m->bp1[0] || v1 >= m->bp1[m->n1] || v2 <= m->bp2[0] ||
        v2 >= m->bp2[m->n2])
        return 0;
    int i = search_last(m->bp1, m->n1, v1);
    int j = search_last(m->bp2, m->n2, v2);
    L->i = i;
    L->j = j;
    L->h1 = m->bp1[i + 1] - m->bp1[i];
    L->h2 = m->bp2[j + 1] - m->bp2[j];
    L->xi1 = (v1 - m->bp1[i]) / L->h1;
    L->xi2 = (v2 - m->bp2[j]) / L->h2;
    return 1;
}

/* fast_eval_particle[_grad]! (MantisWrappers.jl:219-289): k = j1 + 3*j2 */
static void eval_particle(const om_mesh *m, const loc_t *L, double *vals,
                          double *dx1, double *dx2, int *gids) {
    double B1[3], dB1[3], B2[3], dB2[3], p1[3], dp1[3], p2[3], dp2[3];
    bern2(L->xi1, B1, dB1);
    bern2(L->xi2, B2, dB2);
    extract3(m->C1 + 9 * L->i, B1, p1);
    extract3(m->C2 + 9 * L->j, B2, p2);
    if (dx1) {
        extract3(m->C1 + 9 * L->i, dB1, dp1);
        extract3(m->C2 + 9 * L->j, dB2, dp2);
    }
    int k = 0;
    for (int j2 = 0; j2 < 3; j2++)
        for (int j1 = 0; j1 < 3; j1++) {
            vals[k] = p1[j1] * p2[j2];
            if (dx1) {
                dx1[k] = dp1[j1] * p2[j2];
                dx2[k] = p1[j1] * dp2[j2];
            }
            gids[k] = (L->i + j1) + (L->j + j2) * m->nd1;
            k++;
        }
}

/* ------------------------------------------------------------- mass matrix */

static void assemble_mass_band(om_mesh *m) {
    int nd = m->n_dofs, bw = m->bw;
    double *A = calloc((size_t)nd * (bw + 1), sizeof(double)); /* A[i][bw - (i-j)] */
    double gx[3], gw[3];
    gauss_legendre01(3, gx, gw);
    for (int ej = 0; ej < m->n2; ej++)
        for (int ei = 0; ei < m->n1; ei++) {
            double h1 = m->bp1[ei + 1] - m->bp1[ei];
            double h2 = m->bp2[ej + 1] - m->bp2[ej];
            double jac = h1 * h2;
            for (int q2 = 0; q2 < 3; q2++)
                for (int q1 = 0; q1 < 3; q1++) {
                    double B1[3], B2[3], p1[3], p2[3];
                    bern2(gx[q1], B1, NULL);
                    bern2(gx[q2], B2, NULL);
                    extract3(m->C1 + 9 * ei, B1, p1);
                    extract3(m->C2 + 9 * ej, B2, p2);
                    double wq = gw[q1] * gw[q2];
                    for (int a2 = 0; a2 < 3; a2++)
                        for (int a1 = 0; a1 < 3; a1++) {
                            int gi = (ei + a1) + (ej + a2) * m->nd1;
                            double fi = p1[a1] * p2[a2];
                            for (int b2 = 0; b2 < 3; b2++)
                                for (int b1 = 0; b1 < 3; b1++) {
                                    int gj = (ei + b1) + (ej + b2) * m->nd1;
                                    if (gj > gi) continue;
                                    double fj = p1[b1] * p2[b2];
                                    A[(size_t)gi * (bw + 1) + (bw - (gi - gj))] +=
                                        fi * fj * wq * jac;
                                }
                        }
                }
        }
    /* banded Cholesky, in place */
    for (int i = 0; i < nd; i++) {
        int j0 = i - bw < 0 ? 0 : i - bw;
        for (int j = j0; j <= i; j++) {
            double s = A[(size_t)i * (bw + 1) + (bw - (i - j))];
            int k0 = (i - bw > j - bw ? i - bw : j - bw);
            if (k0 < 0) k0 = 0;
            for (int k = k0; k < j; k++)
                s -= A[(size_t)i * (bw + 1) + (bw - (i - k))] *
                     A[(size_t)j * (bw + 1) + (bw - (j - k))];
            if (j == i)
                A[(size_t)i * (bw + 1) + bw] = sqrt(s);
            else
                A[(size_t)i * (bw + 1) + (bw - (i - j))] =
                    s / A[(size_t)j * (bw + 1) + bw];
        }
    }
    m->Lb = A;
}

/* 1D mass matrix of dimension d (3-point GL per element, the same rule as the
 * 2D assembly, of which M = M2 (x) M1 is the Kronecker product) and its banded
 * Cholesky factor, half bandwidth 2. */
static double *mass1d_factor(const double *bp, int n, const double *C) {
    int nd = n + 2;
    double *A = calloc((size_t)nd * 3, sizeof(double)); /* A[i][2 - (i-j)] */
    double gx[3], gw[3];
    gauss_legendre01(3, gx, gw);
    for (int e = 0; e < n; e++) {
        double h = bp[e + 1] - bp[e];
        for (int q = 0; q < 3; q++) {
            double B[3], p[3];
            bern2(gx[q], B, NULL);
            extract3(C + 9 * e, B, p);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b <= a; b++)
                    A[(size_t)(e + a) * 3 + (2 - (a - b))] += p[a] * p[b] * gw[q] * h;
        }
    }
    for (int i = 0; i < nd; i++) {
        int j0 = i - 2 < 0 ? 0 : i - 2;
        for (int j = j0; j <= i; j++) {
            double s = A[(size_t)i * 3 + (2 - (i - j))];
            int k0 = j - 2 > j0 ? j - 2 : j0;
            for (int k = k0; k < j; k++)
                s -= A[(size_t)i * 3 + (2 - (i - k))] * A[(size_t)j * 3 + (2 - (j - k))];
            if (j == i) A[(size_t)i * 3 + 2] = sqrt(s);
            else A[(size_t)i * 3 + (2 - (i - j))] = s / A[(size_t)j * 3 + 2];
        }
    }
    return A;
}

/* x <- M^{-1} x for one line of a 1D factor L (length nd, stride st) */
static void line_solve(const double *L, int nd, double *x, size_t st) {
    for (int i = 0; i < nd; i++) {
        double s = x[i * st];
        for (int k = (i - 2 < 0 ? 0 : i - 2); k < i; k++) s -= L[(size_t)i * 3 + (2 - (i - k))] * x[k * st];
        x[i * st] = s / L[(size_t)i * 3 + 2];
    }
    for (int i = nd - 1; i >= 0; i--) {
        double s = x[i * st];
        for (int k = i + 1; k <= (i + 2 < nd ? i + 2 : nd - 1); k++)
            s -= L[(size_t)k * 3 + (2 - (k - i))] * x[k * st];
        x[i * st] = s / L[(size_t)i * 3 + 2];
    }
}

/* dense inverse of the 1D mass matrix from its factor (columns solved one by one) */
static double *dense_inverse(const double *L, int nd) {
    double *I = calloc((size_t)nd * nd, sizeof(double));
    for (int j = 0; j < nd; j++) {
        I[(size_t)j * nd + j] = 1.0;
        line_solve(L, nd, I + (size_t)j * nd, 1);   /* column j (symmetric) */
    }
    return I;
}

void om_set_mass_solver(om_mesh *m, int kind) {
    m->mass_kind = (kind == 1 || kind == 2) ? kind : 0;
    if (m->mass_kind >= 1 && !m->L1) {
        m->L1 = mass1d_factor(m->bp1, m->n1, m->C1);
        m->L2 = mass1d_factor(m->bp2, m->n2, m->C2);
    }
    if (m->mass_kind == 2 && !m->I1) {
        m->I1 = dense_inverse(m->L1, m->nd1);
        m->I2 = dense_inverse(m->L2, m->nd2);
    }
}

void om_mass_solve(const om_mesh *m, const double *rhs, double *out) {
    int nd = m->n_dofs, bw = m->bw;
    if (m->mass_kind == 2) {
        /* out = M1^{-1} B M2^{-1} by dense products with the 1D inverses */
        int n1 = m->nd1, n2 = m->nd2;
        double *y = malloc(sizeof(double) * nd);
        for (int i2 = 0; i2 < n2; i2++)
            for (int i1 = 0; i1 < n1; i1++) {
                double s = 0.0;
                for (int k = 0; k < n1; k++) s = fma(m->I1[(size_t)k * n1 + i1], rhs[(size_t)i2 * n1 + k], s);
                y[(size_t)i2 * n1 + i1] = s;
            }
        for (int i2 = 0; i2 < n2; i2++)
            for (int i1 = 0; i1 < n1; i1++) {
                double s = 0.0;
                for (int k = 0; k < n2; k++) s = fma(y[(size_t)k * n1 + i1], m->I2[(size_t)k * n2 + i2], s);
                out[(size_t)i2 * n1 + i1] = s;
            }
        free(y);
        return;
    }
    if (m->mass_kind == 1) {
        /* M = M2 (x) M1 with index i1 + i2 nd1: solve along i1, then along i2 */
        memcpy(out, rhs, sizeof(double) * nd);
        for (int i2 = 0; i2 < m->nd2; i2++) line_solve(m->L1, m->nd1, out + (size_t)i2 * m->nd1, 1);
        for (int i1 = 0; i1 < m->nd1; i1++) line_solve(m->L2, m->nd2, out + i1, m->nd1);
        return;
    }
    const double *A = m->Lb;
    double *y = malloc(sizeof(double) * nd);
    for (int i = 0; i < nd; i++) {
        double s = rhs[i];
        int k0 = i - bw < 0 ? 0 : i - bw;
        for (int k = k0; k < i; k++) s -= A[(size_t)i * (bw + 1) + (bw - (i - k))] * y[k];
        y[i] = s / A[(size_t)i * (bw + 1) + bw];
    }
    for (int i = nd - 1; i >= 0; i--) {
        double s = y[i];
        int k1 = i + bw >= nd ? nd - 1 : i + bw;
        for (int k = i + 1; k <= k1; k++) s -= A[(size_t)k * (bw + 1) + (bw - (k - i))] * out[k];
        out[i] = s / A[(size_t)i * (bw + 1) + bw];
    }
    free(y);
}

void om_mass_matrix_dense(const om_mesh *m, double *out) {
    int nd = m->n_dofs, bw = m->bw;
    /* rebuild L L^T from the factor */
    memset(out, 0, sizeof(double) * (size_t)nd * nd);
    for (int i = 0; i < nd; i++)
        for (int j = (i - bw < 0 ? 0 : i - bw); j <= i; j++) {
            double s = 0.0;
            int k0 = i - bw > j - bw ? i - bw : j - bw;
            if (k0 < 0) k0 = 0;
            for (int k = k0; k <= j; k++)
                s += m->Lb[(size_t)i * (bw + 1) + (bw - (i - k))] *
                     m->Lb[(size_t)j * (bw + 1) + (bw - (j - k))];
            out[(size_t)i * nd + j] = s;
            out[(size_t)j * nd + i] = s;
        }
}

/* -------------------------------------------------------------- workspace */

om_mesh *om_create(const double *bp1, int nb1, const double *bp2, int nb2,
                   int nquad, int use_logsq) {
    if (nb1 < 2 || nb2 < 2 || nquad < 1 || nquad > 32) return NULL;
    om_mesh *m = calloc(1, sizeof(om_mesh));
    m->n1 = nb1 - 1;
    m->n2 = nb2 - 1;
    m->bp1 = malloc(sizeof(double) * nb1);
    m->bp2 = malloc(sizeof(double) * nb2);
    memcpy(m->bp1, bp1, sizeof(double) * nb1);
    memcpy(m->bp2, bp2, sizeof(double) * nb2);
    m->nd1 = m->n1 + 2;
    m->nd2 = m->n2 + 2;
    m->n_dofs = m->nd1 * m->nd2;
    m->n_el = m->n1 * m->n2;
    m->C1 = malloc(sizeof(double) * 9 * m->n1);
    m->C2 = malloc(sizeof(double) * 9 * m->n2);
    build_extraction(m->bp1, m->n1, m->C1);
    build_extraction(m->bp2, m->n2, m->C2);
    m->nq = nquad;
    gauss_legendre01(nquad, m->qx, m->qw);
    m->bw = 2 * m->nd1 + 2;
    m->use_logsq = use_logsq;
    assemble_mass_band(m);
    return m;
}

void om_destroy(om_mesh *m) {
    if (!m) return;
    free(m->bp1); free(m->bp2); free(m->C1); free(m->C2); free(m->Lb);
    free(m->L1); free(m->L2); free(m->I1); free(m->I2);
    free(m);
}

int om_n_dofs(const om_mesh *m) { return m->n_dofs; }
int om_nd1(const om_mesh *m) { return m->nd1; }

void om_extraction(const om_mesh *m, int dim, double *out) {
    if (dim == 1) memcpy(out, m->C1, sizeof(double) * 9 * m->n1);
    else memcpy(out, m->C2, sizeof(double) * 9 * m->n2);
}

void om_quadrature(const om_mesh *m, double *x, double *w) {
    memcpy(x, m->qx, sizeof(double) * m->nq);
    memcpy(w, m->qw, sizeof(double) * m->nq);
}

/* -------------------------------------------------------------- projection */

void om_l2_rhs(const om_mesh *m, const double *v, const double *w, int N,
               double *rhs) {
    memset(rhs, 0, sizeof(double) * m->n_dofs);
    for (int a = 0; a < N; a++) {
        loc_t L;
        if (!locate(m, v[a], v[N + a], &L)) continue;
        double vals[9];
        int gids[9];
        eval_particle(m, &L, vals, NULL, NULL, gids);
        for (int j = 0; j < 9; j++) rhs[gids[j]] += w[a] * vals[j];
    }
}

/* l2_project! (functions.jl:121-134) */
void om_l2_project(const om_mesh *m, const double *v, const double *w, int N,
                   double *f_out) {
    double *rhs = malloc(sizeof(double) * m->n_dofs);
    om_l2_rhs(m, v, w, N, rhs);
    om_mass_solve(m, rhs, f_out);
    free(rhs);
}

/* field value and basis at quadrature point (q1, q2) of element (ei, ej) */
static double field_at_qp(const om_mesh *m, const double *c, int ei, int ej,
                          int q1, int q2, double *phi, int *gids) {
    double B1[3], B2[3], p1[3], p2[3];
    bern2(m->qx[q1], B1, NULL);
    bern2(m->qx[q2], B2, NULL);
    extract3(m->C1 + 9 * ei, B1, p1);
    extract3(m->C2 + 9 * ej, B2, p2);
    double f = 0.0;
    int k = 0;
    for (int j2 = 0; j2 < 3; j2++)
        for (int j1 = 0; j1 < 3; j1++) {
            phi[k] = p1[j1] * p2[j2];
            gids[k] = (ei + j1) + (ej + j2) * m->nd1;
            f += c[gids[k]] * phi[k];
            k++;
        }
    return f;
}

/* compute_entropy (functions.jl:137-155) */
double om_entropy(const om_mesh *m, const double *f) {
    double S = 0.0;
    for (int ej = 0; ej < m->n2; ej++)
        for (int ei = 0; ei < m->n1; ei++) {
            double jac = (m->bp1[ei + 1] - m->bp1[ei]) * (m->bp2[ej + 1] - m->bp2[ej]);
            for (int q2 = 0; q2 < m->nq; q2++)
                for (int q1 = 0; q1 < m->nq; q1++) {
                    double phi[9];
                    int gids[9];
                    double fv = field_at_qp(m, f, ei, ej, q1, q2, phi, gids);
                    double wq = m->qw[q1] * m->qw[q2];
                    if (m->use_logsq) {
                        if (fv * fv > 1e-60)
                            S -= fv * 0.5 * log(fv * fv) * wq * jac;
                    } else if (fv > 1e-30) {
                        S -= fv * log(fv) * wq * jac;
                    }
                }
        }
    return S;
}

/* Post-step diagnostics of the time loop (main.jl:298-307): out6 = entropy S of
 * the projection of v, energy 1/2 sum w |v|^2 (compute_energy, functions.jl:355-358),
 * momentum sum w v (compute_momentum, :349-353), ||f_s - f_p||_2 with f_p the
 * element-constant histogram density (compute_fs_minus_fp_l2, :315-347) and the
 * negative-part L1 norm of f_s (compute_negative_part_l1, :300-313), both on the
 * N_QUAD Gauss grid. Element masses are summed over the markers located in
 * each element, as the reference does. */
void om_diagnostics(const om_mesh *m, const double *v, const double *w, int N, double *out6) {
    double *f = malloc(sizeof(double) * m->n_dofs);
    double *emass = calloc((size_t)m->n1 * m->n2, sizeof(double));
    om_l2_project(m, v, w, N, f);
    double E = 0.0, P1 = 0.0, P2 = 0.0;
    for (int a = 0; a < N; a++) {
        P1 += w[a] * v[a];
        P2 += w[a] * v[N + a];
        E += w[a] * (v[a] * v[a] + v[N + a] * v[N + a]);
        loc_t L;
        if (locate(m, v[a], v[N + a], &L)) emass[L.i + L.j * m->n1] += w[a];
    }
    double sumsq = 0.0, neg = 0.0;
    for (int ej = 0; ej < m->n2; ej++)
        for (int ei = 0; ei < m->n1; ei++) {
            double jac = (m->bp1[ei + 1] - m->bp1[ei]) * (m->bp2[ej + 1] - m->bp2[ej]);
            double fp = emass[ei + ej * m->n1] / jac;
            for (int q2 = 0; q2 < m->nq; q2++)
                for (int q1 = 0; q1 < m->nq; q1++) {
                    double phi[9];
                    int gids[9];
                    double fv = field_at_qp(m, f, ei, ej, q1, q2, phi, gids);
                    double wq = m->qw[q1] * m->qw[q2];
                    if (fv < 0.0) neg += (-fv) * wq * jac;
                    double d = fv - fp;
                    sumsq += d * d * wq * jac;
                }
        }
    out6[0] = om_entropy(m, f);
    out6[1] = 0.5 * E;
    out6[2] = P1;
    out6[3] = P2;
    out6[4] = sqrt(sumsq);
    out6[5] = neg;
    free(f);
    free(emass);
}

/* compute_r! (functions.jl:158-179) */
void om_compute_r(const om_mesh *m, const double *f, double *r) {
    memset(r, 0, sizeof(double) * m->n_dofs);
    for (int ej = 0; ej < m->n2; ej++)
        for (int ei = 0; ei < m->n1; ei++) {
            double jac = (m->bp1[ei + 1] - m->bp1[ei]) * (m->bp2[ej + 1] - m->bp2[ej]);
            for (int q2 = 0; q2 < m->nq; q2++)
                for (int q1 = 0; q1 < m->nq; q1++) {
                    double phi[9];
                    int gids[9];
                    double fv = field_at_qp(m, f, ei, ej, q1, q2, phi, gids);
                    double integrand;
                    if (m->use_logsq)
                        integrand = fv * fv > 1e-60 ? (1 + 0.5 * log(fv * fv)) : 0.0;
                    else
                        integrand = fv > 1e-30 ? (1 + log(fv)) : 0.0;
                    double wq = m->qw[q1] * m->qw[q2];
                    for (int j = 0; j < 9; j++)
                        r[gids[j]] += integrand * phi[j] * wq * jac;
                }
        }
}

/* compute_G! (functions.jl:182-202) */
void om_compute_G(const om_mesh *m, const double *v, int N, const double *Lv,
                  double *G) {
    for (int a = 0; a < N; a++) {
        G[a] = 0.0;
        G[N + a] = 0.0;
        loc_t L;
        if (!locate(m, v[a], v[N + a], &L)) continue;
        double vals[9], dx1[9], dx2[9];
        int gids[9];
        eval_particle(m, &L, vals, dx1, dx2, gids);
        double ih1 = 1.0 / L.h1, ih2 = 1.0 / L.h2;
        double acc1 = 0.0, acc2 = 0.0;
        for (int j = 0; j < 9; j++) {
            double c = Lv[gids[j]];
            acc1 += c * dx1[j] * ih1;
            acc2 += c * dx2[j] * ih2;
        }
        G[a] = acc1;
        G[N + a] = acc2;
    }
}

/* eval_loggrad_at_particles! (functions.jl:37-64) */
void om_loggrad(const om_mesh *m, const double *v, int N, const double *fc,
                double *g) {
    for (int a = 0; a < N; a++) {
        loc_t L;
        if (!locate(m, v[a], v[N + a], &L)) {
            g[a] = 0.0;
            g[N + a] = 0.0;
            continue;
        }
        double vals[9], dx1[9], dx2[9];
        int gids[9];
        eval_particle(m, &L, vals, dx1, dx2, gids);
        double ih1 = 1.0 / L.h1, ih2 = 1.0 / L.h2;
        double f = 0.0, d1 = 0.0, d2 = 0.0;
        for (int j = 0; j < 9; j++) {
            double c = fc[gids[j]];
            f += c * vals[j];
            d1 += c * dx1[j] * ih1;
            d2 += c * dx2[j] * ih2;
        }
        double invf = 1.0 / fmax(fabs(f), FS_FLOOR);
        double g1 = d1 * invf, g2 = d2 * invf;
        g[a] = g1 < -G_MAX ? -G_MAX : (g1 > G_MAX ? G_MAX : g1);
        g[N + a] = g2 < -G_MAX ? -G_MAX : (g2 > G_MAX ? G_MAX : g2);
    }
}

double om_eval_field(const om_mesh *m, const double *c, double x1, double x2) {
    loc_t L;
    if (!locate(m, x1, x2, &L)) return 0.0;
    double vals[9];
    int gids[9];
    eval_particle(m, &L, vals, NULL, NULL, gids);
    double f = 0.0;
    for (int j = 0; j < 9; j++) f += c[gids[j]] * vals[j];
    return f;
}

/* --------------------------------------------------------------- pair sums */

static int set_threads(int nthreads) {
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

static inline int outside(const om_mesh *m, double a, double b) {
    return a <= m->bp1[0] || a >= m->bp1[m->n1] || b <= m->bp2[0] || b >= m->bp2[m->n2];
}

/* one target row of compute_collision! (functions.jl:211-234) */
static void collision_row(const om_mesh *m, const double *v, const double *w,
                          const double *G, int N, int g, double *o1, double *o2) {
    double vg1 = v[g], vg2 = v[N + g];
    *o1 = 0.0;
    *o2 = 0.0;
    if (outside(m, vg1, vg2)) return;
    double Gg1 = G[g], Gg2 = G[N + g];
    double acc1 = 0.0, acc2 = 0.0;
    for (int a = 0; a < N; a++) {
        if (a == g) continue;
        double va1 = v[a], va2 = v[N + a];
        if (outside(m, va1, va2)) continue;
        double d1 = vg1 - va1;
        double d2 = vg2 - va2;
        double dist2 = d1 * d1 + d2 * d2;
        if (dist2 < 1e-24) continue;
        double dist = sqrt(dist2);
        double g1 = G[a] - Gg1;
        double g2 = G[N + a] - Gg2;
        double dvg = (d1 * g1 + d2 * g2) / dist2;
        double inv = 1.0 / dist;
        acc1 += w[a] * (g1 - d1 * dvg) * inv;
        acc2 += w[a] * (g2 - d2 * dvg) * inv;
    }
    *o1 = acc1;
    *o2 = acc2;
}

/* compute_collision! (functions.jl:205-237): threaded over gamma as
 * Threads.@threads does at functions.jl:210 */
void om_collision(const om_mesh *m, const double *v, const double *w,
                  const double *G, int N, double *dot_v, int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int g = 0; g < N; g++) collision_row(m, v, w, G, N, g, &dot_v[g], &dot_v[N + g]);
}

void om_collision_rows(const om_mesh *m, const double *v, const double *w,
                       const double *G, int N, const int *rows, int nrows,
                       double *out, int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
    for (int r = 0; r < nrows; r++)
        collision_row(m, v, w, G, N, rows[r], &out[r], &out[nrows + r]);
}

/* compute_collision_metric! (functions.jl:249-290) */
void om_collision_metric(const om_mesh *m, const double *v, const double *w,
                         const double *G, int N, double *dot_v, double *A,
                         int nthreads) {
    int nt = set_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nt)
    for (int g = 0; g < N; g++) {
        double vg1 = v[g], vg2 = v[N + g];
        dot_v[g] = dot_v[N + g] = 0.0;
        A[g] = A[N + g] = A[2 * N + g] = 0.0;
        if (outside(m, vg1, vg2)) continue;
        double Gg1 = G[g], Gg2 = G[N + g];
        double acc1 = 0.0, acc2 = 0.0, a11 = 0.0, a12 = 0.0, a22 = 0.0;
        for (int a = 0; a < N; a++) {
            if (a == g) continue;
            double va1 = v[a], va2 = v[N + a];
            if (outside(m, va1, va2)) continue;
            double d1 = vg1 - va1;
            double d2 = vg2 - va2;
            double dist2 = d1 * d1 + d2 * d2;
            if (dist2 < 1e-24) continue;
            double dist = sqrt(dist2);
            double g1 = G[a] - Gg1;
            double g2 = G[N + a] - Gg2;
            double dvg = (d1 * g1 + d2 * g2) / dist2;
            double inv = 1.0 / dist;
            acc1 += w[a] * (g1 - d1 * dvg) * inv;
            acc2 += w[a] * (g2 - d2 * dvg) * inv;
            double s = w[a] * inv;
            a11 += s * (1 - d1 * d1 / dist2);
            a12 -= s * d1 * d2 / dist2;
            a22 += s * (1 - d2 * d2 / dist2);
        }
        dot_v[g] = acc1;
        dot_v[N + g] = acc2;
        A[g] = a11;
        A[N + g] = a12;
        A[2 * N + g] = a22;
    }
}

/* ---------------------------------------------------------------------- LB */

void om_moments(const double *v, const double *w, int N, double *out) {
    double n = 0.0, U1 = 0.0, U2 = 0.0, Q = 0.0;
    for (int a = 0; a < N; a++) {
        double wa = w[a], x = v[a], y = v[N + a];
        n += wa;
        U1 += wa * x;
        U2 += wa * y;
        Q += wa * (x * x + y * y);
    }
    out[0] = n; out[1] = U1; out[2] = U2; out[3] = Q;
}

/* dense LU with partial pivoting, as Julia's `\` (LAPACK getrf/getrs) */
static int lu_solve(int n, double *A, double *b) {
    int piv[32];
    for (int k = 0; k < n; k++) {
        int p = k;
        double mx = fabs(A[k * n + k]);
        for (int i = k + 1; i < n; i++)
            if (fabs(A[i * n + k]) > mx) { mx = fabs(A[i * n + k]); p = i; }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < n; j++) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
        if (A[k * n + k] == 0.0) return 1;
        for (int i = k + 1; i < n; i++) {
            A[i * n + k] /= A[k * n + k];
            for (int j = k + 1; j < n; j++) A[i * n + j] -= A[i * n + k] * A[k * n + j];
        }
    }
    for (int k = 0; k < n; k++) if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
    for (int i = 0; i < n; i++) for (int j = 0; j < i; j++) b[i] -= A[i * n + j] * b[j];
    for (int i = n - 1; i >= 0; i--) {
        for (int j = i + 1; j < n; j++) b[i] -= A[i * n + j] * b[j];
        b[i] /= A[i * n + i];
    }
    return 0;
}

void om_drift_multipliers(const double *v, const double *w, const double *g,
                          int N, double n, double U1, double U2, double Q,
                          double *out) {
    double Sg1 = 0.0, Sg2 = 0.0, P = 0.0;
    for (int a = 0; a < N; a++) {
        double g1 = g[a], g2 = g[N + a], wa = w[a];
        Sg1 += wa * g1;
        Sg2 += wa * g2;
        P += wa * (v[a] * g1 + v[N + a] * g2);
    }
    double M[9] = {n, 0.0, U1, 0.0, n, U2, U1, U2, Q};
    double rhs[3] = {-Sg1, -Sg2, -P};
    lu_solve(3, M, rhs);
    out[0] = rhs[0]; out[1] = rhs[1]; out[2] = rhs[2];
}

void om_lb_velocity(double *dot_v, const double *v, const double *g, int N,
                    double A1, double A2, double B, double nu) {
    for (int a = 0; a < N; a++) {
        dot_v[a] = -nu * (g[a] + A1 + B * v[a]);
        dot_v[N + a] = -nu * (g[N + a] + A2 + B * v[N + a]);
    }
}

/* ------------------------------------------------------------ Picard map */

/* compute_entropy_gradient! (solver.jl:62-74) */
static void entropy_gradient(const om_mesh *m, double *dS, const double *v,
                             const double *w, int N, double *fbuf, double *r,
                             double *L, double *G) {
    om_l2_project(m, v, w, N, fbuf);
    om_compute_r(m, fbuf, r);
    om_mass_solve(m, r, L);
    om_compute_G(m, v, N, L, G);
    for (int a = 0; a < N; a++) {
        dS[a] = -w[a] * G[a];
        dS[N + a] = -w[a] * G[N + a];
    }
}

/* picard_map! (solver.jl:176-227), with landau_geff! (solver.jl:86-113) */
void om_picard_map(const om_mesh *m, const om_opts *o, double *v_out,
                   const double *v_in, const double *v0, const double *w,
                   int N, double S0, double dt) {
    int nd = m->n_dofs;
    double *v_mid = malloc(sizeof(double) * 2 * N);
    double *dv = malloc(sizeof(double) * 2 * N);
    double *dS = malloc(sizeof(double) * 2 * N);
    double *Geff = malloc(sizeof(double) * 2 * N);
    double *dotv = malloc(sizeof(double) * 2 * N);
    double *Gb = malloc(sizeof(double) * 2 * N);
    double *fbuf = malloc(sizeof(double) * nd);
    double *r = malloc(sizeof(double) * nd);
    double *L = malloc(sizeof(double) * nd);
    for (int i = 0; i < 2 * N; i++) {
        v_mid[i] = 0.5 * (v0[i] + v_in[i]);
        dv[i] = v_in[i] - v0[i];
    }
    if (o->model == 1) {
        /* LB: direct clamped log-gradient base (solver.jl:185-210) */
        om_l2_project(m, v_mid, w, N, fbuf);
        om_loggrad(m, v_mid, N, fbuf, Geff);
        if (o->use_gonzalez) {
            om_l2_project(m, v_in, w, N, fbuf);
            double S1 = om_entropy(m, fbuf);
            double dot = 0.0, nrm2 = 0.0;
            for (int a = 0; a < N; a++) {
                dot -= w[a] * (dv[a] * Geff[a] + dv[N + a] * Geff[N + a]);
                nrm2 += dv[a] * dv[a] + dv[N + a] * dv[N + a];
            }
            double lam = nrm2 > 1e-30 ? (S1 - S0 - dot) / nrm2 : 0.0;
            for (int a = 0; a < N; a++) {
                double iw = 1.0 / w[a];
                Geff[a] -= lam * dv[a] * iw;
                Geff[N + a] -= lam * dv[N + a] * iw;
            }
        }
        double mo[4], ab[3];
        om_moments(v_mid, w, N, mo);
        om_drift_multipliers(v_mid, w, Geff, N, mo[0], mo[1], mo[2], mo[3], ab);
        om_lb_velocity(dotv, v_mid, Geff, N, ab[0], ab[1], ab[2], o->nu);
    } else {
        entropy_gradient(m, dS, v_mid, w, N, fbuf, r, L, Gb);
        double corr = 0.0;
        if (o->use_gonzalez) {
            om_l2_project(m, v_in, w, N, fbuf);
            double S1 = om_entropy(m, fbuf);
            double dot = 0.0, nrm2 = 0.0;
            for (int a = 0; a < N; a++) {
                dot += dv[a] * dS[a] + dv[N + a] * dS[N + a];
                nrm2 += dv[a] * dv[a] + dv[N + a] * dv[N + a];
            }
            corr = nrm2 > 1e-30 ? (S1 - S0 - dot) / nrm2 : 0.0;
        }
        for (int a = 0; a < N; a++) {
            double iw = 1.0 / w[a];
            Geff[a] = -(dS[a] + corr * dv[a]) * iw;
            Geff[N + a] = -(dS[N + a] + corr * dv[N + a]) * iw;
        }
        om_collision(m, v_mid, w, Geff, N, dotv, o->nthreads);
    }
    for (int i = 0; i < 2 * N; i++) v_out[i] = v0[i] + dt * dotv[i];
    free(v_mid); free(dv); free(dS); free(Geff); free(dotv); free(Gb);
    free(fbuf); free(r); free(L);
}

static double norm2v(const double *x, int n) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}

/* step_anderson! (solver.jl:300-423) */
void om_step_anderson(const om_mesh *m, const om_opts *o, double *v1,
                      const double *v0, const double *w, int N, double S0,
                      double dt, double *out4) {
    int n = 2 * N, mm = o->m;
    double *Gv = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n);
    double *rp = malloc(sizeof(double) * n), *Gp = malloc(sizeof(double) * n);
    double *vold = malloc(sizeof(double) * n), *vbest = malloc(sizeof(double) * n);
    double *dF = calloc((size_t)n * mm, sizeof(double));
    double *dG = calloc((size_t)n * mm, sizeof(double));
    double restart = o->restart_factor > 0 ? o->restart_factor : INFINITY;
    int history = 0, slot = 0, n_restart = 0;
    double nrm_r0 = 0.0, nrm_r = 0.0, nrm_best = INFINITY, nrm_best_window = INFINITY;
    memcpy(vbest, v1, sizeof(double) * n);
    for (int k = 1; k <= o->max_iter; k++) {
        memcpy(vold, v1, sizeof(double) * n);
        om_picard_map(m, o, Gv, v1, v0, w, N, S0, dt);
        for (int i = 0; i < n; i++) r[i] = Gv[i] - v1[i];
        nrm_r = norm2v(r, n);
        if (k == 1) nrm_r0 = nrm_r;
        if (nrm_r < nrm_best) {
            nrm_best = nrm_r;
            memcpy(vbest, o->exit_picard_step ? Gv : v1, sizeof(double) * n);
        }
        double eff_tol = fmax(o->tol * (norm2v(v1, n) + 1e-30), o->abs_floor);
        if (nrm_r < eff_tol) {
            if (o->exit_picard_step) memcpy(v1, Gv, sizeof(double) * n);
            out4[0] = k; out4[1] = nrm_r; out4[2] = n_restart; out4[3] = nrm_r0;
            goto done;
        }
        if (k > o->stag_window && k % o->stag_window == 0) {
            double rel = (nrm_best_window - nrm_best) / (nrm_best_window + 1e-30);
            if (rel < o->stag_rel_tol) {
                memcpy(v1, vbest, sizeof(double) * n);
                out4[0] = k; out4[1] = nrm_best; out4[2] = n_restart; out4[3] = nrm_r0;
                goto done;
            }
            nrm_best_window = nrm_best;
        }
        int just_restarted = 0;
        if (k > 1 && nrm_r > restart * nrm_best) {
            history = 0;
            slot = 0;
            n_restart++;
            just_restarted = 1;
        }
        double damp = k > o->damp_decay_start ? o->damping * o->damp_decay_factor : o->damping;
        if (k == 1 || just_restarted || !o->use_anderson) {
            for (int i = 0; i < n; i++) v1[i] = damp * Gv[i] + (1 - damp) * vold[i];
        } else {
            slot = slot % mm + 1; /* mod1(slot + 1, m) */
            history = history + 1 < mm ? history + 1 : mm;
            double *F = dF + (size_t)(slot - 1) * n, *Gc = dG + (size_t)(slot - 1) * n;
            for (int i = 0; i < n; i++) { F[i] = r[i] - rp[i]; Gc[i] = Gv[i] - Gp[i]; }
            double ATA[64], ATr[8];
            for (int a = 0; a < history; a++) {
                for (int b = 0; b < history; b++) {
                    double s = 0.0;
                    const double *Fa = dF + (size_t)a * n, *Fb = dF + (size_t)b * n;
                    for (int i = 0; i < n; i++) s += Fa[i] * Fb[i];
                    ATA[a * history + b] = s;
                }
                double s = 0.0;
                const double *Fa = dF + (size_t)a * n;
                for (int i = 0; i < n; i++) s += Fa[i] * r[i];
                ATr[a] = s;
            }
            double dm = 0.0;
            for (int j = 0; j < history; j++) dm += ATA[j * history + j];
            dm /= history;
            double l2 = o->reg_factor * dm + 1e-30;
            for (int j = 0; j < history; j++) ATA[j * history + j] += l2;
            lu_solve(history, ATA, ATr);
            for (int i = 0; i < n; i++) {
                double s = Gv[i];
                for (int j = 0; j < history; j++) s += -1.0 * dG[(size_t)j * n + i] * ATr[j];
                v1[i] = damp * s + (1 - damp) * vold[i];
            }
        }
        memcpy(rp, r, sizeof(double) * n);
        memcpy(Gp, Gv, sizeof(double) * n);
    }
    memcpy(v1, vbest, sizeof(double) * n);
    out4[0] = o->max_iter; out4[1] = nrm_best; out4[2] = n_restart; out4[3] = nrm_r0;
done:
    free(Gv); free(r); free(rp); free(Gp); free(vold); free(vbest); free(dF); free(dG);
}

/* Explicit predictor of the time loop (main.jl:233-245). */
void om_predictor(const om_mesh *m, const om_opts *o, double *v1,
                  const double *v, const double *w, int N, double dt) {
    int nd = m->n_dofs;
    double *fc = malloc(sizeof(double) * nd), *r = malloc(sizeof(double) * nd);
    double *L = malloc(sizeof(double) * nd);
    double *G = malloc(sizeof(double) * 2 * N), *dotv = malloc(sizeof(double) * 2 * N);
    om_l2_project(m, v, w, N, fc);
    if (o->model == 1) {
        double mo[4], ab[3];
        om_loggrad(m, v, N, fc, G);
        om_moments(v, w, N, mo);
        om_drift_multipliers(v, w, G, N, mo[0], mo[1], mo[2], mo[3], ab);
        om_lb_velocity(dotv, v, G, N, ab[0], ab[1], ab[2], o->nu);
    } else {
        om_compute_r(m, fc, r);
        om_mass_solve(m, r, L);
        om_compute_G(m, v, N, L, G);
        om_collision(m, v, w, G, N, dotv, o->nthreads);
    }
    for (int i = 0; i < 2 * N; i++) v1[i] = v[i] + dt * dotv[i];
    free(fc); free(r); free(L); free(G); free(dotv);
}

/* ---------------------------------------------------------- defect correction */

/* Hessian of the spline field L at markers v: (d11, d12, d22) L with the P2
 * basis' second derivatives d^2 B / dxi^2 = (2, -4, 2); 0 outside the domain.
 * H is 3N: H11, H12, H22. */
static void hessian_L(const om_mesh *m, const double *v, int N, const double *Lv, double *H) {
    static const double d2B[3] = {2.0, -4.0, 2.0};
    for (int a = 0; a < N; a++) {
        H[a] = H[N + a] = H[2 * N + a] = 0.0;
        loc_t L;
        if (!locate(m, v[a], v[N + a], &L)) continue;
        double B1[3], dB1[3], B2[3], dB2[3], p1[3], dp1[3], q1[3], p2[3], dp2[3], q2[3];
        bern2(L.xi1, B1, dB1);
        bern2(L.xi2, B2, dB2);
        extract3(m->C1 + 9 * L.i, B1, p1);
        extract3(m->C1 + 9 * L.i, dB1, dp1);
        extract3(m->C1 + 9 * L.i, d2B, q1);
        extract3(m->C2 + 9 * L.j, B2, p2);
        extract3(m->C2 + 9 * L.j, dB2, dp2);
        extract3(m->C2 + 9 * L.j, d2B, q2);
        double ih1 = 1.0 / L.h1, ih2 = 1.0 / L.h2, h11 = 0.0, h12 = 0.0, h22 = 0.0;
        for (int j2 = 0; j2 < 3; j2++)
            for (int j1 = 0; j1 < 3; j1++) {
                double c = Lv[(L.i + j1) + (L.j + j2) * m->nd1];
                h11 += c * (q1[j1] * p2[j2]) * (ih1 * ih1);
                h12 += c * (dp1[j1] * dp2[j2]) * (ih1 * ih2);
                h22 += c * (p1[j1] * q2[j2]) * (ih2 * ih2);
            }
        H[a] = h11;
        H[N + a] = h12;
        H[2 * N + a] = h22;
    }
}

void om_hessian_L(const om_mesh *m, const double *v, int N, const double *Lv, double *H) {
    hessian_L(m, v, N, Lv, H);
}

/* landau_geff! (solver.jl:86-113) at v_in: G_eff and (optionally) v_mid; with
 * H != NULL also the Hessian of L at v_mid and the Gonzalez lambda */
static void landau_geff_h(const om_mesh *m, int gonzalez, double *Geff, double *vmid,
                          const double *v_in, const double *v0, const double *w, int N, double S0,
                          double *H, double *lam_out);
static void landau_geff(const om_mesh *m, int gonzalez, double *Geff, double *vmid,
                        const double *v_in, const double *v0, const double *w, int N, double S0) {
    landau_geff_h(m, gonzalez, Geff, vmid, v_in, v0, w, N, S0, NULL, NULL);
}
static void landau_geff_h(const om_mesh *m, int gonzalez, double *Geff, double *vmid,
                          const double *v_in, const double *v0, const double *w, int N, double S0,
                          double *H, double *lam_out) {
    int nd = m->n_dofs;
    double *dv = malloc(sizeof(double) * 2 * N), *dS = malloc(sizeof(double) * 2 * N);
    double *Gb = malloc(sizeof(double) * 2 * N);
    double *fbuf = malloc(sizeof(double) * nd), *r = malloc(sizeof(double) * nd);
    double *L = malloc(sizeof(double) * nd);
    for (int i = 0; i < 2 * N; i++) {
        vmid[i] = 0.5 * (v0[i] + v_in[i]);
        dv[i] = v_in[i] - v0[i];
    }
    entropy_gradient(m, dS, vmid, w, N, fbuf, r, L, Gb);
    if (H) hessian_L(m, vmid, N, L, H);
    double corr = 0.0;
    if (gonzalez) {
        om_l2_project(m, v_in, w, N, fbuf);
        double S1 = om_entropy(m, fbuf);
        double dot = 0.0, nrm2 = 0.0;
        for (int a = 0; a < N; a++) {
            dot += dv[a] * dS[a] + dv[N + a] * dS[N + a];
            nrm2 += dv[a] * dv[a] + dv[N + a] * dv[N + a];
        }
        corr = nrm2 > 1e-30 ? (S1 - S0 - dot) / nrm2 : 0.0;
    }
    if (lam_out) *lam_out = corr;
    for (int a = 0; a < N; a++) {
        double iw = 1.0 / w[a];
        Geff[a] = -(dS[a] + corr * dv[a]) * iw;
        Geff[N + a] = -(dS[N + a] + corr * dv[N + a]) * iw;
    }
    free(dv); free(dS); free(Gb); free(fbuf); free(r); free(L);
}

typedef struct {
    const om_mesh *m;
    int gonzalez, N;
    const double *v0, *w, *Gv, *A, *Gk;
    double S0, dt;
    double *Geff, *vmid;
    int precond;       /* block-Newton preconditioning of the inner iteration */
    double *H, lam;    /* Hessian of L at v_mid and lambda of the last map      */
} frozen_ctx;

/* frozen_map! (solver.jl:585-595) */
static void frozen_map(frozen_ctx *f, double *out, const double *u) {
    int N = f->N;
    landau_geff_h(f->m, f->gonzalez, f->Geff, f->vmid, u, f->v0, f->w, N, f->S0,
                  f->precond ? f->H : NULL, f->precond ? &f->lam : NULL);
    for (int a = 0; a < N; a++) {
        double d1 = f->Geff[a] - f->Gk[a];
        double d2 = f->Geff[N + a] - f->Gk[N + a];
        out[a] = f->Gv[a] - f->dt * (f->A[a] * d1 + f->A[N + a] * d2);
        out[N + a] = f->Gv[N + a] - f->dt * (f->A[N + a] * d1 + f->A[2 * N + a] * d2);
    }
}

/* Block-Newton preconditioner of the inner iteration (the library's
 * extension; precond = 0 is the reference's iteration). Per marker, the
 * residual R(u) = Phi(u) - u has the local Jacobian -(I + dt A M) with
 * M = H/2 - (lambda/w) I (H the Hessian of L at v_mid: G_eff = G(v_mid) -
 * lambda dv / w, v_mid = (u + v0)/2); r <- (I + dt A M)^{-1} r, the 2x2 solve
 * skipped where |det| < 0.1. precond = 2 drops the lambda/w term (M = H/2).
 * The fixed points are unchanged. */
static void precondition(const frozen_ctx *f, double *r) {
    int N = f->N;
    for (int a = 0; a < N; a++) {
        double iw = 1.0 / f->w[a];
        double A11 = f->A[a], A12 = f->A[N + a], A22 = f->A[2 * N + a];
        double lt = f->precond == 1 ? f->lam * iw : 0.0;   /* mode 2: Hessian only */
        double M11 = 0.5 * f->H[a] - lt, M12 = 0.5 * f->H[N + a];
        double M22 = 0.5 * f->H[2 * N + a] - lt;
        double P11 = 1.0 + f->dt * (A11 * M11 + A12 * M12);
        double P12 = f->dt * (A11 * M12 + A12 * M22);
        double P21 = f->dt * (A12 * M11 + A22 * M12);
        double P22 = 1.0 + f->dt * (A12 * M12 + A22 * M22);
        double det = P11 * P22 - P12 * P21;
        if (!(fabs(det) >= 0.1)) continue;
        double r1 = r[a], r2 = r[N + a];
        r[a] = (P22 * r1 - P12 * r2) / det;
        r[N + a] = (P11 * r2 - P21 * r1) / det;
    }
}

/* _anderson_inner! (solver.jl:492-526); returns the number of map evaluations.
 * With fc->precond, Anderson runs on u + P^{-1} r; the stopping test stays on
 * the plain residual r. */
static int anderson_inner(frozen_ctx *fc, double *u, double tol, int maxit, int mm,
                          double damping, double reg_factor) {
    int n = 2 * fc->N;
    double *Fu = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n);
    double *rp = malloc(sizeof(double) * n), *Fp = malloc(sizeof(double) * n);
    double *uold = malloc(sizeof(double) * n);
    double *dF = calloc((size_t)n * mm, sizeof(double)), *dG = calloc((size_t)n * mm, sizeof(double));
    int hist = 0, slot = 0, ret = maxit;
    for (int k = 1; k <= maxit; k++) {
        memcpy(uold, u, sizeof(double) * n);
        frozen_map(fc, Fu, u);
        for (int i = 0; i < n; i++) r[i] = Fu[i] - u[i];
        if (norm2v(r, n) < tol) {
            memcpy(u, Fu, sizeof(double) * n);
            ret = k;
            break;
        }
        if (fc->precond) {
            precondition(fc, r);
            for (int i = 0; i < n; i++) Fu[i] = u[i] + r[i];
        }
        if (k == 1) {
            for (int i = 0; i < n; i++) u[i] = damping * Fu[i] + (1 - damping) * uold[i];
        } else {
            slot = slot % mm + 1;
            hist = hist + 1 < mm ? hist + 1 : mm;
            double *F = dF + (size_t)(slot - 1) * n, *Gc = dG + (size_t)(slot - 1) * n;
            for (int i = 0; i < n; i++) { F[i] = r[i] - rp[i]; Gc[i] = Fu[i] - Fp[i]; }
            double ATA[64], ATr[8];
            for (int a = 0; a < hist; a++) {
                for (int b = 0; b < hist; b++) {
                    double s = 0.0;
                    for (int i = 0; i < n; i++) s += dF[(size_t)a * n + i] * dF[(size_t)b * n + i];
                    ATA[a * hist + b] = s;
                }
                double s = 0.0;
                for (int i = 0; i < n; i++) s += dF[(size_t)a * n + i] * r[i];
                ATr[a] = s;
            }
            double dm = 0.0;
            for (int j = 0; j < hist; j++) dm += ATA[j * hist + j];
            double l2 = reg_factor * dm / hist + 1e-30;
            for (int j = 0; j < hist; j++) ATA[j * hist + j] += l2;
            lu_solve(hist, ATA, ATr);
            for (int i = 0; i < n; i++) {
                double s = Fu[i];
                for (int j = 0; j < hist; j++) s += -1.0 * dG[(size_t)j * n + i] * ATr[j];
                u[i] = damping * s + (1 - damping) * uold[i];
            }
        }
        memcpy(rp, r, sizeof(double) * n);
        memcpy(Fp, Fu, sizeof(double) * n);
    }
    free(Fu); free(r); free(rp); free(Fp); free(uold); free(dF); free(dG);
    return ret;
}

/* Anderson mixing of the outer iterates of step_defect! (outer_m > 0; the
 * library's extension, outer_m = 0 is the reference's iteration). The outer
 * step v_k -> u_k = D(v_k) (the inner solution) is mixed over the last outer_m
 * pairs: with r_j = u_j - v_j, dF_j = r_j - r_{j-1}, dU_j = u_j - u_{j-1},
 * v_{k+1} = u_k - dU gamma, gamma = (dF'dF + l2 I) \ dF' r_k, l2 as in
 * _anderson_inner! (solver.jl:514-518). The window restarts on the first outer
 * step and when the outer residual exceeds twice its best since the restart
 * (then v_{k+1} = u_k). */
typedef struct {
    int m, hist, slot, k;
    double best;
    double *vk, *u, *r, *rp, *up, *dF, *dU;
} outer_aa;

static void outer_aa_step(outer_aa *A, double *v1, int n, double nrm, double reg_factor) {
    int k = A->k + 1;
    for (int i = 0; i < n; i++) { A->u[i] = v1[i]; A->r[i] = v1[i] - A->vk[i]; }
    if (k == 1 || nrm > 2.0 * A->best) {
        A->k = 1;
        A->hist = 0;
        A->slot = 0;
        A->best = nrm;
    } else {
        A->k = k;
        if (nrm < A->best) A->best = nrm;
        A->slot = A->slot % A->m + 1;
        A->hist = A->hist + 1 < A->m ? A->hist + 1 : A->m;
        double *F = A->dF + (size_t)(A->slot - 1) * n, *U = A->dU + (size_t)(A->slot - 1) * n;
        for (int i = 0; i < n; i++) { F[i] = A->r[i] - A->rp[i]; U[i] = A->u[i] - A->up[i]; }
        int h = A->hist;
        double ATA[64], ATr[8];
        for (int a = 0; a < h; a++) {
            for (int b = 0; b < h; b++) {
                double s = 0.0;
                for (int i = 0; i < n; i++) s += A->dF[(size_t)a * n + i] * A->dF[(size_t)b * n + i];
                ATA[a * h + b] = s;
            }
            double s = 0.0;
            for (int i = 0; i < n; i++) s += A->dF[(size_t)a * n + i] * A->r[i];
            ATr[a] = s;
        }
        double dm = 0.0;
        for (int j = 0; j < h; j++) dm += ATA[j * h + j];
        double l2 = reg_factor * dm / h + 1e-30;
        for (int j = 0; j < h; j++) ATA[j * h + j] += l2;
        lu_solve(h, ATA, ATr);
        for (int i = 0; i < n; i++) {
            double s = A->u[i];
            for (int j = 0; j < h; j++) s -= A->dU[(size_t)j * n + i] * ATr[j];
            v1[i] = s;
        }
    }
    memcpy(A->rp, A->r, sizeof(double) * n);
    memcpy(A->up, A->u, sizeof(double) * n);
}

/* step_defect! (solver.jl:569-634). out4 = outer, residual, inner, initial residual */
void om_step_defect(const om_mesh *m, const om_opts *o, double eta, int max_inner,
                    int stag_window, int outer_m, int precond, double *v1, const double *v0,
                    const double *w, int N, double S0, double dt, double *out4) {
    int n = 2 * N;
    double *Geff = malloc(sizeof(double) * n), *vmid = malloc(sizeof(double) * n);
    double *dotv = malloc(sizeof(double) * n), *A = malloc(sizeof(double) * 3 * N);
    double *Gv = malloc(sizeof(double) * n), *r = malloc(sizeof(double) * n);
    double *Gk = malloc(sizeof(double) * n), *vbest = malloc(sizeof(double) * n);
    double nrm0 = 0.0, nrm_best = INFINITY, nrm_best_window = INFINITY;
    int inner = 0;
    memcpy(vbest, v1, sizeof(double) * n);
    frozen_ctx fc = {m, o->use_gonzalez, N, v0, w, Gv, A, Gk, S0, dt, NULL, NULL, precond,
                     NULL, 0.0};
    double *Hbuf = precond ? malloc(sizeof(double) * 3 * N) : NULL;
    fc.H = Hbuf;
    double *fGeff = malloc(sizeof(double) * n), *fvmid = malloc(sizeof(double) * n);
    fc.Geff = fGeff;
    fc.vmid = fvmid;
    outer_aa aa = {outer_m, 0, 0, 0, INFINITY, NULL, NULL, NULL, NULL, NULL, NULL, NULL};
    if (outer_m > 0) {
        aa.vk = malloc(sizeof(double) * n); aa.u = malloc(sizeof(double) * n);
        aa.r = malloc(sizeof(double) * n); aa.rp = malloc(sizeof(double) * n);
        aa.up = malloc(sizeof(double) * n);
        aa.dF = calloc((size_t)n * outer_m, sizeof(double));
        aa.dU = calloc((size_t)n * outer_m, sizeof(double));
    }
    for (int k = 1; k <= o->max_iter; k++) {
        landau_geff(m, o->use_gonzalez, Geff, vmid, v1, v0, w, N, S0);
        om_collision_metric(m, vmid, w, Geff, N, dotv, A, o->nthreads);
        for (int i = 0; i < n; i++) {
            Gv[i] = v0[i] + dt * dotv[i];
            r[i] = Gv[i] - v1[i];
        }
        double nrm = norm2v(r, n);
        if (k == 1) nrm0 = nrm;
        if (nrm < nrm_best) {
            nrm_best = nrm;
            memcpy(vbest, Gv, sizeof(double) * n);
        }
        if (nrm < fmax(o->tol * (norm2v(v1, n) + 1e-30), o->abs_floor)) {
            memcpy(v1, Gv, sizeof(double) * n);
            out4[0] = k; out4[1] = nrm; out4[2] = inner; out4[3] = nrm0;
            goto done;
        }
        if (k > stag_window && k % stag_window == 0) {
            if ((nrm_best_window - nrm_best) / (nrm_best_window + 1e-30) < o->stag_rel_tol) {
                memcpy(v1, vbest, sizeof(double) * n);
                out4[0] = k; out4[1] = nrm_best; out4[2] = inner; out4[3] = nrm0;
                goto done;
            }
            nrm_best_window = nrm_best;
        }
        memcpy(Gk, Geff, sizeof(double) * n);
        if (outer_m > 0) memcpy(aa.vk, v1, sizeof(double) * n);
        inner += anderson_inner(&fc, v1, fmax(eta * nrm, 0.5 * o->abs_floor), max_inner, o->m,
                                o->damping, o->reg_factor);
        if (outer_m > 0) outer_aa_step(&aa, v1, n, nrm, o->reg_factor);
    }
    memcpy(v1, vbest, sizeof(double) * n);
    out4[0] = o->max_iter; out4[1] = nrm_best; out4[2] = inner; out4[3] = nrm0;
done:
    free(Geff); free(vmid); free(dotv); free(A); free(Gv); free(r); free(Gk); free(vbest);
    free(fGeff); free(fvmid);
    free(aa.vk); free(aa.u); free(aa.r); free(aa.rp); free(aa.up); free(aa.dF); free(aa.dU);
    free(Hbuf);
}

/* ------------------------------------------------------------ Newton-Krylov */

/* Symmetric Givens reflection of newton_krylov.jl:37-58 (_sym_givens). */
static void sym_givens(double a, double b, double *c, double *s, double *rho) {
    if (b == 0.0) {
        *c = (a > 0) - (a < 0) + (a == 0.0);
        *s = 0.0;
        *rho = fabs(a);
    } else if (a == 0.0) {
        *c = 0.0;
        *s = (b > 0) - (b < 0);
        *rho = fabs(b);
    } else if (fabs(b) > fabs(a)) {
        double t = a / b;
        *s = ((b > 0) - (b < 0)) / sqrt(1.0 + t * t);
        *c = *s * t;
        *rho = b / *s;
    } else {
        double t = b / a;
        *c = ((a > 0) - (a < 0)) / sqrt(1.0 + t * t);
        *s = *c * t;
        *rho = a / *c;
    }
}

typedef struct {
    const om_mesh *m;
    const om_opts *o;
    const double *v0, *w;
    int N;
    double S0, dt;
    double *Gv;
    int n_evals;
} nk_ctx;

/* residual!(F, v) of step_newton! (solver.jl:465-472): F = v - G(v) */
static void nk_residual(nk_ctx *c, double *F, const double *x) {
    om_picard_map(c->m, c->o, c->Gv, x, c->v0, c->w, c->N, c->S0, c->dt);
    for (int i = 0; i < 2 * c->N; i++) F[i] = x[i] - c->Gv[i];
    c->n_evals++;
}

/* gmres! (newton_krylov.jl:74-130) with A u = (F(x + h u) - F(x)) / h,
 * h = fd_h / ||u|| (the jvp! of newton_krylov!, :215-222). Returns k. */
static int nk_gmres(nk_ctx *c, int n, double *xs, const double *x, const double *Fx,
                    double rtol, int itmax, int mem, double fd_h, double *V, double *R,
                    double *cs, double *sn, double *z, double *wv, double *xp, double *Fp) {
    int kmax = itmax < mem ? itmax : mem;
    for (int i = 0; i < n; i++) xs[i] = 0.0;
    double beta = norm2v(Fx, n);
    if (beta == 0.0) return 0;
    double eps = rtol * beta;
    double btol = pow(2.220446049250313e-16, 0.75);
    for (int i = 0; i <= mem; i++) z[i] = 0.0;
    z[0] = beta;
    for (int i = 0; i < n; i++) V[i] = Fx[i] / beta;
    int k = 0;
    while (k < kmax) {
        k++;
        const double *u = V + (size_t)(k - 1) * n;
        double h = fd_h / norm2v(u, n);
        for (int i = 0; i < n; i++) xp[i] = x[i] + h * u[i];
        nk_residual(c, Fp, xp);
        for (int i = 0; i < n; i++) wv[i] = (Fp[i] - Fx[i]) / h;
        for (int i = 0; i < k; i++) {     /* modified Gram-Schmidt */
            const double *vi = V + (size_t)i * n;
            double hh = 0.0;
            for (int j = 0; j < n; j++) hh += vi[j] * wv[j];
            R[(size_t)i * mem + (k - 1)] = hh;
            for (int j = 0; j < n; j++) wv[j] -= hh * vi[j];
        }
        double hnext = norm2v(wv, n);
        for (int i = 0; i < k - 1; i++) {
            double a = R[(size_t)i * mem + (k - 1)], b = R[(size_t)(i + 1) * mem + (k - 1)];
            double tmp = cs[i] * a + sn[i] * b;
            R[(size_t)(i + 1) * mem + (k - 1)] = sn[i] * a - cs[i] * b;
            R[(size_t)i * mem + (k - 1)] = tmp;
        }
        double rho;
        sym_givens(R[(size_t)(k - 1) * mem + (k - 1)], hnext, &cs[k - 1], &sn[k - 1], &rho);
        R[(size_t)(k - 1) * mem + (k - 1)] = rho;
        z[k] = sn[k - 1] * z[k - 1];
        z[k - 1] = cs[k - 1] * z[k - 1];
        double rnorm = fabs(z[k]);
        if (rnorm <= eps || hnext <= btol) break;
        if (k < kmax)
            for (int i = 0; i < n; i++) V[(size_t)k * n + i] = wv[i] / hnext;
    }
    for (int i = k - 1; i >= 0; i--) {
        double acc = z[i];
        for (int j = i + 1; j < k; j++) acc -= R[(size_t)i * mem + j] * z[j];
        z[i] = fabs(R[(size_t)i * mem + i]) <= btol ? 0.0 : acc / R[(size_t)i * mem + i];
    }
    for (int i = 0; i < k; i++)
        for (int j = 0; j < n; j++) xs[j] += z[i] * V[(size_t)i * n + j];
    return k;
}

void om_step_newton(const om_mesh *m, const om_opts *o, int krylov_max, double fd_h,
                    double eta_max, double *v1, const double *v0, const double *w, int N,
                    double S0, double dt, double *out5) {
    int n = 2 * N, mem = krylov_max;
    nk_ctx c = {m, o, v0, w, N, S0, dt, malloc(sizeof(double) * n), 0};
    double *F = malloc(sizeof(double) * n), *Ft = malloc(sizeof(double) * n);
    double *xt = malloc(sizeof(double) * n), *xp = malloc(sizeof(double) * n);
    double *Fp = malloc(sizeof(double) * n), *d = malloc(sizeof(double) * n);
    double *xb = malloc(sizeof(double) * n), *Fb = malloc(sizeof(double) * n);
    double *wv = malloc(sizeof(double) * n);
    double *V = malloc(sizeof(double) * (size_t)n * (mem + 1));
    double *R = calloc((size_t)mem * mem, sizeof(double));
    double *cs = calloc(mem, sizeof(double)), *sn = calloc(mem, sizeof(double));
    double *z = calloc(mem + 1, sizeof(double));
    /* step_newton! (solver.jl:460-486): tolerance taken once at the predictor */
    double tol = fmax(o->tol * (norm2v(v1, n) + 1e-30), o->abs_floor);
    double *x = v1;
    nk_residual(&c, F, x);
    double rnorm = norm2v(F, n), rnorm0 = rnorm, rbest = rnorm, eta = eta_max, rprev = rnorm;
    memcpy(xb, x, sizeof(double) * n);
    memcpy(Fb, F, sizeof(double) * n);
    int n_newton = 0, status = 2; /* 0 converged, 1 stalled, 2 budget */
    const double gamma = 0.9, armijo = 1e-4;
    const int max_backtrack = 8;
    for (;;) {
        if (rnorm < tol) { status = 0; break; }
        int budget = o->max_iter - c.n_evals;
        if (budget < 2) break;
        if (n_newton > 0) {
            double ew = gamma * (rnorm / rprev) * (rnorm / rprev);
            double safe = gamma * eta * eta;
            if (safe > 0.1) ew = fmax(ew, safe);
            eta = fmin(fmax(ew, 0.5 * tol / rnorm), eta_max);
        }
        int itmax = krylov_max < budget - 1 ? krylov_max : budget - 1;
        nk_gmres(&c, n, d, x, F, eta, itmax, mem, fd_h, V, R, cs, sn, z, wv, xp, Fp);
        n_newton++;
        double lam = 1.0, rt = INFINITY;
        int accepted = 0;
        for (int bt = 0; bt <= max_backtrack; bt++) {
            for (int i = 0; i < n; i++) xt[i] = x[i] - lam * d[i];
            nk_residual(&c, Ft, xt);
            rt = norm2v(Ft, n);
            if (rt <= (1.0 - armijo * lam * (1.0 - eta)) * rnorm) { accepted = 1; break; }
            if (c.n_evals >= o->max_iter) break;
            lam /= 2.0;
        }
        if (rt < rbest) {
            rbest = rt;
            memcpy(xb, xt, sizeof(double) * n);
            memcpy(Fb, Ft, sizeof(double) * n);
        }
        if (!accepted) { status = c.n_evals >= o->max_iter ? 2 : 1; break; }
        memcpy(x, xt, sizeof(double) * n);
        memcpy(F, Ft, sizeof(double) * n);
        rprev = rnorm;
        rnorm = rt;
    }
    if (status != 0 && rbest < rnorm) {
        memcpy(x, xb, sizeof(double) * n);
        memcpy(F, Fb, sizeof(double) * n);
        rnorm = rbest;
    }
    if (o->exit_picard_step)                  /* v1 -= F: the Picard update G(v) */
        for (int i = 0; i < n; i++) x[i] -= F[i];
    out5[0] = c.n_evals; out5[1] = rnorm; out5[2] = n_newton; out5[3] = rnorm0; out5[4] = status;
    free(c.Gv); free(F); free(Ft); free(xt); free(xp); free(Fp); free(d); free(xb); free(Fb);
    free(wv); free(V); free(R); free(cs); free(sn); free(z);
}
