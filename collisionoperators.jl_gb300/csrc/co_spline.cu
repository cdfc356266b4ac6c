// co_spline.cu -- the P_DEG=2 particle <-> spline stage on the device.
//
// Replaces projection_gpu.jl (atomic scatter, gathers) and the CPU parts of
// the chain (mass solve, quadrature) with deterministic kernels:
//   1. locate:   cell id and reference coordinates per marker, per-chunk cell
//                histograms (integer, so order-independent);
//   2. sort:     stable counting sort of the in-domain markers by cell
//                (chunk-major offsets + warp-sequential ranks), which also
//                compacts away out-of-domain markers;
//   3. scatter:  b = sum_a w_a phi_k(v_a) as a segmented sum per (cell, local
//                basis) in marker order, then a fixed 3x3-cell gather per dof;
//   4. solve:    M = M1 (x) M2 (tensor-product mass matrix), so M^{-1} b is two
//                small dense products with the 1D inverses;
//   5. quadrature for r (functions.jl:158-179) and S (functions.jl:137-155),
//                one block per element, fixed-order reductions;
//   6. gathers:  grad L (functions.jl:182-202) and the clamped log-gradient
//                (functions.jl:37-64) per marker.
// Everything is FP64 and bitwise reproducible run to run.
#include "co_internal.cuh"
#include "co_reduce.cuh"

// ---------------------------------------------------------------- basis

// _bernstein_eval! for p = 2 (MantisWrappers.jl:201-216), same expressions.
__device__ __forceinline__ void bern2(double xi, double *B, double *dB) {
    double om = 1.0 - xi;
    B[0] = om * om;
    B[1] = 2.0 * xi * om;
    B[2] = xi * xi;
    if (dB) {
        dB[0] = 2.0 * (0.0 - om);
        dB[1] = 2.0 * (om - xi);
        dB[2] = 2.0 * xi;
    }
}

// phi[j] = sum_k C[k][j] B[k]  (mul!(phi, transpose(C), B))
__device__ __forceinline__ void extract3(const double *__restrict__ c, const double *B,
                                         double *phi) {
#pragma unroll
    for (int j = 0; j < 3; j++) phi[j] = c[0 * 3 + j] * B[0] + c[1 * 3 + j] * B[1] + c[2 * 3 + j] * B[2];
}

// searchsortedlast - 1 on bp[0..n] for bp[0] < x < bp[n] (_cell_search,
// projection_gpu.jl:20-32)
__device__ __forceinline__ int cell_search(const double *__restrict__ bp, int n, double x) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (bp[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

// p_j(x) (and dp_j/dx) of the three cell-local basis functions from the cell's
// monomial table P[j] = (alpha, beta, gamma, 2 gamma): the extraction product
// C^T B(x) of extract3/bern2 in 2-3 FMAs per function (equal to it within a few
// ulps; FP64 issue is the bound of the marker kernels on this GPU)
__device__ __forceinline__ void basis_mono(const double *__restrict__ P, double x, double *p,
                                           double *dp) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const double *q = P + 4 * j;
        p[j] = fma(fma(q[2], x, q[1]), x, q[0]);
        if (dp) dp[j] = fma(q[3], x, q[1]);
    }
}

// ---------------------------------------------------------------- kernels

// One marker set of a locate launch. With v0 set, x is v_in and the located
// points are v_mid = 0.5 (v0 + v_in), written to vmid beside dv = v_in - v0
// (solver.jl:181-182); otherwise x itself is located.
struct co_locate_job {
    const double *x, *v0;
    double *vmid, *dv;
    int *cell;
    double *xi;
    int *hist;
};

// locate_particle (MantisWrappers.jl:168-179) + per-chunk cell histogram, for
// one or two marker sets (blockIdx.y). The reference coordinate is (v - bp[i])
// times the cell's reciprocal width (within one ulp of the quotient; an FP64
// division costs ~10 FP64 issue slots on this GPU).
__global__ void __launch_bounds__(CO_CHUNK)
k_locate_hist(co_locate_job j0, co_locate_job j1, int N, const double *__restrict__ bp1,
              int n1, const double *__restrict__ bp2, int n2, const double *__restrict__ ih1,
              const double *__restrict__ ih2, int n_el) {
    extern __shared__ int hs[];
    const co_locate_job J = blockIdx.y ? j1 : j0;
    for (int i = threadIdx.x; i < n_el; i += blockDim.x) hs[i] = 0;
    __syncthreads();
    int a = blockIdx.x * CO_CHUNK + threadIdx.x;
    if (a < N) {
        double v1 = J.x[a], v2 = J.x[N + a];
        if (J.v0) {
            const double b1 = J.v0[a], b2 = J.v0[N + a];
            const double m1 = 0.5 * (b1 + v1), m2 = 0.5 * (b2 + v2);
            J.vmid[a] = m1;
            J.vmid[N + a] = m2;
            J.dv[a] = v1 - b1;
            J.dv[N + a] = v2 - b2;
            v1 = m1;
            v2 = m2;
        }
        int c = -1;
        double x1 = 0.0, x2 = 0.0;
        if (!(v1 <= bp1[0] || v1 >= bp1[n1] || v2 <= bp2[0] || v2 >= bp2[n2])) {
            int i = cell_search(bp1, n1, v1);
            int j = cell_search(bp2, n2, v2);
            x1 = (v1 - bp1[i]) * ih1[i];
            x2 = (v2 - bp2[j]) * ih2[j];
            c = i + j * n1;
            atomicAdd(&hs[c], 1);
        }
        J.cell[a] = c;
        J.xi[a] = x1;
        J.xi[N + a] = x2;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_el; i += blockDim.x)
        J.hist[(size_t)blockIdx.x * n_el + i] = hs[i];
}

// Per cell: exclusive offsets of each chunk within the cell, and the count;
// then the last block of each marker set to finish (arrival counter
// tickets[set]) forms the exclusive scan of the counts, cstart[0..n_el] (the
// cell starts of the sorted order). Integer sums: exact, whatever the order.
__global__ void __launch_bounds__(256)
k_cellcount(co_sortset s0, co_sortset s1, int nchunk, int n_el, unsigned *tickets) {
    const co_sortset S = blockIdx.y ? s1 : s0;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n_el) {
        const int *__restrict__ hist = S.hist;
        int *__restrict__ hoff = S.hoff;
        int run = 0, k = 0;
        // eight chunk counts loaded ahead of the running sum: one L2 round trip
        // per eight chunks instead of per chunk
        for (; k + 8 <= nchunk; k += 8) {
            int h[8];
#pragma unroll
            for (int u = 0; u < 8; u++) h[u] = hist[(size_t)(k + u) * n_el + c];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                hoff[(size_t)(k + u) * n_el + c] = run;
                run += h[u];
            }
        }
        for (; k < nchunk; k++) {
            int h = hist[(size_t)k * n_el + c];
            hoff[(size_t)k * n_el + c] = run;
            run += h;
        }
        S.count[c] = run;
    }
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&tickets[blockIdx.y], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (threadIdx.x == 0) tickets[blockIdx.y] = 0u;
    // exclusive scan of count[0..n_el) by this block; the counts of the other
    // blocks are read through L2 (__ldcg), past this SM's L1
    __shared__ int sh[256];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (n_el + nt - 1) / nt;
    const int b0 = t * per, b1 = min(n_el, b0 + per);
    int sum = 0;
    for (int i = b0; i < b1; i++) sum += __ldcg(&S.count[i]);
    sh[t] = sum;
    __syncthreads();
    for (int o = 1; o < nt; o <<= 1) {   // Hillis-Steele inclusive scan of the thread sums
        const int v = t >= o ? sh[t - o] : 0;
        __syncthreads();
        sh[t] += v;
        __syncthreads();
    }
    int run = t > 0 ? sh[t - 1] : 0;
    for (int i = b0; i < b1; i++) {
        S.cstart[i] = run;
        run += __ldcg(&S.count[i]);
    }
    if (t == nt - 1) S.cstart[n_el] = sh[nt - 1];
}

// Stable placement: rank of each marker among the markers of its cell that
// precede it in its chunk, warps taking turns in index order. The sorted
// weights and the six cell-local basis values per marker are written for the
// scatter.
__global__ void __launch_bounds__(CO_CHUNK)
k_perm(co_sortset s0, co_sortset s1, int N, int n_el, int n1, const double *__restrict__ w,
       const double *__restrict__ P1, const double *__restrict__ P2) {
    extern __shared__ int run[];
    const co_sortset S = blockIdx.y ? s1 : s0;
    for (int i = threadIdx.x; i < n_el; i += blockDim.x) run[i] = 0;
    __syncthreads();
    int a = blockIdx.x * CO_CHUNK + threadIdx.x;
    int c = a < N ? S.cell[a] : -2;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned peers = __match_any_sync(0xffffffffu, c);
    int rank = __popc(peers & ((1u << lane) - 1u));
    int leader = __ffs(peers) - 1;
    int base = 0;
    for (int wv = 0; wv < (CO_CHUNK >> 5); wv++) {
        if (warp == wv) {
            int b = 0;
            if (c >= 0 && lane == leader) {
                b = run[c];
                run[c] = b + __popc(peers);
            }
            base = __shfl_sync(0xffffffffu, b, leader);
        }
        __syncthreads();
    }
    if (a >= N) return;
    if (c < 0) {
        S.inv[a] = -1;
        return;
    }
    int pos = S.cstart[c] + S.hoff[(size_t)blockIdx.x * n_el + c] + base + rank;
    S.perm[pos] = a;
    S.inv[a] = pos;
    S.scell[pos] = c;
    S.sw[pos] = w[a];
    int i = c % n1, j = c / n1;
    double *o = S.sphi + (size_t)pos * 6;
    basis_mono(P1 + 12 * i, S.xi[a], o, nullptr);
    basis_mono(P2 + 12 * j, S.xi[N + a], o + 3, nullptr);
}

// Segmented sum per (cell, local basis j1 + 3 j2): one block of 4 warps per
// cell, thread t takes the cell's markers t, t + 128, ... in sorted (index)
// order; each warp combines its lanes by a fixed shuffle tree and warp 0 adds
// the four warp sums in warp order. Cells are very uneven (the central cell of
// a Gaussian holds ~45x the mean), so four warps share the long segments;
// empty cells leave at once and warps past the segment's end skip the tree.
// Deterministic run to run.
__global__ void __launch_bounds__(128)
k_cellsum(co_sortset s0, co_sortset s1, int n_el) {
    __shared__ double part[4][9];
    const co_sortset S = blockIdx.y ? s1 : s0;
    const int c = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (c >= n_el) return;
    const double *__restrict__ sw = S.sw;
    const double *__restrict__ sphi = S.sphi;
    double *__restrict__ bS = S.bS;
    const int p0 = S.cstart[c], p1 = S.cstart[c + 1];
    if (p0 == p1) {
        if (threadIdx.x < 9) bS[(size_t)c * 9 + threadIdx.x] = 0.0;
        return;
    }
    double acc[9];
#pragma unroll
    for (int j = 0; j < 9; j++) acc[j] = 0.0;
    const bool active = p0 + warp * 32 < p1;
    if (active) {
        for (int p = p0 + threadIdx.x; p < p1; p += 128) {
            const double *ph = sphi + (size_t)p * 6;
            const double w = sw[p];
            // w phi1 once, then nine FMAs: GB300 issues FP64 at 1/64 of the
            // FP32 rate, and the densest cell is the critical path
            const double a0 = w * ph[0], a1 = w * ph[1], a2 = w * ph[2];
            const double b0 = ph[3], b1 = ph[4], b2 = ph[5];
            acc[0] = fma(a0, b0, acc[0]);
            acc[1] = fma(a1, b0, acc[1]);
            acc[2] = fma(a2, b0, acc[2]);
            acc[3] = fma(a0, b1, acc[3]);
            acc[4] = fma(a1, b1, acc[4]);
            acc[5] = fma(a2, b1, acc[5]);
            acc[6] = fma(a0, b2, acc[6]);
            acc[7] = fma(a1, b2, acc[7]);
            acc[8] = fma(a2, b2, acc[8]);
        }
        // the nine lane sums by recursive halving (16 FP64 adds per lane instead
        // of 45 for nine shuffle trees: at GB300's FP64 rate the trees cost more
        // than the scatter itself)
        double v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = j < 9 ? acc[j] : 0.0;
        const double sj = co_warp_sum16(v, lane);   // value (lane >> 1)
        if ((lane & 1) == 0 && (lane >> 1) < 9) part[warp][lane >> 1] = sj;
    } else if (lane < 9) {
        part[warp][lane] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        const int j = threadIdx.x;
        bS[(size_t)c * 9 + j] = ((part[0][j] + part[1][j]) + part[2][j]) + part[3][j];
    }
}

// dof k = (k1, k2) gathers the <= 9 cell-local entries that touch it; one or
// two (src, out) pairs (blockIdx.y)
__global__ void k_dofgather(const double *__restrict__ src0, double *__restrict__ out0,
                            const double *__restrict__ src1, double *__restrict__ out1, int n1,
                            int n2, int nd1, int nd2) {
    const double *__restrict__ src = blockIdx.y ? src1 : src0;
    double *__restrict__ out = blockIdx.y ? out1 : out0;
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nd1 * nd2) return;
    int k1 = k % nd1, k2 = k / nd1;
    double acc = 0.0;
    for (int b = 0; b < 3; b++) {
        int jj = k2 - b;
        if (jj < 0 || jj >= n2) continue;
        for (int a = 0; a < 3; a++) {
            int i = k1 - a;
            if (i < 0 || i >= n1) continue;
            acc += src[(size_t)(i + jj * n1) * 9 + a + 3 * b];
        }
    }
    out[k] = acc;
}

// The mass solve f = M1^{-1} B M2^{-1} (M = M2 (x) M1, first index fastest) as
// two dense products with the 1D inverses. One warp per eight consecutive
// outputs i1 .. i1 + 7 of one column i2: lane l adds the terms k = l, l + 32,
// ... of all eight (the eight inverse-matrix entries of a k are contiguous, the
// right-hand-side entry is shared), then co_warp_sum<8> adds the lanes (9 FP64
// adds per lane for the eight outputs instead of 5 per output). One or two
// right-hand sides (blockIdx.y). Fixed order, deterministic.
#define MASS_OUT 8
// y[i1, i2] = sum_k M1^{-1}[i1, k] b[k, i2]
__global__ void __launch_bounds__(256)
k_mass1(const double *__restrict__ Minv1, const double *__restrict__ b0,
        double *__restrict__ y0, const double *__restrict__ b1, double *__restrict__ y1,
        int nd1, int nd2) {
    const double *__restrict__ b = blockIdx.y ? b1 : b0;
    double *__restrict__ y = blockIdx.y ? y1 : y0;
    const int ng1 = (nd1 + MASS_OUT - 1) / MASS_OUT;
    const int wi = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (wi >= ng1 * nd2) return;
    const int i1b = (wi % ng1) * MASS_OUT, i2 = wi / ng1;
    const double *col = b + (size_t)i2 * nd1;
    double s[MASS_OUT];
#pragma unroll
    for (int o = 0; o < MASS_OUT; o++) s[o] = 0.0;
    // Minv1 is exactly symmetric (symmetrised at set-up): row i1 read as column i1
    for (int k = lane; k < nd1; k += 32) {
        const double bk = col[k];
        const double *mrow = Minv1 + (size_t)k * nd1;
#pragma unroll
        for (int o = 0; o < MASS_OUT; o++)
            if (i1b + o < nd1) s[o] = fma(mrow[i1b + o], bk, s[o]);
    }
    const double r = co_warp_sum<MASS_OUT>(s, lane);   // output lane >> 2
    const int o = lane >> 2;
    if ((lane & 3) == 0 && i1b + o < nd1) y[(size_t)i2 * nd1 + i1b + o] = r;
}

// The dof gather and the first mass product in one launch: one block per
// column i2 (and marker set, blockIdx.y) gathers b[:, i2] from the cell-local
// entries src[e][9] into shared memory (k_dofgather's sums), then its warps form
// the outputs of k_mass1 for that column, eight per warp, with k_mass1's
// arithmetic. Dynamic shared memory: nd1 doubles.
__global__ void __launch_bounds__(256)
k_gather_mass1(const double *__restrict__ src0, double *__restrict__ y0,
               const double *__restrict__ src1, double *__restrict__ y1,
               const double *__restrict__ Minv1, int n1, int n2, int nd1, int nd2) {
    extern __shared__ double col[];
    const double *__restrict__ src = blockIdx.y ? src1 : src0;
    double *__restrict__ y = blockIdx.y ? y1 : y0;
    const int i2 = blockIdx.x;
    for (int k1 = threadIdx.x; k1 < nd1; k1 += blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < 3; b++) {
            int jj = i2 - b;
            if (jj < 0 || jj >= n2) continue;
            for (int a = 0; a < 3; a++) {
                int i = k1 - a;
                if (i < 0 || i >= n1) continue;
                acc += src[(size_t)(i + jj * n1) * 9 + a + 3 * b];
            }
        }
        col[k1] = acc;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int ng1 = (nd1 + MASS_OUT - 1) / MASS_OUT;
    for (int g = warp; g < ng1; g += nw) {
        const int i1b = g * MASS_OUT;
        double s[MASS_OUT];
#pragma unroll
        for (int o = 0; o < MASS_OUT; o++) s[o] = 0.0;
        for (int k = lane; k < nd1; k += 32) {
            const double bk = col[k];
            const double *mrow = Minv1 + (size_t)k * nd1;
#pragma unroll
            for (int o = 0; o < MASS_OUT; o++)
                if (i1b + o < nd1) s[o] = fma(mrow[i1b + o], bk, s[o]);
        }
        const double r = co_warp_sum<MASS_OUT>(s, lane);   // output lane >> 2
        const int o = lane >> 2;
        if ((lane & 3) == 0 && i1b + o < nd1) y[(size_t)i2 * nd1 + i1b + o] = r;
    }
}

// out[i1, i2] = sum_k y[i1, k] M2^{-1}[k, i2]
__global__ void __launch_bounds__(256)
k_mass2(const double *__restrict__ Minv2, const double *__restrict__ y0,
        double *__restrict__ out0, const double *__restrict__ y1, double *__restrict__ out1,
        int nd1, int nd2) {
    const double *__restrict__ y = blockIdx.y ? y1 : y0;
    double *__restrict__ out = blockIdx.y ? out1 : out0;
    const int ng1 = (nd1 + MASS_OUT - 1) / MASS_OUT;
    const int wi = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (wi >= ng1 * nd2) return;
    const int i1b = (wi % ng1) * MASS_OUT, i2 = wi / ng1;
    double s[MASS_OUT];
#pragma unroll
    for (int o = 0; o < MASS_OUT; o++) s[o] = 0.0;
    for (int k = lane; k < nd2; k += 32) {
        const double mk = Minv2[(size_t)k * nd2 + i2];
        const double *yrow = y + (size_t)k * nd1;
#pragma unroll
        for (int o = 0; o < MASS_OUT; o++)
            if (i1b + o < nd1) s[o] = fma(yrow[i1b + o], mk, s[o]);
    }
    const double r = co_warp_sum<MASS_OUT>(s, lane);   // output lane >> 2
    const int o = lane >> 2;
    if ((lane & 3) == 0 && i1b + o < nd1) out[(size_t)i2 * nd1 + i1b + o] = r;
}

// Element quadrature for r-local (mode 0, functions.jl:158-179) or the entropy
// partial (mode 1, functions.jl:137-155). One thread per (element, Gauss row
// q1): nq threads per element and 128 / nq elements per block, so the lanes
// stay busy for any nq. GB300 issues FP64 at 1/64 of the FP32 rate and these
// kernels are FP64-issue bound, so the tensor-product form is used throughout:
//   g_b(q1)      = sum_a c_ab p1_a(q1)                 (once per row)
//   f(q1, q2)    = sum_b g_b(q1) p2_b(q2)
//   H_b(q1)      = sum_q2 h(q1, q2) p2_b(q2),  h = integrand * w_q * |e|
//   r_ab         = sum_q1 p1_a(q1) H_b(q1)             (rows added in order)
// about 400 FP64 operations and nq^2 logarithms per element instead of ~30 per
// Gauss point plus the logarithm. Fixed summation order: deterministic. Two jobs
// may share a launch (blockIdx.y selects), e.g. r at v_mid and S at v_in.
struct co_elem_job {
    const double *fc;   // spline coefficients (n_dofs)
    int mode;           // 0: r-local -> out[e][9]; 1: entropy partial -> out[e]
    double *out;
};

#define ELEM_THREADS 128
__global__ void __launch_bounds__(ELEM_THREADS)
k_elem(co_elem_job j0, co_elem_job j1, int n1, int n2, int nd1, int nq,
       const double *__restrict__ Tq1, const double *__restrict__ Tq2,
       const double *__restrict__ qw, const double *__restrict__ bp1,
       const double *__restrict__ bp2, int logsq) {
    __shared__ double part[ELEM_THREADS * 9];
    const co_elem_job jb = blockIdx.y ? j1 : j0;
    const int mode = jb.mode;
    const int epb = ELEM_THREADS / nq;
    const int t = threadIdx.x, el = t / nq, q1 = t - el * nq;
    const int e = blockIdx.x * epb + el;
    const int n_el = n1 * n2;
    if (el < epb && e < n_el) {
        const int i = e % n1, j = e / n1;
        const double jac = (bp1[i + 1] - bp1[i]) * (bp2[j + 1] - bp2[j]);
        const double *fc = jb.fc;
        double p1[3], g[3];
#pragma unroll
        for (int a = 0; a < 3; a++) p1[a] = Tq1[((size_t)i * 3 + a) * nq + q1];
#pragma unroll
        for (int bb = 0; bb < 3; bb++) {
            const double *cr = fc + i + (j + bb) * nd1;
            double v = cr[0] * p1[0];
            v = fma(cr[1], p1[1], v);
            g[bb] = fma(cr[2], p1[2], v);
        }
        const double wq1 = qw[q1];
        double H0 = 0.0, H1 = 0.0, H2 = 0.0, sv = 0.0;
        const double *T2 = Tq2 + (size_t)j * 3 * nq;
        for (int q2 = 0; q2 < nq; q2++) {
            const double p20 = T2[q2], p21 = T2[nq + q2], p22 = T2[2 * nq + q2];
            double f = g[0] * p20;
            f = fma(g[1], p21, f);
            f = fma(g[2], p22, f);
            const double wj = wq1 * qw[q2] * jac;
            if (mode == 0) {
                double integrand;
                if (logsq)
                    integrand = f * f > 1e-60 ? (1 + 0.5 * log(f * f)) : 0.0;
                else
                    integrand = f > 1e-30 ? (1 + log(f)) : 0.0;
                const double h = integrand * wj;
                H0 = fma(h, p20, H0);
                H1 = fma(h, p21, H1);
                H2 = fma(h, p22, H2);
            } else if (logsq) {
                if (f * f > 1e-60) sv += -(f * 0.5 * log(f * f) * wj);
            } else if (f > 1e-30) {
                sv += -(f * log(f) * wj);
            }
        }
        double *o = part + (size_t)t * 9;
        if (mode == 0) {
#pragma unroll
            for (int a = 0; a < 3; a++) {
                o[a] = p1[a] * H0;
                o[3 + a] = p1[a] * H1;
                o[6 + a] = p1[a] * H2;
            }
        } else {
            o[0] = sv;
        }
    }
    __syncthreads();
    const int ncomp = mode == 0 ? 9 : 1;
    for (int k = t; k < epb * ncomp; k += blockDim.x) {
        const int el2 = k / ncomp, comp = k - el2 * ncomp;
        const int e2 = blockIdx.x * epb + el2;
        if (e2 >= n_el) continue;
        const double *src = part + (size_t)el2 * nq * 9 + comp;
        double s = 0.0;
        for (int r = 0; r < nq; r++) s += src[r * 9];
        jb.out[(size_t)e2 * ncomp + comp] = s;
    }
}

// Post-step diagnostics per element on the N_QUAD Gauss grid (main.jl:298-307):
// D[e] = {entropy partial (compute_entropy, functions.jl:137-155), negative part
// of f_s (compute_negative_part_l1, :300-313), (f_s - f_p)^2 with f_p the
// element's marker mass over its area (compute_fs_minus_fp_l2, :315-347)}. The
// element's marker mass is the sum of its nine cell-sum entries bS[e][k] =
// sum_{a in e} w_a phi_k(v_a): the nine local basis functions sum to 1 there.
__global__ void __launch_bounds__(64)
k_diag_elem(const double *__restrict__ fc, int n1, int nd1, int nq,
            const double *__restrict__ Tq1, const double *__restrict__ Tq2,
            const double *__restrict__ qw, const double *__restrict__ bp1,
            const double *__restrict__ bp2, int logsq, const double *__restrict__ bS,
            double *__restrict__ D) {
    __shared__ double contrib[64 * 3];
    __shared__ double cs[9];
    __shared__ double fp_sh;
    int e = blockIdx.x;
    int i = e % n1, j = e / n1;
    int t = threadIdx.x;
    double jac = (bp1[i + 1] - bp1[i]) * (bp2[j + 1] - bp2[j]);
    if (t < 9) cs[t] = fc[(i + t % 3) + (j + t / 3) * nd1];
    if (t == 0) {
        double m = 0.0;
        for (int k = 0; k < 9; k++) m += bS[(size_t)e * 9 + k];
        fp_sh = m / jac;
    }
    __syncthreads();
    int nqq = nq * nq;
    if (t < nqq) {
        int q1 = t % nq, q2 = t / nq;
        double p1[3], p2[3];
        for (int a = 0; a < 3; a++) {
            p1[a] = Tq1[((size_t)i * 3 + a) * nq + q1];
            p2[a] = Tq2[((size_t)j * 3 + a) * nq + q2];
        }
        double f = 0.0;
        for (int b = 0; b < 3; b++)
            for (int a = 0; a < 3; a++) f += cs[a + 3 * b] * (p1[a] * p2[b]);
        double wq = qw[q1] * qw[q2];
        double s = 0.0;
        if (logsq) {
            if (f * f > 1e-60) s = -(f * 0.5 * log(f * f) * wq * jac);
        } else if (f > 1e-30) {
            s = -(f * log(f) * wq * jac);
        }
        double d = f - fp_sh;
        contrib[t * 3 + 0] = s;
        contrib[t * 3 + 1] = f < 0.0 ? (-f) * wq * jac : 0.0;
        contrib[t * 3 + 2] = d * d * wq * jac;
    }
    __syncthreads();
    if (t < 3) {
        double s = 0.0;
        for (int q = 0; q < nqq; q++) s += contrib[q * 3 + t];
        D[(size_t)e * 3 + t] = s;
    }
}

// block partials of sum w v1, sum w v2, sum w |v|^2 over all markers
// (compute_momentum / compute_energy, functions.jl:349-358)
__global__ void __launch_bounds__(CO_RED_THREADS)
k_marker_moments(const double *__restrict__ v, const double *__restrict__ w, int N,
                 double *__restrict__ red) {
    __shared__ double sh[32];
    double p1 = 0.0, p2 = 0.0, e = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        double x1 = v[a], x2 = v[N + a], wa = w[a];
        p1 += wa * x1;
        p2 += wa * x2;
        e += wa * (x1 * x1 + x2 * x2);
    }
    double s1 = co_block_sum(p1, sh);
    double s2 = co_block_sum(p2, sh);
    double s3 = co_block_sum(e, sh);
    if (threadIdx.x == 0) {
        red[blockIdx.x * 3 + 0] = s1;
        red[blockIdx.x * 3 + 1] = s2;
        red[blockIdx.x * 3 + 2] = s3;
    }
}

// out = {S, E, P1, P2, ||f_s - f_p||_2, negative part}, fixed-order sums
__global__ void __launch_bounds__(256)
k_diag_final(const double *__restrict__ D, int n_el, const double *__restrict__ red, int nred,
             double *__restrict__ out) {
    __shared__ double sh[32];
    double S = co_sum_partials(D, n_el, 3, 0, sh);
    double neg = co_sum_partials(D, n_el, 3, 1, sh);
    double sq = co_sum_partials(D, n_el, 3, 2, sh);
    double p1 = co_sum_partials(red, nred, 3, 0, sh);
    double p2 = co_sum_partials(red, nred, 3, 1, sh);
    double e = co_sum_partials(red, nred, 3, 2, sh);
    if (threadIdx.x == 0) {
        out[0] = S;
        out[1] = 0.5 * e;
        out[2] = p1;
        out[3] = p2;
        out[4] = sqrt(sq);
        out[5] = neg;
    }
}

// S = sum_e Ep[e] in a fixed order (one block)
__global__ void __launch_bounds__(256)
k_sum_to(const double *__restrict__ Ep, int n, double *__restrict__ out) {
    __shared__ double sh[32];
    double s = co_sum_partials(Ep, n, 1, 0, sh);
    if (threadIdx.x == 0) *out = s;
}

// compute_G! (functions.jl:182-202) at markers x, optionally with dS = -w G
// (solver.jl:69-72) and the Gonzalez partials dv.dS, |dv|^2 (solver.jl:98-103).
__global__ void __launch_bounds__(CO_RED_THREADS)
k_grad_L(const double *__restrict__ x, int N, const int *__restrict__ cell,
         const double *__restrict__ xi, const double *__restrict__ Lc, int n1, int nd1,
         const double *__restrict__ IH1, const double *__restrict__ IH2,
         const double *__restrict__ P1, const double *__restrict__ P2,
         double *__restrict__ G, const double *__restrict__ w, double *__restrict__ dS,
         const double *__restrict__ dv, double *__restrict__ red, co_lambda_job lam) {
    __shared__ double sh[32];
    double pdot = 0.0, pn2 = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        int c = cell[a];
        double acc1 = 0.0, acc2 = 0.0;
        if (c >= 0) {
            int i = c % n1, j = c / n1;
            double p1[3], dp1[3], p2[3], dp2[3];
            basis_mono(P1 + 12 * i, xi[a], p1, dp1);
            basis_mono(P2 + 12 * j, xi[N + a], p2, dp2);
            // tensor-product form: dL/dx1 = (1/h1) sum_b p2_b sum_q L_qb dp1_q and
            // dL/dx2 = (1/h2) sum_b dp2_b sum_q L_qb p1_q (26 FP64 operations
            // instead of 54 for the nine terms one by one)
            double t1 = 0.0, t2 = 0.0;
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const double *Lr = Lc + i + (j + b) * nd1;
                double s1 = Lr[0] * dp1[0], s2 = Lr[0] * p1[0];
                s1 = fma(Lr[1], dp1[1], s1);
                s2 = fma(Lr[1], p1[1], s2);
                s1 = fma(Lr[2], dp1[2], s1);
                s2 = fma(Lr[2], p1[2], s2);
                t1 = fma(s1, p2[b], t1);
                t2 = fma(s2, dp2[b], t2);
            }
            acc1 = t1 * IH1[i];
            acc2 = t2 * IH2[j];
        }
        G[a] = acc1;
        G[N + a] = acc2;
        if (dS) {
            double s1 = -w[a] * acc1, s2 = -w[a] * acc2;
            dS[a] = s1;
            dS[N + a] = s2;
            if (red) {
                double d1 = dv[a], d2 = dv[N + a];
                pdot += d1 * s1 + d2 * s2;
                pn2 += d1 * d1 + d2 * d2;
            }
        }
    }
    if (red) {
        double s = co_block_sum(pdot, sh);
        double n = co_block_sum(pn2, sh);
        if (threadIdx.x == 0) {
            red[blockIdx.x * 2 + 0] = s;
            red[blockIdx.x * 2 + 1] = n;
        }
        if (lam.st) {
            // the last block to finish forms the Gonzalez lambda (landau_geff!,
            // solver.jl:98-103) from all blocks' partials: S1 = S(v_in) from the
            // element entropy partials (if given), then lambda = (S1 - S0 - dv.dS)
            // / |dv|^2, the sums in the order of one 256-thread block
            __shared__ int last;
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) last = atomicAdd(lam.ticket, 1u) == gridDim.x - 1;
            __syncthreads();
            if (!last) return;
            __threadfence();
            if (threadIdx.x == 0) *lam.ticket = 0u;
            const int nb = gridDim.x;
            double S1 = lam.Ep ? co_block_sum(co_strided_sum(lam.Ep, threadIdx.x, lam.n_el,
                                                             blockDim.x, 1, 0, 0.0), sh)
                               : 0.0;
            double dot = co_block_sum(co_strided_sum_cg(red, threadIdx.x, nb, blockDim.x, 2, 0,
                                                        0.0), sh);
            double nn = co_block_sum(co_strided_sum_cg(red, threadIdx.x, nb, blockDim.x, 2, 1,
                                                       0.0), sh);
            if (threadIdx.x == 0) {
                if (lam.Ep) lam.st->S1 = S1;
                else S1 = lam.st->S1;
                double l = 0.0;
                if (lam.gonzalez) l = nn > 1e-30 ? (S1 - lam.S0 - dot) / nn : 0.0;
                lam.st->lambda = l;
            }
        }
    }
}

// eval_loggrad_at_particles! (functions.jl:37-64) with the LB Gonzalez partials
// -sum w dv.g and |dv|^2 (solver.jl:198-203).
__global__ void __launch_bounds__(CO_RED_THREADS)
k_loggrad(const double *__restrict__ x, int N, const int *__restrict__ cell,
          const double *__restrict__ xi, const double *__restrict__ fc, int n1, int nd1,
          const double *__restrict__ bp1, const double *__restrict__ bp2,
          const double *__restrict__ C1, const double *__restrict__ C2,
          double *__restrict__ g, const double *__restrict__ w,
          const double *__restrict__ dv, double *__restrict__ red) {
    __shared__ double sh[32];
    double pdot = 0.0, pn2 = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        int c = cell[a];
        double g1 = 0.0, g2 = 0.0;
        if (c >= 0) {
            int i = c % n1, j = c / n1;
            double h1 = bp1[i + 1] - bp1[i], h2 = bp2[j + 1] - bp2[j];
            double ih1 = 1.0 / h1, ih2 = 1.0 / h2;
            double B1[3], dB1[3], B2[3], dB2[3], p1[3], dp1[3], p2[3], dp2[3];
            bern2(xi[a], B1, dB1);
            bern2(xi[N + a], B2, dB2);
            extract3(C1 + 9 * i, B1, p1);
            extract3(C1 + 9 * i, dB1, dp1);
            extract3(C2 + 9 * j, B2, p2);
            extract3(C2 + 9 * j, dB2, dp2);
            double f = 0.0, d1 = 0.0, d2 = 0.0;
            for (int b = 0; b < 3; b++)
                for (int q = 0; q < 3; q++) {
                    double cv = fc[(i + q) + (j + b) * nd1];
                    f += cv * (p1[q] * p2[b]);
                    d1 += cv * (dp1[q] * p2[b]) * ih1;
                    d2 += cv * (p1[q] * dp2[b]) * ih2;
                }
            double invf = 1.0 / fmax(fabs(f), CO_FS_FLOOR);
            g1 = fmin(fmax(d1 * invf, -CO_G_MAX), CO_G_MAX);
            g2 = fmin(fmax(d2 * invf, -CO_G_MAX), CO_G_MAX);
        }
        g[a] = g1;
        g[N + a] = g2;
        if (red) {
            double e1 = dv[a], e2 = dv[N + a];
            pdot -= w[a] * (e1 * g1 + e2 * g2);
            pn2 += e1 * e1 + e2 * e2;
        }
    }
    if (red) {
        double s = co_block_sum(pdot, sh);
        double n = co_block_sum(pn2, sh);
        if (threadIdx.x == 0) {
            red[blockIdx.x * 2 + 0] = s;
            red[blockIdx.x * 2 + 1] = n;
        }
    }
}

// Hessian of the spline field L at markers x (cell/xi of x's last sort):
// H = (d11 L, d12 L, d22 L) with the P2 basis' second derivatives
// d^2 B / dxi^2 = (2, -4, 2); 0 outside the domain. Used by the block-Newton
// preconditioner of the defect correction's inner iteration.
__global__ void k_hess_L(int N, const int *__restrict__ cell, const double *__restrict__ xi,
                         const double *__restrict__ Lc, int n1, int nd1,
                         const double *__restrict__ bp1, const double *__restrict__ bp2,
                         const double *__restrict__ C1, const double *__restrict__ C2,
                         double *__restrict__ H) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    int c = cell[a];
    double h11 = 0.0, h12 = 0.0, h22 = 0.0;
    if (c >= 0) {
        int i = c % n1, j = c / n1;
        double ih1 = 1.0 / (bp1[i + 1] - bp1[i]), ih2 = 1.0 / (bp2[j + 1] - bp2[j]);
        const double d2B[3] = {2.0, -4.0, 2.0};
        double B1[3], dB1[3], B2[3], dB2[3], p1[3], dp1[3], q1[3], p2[3], dp2[3], q2[3];
        bern2(xi[a], B1, dB1);
        bern2(xi[N + a], B2, dB2);
        extract3(C1 + 9 * i, B1, p1);
        extract3(C1 + 9 * i, dB1, dp1);
        extract3(C1 + 9 * i, d2B, q1);
        extract3(C2 + 9 * j, B2, p2);
        extract3(C2 + 9 * j, dB2, dp2);
        extract3(C2 + 9 * j, d2B, q2);
        for (int b = 0; b < 3; b++)
            for (int q = 0; q < 3; q++) {
                double Lv = Lc[(i + q) + (j + b) * nd1];
                h11 += Lv * (q1[q] * p2[b]) * (ih1 * ih1);
                h12 += Lv * (dp1[q] * dp2[b]) * (ih1 * ih2);
                h22 += Lv * (p1[q] * q2[b]) * (ih2 * ih2);
            }
    }
    H[a] = h11;
    H[N + a] = h12;
    H[2 * (size_t)N + a] = h22;
}

// Warm-start features per marker at the step's start x (after the predictor),
// FP32 rows of CO_WS_NFEAT: 0-1 the predictor velocity vdot, 2-3 G (entropy
// gradient), 4-5 the clamped grad f_s / f_s, 6 log max(f_s, 1e-30), 7-9 the
// Hessian of L (H11, H12, H22), 10-12 the FP32 pair metric A (A11, A12, A22);
// columns 13-14 (the predictor's first residual / dt) are written afterwards.
// H and A are the two factors of the local stiffness dt A H / 2 of the implicit
// step, so the network sees the quantities a local Newton correction needs.
__global__ void k_features(int N, const int *__restrict__ cell, const double *__restrict__ xi,
                           const double *__restrict__ fc, int n1, int nd1,
                           const double *__restrict__ bp1, const double *__restrict__ bp2,
                           const double *__restrict__ C1, const double *__restrict__ C2,
                           const double *__restrict__ G, const double *__restrict__ vdot,
                           const double *__restrict__ H, const double *__restrict__ A,
                           float *__restrict__ X) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    int c = cell[a];
    double f = 0.0, g1 = 0.0, g2 = 0.0;
    if (c >= 0) {
        int i = c % n1, j = c / n1;
        double ih1 = 1.0 / (bp1[i + 1] - bp1[i]), ih2 = 1.0 / (bp2[j + 1] - bp2[j]);
        double B1[3], dB1[3], B2[3], dB2[3], p1[3], dp1[3], p2[3], dp2[3];
        bern2(xi[a], B1, dB1);
        bern2(xi[N + a], B2, dB2);
        extract3(C1 + 9 * i, B1, p1);
        extract3(C1 + 9 * i, dB1, dp1);
        extract3(C2 + 9 * j, B2, p2);
        extract3(C2 + 9 * j, dB2, dp2);
        double d1 = 0.0, d2 = 0.0;
        for (int b = 0; b < 3; b++)
            for (int q = 0; q < 3; q++) {
                double cv = fc[(i + q) + (j + b) * nd1];
                f += cv * (p1[q] * p2[b]);
                d1 += cv * (dp1[q] * p2[b]) * ih1;
                d2 += cv * (p1[q] * dp2[b]) * ih2;
            }
        double invf = 1.0 / fmax(fabs(f), CO_FS_FLOOR);
        g1 = fmin(fmax(d1 * invf, -CO_G_MAX), CO_G_MAX);
        g2 = fmin(fmax(d2 * invf, -CO_G_MAX), CO_G_MAX);
    }
    float *o = X + (size_t)a * CO_WS_NFEAT;
    o[0] = (float)vdot[a];
    o[1] = (float)vdot[N + a];
    o[2] = (float)G[a];
    o[3] = (float)G[N + a];
    o[4] = (float)g1;
    o[5] = (float)g2;
    o[6] = (float)log(fmax(f, CO_FS_FLOOR));
    for (int k = 0; k < 3; k++) {
        o[7 + k] = (float)H[(size_t)k * N + a];
        o[10 + k] = (float)A[(size_t)k * N + a];
    }
}

// columns 13-14 of the features: the predictor's first residual r / dt
__global__ void k_features_res(int N, const double *__restrict__ r, double inv_dt,
                               float *__restrict__ X) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    X[(size_t)a * CO_WS_NFEAT + 13] = (float)(r[a] * inv_dt);
    X[(size_t)a * CO_WS_NFEAT + 14] = (float)(r[N + a] * inv_dt);
}

// ---------------------------------------------------------------- host side

// set 0: the context's primary sort/projection buffers
static co_sortset primary_set(co_ctx *c) {
    co_bufs &b = c->mb;
    co_sortset s;
    s.cell = b.cell;
    s.inv = b.inv;
    s.perm = b.perm;
    s.scell = b.scell;
    s.hist = b.hist;
    s.hoff = b.hoff;
    s.count = b.count;
    s.cstart = b.cstart;
    s.xi = b.xi;
    s.sw = b.sw;
    s.sphi = b.sphi;
    s.bS = c->bS;
    s.b = c->b;
    s.y = c->y;
    return s;
}

void co_sortset_free(co_ctx *c) {
    co_sortset &g = c->gs;
    void *p[] = {g.cell, g.inv, g.perm, g.scell, g.hist, g.hoff, g.count, g.cstart,
                 g.xi, g.sw, g.sphi, g.bS, g.b, g.y};
    for (void *q : p)
        if (q) cudaFree(q);
    memset(&g, 0, sizeof(g));
    c->gs_cap = 0;
}

// set 1 at the context's marker capacity
static int ensure_gs(co_ctx *c) {
    if (c->gs_cap == c->mb.cap && c->gs.cell) return CO_OK;
    co_sortset_free(c);
    co_sortset &g = c->gs;
    const size_t cap = (size_t)c->mb.cap, nch = (size_t)c->mb.nchunk_cap, ne = c->n_el;
    bool ok = cudaMalloc(&g.cell, sizeof(int) * cap) == cudaSuccess &&
              cudaMalloc(&g.inv, sizeof(int) * cap) == cudaSuccess &&
              cudaMalloc(&g.perm, sizeof(int) * cap) == cudaSuccess &&
              cudaMalloc(&g.scell, sizeof(int) * cap) == cudaSuccess &&
              cudaMalloc(&g.hist, sizeof(int) * nch * ne) == cudaSuccess &&
              cudaMalloc(&g.hoff, sizeof(int) * nch * ne) == cudaSuccess &&
              cudaMalloc(&g.count, sizeof(int) * ne) == cudaSuccess &&
              cudaMalloc(&g.cstart, sizeof(int) * (ne + 1)) == cudaSuccess &&
              cudaMalloc(&g.xi, sizeof(double) * 2 * cap) == cudaSuccess &&
              cudaMalloc(&g.sw, sizeof(double) * cap) == cudaSuccess &&
              cudaMalloc(&g.sphi, sizeof(double) * 6 * cap) == cudaSuccess &&
              cudaMalloc(&g.bS, sizeof(double) * 9 * ne) == cudaSuccess &&
              cudaMalloc(&g.b, sizeof(double) * c->n_dofs) == cudaSuccess &&
              cudaMalloc(&g.y, sizeof(double) * c->n_dofs) == cudaSuccess;
    if (!ok) {
        co_sortset_free(c);
        return CO_ERR_NOMEM;
    }
    c->gs_cap = c->mb.cap;
    return CO_OK;
}

// locate + stable sort of one or two marker sets (jobs j0 -> set 0, j1 -> set 1)
static int sort_sets(co_ctx *c, const co_locate_job &j0, const co_locate_job &j1, int nsets,
                     int N) {
    co_bufs &b = c->mb;
    const co_sortset s0 = primary_set(c), s1 = nsets > 1 ? c->gs : s0;
    int nchunk = co_cdiv(N, CO_CHUNK);
    if (nchunk == 0) nchunk = 1;
    size_t sm = sizeof(int) * (size_t)c->n_el;
    if (N > 0) {
        k_locate_hist<<<dim3(nchunk, nsets), CO_CHUNK, sm, c->stream>>>(
            j0, j1, N, c->bp1, c->n1, c->bp2, c->n2, c->ih1, c->ih2, c->n_el);
        c->launches++;
    } else {
        CO_CK(cudaMemsetAsync(s0.hist, 0, sizeof(int) * c->n_el, c->stream));
        if (nsets > 1) CO_CK(cudaMemsetAsync(s1.hist, 0, sizeof(int) * c->n_el, c->stream));
    }
    k_cellcount<<<dim3(co_cdiv(c->n_el, 256), nsets), 256, 0, c->stream>>>(
        s0, s1, N > 0 ? nchunk : 1, c->n_el, c->tickets);
    c->launches++;
    if (N > 0) {
        k_perm<<<dim3(nchunk, nsets), CO_CHUNK, sm, c->stream>>>(s0, s1, N, c->n_el, c->n1,
                                                                 b.w, c->P1, c->P2);
        c->launches++;
    }
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// locate + stable sort of markers x (N) into set 0. Results: mb.cell, mb.xi,
// mb.perm, mb.inv, mb.scell, mb.sw, mb.sphi, cstart (M_in = cstart[n_el]).
int co_sort_markers(co_ctx *c, const double *x, int N) {
    co_bufs &b = c->mb;
    co_locate_job j = {x, nullptr, nullptr, nullptr, b.cell, b.xi, b.hist};
    return sort_sets(c, j, j, 1, N);
}

int co_sort_mid(co_ctx *c, const double *vin, const double *v0, int N, int two) {
    co_bufs &b = c->mb;
    int rc;
    if (two && (rc = ensure_gs(c))) return rc;
    co_locate_job j0 = {vin, v0, b.vmid, b.dv, b.cell, b.xi, b.hist};
    co_locate_job j1 = j0;
    if (two) j1 = {vin, nullptr, nullptr, nullptr, c->gs.cell, c->gs.xi, c->gs.hist};
    return sort_sets(c, j0, j1, two ? 2 : 1, N);
}

static int mass_solve_two(co_ctx *c, const double *r0, double *y0, double *o0,
                          const double *r1, double *y1, double *o1, int nsets) {
    // one warp per MASS_OUT outputs of a column, eight warps per block
    const int nw = co_cdiv(c->nd1, MASS_OUT) * c->nd2;
    k_mass1<<<dim3(co_cdiv(nw, 8), nsets), 256, 0, c->stream>>>(c->Minv1, r0, y0, r1, y1,
                                                                 c->nd1, c->nd2);
    k_mass2<<<dim3(co_cdiv(nw, 8), nsets), 256, 0, c->stream>>>(c->Minv2, y0, o0, y1, o1,
                                                                 c->nd1, c->nd2);
    c->launches += 2;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_mass_solve_dev(co_ctx *c, const double *rhs, double *out) {
    return mass_solve_two(c, rhs, c->y, out, rhs, c->y, out, 1);
}

// cell sums -> (dof gather + M1^{-1}) -> M2^{-1}, for one or two marker sets
static int gather_solve_two(co_ctx *c, const double *e0, double *y0, double *o0,
                            const double *e1, double *y1, double *o1, int nsets) {
    k_gather_mass1<<<dim3(c->nd2, nsets), 256, sizeof(double) * c->nd1, c->stream>>>(
        e0, y0, e1, y1, c->Minv1, c->n1, c->n2, c->nd1, c->nd2);
    const int nw = co_cdiv(c->nd1, MASS_OUT) * c->nd2;
    k_mass2<<<dim3(co_cdiv(nw, 8), nsets), 256, 0, c->stream>>>(c->Minv2, y0, o0, y1, o1,
                                                                 c->nd1, c->nd2);
    c->launches += 2;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_project_two(co_ctx *c, double *f0, double *f1, int two) {
    const int nsets = two ? 2 : 1;
    const co_sortset s0 = primary_set(c), s1 = two ? c->gs : s0;
    k_cellsum<<<dim3(c->n_el, nsets), 128, 0, c->stream>>>(s0, s1, c->n_el);
    c->launches++;
    CO_CK(cudaGetLastError());
    return gather_solve_two(c, s0.bS, s0.y, f0, s1.bS, s1.y, two ? f1 : f0, nsets);
}

// after co_sort_markers: b = scatter, f = M^{-1} b
int co_project_sorted(co_ctx *c, double *f_out) { return co_project_two(c, f_out, f_out, 0); }

int co_r_and_entropy_dev(co_ctx *c, const double *f, double *r, const double *fS) {
    co_elem_job jr = {f, 0, c->E};
    co_elem_job js = {fS, 1, c->Ep};
    k_elem<<<dim3(co_cdiv(c->n_el, ELEM_THREADS / c->nq), fS ? 2 : 1), ELEM_THREADS, 0,
             c->stream>>>(jr, js, c->n1, c->n2, c->nd1, c->nq, c->Tq1, c->Tq2, c->qw, c->bp1,
                          c->bp2, (c->flags & CO_FLAG_LOGSQ) ? 1 : 0);
    k_dofgather<<<dim3(co_cdiv(c->n_dofs, 128), 1), 128, 0, c->stream>>>(
        c->E, r, c->E, r, c->n1, c->n2, c->nd1, c->nd2);
    c->launches += 2;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_r_solve_dev(co_ctx *c, const double *f, double *L, const double *fS) {
    co_elem_job jr = {f, 0, c->E};
    co_elem_job js = {fS, 1, c->Ep};
    k_elem<<<dim3(co_cdiv(c->n_el, ELEM_THREADS / c->nq), fS ? 2 : 1), ELEM_THREADS, 0,
             c->stream>>>(jr, js, c->n1, c->n2, c->nd1, c->nq, c->Tq1, c->Tq2, c->qw, c->bp1,
                          c->bp2, (c->flags & CO_FLAG_LOGSQ) ? 1 : 0);
    c->launches++;
    CO_CK(cudaGetLastError());
    return gather_solve_two(c, c->E, c->y, L, c->E, c->y, L, 1);
}

int co_compute_r_dev(co_ctx *c, const double *f, double *r) {
    return co_r_and_entropy_dev(c, f, r, nullptr);
}

int co_entropy_parts_dev(co_ctx *c, const double *f) {
    co_elem_job js = {f, 1, c->Ep};
    k_elem<<<dim3(co_cdiv(c->n_el, ELEM_THREADS / c->nq), 1), ELEM_THREADS, 0, c->stream>>>(
        js, js, c->n1, c->n2, c->nd1, c->nq, c->Tq1, c->Tq2, c->qw, c->bp1, c->bp2,
        (c->flags & CO_FLAG_LOGSQ) ? 1 : 0);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_entropy_finalize_dev(co_ctx *c, double *S_dev) {
    k_sum_to<<<1, 256, 0, c->stream>>>(c->Ep, c->n_el, S_dev);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// post-step diagnostics of markers x (device) with weights in mb.w -> out6 (device)
int co_diagnostics_impl(co_ctx *c, const double *x, int N, double *out6) {
    int rc;
    if ((rc = co_sort_markers(c, x, N))) return rc;
    if ((rc = co_project_sorted(c, c->f))) return rc;
    double *D = c->E;   // n_el x 9 scratch; the diagnostics use n_el x 3
    k_diag_elem<<<c->n_el, 64, 0, c->stream>>>(c->f, c->n1, c->nd1, c->nq, c->Tq1, c->Tq2, c->qw,
                                               c->bp1, c->bp2, (c->flags & CO_FLAG_LOGSQ) ? 1 : 0,
                                               c->bS, D);
    int g = co_cdiv(N > 0 ? N : 1, CO_RED_THREADS);
    if (g > c->mb.red_cap) g = c->mb.red_cap;
    k_marker_moments<<<g, CO_RED_THREADS, 0, c->stream>>>(x, c->mb.w, N, c->mb.red);
    k_diag_final<<<1, 256, 0, c->stream>>>(D, c->n_el, c->mb.red, g, out6);
    c->launches += 3;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

static int red_grid(co_ctx *c, int N) {
    int g = co_cdiv(N, CO_RED_THREADS);
    if (g > c->mb.red_cap) g = c->mb.red_cap;
    if (g < 1) g = 1;
    return g;
}

// gradient gather at x (cell/xi from the last locate of x)
int co_grad_L_dev(co_ctx *c, const double *x, int N, const double *L, double *G,
                  const double *w, double *dS, const double *dv, double *red) {
    if (N == 0) return CO_OK;
    co_lambda_job none = {};
    k_grad_L<<<red_grid(c, N), CO_RED_THREADS, 0, c->stream>>>(
        x, N, c->mb.cell, c->mb.xi, L, c->n1, c->nd1, c->ih1, c->ih2, c->P1, c->P2, G, w, dS, dv,
        red, none);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_grad_L_lambda_dev(co_ctx *c, const double *x, int N, const double *L, double *G,
                         const double *w, double *dS, const double *dv, double *red,
                         double S0, int gonzalez, const double *Ep) {
    if (N == 0) return CO_ERR_ARG;
    co_lambda_job lam = {c->st, S0, gonzalez, Ep, c->n_el, c->tickets + CO_TICKET_LAMBDA};
    k_grad_L<<<red_grid(c, N), CO_RED_THREADS, 0, c->stream>>>(
        x, N, c->mb.cell, c->mb.xi, L, c->n1, c->nd1, c->ih1, c->ih2, c->P1, c->P2, G, w, dS, dv,
        red, lam);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_loggrad_dev(co_ctx *c, const double *x, int N, const double *f, double *g,
                   const double *w, const double *dv, double *red) {
    if (N == 0) return CO_OK;
    k_loggrad<<<red_grid(c, N), CO_RED_THREADS, 0, c->stream>>>(
        x, N, c->mb.cell, c->mb.xi, f, c->n1, c->nd1, c->bp1, c->bp2, c->C1, c->C2, g, w, dv, red);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// dynamic shared memory of the sort kernels (one int per cell)
int co_spline_configure(co_ctx *c) {
    int bytes = (int)(sizeof(int) * (size_t)c->n_el);
    if (bytes > 48 * 1024) {
        if (bytes > 200 * 1024) return CO_ERR_UNSUPPORTED;
        CO_CK(cudaFuncSetAttribute(k_locate_hist, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
        CO_CK(cudaFuncSetAttribute(k_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    }
    return CO_OK;
}

// ------------------------------------------------------------- capacity

template <typename T>
static int grow(T **p, size_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc((void **)p, n * sizeof(T)) != cudaSuccess) return CO_ERR_NOMEM;
    return CO_OK;
}

int co_ensure_capacity(co_ctx *c, int N, int m) {
    co_bufs &b = c->mb;
    int rc;
    if (N > b.cap) {
        int cap = N < 1024 ? 1024 : N;
        cap = (cap + 255) / 256 * 256;  // packed pair operands are padded to whole tiles
        size_t n2 = 2 * (size_t)cap;
        double **d2[] = {&b.vmid, &b.dv, &b.G, &b.dS, &b.Gv, &b.r, &b.rp, &b.Gp,
                         &b.vbest, &b.v1, &b.v0, &b.vin, &b.dotv, &b.xi};
        for (double **p : d2)
            if ((rc = grow(p, n2))) return rc;
        if ((rc = grow(&b.w, (size_t)cap))) return rc;
        if ((rc = grow(&b.cell, (size_t)cap))) return rc;
        if ((rc = grow(&b.inv, (size_t)cap))) return rc;
        if ((rc = grow(&b.perm, (size_t)cap))) return rc;
        if ((rc = grow(&b.scell, (size_t)cap))) return rc;
        if ((rc = grow(&b.sw, (size_t)cap))) return rc;
        if ((rc = grow(&b.sphi, 6 * (size_t)cap))) return rc;
        if ((rc = grow(&b.px, (size_t)cap))) return rc;
        if ((rc = grow(&b.pg, (size_t)cap))) return rc;
        if ((rc = grow(&b.pw, (size_t)cap))) return rc;
        if ((rc = grow(&b.pf_x, (size_t)cap))) return rc;
        if ((rc = grow(&b.pf_g, (size_t)cap))) return rc;
        if ((rc = grow(&b.pf_w, (size_t)cap))) return rc;
        if ((rc = grow(&b.pf_wl, (size_t)cap))) return rc;
        if ((rc = grow(&b.pdot, n2))) return rc;
        if ((rc = grow(&b.pA, 3 * (size_t)cap))) return rc;
        int nchunk = co_cdiv(cap, CO_CHUNK);
        if ((rc = grow(&b.hist, (size_t)nchunk * c->n_el))) return rc;
        if ((rc = grow(&b.hoff, (size_t)nchunk * c->n_el))) return rc;
        b.nchunk_cap = nchunk;
        b.cap = cap;
        // set 1 is allocated with set 0, never on first use: the Picard maps
        // that use it are captured into CUDA graphs, where no allocation may run
        if ((rc = ensure_gs(c))) return rc;
        double **lazy[] = {&b.Gk, &b.Phi, &b.Adef, &b.aa, &b.pc};  // re-created at the new size on use
        for (double **q : lazy) {
            if (*q) cudaFree(*q);
            *q = nullptr;
        }
        b.aa_m = 0;
        if (b.m_cap > 0) {
            if ((rc = grow(&b.dF, n2 * b.m_cap))) return rc;
            if ((rc = grow(&b.dG, n2 * b.m_cap))) return rc;
        }
    }
    if (m > b.m_cap) {
        size_t n2 = 2 * (size_t)b.cap;
        if ((rc = grow(&b.dF, n2 * m))) return rc;
        if ((rc = grow(&b.dG, n2 * m))) return rc;
        b.m_cap = m;
    }
    return CO_OK;
}

// Hessian of c->L at x (cell/xi of x's last sort) -> H (3N)
int co_hess_L_dev(co_ctx *c, int N, double *H) {
    if (N == 0) return CO_OK;
    k_hess_L<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, c->mb.cell, c->mb.xi, c->L, c->n1, c->nd1,
                                                     c->bp1, c->bp2, c->C1, c->C2, H);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// features at the last sorted markers (cell/xi of that sort, coefficients in
// c->f, G and dotv in the marker buffers, H and A as given)
int co_features_dev(co_ctx *c, int N, const double *H, const double *A, float *X) {
    if (N == 0) return CO_OK;
    k_features<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, c->mb.cell, c->mb.xi, c->f, c->n1,
                                                       c->nd1, c->bp1, c->bp2, c->C1, c->C2,
                                                       c->mb.G, c->mb.dotv, H, A, X);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_features_res_dev(co_ctx *c, int N, const double *r, double dt, float *X) {
    if (N == 0) return CO_OK;
    k_features_res<<<co_cdiv(N, 256), 256, 0, c->stream>>>(N, r, 1.0 / dt, X);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}
