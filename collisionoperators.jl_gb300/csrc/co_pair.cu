// co_pair.cu -- the O(N^2) Landau pair sum (functions.jl:205-237) on sm_103a.
//
// N-body layout: the in-domain markers are compacted and cell-sorted by the
// spline stage; the pack kernel lays their operands out contiguously (px, pg,
// pw). A block owns a tile of targets gamma (one per thread) and streams the
// sources alpha through shared memory in tiles; the alpha range can be split
// into slices whose partial sums are added afterwards in slice order, so
// results are bitwise reproducible for a given N.
//
// FP64 form (the reference's Float64 path): on GB300 FP64 issues at 1/64 of
// the FP32 rate, so the per-pair FP64 instruction count is what sets the time.
// The pair body is 20 FP64 instructions:
//   d (2), |d|^2 (2), 1/|d| refinement (5), G difference (2), d.g (2),
//   1/|d|^2 and (d.g)/|d|^2 (2), projection (2), w/|d| (1), accumulate (2).
// 1/|d| starts from a single-precision seed built from the FP64 bit pattern
// with integer operations (no FP64 conversion instructions) and MUFU.RSQ, then
// one third-order Newton step y += y e (1/2 + 3/8 e), e = 1 - x y^2, which
// takes the ~2^-20 seed error to below 2^-53 (the same idea as the
// reference's f32 seed + two Newton steps, collision_gpu.jl:36-44, with one
// higher-order step in place of two quadratic ones). The |d|^2 < 1e-24 guard
// (functions.jl:224) is an integer compare on the bit pattern.
//
// Mixed form (the precision form of the solver): the pair arithmetic runs in FP32 on
// FP64-centred differences -- each coordinate is split into an FP32 head and
// tail (x = xh + xl), so d = (xh_g - xh_a) + (xl_g - xl_a) is accurate to an
// FP32 rounding of d itself even for close pairs -- and the per-tile FP32
// partial sums are accumulated in FP64.
#include "co_internal.cuh"
#include "co_reduce.cuh"

#define PAIR_TPB 128

// bit pattern of 1e-24 (functions.jl:224 guard)
#define CO_R2_MIN_BITS 0x3B282DB34012B251LL

__device__ __forceinline__ double rsqrt_seed64(double x) {
    // FP32 value of x from its high word (x in [1e-30, 1e30], positive)
    int hi = __double2hiint(x);
    float xf = __int_as_float((hi - (896 << 20)) << 3);
    float yf = rsqrtf(xf);
    int fb = __float_as_int(yf);
    return __hiloint2double((fb >> 3) + (896 << 20), fb << 29);
}

__device__ __forceinline__ void pair64(double xg1, double xg2, double Gg1, double Gg2,
                                       double xa1, double xa2, double Ga1, double Ga2,
                                       double wa, double &acc1, double &acc2) {
    double d1 = xg1 - xa1;
    double d2 = xg2 - xa2;
    double r2 = d1 * d1;
    r2 = fma(d2, d2, r2);
    bool ok = __double_as_longlong(r2) >= CO_R2_MIN_BITS;
    double xr = ok ? r2 : 1.0;
    double y = rsqrt_seed64(xr);
    double t = xr * y;
    double e = fma(-t, y, 1.0);
    double p = fma(0.375, e, 0.5);
    double ye = y * e;
    y = fma(ye, p, y);
    double g1 = Ga1 - Gg1;
    double g2 = Ga2 - Gg2;
    double dg = d1 * g1;
    dg = fma(d2, g2, dg);
    double y2 = y * y;
    double cc = dg * y2;
    double t1 = fma(-d1, cc, g1);
    double t2 = fma(-d2, cc, g2);
    double s = wa * y;
    s = ok ? s : 0.0;
    acc1 = fma(s, t1, acc1);
    acc2 = fma(s, t2, acc2);
}

// F and the metric A (functions.jl:249-290 / collision_gpu.jl:289-339)
__device__ __forceinline__ void pair64_metric(double xg1, double xg2, double Gg1, double Gg2,
                                              double xa1, double xa2, double Ga1, double Ga2,
                                              double wa, double &acc1, double &acc2,
                                              double &a11, double &a12, double &a22) {
    double d1 = xg1 - xa1;
    double d2 = xg2 - xa2;
    double q11 = d1 * d1, q22 = d2 * d2;
    double r2 = q11 + q22;
    bool ok = __double_as_longlong(r2) >= CO_R2_MIN_BITS;
    double xr = ok ? r2 : 1.0;
    double y = rsqrt_seed64(xr);
    double t = xr * y;
    double e = fma(-t, y, 1.0);
    double p = fma(0.375, e, 0.5);
    double ye = y * e;
    y = fma(ye, p, y);
    double g1 = Ga1 - Gg1;
    double g2 = Ga2 - Gg2;
    double dg = d1 * g1;
    dg = fma(d2, g2, dg);
    double y2 = y * y;
    double cc = dg * y2;
    double t1 = fma(-d1, cc, g1);
    double t2 = fma(-d2, cc, g2);
    double s = wa * y;
    s = ok ? s : 0.0;
    acc1 = fma(s, t1, acc1);
    acc2 = fma(s, t2, acc2);
    a11 = fma(s, fma(-q11, y2, 1.0), a11);
    a12 = fma(-s, (d1 * d2) * y2, a12);
    a22 = fma(s, fma(-q22, y2, 1.0), a22);
}

// out layout: partial[slice][comp][M] with stride ld
template <bool METRIC>
__global__ void __launch_bounds__(PAIR_TPB)
k_pair64(const double2 *__restrict__ px, const double2 *__restrict__ pg,
         const double *__restrict__ pw, const int *__restrict__ Mp, int slice_len,
         double *__restrict__ out, size_t ld) {
    __shared__ double2 sx[PAIR_TPB];
    __shared__ double2 sg[PAIR_TPB];
    __shared__ double sw[PAIR_TPB];
    const int M = *Mp;
    const int g0 = blockIdx.x * PAIR_TPB;
    if (g0 >= M) return;
    const int g = g0 + threadIdx.x;
    const int sl = blockIdx.y;
    const int a0 = sl * slice_len;
    const int a1 = min(M, a0 + slice_len);
    double2 xg = make_double2(0.0, 0.0), Gg = make_double2(0.0, 0.0);
    if (g < M) {
        xg = px[g];
        Gg = pg[g];
    }
    double acc1 = 0.0, acc2 = 0.0, a11 = 0.0, a12 = 0.0, a22 = 0.0;
    for (int base = a0; base < a1; base += PAIR_TPB) {
        int a = base + threadIdx.x;
        if (a < a1) {
            sx[threadIdx.x] = px[a];
            sg[threadIdx.x] = pg[a];
            sw[threadIdx.x] = pw[a];
        } else {  // inert padding: far away, zero weight
            sx[threadIdx.x] = make_double2(1e3, 1e3);
            sg[threadIdx.x] = make_double2(0.0, 0.0);
            sw[threadIdx.x] = 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < PAIR_TPB; k++) {
            double2 xa = sx[k], Ga = sg[k];
            if (METRIC)
                pair64_metric(xg.x, xg.y, Gg.x, Gg.y, xa.x, xa.y, Ga.x, Ga.y, sw[k], acc1, acc2,
                              a11, a12, a22);
            else
                pair64(xg.x, xg.y, Gg.x, Gg.y, xa.x, xa.y, Ga.x, Ga.y, sw[k], acc1, acc2);
        }
        __syncthreads();
    }
    if (g < M) {
        const int nc = METRIC ? 5 : 2;
        double *o = out + (size_t)sl * nc * ld;
        o[g] = acc1;
        o[ld + g] = acc2;
        if (METRIC) {
            o[2 * ld + g] = a11;
            o[3 * ld + g] = a12;
            o[4 * ld + g] = a22;
        }
    }
}

// FP32 pair body on head/tail-split operands
__device__ __forceinline__ void pair32(const float4 &xg, const float4 &Gg, const float4 &xa,
                                       const float4 &Ga, float wa, float &acc1, float &acc2) {
    float d1 = (xg.x - xa.x) + (xg.z - xa.z);
    float d2 = (xg.y - xa.y) + (xg.w - xa.w);
    float g1 = (Ga.x - Gg.x) + (Ga.z - Gg.z);
    float g2 = (Ga.y - Gg.y) + (Ga.w - Gg.w);
    float r2 = d1 * d1;
    r2 = fmaf(d2, d2, r2);
    float y = rsqrtf(r2);
    y = r2 >= 1e-24f ? y : 0.0f;
    float dg = d1 * g1;
    dg = fmaf(d2, g2, dg);
    float y2 = y * y;
    float cc = dg * y2;
    float t1 = fmaf(-d1, cc, g1);
    float t2 = fmaf(-d2, cc, g2);
    float s = wa * y;
    acc1 = fmaf(s, t1, acc1);
    acc2 = fmaf(s, t2, acc2);
}

#define PAIR32_TILE 256
__global__ void __launch_bounds__(PAIR_TPB)
k_pair32(const float4 *__restrict__ pfx, const float4 *__restrict__ pfg,
         const float *__restrict__ pfw, const int *__restrict__ Mp, int slice_len,
         double *__restrict__ out, size_t ld) {
    __shared__ float4 sx[PAIR32_TILE];
    __shared__ float4 sg[PAIR32_TILE];
    __shared__ float sw[PAIR32_TILE];
    const int M = *Mp;
    const int g0 = blockIdx.x * PAIR_TPB;
    if (g0 >= M) return;
    const int g = g0 + threadIdx.x;
    const int sl = blockIdx.y;
    const int a0 = sl * slice_len;
    const int a1 = min(M, a0 + slice_len);
    float4 xg = make_float4(0.f, 0.f, 0.f, 0.f), Gg = xg;
    if (g < M) {
        xg = pfx[g];
        Gg = pfg[g];
    }
    double acc1 = 0.0, acc2 = 0.0;
    for (int base = a0; base < a1; base += PAIR32_TILE) {
        for (int k = threadIdx.x; k < PAIR32_TILE; k += PAIR_TPB) {
            int a = base + k;
            if (a < a1) {
                sx[k] = pfx[a];
                sg[k] = pfg[a];
                sw[k] = pfw[a];
            } else {
                sx[k] = make_float4(1e3f, 1e3f, 0.f, 0.f);
                sg[k] = make_float4(0.f, 0.f, 0.f, 0.f);
                sw[k] = 0.f;
            }
        }
        __syncthreads();
        float t1 = 0.f, t2 = 0.f;
#pragma unroll 8
        for (int k = 0; k < PAIR32_TILE; k++) pair32(xg, Gg, sx[k], sg[k], sw[k], t1, t2);
        acc1 += (double)t1;
        acc2 += (double)t2;
        __syncthreads();
    }
    if (g < M) {
        double *o = out + (size_t)sl * 2 * ld;
        o[g] = acc1;
        o[ld + g] = acc2;
    }
}

// ------------------------------------------------------------------ metric (FP32)
//
// A_g = sum_a w_a U(v_g - v_a), U(z) = (I - z z^T/|z|^2)/|z|  (functions.jl:278-281),
// evaluated in FP32 on the head parts of the packed operands. Used only as the
// frozen metric of the defect-correction inner model (solver.jl:585-595), where
// it shapes the convergence rate but not the fixed point: the outer residual is
// always an FP64 (or, in the mixed form, FP32-then-FP64) Picard map.
__global__ void __launch_bounds__(PAIR_TPB)
k_metric32(const float4 *__restrict__ pfx, const float *__restrict__ pfw,
           const int *__restrict__ Mp, double *__restrict__ out, size_t ld) {
    __shared__ float2 sx[PAIR32_TILE];
    __shared__ float sw[PAIR32_TILE];
    const int M = *Mp;
    const int g0 = blockIdx.x * PAIR_TPB;
    if (g0 >= M) return;
    const int g = g0 + threadIdx.x;
    float2 xg = make_float2(0.f, 0.f);
    if (g < M) {
        float4 t = pfx[g];
        xg = make_float2(t.x + t.z, t.y + t.w);
    }
    double A11 = 0.0, A12 = 0.0, A22 = 0.0;
    for (int base = 0; base < M; base += PAIR32_TILE) {
        for (int k = threadIdx.x; k < PAIR32_TILE; k += PAIR_TPB) {
            int a = base + k;
            if (a < M) {
                float4 t = pfx[a];
                sx[k] = make_float2(t.x + t.z, t.y + t.w);
                sw[k] = pfw[a];
            } else {
                sx[k] = make_float2(1e3f, 1e3f);
                sw[k] = 0.f;
            }
        }
        __syncthreads();
        float a11 = 0.f, a12 = 0.f, a22 = 0.f;
#pragma unroll 8
        for (int k = 0; k < PAIR32_TILE; k++) {
            float d1 = xg.x - sx[k].x, d2 = xg.y - sx[k].y;
            float r2 = fmaf(d2, d2, d1 * d1);
            float y = rsqrtf(r2);
            y = r2 >= 1e-24f ? y : 0.f;
            float s = sw[k] * y;
            float y2 = y * y;
            a11 = fmaf(s, fmaf(-d1 * d1, y2, 1.f), a11);
            a12 = fmaf(-s, d1 * d2 * y2, a12);
            a22 = fmaf(s, fmaf(-d2 * d2, y2, 1.f), a22);
        }
        A11 += (double)a11;
        A12 += (double)a12;
        A22 += (double)a22;
        __syncthreads();
    }
    if (g < M) {
        out[g] = A11;
        out[ld + g] = A12;
        out[2 * ld + g] = A22;
    }
}

// ------------------------------------------------------------------ symmetric
//
// Newton's third law for the pair sum: with d = v_g - v_a and g = G_a - G_g,
// the ordered pair (a, g) sees d' = -d and g' = -g, so its term is
// w_g U(d)(-g)/|d| = -w_g u with u = U(d) g / |d| the unweighted term of
// (g, a). One evaluation of u serves both targets.
//
// Tiles of ST = 128 sorted markers; tile pairs (I, J = I + k mod nt) for
// k = 0..H (H = nt/2; for even nt the k = H pairs are taken once, I < nt/2),
// so every unordered tile pair appears exactly once and every row I has the
// same work. A block owns I and a chunk of KC consecutive k. Inside a tile
// pair the 4 warps take the 4 source sub-tiles in rotation (one warp per
// sub-tile per round); within a warp, lane l pairs its target with source
// (l + q) mod 32 at step q and passes the source's accumulator to lane l - 1
// with a shuffle, so each source accumulator has one owner at every step. The
// target side accumulates in registers across the chunk (gpart); the source
// side of each tile pair is written to its own slot (apart) and everything is
// summed afterwards in a fixed order: bitwise reproducible.
//
// FP64 body: 19 FP64 instructions for u + 4 FMAs for the two accumulations =
// 23 per unordered pair, 11.5 per ordered pair (20 in k_pair64).
#define ST 128

__device__ __forceinline__ void pair_u64(double d1, double d2, double g1, double g2, double &u1,
                                         double &u2) {
    double r2 = d1 * d1;
    r2 = fma(d2, d2, r2);
    bool ok = __double_as_longlong(r2) >= CO_R2_MIN_BITS;
    double xr = ok ? r2 : 1.0;
    double y = rsqrt_seed64(xr);
    double t = xr * y;
    double e = fma(-t, y, 1.0);
    double p = fma(0.375, e, 0.5);
    double ye = y * e;
    y = fma(ye, p, y);
    double dg = d1 * g1;
    dg = fma(d2, g2, dg);
    double y2 = y * y;
    double cc = dg * y2;
    double t1 = fma(-d1, cc, g1);
    double t2 = fma(-d2, cc, g2);
    double ym = ok ? y : 0.0;
    u1 = t1 * ym;
    u2 = t2 * ym;
}

__device__ __forceinline__ bool sym_skip(int nt, int H, int I, int k) {
    return k > 0 && (nt & 1) == 0 && k == H && I >= nt / 2;
}

__global__ void __launch_bounds__(ST)
k_pair64_sym(const double2 *__restrict__ px, const double2 *__restrict__ pg,
             const double *__restrict__ pw, int nt, int H, int KC,
             double *__restrict__ gpart, double *__restrict__ apart) {
    __shared__ double2 sx[ST], sg[ST];
    __shared__ double sw[ST];
    __shared__ double2 sacc[ST];
    const int I = blockIdx.x % nt, chunk = blockIdx.x / nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double2 xg = px[I * ST + tid], Gg = pg[I * ST + tid];
    const double wg = pw[I * ST + tid];
    double ga1 = 0.0, ga2 = 0.0;
    const int k0 = chunk * KC, k1 = min(H + 1, k0 + KC);
    for (int k = k0; k < k1; k++) {
        if (sym_skip(nt, H, I, k)) continue;
        const int J = (I + k) % nt;
        __syncthreads();
        sx[tid] = px[J * ST + tid];
        sg[tid] = pg[J * ST + tid];
        sw[tid] = pw[J * ST + tid];
        sacc[tid] = make_double2(0.0, 0.0);
        __syncthreads();
        if (k == 0) {  // diagonal tile: ordered pairs, self excluded by the guard
#pragma unroll 4
            for (int a = 0; a < ST; a++) {
                double u1, u2;
                double2 xa = sx[a], Ga = sg[a];
                pair_u64(xg.x - xa.x, xg.y - xa.y, Ga.x - Gg.x, Ga.y - Gg.y, u1, u2);
                ga1 = fma(sw[a], u1, ga1);
                ga2 = fma(sw[a], u2, ga2);
            }
            continue;
        }
        for (int r = 0; r < 4; r++) {
            const int base = ((warp + r) & 3) * 32;
            double2 a0 = sacc[base + lane];
            double a1 = a0.x, a2 = a0.y;
#pragma unroll 4
            for (int q = 0; q < 32; q++) {
                const int ai = base + ((lane + q) & 31);
                double2 xa = sx[ai], Ga = sg[ai];
                double wa = sw[ai];
                double u1, u2;
                pair_u64(xg.x - xa.x, xg.y - xa.y, Ga.x - Gg.x, Ga.y - Gg.y, u1, u2);
                ga1 = fma(wa, u1, ga1);
                ga2 = fma(wa, u2, ga2);
                a1 = fma(-wg, u1, a1);
                a2 = fma(-wg, u2, a2);
                a1 = __shfl_sync(0xffffffffu, a1, (lane + 1) & 31);
                a2 = __shfl_sync(0xffffffffu, a2, (lane + 1) & 31);
            }
            sacc[base + lane] = make_double2(a1, a2);
            __syncthreads();
        }
        double *ap = apart + ((size_t)(k - 1) * nt + J) * 2 * ST;
        ap[tid] = sacc[tid].x;
        ap[ST + tid] = sacc[tid].y;
    }
    double *gp = gpart + ((size_t)chunk * nt + I) * 2 * ST;
    gp[tid] = ga1;
    gp[ST + tid] = ga2;
}

// FP32 body on head/tail operands: returns the unweighted term u
__device__ __forceinline__ void pair_u32(const float4 &xg, const float4 &Gg, const float4 &xa,
                                         const float4 &Ga, float &u1, float &u2) {
    float d1 = (xg.x - xa.x) + (xg.z - xa.z);
    float d2 = (xg.y - xa.y) + (xg.w - xa.w);
    float g1 = (Ga.x - Gg.x) + (Ga.z - Gg.z);
    float g2 = (Ga.y - Gg.y) + (Ga.w - Gg.w);
    float r2 = d1 * d1;
    r2 = fmaf(d2, d2, r2);
    float y = rsqrtf(r2);
    y = r2 >= 1e-24f ? y : 0.0f;
    float dg = d1 * g1;
    dg = fmaf(d2, g2, dg);
    float y2 = y * y;
    float cc = dg * y2;
    u1 = fmaf(-d1, cc, g1) * y;
    u2 = fmaf(-d2, cc, g2) * y;
}

// Register-blocked FP32 symmetric kernel: each of the ST threads holds R targets
// (t, t + ST, ...) of a TS = R * ST tile, so every source a thread loads from
// shared memory and every shuffle of the rotating source accumulators serves R
// pair evaluations. Source tile J is handled in NG = TS / 32 groups of 32: in
// round rr warp w takes group (w + rr) mod NG, so each group meets each warp
// once and its accumulators pass from warp to warp through sacc between rounds
// (fixed order, deterministic).
template <int R>
__global__ void __launch_bounds__(ST)
k_pair32_sym(const float4 *__restrict__ pfx, const float4 *__restrict__ pfg,
             const float *__restrict__ pfw, int nt, int H, int KC,
             double *__restrict__ gpart, float *__restrict__ apart) {
    constexpr int TS = R * ST, NG = TS / 32;
    __shared__ float4 sx[TS], sg[TS];
    __shared__ float sw[TS];
    __shared__ float2 sacc[TS];
    const int I = blockIdx.x % nt, chunk = blockIdx.x / nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float4 xg[R], Gg[R];
    float wg[R];
    double ga1[R], ga2[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        xg[r] = pfx[I * TS + r * ST + tid];
        Gg[r] = pfg[I * TS + r * ST + tid];
        wg[r] = pfw[I * TS + r * ST + tid];
        ga1[r] = 0.0;
        ga2[r] = 0.0;
    }
    const int k0 = chunk * KC, k1 = min(H + 1, k0 + KC);
    for (int k = k0; k < k1; k++) {
        if (sym_skip(nt, H, I, k)) continue;
        const int J = (I + k) % nt;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < R; r++) {
            sx[r * ST + tid] = pfx[J * TS + r * ST + tid];
            sg[r * ST + tid] = pfg[J * TS + r * ST + tid];
            sw[r * ST + tid] = pfw[J * TS + r * ST + tid];
            sacc[r * ST + tid] = make_float2(0.f, 0.f);
        }
        __syncthreads();
        float t1[R], t2[R];
#pragma unroll
        for (int r = 0; r < R; r++) t1[r] = t2[r] = 0.f;
        if (k == 0) {  // diagonal tile: ordered pairs, self excluded by the guard
#pragma unroll 4
            for (int a = 0; a < TS; a++) {
                const float4 xa = sx[a], Ga = sg[a];
                const float wa = sw[a];
#pragma unroll
                for (int r = 0; r < R; r++) {
                    float u1, u2;
                    pair_u32(xg[r], Gg[r], xa, Ga, u1, u2);
                    t1[r] = fmaf(wa, u1, t1[r]);
                    t2[r] = fmaf(wa, u2, t2[r]);
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                ga1[r] += (double)t1[r];
                ga2[r] += (double)t2[r];
            }
            continue;
        }
        for (int rr = 0; rr < NG; rr++) {
            const int base = ((warp + rr) % NG) * 32;
            float2 a0 = sacc[base + lane];
            float a1 = a0.x, a2 = a0.y;
#pragma unroll 4
            for (int q = 0; q < 32; q++) {
                const int ai = base + ((lane + q) & 31);
                const float4 xa = sx[ai], Ga = sg[ai];
                const float wa = sw[ai];
#pragma unroll
                for (int r = 0; r < R; r++) {
                    float u1, u2;
                    pair_u32(xg[r], Gg[r], xa, Ga, u1, u2);
                    t1[r] = fmaf(wa, u1, t1[r]);
                    t2[r] = fmaf(wa, u2, t2[r]);
                    a1 = fmaf(-wg[r], u1, a1);
                    a2 = fmaf(-wg[r], u2, a2);
                }
                a1 = __shfl_sync(0xffffffffu, a1, (lane + 1) & 31);
                a2 = __shfl_sync(0xffffffffu, a2, (lane + 1) & 31);
            }
            sacc[base + lane] = make_float2(a1, a2);
            __syncthreads();
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            ga1[r] += (double)t1[r];
            ga2[r] += (double)t2[r];
        }
        float *ap = apart + ((size_t)(k - 1) * nt + J) * 2 * TS;
#pragma unroll
        for (int r = 0; r < R; r++) {
            ap[r * ST + tid] = sacc[r * ST + tid].x;
            ap[TS + r * ST + tid] = sacc[r * ST + tid].y;
        }
    }
    double *gp = gpart + ((size_t)chunk * nt + I) * 2 * TS;
#pragma unroll
    for (int r = 0; r < R; r++) {
        gp[r * ST + tid] = ga1[r];
        gp[TS + r * ST + tid] = ga2[r];
    }
}

// ------------------------------------------------------------------ double-single
//
// The same symmetric pair sum in double-single arithmetic: every value is an
// unevaluated sum hi + lo of two FP32 numbers (about 44 significant bits), built
// from the error-free transformations of Dekker (1971) and Knuth (TAOCP vol. 2):
// two_sum (6 adds), fast_two_sum (3), two_prod via FMA (2). The intrinsics
// __fadd_rn/__fsub_rn/__fmul_rn/__fmaf_rn keep the compiler from contracting
// these sequences. 1/|d| is one Newton step from the MUFU seed. Each unordered
// pair (both orders) costs about 190 FP32 instructions against 20 FP64
// instructions in k_pair64_sym, i.e. about 7x less issue time on a part whose
// FP32:FP64 rate is 64:1, at ~1e-13 relative accuracy per term; momentum stays
// exact to the accumulation round-off because each pair's term is computed once
// and added with both signs. Used for the FP64 stage of the mixed precision form.
struct dsf {
    float h, l;
};

__device__ __forceinline__ dsf ds_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ dsf ds_fast(float a, float b) {
    float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dsf ds_add(dsf a, dsf b) {
    dsf s = ds_two_sum(a.h, b.h);
    return ds_fast(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dsf ds_sub(dsf a, dsf b) { return ds_add(a, {-b.h, -b.l}); }
__device__ __forceinline__ dsf ds_mul(dsf a, dsf b) {
    float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ds_fast(p, e);
}
// Unnormalised double-single values: an intermediate that only feeds a
// product or a sum is kept as an exact pair (h, l) whose l may exceed
// ulp(h)/2 by a few ulps; the value h + l carries the same ~2^-44 accuracy,
// and skipping the renormalising fast_two_sum saves 3 instructions each time.
// The products drop the l*l term, so a factor whose l can be large relative to
// h (a difference of nearly equal inputs) is renormalised first.
__device__ __forceinline__ dsf ds_mul_u(dsf a, dsf b) {   // a b, unnormalised
    float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return {p, e};
}
__device__ __forceinline__ dsf ds_sqr_u(dsf a) {          // a^2, unnormalised
    float p = __fmul_rn(a.h, a.h);
    float e = __fmaf_rn(a.h, a.h, -p);
    e = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e);
    return {p, e};
}
__device__ __forceinline__ dsf ds_add_u(dsf a, dsf b) {   // a + b, unnormalised
    dsf s = ds_two_sum(a.h, b.h);
    return {s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l))};
}
__device__ __forceinline__ dsf ds_norm(dsf a) { return ds_fast(a.h, a.l); }
// acc += x with acc kept unnormalised (renormalised by the caller every 32 terms)
__device__ __forceinline__ void ds_acc(dsf &acc, dsf x) {
    dsf s = ds_two_sum(acc.h, x.h);
    acc.h = s.h;
    acc.l = __fadd_rn(acc.l, __fadd_rn(x.l, s.l));
}

// Pair term of the symmetric sum in double-single. In two dimensions the
// projection of g = G_a - G_g off d = x_g - x_a is
//   g - d (d.g)/|d|^2 = c (d2, -d1) / |d|^2,   c = g1 d2 - g2 d1,
// so u = U(d) g / |d| = s (d2, -d1) with s = c / |d|^3 (the same term as
// functions.jl:221-231 in exact arithmetic; c carries the cancellation that
// g - d (d.g)/|d|^2 carries when g is nearly parallel to d). Returns d1, d2 and
// s (0 for |d|^2 < 1e-24). The target gets w_a s (d2, -d1), the source the
// same with -w_g.
__device__ __forceinline__ void pair_s_ds(const float4 &xg, const float4 &Gg, const float4 &xa,
                                          const float4 &Ga, dsf &d1, dsf &d2, dsf &s) {
    // differences are renormalised: for close markers the heads cancel exactly
    // and the tail difference would otherwise be a large l (the products drop l*l)
    d1 = ds_norm(ds_add_u({xg.x, xg.z}, {-xa.x, -xa.z}));
    d2 = ds_norm(ds_add_u({xg.y, xg.w}, {-xa.y, -xa.w}));
    dsf r2 = ds_add_u(ds_sqr_u(d1), ds_sqr_u(d2));
    const bool ok = r2.h >= 1e-24f;
    if (!ok) r2 = {1.f, 0.f};
    // 1/|d|^3 from the MUFU seed y0 ~ 1/sqrt(r2): with e = 1 - r2 y0^2 (~1e-7),
    // 1/|d|^3 = y0^3 (1 - e)^{-3/2} = y0^3 (1 + 3e/2 + 15e^2/8 + O(e^3)). y0^2
    // and y0^3 are formed as exact double-single products and e from them, so
    // the result carries ~1e-14 relative error, as a Newton step on y0 followed
    // by double-single cubing does, in 18 instructions instead of 25.
    const float y0 = rsqrtf(r2.h);
    const float p2 = __fmul_rn(y0, y0);
    const float e2 = __fmaf_rn(y0, y0, -p2);       // y0^2 = p2 + e2 exactly
    float q = __fmul_rn(r2.h, p2);
    float qe = __fmaf_rn(r2.h, p2, -q);
    qe = __fmaf_rn(r2.h, e2, qe);
    qe = __fmaf_rn(r2.l, p2, qe);                  // r2 y0^2 = q + qe
    const float e = __fsub_rn(__fsub_rn(1.0f, q), qe);
    const float p3 = __fmul_rn(p2, y0);
    float e3 = __fmaf_rn(p2, y0, -p3);
    e3 = __fmaf_rn(e2, y0, e3);                    // y0^3 = p3 + e3
    const float corr = __fmul_rn(e, __fmaf_rn(1.875f, e, 1.5f));
    const dsf y3 = {p3, __fmaf_rn(p3, corr, e3)};
    const dsf g1 = ds_norm(ds_add_u({Ga.x, Ga.z}, {-Gg.x, -Gg.z}));
    const dsf g2 = ds_norm(ds_add_u({Ga.y, Ga.w}, {-Gg.y, -Gg.w}));
    const dsf m2 = ds_mul_u(g2, d1);
    const dsf c = ds_norm(ds_add_u(ds_mul_u(g1, d2), {-m2.h, -m2.l}));
    s = ds_mul_u(c, y3);
    if (!ok) s = {0.f, 0.f};
}

// Tile pairs whose 2 x 128 markers all carry one weight w0 (the common case:
// equal-weight markers) take the unweighted loop: the terms s (d2, -d1) are
// summed without the per-pair weight products and w0 multiplies the FP64 fold
// (16 of ~190 instructions per pair saved). A block vote on the loaded tile
// decides per tile pair; padding (weight 0) and unequal weights take the
// weighted loop.
__global__ void __launch_bounds__(ST)
k_pair_ds_sym(const float4 *__restrict__ pfx, const float4 *__restrict__ pfg,
              const float *__restrict__ pfw, const float *__restrict__ pfwl, int nt, int H,
              int KC, double *__restrict__ gpart, double *__restrict__ apart) {
    __shared__ float4 sx[ST], sg[ST];
    __shared__ float2 sw[ST];
    __shared__ float4 sacc[ST];  // {a1.h, a1.l, a2.h, a2.l}
    const int I = blockIdx.x % nt, chunk = blockIdx.x / nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float4 xg = pfx[I * ST + tid], Gg = pfg[I * ST + tid];
    const dsf wg = {pfw[I * ST + tid], pfwl[I * ST + tid]};
    const float2 w0 = make_float2(pfw[I * ST], pfwl[I * ST]);
    const double w0d = (double)w0.x + (double)w0.y;
    const bool own_same = wg.h == w0.x && wg.l == w0.y && w0.x != 0.f;
    dsf ga1 = {0.f, 0.f}, ga2 = {0.f, 0.f};
    double gd1 = 0.0, gd2 = 0.0;
    const int k0 = chunk * KC, k1 = min(H + 1, k0 + KC);
    for (int k = k0; k < k1; k++) {
        if (sym_skip(nt, H, I, k)) continue;
        const int J = (I + k) % nt;
        __syncthreads();
        sx[tid] = pfx[J * ST + tid];
        sg[tid] = pfg[J * ST + tid];
        const float2 wa = make_float2(pfw[J * ST + tid], pfwl[J * ST + tid]);
        sw[tid] = wa;
        sacc[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
        const bool uni =
            __syncthreads_and(own_same && wa.x == w0.x && wa.y == w0.y) != 0;
        if (k == 0) {
            if (uni) {
                for (int a = 0; a < ST; a++) {
                    dsf d1, d2, sp;
                    pair_s_ds(xg, Gg, sx[a], sg[a], d1, d2, sp);
                    const dsf t2 = ds_mul_u(sp, d1);
                    ds_acc(ga1, ds_mul_u(sp, d2));
                    ds_acc(ga2, {-t2.h, -t2.l});
                    if ((a & 31) == 31) {
                        ga1 = ds_norm(ga1);
                        ga2 = ds_norm(ga2);
                    }
                }
            } else {
                for (int a = 0; a < ST; a++) {
                    dsf d1, d2, sp;
                    pair_s_ds(xg, Gg, sx[a], sg[a], d1, d2, sp);
                    const dsf ws = ds_mul_u({sw[a].x, sw[a].y}, sp);
                    ds_acc(ga1, ds_mul_u(ws, d2));
                    ds_acc(ga2, ds_mul_u(ws, {-d1.h, -d1.l}));
                    if ((a & 31) == 31) {
                        ga1 = ds_norm(ga1);
                        ga2 = ds_norm(ga2);
                    }
                }
            }
        } else {
            for (int r = 0; r < 4; r++) {
                const int base = ((warp + r) & 3) * 32;
                float4 a0 = sacc[base + lane];
                dsf a1 = {a0.x, a0.y}, a2 = {a0.z, a0.w};
                if (uni) {
                    // target += s (d2, -d1); source accumulates the same terms,
                    // its factor -w0 applied at the write-out
#pragma unroll 2
                    for (int q = 0; q < 32; q++) {
                        const int ai = base + ((lane + q) & 31);
                        dsf d1, d2, sp;
                        pair_s_ds(xg, Gg, sx[ai], sg[ai], d1, d2, sp);
                        const dsf t1 = ds_mul_u(sp, d2);
                        const dsf t2 = ds_mul_u(sp, d1);
                        const dsf nt2 = {-t2.h, -t2.l};
                        ds_acc(ga1, t1);
                        ds_acc(ga2, nt2);
                        ds_acc(a1, t1);
                        ds_acc(a2, nt2);
                        const int src = (lane + 1) & 31;
                        a1.h = __shfl_sync(0xffffffffu, a1.h, src);
                        a1.l = __shfl_sync(0xffffffffu, a1.l, src);
                        a2.h = __shfl_sync(0xffffffffu, a2.h, src);
                        a2.l = __shfl_sync(0xffffffffu, a2.l, src);
                    }
                } else {
#pragma unroll 2
                    for (int q = 0; q < 32; q++) {
                        const int ai = base + ((lane + q) & 31);
                        dsf d1, d2, sp;
                        pair_s_ds(xg, Gg, sx[ai], sg[ai], d1, d2, sp);
                        const dsf ws = ds_mul_u({sw[ai].x, sw[ai].y}, sp);   // w_a s
                        const dsf wn = ds_mul_u({-wg.h, -wg.l}, sp);         // -w_g s
                        const dsf nd1 = {-d1.h, -d1.l};
                        ds_acc(ga1, ds_mul_u(ws, d2));
                        ds_acc(ga2, ds_mul_u(ws, nd1));
                        ds_acc(a1, ds_mul_u(wn, d2));
                        ds_acc(a2, ds_mul_u(wn, nd1));
                        const int src = (lane + 1) & 31;
                        a1.h = __shfl_sync(0xffffffffu, a1.h, src);
                        a1.l = __shfl_sync(0xffffffffu, a1.l, src);
                        a2.h = __shfl_sync(0xffffffffu, a2.h, src);
                        a2.l = __shfl_sync(0xffffffffu, a2.l, src);
                    }
                }
                a1 = ds_norm(a1);
                a2 = ds_norm(a2);
                ga1 = ds_norm(ga1);
                ga2 = ds_norm(ga2);
                sacc[base + lane] = make_float4(a1.h, a1.l, a2.h, a2.l);
                __syncthreads();
            }
            double *ap = apart + ((size_t)(k - 1) * nt + J) * 2 * ST;
            float4 v = sacc[tid];
            const double sf = uni ? -w0d : 1.0;
            ap[tid] = sf * ((double)v.x + (double)v.y);
            ap[ST + tid] = sf * ((double)v.z + (double)v.w);
        }
        // fold the tile pair's target-side double-single sum into FP64
        const double tf = uni ? w0d : 1.0;
        gd1 += tf * ((double)ga1.h + (double)ga1.l);
        gd2 += tf * ((double)ga2.h + (double)ga2.l);
        ga1 = {0.f, 0.f};
        ga2 = {0.f, 0.f};
    }
    double *gp = gpart + ((size_t)chunk * nt + I) * 2 * ST;
    gp[tid] = gd1;
    gp[ST + tid] = gd2;
}

// Symmetric FP32 metric: U(d) = (I - d d^T/|d|^2)/|d| is even in d, so one
// evaluation adds w_a U to A_g and w_g U to A_a (same tiling and rotation as
// k_pair32_sym; head+tail differences). Partials: 3 components.
__device__ __forceinline__ void metric_u32(const float4 &xg, const float4 &xa, float &u11,
                                           float &u12, float &u22) {
    float d1 = (xg.x - xa.x) + (xg.z - xa.z);
    float d2 = (xg.y - xa.y) + (xg.w - xa.w);
    float q11 = d1 * d1, q22 = d2 * d2;
    float r2 = q11 + q22;
    float y = rsqrtf(r2);
    y = r2 >= 1e-24f ? y : 0.0f;
    float y2 = y * y;
    u11 = y * fmaf(-q11, y2, 1.f);
    u12 = -y * (d1 * d2 * y2);
    u22 = y * fmaf(-q22, y2, 1.f);
}

__global__ void __launch_bounds__(ST)
k_metric32_sym(const float4 *__restrict__ pfx, const float *__restrict__ pfw, int nt, int H,
               int KC, double *__restrict__ gpart, float *__restrict__ apart) {
    __shared__ float4 sx[ST];
    __shared__ float sw[ST];
    __shared__ float4 sacc[ST];
    const int I = blockIdx.x % nt, chunk = blockIdx.x / nt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float4 xg = pfx[I * ST + tid];
    const float wg = pfw[I * ST + tid];
    double g11 = 0.0, g12 = 0.0, g22 = 0.0;
    const int k0 = chunk * KC, k1 = min(H + 1, k0 + KC);
    for (int k = k0; k < k1; k++) {
        if (sym_skip(nt, H, I, k)) continue;
        const int J = (I + k) % nt;
        __syncthreads();
        sx[tid] = pfx[J * ST + tid];
        sw[tid] = pfw[J * ST + tid];
        sacc[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
        __syncthreads();
        float t11 = 0.f, t12 = 0.f, t22 = 0.f;
        if (k == 0) {
#pragma unroll 8
            for (int a = 0; a < ST; a++) {
                float u11, u12, u22;
                metric_u32(xg, sx[a], u11, u12, u22);
                t11 = fmaf(sw[a], u11, t11);
                t12 = fmaf(sw[a], u12, t12);
                t22 = fmaf(sw[a], u22, t22);
            }
        } else {
            for (int r = 0; r < 4; r++) {
                const int base = ((warp + r) & 3) * 32;
                float4 a0 = sacc[base + lane];
                float a11 = a0.x, a12 = a0.y, a22 = a0.z;
#pragma unroll 8
                for (int q = 0; q < 32; q++) {
                    const int ai = base + ((lane + q) & 31);
                    float u11, u12, u22;
                    metric_u32(xg, sx[ai], u11, u12, u22);
                    const float wa = sw[ai];
                    t11 = fmaf(wa, u11, t11);
                    t12 = fmaf(wa, u12, t12);
                    t22 = fmaf(wa, u22, t22);
                    a11 = fmaf(wg, u11, a11);
                    a12 = fmaf(wg, u12, a12);
                    a22 = fmaf(wg, u22, a22);
                    const int src = (lane + 1) & 31;
                    a11 = __shfl_sync(0xffffffffu, a11, src);
                    a12 = __shfl_sync(0xffffffffu, a12, src);
                    a22 = __shfl_sync(0xffffffffu, a22, src);
                }
                sacc[base + lane] = make_float4(a11, a12, a22, 0.f);
                __syncthreads();
            }
            float *ap = apart + ((size_t)(k - 1) * nt + J) * 3 * ST;
            float4 v = sacc[tid];
            ap[tid] = v.x;
            ap[ST + tid] = v.y;
            ap[2 * ST + tid] = v.z;
        }
        g11 += (double)t11;
        g12 += (double)t12;
        g22 += (double)t22;
    }
    double *gp = gpart + ((size_t)chunk * nt + I) * 3 * ST;
    gp[tid] = g11;
    gp[ST + tid] = g12;
    gp[2 * ST + tid] = g22;
}

__global__ void k_metric_reduce(const double *__restrict__ gpart, const float *__restrict__ apart,
                                int nt, int H, int nchunk, double *__restrict__ dst, size_t ld) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nt * ST) return;
    int K = p / ST, t = p - K * ST;
    double s[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < nchunk; c++) {
        const double *gp = gpart + ((size_t)c * nt + K) * 3 * ST;
        for (int q = 0; q < 3; q++) s[q] += gp[q * ST + t];
    }
    for (int k = 1; k <= H; k++) {
        int I = (K - k + nt) % nt;
        if (sym_skip(nt, H, I, k)) continue;
        const float *ap = apart + ((size_t)(k - 1) * nt + K) * 3 * ST;
        for (int q = 0; q < 3; q++) s[q] += (double)ap[q * ST + t];
    }
    for (int q = 0; q < 3; q++) dst[(size_t)q * ld + p] = s[q];
}

// vdot[p] = sum over chunks of the target-side partials + sum over k of the
// source-side partials, in that fixed order
template <typename TA>
__global__ void k_sym_reduce(const double *__restrict__ gpart, const TA *__restrict__ apart,
                             int nt, int H, int nchunk, int TS, double *__restrict__ dst,
                             size_t ld) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nt * TS) return;
    int K = p / TS, t = p - K * TS;
    double s1 = 0.0, s2 = 0.0;
    for (int c = 0; c < nchunk; c++) {
        const double *gp = gpart + ((size_t)c * nt + K) * 2 * TS;
        s1 += gp[t];
        s2 += gp[TS + t];
    }
    for (int k = 1; k <= H; k++) {
        int I = (K - k + nt) % nt;
        if (sym_skip(nt, H, I, k)) continue;
        const TA *ap = apart + ((size_t)(k - 1) * nt + K) * 2 * TS;
        s1 += (double)ap[t];
        s2 += (double)ap[TS + t];
    }
    dst[p] = s1;
    dst[ld + p] = s2;
}

// sum the slice partials of components [c0, c0+nc) in slice order into
// dst (nc x ld); the partials hold ncomp components per slice
__global__ void k_slice_reduce(const double *__restrict__ part, int split, int ncomp, int c0,
                               int nc, size_t ld, const int *__restrict__ Mp,
                               double *__restrict__ dst) {
    int M = *Mp;
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= M) return;
    for (int c = 0; c < nc; c++) {
        double s = 0.0;
        for (int sl = 0; sl < split; sl++) s += part[((size_t)sl * ncomp + c0 + c) * ld + g];
        dst[(size_t)c * ld + g] = s;
    }
}

// Landau pack: lambda from the device state, G_eff = -(dS + lambda dv)/w
// (solver.jl:107-111), operands in sorted order.
__global__ void k_pack_landau(const int *__restrict__ perm, const int *__restrict__ Mp, int Mpad, int N,
                              const double *__restrict__ vmid, const double *__restrict__ dS,
                              const double *__restrict__ dv, const double *__restrict__ w,
                              const co_solver_state *__restrict__ st, int use_lambda,
                              int mode, double2 *__restrict__ px, double2 *__restrict__ pg,
                              double *__restrict__ pw, float4 *__restrict__ pfx,
                              float4 *__restrict__ pfg, float *__restrict__ pfw, float *__restrict__ pfwl) {
    int M = *Mp;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Mpad) return;
    if (p >= M) {  // inert padding up to the tile boundary: far away, zero weight
        if (mode & 2) {
            pfx[p] = make_float4(1e3f, 1e3f, 0.f, 0.f);
            pfg[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            pfw[p] = 0.f;
            pfwl[p] = 0.f;
        }
        if (mode & 1) {
            px[p] = make_double2(1e3, 1e3);
            pg[p] = make_double2(0.0, 0.0);
            pw[p] = 0.0;
        }
        return;
    }
    int a = perm[p];
    double lam = use_lambda ? st->lambda : 0.0;
    double iw = 1.0 / w[a];
    double x1 = vmid[a], x2 = vmid[N + a];
    double G1 = -(dS[a] + lam * dv[a]) * iw;
    double G2 = -(dS[N + a] + lam * dv[N + a]) * iw;
    if (mode & 2) {
        float x1h = (float)x1, x2h = (float)x2, G1h = (float)G1, G2h = (float)G2;
        pfx[p] = make_float4(x1h, x2h, (float)(x1 - (double)x1h), (float)(x2 - (double)x2h));
        pfg[p] = make_float4(G1h, G2h, (float)(G1 - (double)G1h), (float)(G2 - (double)G2h));
        float wh = (float)w[a];
        pfw[p] = wh;
        pfwl[p] = (float)(w[a] - (double)wh);
    }
    if (mode & 1) {
        px[p] = make_double2(x1, x2);
        pg[p] = make_double2(G1, G2);
        pw[p] = w[a];
    }
}

// Hook pack: operands straight from (v, G, w) (COLLISION_FN semantics).
__global__ void k_pack_plain(const int *__restrict__ perm, const int *__restrict__ Mp, int Mpad, int N,
                             const double *__restrict__ v, const double *__restrict__ G,
                             const double *__restrict__ w, int mode,
                             double2 *__restrict__ px, double2 *__restrict__ pg,
                             double *__restrict__ pw, float4 *__restrict__ pfx,
                             float4 *__restrict__ pfg, float *__restrict__ pfw, float *__restrict__ pfwl) {
    int M = *Mp;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Mpad) return;
    if (p >= M) {  // inert padding up to the tile boundary: far away, zero weight
        if (mode & 2) {
            pfx[p] = make_float4(1e3f, 1e3f, 0.f, 0.f);
            pfg[p] = make_float4(0.f, 0.f, 0.f, 0.f);
            pfw[p] = 0.f;
            pfwl[p] = 0.f;
        }
        if (mode & 1) {
            px[p] = make_double2(1e3, 1e3);
            pg[p] = make_double2(0.0, 0.0);
            pw[p] = 0.0;
        }
        return;
    }
    int a = perm[p];
    double x1 = v[a], x2 = v[N + a], G1 = G[a], G2 = G[N + a];
    if (mode & 2) {
        float x1h = (float)x1, x2h = (float)x2, G1h = (float)G1, G2h = (float)G2;
        pfx[p] = make_float4(x1h, x2h, (float)(x1 - (double)x1h), (float)(x2 - (double)x2h));
        pfg[p] = make_float4(G1h, G2h, (float)(G1 - (double)G1h), (float)(G2 - (double)G2h));
        float wh = (float)w[a];
        pfw[p] = wh;
        pfwl[p] = (float)(w[a] - (double)wh);
    }
    if (mode & 1) {
        px[p] = make_double2(x1, x2);
        pg[p] = make_double2(G1, G2);
        pw[p] = w[a];
    }
}

// Gv = v0 + dt * vdot (solver.jl:225), vdot unpacked from sorted order (0 for
// out-of-domain markers); optionally r = Gv - v1 and block partials of |r|^2,
// |v1|^2 for step_anderson! (solver.jl:339-349).
__global__ void __launch_bounds__(CO_RED_THREADS)
k_unpack_update(const int *__restrict__ inv, int N, const double *__restrict__ pdot, size_t ld,
                double dt, const double *__restrict__ v0, double *__restrict__ Gv,
                double *__restrict__ dotv, const double *__restrict__ v1, double *__restrict__ r,
                double *__restrict__ red) {
    __shared__ double sh[32];
    double sr = 0.0, sv = 0.0;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
        int p = inv[a];
        double q1 = 0.0, q2 = 0.0;
        if (p >= 0) {
            q1 = pdot[p];
            q2 = pdot[ld + p];
        }
        if (dotv) {
            dotv[a] = q1;
            dotv[N + a] = q2;
        }
        if (Gv) {
            double g1 = v0[a] + dt * q1, g2 = v0[N + a] + dt * q2;
            Gv[a] = g1;
            Gv[N + a] = g2;
            if (r) {
                double x1 = v1[a], x2 = v1[N + a];
                double r1 = g1 - x1, r2 = g2 - x2;
                r[a] = r1;
                r[N + a] = r2;
                sr += r1 * r1 + r2 * r2;
                sv += x1 * x1 + x2 * x2;
            }
        }
    }
    if (red) {
        double a = co_block_sum(sr, sh);
        double b = co_block_sum(sv, sh);
        if (threadIdx.x == 0) {
            red[blockIdx.x * 2 + 0] = a;
            red[blockIdx.x * 2 + 1] = b;
        }
    }
}

// unpack A (3 comps) for COLLMETRIC_FN
__global__ void k_unpack_A(const int *__restrict__ inv, int N, const double *__restrict__ pA,
                           size_t ld, double *__restrict__ A) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    int p = inv[a];
    for (int c = 0; c < 3; c++) A[(size_t)c * N + a] = p >= 0 ? pA[(size_t)c * ld + p] : 0.0;
}

// ------------------------------------------------------------------ host

static int choose_split(co_ctx *c, int M, int tpb, int force) {
    if (force > 0) return force;
    int tiles = co_cdiv(M, tpb);
    if (tiles < 1) tiles = 1;
    int want = co_cdiv(4LL * c->nsm, tiles);
    int max_split = co_cdiv(M, 256);
    if (max_split < 1) max_split = 1;
    if (want > max_split) want = max_split;
    if (want < 1) want = 1;
    return want;
}

static int ensure_part(co_ctx *c, size_t n) {
    if (n <= c->mb.part_cap) return CO_OK;
    if (c->mb.part) cudaFree(c->mb.part);
    c->mb.part = nullptr;
    if (cudaMalloc(&c->mb.part, n * sizeof(double)) != cudaSuccess) return CO_ERR_NOMEM;
    c->mb.part_cap = n;
    return CO_OK;
}

// M is an upper bound (N); the true count sits at cstart[n_el] on the device.
static int pair_sym(co_ctx *c, int Mub, int fp64);

int co_pair_fp64(co_ctx *c, int Mub, int with_metric) {
    if (Mub <= 0) return CO_OK;
    if (!with_metric && c->pair_symmetric && co_cdiv(Mub, ST) >= 4) return pair_sym(c, Mub, 1);
    const int *Mp = c->mb.cstart + c->n_el;
    size_t ld = (size_t)c->mb.cap;
    int split = choose_split(c, Mub, PAIR_TPB, c->pair_split_fp64);
    int slice = co_cdiv(Mub, split);
    slice = co_cdiv(slice, PAIR_TPB) * PAIR_TPB;
    split = co_cdiv(Mub, slice);
    int nc = with_metric ? 5 : 2;
    dim3 grid(co_cdiv(Mub, PAIR_TPB), split);
    double *dst = c->mb.pdot;
    if (split > 1 || with_metric) {
        int rc = ensure_part(c, (size_t)split * nc * ld);
        if (rc) return rc;
        dst = c->mb.part;
    }
    co_prof_begin(c, 1);
    if (with_metric)
        k_pair64<true><<<grid, PAIR_TPB, 0, c->stream>>>(c->mb.px, c->mb.pg, c->mb.pw, Mp, slice,
                                                         dst, ld);
    else
        k_pair64<false><<<grid, PAIR_TPB, 0, c->stream>>>(c->mb.px, c->mb.pg, c->mb.pw, Mp, slice,
                                                          dst, ld);
    co_prof_end(c);
    c->launches++;
    if (with_metric) {
        // components 0,1 -> pdot ; 2,3,4 -> pA
        k_slice_reduce<<<co_cdiv(Mub, 256), 256, 0, c->stream>>>(dst, split, 5, 0, 2, ld, Mp,
                                                                c->mb.pdot);
        k_slice_reduce<<<co_cdiv(Mub, 256), 256, 0, c->stream>>>(dst, split, 5, 2, 3, ld, Mp,
                                                                c->mb.pA);
        c->launches += 2;
    } else if (split > 1) {
        k_slice_reduce<<<co_cdiv(Mub, 256), 256, 0, c->stream>>>(dst, split, 2, 0, 2, ld, Mp,
                                                                c->mb.pdot);
        c->launches++;
    }
    CO_CK(cudaGetLastError());
    return CO_OK;
}

#define SYM_KC 8

// symmetric pair sum on the padded operands (Mpad = nt * ST);
// kind: 0 FP32, 1 FP64, 2 double-single
static int pair_sym(co_ctx *c, int Mub, int kind) {
    const int fp64 = kind != 0;  // partials of the source side in double
    int nt = co_cdiv(Mub, ST);
    int H = nt / 2;
    int KC = SYM_KC;
    int nchunk = co_cdiv(H + 1, KC);
    size_t gsz = (size_t)nchunk * nt * 2 * ST;               // doubles
    size_t asz = (size_t)(H > 0 ? H : 1) * nt * 2 * ST;      // doubles (fp64) / floats (fp32)
    size_t need = gsz + (fp64 ? asz : (asz + 1) / 2);
    if (!fp64) {   // the FP32 kernel's 256-marker tiles
        const int nt2 = co_cdiv(Mub, 2 * ST), H2 = nt2 / 2, nchunk2 = co_cdiv(H2 + 1, KC);
        const size_t g2 = (size_t)nchunk2 * nt2 * 4 * ST;
        const size_t a2 = (size_t)(H2 > 0 ? H2 : 1) * nt2 * 4 * ST;
        need = g2 + (a2 + 1) / 2;
    }
    int rc = ensure_part(c, need);
    if (rc) return rc;
    double *gpart = c->mb.part;
    co_prof_begin(c, kind == 1 ? 1 : (kind == 2 ? 2 : 0));
    if (kind == 2) {
        double *apart = c->mb.part + gsz;
        k_pair_ds_sym<<<nt * nchunk, ST, 0, c->stream>>>(c->mb.pf_x, c->mb.pf_g, c->mb.pf_w,
                                                         c->mb.pf_wl, nt, H, KC, gpart, apart);
        co_prof_end(c);
        k_sym_reduce<double><<<co_cdiv((long long)nt * ST, 256), 256, 0, c->stream>>>(
            gpart, apart, nt, H, nchunk, ST, c->mb.pdot, (size_t)c->mb.cap);
    } else if (fp64) {
        double *apart = c->mb.part + gsz;
        k_pair64_sym<<<nt * nchunk, ST, 0, c->stream>>>(c->mb.px, c->mb.pg, c->mb.pw, nt, H, KC,
                                                        gpart, apart);
        co_prof_end(c);
        k_sym_reduce<double><<<co_cdiv((long long)nt * ST, 256), 256, 0, c->stream>>>(
            gpart, apart, nt, H, nchunk, ST, c->mb.pdot, (size_t)c->mb.cap);
    } else {
        // FP32: two targets per thread on 256-marker tiles (Mpad is a multiple of
        // 256 and the tile count has been checked by the caller)
        constexpr int R32 = 2, TS32 = R32 * ST;
        const int nt2 = co_cdiv(Mub, TS32), H2 = nt2 / 2, nchunk2 = co_cdiv(H2 + 1, KC);
        const size_t gsz2 = (size_t)nchunk2 * nt2 * 2 * TS32;
        float *apart = (float *)(c->mb.part + gsz2);
        k_pair32_sym<R32><<<nt2 * nchunk2, ST, 0, c->stream>>>(c->mb.pf_x, c->mb.pf_g,
                                                               c->mb.pf_w, nt2, H2, KC,
                                                               gpart, apart);
        co_prof_end(c);
        k_sym_reduce<float><<<co_cdiv((long long)nt2 * TS32, 256), 256, 0, c->stream>>>(
            gpart, apart, nt2, H2, nchunk2, TS32, c->mb.pdot, (size_t)c->mb.cap);
    }
    c->launches += 2;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_pair_fp32(co_ctx *c, int Mub) {
    if (Mub <= 0) return CO_OK;
    if (c->pair_symmetric && co_cdiv(Mub, 2 * ST) >= 4) return pair_sym(c, Mub, 0);
    if (Mub <= 0) return CO_OK;
    const int *Mp = c->mb.cstart + c->n_el;
    size_t ld = (size_t)c->mb.cap;
    int split = choose_split(c, Mub, PAIR_TPB, c->pair_split_fp32);
    int slice = co_cdiv(Mub, split);
    slice = co_cdiv(slice, PAIR32_TILE) * PAIR32_TILE;
    split = co_cdiv(Mub, slice);
    dim3 grid(co_cdiv(Mub, PAIR_TPB), split);
    double *dst = c->mb.pdot;
    if (split > 1) {
        int rc = ensure_part(c, (size_t)split * 2 * ld);
        if (rc) return rc;
        dst = c->mb.part;
    }
    co_prof_begin(c, 0);
    k_pair32<<<grid, PAIR_TPB, 0, c->stream>>>(c->mb.pf_x, c->mb.pf_g, c->mb.pf_w, Mp, slice, dst,
                                               ld);
    co_prof_end(c);
    c->launches++;
    if (split > 1) {
        k_slice_reduce<<<co_cdiv(Mub, 256), 256, 0, c->stream>>>(dst, split, 2, 0, 2, ld, Mp,
                                                                c->mb.pdot);
        c->launches++;
    }
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_pack_plain(co_ctx *c, int N, int Mub, int precision, const double *x, const double *G) {
    if (Mub <= 0) return CO_OK;
    const int *Mp = c->mb.cstart + c->n_el;
    co_bufs &b = c->mb;
    int Mpad = co_cdiv(Mub, 256) * 256;  // whole tiles of up to 256 markers
    k_pack_plain<<<co_cdiv(Mpad, 256), 256, 0, c->stream>>>(b.perm, Mp, Mpad, N, x, G, b.w,
                                                            co_pack_mode(precision), b.px, b.pg,
                                                            b.pw, b.pf_x, b.pf_g, b.pf_w, b.pf_wl);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_pack_landau(co_ctx *c, int N, int Mub, int precision, int gonzalez) {
    if (Mub <= 0) return CO_OK;
    const int *Mp = c->mb.cstart + c->n_el;
    co_bufs &b = c->mb;
    int Mpad = co_cdiv(Mub, 256) * 256;  // whole tiles of up to 256 markers
    k_pack_landau<<<co_cdiv(Mpad, 256), 256, 0, c->stream>>>(
        b.perm, Mp, Mpad, N, b.vmid, b.dS, b.dv, b.w, c->st, gonzalez, co_pack_mode(precision),
        b.px, b.pg, b.pw, b.pf_x, b.pf_g, b.pf_w, b.pf_wl);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_unpack_update(co_ctx *c, int N, double dt, double *Gv, const double *v0,
                     const double *v1, double *r, double *red) {
    if (N == 0) return CO_OK;
    int g = co_cdiv(N, CO_RED_THREADS);
    if (g > c->mb.red_cap) g = c->mb.red_cap;
    k_unpack_update<<<g, CO_RED_THREADS, 0, c->stream>>>(c->mb.inv, N, c->mb.pdot,
                                                         (size_t)c->mb.cap, dt, v0, Gv,
                                                         c->mb.dotv, v1, r, red);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_unpack_A(co_ctx *c, int N, double *A) {
    if (N == 0) return CO_OK;
    k_unpack_A<<<co_cdiv(N, 256), 256, 0, c->stream>>>(c->mb.inv, N, c->mb.pA, (size_t)c->mb.cap,
                                                       A);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

int co_metric32(co_ctx *c, int Mub) {
    if (Mub <= 0) return CO_OK;
    if (c->pair_symmetric && co_cdiv(Mub, ST) >= 4) {
        int nt = co_cdiv(Mub, ST), H = nt / 2, KC = SYM_KC, nchunk = co_cdiv(H + 1, KC);
        size_t gsz = (size_t)nchunk * nt * 3 * ST;
        size_t asz = (size_t)(H > 0 ? H : 1) * nt * 3 * ST;  // floats
        int rc = ensure_part(c, gsz + (asz + 1) / 2);
        if (rc) return rc;
        float *apart = (float *)(c->mb.part + gsz);
        k_metric32_sym<<<nt * nchunk, ST, 0, c->stream>>>(c->mb.pf_x, c->mb.pf_w, nt, H, KC,
                                                          c->mb.part, apart);
        k_metric_reduce<<<co_cdiv((long long)nt * ST, 256), 256, 0, c->stream>>>(
            c->mb.part, apart, nt, H, nchunk, c->mb.pA, (size_t)c->mb.cap);
        c->launches += 2;
        CO_CK(cudaGetLastError());
        return CO_OK;
    }
    const int *Mp = c->mb.cstart + c->n_el;
    k_metric32<<<co_cdiv(Mub, PAIR_TPB), PAIR_TPB, 0, c->stream>>>(c->mb.pf_x, c->mb.pf_w, Mp,
                                                                   c->mb.pA, (size_t)c->mb.cap);
    c->launches++;
    CO_CK(cudaGetLastError());
    return CO_OK;
}

// FP64-equivalent pair sum in double-single arithmetic (symmetric kernel);
// falls back to the FP64 kernel below 4 tiles
int co_pair_ds(co_ctx *c, int Mub) {
    if (Mub <= 0) return CO_OK;
    if (co_cdiv(Mub, ST) >= 4) return pair_sym(c, Mub, 2);
    return co_pair_fp64(c, Mub, 0);
}

// ================================================================== batched
//
// Many independent ensembles in one persistent launch: the work items of all
// Landau instances -- (instance, tile I, chunk of k) as in k_pair64_sym, with a
// tile of T = 32 W markers -- are handed out through an atomic counter, so the
// grid size and the tile shape are free parameters (chosen by the autotuner of
// the batch engine). Items of instances whose solve has finished are skipped.
// Every item writes its own partial slots, so the result does not depend on
// which block ran which item.
template <int W>
__global__ void __launch_bounds__(32 * W)
k_pair64_sym_batch(const co_bwork *__restrict__ works, int n_inst, int total, int KC,
                   unsigned *__restrict__ counter) {
    constexpr int T = 32 * W;
    __shared__ double2 sx[T], sg[T];
    __shared__ double sw[T];
    __shared__ double2 sacc[T];
    __shared__ int s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int item = s_item;
        __syncthreads();
        if (item >= total) return;
        int lo = 0, hi = n_inst;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (works[mid].blk0 <= item) lo = mid; else hi = mid;
        }
        const co_bwork wk = works[lo];
        if (wk.st->done) continue;
        const int b = item - wk.blk0;
        const int nt = wk.nt, H = wk.H;
        const int I = b % nt, chunk = b / nt;
        const double2 xg = wk.px[I * T + tid], Gg = wk.pg[I * T + tid];
        const double wg = wk.pw[I * T + tid];
        double ga1 = 0.0, ga2 = 0.0;
        const int k0 = chunk * KC, k1 = min(H + 1, k0 + KC);
        for (int k = k0; k < k1; k++) {
            if (sym_skip(nt, H, I, k)) continue;
            const int J = (I + k) % nt;
            __syncthreads();
            sx[tid] = wk.px[J * T + tid];
            sg[tid] = wk.pg[J * T + tid];
            sw[tid] = wk.pw[J * T + tid];
            sacc[tid] = make_double2(0.0, 0.0);
            __syncthreads();
            if (k == 0) {
#pragma unroll 4
                for (int a = 0; a < T; a++) {
                    double u1, u2;
                    double2 xa = sx[a], Ga = sg[a];
                    pair_u64(xg.x - xa.x, xg.y - xa.y, Ga.x - Gg.x, Ga.y - Gg.y, u1, u2);
                    ga1 = fma(sw[a], u1, ga1);
                    ga2 = fma(sw[a], u2, ga2);
                }
                continue;
            }
            for (int r = 0; r < W; r++) {
                const int base = ((warp + r) % W) * 32;
                double2 a0 = sacc[base + lane];
                double a1 = a0.x, a2 = a0.y;
#pragma unroll 4
                for (int q = 0; q < 32; q++) {
                    const int ai = base + ((lane + q) & 31);
                    double2 xa = sx[ai], Ga = sg[ai];
                    double wa = sw[ai];
                    double u1, u2;
                    pair_u64(xg.x - xa.x, xg.y - xa.y, Ga.x - Gg.x, Ga.y - Gg.y, u1, u2);
                    ga1 = fma(wa, u1, ga1);
                    ga2 = fma(wa, u2, ga2);
                    a1 = fma(-wg, u1, a1);
                    a2 = fma(-wg, u2, a2);
                    a1 = __shfl_sync(0xffffffffu, a1, (lane + 1) & 31);
                    a2 = __shfl_sync(0xffffffffu, a2, (lane + 1) & 31);
                }
                sacc[base + lane] = make_double2(a1, a2);
                __syncthreads();
            }
            double *ap = wk.apart + ((size_t)(k - 1) * nt + J) * 2 * T;
            ap[tid] = sacc[tid].x;
            ap[T + tid] = sacc[tid].y;
        }
        double *gp = wk.gpart + ((size_t)chunk * nt + I) * 2 * T;
        gp[tid] = ga1;
        gp[T + tid] = ga2;
    }
}

// fixed-order reduction of every instance's partials (blockIdx.y = instance)
__global__ void k_sym_reduce_batch(const co_bwork *__restrict__ works, int T) {
    const co_bwork wk = works[blockIdx.y];
    if (wk.st->done) return;
    const int nt = wk.nt, H = wk.H;
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nt * T) return;
    int K = p / T, t = p - K * T;
    double s1 = 0.0, s2 = 0.0;
    for (int c = 0; c < wk.nchunk; c++) {
        const double *gp = wk.gpart + ((size_t)c * nt + K) * 2 * T;
        s1 += gp[t];
        s2 += gp[T + t];
    }
    for (int k = 1; k <= H; k++) {
        int I = (K - k + nt) % nt;
        if (sym_skip(nt, H, I, k)) continue;
        const double *ap = wk.apart + ((size_t)(k - 1) * nt + K) * 2 * T;
        s1 += ap[t];
        s2 += ap[T + t];
    }
    wk.pdot[p] = s1;
    wk.pdot[wk.ld + p] = s2;
}

// Fill the work table of a batch for tile width T = 32 W and chunk KC; makes
// sure every instance's partial buffer is large enough. Returns the number of
// work items.
int co_batch_work_table(co_ctx *const *ctxs, const co_solver_state *const *states, int n,
                        int W, int KC, co_bwork *tab, int *max_pos) {
    const int T = 32 * W;
    int blk = 0, mp = 0;
    for (int i = 0; i < n; i++) {
        co_ctx *c = ctxs[i];
        co_bwork &wk = tab[i];
        int N = c->batch_N;
        int nt = co_cdiv(N, T), H = nt / 2, nchunk = co_cdiv(H + 1, KC);
        size_t gsz = (size_t)nchunk * nt * 2 * T, asz = (size_t)(H > 0 ? H : 1) * nt * 2 * T;
        if (c->batch_landau) {
            int rc = ensure_part(c, gsz + asz);
            if (rc) return -rc;
        }
        wk.px = c->mb.px;
        wk.pg = c->mb.pg;
        wk.pw = c->mb.pw;
        wk.gpart = c->mb.part;
        wk.apart = c->mb.part + gsz;
        wk.pdot = c->mb.pdot;
        wk.ld = (size_t)c->mb.cap;
        wk.st = states[i];
        wk.nt = c->batch_landau ? nt : 0;   // LB instances have no pair sum
        wk.H = H;
        wk.nchunk = nchunk;
        wk.blk0 = blk;
        blk += c->batch_landau ? nt * nchunk : 0;
        if (c->batch_landau && nt * T > mp) mp = nt * T;
    }
    *max_pos = mp;
    return blk;
}

// one batched symmetric FP64 pair sum over all Landau instances
int co_pair64_batch(cudaStream_t s, const co_bwork *d_tab, int n, int total, int W, int KC,
                    int grid, unsigned *d_counter, int max_pos) {
    if (total <= 0) return CO_OK;
    CO_CK(cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s));
    switch (W) {
        case 2: k_pair64_sym_batch<2><<<grid, 64, 0, s>>>(d_tab, n, total, KC, d_counter); break;
        case 4: k_pair64_sym_batch<4><<<grid, 128, 0, s>>>(d_tab, n, total, KC, d_counter); break;
        case 8: k_pair64_sym_batch<8><<<grid, 256, 0, s>>>(d_tab, n, total, KC, d_counter); break;
        default: return CO_ERR_ARG;
    }
    dim3 rg(co_cdiv(max_pos, 256), n);
    k_sym_reduce_batch<<<rg, 256, 0, s>>>(d_tab, 32 * W);
    CO_CK(cudaGetLastError());
    return CO_OK;
}
