// co_noalloc.cu -- the FP64 Landau pair sum (COLLISION_FN semantics,
// functions.jl:205-237) for callers that cannot allocate device memory.
//
// Who needs it: a host that owns all device memory itself -- for example a
// Julia process whose CUDA.jl memory pool manages the GPU, or an application
// that must not allocate between time steps -- cannot create a co_ctx (context
// creation allocates tables and marker buffers). This entry point takes device
// pointers for every input and output and allocates nothing: its only scratch
// (the per-slice partial sums of the split pair loop) is a file-scope
// __device__ array of fixed size, which every GPU that loads the library holds
// until the process exits.
//
// Limits and behaviour:
//   - N <= CO_NOALLOC_MAX_N (32,768 markers); larger N returns CO_ERR_SIZE
//     before any device work.
//   - The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress, with that device current, and caches it; make that
//     first call before any stream capture.
//   - All calls share the one array. Every partial the reduction reads is
//     written earlier in the same call, so leftover contents of a previous call
//     are never read; the one word that must start at zero (the non-finite
//     flag) is cleared by each call. Two calls whose kernels overlap on the GPU
//     (different streams, or different host threads) race on the array and must
//     be serialised by the caller.
//   - Inputs are checked for NaN/Inf first, on the GPU: the call waits for that
//     check (and so for the work queued before it on the caller's stream) and
//     returns CO_ERR_NONFINITE without touching dot_v if one is found, as the
//     context entry points do. The pair sum itself is then enqueued on the
//     caller's stream and not synchronised.
//
// Arithmetic: one-sided FP64 pair loop with the reference's masks (targets
// outside (bp[1], bp[end]) get 0, sources outside are skipped, |d|^2 < 1e-24
// skipped), the same rsqrt refinement as the library's FP64 pair kernel, and a
// fixed-order sum over alpha slices.
#include <mutex>

#include "co_internal.cuh"

#define CO_NOALLOC_MAX_N 32768
#define CO_NOALLOC_SLICES 8
#define NA_TPB 128
#define NA_R2_MIN_BITS 0x3B282DB34012B251LL  // bit pattern of 1e-24

// 8 slices x 2 components x 32768 markers of FP64 = 4 MiB per device, then a
// 256-byte tail whose first word is the non-finite flag of the current call
#define CO_NOALLOC_PART (CO_NOALLOC_SLICES * 2 * CO_NOALLOC_MAX_N)
static __device__ __align__(256) double g_noalloc_part[CO_NOALLOC_PART + 32];

static std::mutex g_noalloc_mu;
static double *g_noalloc_addr[64];  // device address of g_noalloc_part, per device

__device__ __forceinline__ double na_rsqrt(double x) {
    int hi = __double2hiint(x);
    float xf = __int_as_float((hi - (896 << 20)) << 3);
    float yf = rsqrtf(xf);
    int fb = __float_as_int(yf);
    double y = __hiloint2double((fb >> 3) + (896 << 20), fb << 29);
    double t = x * y;
    double e = fma(-t, y, 1.0);
    double p = fma(0.375, e, 0.5);
    double ye = y * e;
    return fma(ye, p, y);
}

__device__ __forceinline__ bool na_inside(double a, double b, double lo1, double hi1, double lo2,
                                          double hi2) {
    return !(a <= lo1 || a >= hi1 || b <= lo2 || b >= hi2);
}

// part[(sl * 2 + c) * N + g]: partial over the alpha range of slice sl
__global__ void __launch_bounds__(NA_TPB)
k_noalloc_pair(const double *__restrict__ v, const double *__restrict__ w,
               const double *__restrict__ G, int N, double lo1, double hi1, double lo2,
               double hi2, int slice_len, double *__restrict__ part) {
    __shared__ double sx1[NA_TPB], sx2[NA_TPB], sg1[NA_TPB], sg2[NA_TPB], sw[NA_TPB];
    const int g = blockIdx.x * NA_TPB + threadIdx.x;
    const int sl = blockIdx.y;
    const int a0 = sl * slice_len;
    const int a1 = min(N, a0 + slice_len);
    double xg1 = 0.0, xg2 = 0.0, Gg1 = 0.0, Gg2 = 0.0;
    bool gin = false;
    if (g < N) {
        xg1 = v[g];
        xg2 = v[N + g];
        Gg1 = G[g];
        Gg2 = G[N + g];
        gin = na_inside(xg1, xg2, lo1, hi1, lo2, hi2);
    }
    double acc1 = 0.0, acc2 = 0.0;
    for (int base = a0; base < a1; base += NA_TPB) {
        int a = base + threadIdx.x;
        double x1 = 1e3, x2 = 1e3, q1 = 0.0, q2 = 0.0, wa = 0.0;
        if (a < a1) {
            double y1 = v[a], y2 = v[N + a];
            if (na_inside(y1, y2, lo1, hi1, lo2, hi2)) {
                x1 = y1;
                x2 = y2;
                q1 = G[a];
                q2 = G[N + a];
                wa = w[a];
            }
        }
        sx1[threadIdx.x] = x1;
        sx2[threadIdx.x] = x2;
        sg1[threadIdx.x] = q1;
        sg2[threadIdx.x] = q2;
        sw[threadIdx.x] = wa;
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < NA_TPB; k++) {
            double d1 = xg1 - sx1[k];
            double d2 = xg2 - sx2[k];
            double r2 = d1 * d1;
            r2 = fma(d2, d2, r2);
            bool ok = __double_as_longlong(r2) >= NA_R2_MIN_BITS;
            double y = na_rsqrt(ok ? r2 : 1.0);
            double g1 = sg1[k] - Gg1;
            double g2 = sg2[k] - Gg2;
            double dg = d1 * g1;
            dg = fma(d2, g2, dg);
            double cc = dg * (y * y);
            double t1 = fma(-d1, cc, g1);
            double t2 = fma(-d2, cc, g2);
            double s = ok ? sw[k] * y : 0.0;
            acc1 = fma(s, t1, acc1);
            acc2 = fma(s, t2, acc2);
        }
        __syncthreads();
    }
    if (g < N) {
        part[((size_t)sl * 2 + 0) * N + g] = gin ? acc1 : 0.0;
        part[((size_t)sl * 2 + 1) * N + g] = gin ? acc2 : 0.0;
    }
}

// flag = 1 if any of v (2N), w (N), G (2N) is NaN or Inf
__global__ void k_noalloc_check(const double *__restrict__ v, const double *__restrict__ w,
                                const double *__restrict__ G, int N, unsigned *flag) {
    int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        bad |= !isfinite(v[i]) | !isfinite(v[N + i]) | !isfinite(w[i]) | !isfinite(G[i]) |
               !isfinite(G[N + i]);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1u);
}

__global__ void k_noalloc_reduce(const double *__restrict__ part, int N, int split,
                                 double *__restrict__ dot_v) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= N) return;
    double s1 = 0.0, s2 = 0.0;
    for (int sl = 0; sl < split; sl++) {
        s1 += part[((size_t)sl * 2 + 0) * N + g];
        s2 += part[((size_t)sl * 2 + 1) * N + g];
    }
    dot_v[g] = s1;
    dot_v[N + g] = s2;
}

// device address of the scratch array on the current device (set up once)
static int noalloc_scratch(double **out) {
    int dev = 0;
    CO_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return CO_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_noalloc_part) != cudaSuccess || !ptr) return CO_ERR_CUDA;
        g_noalloc_addr[dev] = (double *)ptr;
    }
    *out = g_noalloc_addr[dev];
    return CO_OK;
}

extern "C" int co_collision_noalloc(const double *v, const double *w, const double *G,
                                    double *dot_v, int N, double lo1, double hi1, double lo2,
                                    double hi2, void *stream) {
    if (N < 0 || (N > 0 && (!v || !w || !G || !dot_v))) return CO_ERR_ARG;
    if (!(lo1 < hi1) || !(lo2 < hi2)) return CO_ERR_ARG;
    if (N > CO_NOALLOC_MAX_N) return CO_ERR_SIZE;
    if (N == 0) return CO_OK;
    double *part = nullptr;
    int rc = noalloc_scratch(&part);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned *flag = (unsigned *)(part + CO_NOALLOC_PART);
    unsigned bad = 0;
    CO_CK(cudaMemsetAsync(flag, 0, sizeof(unsigned), s));
    k_noalloc_check<<<co_cdiv(N, 256) < 304 ? co_cdiv(N, 256) : 304, 256, 0, s>>>(v, w, G, N,
                                                                                flag);
    CO_CK(cudaGetLastError());
    CO_CK(cudaMemcpyAsync(&bad, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CO_CK(cudaStreamSynchronize(s));
    if (bad) return CO_ERR_NONFINITE;
    const int tiles = co_cdiv(N, NA_TPB);
    int split = co_cdiv(608, tiles);  // about 4 blocks per SM on 152 SMs
    if (split > CO_NOALLOC_SLICES) split = CO_NOALLOC_SLICES;
    if (split < 1) split = 1;
    int slice = co_cdiv(co_cdiv(N, split), NA_TPB) * NA_TPB;
    split = co_cdiv(N, slice);
    dim3 grid(tiles, split);
    k_noalloc_pair<<<grid, NA_TPB, 0, s>>>(v, w, G, N, lo1, hi1, lo2, hi2, slice, part);
    k_noalloc_reduce<<<co_cdiv(N, 256), 256, 0, s>>>(part, N, split, dot_v);
    CO_CK(cudaGetLastError());
    return CO_OK;
}
