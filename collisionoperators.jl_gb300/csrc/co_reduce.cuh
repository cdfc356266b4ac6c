// co_reduce.cuh -- fixed-order block reductions (deterministic run to run).
#pragma once
#include <cuda_runtime.h>

// Sum of one double over a block of blockDim.x (multiple of 32, <= 1024)
// threads; every thread gets the result. Fixed shuffle tree, then warp
// partials summed in warp order by warp 0.
__device__ __forceinline__ double co_block_sum(double v, double *sh /* >= 32 */) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    int nw = blockDim.x >> 5;
    if (warp == 0) {
        double s = lane < nw ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[0] = s;
    }
    __syncthreads();
    double r = sh[0];
    __syncthreads();
    return r;
}

// s += v[i0], v[i0 + step], ... (i < n) in that order. The loads are issued
// eight at a time ahead of the adds, so a thread waits for one L2 round trip
// per eight terms rather than per term; the additions keep their order.
__device__ __forceinline__ double co_strided_sum(const double *v, int i0, int n, int step,
                                                 int ncomp, int comp, double s) {
    int i = i0;
    for (; i + 7 * step < n; i += 8 * step) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; u++) t[u] = v[(size_t)(i + u * step) * ncomp + comp];
#pragma unroll
        for (int u = 0; u < 8; u++) s += t[u];
    }
    for (; i < n; i += step) s += v[(size_t)i * ncomp + comp];
    return s;
}

// co_strided_sum with the loads through L2 (__ldcg), for partials that other
// blocks of the same launch wrote (the last-block-done pattern)
__device__ __forceinline__ double co_strided_sum_cg(const double *v, int i0, int n, int step,
                                                    int ncomp, int comp, double s) {
    int i = i0;
    for (; i + 7 * step < n; i += 8 * step) {
        double t[8];
#pragma unroll
        for (int u = 0; u < 8; u++) t[u] = __ldcg(&v[(size_t)(i + u * step) * ncomp + comp]);
#pragma unroll
        for (int u = 0; u < 8; u++) s += t[u];
    }
    for (; i < n; i += step) s += __ldcg(&v[(size_t)i * ncomp + comp]);
    return s;
}

// Sum of red[0..n) * (stride) component `comp` by one block, fixed order:
// thread t sums entries t, t+B, ... in order, then co_block_sum.
__device__ __forceinline__ double co_sum_partials(const double *red, int n, int ncomp,
                                                   int comp, double *sh) {
    double s = co_strided_sum(red, threadIdx.x, n, blockDim.x, ncomp, comp, 0.0);
    return co_block_sum(s, sh);
}

// Sums each of the V values v[0..V) (V = 2, 4, 8 or 16) over the 32 lanes of a
// warp by recursive halving: at each level a lane keeps the half of its values
// that its lane bit selects and adds the partner's copy of that half; once one
// value is left, plain butterfly levels finish the sum. The adds per lane are
// V - 1 + (6 - log2 V) instead of 5 V for V shuffle trees, which matters at
// GB300's FP64 rate. Returns the sum of value lane >> (5 - log2 V) (lanes that
// differ only in the low bits hold the same sum). Fixed order, deterministic.
// v is overwritten.
template <int V>
__device__ __forceinline__ double co_warp_sum(double (&v)[V], int lane) {
    static_assert(V == 2 || V == 4 || V == 8 || V == 16, "V must be 2, 4, 8 or 16");
    int bit = 16;
#pragma unroll
    for (int half = V / 2; half >= 1; half >>= 1, bit >>= 1) {
        const bool up = (lane & bit) != 0;
#pragma unroll
        for (int i = 0; i < half; i++) {
            const double send = up ? v[i] : v[half + i];
            const double keep = up ? v[half + i] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, bit);
        }
    }
    double s = v[0];
#pragma unroll
    for (; bit >= 1; bit >>= 1) s += __shfl_xor_sync(0xffffffffu, s, bit);
    return s;
}

__device__ __forceinline__ double co_warp_sum16(double (&v)[16], int lane) {
    return co_warp_sum<16>(v, lane);
}
