// co_mlp.cu -- the learned warm start: a small MLP trained and evaluated by
// this library's own kernels.
//
// Network: n_in -> 64 -> 64 -> 64 -> n_out, GELU (erf form) after the three
// hidden layers. The weight matrices are BF16 (the copy every kernel reads); an
// FP32 master copy and the Adam moments live beside them; biases are FP32.
// Every kernel converts the BF16 weights to FP32 in shared memory and
// accumulates in FP32. One sample per thread for the forward and the
// per-sample backward pass; the weight gradients are reduced over the
// minibatch by one thread per parameter in a fixed sample order, so training
// is deterministic run to run. Loss: mean squared error over samples and
// outputs.
//
// Used as the warm start of the implicit step: the network maps per-marker
// features at the start of a step (velocity, entropy gradient, predictor
// velocity, log-density and its gradient) to the normalised correction
// (v_converged - v_Euler)/dt^2, in the spirit of the reference's planned
// "Euler + dt^2 * delta" correction (Parameters.jl:108-112). The solver keeps
// the last word: the caller keeps the plain predictor whenever the learned
// proposal's first residual is larger.
#include <cuda_bf16.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "co_internal.cuh"

#define MLP_H 64
#define MLP_MAX_IN 16
#define MLP_MAX_OUT 4
#define MLP_TPB 64

struct co_mlp {
    int device;
    int n_in, n_out;
    size_t P;                    // number of parameters
    float *master;               // FP32 parameters (layout below)
    __nv_bfloat16 *wbf;          // BF16 copy of all parameters (weights used in BF16)
    float *grad, *m1, *m2;       // gradient and Adam moments
    int step;
    // training scratch
    float *z;                    // B x 3 x H pre-activations
    float *y;                    // B x n_out outputs
    float *d;                    // B x (3 H + n_out) deltas
    int cap;
    // feature and output normalisation applied by co_mlp_forward (inference):
    // [mean (MLP_MAX_IN), 1/std (MLP_MAX_IN), out std (MLP_MAX_OUT), out mean
    // (MLP_MAX_OUT)]; NULL = none. Training kernels see normalised data as given.
    float *norm;
};
#define MLP_NORM_FLOATS (2 * MLP_MAX_IN + 2 * MLP_MAX_OUT)

// parameter offsets: W0 [H][n_in], b0 [H], W1 [H][H], b1 [H], W2 [H][H], b2 [H],
// W3 [n_out][H], b3 [n_out]
struct mlp_off {
    int W0, b0, W1, b1, W2, b2, W3, b3, P;
};
__host__ __device__ inline mlp_off mlp_offsets(int n_in, int n_out) {
    mlp_off o;
    o.W0 = 0;
    o.b0 = o.W0 + MLP_H * n_in;
    o.W1 = o.b0 + MLP_H;
    o.b1 = o.W1 + MLP_H * MLP_H;
    o.W2 = o.b1 + MLP_H;
    o.b2 = o.W2 + MLP_H * MLP_H;
    o.W3 = o.b2 + MLP_H;
    o.b3 = o.W3 + n_out * MLP_H;
    o.P = o.b3 + n_out;
    return o;
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_d(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
           x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// weights (BF16 -> FP32) and biases into shared memory
__device__ void mlp_load(const __nv_bfloat16 *__restrict__ wbf, const float *__restrict__ master,
                         mlp_off o, int n_in, int n_out, float *sp) {
    for (int i = threadIdx.x; i < o.P; i += blockDim.x) {
        bool is_bias = (i >= o.b0 && i < o.W1) || (i >= o.b1 && i < o.W2) ||
                       (i >= o.b2 && i < o.W3) || i >= o.b3;
        sp[i] = is_bias ? master[i] : __bfloat162float(wbf[i]);
    }
    __syncthreads();
}

// forward pass of one sample; z (if given) receives the three pre-activations
__device__ __forceinline__ void mlp_fwd(const float *sp, mlp_off o, int n_in, int n_out,
                                        const float *x, float *z, float *out) {
    float a[MLP_H], b[MLP_H];
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        float s = sp[o.b0 + j];
#pragma unroll
        for (int i = 0; i < MLP_MAX_IN; i++)
            if (i < n_in) s = fmaf(sp[o.W0 + j * n_in + i], x[i], s);
        if (z) z[j] = s;
        a[j] = gelu(s);
    }
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        float s = sp[o.b1 + j];
#pragma unroll
        for (int i = 0; i < MLP_H; i++) s = fmaf(sp[o.W1 + j * MLP_H + i], a[i], s);
        if (z) z[MLP_H + j] = s;
        b[j] = gelu(s);
    }
#pragma unroll
    for (int j = 0; j < MLP_H; j++) {
        float s = sp[o.b2 + j];
#pragma unroll
        for (int i = 0; i < MLP_H; i++) s = fmaf(sp[o.W2 + j * MLP_H + i], b[i], s);
        if (z) z[2 * MLP_H + j] = s;
        a[j] = gelu(s);
    }
#pragma unroll
    for (int k = 0; k < MLP_MAX_OUT; k++) {
        if (k < n_out) {
            float s = sp[o.b3 + k];
#pragma unroll
            for (int i = 0; i < MLP_H; i++) s = fmaf(sp[o.W3 + k * MLP_H + i], a[i], s);
            out[k] = s;
        }
    }
}

__global__ void __launch_bounds__(MLP_TPB)
k_mlp_forward(const __nv_bfloat16 *__restrict__ wbf, const float *__restrict__ master, int n_in,
              int n_out, const float *__restrict__ X, int B, float *__restrict__ Y,
              float *__restrict__ Z, const float *__restrict__ norm) {
    extern __shared__ float sp[];
    mlp_off o = mlp_offsets(n_in, n_out);
    mlp_load(wbf, master, o, n_in, n_out, sp);
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    float x[MLP_MAX_IN], out[MLP_MAX_OUT];
#pragma unroll
    for (int i = 0; i < MLP_MAX_IN; i++) {
        float xi = i < n_in ? X[(size_t)s * n_in + i] : 0.f;
        if (norm && i < n_in) xi = (xi - norm[i]) * norm[MLP_MAX_IN + i];
        x[i] = xi;
    }
    mlp_fwd(sp, o, n_in, n_out, x, Z ? Z + (size_t)s * 3 * MLP_H : nullptr, out);
#pragma unroll
    for (int k = 0; k < MLP_MAX_OUT; k++)
        if (k < n_out) {
            float y = out[k];
            if (norm) y = fmaf(y, norm[2 * MLP_MAX_IN + k], norm[2 * MLP_MAX_IN + MLP_MAX_OUT + k]);
            Y[(size_t)s * n_out + k] = y;
        }
}

// per-sample deltas: D[s] = [dz0 (H), dz1 (H), dz2 (H), dy (n_out)]
__global__ void __launch_bounds__(MLP_TPB)
k_mlp_backward(const __nv_bfloat16 *__restrict__ wbf, const float *__restrict__ master, int n_in,
               int n_out, const float *__restrict__ Z, const float *__restrict__ Y,
               const float *__restrict__ T, int B, float *__restrict__ D) {
    extern __shared__ float sp[];
    mlp_off o = mlp_offsets(n_in, n_out);
    mlp_load(wbf, master, o, n_in, n_out, sp);
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const float *z = Z + (size_t)s * 3 * MLP_H;
    float *dd = D + (size_t)s * (3 * MLP_H + n_out);
    float dy[MLP_MAX_OUT];
    const float scale = 2.0f / ((float)B * (float)n_out);
#pragma unroll
    for (int k = 0; k < MLP_MAX_OUT; k++) {
        dy[k] = k < n_out ? scale * (Y[(size_t)s * n_out + k] - T[(size_t)s * n_out + k]) : 0.f;
        if (k < n_out) dd[3 * MLP_H + k] = dy[k];
    }
    float g[MLP_H], h[MLP_H];
#pragma unroll
    for (int i = 0; i < MLP_H; i++) {  // dz2 = W3^T dy * gelu'(z2)
        float sacc = 0.f;
#pragma unroll
        for (int k = 0; k < MLP_MAX_OUT; k++)
            if (k < n_out) sacc = fmaf(sp[o.W3 + k * MLP_H + i], dy[k], sacc);
        g[i] = sacc * gelu_d(z[2 * MLP_H + i]);
        dd[2 * MLP_H + i] = g[i];
    }
#pragma unroll
    for (int i = 0; i < MLP_H; i++) {  // dz1 = W2^T dz2 * gelu'(z1)
        float sacc = 0.f;
#pragma unroll
        for (int j = 0; j < MLP_H; j++) sacc = fmaf(sp[o.W2 + j * MLP_H + i], g[j], sacc);
        h[i] = sacc * gelu_d(z[MLP_H + i]);
        dd[MLP_H + i] = h[i];
    }
#pragma unroll
    for (int i = 0; i < MLP_H; i++) {  // dz0 = W1^T dz1 * gelu'(z0)
        float sacc = 0.f;
#pragma unroll
        for (int j = 0; j < MLP_H; j++) sacc = fmaf(sp[o.W1 + j * MLP_H + i], h[j], sacc);
        dd[i] = sacc * gelu_d(z[i]);
    }
}

// one thread per parameter: sum over the minibatch in sample order
__global__ void k_mlp_wgrad(int n_in, int n_out, const float *__restrict__ X,
                            const float *__restrict__ Z, const float *__restrict__ D, int B,
                            float *__restrict__ grad) {
    mlp_off o = mlp_offsets(n_in, n_out);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= o.P) return;
    const int DS = 3 * MLP_H + n_out;
    float s = 0.f;
    if (p < o.b0) {                      // W0[j][i]: dz0_j x_i
        int j = p / n_in, i = p - j * n_in;
        for (int b = 0; b < B; b++) s = fmaf(D[(size_t)b * DS + j], X[(size_t)b * n_in + i], s);
    } else if (p < o.W1) {               // b0
        int j = p - o.b0;
        for (int b = 0; b < B; b++) s += D[(size_t)b * DS + j];
    } else if (p < o.b1) {               // W1[j][i]: dz1_j gelu(z0_i)
        int q = p - o.W1, j = q / MLP_H, i = q - j * MLP_H;
        for (int b = 0; b < B; b++)
            s = fmaf(D[(size_t)b * DS + MLP_H + j], gelu(Z[(size_t)b * 3 * MLP_H + i]), s);
    } else if (p < o.W2) {
        int j = p - o.b1;
        for (int b = 0; b < B; b++) s += D[(size_t)b * DS + MLP_H + j];
    } else if (p < o.b2) {               // W2[j][i]: dz2_j gelu(z1_i)
        int q = p - o.W2, j = q / MLP_H, i = q - j * MLP_H;
        for (int b = 0; b < B; b++)
            s = fmaf(D[(size_t)b * DS + 2 * MLP_H + j],
                     gelu(Z[(size_t)b * 3 * MLP_H + MLP_H + i]), s);
    } else if (p < o.W3) {
        int j = p - o.b2;
        for (int b = 0; b < B; b++) s += D[(size_t)b * DS + 2 * MLP_H + j];
    } else if (p < o.b3) {               // W3[k][i]: dy_k gelu(z2_i)
        int q = p - o.W3, k = q / MLP_H, i = q - k * MLP_H;
        for (int b = 0; b < B; b++)
            s = fmaf(D[(size_t)b * DS + 3 * MLP_H + k],
                     gelu(Z[(size_t)b * 3 * MLP_H + 2 * MLP_H + i]), s);
    } else {
        int k = p - o.b3;
        for (int b = 0; b < B; b++) s += D[(size_t)b * DS + 3 * MLP_H + k];
    }
    grad[p] = s;
}

__global__ void k_mlp_adam(int P, float lr, float b1, float b2, float eps, int step,
                           float *__restrict__ master, __nv_bfloat16 *__restrict__ wbf,
                           const float *__restrict__ grad, float *__restrict__ m1,
                           float *__restrict__ m2) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    float g = grad[p];
    float a = b1 * m1[p] + (1.f - b1) * g;
    float v = b2 * m2[p] + (1.f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    float ah = a / (1.f - powf(b1, (float)step));
    float vh = v / (1.f - powf(b2, (float)step));
    float w = master[p] - lr * ah / (sqrtf(vh) + eps);
    master[p] = w;
    wbf[p] = __float2bfloat16_rn(w);
}

__global__ void k_mlp_refresh(int P, const float *__restrict__ master, __nv_bfloat16 *__restrict__ wbf) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) wbf[p] = __float2bfloat16_rn(master[p]);
}

// ---------------------------------------------------------------- host

static int mlp_ensure(co_mlp *m, int B) {
    if (B <= m->cap) return CO_OK;
    cudaFree(m->z);
    cudaFree(m->y);
    cudaFree(m->d);
    m->z = m->y = m->d = nullptr;
    if (cudaMalloc(&m->z, sizeof(float) * (size_t)B * 3 * MLP_H) != cudaSuccess ||
        cudaMalloc(&m->y, sizeof(float) * (size_t)B * m->n_out) != cudaSuccess ||
        cudaMalloc(&m->d, sizeof(float) * (size_t)B * (3 * MLP_H + m->n_out)) != cudaSuccess)
        return CO_ERR_NOMEM;
    m->cap = B;
    return CO_OK;
}

extern "C" int co_mlp_create(int n_in, int n_out, unsigned seed, int device, co_mlp **out) {
    if (!out || n_in < 1 || n_in > MLP_MAX_IN || n_out < 1 || n_out > MLP_MAX_OUT)
        return CO_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return CO_ERR_NODEVICE;
    CO_CK(cudaSetDevice(device));
    co_mlp *m = (co_mlp *)calloc(1, sizeof(co_mlp));
    m->device = device;
    m->n_in = n_in;
    m->n_out = n_out;
    mlp_off o = mlp_offsets(n_in, n_out);
    m->P = o.P;
    // He-style init with a small LCG (deterministic from the seed)
    std::vector<float> h(o.P, 0.f);
    unsigned long long st = 0x9E3779B97F4A7C15ull ^ seed;
    auto unif = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return ((st >> 40) & 0xFFFFFF) / 16777216.0f * 2.f - 1.f;
    };
    for (int i = o.W0; i < o.b0; i++) h[i] = unif() * sqrtf(3.f * 2.f / n_in);
    for (int i = o.W1; i < o.b1; i++) h[i] = unif() * sqrtf(3.f * 2.f / MLP_H);
    for (int i = o.W2; i < o.b2; i++) h[i] = unif() * sqrtf(3.f * 2.f / MLP_H);
    for (int i = o.W3; i < o.b3; i++) h[i] = unif() * sqrtf(3.f / MLP_H) * 0.1f;
    if (cudaMalloc(&m->master, sizeof(float) * o.P) != cudaSuccess ||
        cudaMalloc(&m->wbf, sizeof(__nv_bfloat16) * o.P) != cudaSuccess ||
        cudaMalloc(&m->grad, sizeof(float) * o.P) != cudaSuccess ||
        cudaMalloc(&m->m1, sizeof(float) * o.P) != cudaSuccess ||
        cudaMalloc(&m->m2, sizeof(float) * o.P) != cudaSuccess) {
        co_mlp_destroy(m);
        return CO_ERR_NOMEM;
    }
    cudaMemcpy(m->master, h.data(), sizeof(float) * o.P, cudaMemcpyHostToDevice);
    cudaMemset(m->m1, 0, sizeof(float) * o.P);
    cudaMemset(m->m2, 0, sizeof(float) * o.P);
    k_mlp_refresh<<<co_cdiv(o.P, 256), 256>>>((int)o.P, m->master, m->wbf);
    int smem = (int)(sizeof(float) * o.P);
    cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        co_mlp_destroy(m);
        return CO_ERR_CUDA;
    }
    *out = m;
    return CO_OK;
}

extern "C" int co_mlp_destroy(co_mlp *m) {
    if (!m) return CO_ERR_ARG;
    cudaSetDevice(m->device);
    void *ptrs[] = {m->master, m->wbf, m->grad, m->m1, m->m2, m->z, m->y, m->d, m->norm};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    free(m);
    return CO_OK;
}

extern "C" int co_mlp_num_params(const co_mlp *m, int *P) {
    if (!m || !P) return CO_ERR_ARG;
    *P = (int)m->P;
    return CO_OK;
}

extern "C" int co_mlp_set_params(co_mlp *m, const float *host) {
    if (!m || !host) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(m->device));
    CO_CK(cudaMemcpy(m->master, host, sizeof(float) * m->P, cudaMemcpyHostToDevice));
    CO_CK(cudaMemset(m->m1, 0, sizeof(float) * m->P));
    CO_CK(cudaMemset(m->m2, 0, sizeof(float) * m->P));
    m->step = 0;
    k_mlp_refresh<<<co_cdiv(m->P, 256), 256>>>((int)m->P, m->master, m->wbf);
    CO_CK(cudaDeviceSynchronize());
    return CO_OK;
}

extern "C" int co_mlp_get_params(const co_mlp *m, float *host) {
    if (!m || !host) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(m->device));
    CO_CK(cudaMemcpy(host, m->master, sizeof(float) * m->P, cudaMemcpyDeviceToHost));
    return CO_OK;
}

extern "C" int co_mlp_set_normalization(co_mlp *m, const double *x_mean, const double *x_std,
                                        const double *y_mean, const double *y_std) {
    if (!m) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(m->device));
    if (!x_mean) {
        if (m->norm) cudaFree(m->norm);
        m->norm = nullptr;
        return CO_OK;
    }
    if (!x_std || !y_mean || !y_std) return CO_ERR_ARG;
    float h[MLP_NORM_FLOATS] = {0.f};
    for (int i = 0; i < m->n_in; i++) {
        if (!(x_std[i] > 0.0) || !isfinite(x_mean[i])) return CO_ERR_ARG;
        h[i] = (float)x_mean[i];
        h[MLP_MAX_IN + i] = (float)(1.0 / x_std[i]);
    }
    for (int k = 0; k < m->n_out; k++) {
        if (!isfinite(y_std[k]) || !isfinite(y_mean[k])) return CO_ERR_ARG;
        h[2 * MLP_MAX_IN + k] = (float)y_std[k];
        h[2 * MLP_MAX_IN + MLP_MAX_OUT + k] = (float)y_mean[k];
    }
    if (!m->norm && cudaMalloc(&m->norm, sizeof(h)) != cudaSuccess) return CO_ERR_NOMEM;
    CO_CK(cudaMemcpy(m->norm, h, sizeof(h), cudaMemcpyHostToDevice));
    return CO_OK;
}

// Y = net(X) for B samples (device pointers, row-major B x n_in / B x n_out),
// with the normalisation of co_mlp_set_normalization applied if set
extern "C" int co_mlp_forward(co_mlp *m, const float *X, int B, float *Y, void *stream) {
    if (!m || B < 0 || (B > 0 && (!X || !Y))) return CO_ERR_ARG;
    if (B == 0) return CO_OK;
    CO_CK(cudaSetDevice(m->device));
    int smem = (int)(sizeof(float) * m->P);
    k_mlp_forward<<<co_cdiv(B, MLP_TPB), MLP_TPB, smem, (cudaStream_t)stream>>>(
        m->wbf, m->master, m->n_in, m->n_out, X, B, Y, nullptr, m->norm);
    CO_CK(cudaGetLastError());
    return CO_OK;
}

static int mlp_grad(co_mlp *m, const float *X, const float *T, int B, float *loss) {
    int rc = mlp_ensure(m, B);
    if (rc) return rc;
    int smem = (int)(sizeof(float) * m->P);
    k_mlp_forward<<<co_cdiv(B, MLP_TPB), MLP_TPB, smem>>>(m->wbf, m->master, m->n_in, m->n_out, X,
                                                         B, m->y, m->z, nullptr);
    k_mlp_backward<<<co_cdiv(B, MLP_TPB), MLP_TPB, smem>>>(m->wbf, m->master, m->n_in, m->n_out,
                                                          m->z, m->y, T, B, m->d);
    k_mlp_wgrad<<<co_cdiv(m->P, 128), 128>>>(m->n_in, m->n_out, X, m->z, m->d, B, m->grad);
    CO_CK(cudaGetLastError());
    if (loss) {
        std::vector<float> y((size_t)B * m->n_out), t((size_t)B * m->n_out);
        CO_CK(cudaMemcpy(y.data(), m->y, sizeof(float) * y.size(), cudaMemcpyDeviceToHost));
        CO_CK(cudaMemcpy(t.data(), T, sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
        double s = 0.0;
        for (size_t i = 0; i < y.size(); i++) s += (double)(y[i] - t[i]) * (y[i] - t[i]);
        *loss = (float)(s / (double)y.size());
    }
    return CO_OK;
}

// gradients of the mean squared error w.r.t. all parameters (host array of P)
extern "C" int co_mlp_gradients(co_mlp *m, const float *X, const float *T, int B, float *grad,
                                float *loss) {
    if (!m || !X || !T || !grad || B < 1) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(m->device));
    int rc = mlp_grad(m, X, T, B, loss);
    if (rc) return rc;
    CO_CK(cudaMemcpy(grad, m->grad, sizeof(float) * m->P, cudaMemcpyDeviceToHost));
    return CO_OK;
}

// one Adam step on a minibatch (device X: B x n_in, T: B x n_out)
extern "C" int co_mlp_train_step(co_mlp *m, const float *X, const float *T, int B, float lr,
                                 float *loss) {
    if (!m || !X || !T || B < 1) return CO_ERR_ARG;
    CO_CK(cudaSetDevice(m->device));
    int rc = mlp_grad(m, X, T, B, loss);
    if (rc) return rc;
    m->step += 1;
    k_mlp_adam<<<co_cdiv(m->P, 256), 256>>>((int)m->P, lr, 0.9f, 0.999f, 1e-8f, m->step,
                                            m->master, m->wbf, m->grad, m->m1, m->m2);
    CO_CK(cudaGetLastError());
    return CO_OK;
}
