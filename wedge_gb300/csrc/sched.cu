// Training and checking kernels of the scheduler network (see sched.cuh).
//
// A block of NH = 64 threads takes a contiguous run of samples, one sample at
// a time: thread k owns hidden neuron k of both layers, so it keeps the
// gradient rows it owns (W1[k][:], W2[k][:], W3[:][k], b1[k], b2[k]) in
// registers across the run and writes them once.  The per-block partial
// gradients are then summed in block order by one kernel and applied by an
// Adam step, so a training run is deterministic for a given sample order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "engine.cuh"
#include "sched.cuh"

namespace wedge {

constexpr int MLP_THREADS = NH;
constexpr int SAMPLES_PER_BLOCK = 16;

struct MlpShared {
    float net[WEDGE_SCHED_BLOB];
    float raw[NF], xs[NF], h1[NH], h2[NH], out[NO], dy[NO], dh2[NH];
};

// forward of samples [blockIdx.x * per_block, ...): out[n][NO]
__global__ void __launch_bounds__(MLP_THREADS) mlp_forward_kernel(const float* __restrict__ net, const float* X,
                                                                  uint32_t n, uint32_t per_block, float* out)
{
    __shared__ MlpShared sh;
    for (int i = threadIdx.x; i < WEDGE_SCHED_BLOB; i += blockDim.x)
        sh.net[i] = net[i];
    __syncthreads();
    const uint32_t s0 = blockIdx.x * per_block;
    for (uint32_t s = s0; s < n && s < s0 + per_block; ++s) {
        if (threadIdx.x < NF)
            sh.raw[threadIdx.x] = X[(uint64_t)s * NF + threadIdx.x];
        __syncthreads();
        sched_forward_block(sh.net, sh.raw, sh.xs, sh.h1, sh.h2, sh.out);
        if (threadIdx.x < NO)
            out[(uint64_t)s * NO + threadIdx.x] = sh.out[threadIdx.x];
        __syncthreads();
    }
}

// Loss (sum over measured outputs of (y - target)^2, divided by `norm`) and its
// gradient for the samples idx[b*per_block ...] (idx == nullptr: the identity).
// partial[b][WEDGE_SCHED_PARAMS] gets the block's gradient, loss_part[b] its loss.
__global__ void __launch_bounds__(MLP_THREADS) mlp_grad_kernel(const float* __restrict__ net, const float* X,
                                                               const float* Y, const float* M, const uint32_t* idx,
                                                               uint32_t n, uint32_t per_block, float norm,
                                                               float* partial, double* loss_part)
{
    __shared__ MlpShared sh;
    const int k = threadIdx.x;
    for (int i = k; i < WEDGE_SCHED_BLOB; i += blockDim.x)
        sh.net[i] = net[i];
    float gW1[NF], gW2[NH], gW3[NO];
    float gb1 = 0.0f, gb2 = 0.0f, gb3 = 0.0f;
#pragma unroll
    for (int i = 0; i < NF; ++i)
        gW1[i] = 0.0f;
#pragma unroll
    for (int j = 0; j < NH; ++j)
        gW2[j] = 0.0f;
#pragma unroll
    for (int o = 0; o < NO; ++o)
        gW3[o] = 0.0f;
    double loss = 0.0;
    __syncthreads();
    const uint32_t s0 = blockIdx.x * per_block;
    for (uint32_t r = s0; r < n && r < s0 + per_block; ++r) {
        const uint32_t s = idx ? idx[r] : r;
        if (k < NF)
            sh.raw[k] = X[(uint64_t)s * NF + k];
        __syncthreads();
        sched_forward_block(sh.net, sh.raw, sh.xs, sh.h1, sh.h2, sh.out);
        if (k < NO) {
            const float m = M[(uint64_t)s * NO + k];
            const float e = (m != 0.0f) ? sh.out[k] - Y[(uint64_t)s * NO + k] : 0.0f;
            loss += (double)e * (double)e;
            sh.dy[k] = 2.0f * e / norm;
            gb3 += sh.dy[k];
        }
        __syncthreads();
        // layer 3 and the hidden-2 error of neuron k
        const float h2k = sh.h2[k];
        float d2 = 0.0f;
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            gW3[o] = __fmaf_rn(sh.dy[o], h2k, gW3[o]);
            d2 = __fmaf_rn(sh.net[OFF_W3 + o * NH + k], sh.dy[o], d2);
        }
        d2 = (h2k > 0.0f) ? d2 : 0.0f;
        sh.dh2[k] = d2;
        gb2 += d2;
        __syncthreads();
        // layer 2 row k, and the hidden-1 error of neuron k (column k of W2)
        float d1 = 0.0f;
#pragma unroll
        for (int j = 0; j < NH; ++j) {
            gW2[j] = __fmaf_rn(d2, sh.h1[j], gW2[j]);
            d1 = __fmaf_rn(sh.net[OFF_W2 + j * NH + k], sh.dh2[j], d1);
        }
        d1 = (sh.h1[k] > 0.0f) ? d1 : 0.0f;
        gb1 += d1;
#pragma unroll
        for (int i = 0; i < NF; ++i)
            gW1[i] = __fmaf_rn(d1, sh.xs[i], gW1[i]);
        __syncthreads(); /* the next sample overwrites the shared activations */
    }
    float* p = partial + (uint64_t)blockIdx.x * WEDGE_SCHED_PARAMS;
    constexpr int W1 = OFF_W1 - OFF_W1, B1 = OFF_B1 - OFF_W1, W2 = OFF_W2 - OFF_W1, B2 = OFF_B2 - OFF_W1,
                  W3 = OFF_W3 - OFF_W1, B3 = OFF_B3 - OFF_W1;
#pragma unroll
    for (int i = 0; i < NF; ++i)
        p[W1 + k * NF + i] = gW1[i];
    p[B1 + k] = gb1;
#pragma unroll
    for (int j = 0; j < NH; ++j)
        p[W2 + k * NH + j] = gW2[j];
    p[B2 + k] = gb2;
#pragma unroll
    for (int o = 0; o < NO; ++o)
        p[W3 + o * NH + k] = gW3[o];
    if (k < NO)
        p[B3 + k] = gb3;
    // block loss: threads 0..NO-1 hold parts
    __shared__ double sl[NO];
    if (k < NO)
        sl[k] = loss;
    __syncthreads();
    if (k == 0) {
        double a = 0.0;
        for (int o = 0; o < NO; ++o)
            a += sl[o];
        loss_part[blockIdx.x] = a / (double)norm;
    }
}

// grad[p] = sum over blocks, in block order
__global__ void mlp_reduce_kernel(const float* partial, uint32_t nblocks, float* grad)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)WEDGE_SCHED_PARAMS)
        return;
    float a = 0.0f;
    for (uint32_t b = 0; b < nblocks; ++b)
        a += partial[(uint64_t)b * WEDGE_SCHED_PARAMS + p];
    grad[p] = a;
}

// Adam (Kingma & Ba, 2015) on the trainable part of the blob; bc1/bc2 = 1 - beta^t
__global__ void mlp_adam_kernel(float* net, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                                float eps, float bc1, float bc2)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)WEDGE_SCHED_PARAMS)
        return;
    const float g = grad[p];
    const float mm = beta1 * m[p] + (1.0f - beta1) * g;
    const float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float mh = mm / bc1, vh = vv / bc2;
    net[OFF_W1 + p] -= lr * mh / (sqrtf(vh) + eps);
}

namespace {

struct DevBuf {
    void* p = nullptr;
    ~DevBuf()
    {
        if (p)
            cudaFree(p);
    }
    template <class T>
    T* as()
    {
        return static_cast<T*>(p);
    }
};

int to_device(DevBuf& b, const void* host, size_t bytes)
{
    WEDGE_CHECK(cudaMalloc(&b.p, bytes ? bytes : 16));
    if (bytes)
        WEDGE_CHECK(cudaMemcpy(b.p, host, bytes, cudaMemcpyHostToDevice));
    return WEDGE_OK;
}

uint32_t blocks_for(uint64_t n) { return (uint32_t)((n + SAMPLES_PER_BLOCK - 1) / SAMPLES_PER_BLOCK); }

uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace
}  // namespace wedge

using namespace wedge;

extern "C" int wedge_mlp_forward(const float* blob, const float* X, uint64_t n, float* out)
{
    if (!blob || (n && (!X || !out)) || n > 0xFFFFFFFFull)
        return WEDGE_ERR_ARG;
    if (n == 0)
        return WEDGE_OK;
    DevBuf dnet, dx, dout;
    int rc;
    if ((rc = to_device(dnet, blob, sizeof(float) * WEDGE_SCHED_BLOB)) || (rc = to_device(dx, X, sizeof(float) * NF * n)))
        return rc;
    WEDGE_CHECK(cudaMalloc(&dout.p, sizeof(float) * NO * n));
    mlp_forward_kernel<<<blocks_for(n), MLP_THREADS>>>(dnet.as<float>(), dx.as<float>(), (uint32_t)n, SAMPLES_PER_BLOCK,
                                                       dout.as<float>());
    WEDGE_CHECK(cudaGetLastError());
    WEDGE_CHECK(cudaMemcpy(out, dout.p, sizeof(float) * NO * n, cudaMemcpyDeviceToHost));
    return WEDGE_OK;
}

extern "C" int wedge_mlp_loss_grad(const float* blob, const float* X, const float* Y, const float* M, uint64_t n,
                                   double* loss, float* grad)
{
    if (!blob || !loss || !grad || n == 0 || !X || !Y || !M || n > 0xFFFFFFFFull)
        return WEDGE_ERR_ARG;
    const uint32_t nb = blocks_for(n);
    DevBuf dnet, dx, dy, dm, dpart, dloss, dgrad;
    int rc;
    if ((rc = to_device(dnet, blob, sizeof(float) * WEDGE_SCHED_BLOB)) || (rc = to_device(dx, X, sizeof(float) * NF * n)) ||
        (rc = to_device(dy, Y, sizeof(float) * NO * n)) || (rc = to_device(dm, M, sizeof(float) * NO * n)))
        return rc;
    WEDGE_CHECK(cudaMalloc(&dpart.p, sizeof(float) * WEDGE_SCHED_PARAMS * nb));
    WEDGE_CHECK(cudaMalloc(&dloss.p, sizeof(double) * nb));
    WEDGE_CHECK(cudaMalloc(&dgrad.p, sizeof(float) * WEDGE_SCHED_PARAMS));
    mlp_grad_kernel<<<nb, MLP_THREADS>>>(dnet.as<float>(), dx.as<float>(), dy.as<float>(), dm.as<float>(), nullptr,
                                         (uint32_t)n, SAMPLES_PER_BLOCK, (float)n, dpart.as<float>(),
                                         dloss.as<double>());
    mlp_reduce_kernel<<<(WEDGE_SCHED_PARAMS + 255) / 256, 256>>>(dpart.as<float>(), nb, dgrad.as<float>());
    WEDGE_CHECK(cudaGetLastError());
    WEDGE_CHECK(cudaMemcpy(grad, dgrad.p, sizeof(float) * WEDGE_SCHED_PARAMS, cudaMemcpyDeviceToHost));
    double* lp = (double*)malloc(sizeof(double) * nb);
    if (!lp)
        return WEDGE_ERR_OOM;
    cudaError_t e = cudaMemcpy(lp, dloss.p, sizeof(double) * nb, cudaMemcpyDeviceToHost);
    double a = 0.0;
    for (uint32_t b = 0; b < nb; ++b)
        a += lp[b];
    free(lp);
    if (e != cudaSuccess)
        return cuda_status(e);
    *loss = a;
    return WEDGE_OK;
}

extern "C" int wedge_mlp_train(float* blob, const float* X, const float* Y, const float* M, uint64_t n,
                               uint32_t epochs, uint32_t batch, float lr, uint64_t seed, double* final_loss)
{
    if (!blob || n == 0 || !X || !Y || !M || batch == 0 || n > 0xFFFFFFFFull || !(lr > 0.0f))
        return WEDGE_ERR_ARG;
    if (batch > n)
        batch = (uint32_t)n;
    const uint32_t nb = blocks_for(batch);
    DevBuf dnet, dx, dy, dm, dpart, dloss, dgrad, dmom, dvel, didx;
    int rc;
    if ((rc = to_device(dnet, blob, sizeof(float) * WEDGE_SCHED_BLOB)) || (rc = to_device(dx, X, sizeof(float) * NF * n)) ||
        (rc = to_device(dy, Y, sizeof(float) * NO * n)) || (rc = to_device(dm, M, sizeof(float) * NO * n)))
        return rc;
    WEDGE_CHECK(cudaMalloc(&dpart.p, sizeof(float) * WEDGE_SCHED_PARAMS * nb));
    WEDGE_CHECK(cudaMalloc(&dloss.p, sizeof(double) * nb));
    WEDGE_CHECK(cudaMalloc(&dgrad.p, sizeof(float) * WEDGE_SCHED_PARAMS));
    WEDGE_CHECK(cudaMalloc(&dmom.p, sizeof(float) * WEDGE_SCHED_PARAMS));
    WEDGE_CHECK(cudaMalloc(&dvel.p, sizeof(float) * WEDGE_SCHED_PARAMS));
    WEDGE_CHECK(cudaMalloc(&didx.p, sizeof(uint32_t) * n));
    WEDGE_CHECK(cudaMemset(dmom.p, 0, sizeof(float) * WEDGE_SCHED_PARAMS));
    WEDGE_CHECK(cudaMemset(dvel.p, 0, sizeof(float) * WEDGE_SCHED_PARAMS));
    uint32_t* perm = (uint32_t*)malloc(sizeof(uint32_t) * n);
    if (!perm)
        return WEDGE_ERR_OOM;
    for (uint64_t i = 0; i < n; ++i)
        perm[i] = (uint32_t)i;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    float bc1 = 1.0f, bc2 = 1.0f;
    uint64_t state = seed;
    int err = WEDGE_OK;
    for (uint32_t ep = 0; ep < epochs && err == WEDGE_OK; ++ep) {
        for (uint64_t i = n - 1; i > 0; --i) { /* Fisher-Yates with a splitmix64 stream */
            state = mix64(state);
            const uint64_t j = state % (i + 1);
            const uint32_t t = perm[i];
            perm[i] = perm[j];
            perm[j] = t;
        }
        if (cudaMemcpy(didx.p, perm, sizeof(uint32_t) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
            err = WEDGE_ERR_CUDA;
            break;
        }
        for (uint64_t b0 = 0; b0 < n; b0 += batch) {
            const uint32_t bn = (uint32_t)((n - b0) < batch ? (n - b0) : batch);
            const uint32_t blocks = blocks_for(bn);
            mlp_grad_kernel<<<blocks, MLP_THREADS>>>(dnet.as<float>(), dx.as<float>(), dy.as<float>(), dm.as<float>(),
                                                     didx.as<uint32_t>() + b0, bn, SAMPLES_PER_BLOCK, (float)bn,
                                                     dpart.as<float>(), dloss.as<double>());
            mlp_reduce_kernel<<<(WEDGE_SCHED_PARAMS + 255) / 256, 256>>>(dpart.as<float>(), blocks, dgrad.as<float>());
            bc1 *= beta1;
            bc2 *= beta2;
            mlp_adam_kernel<<<(WEDGE_SCHED_PARAMS + 255) / 256, 256>>>(dnet.as<float>(), dgrad.as<float>(),
                                                                       dmom.as<float>(), dvel.as<float>(), lr, beta1,
                                                                       beta2, eps, 1.0f - bc1, 1.0f - bc2);
        }
        if (cudaGetLastError() != cudaSuccess)
            err = WEDGE_ERR_CUDA;
    }
    free(perm);
    if (err)
        return err;
    WEDGE_CHECK(cudaMemcpy(blob, dnet.p, sizeof(float) * WEDGE_SCHED_BLOB, cudaMemcpyDeviceToHost));
    if (final_loss) {
        float* g = (float*)malloc(sizeof(float) * WEDGE_SCHED_PARAMS);
        if (!g)
            return WEDGE_ERR_OOM;
        const int r = wedge_mlp_loss_grad(blob, X, Y, M, n, final_loss, g);
        free(g);
        return r;
    }
    return WEDGE_OK;
}
