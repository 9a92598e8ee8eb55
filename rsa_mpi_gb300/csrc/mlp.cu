// mlp.cu -- the 16-64-64-2 network of the learned subdivision schedule: BF16 weights, FP32 accumulation.
//
// Layout of the 5378 weights (row major): W1[64][16], b1[64], W2[64][64], b2[64], W3[2][64], b3[2].
// Forward: h1 = relu(W1 x + b1), h2 = relu(W2 h1 + b2), y = W3 h2 + b3.  The two outputs are the
// predicted remaining time after each action (y[0] = one more dart pass, y[1] = subdivide now).
//
// Training: mean squared error over the outputs whose target is finite (the action taken), gradients of
// every weight accumulated in FP32, SGD on FP32 master weights, BF16 copies refreshed after each step.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/rsagpu.h"
#include "rsa_ops.h"

namespace rsagpu {
namespace {

constexpr int NI = 16, NH = 64, NO = 2;
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NO * NH;
constexpr int NW = OB3 + NO;  // 5378
static_assert(NW == 5378, "weight layout");

__device__ __forceinline__ float bf(const __nv_bfloat16* w, int i) { return __bfloat162float(w[i]); }

// One block of NH threads per group of samples; thread j owns hidden unit j of both layers.
__device__ __forceinline__ void forward_one(const __nv_bfloat16* w, const float* x, float* h1, float* h2, float* y,
                                            int j) {
    float a = bf(w, OB1 + j);
#pragma unroll
    for (int i = 0; i < NI; i++) a += bf(w, OW1 + j * NI + i) * x[i];
    h1[j] = a > 0.f ? a : 0.f;
    __syncthreads();
    float b = bf(w, OB2 + j);
#pragma unroll 8
    for (int i = 0; i < NH; i++) b += bf(w, OW2 + j * NH + i) * h1[i];
    h2[j] = b > 0.f ? b : 0.f;
    __syncthreads();
    if (j < NO) {
        float c = bf(w, OB3 + j);
#pragma unroll 8
        for (int i = 0; i < NH; i++) c += bf(w, OW3 + j * NH + i) * h2[i];
        y[j] = c;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NH) k_mlp_forward(const __nv_bfloat16* wg, const float* x, uint64_t n, float* y) {
    __shared__ __nv_bfloat16 w[NW];
    __shared__ float xs[NI], h1[NH], h2[NH], ys[NO];
    for (int i = threadIdx.x; i < NW; i += NH) w[i] = wg[i];
    __syncthreads();
    for (uint64_t s = blockIdx.x; s < n; s += gridDim.x) {
        if (threadIdx.x < NI) xs[threadIdx.x] = x[s * NI + threadIdx.x];
        __syncthreads();
        forward_one(w, xs, h1, h2, ys, threadIdx.x);
        if (threadIdx.x < NO) y[s * NO + threadIdx.x] = ys[threadIdx.x];
        __syncthreads();
    }
}

// Gradients of the mean squared error; n_valid = number of finite targets over the batch.
__global__ void __launch_bounds__(NH) k_mlp_grad(const __nv_bfloat16* wg, const float* x, const float* t, uint64_t n,
                                                 float inv_valid, float* grad, float* loss) {
    __shared__ __nv_bfloat16 w[NW];
    __shared__ float xs[NI], h1[NH], h2[NH], ys[NO], dy[NO], dh2[NH];
    const int j = threadIdx.x;
    for (int i = j; i < NW; i += NH) w[i] = wg[i];
    __syncthreads();
    // per-thread gradient rows in registers: W1 row j, b1[j], W2 row j, b2[j]; W3/b3 by threads < NO
    float gW1[NI], gW2[NH], gb1 = 0.f, gb2 = 0.f, gW3[NH], gb3 = 0.f, lsum = 0.f;
#pragma unroll
    for (int i = 0; i < NI; i++) gW1[i] = 0.f;
#pragma unroll
    for (int i = 0; i < NH; i++) {
        gW2[i] = 0.f;
        gW3[i] = 0.f;
    }
    for (uint64_t s = blockIdx.x; s < n; s += gridDim.x) {
        if (j < NI) xs[j] = x[s * NI + j];
        __syncthreads();
        forward_one(w, xs, h1, h2, ys, j);
        if (j < NO) {
            const float tv = t[s * NO + j];
            const bool valid = isfinite(tv);
            const float e = valid ? ys[j] - tv : 0.f;
            dy[j] = 2.f * e * inv_valid;
            lsum += e * e * inv_valid;
        }
        __syncthreads();
        // output layer: thread o < NO owns row o of W3
        if (j < NO) {
#pragma unroll 8
            for (int i = 0; i < NH; i++) gW3[i] += dy[j] * h2[i];
            gb3 += dy[j];
        }
        // hidden layer 2: dh2[j] = sum_o W3[o][j] dy[o] * relu'(h2[j])
        float d2 = 0.f;
#pragma unroll
        for (int o = 0; o < NO; o++) d2 += bf(w, OW3 + o * NH + j) * dy[o];
        d2 = h2[j] > 0.f ? d2 : 0.f;
        dh2[j] = d2;
#pragma unroll 8
        for (int i = 0; i < NH; i++) gW2[i] += d2 * h1[i];
        gb2 += d2;
        __syncthreads();
        // hidden layer 1: dh1[j] = sum_k W2[k][j] dh2[k] * relu'(h1[j])
        float d1 = 0.f;
#pragma unroll 8
        for (int k = 0; k < NH; k++) d1 += bf(w, OW2 + k * NH + j) * dh2[k];
        d1 = h1[j] > 0.f ? d1 : 0.f;
#pragma unroll
        for (int i = 0; i < NI; i++) gW1[i] += d1 * xs[i];
        gb1 += d1;
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < NI; i++) atomicAdd(grad + OW1 + j * NI + i, gW1[i]);
    atomicAdd(grad + OB1 + j, gb1);
#pragma unroll 8
    for (int i = 0; i < NH; i++) atomicAdd(grad + OW2 + j * NH + i, gW2[i]);
    atomicAdd(grad + OB2 + j, gb2);
    if (j < NO) {
#pragma unroll 8
        for (int i = 0; i < NH; i++) atomicAdd(grad + OW3 + j * NH + i, gW3[i]);
        atomicAdd(grad + OB3 + j, gb3);
        atomicAdd(loss, lsum);
    }
}

__global__ void k_sgd(float* master, __nv_bfloat16* wb, const float* grad, float lr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NW) return;
    master[i] -= lr * grad[i];
    wb[i] = __float2bfloat16_rn(master[i]);
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

int cuda_fail(cudaError_t e) {
    set_last_error(cudaGetErrorString(e));
    return RSAGPU_ERR_CUDA;
}

}  // namespace

// Decision of the learned schedule for one round: y = MLP(features) on the device (weights resident).
int mlp_decide(const uint16_t* d_weights, const float* d_features, float* d_out, cudaStream_t s) {
    k_mlp_forward<<<1, NH, 0, s>>>((const __nv_bfloat16*)d_weights, d_features, 1, d_out);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RSAGPU_OK : cuda_fail(e);
}

}  // namespace rsagpu

using namespace rsagpu;

extern "C" int rsagpu_mlp_forward(const uint16_t* weights_bf16, const float* x, uint64_t n, float* y) {
    if (!weights_bf16 || (n > 0 && (!x || !y))) {
        set_last_error("rsagpu_mlp_forward: null argument");
        return RSAGPU_ERR_ARG;
    }
    if (n == 0) return RSAGPU_OK;
    DevBuf w, dx, dy;
    cudaError_t e;
    if ((e = cudaMalloc(&w.p, NW * sizeof(uint16_t))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&dx.p, n * NI * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&dy.p, n * NO * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    cudaMemcpy(w.p, weights_bf16, NW * sizeof(uint16_t), cudaMemcpyHostToDevice);
    cudaMemcpy(dx.p, x, n * NI * sizeof(float), cudaMemcpyHostToDevice);
    const unsigned nb = (unsigned)std::min<uint64_t>(n, 152 * 16);
    k_mlp_forward<<<nb, NH>>>((const __nv_bfloat16*)w.p, (const float*)dx.p, n, (float*)dy.p);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMemcpy(y, dy.p, n * NO * sizeof(float), cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_fail(e);
    return RSAGPU_OK;
}

extern "C" int rsagpu_mlp_train_step(float* master_weights, uint16_t* weights_bf16, const float* x, const float* target,
                                     uint64_t n, float lr, float* loss_out, float* grad_out) {
    if (!master_weights || !weights_bf16 || !x || !target || n == 0) {
        set_last_error("rsagpu_mlp_train_step: null argument or empty batch");
        return RSAGPU_ERR_ARG;
    }
    uint64_t valid = 0;
    for (uint64_t i = 0; i < n * NO; i++) valid += std::isfinite(target[i]) ? 1 : 0;
    if (valid == 0) {
        set_last_error("rsagpu_mlp_train_step: no finite target");
        return RSAGPU_ERR_ARG;
    }
    DevBuf m, wb, dx, dt, g, l;
    cudaError_t e;
    if ((e = cudaMalloc(&m.p, NW * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&wb.p, NW * sizeof(uint16_t))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&dx.p, n * NI * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&dt.p, n * NO * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&g.p, NW * sizeof(float))) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaMalloc(&l.p, sizeof(float))) != cudaSuccess) return cuda_fail(e);
    cudaMemcpy(m.p, master_weights, NW * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(wb.p, weights_bf16, NW * sizeof(uint16_t), cudaMemcpyHostToDevice);
    cudaMemcpy(dx.p, x, n * NI * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dt.p, target, n * NO * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemset(g.p, 0, NW * sizeof(float));
    cudaMemset(l.p, 0, sizeof(float));
    const unsigned nb = (unsigned)std::min<uint64_t>((n + 15) / 16, 152 * 4);
    k_mlp_grad<<<nb, NH>>>((const __nv_bfloat16*)wb.p, (const float*)dx.p, (const float*)dt.p, n, 1.0f / (float)valid,
                           (float*)g.p, (float*)l.p);
    k_sgd<<<(NW + 255) / 256, 256>>>((float*)m.p, (__nv_bfloat16*)wb.p, (const float*)g.p, lr);
    count_launch(2);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e);
    cudaMemcpy(master_weights, m.p, NW * sizeof(float), cudaMemcpyDeviceToHost);
    cudaMemcpy(weights_bf16, wb.p, NW * sizeof(uint16_t), cudaMemcpyDeviceToHost);
    if (grad_out) cudaMemcpy(grad_out, g.p, NW * sizeof(float), cudaMemcpyDeviceToHost);
    float loss = 0;
    if ((e = cudaMemcpy(&loss, l.p, sizeof(float), cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_fail(e);
    if (loss_out) *loss_out = loss;
    return RSAGPU_OK;
}
