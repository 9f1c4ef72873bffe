// Learned SCF warm start: a small MLP (din -> 128 -> 128 -> 128 -> dout, SiLU) with BF16 weights,
// FP32 accumulation, FP32 master weights and Adam, trained and evaluated by these kernels.
//
// Forward: one CTA of 128 threads per 32 samples; activations of the 32 samples stay in shared
// memory, thread t computes hidden unit t for all of them (weights read as bf16 pairs).
// Backward: the same tiling in reverse; per-CTA weight gradients are reduced in shared memory and
// added to the FP32 gradient buffers with atomics.  Adam updates the FP32 masters and refreshes
// the BF16 copies used by the next forward pass.
// No counterpart in the reference (FORGE starts from the non-interacting guess or a checkpoint).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "forge_internal.cuh"

namespace forge {

constexpr int MLP_W = 128;     // hidden width
constexpr int MLP_S = 32;      // samples per CTA
constexpr int MLP_MAXIN = 64;  // max input features
constexpr int MLP_MAXOUT = 8;  // max outputs

struct MlpDims {
    int din, dout;
    // parameter offsets (elements) in the flat parameter vector
    int64_t w0, b0, w1, b1, w2, b2, w3, b3, total;
};

inline MlpDims mlp_dims(int din, int dout) {
    MlpDims d{din, dout, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    int64_t o = 0;
    d.w0 = o; o += (int64_t)MLP_W * din;
    d.b0 = o; o += MLP_W;
    d.w1 = o; o += (int64_t)MLP_W * MLP_W;
    d.b1 = o; o += MLP_W;
    d.w2 = o; o += (int64_t)MLP_W * MLP_W;
    d.b2 = o; o += MLP_W;
    d.w3 = o; o += (int64_t)dout * MLP_W;
    d.b3 = o; o += dout;
    d.total = o;
    return d;
}

__device__ inline float silu(float x) { return x / (1.f + __expf(-x)); }
__device__ inline float dsilu(float x) {
    const float s = 1.f / (1.f + __expf(-x));
    return s * (1.f + x * (1.f - s));
}

// pre-activations are stored (Z0, Z1, Z2: B x 128) for the backward pass
__global__ void __launch_bounds__(MLP_W) k_mlp_forward(MlpDims d, const __nv_bfloat16* __restrict__ W,
                                                       const float* __restrict__ X, int64_t n, float* __restrict__ Y,
                                                       float* __restrict__ Z) {
    __shared__ float h[MLP_S][MLP_W + 1];
    __shared__ float xin[MLP_S][MLP_MAXIN + 1];
    const int t = threadIdx.x;
    const int64_t s0 = (int64_t)blockIdx.x * MLP_S;
    for (int q = t; q < MLP_S * d.din; q += MLP_W) {
        const int s = q / d.din, f = q - s * d.din;
        xin[s][f] = (s0 + s < n) ? X[(s0 + s) * d.din + f] : 0.f;
    }
    __syncthreads();
    float acc[MLP_S];
    // layer 0
    {
        const float bias = __bfloat162float(W[d.b0 + t]);
#pragma unroll
        for (int s = 0; s < MLP_S; ++s) acc[s] = bias;
        for (int f = 0; f < d.din; ++f) {
            const float w = __bfloat162float(W[d.w0 + (int64_t)t * d.din + f]);
#pragma unroll
            for (int s = 0; s < MLP_S; ++s) acc[s] = fmaf(w, xin[s][f], acc[s]);
        }
#pragma unroll
        for (int s = 0; s < MLP_S; ++s) {
            if (Z && s0 + s < n) Z[(s0 + s) * 3 * MLP_W + t] = acc[s];
            h[s][t] = silu(acc[s]);
        }
    }
    __syncthreads();
    // layers 1 and 2
    for (int layer = 1; layer <= 2; ++layer) {
        const int64_t wo = layer == 1 ? d.w1 : d.w2, bo = layer == 1 ? d.b1 : d.b2;
        const float bias = __bfloat162float(W[bo + t]);
#pragma unroll
        for (int s = 0; s < MLP_S; ++s) acc[s] = bias;
        for (int f = 0; f < MLP_W; ++f) {
            const float w = __bfloat162float(W[wo + (int64_t)t * MLP_W + f]);
#pragma unroll
            for (int s = 0; s < MLP_S; ++s) acc[s] = fmaf(w, h[s][f], acc[s]);
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < MLP_S; ++s) {
            if (Z && s0 + s < n) Z[(s0 + s) * 3 * MLP_W + layer * MLP_W + t] = acc[s];
            h[s][t] = silu(acc[s]);
        }
        __syncthreads();
    }
    // output layer: thread t < dout * MLP_S computes one (sample, output)
    for (int q = t; q < MLP_S * d.dout; q += MLP_W) {
        const int s = q / d.dout, o = q - s * d.dout;
        float a = __bfloat162float(W[d.b3 + o]);
        for (int f = 0; f < MLP_W; ++f) a = fmaf(__bfloat162float(W[d.w3 + (int64_t)o * MLP_W + f]), h[s][f], a);
        if (s0 + s < n) Y[(s0 + s) * d.dout + o] = a;
    }
}

// loss = sum_s sum_o wt_o (y - target)^2 / n ; G: FP32 gradient (flat, same layout as W)
__global__ void __launch_bounds__(MLP_W) k_mlp_backward(MlpDims d, const __nv_bfloat16* __restrict__ W,
                                                        const float* __restrict__ X, const float* __restrict__ Y,
                                                        const float* __restrict__ Tgt, const float* __restrict__ wt,
                                                        const float* __restrict__ Z, int64_t n,
                                                        float* __restrict__ G, float* __restrict__ loss) {
    __shared__ float a[MLP_S][MLP_W + 1];   // activations of the current layer input
    __shared__ float g[MLP_S][MLP_W + 1];   // gradient w.r.t. pre-activations of the current layer
    __shared__ float dy[MLP_S][MLP_MAXOUT];
    __shared__ float xin[MLP_S][MLP_MAXIN + 1];
    const int t = threadIdx.x;
    const int64_t s0 = (int64_t)blockIdx.x * MLP_S;
    float lsum = 0.f;
    for (int q = t; q < MLP_S * d.dout; q += MLP_W) {
        const int s = q / d.dout, o = q - s * d.dout;
        float e = 0.f;
        if (s0 + s < n) {
            const float r = Y[(s0 + s) * d.dout + o] - Tgt[(s0 + s) * d.dout + o];
            e = 2.f * wt[o] * r / (float)n;
            lsum += wt[o] * r * r / (float)n;
        }
        dy[s][o] = e;
    }
    for (int q = t; q < MLP_S * d.din; q += MLP_W) {
        const int s = q / d.din, f = q - s * d.din;
        xin[s][f] = (s0 + s < n) ? X[(s0 + s) * d.din + f] : 0.f;
    }
    // a = h3 = silu(Z2)
#pragma unroll 4
    for (int s = 0; s < MLP_S; ++s) a[s][t] = (s0 + s < n) ? silu(Z[(s0 + s) * 3 * MLP_W + 2 * MLP_W + t]) : 0.f;
    __syncthreads();
    if (lsum != 0.f) atomicAdd(loss, lsum);
    // output layer grads: dW3[o][t] = sum_s dy[s][o] a[s][t]; db3
    for (int o = 0; o < d.dout; ++o) {
        float gw = 0.f;
        for (int s = 0; s < MLP_S; ++s) gw = fmaf(dy[s][o], a[s][t], gw);
        atomicAdd(&G[d.w3 + (int64_t)o * MLP_W + t], gw);
        if (t == 0) {
            float gb = 0.f;
            for (int s = 0; s < MLP_S; ++s) gb += dy[s][o];
            atomicAdd(&G[d.b3 + o], gb);
        }
    }
    // g = (W3^T dy) * silu'(Z2)
    for (int s = 0; s < MLP_S; ++s) {
        float v = 0.f;
        for (int o = 0; o < d.dout; ++o) v = fmaf(__bfloat162float(W[d.w3 + (int64_t)o * MLP_W + t]), dy[s][o], v);
        g[s][t] = (s0 + s < n) ? v * dsilu(Z[(s0 + s) * 3 * MLP_W + 2 * MLP_W + t]) : 0.f;
    }
    __syncthreads();
    // hidden layers 2 and 1
    for (int layer = 2; layer >= 1; --layer) {
        const int64_t wo = layer == 2 ? d.w2 : d.w1, bo = layer == 2 ? d.b2 : d.b1;
        // a = input of this layer = silu(Z[layer-1])
#pragma unroll 4
        for (int s = 0; s < MLP_S; ++s)
            a[s][t] = (s0 + s < n) ? silu(Z[(s0 + s) * 3 * MLP_W + (layer - 1) * MLP_W + t]) : 0.f;
        __syncthreads();
        // dW[t][f] for fixed t (output unit) over f: thread t owns row t
        for (int f = 0; f < MLP_W; ++f) {
            float gw = 0.f;
#pragma unroll 8
            for (int s = 0; s < MLP_S; ++s) gw = fmaf(g[s][t], a[s][f], gw);
            atomicAdd(&G[wo + (int64_t)t * MLP_W + f], gw);
        }
        {
            float gb = 0.f;
            for (int s = 0; s < MLP_S; ++s) gb += g[s][t];
            atomicAdd(&G[bo + t], gb);
        }
        // g_prev[s][t] = sum_u W[u][t] g[s][u] * silu'(Z[layer-1][t])
        float gp[MLP_S];
#pragma unroll
        for (int s = 0; s < MLP_S; ++s) gp[s] = 0.f;
        for (int u = 0; u < MLP_W; ++u) {
            const float w = __bfloat162float(W[wo + (int64_t)u * MLP_W + t]);
#pragma unroll
            for (int s = 0; s < MLP_S; ++s) gp[s] = fmaf(w, g[s][u], gp[s]);
        }
        __syncthreads();
#pragma unroll
        for (int s = 0; s < MLP_S; ++s)
            g[s][t] = (s0 + s < n) ? gp[s] * dsilu(Z[(s0 + s) * 3 * MLP_W + (layer - 1) * MLP_W + t]) : 0.f;
        __syncthreads();
    }
    // first layer: dW0[t][f] = sum_s g[s][t] x[s][f]
    for (int f = 0; f < d.din; ++f) {
        float gw = 0.f;
        for (int s = 0; s < MLP_S; ++s) gw = fmaf(g[s][t], xin[s][f], gw);
        atomicAdd(&G[d.w0 + (int64_t)t * d.din + f], gw);
    }
    {
        float gb = 0.f;
        for (int s = 0; s < MLP_S; ++s) gb += g[s][t];
        atomicAdd(&G[d.b0 + t], gb);
    }
}

__global__ void k_adam(float* __restrict__ Wm, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ G, __nv_bfloat16* __restrict__ Wb, int64_t total, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const float g = G[q];
        const float mq = b1 * m[q] + (1.f - b1) * g;
        const float vq = b2 * v[q] + (1.f - b2) * g * g;
        m[q] = mq;
        v[q] = vq;
        const float w = Wm[q] - lr * (mq / c1) / (sqrtf(vq / c2) + eps);
        Wm[q] = w;
        Wb[q] = __float2bfloat16(w);
    }
}

__global__ void k_to_bf16(const float* __restrict__ Wm, __nv_bfloat16* __restrict__ Wb, int64_t total) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x)
        Wb[q] = __float2bfloat16(Wm[q]);
}

}  // namespace forge

using namespace forge;

struct forge_mlp {
    MlpDims d;
    cudaStream_t st = nullptr;
    DevBuf Wm, Wb, m, v, G, X, Y, T, Z, wt, loss;
    int64_t cap = 0, step = 0;
};

namespace {
int mlp_capacity(forge_mlp* h, int64_t n) {
    if (n <= h->cap) return 0;
    const MlpDims& d = h->d;
    FORGE_TRY(h->X.ensure(n * d.din * sizeof(float)));
    FORGE_TRY(h->Y.ensure(n * d.dout * sizeof(float)));
    FORGE_TRY(h->T.ensure(n * d.dout * sizeof(float)));
    FORGE_TRY(h->Z.ensure(n * 3 * MLP_W * sizeof(float)));
    h->cap = n;
    return 0;
}
}  // namespace

extern "C" {

int forge_gpu_mlp_create(int64_t din, int64_t dout, uint64_t seed, forge_mlp** out) {
    if (!out || din < 1 || din > MLP_MAXIN || dout < 1 || dout > MLP_MAXOUT) {
        set_error(FORGE_ERR_ARG, "mlp_create: din must be 1..%d and dout 1..%d", MLP_MAXIN, MLP_MAXOUT);
        return FORGE_ERR_ARG;
    }
    forge_mlp* h = new forge_mlp();
    h->d = mlp_dims((int)din, (int)dout);
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        set_error(FORGE_ERR_CUDA, "mlp_create: no CUDA device");
        return FORGE_ERR_CUDA;
    }
    const int64_t P = h->d.total;
    int rc = 0;
    if ((rc = h->Wm.ensure(P * 4)) || (rc = h->Wb.ensure(P * 2)) || (rc = h->m.ensure(P * 4)) ||
        (rc = h->v.ensure(P * 4)) || (rc = h->G.ensure(P * 4)) || (rc = h->wt.ensure(MLP_MAXOUT * 4)) ||
        (rc = h->loss.ensure(4))) {
        forge_gpu_mlp_destroy(h);
        return rc;
    }
    // He-style initialisation (deterministic LCG on the host)
    std::vector<float> w(P, 0.f);
    uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto rnd = [&]() {
        s = s * 6364136223846793005ULL + 1442695040888963407ULL;
        return ((double)(s >> 11) / 9007199254740992.0) * 2.0 - 1.0;
    };
    const MlpDims& d = h->d;
    auto fill = [&](int64_t off, int64_t cnt, double scale) {
        for (int64_t q = 0; q < cnt; ++q) w[off + q] = (float)(rnd() * scale);
    };
    fill(d.w0, (int64_t)MLP_W * d.din, std::sqrt(3.0 / d.din));
    fill(d.w1, (int64_t)MLP_W * MLP_W, std::sqrt(3.0 / MLP_W));
    fill(d.w2, (int64_t)MLP_W * MLP_W, std::sqrt(3.0 / MLP_W));
    fill(d.w3, (int64_t)d.dout * MLP_W, std::sqrt(3.0 / MLP_W) * 0.1);
    std::vector<float> ones(MLP_MAXOUT, 1.f);
    if (cudaMemcpy(h->Wm.ptr, w.data(), P * 4, cudaMemcpyHostToDevice) ||
        cudaMemset(h->m.ptr, 0, P * 4) || cudaMemset(h->v.ptr, 0, P * 4) ||
        cudaMemcpy(h->wt.ptr, ones.data(), MLP_MAXOUT * 4, cudaMemcpyHostToDevice)) {
        forge_gpu_mlp_destroy(h);
        set_error(FORGE_ERR_CUDA, "mlp_create: upload failed");
        return FORGE_ERR_CUDA;
    }
    k_to_bf16<<<64, 256, 0, h->st>>>(h->Wm.as<float>(), h->Wb.as<__nv_bfloat16>(), P);
    cudaStreamSynchronize(h->st);
    *out = h;
    return 0;
}

int forge_gpu_mlp_destroy(forge_mlp* h) {
    if (!h) return 0;
    DevBuf* b[] = {&h->Wm, &h->Wb, &h->m, &h->v, &h->G, &h->X, &h->Y, &h->T, &h->Z, &h->wt, &h->loss};
    for (DevBuf* x : b) x->release();
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return 0;
}

int64_t forge_gpu_mlp_num_params(forge_mlp* h) { return h ? h->d.total : 0; }

int forge_gpu_mlp_set_params(forge_mlp* h, const float* W) {
    if (!h || !W) return FORGE_ERR_ARG;
    FORGE_CUDA(cudaMemcpyAsync(h->Wm.ptr, W, h->d.total * 4, cudaMemcpyHostToDevice, h->st));
    k_to_bf16<<<64, 256, 0, h->st>>>(h->Wm.as<float>(), h->Wb.as<__nv_bfloat16>(), h->d.total);
    FORGE_LAUNCH_CHECK();
    FORGE_CUDA(cudaMemsetAsync(h->m.ptr, 0, h->d.total * 4, h->st));
    FORGE_CUDA(cudaMemsetAsync(h->v.ptr, 0, h->d.total * 4, h->st));
    h->step = 0;
    FORGE_CUDA(cudaStreamSynchronize(h->st));
    return 0;
}

// FP32 master parameters (W) and, optionally, the BF16 copies actually used (as floats)
int forge_gpu_mlp_get_params(forge_mlp* h, float* W, float* Wbf16) {
    if (!h) return FORGE_ERR_ARG;
    if (W) FORGE_CUDA(cudaMemcpyAsync(W, h->Wm.ptr, h->d.total * 4, cudaMemcpyDeviceToHost, h->st));
    std::vector<__nv_bfloat16> tmp;
    if (Wbf16) {
        tmp.resize(h->d.total);
        FORGE_CUDA(cudaMemcpyAsync(tmp.data(), h->Wb.ptr, h->d.total * 2, cudaMemcpyDeviceToHost, h->st));
    }
    FORGE_CUDA(cudaStreamSynchronize(h->st));
    if (Wbf16)
        for (int64_t q = 0; q < h->d.total; ++q) Wbf16[q] = __bfloat162float(tmp[q]);
    return 0;
}

int forge_gpu_mlp_set_loss_weights(forge_mlp* h, const float* wt) {
    if (!h || !wt) return FORGE_ERR_ARG;
    FORGE_CUDA(cudaMemcpy(h->wt.ptr, wt, h->d.dout * 4, cudaMemcpyHostToDevice));
    return 0;
}

int forge_gpu_mlp_forward(forge_mlp* h, const float* X, int64_t n, float* Y) {
    if (!h || !X || !Y || n < 1) return FORGE_ERR_ARG;
    FORGE_TRY(mlp_capacity(h, n));
    const MlpDims& d = h->d;
    FORGE_CUDA(cudaMemcpyAsync(h->X.ptr, X, n * d.din * 4, cudaMemcpyHostToDevice, h->st));
    k_mlp_forward<<<(unsigned)((n + MLP_S - 1) / MLP_S), MLP_W, 0, h->st>>>(d, h->Wb.as<__nv_bfloat16>(),
                                                                              h->X.as<float>(), n, h->Y.as<float>(),
                                                                              nullptr);
    FORGE_LAUNCH_CHECK();
    FORGE_CUDA(cudaMemcpyAsync(Y, h->Y.ptr, n * d.dout * 4, cudaMemcpyDeviceToHost, h->st));
    FORGE_CUDA(cudaStreamSynchronize(h->st));
    return 0;
}

// gradient of the weighted MSE w.r.t. the parameters (G, flat) and the loss, at the current weights
int forge_gpu_mlp_gradient(forge_mlp* h, const float* X, const float* Tg, int64_t n, float* G, float* loss) {
    if (!h || !X || !Tg || n < 1) return FORGE_ERR_ARG;
    FORGE_TRY(mlp_capacity(h, n));
    const MlpDims& d = h->d;
    FORGE_CUDA(cudaMemcpyAsync(h->X.ptr, X, n * d.din * 4, cudaMemcpyHostToDevice, h->st));
    FORGE_CUDA(cudaMemcpyAsync(h->T.ptr, Tg, n * d.dout * 4, cudaMemcpyHostToDevice, h->st));
    FORGE_CUDA(cudaMemsetAsync(h->G.ptr, 0, d.total * 4, h->st));
    FORGE_CUDA(cudaMemsetAsync(h->loss.ptr, 0, 4, h->st));
    const unsigned nb = (unsigned)((n + MLP_S - 1) / MLP_S);
    k_mlp_forward<<<nb, MLP_W, 0, h->st>>>(d, h->Wb.as<__nv_bfloat16>(), h->X.as<float>(), n, h->Y.as<float>(),
                                           h->Z.as<float>());
    FORGE_LAUNCH_CHECK();
    k_mlp_backward<<<nb, MLP_W, 0, h->st>>>(d, h->Wb.as<__nv_bfloat16>(), h->X.as<float>(), h->Y.as<float>(),
                                            h->T.as<float>(), h->wt.as<float>(), h->Z.as<float>(), n,
                                            h->G.as<float>(), h->loss.as<float>());
    FORGE_LAUNCH_CHECK();
    if (G) FORGE_CUDA(cudaMemcpyAsync(G, h->G.ptr, d.total * 4, cudaMemcpyDeviceToHost, h->st));
    if (loss) FORGE_CUDA(cudaMemcpyAsync(loss, h->loss.ptr, 4, cudaMemcpyDeviceToHost, h->st));
    FORGE_CUDA(cudaStreamSynchronize(h->st));
    return 0;
}

// Adam training on device-resident data: `epochs` passes of minibatches of size `bs` over the n
// samples in a fixed shuffled order (seeded); returns the mean loss of the last epoch.
int forge_gpu_mlp_train(forge_mlp* h, const float* X, const float* Tg, int64_t n, int64_t epochs, int64_t bs,
                        double lr, uint64_t seed, float* last_loss) {
    if (!h || !X || !Tg || n < 1 || epochs < 1 || bs < 1) return FORGE_ERR_ARG;
    const MlpDims& d = h->d;
    // permuted copies per epoch are built on the host (n is at most a few 10^5)
    std::vector<int64_t> perm(n);
    for (int64_t q = 0; q < n; ++q) perm[q] = q;
    std::vector<float> xb((size_t)n * d.din), tb((size_t)n * d.dout);
    uint64_t s = seed * 2862933555777941757ULL + 3037000493ULL;
    DevBuf dX, dT;
    FORGE_TRY(dX.ensure(n * d.din * 4));
    FORGE_TRY(dT.ensure(n * d.dout * 4));
    FORGE_TRY(mlp_capacity(h, bs));
    float lsum = 0.f;
    for (int64_t ep = 0; ep < epochs; ++ep) {
        for (int64_t q = n - 1; q > 0; --q) {
            s = s * 6364136223846793005ULL + 1442695040888963407ULL;
            int64_t r = (int64_t)((s >> 33) % (uint64_t)(q + 1));
            std::swap(perm[q], perm[r]);
        }
        for (int64_t q = 0; q < n; ++q) {
            std::memcpy(&xb[q * d.din], &X[perm[q] * d.din], d.din * 4);
            std::memcpy(&tb[q * d.dout], &Tg[perm[q] * d.dout], d.dout * 4);
        }
        FORGE_CUDA(cudaMemcpyAsync(dX.ptr, xb.data(), n * d.din * 4, cudaMemcpyHostToDevice, h->st));
        FORGE_CUDA(cudaMemcpyAsync(dT.ptr, tb.data(), n * d.dout * 4, cudaMemcpyHostToDevice, h->st));
        FORGE_CUDA(cudaMemsetAsync(h->loss.ptr, 0, 4, h->st));
        int64_t nbatch = 0;
        for (int64_t b0 = 0; b0 < n; b0 += bs) {
            const int64_t m = (n - b0 < bs) ? n - b0 : bs;
            const float* xp = dX.as<float>() + b0 * d.din;
            const float* tp = dT.as<float>() + b0 * d.dout;
            FORGE_CUDA(cudaMemsetAsync(h->G.ptr, 0, d.total * 4, h->st));
            const unsigned nb = (unsigned)((m + MLP_S - 1) / MLP_S);
            k_mlp_forward<<<nb, MLP_W, 0, h->st>>>(d, h->Wb.as<__nv_bfloat16>(), xp, m, h->Y.as<float>(),
                                                   h->Z.as<float>());
            FORGE_LAUNCH_CHECK();
            k_mlp_backward<<<nb, MLP_W, 0, h->st>>>(d, h->Wb.as<__nv_bfloat16>(), xp, h->Y.as<float>(), tp,
                                                    h->wt.as<float>(), h->Z.as<float>(), m, h->G.as<float>(),
                                                    h->loss.as<float>());
            FORGE_LAUNCH_CHECK();
            ++h->step;
            const float c1 = 1.f - std::pow(0.9f, (float)h->step), c2 = 1.f - std::pow(0.999f, (float)h->step);
            k_adam<<<256, 256, 0, h->st>>>(h->Wm.as<float>(), h->m.as<float>(), h->v.as<float>(), h->G.as<float>(),
                                           h->Wb.as<__nv_bfloat16>(), d.total, (float)lr, 0.9f, 0.999f, 1e-8f, c1, c2);
            FORGE_LAUNCH_CHECK();
            ++nbatch;
        }
        FORGE_CUDA(cudaMemcpyAsync(&lsum, h->loss.ptr, 4, cudaMemcpyDeviceToHost, h->st));
        FORGE_CUDA(cudaStreamSynchronize(h->st));
        lsum /= (float)nbatch;
    }
    dX.release();
    dT.release();
    if (last_loss) *last_loss = lsum;
    return 0;
}

}  // extern "C"
