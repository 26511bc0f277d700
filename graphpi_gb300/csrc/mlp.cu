// Learned schedule cost model: a two-layer perceptron (in -> hidden ReLU ->
// 1), fp32, trained full-batch with Adam on the GPU.  It scores candidate
// loop orders by predicted log runtime, the role the reference gives its
// analytic model (Schedule::our_estimate_schedule_restrict,
// src/schedule.cpp:1487-1574).  No reference counterpart.
//
// Parameters are one flat array: W1[hidden][in], b1[hidden], W2[hidden], b2.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "gpm_internal.h"

namespace gpm {

#define MLP_CK(call)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            set_error("%s failed: %s", #call, cudaGetErrorString(e_));                            \
            return e_ == cudaErrorMemoryAllocation ? GPM_ERR_OOM : GPM_ERR_CUDA;                 \
        }                                                                                         \
    } while (0)

constexpr int kMlpMaxIn = 128;
constexpr int kMlpMaxHidden = 256;

// One block per row (grid-stride); thread j owns hidden unit j.
__global__ void mlp_forward_kernel(const float* __restrict__ X, int N, int D, int H, const float* __restrict__ P,
                                   float* __restrict__ Hact, float* __restrict__ Y) {
    __shared__ float xs[kMlpMaxIn];
    __shared__ float red[kMlpMaxHidden / 32];
    const float* W1 = P;
    const float* b1 = W1 + (size_t)H * D;
    const float* W2 = b1 + H;
    const float b2 = W2[H];
    const int j = threadIdx.x;
    for (int r = blockIdx.x; r < N; r += gridDim.x) {
        for (int k = j; k < D; k += blockDim.x) xs[k] = X[(size_t)r * D + k];
        __syncthreads();
        float h = 0.f;
        if (j < H) {
            float a = b1[j];
            const float* w = W1 + (size_t)j * D;
            for (int k = 0; k < D; ++k) a = fmaf(w[k], xs[k], a);
            h = a > 0.f ? a : 0.f;
            if (Hact) Hact[(size_t)r * H + j] = h;
        }
        float part = j < H ? W2[j] * h : 0.f;
        for (int o = 16; o >= 1; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((j & 31) == 0) red[j >> 5] = part;
        __syncthreads();
        if (j == 0) {
            float y = b2;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) y += red[w];
            Y[r] = y;
        }
        __syncthreads();
    }
}

// Gradients of mean squared error, accumulated per block in shared memory
// and added to G once per block.  loss receives the mean squared error.
__global__ void mlp_backward_kernel(const float* __restrict__ X, const float* __restrict__ T, int N, int D, int H,
                                    const float* __restrict__ P, const float* __restrict__ Hact,
                                    const float* __restrict__ Y, float* __restrict__ G, float* __restrict__ loss) {
    extern __shared__ float acc[];  // H*D + H + H + 1 + D
    const int j = threadIdx.x;
    const int nparam = H * D + 2 * H + 1;
    float* xs = acc + nparam;
    for (int i = j; i < nparam; i += blockDim.x) acc[i] = 0.f;
    __syncthreads();
    const float* W2 = P + (size_t)H * D + H;
    float lsum = 0.f;
    for (int r = blockIdx.x; r < N; r += gridDim.x) {
        for (int k = j; k < D; k += blockDim.x) xs[k] = X[(size_t)r * D + k];
        __syncthreads();
        const float diff = Y[r] - T[r];
        const float dy = 2.f * diff / (float)N;
        if (j == 0) {
            acc[nparam - 1] += dy;
            lsum += diff * diff / (float)N;
        }
        if (j < H) {
            const float h = Hact[(size_t)r * H + j];
            acc[H * D + H + j] += dy * h;
            const float dh = h > 0.f ? dy * W2[j] : 0.f;
            acc[H * D + j] += dh;
            float* gw = acc + (size_t)j * D;
            for (int k = 0; k < D; ++k) gw[k] = fmaf(dh, xs[k], gw[k]);
        }
        __syncthreads();
    }
    for (int i = j; i < nparam; i += blockDim.x)
        if (acc[i] != 0.f) atomicAdd(&G[i], acc[i]);
    if (j == 0 && lsum != 0.f) atomicAdd(loss, lsum);
}

__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M,
                            float* __restrict__ V, int n, float lr, float beta1, float beta2, float eps, float c1,
                            float c2, float wd) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float g = G[i] + wd * P[i];
        const float m = beta1 * M[i] + (1.f - beta1) * g;
        const float v = beta2 * V[i] + (1.f - beta2) * g * g;
        M[i] = m;
        V[i] = v;
        P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

}  // namespace gpm

using namespace gpm;

struct gpm_mlp {
    int in = 0, hidden = 0, nparam = 0;
    int device = 0;
    float* P = nullptr;  // device parameters
    float* M = nullptr;  // Adam moments
    float* V = nullptr;
    long long step = 0;
    ~gpm_mlp() {
        if (P) cudaFree(P);
        if (M) cudaFree(M);
        if (V) cudaFree(V);
    }
};

namespace {

struct Batch {
    float* X = nullptr;
    float* T = nullptr;
    float* Y = nullptr;
    float* H = nullptr;
    float* G = nullptr;
    float* loss = nullptr;
    ~Batch() {
        for (float* p : {X, T, Y, H, G, loss})
            if (p) cudaFree(p);
    }
};

int upload(gpm_mlp* m, const float* X, const float* T, int N, Batch& b, bool need_grad) {
    MLP_CK(cudaMalloc(&b.X, sizeof(float) * (size_t)N * m->in));
    MLP_CK(cudaMalloc(&b.Y, sizeof(float) * (size_t)N));
    MLP_CK(cudaMemcpy(b.X, X, sizeof(float) * (size_t)N * m->in, cudaMemcpyHostToDevice));
    if (need_grad) {
        MLP_CK(cudaMalloc(&b.T, sizeof(float) * (size_t)N));
        MLP_CK(cudaMalloc(&b.H, sizeof(float) * (size_t)N * m->hidden));
        MLP_CK(cudaMalloc(&b.G, sizeof(float) * (size_t)m->nparam));
        MLP_CK(cudaMalloc(&b.loss, sizeof(float)));
        MLP_CK(cudaMemcpy(b.T, T, sizeof(float) * (size_t)N, cudaMemcpyHostToDevice));
    }
    return GPM_OK;
}

int threads_for(int hidden) { return ((hidden + 31) / 32) * 32; }

int grid_for(int N) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, std::min(N, sms * 4));
}

size_t bwd_smem(const gpm_mlp* m) { return sizeof(float) * ((size_t)m->hidden * m->in + 2 * m->hidden + 1 + m->in); }

int forward_backward(gpm_mlp* m, Batch& b, int N, bool grad) {
    const int th = threads_for(m->hidden), gr = grid_for(N);
    mlp_forward_kernel<<<gr, th>>>(b.X, N, m->in, m->hidden, m->P, grad ? b.H : nullptr, b.Y);
    MLP_CK(cudaGetLastError());
    if (!grad) return GPM_OK;
    MLP_CK(cudaMemset(b.G, 0, sizeof(float) * (size_t)m->nparam));
    MLP_CK(cudaMemset(b.loss, 0, sizeof(float)));
    mlp_backward_kernel<<<gr, th, bwd_smem(m)>>>(b.X, b.T, N, m->in, m->hidden, m->P, b.H, b.Y, b.G, b.loss);
    MLP_CK(cudaGetLastError());
    return GPM_OK;
}

}  // namespace

extern "C" {

GPM_API int gpm_mlp_create(int32_t in_dim, int32_t hidden, uint64_t seed, gpm_mlp** out) {
    clear_error();
    if (!out || in_dim < 1 || in_dim > kMlpMaxIn || hidden < 1 || hidden > kMlpMaxHidden) {
        set_error("gpm_mlp_create: in_dim must be 1..%d and hidden 1..%d", kMlpMaxIn, kMlpMaxHidden);
        return GPM_ERR_INVALID_ARG;
    }
    gpm_mlp* m = new gpm_mlp();
    m->in = in_dim;
    m->hidden = hidden;
    m->nparam = hidden * in_dim + 2 * hidden + 1;
    cudaGetDevice(&m->device);
    // He-style init from a counter-based generator
    std::vector<float> p(m->nparam, 0.f);
    uint64_t x = seed ^ 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (float)((double)(z >> 11) / 9007199254740992.0);
    };
    const float s1 = std::sqrt(6.f / (float)in_dim), s2 = std::sqrt(6.f / (float)hidden);
    for (int i = 0; i < hidden * in_dim; ++i) p[i] = (2.f * uni() - 1.f) * s1;
    for (int i = 0; i < hidden; ++i) p[hidden * in_dim + hidden + i] = (2.f * uni() - 1.f) * s2;
    if (cudaMalloc(&m->P, sizeof(float) * m->nparam) != cudaSuccess ||
        cudaMalloc(&m->M, sizeof(float) * m->nparam) != cudaSuccess ||
        cudaMalloc(&m->V, sizeof(float) * m->nparam) != cudaSuccess ||
        cudaMemcpy(m->P, p.data(), sizeof(float) * m->nparam, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->M, 0, sizeof(float) * m->nparam) != cudaSuccess ||
        cudaMemset(m->V, 0, sizeof(float) * m->nparam) != cudaSuccess) {
        set_error("gpm_mlp_create: %s", cudaGetErrorString(cudaGetLastError()));
        delete m;
        return GPM_ERR_CUDA;
    }
    if (bwd_smem(m) > 48 * 1024)
        cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem(m));
    *out = m;
    return GPM_OK;
}

GPM_API int gpm_mlp_destroy(gpm_mlp* m) {
    delete m;
    return GPM_OK;
}

GPM_API int gpm_mlp_params(gpm_mlp* m, float* host, int32_t n, int32_t set) {
    clear_error();
    if (!m || !host || n != m->nparam) {
        set_error("gpm_mlp_params: need %d floats", m ? m->nparam : -1);
        return GPM_ERR_INVALID_ARG;
    }
    if (set) {
        MLP_CK(cudaMemcpy(m->P, host, sizeof(float) * n, cudaMemcpyHostToDevice));
        MLP_CK(cudaMemset(m->M, 0, sizeof(float) * n));
        MLP_CK(cudaMemset(m->V, 0, sizeof(float) * n));
        m->step = 0;
    } else {
        MLP_CK(cudaMemcpy(host, m->P, sizeof(float) * n, cudaMemcpyDeviceToHost));
    }
    return GPM_OK;
}

GPM_API int gpm_mlp_forward(gpm_mlp* m, const float* X, int32_t n_rows, float* Y) {
    clear_error();
    if (!m || !X || !Y || n_rows < 1) return GPM_ERR_INVALID_ARG;
    Batch b;
    int rc = upload(m, X, nullptr, n_rows, b, false);
    if (rc) return rc;
    rc = forward_backward(m, b, n_rows, false);
    if (rc) return rc;
    MLP_CK(cudaMemcpy(Y, b.Y, sizeof(float) * n_rows, cudaMemcpyDeviceToHost));
    return GPM_OK;
}

GPM_API int gpm_mlp_gradients(gpm_mlp* m, const float* X, const float* T, int32_t n_rows, float* grads,
                              float* loss) {
    clear_error();
    if (!m || !X || !T || !grads || n_rows < 1) return GPM_ERR_INVALID_ARG;
    Batch b;
    int rc = upload(m, X, T, n_rows, b, true);
    if (rc) return rc;
    rc = forward_backward(m, b, n_rows, true);
    if (rc) return rc;
    MLP_CK(cudaMemcpy(grads, b.G, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost));
    if (loss) MLP_CK(cudaMemcpy(loss, b.loss, sizeof(float), cudaMemcpyDeviceToHost));
    return GPM_OK;
}

GPM_API int gpm_mlp_train(gpm_mlp* m, const float* X, const float* T, int32_t n_rows, int32_t epochs, float lr,
                          float weight_decay, float* final_loss) {
    clear_error();
    if (!m || !X || !T || n_rows < 1 || epochs < 1 || !(lr > 0.f)) return GPM_ERR_INVALID_ARG;
    Batch b;
    int rc = upload(m, X, T, n_rows, b, true);
    if (rc) return rc;
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const int ag = std::max(1, std::min(1024, (m->nparam + 255) / 256));
    for (int e = 0; e < epochs; ++e) {
        rc = forward_backward(m, b, n_rows, true);
        if (rc) return rc;
        ++m->step;
        const float c1 = 1.f - std::pow(beta1, (float)m->step), c2 = 1.f - std::pow(beta2, (float)m->step);
        adam_kernel<<<ag, 256>>>(m->P, b.G, m->M, m->V, m->nparam, lr, beta1, beta2, eps, c1, c2, weight_decay);
        MLP_CK(cudaGetLastError());
    }
    MLP_CK(cudaDeviceSynchronize());
    if (final_loss) MLP_CK(cudaMemcpy(final_loss, b.loss, sizeof(float), cudaMemcpyDeviceToHost));
    return GPM_OK;
}

}  // extern "C"
