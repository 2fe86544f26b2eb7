// mlp.cu - training and inference kernels of the SHAKE-seeding network (mlp.cuh).
//
//   k_mlp_forward  one thread per sample
//   k_mlp_grad     a block of 128 samples: forward with stored pre-activations, backward deltas,
//                  then the batch sums of the weight gradients (each thread a slice of the
//                  parameters, summing over the block's samples in shared memory), one global
//                  atomic per parameter and block
//   k_mlp_adam     Adam step on the FP32 master weights
// The loss is the mean squared error in normalised output units.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "ctx.h"
#include "mlp.cuh"

namespace mdg {

namespace {

using namespace mlp;
constexpr int kB = 128;  // samples per gradient block

__global__ void k_mlp_round(const float* master, float* wr, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        wr[i] = i < NPARAM ? bf16r(master[i]) : master[i];
}

__global__ void k_mlp_forward(const float* Wg, const float* X, float* Y, int n) {
    __shared__ float W[NW];
    for (int i = threadIdx.x; i < NW; i += blockDim.x) W[i] = Wg[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float in[NI], out[NO];
    for (int i = 0; i < NI; ++i) in[i] = X[s * NI + i];
    forward(W, in, out);
    for (int c = 0; c < NO; ++c) Y[s * NO + c] = out[c];
}

// shared layout of k_mlp_grad
struct GradSmem {
    float W[NW];
    float x[kB][NI + 1];
    float z1[kB][NH + 1];
    float z2[kB][NH + 1];
    float d1[kB][NH + 1];
    float d2[kB][NH + 1];
    float d3[kB][4];
};

// gradient of sum_s ||(y_s - t_s)/ystd||^2 / nb over the samples idx[b0 .. b0+nb)
__global__ void __launch_bounds__(kB) k_mlp_grad(const float* Wg, const float* X, const float* T, const int* idx,
                                                 int b0, int nb, float inv_norm, float* grad, float* loss) {
    extern __shared__ __align__(16) unsigned char smraw[];
    GradSmem& S = *reinterpret_cast<GradSmem*>(smraw);
    for (int i = threadIdx.x; i < NW; i += blockDim.x) S.W[i] = Wg[i];
    __syncthreads();
    const float* W = S.W;
    const int t = threadIdx.x;
    const int sidx = blockIdx.x * kB + t;
    const bool ok = sidx < nb;
    float lsum = 0.f;
    {
        float x[NI];
        const int g = ok ? idx[b0 + sidx] : 0;
#pragma unroll
        for (int i = 0; i < NI; ++i) x[i] = ok ? (X[(size_t)g * NI + i] - W[OXM + i]) * W[OXS + i] : 0.f;
#pragma unroll
        for (int i = 0; i < NI; ++i) S.x[t][i] = x[i];
        float h1[NH];
        for (int o = 0; o < NH; ++o) {
            float z = W[OB1 + o];
#pragma unroll
            for (int i = 0; i < NI; ++i) z = fmaf(W[OW1 + o * NI + i], x[i], z);
            S.z1[t][o] = z;
            h1[o] = silu(z);
        }
        float y[NO] = {W[OB3], W[OB3 + 1], W[OB3 + 2]};
        for (int o = 0; o < NH; ++o) {
            float z = W[OB2 + o];
#pragma unroll 16
            for (int i = 0; i < NH; ++i) z = fmaf(W[OW2 + o * NH + i], h1[i], z);
            S.z2[t][o] = z;
            const float h = silu(z);
#pragma unroll
            for (int c = 0; c < NO; ++c) y[c] = fmaf(W[OW3 + c * NH + o], h, y[c]);
        }
        float d3[NO];
#pragma unroll
        for (int c = 0; c < NO; ++c) {
            const float tn = ok ? (T[(size_t)g * NO + c] - W[OYM + c]) / W[OYS + c] : 0.f;
            const float e = ok ? y[c] - tn : 0.f;
            lsum += e * e;
            d3[c] = 2.0f * e * inv_norm;
            S.d3[t][c] = d3[c];
        }
        for (int o = 0; o < NH; ++o) {
            float a = 0.f;
#pragma unroll
            for (int c = 0; c < NO; ++c) a = fmaf(W[OW3 + c * NH + o], d3[c], a);
            S.d2[t][o] = a * silu_d(S.z2[t][o]);
        }
        for (int i = 0; i < NH; ++i) {
            float a = 0.f;
            for (int o = 0; o < NH; ++o) a = fmaf(W[OW2 + o * NH + i], S.d2[t][o], a);
            S.d1[t][i] = a * silu_d(S.z1[t][i]);
        }
    }
    __syncthreads();
    const int ns = min(kB, nb - blockIdx.x * kB);
    for (int p = t; p < NPARAM; p += blockDim.x) {
        float gsum = 0.f;
        if (p < OB1) {
            const int o = p / NI, i = p % NI;
            for (int s = 0; s < ns; ++s) gsum = fmaf(S.d1[s][o], S.x[s][i], gsum);
        } else if (p < OW2) {
            const int o = p - OB1;
            for (int s = 0; s < ns; ++s) gsum += S.d1[s][o];
        } else if (p < OB2) {
            const int o = (p - OW2) / NH, i = (p - OW2) % NH;
            for (int s = 0; s < ns; ++s) gsum = fmaf(S.d2[s][o], silu(S.z1[s][i]), gsum);
        } else if (p < OW3) {
            const int o = p - OB2;
            for (int s = 0; s < ns; ++s) gsum += S.d2[s][o];
        } else if (p < OB3) {
            const int c = (p - OW3) / NH, i = (p - OW3) % NH;
            for (int s = 0; s < ns; ++s) gsum = fmaf(S.d3[s][c], silu(S.z2[s][i]), gsum);
        } else {
            const int c = p - OB3;
            for (int s = 0; s < ns; ++s) gsum += S.d3[s][c];
        }
        atomicAdd(&grad[p], gsum);
    }
    lsum = warp_sum(lsum);
    if ((t & 31) == 0) atomicAdd(loss, lsum);
}

__global__ void k_mlp_adam(float* w, float* g, float* m, float* v, int n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        g[i] = 0.f;
    }
}

struct DevBuf {
    std::vector<void*> p;
    void* get(size_t bytes) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
        p.push_back(q);
        return q;
    }
    ~DevBuf() {
        for (void* q : p) cudaFree(q);
    }
};

}  // namespace

int mlp_nw() { return NW; }

// Normalisation statistics into the blob (host)
static void set_stats(float* blob, const float* X, const float* Y, int64_t n) {
    for (int i = 0; i < NI; ++i) {
        double s = 0, s2 = 0;
        for (int64_t k = 0; k < n; ++k) {
            s += X[k * NI + i];
            s2 += (double)X[k * NI + i] * X[k * NI + i];
        }
        const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-30);
        blob[OXM + i] = (float)mu;
        blob[OXS + i] = (float)(1.0 / std::sqrt(var));
    }
    for (int c = 0; c < NO; ++c) {
        double s = 0, s2 = 0;
        for (int64_t k = 0; k < n; ++k) {
            s += Y[k * NO + c];
            s2 += (double)Y[k * NO + c] * Y[k * NO + c];
        }
        const double mu = s / n, var = std::max(s2 / n - mu * mu, 1e-30);
        blob[OYM + c] = (float)mu;
        blob[OYS + c] = (float)std::sqrt(var);
    }
}

int mlp_forward_host(const float* w, const float* X, int64_t n, float* Y, std::string& err) {
    DevBuf b;
    float* dw = (float*)b.get(sizeof(float) * NW);
    float* dwr = (float*)b.get(sizeof(float) * NW);
    float* dx = (float*)b.get(sizeof(float) * NI * std::max<int64_t>(n, 1));
    float* dy = (float*)b.get(sizeof(float) * NO * std::max<int64_t>(n, 1));
    if (!dw || !dwr || !dx || !dy) return err = "mlp: cudaMalloc failed", MDG_E_CUDA;
    cudaMemcpy(dw, w, sizeof(float) * NW, cudaMemcpyHostToDevice);
    cudaMemcpy(dx, X, sizeof(float) * NI * n, cudaMemcpyHostToDevice);
    k_mlp_round<<<20, 256>>>(dw, dwr, NW);
    k_mlp_forward<<<(int)((n + 127) / 128), 128>>>(dwr, dx, dy, (int)n);
    if (cudaDeviceSynchronize() != cudaSuccess) return err = "mlp: forward kernel failed", MDG_E_CUDA;
    cudaMemcpy(Y, dy, sizeof(float) * NO * n, cudaMemcpyDeviceToHost);
    return MDG_OK;
}

// Gradient of the mean loss over all n samples at weights w (for checks against a CPU restatement).
int mlp_grad_host(const float* w, const float* X, const float* Y, int64_t n, float* grad, float* loss,
                  std::string& err) {
    DevBuf b;
    float* dw = (float*)b.get(sizeof(float) * NW);
    float* dwr = (float*)b.get(sizeof(float) * NW);
    float* dx = (float*)b.get(sizeof(float) * NI * n);
    float* dy = (float*)b.get(sizeof(float) * NO * n);
    float* dg = (float*)b.get(sizeof(float) * NPARAM);
    float* dl = (float*)b.get(sizeof(float));
    int* di = (int*)b.get(sizeof(int) * n);
    if (!dw || !dwr || !dx || !dy || !dg || !dl || !di) return err = "mlp: cudaMalloc failed", MDG_E_CUDA;
    std::vector<int> idx(n);
    for (int64_t k = 0; k < n; ++k) idx[k] = (int)k;
    cudaMemcpy(dw, w, sizeof(float) * NW, cudaMemcpyHostToDevice);
    cudaMemcpy(dx, X, sizeof(float) * NI * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, Y, sizeof(float) * NO * n, cudaMemcpyHostToDevice);
    cudaMemcpy(di, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    cudaMemset(dg, 0, sizeof(float) * NPARAM);
    cudaMemset(dl, 0, sizeof(float));
    if (allow_max_smem(k_mlp_grad) != cudaSuccess)
        return err = "mlp: attribute", MDG_E_CUDA;
    k_mlp_round<<<20, 256>>>(dw, dwr, NW);
    k_mlp_grad<<<(int)((n + kB - 1) / kB), kB, sizeof(GradSmem)>>>(dwr, dx, dy, di, 0, (int)n, 1.0f / (float)n, dg, dl);
    if (cudaDeviceSynchronize() != cudaSuccess) return err = "mlp: gradient kernel failed", MDG_E_CUDA;
    cudaMemcpy(grad, dg, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost);
    float l = 0.f;
    cudaMemcpy(&l, dl, sizeof(float), cudaMemcpyDeviceToHost);
    if (loss) *loss = l / (float)n;
    return MDG_OK;
}

// Adam training from a seeded initialisation; w_out receives the full blob, loss_out per epoch.
int mlp_train_host(const float* X, const float* Y, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                   float* w_out, float* loss_out, std::string& err) {
    if (n < 1 || epochs < 1 || batch < 1) return err = "mlp_train: bad argument", MDG_E_ARG;
    std::vector<float> blob(NW, 0.f);
    set_stats(blob.data(), X, Y, n);
    std::mt19937_64 rng(seed);
    auto init = [&](int off, int fan_in, int count) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / (float)fan_in));
        for (int k = 0; k < count; ++k) blob[off + k] = nd(rng);
    };
    init(OW1, NI, NH * NI);
    init(OW2, NH, NH * NH);
    init(OW3, NH, NO * NH);
    for (int k = 0; k < NO * NH; ++k) blob[OW3 + k] *= 0.1f;
    DevBuf b;
    float* dw = (float*)b.get(sizeof(float) * NW);
    float* dwr = (float*)b.get(sizeof(float) * NW);
    float* dm = (float*)b.get(sizeof(float) * NPARAM);
    float* dv = (float*)b.get(sizeof(float) * NPARAM);
    float* dg = (float*)b.get(sizeof(float) * NPARAM);
    float* dl = (float*)b.get(sizeof(float));
    float* dx = (float*)b.get(sizeof(float) * NI * n);
    float* dy = (float*)b.get(sizeof(float) * NO * n);
    int* di = (int*)b.get(sizeof(int) * n);
    if (!dw || !dwr || !dm || !dv || !dg || !dl || !dx || !dy || !di) return err = "mlp_train: cudaMalloc failed", MDG_E_CUDA;
    cudaMemcpy(dw, blob.data(), sizeof(float) * NW, cudaMemcpyHostToDevice);
    cudaMemcpy(dx, X, sizeof(float) * NI * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, Y, sizeof(float) * NO * n, cudaMemcpyHostToDevice);
    cudaMemset(dm, 0, sizeof(float) * NPARAM);
    cudaMemset(dv, 0, sizeof(float) * NPARAM);
    cudaMemset(dg, 0, sizeof(float) * NPARAM);
    if (allow_max_smem(k_mlp_grad) != cudaSuccess)
        return err = "mlp_train: attribute", MDG_E_CUDA;
    std::vector<int> idx(n);
    for (int64_t k = 0; k < n; ++k) idx[k] = (int)k;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    int64_t stepn = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(idx.begin(), idx.end(), rng);
        cudaMemcpy(di, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        cudaMemset(dl, 0, sizeof(float));
        const float lr_ep = lr * 0.5f * (1.0f + std::cos(3.14159265f * (float)ep / (float)epochs));
        for (int64_t b0 = 0; b0 < n; b0 += batch) {
            const int nb = (int)std::min<int64_t>(batch, n - b0);
            ++stepn;
            k_mlp_round<<<20, 256>>>(dw, dwr, NW);
            k_mlp_grad<<<(nb + kB - 1) / kB, kB, sizeof(GradSmem)>>>(dwr, dx, dy, di, (int)b0, nb, 1.0f / (float)nb, dg, dl);
            const float c1 = 1.f - std::pow(b1, (float)stepn), c2 = 1.f - std::pow(b2, (float)stepn);
            k_mlp_adam<<<20, 256>>>(dw, dg, dm, dv, NPARAM, lr_ep, b1, b2, eps, c1, c2);
        }
        float l = 0.f;
        cudaMemcpy(&l, dl, sizeof(float), cudaMemcpyDeviceToHost);
        if (loss_out) loss_out[ep] = l / (float)n;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return err = "mlp_train: kernel failed", MDG_E_CUDA;
    cudaMemcpy(w_out, dw, sizeof(float) * NW, cudaMemcpyDeviceToHost);
    return MDG_OK;
}

}  // namespace mdg
