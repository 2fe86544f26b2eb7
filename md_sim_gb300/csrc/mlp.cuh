// mlp.cuh - the SHAKE-seeding network: 9 -> 64 -> 64 -> 3, SiLU, used by the SHAKE kernel
// (inference) and by the training kernels of mlp.cu.
//
// Parameter blob (float32, MLP_NW values): W1[64][9] b1[64] W2[64][64] b2[64] W3[3][64] b3[3],
// then input mean[9], input 1/std[9], output mean[3], output std[3].  Kernels compute with the
// weights rounded to BF16 and accumulate in FP32.
#pragma once

#include <cuda_bf16.h>

namespace mdg {
namespace mlp {

constexpr int NI = 9, NH = 64, NO = 3;
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NO * NH;
constexpr int NPARAM = OB3 + NO;  // trained parameters (4995)
constexpr int OXM = NPARAM, OXS = OXM + NI, OYM = OXS + NI, OYS = OYM + NO;
constexpr int NW = OYS + NO;      // full blob (5019)

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_d(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float bf16r(float w) { return __bfloat162float(__float2bfloat16_rn(w)); }

// Features of a 3-constraint molecule from the unconstrained bonds p_c and the previous bonds r_c
// (both minimum-imaged) and the constraint lengths squared l2_c.
__device__ __forceinline__ void features(const double p[3][3], const double r[3][3], const double l2[3], float f[9]) {
    for (int c = 0; c < 3; ++c) {
        const int d = (c + 1) % 3;
        const double pp = p[c][0] * p[c][0] + p[c][1] * p[c][1] + p[c][2] * p[c][2];
        const double pr = p[c][0] * r[c][0] + p[c][1] * r[c][1] + p[c][2] * r[c][2];
        const double pq = p[c][0] * r[d][0] + p[c][1] * r[d][1] + p[c][2] * r[d][2];
        f[c] = (float)((l2[c] - pp) / l2[c]);
        f[3 + c] = (float)(pr / l2[c]);
        f[6 + c] = (float)(pq / sqrt(l2[c] * l2[d]));
    }
}

// Forward pass with weights W (already BF16-rounded floats, e.g. in shared memory).
__device__ __forceinline__ void forward(const float* W, const float in[9], float out[3]) {
    float x[NI];
#pragma unroll
    for (int i = 0; i < NI; ++i) x[i] = (in[i] - W[OXM + i]) * W[OXS + i];
    float h1[NH];
#pragma unroll 8
    for (int o = 0; o < NH; ++o) {
        float z = W[OB1 + o];
#pragma unroll
        for (int i = 0; i < NI; ++i) z = fmaf(W[OW1 + o * NI + i], x[i], z);
        h1[o] = silu(z);
    }
    float y[NO] = {W[OB3 + 0], W[OB3 + 1], W[OB3 + 2]};
#pragma unroll 4
    for (int o = 0; o < NH; ++o) {
        float z = W[OB2 + o];
#pragma unroll
        for (int i = 0; i < NH; ++i) z = fmaf(W[OW2 + o * NH + i], h1[i], z);
        const float h = silu(z);
#pragma unroll
        for (int c = 0; c < NO; ++c) y[c] = fmaf(W[OW3 + c * NH + o], h, y[c]);
    }
#pragma unroll
    for (int c = 0; c < NO; ++c) out[c] = y[c] * W[OYS + c] + W[OYM + c];
}

// The same forward pass by a whole block (at least 64 threads; every thread calls it): thread o
// computes hidden unit o of each layer and threads 0-2 the outputs, each with the operations of
// forward() in its order, so the outputs are identical to it.  in and out live in shared memory;
// h is shared scratch of 2 * NH floats.
__device__ __forceinline__ void forward_block(const float* W, const float* in, float* h, float* out) {
    const int o = threadIdx.x;
    if (o < NH) {
        float z = W[OB1 + o];
#pragma unroll
        for (int i = 0; i < NI; ++i) z = fmaf(W[OW1 + o * NI + i], (in[i] - W[OXM + i]) * W[OXS + i], z);
        h[o] = silu(z);
    }
    __syncthreads();
    if (o < NH) {
        float z = W[OB2 + o];
#pragma unroll 8
        for (int i = 0; i < NH; ++i) z = fmaf(W[OW2 + o * NH + i], h[i], z);
        h[NH + o] = silu(z);
    }
    __syncthreads();
    if (o < NO) {
        float y = W[OB3 + o];
        for (int k = 0; k < NH; ++k) y = fmaf(W[OW3 + o * NH + k], h[NH + k], y);
        out[o] = y * W[OYS + o] + W[OYM + o];
    }
    __syncthreads();
}

}  // namespace mlp
}  // namespace mdg
