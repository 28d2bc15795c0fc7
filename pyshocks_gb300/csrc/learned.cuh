// Learned-weight WENO reconstruction: an MLP 5 -> 32 -> 32 -> 3 (tanh, tanh,
// softmax) maps the normalised 5-point stencil of a face to the weights of the
// three WENO-JS5 sub-stencils (src/pyshocks/weno.py:206-244); the face value is
// the convex combination sum_k omega_k uhat_k, so the flux stays conservative.
// Where the network puts more than `band` of its weight on sub-stencils that
// WENO-JS marks as crossing a discontinuity (JS weight below `tau`), the plain
// WENO-JS weights are used instead (per face).
//
// Inference runs on the tensor cores: each warp evaluates 16 faces at a time
// with mma.sync m16n8k16 (bf16 inputs, fp32 accumulate); the layer outputs stay
// in registers and feed the next layer's A fragments directly. Training uses a
// per-thread fp32 forward/backward (learned.cu).
//
// Parameter vector (1347 floats): W1[32][5], b1[32], W2[32][32], b2[32],
// W3[3][32], b3[3] (row-major).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace shk {

constexpr int kMlpIn = 5, kMlpH = 32, kMlpOut = 3;
constexpr int kMlpParams = kMlpH * kMlpIn + kMlpH + kMlpH * kMlpH + kMlpH + kMlpOut * kMlpH + kMlpOut;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpOut * kMlpH;
constexpr float kNormEps = 1.0e-12f;

struct LearnedParams {
    const float* mlp;  // kMlpParams floats (device)
    float eps;         // WENO-JS epsilon of the fallback
    float tau;         // JS weight below which a sub-stencil counts as non-smooth
    float band;        // largest network weight allowed on non-smooth sub-stencils
};

// x = (s - mean) / (max - min + 1e-12)
__device__ __forceinline__ void mlp_normalise(const float s[5], float x[5]) {
    float m = (s[0] + s[1] + s[2] + s[3] + s[4]) * 0.2f;
    float lo = fminf(fminf(fminf(s[0], s[1]), fminf(s[2], s[3])), s[4]);
    float hi = fmaxf(fmaxf(fmaxf(s[0], s[1]), fmaxf(s[2], s[3])), s[4]);
    const float inv = 1.0f / (hi - lo + kNormEps);
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = (s[k] - m) * inv;
}

// sub-stencil values at the right face (weno.py:231-239)
__device__ __forceinline__ void mlp_substencils(const float s[5], float uh[3]) {
    uh[0] = (2.0f * s[0] - 7.0f * s[1] + 11.0f * s[2]) * (1.0f / 6.0f);
    uh[1] = (-s[1] + 5.0f * s[2] + 2.0f * s[3]) * (1.0f / 6.0f);
    uh[2] = (2.0f * s[2] + 5.0f * s[3] - s[4]) * (1.0f / 6.0f);
}

// WENO-JS5 weights of the right face (weno.py:247-256), fp32
__device__ __forceinline__ void js_weights_f32(const float s[5], float eps, float w[3]) {
    const float q10 = s[0] - 2.0f * s[1] + s[2], q20 = s[0] - 4.0f * s[1] + 3.0f * s[2];
    const float q11 = s[1] - 2.0f * s[2] + s[3], q21 = s[1] - s[3];
    const float q12 = s[2] - 2.0f * s[3] + s[4], q22 = 3.0f * s[2] - 4.0f * s[3] + s[4];
    const float b0 = (13.0f / 12.0f) * q10 * q10 + 0.25f * q20 * q20;
    const float b1 = (13.0f / 12.0f) * q11 * q11 + 0.25f * q21 * q21;
    const float b2 = (13.0f / 12.0f) * q12 * q12 + 0.25f * q22 * q22;
    const float e0 = eps + b0, e1 = eps + b1, e2 = eps + b2;
    const float a0 = 0.1f / (e0 * e0), a1 = 0.6f / (e1 * e1), a2 = 0.3f / (e2 * e2);
    const float inv = 1.0f / (a0 + a1 + a2);
    w[0] = a0 * inv;
    w[1] = a1 * inv;
    w[2] = a2 * inv;
}

// face value from network logits z, with the JS trust band
__device__ __forceinline__ float learned_face(const float s[5], float z0, float z1, float z2,
                                              const LearnedParams& lp) {
    const float zm = fmaxf(fmaxf(z0, z1), z2);
    const float e0 = __expf(z0 - zm), e1 = __expf(z1 - zm), e2 = __expf(z2 - zm);
    const float inv = 1.0f / (e0 + e1 + e2);
    float w[3] = {e0 * inv, e1 * inv, e2 * inv};
    float wj[3];
    js_weights_f32(s, lp.eps, wj);
    const float excess = (wj[0] < lp.tau ? w[0] : 0.0f) + (wj[1] < lp.tau ? w[1] : 0.0f) +
                         (wj[2] < lp.tau ? w[2] : 0.0f);
    if (excess > lp.band) {
        w[0] = wj[0];
        w[1] = wj[1];
        w[2] = wj[2];
    }
    float uh[3];
    mlp_substencils(s, uh);
    return w[0] * uh[0] + w[1] * uh[1] + w[2] * uh[2];
}

// ---- tensor-core inference --------------------------------------------------

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float& d0, float& d1, float& d2, float& d3, uint32_t a0,
                                         uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// B fragments of the three layers for this lane (g = lane/4, t = lane%4):
// layer l: out = act . W^T, B[k][n] = W[n][k]; b0 = (k=2t,2t+1), b1 = (k=2t+8,2t+9), n = g
struct MlpFrags {
    uint32_t w1[4][2];     // 4 n-tiles, K = 16 (5 inputs, bias column 5, zeros)
    uint32_t w2[4][2][2];  // 4 n-tiles x 2 k-tiles
    uint32_t w3[2][2];     // 1 n-tile (3 outputs + 5 zero rows) x 2 k-tiles
    float b2[4][2];        // bias of layer 2 for columns nt*8 + 2t, +1
    float b3[2];           // bias of layer 3 for columns 2t, 2t+1
};

__device__ __forceinline__ void mlp_load_frags(const float* __restrict__ P, MlpFrags& f) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto w1e = [&](int n, int k) -> float {
        if (k < kMlpIn) return P[kOffW1 + n * kMlpIn + k];
        if (k == kMlpIn) return P[kOffB1 + n];
        return 0.0f;
    };
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + g;
        f.w1[nt][0] = pack_bf16(w1e(n, 2 * t), w1e(n, 2 * t + 1));
        f.w1[nt][1] = pack_bf16(w1e(n, 2 * t + 8), w1e(n, 2 * t + 9));
#pragma unroll
        for (int kt = 0; kt < 2; ++kt) {
            const float* row = P + kOffW2 + n * kMlpH + kt * 16;
            f.w2[nt][kt][0] = pack_bf16(row[2 * t], row[2 * t + 1]);
            f.w2[nt][kt][1] = pack_bf16(row[2 * t + 8], row[2 * t + 9]);
        }
        f.b2[nt][0] = P[kOffB2 + nt * 8 + 2 * t];
        f.b2[nt][1] = P[kOffB2 + nt * 8 + 2 * t + 1];
    }
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        if (g < kMlpOut) {
            const float* row = P + kOffW3 + g * kMlpH + kt * 16;
            f.w3[kt][0] = pack_bf16(row[2 * t], row[2 * t + 1]);
            f.w3[kt][1] = pack_bf16(row[2 * t + 8], row[2 * t + 9]);
        } else {
            f.w3[kt][0] = 0u;
            f.w3[kt][1] = 0u;
        }
    }
    f.b3[0] = (2 * t < kMlpOut) ? P[kOffB3 + 2 * t] : 0.0f;
    f.b3[1] = (2 * t + 1 < kMlpOut) ? P[kOffB3 + 2 * t + 1] : 0.0f;
}

// Logits of 16 faces (rows g and g+8 of this lane's group). xg / xg8: the
// normalised stencils of rows g and g+8 (every lane of the group passes its
// rows). Returns, in every lane, the logits (z0, z1, z2) of row g (zr) and of
// row g+8 (zs), gathered from the accumulator layout by shuffles.
__device__ __forceinline__ void mlp_mma_logits(const MlpFrags& f, const float xg[5],
                                               const float xg8[5], float zr[3], float zs[3]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    // layer-1 A fragment: columns 2t, 2t+1 (and 2t+8.. = 0): x0..x4, 1 (bias), 0
    auto col = [&](const float x[5], int c) -> float {
        return c < kMlpIn ? x[c] : (c == kMlpIn ? 1.0f : 0.0f);
    };
    const uint32_t a0 = pack_bf16(col(xg, 2 * t), col(xg, 2 * t + 1));
    const uint32_t a1 = pack_bf16(col(xg8, 2 * t), col(xg8, 2 * t + 1));
    float h[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        h[nt][0] = h[nt][1] = h[nt][2] = h[nt][3] = 0.0f;
        mma_bf16(h[nt][0], h[nt][1], h[nt][2], h[nt][3], a0, a1, 0u, 0u, f.w1[nt][0], f.w1[nt][1]);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[nt][i] = tanh_fast(h[nt][i]);
    }
    // layer 2: A (16 x 32) from the layer-1 accumulators, 2 k-tiles
    uint32_t A2[2][4];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        A2[kt][0] = pack_bf16(h[2 * kt][0], h[2 * kt][1]);
        A2[kt][1] = pack_bf16(h[2 * kt][2], h[2 * kt][3]);
        A2[kt][2] = pack_bf16(h[2 * kt + 1][0], h[2 * kt + 1][1]);
        A2[kt][3] = pack_bf16(h[2 * kt + 1][2], h[2 * kt + 1][3]);
    }
    float q[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        q[nt][0] = q[nt][2] = f.b2[nt][0];
        q[nt][1] = q[nt][3] = f.b2[nt][1];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt)
            mma_bf16(q[nt][0], q[nt][1], q[nt][2], q[nt][3], A2[kt][0], A2[kt][1], A2[kt][2],
                     A2[kt][3], f.w2[nt][kt][0], f.w2[nt][kt][1]);
#pragma unroll
        for (int i = 0; i < 4; ++i) q[nt][i] = tanh_fast(q[nt][i]);
    }
    uint32_t A3[2][4];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
        A3[kt][0] = pack_bf16(q[2 * kt][0], q[2 * kt][1]);
        A3[kt][1] = pack_bf16(q[2 * kt][2], q[2 * kt][3]);
        A3[kt][2] = pack_bf16(q[2 * kt + 1][0], q[2 * kt + 1][1]);
        A3[kt][3] = pack_bf16(q[2 * kt + 1][2], q[2 * kt + 1][3]);
    }
    float z0 = f.b3[0], z1 = f.b3[1], z2 = f.b3[0], z3 = f.b3[1];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
        mma_bf16(z0, z1, z2, z3, A3[kt][0], A3[kt][1], A3[kt][2], A3[kt][3], f.w3[kt][0],
                 f.w3[kt][1]);
    // lane t=0 of the group holds (row g: z[0], z[1]; row g+8: z[0], z[1]),
    // lane t=1 holds (row g: z[2], pad; row g+8: z[2], pad)
    const int base = lane & ~3;
    zr[0] = __shfl_sync(0xffffffffu, z0, base);
    zr[1] = __shfl_sync(0xffffffffu, z1, base);
    zr[2] = __shfl_sync(0xffffffffu, z0, base + 1);
    zs[0] = __shfl_sync(0xffffffffu, z2, base);
    zs[1] = __shfl_sync(0xffffffffu, z3, base);
    zs[2] = __shfl_sync(0xffffffffu, z2, base + 1);
}

}  // namespace shk
