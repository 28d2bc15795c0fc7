// Learned-weight WENO reconstruction: an MLP 5 -> 32 -> 32 -> 3 (tanh, tanh,
// softmax) maps the normalised 5-point stencil of a face to the weights of the
// three WENO-JS5 sub-stencils (src/pyshocks/weno.py:206-244); the face value is
// the convex combination sum_k omega_k uhat_k, so the flux stays conservative.
// The trust band: where the network puts more than `band` of its weight on
// sub-stencils that WENO-JS marks as crossing a discontinuity (JS weight below
// `tau`), or moves any weight more than `dev` away from the WENO-JS weight, the
// plain WENO-JS weights are used instead (per face).
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
    float dev;         // largest |omega_k - omega_JS,k| allowed
};

__device__ __forceinline__ bool outside_band(const float w[3], const float wj[3],
                                             const LearnedParams& lp) {
    const float excess = (wj[0] < lp.tau ? w[0] : 0.0f) + (wj[1] < lp.tau ? w[1] : 0.0f) +
                         (wj[2] < lp.tau ? w[2] : 0.0f);
    const float d = fmaxf(fmaxf(fabsf(w[0] - wj[0]), fabsf(w[1] - wj[1])), fabsf(w[2] - wj[2]));
    return excess > lp.band || d > lp.dev;
}

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
    if (outside_band(w, wj, lp)) {
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

// ---- 32 faces per warp iteration ---------------------------------------------
// Lane (g, t) owns one face: row g (t = 0) / g+8 (t = 1) of m16 tile A, row g
// (t = 2) / g+8 (t = 3) of tile B. The owner holds its stencil *shifted by the
// cell value* (ds_k = s_k - s_2: the weights are shift-invariant and the face
// value is s_2 + sum_k omega_k (uhat_k - s_2), so float differences serve
// float and double states alike), computes its normalised input, and at the
// end its face correction. The A fragments of both tiles are gathered by
// shuffles; hidden layers apply tanh to packed bf16 pairs (tanh.approx.bf16x2),
// which are exactly the next layer's A fragments.

__device__ __forceinline__ uint32_t tanh_bf16x2(uint32_t x) {
    uint32_t y;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(y) : "r"(x));
    return y;
}

// hidden layers + output of one m16 tile; a0/a1: layer-1 A registers (rows g, g+8)
__device__ __forceinline__ void mlp_tile(const MlpFrags& f, uint32_t a0, uint32_t a1, float& z0,
                                         float& z1, float& z2, float& z3) {
    uint32_t A2[2][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
        mma_bf16(c0, c1, c2, c3, a0, a1, 0u, 0u, f.w1[nt][0], f.w1[nt][1]);
        A2[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(c0, c1));
        A2[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(c2, c3));
    }
    uint32_t A3[2][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        float c0 = f.b2[nt][0], c1 = f.b2[nt][1], c2 = f.b2[nt][0], c3 = f.b2[nt][1];
#pragma unroll
        for (int kt = 0; kt < 2; ++kt)
            mma_bf16(c0, c1, c2, c3, A2[kt][0], A2[kt][1], A2[kt][2], A2[kt][3], f.w2[nt][kt][0],
                     f.w2[nt][kt][1]);
        A3[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(c0, c1));
        A3[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(c2, c3));
    }
    z0 = f.b3[0]; z1 = f.b3[1]; z2 = f.b3[0]; z3 = f.b3[1];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt)
        mma_bf16(z0, z1, z2, z3, A3[kt][0], A3[kt][1], A3[kt][2], A3[kt][3], f.w3[kt][0], f.w3[kt][1]);
}

// The face correction sum_k omega_k (uhat_k - s_2) of this lane's face from its
// shifted stencil ds (ds[2] = 0), with the WENO-JS trust band. All 32 lanes
// must call it (shuffles); `valid` only masks nothing -- every lane passes a
// finite stencil.
__device__ __forceinline__ float learned_delta32(const MlpFrags& f, const float ds[5],
                                                 const LearnedParams& lp) {
    const int lane = threadIdx.x & 31, t = lane & 3, base = lane & ~3;
    // normalised input and its packed column pairs (x0,x1) (x2,x3) (x4,1)
    float x[5];
    mlp_normalise(ds, x);
    const uint32_t p0 = pack_bf16(x[0], x[1]), p1 = pack_bf16(x[2], x[3]), p2 = pack_bf16(x[4], 1.0f);
    // A registers of lane (g, t): columns 2t, 2t+1 of rows g and g+8 of each tile,
    // owned by lanes base+0 (A, g), base+1 (A, g+8), base+2 (B, g), base+3 (B, g+8)
    uint32_t a[4];
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const uint32_t q0 = __shfl_sync(0xffffffffu, p0, base + o);
        const uint32_t q1 = __shfl_sync(0xffffffffu, p1, base + o);
        const uint32_t q2 = __shfl_sync(0xffffffffu, p2, base + o);
        a[o] = t == 0 ? q0 : (t == 1 ? q1 : (t == 2 ? q2 : 0u));
    }
    float zA0, zA1, zA2, zA3, zB0, zB1, zB2, zB3;
    mlp_tile(f, a[0], a[1], zA0, zA1, zA2, zA3);
    mlp_tile(f, a[2], a[3], zB0, zB1, zB2, zB3);
    // logits of the owned row: z[0], z[1] from lane base+0, z[2] from lane base+1
    const float u0 = __shfl_sync(0xffffffffu, zA0, base), u1 = __shfl_sync(0xffffffffu, zA1, base);
    const float u2 = __shfl_sync(0xffffffffu, zA2, base), u3 = __shfl_sync(0xffffffffu, zA3, base);
    const float v0 = __shfl_sync(0xffffffffu, zB0, base), v1 = __shfl_sync(0xffffffffu, zB1, base);
    const float v2 = __shfl_sync(0xffffffffu, zB2, base), v3 = __shfl_sync(0xffffffffu, zB3, base);
    const float w0 = __shfl_sync(0xffffffffu, zA0, base + 1), w1 = __shfl_sync(0xffffffffu, zA2, base + 1);
    const float y0 = __shfl_sync(0xffffffffu, zB0, base + 1), y1 = __shfl_sync(0xffffffffu, zB2, base + 1);
    float z0, z1, z2;
    if (t == 0) { z0 = u0; z1 = u1; z2 = w0; }
    else if (t == 1) { z0 = u2; z1 = u3; z2 = w1; }
    else if (t == 2) { z0 = v0; z1 = v1; z2 = y0; }
    else { z0 = v2; z1 = v3; z2 = y1; }
    // softmax, trust band, correction
    const float zm = fmaxf(fmaxf(z0, z1), z2);
    const float e0 = __expf(z0 - zm), e1 = __expf(z1 - zm), e2 = __expf(z2 - zm);
    const float inv = __frcp_rn(e0 + e1 + e2);
    float w[3] = {e0 * inv, e1 * inv, e2 * inv};
    float wj[3];
    js_weights_f32(ds, lp.eps, wj);
    if (outside_band(w, wj, lp)) {
        w[0] = wj[0];
        w[1] = wj[1];
        w[2] = wj[2];
    }
    float uh[3];
    mlp_substencils(ds, uh);  // uhat_k - s_2 (ds[2] = 0)
    return w[0] * uh[0] + w[1] * uh[1] + w[2] * uh[2];
}

// ---- backward of one learned face value (adjoint) ----------------------------
// Wr: the parameters with the weights rounded to bfloat16 exactly as the
// tensor-core forward uses them (layer-2/3 biases stay fp32), staged in shared
// memory by learned_stage_params. The forward is recomputed per face in fp32
// with the same roundings of inputs and activations and the same tanh/exp
// approximations, so the value differentiated is the one the flux kernel
// produced; roundings pass the cotangent straight through. max/min of the
// normalisation split the cotangent evenly at ties (torch/JAX convention).

__device__ __forceinline__ float round_bf16(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

__device__ __forceinline__ void learned_stage_params(const float* __restrict__ P, float* Wr) {
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
        const bool keep = (i >= kOffB2 && i < kOffW3) || i >= kOffB3;
        Wr[i] = keep ? P[i] : round_bf16(P[i]);
    }
}

// d(face value)/d(stencil) scaled by ub; returns ds[5]. The stencil may be
// passed shifted by any constant (the face value moves with it, the weights do
// not), so callers pass differences to the cell value as the forward does.
__device__ __forceinline__ float bf16_tanh(float x) {
    const uint32_t y = tanh_bf16x2(pack_bf16(x, 0.0f));
    return __uint_as_float(y << 16);
}

__device__ __forceinline__ void learned_face_vjp(const float s_in[5], float ub, const float* Wr,
                                                 const LearnedParams& lp, float ds[5]) {
    float s[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) s[k] = s_in[k] - s_in[2];
    float uh[3];
    mlp_substencils(s, uh);
    // WENO-JS weights and fallback decision (as learned_face)
    const float q10 = s[0] - 2.0f * s[1] + s[2], q20 = s[0] - 4.0f * s[1] + 3.0f * s[2];
    const float q11 = s[1] - 2.0f * s[2] + s[3], q21 = s[1] - s[3];
    const float q12 = s[2] - 2.0f * s[3] + s[4], q22 = 3.0f * s[2] - 4.0f * s[3] + s[4];
    const float be[3] = {(13.0f / 12.0f) * q10 * q10 + 0.25f * q20 * q20,
                         (13.0f / 12.0f) * q11 * q11 + 0.25f * q21 * q21,
                         (13.0f / 12.0f) * q12 * q12 + 0.25f * q22 * q22};
    float wj[3];
    {
        const float e0 = lp.eps + be[0], e1 = lp.eps + be[1], e2 = lp.eps + be[2];
        const float a0 = 0.1f / (e0 * e0), a1 = 0.6f / (e1 * e1), a2 = 0.3f / (e2 * e2);
        const float inv = 1.0f / (a0 + a1 + a2);
        wj[0] = a0 * inv; wj[1] = a1 * inv; wj[2] = a2 * inv;
    }
    // network forward with the inference roundings
    float x[5];
    mlp_normalise(s, x);
    float xr[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xr[k] = round_bf16(x[k]);
    float h1[kMlpH], h2[kMlpH];
    for (int a = 0; a < kMlpH; ++a) {
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < kMlpIn; ++k) acc = fmaf(Wr[kOffW1 + a * kMlpIn + k], xr[k], acc);
        acc += Wr[kOffB1 + a];
        h1[a] = bf16_tanh(acc);
    }
    for (int a = 0; a < kMlpH; ++a) {
        float acc = Wr[kOffB2 + a];
        for (int k = 0; k < kMlpH; ++k) acc = fmaf(Wr[kOffW2 + a * kMlpH + k], h1[k], acc);
        h2[a] = bf16_tanh(acc);
    }
    float z[3];
    for (int o = 0; o < 3; ++o) {
        float acc = Wr[kOffB3 + o];
        for (int k = 0; k < kMlpH; ++k) acc = fmaf(Wr[kOffW3 + o * kMlpH + k], h2[k], acc);
        z[o] = acc;
    }
    const float zm = fmaxf(fmaxf(z[0], z[1]), z[2]);
    const float e0 = __expf(z[0] - zm), e1 = __expf(z[1] - zm), e2 = __expf(z[2] - zm);
    const float einv = 1.0f / (e0 + e1 + e2);
    const float w[3] = {e0 * einv, e1 * einv, e2 * einv};
    const bool fallback = outside_band(w, wj, lp);
    const float* wt = fallback ? wj : w;
    // direct part: sum_k omega_k d uhat_k / ds (6 uhat taps: (2,-7,11,0,0) (0,-1,5,2,0) (0,0,2,5,-1))
    const float c6 = ub * (1.0f / 6.0f);
    ds[0] = c6 * (2.0f * wt[0]);
    ds[1] = c6 * (-7.0f * wt[0] - wt[1]);
    ds[2] = c6 * (11.0f * wt[0] + 5.0f * wt[1] + 2.0f * wt[2]);
    ds[3] = c6 * (2.0f * wt[1] + 5.0f * wt[2]);
    ds[4] = c6 * (-wt[2]);
    const float u = wt[0] * uh[0] + wt[1] * uh[1] + wt[2] * uh[2];
    if (fallback) {
        // d u / d beta_l = -2 omega_l (uhat_l - u) / (eps + beta_l)
        float bb[3];
        for (int l = 0; l < 3; ++l) bb[l] = -2.0f * ub * wj[l] * (uh[l] - u) / (lp.eps + be[l]);
        // d beta_l / ds = 13/6 q1_l dq1_l + 1/2 q2_l dq2_l
        const float a0 = (13.0f / 6.0f) * q10 * bb[0], c0 = 0.5f * q20 * bb[0];
        const float a1 = (13.0f / 6.0f) * q11 * bb[1], c1 = 0.5f * q21 * bb[1];
        const float a2 = (13.0f / 6.0f) * q12 * bb[2], c2 = 0.5f * q22 * bb[2];
        ds[0] += a0 + c0;
        ds[1] += -2.0f * a0 - 4.0f * c0 + a1 + c1;
        ds[2] += a0 + 3.0f * c0 - 2.0f * a1 + a2 + 3.0f * c2;
        ds[3] += a1 - c1 - 2.0f * a2 - 4.0f * c2;
        ds[4] += a2 + c2;
        return;
    }
    // softmax and network backward (input gradient only)
    const float dw0 = ub * uh[0], dw1 = ub * uh[1], dw2 = ub * uh[2];
    const float dot = w[0] * dw0 + w[1] * dw1 + w[2] * dw2;
    const float dz[3] = {w[0] * (dw0 - dot), w[1] * (dw1 - dot), w[2] * (dw2 - dot)};
    float da2[kMlpH];
    for (int k = 0; k < kMlpH; ++k) {
        const float dh = Wr[kOffW3 + k] * dz[0] + Wr[kOffW3 + kMlpH + k] * dz[1] +
                         Wr[kOffW3 + 2 * kMlpH + k] * dz[2];
        da2[k] = dh * (1.0f - h2[k] * h2[k]);
    }
    float dx[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < kMlpH; ++k) {
        float dh = 0.0f;
        for (int a = 0; a < kMlpH; ++a) dh = fmaf(Wr[kOffW2 + a * kMlpH + k], da2[a], dh);
        const float da1 = dh * (1.0f - h1[k] * h1[k]);
#pragma unroll
        for (int j = 0; j < kMlpIn; ++j) dx[j] = fmaf(Wr[kOffW1 + k * kMlpIn + j], da1, dx[j]);
    }
    // normalisation x = (s - mean) / (max - min + eps)
    const float m = (s[0] + s[1] + s[2] + s[3] + s[4]) * 0.2f;
    float lo = fminf(fminf(fminf(s[0], s[1]), fminf(s[2], s[3])), s[4]);
    float hi = fmaxf(fmaxf(fmaxf(s[0], s[1]), fmaxf(s[2], s[3])), s[4]);
    const float inv = 1.0f / (hi - lo + kNormEps);
    float sdx = 0.0f, sxd = 0.0f;
    int nhi = 0, nlo = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        sdx += dx[k];
        sxd += dx[k] * (s[k] - m);
        nhi += s[k] == hi;
        nlo += s[k] == lo;
    }
    const float gr = -sxd * inv * inv;  // d/d(range)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float d = inv * (dx[k] - 0.2f * sdx);
        d += gr * ((s[k] == hi ? 1.0f / nhi : 0.0f) - (s[k] == lo ? 1.0f / nlo : 0.0f));
        ds[k] += d;
    }
}

}  // namespace shk

