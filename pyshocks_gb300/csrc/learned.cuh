// Learned-weight WENO reconstruction: an MLP 5 -> 32 -> 32 -> 3 (tanh, tanh,
// softmax) maps the normalised 5-point stencil of a cell, s = v_{c-2..c+2}, to
// the weights of the three WENO-JS5 sub-stencils (src/pyshocks/weno.py:206-244)
// at the cell's right face: omega_R = softmax(z). The cell's left face takes the
// same sub-stencil scores with its own ideal weights, as WENO-JS5 does with its
// shared smoothness indicators (alpha_k = d_k / (eps + beta_k)^2 on the right,
// d_k / (eps + beta_{2-k})^2 on the mirrored left): omega_L = softmax(z2 - ln 3,
// z1, z0 + ln 3), i.e. proportional to (e2 / 3, e1, 3 e0) with e = exp(z). One
// network evaluation serves both faces. Each face value is the convex
// combination sum_k omega_k uhat_k of its sub-stencil values, so the flux stays
// conservative. The trust band, per face: where the network puts more than
// `band` of its weight on sub-stencils that WENO-JS marks as crossing a
// discontinuity (JS weight below `tau`), or moves any weight more than `dev`
// away from the WENO-JS weight (dev >= 1 never triggers), that face uses the
// plain WENO-JS weights.
//
// Inference runs on the tensor cores: each warp evaluates 32 cells at a time
// with mma.sync m16n8k16 (bf16 inputs, fp32 accumulate); the layer outputs stay
// in registers and feed the next layer's A fragments directly. Training uses a
// per-thread fp32 forward/backward (learned.cu).
//
// Parameter vector (1347 floats): W1[32][5], b1[32], W2[32][32], b2[32],
// W3[3][32], b3[3] (row-major).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
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
    float norm_eps;    // floor of the stencil range in the input normalisation
};

// The normalisation floor plays the part of WENO-JS's eps: features far below
// it (a few rounding units on a flat state) reach the network as ~0 inputs, so
// the weights do not follow rounding noise and the scheme's Jacobian stays
// bounded there (with a floor of 1e-12 the linearised learned scheme amplified
// such noise until the adjoint overflowed).
__host__ __device__ inline float norm_floor(float e) { return e > 0.0f ? e : kNormEps; }

__device__ __forceinline__ bool outside_band(const float w[3], const float wj[3],
                                             const LearnedParams& lp) {
    const float excess = (wj[0] < lp.tau ? w[0] : 0.0f) + (wj[1] < lp.tau ? w[1] : 0.0f) +
                         (wj[2] < lp.tau ? w[2] : 0.0f);
    const float d = fmaxf(fmaxf(fabsf(w[0] - wj[0]), fabsf(w[1] - wj[1])), fabsf(w[2] - wj[2]));
    return excess > lp.band || d > lp.dev;
}

// 1/x to ~1 ulp (rcp.approx.ftz.f32, one instruction) for the float weights and
// normalisation of the learned path, where a correctly rounded division buys
// nothing (all arguments here are >= eps-sized normal numbers)
__device__ __forceinline__ float fast_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// x = (s - mean) / (max - min + norm_eps)
__device__ __forceinline__ void mlp_normalise(const float s[5], float x[5], float norm_eps) {
    float m = (s[0] + s[1] + s[2] + s[3] + s[4]) * 0.2f;
    float lo = fminf(fminf(fminf(s[0], s[1]), fminf(s[2], s[3])), s[4]);
    float hi = fmaxf(fmaxf(fmaxf(s[0], s[1]), fmaxf(s[2], s[3])), s[4]);
    const float inv = fast_rcp(hi - lo + norm_eps);
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = (s[k] - m) * inv;
}

// WENO-JS5 smoothness indicators of the three sub-stencils of a cell
// (weno.py:247-256) and the two second/first differences of each
__device__ __forceinline__ void js_betas(const float s[5], float be[3], float q[6]) {
    q[0] = s[0] - 2.0f * s[1] + s[2]; q[1] = s[0] - 4.0f * s[1] + 3.0f * s[2];
    q[2] = s[1] - 2.0f * s[2] + s[3]; q[3] = s[1] - s[3];
    q[4] = s[2] - 2.0f * s[3] + s[4]; q[5] = 3.0f * s[2] - 4.0f * s[3] + s[4];
#pragma unroll
    for (int l = 0; l < 3; ++l)
        be[l] = (13.0f / 12.0f) * q[2 * l] * q[2 * l] + 0.25f * q[2 * l + 1] * q[2 * l + 1];
}

// WENO-JS5 weights of the right face (d = (1, 6, 3)/10 on beta_k) and of the
// mirrored left face (d_k on beta_{2-k}) from the cell's indicators
__device__ __forceinline__ void js_weights_pair(const float be[3], float eps, float wr[3],
                                                float wl[3]) {
    const float e0 = eps + be[0], e1 = eps + be[1], e2 = eps + be[2];
    const float r0 = fast_rcp(e0 * e0), r1 = fast_rcp(e1 * e1), r2 = fast_rcp(e2 * e2);
    const float a1 = 0.6f * r1;
    const float ir = fast_rcp(fmaf(0.1f, r0, fmaf(0.3f, r2, a1)));
    const float il = fast_rcp(fmaf(0.1f, r2, fmaf(0.3f, r0, a1)));
    wr[0] = 0.1f * r0 * ir; wr[1] = a1 * ir; wr[2] = 0.3f * r2 * ir;
    wl[0] = 0.1f * r2 * il; wl[1] = a1 * il; wl[2] = 0.3f * r0 * il;
}

// sub-stencil values minus the cell value, right and left face, from the
// stencil shifted by the cell value (ds[2] = 0)
__device__ __forceinline__ void cell_substencils(const float ds[5], float ur[3], float ul[3]) {
    ur[0] = (2.0f * ds[0] - 7.0f * ds[1]) * (1.0f / 6.0f);
    ur[1] = (2.0f * ds[3] - ds[1]) * (1.0f / 6.0f);
    ur[2] = (5.0f * ds[3] - ds[4]) * (1.0f / 6.0f);
    ul[0] = (2.0f * ds[4] - 7.0f * ds[3]) * (1.0f / 6.0f);
    ul[1] = (2.0f * ds[1] - ds[3]) * (1.0f / 6.0f);
    ul[2] = (5.0f * ds[1] - ds[0]) * (1.0f / 6.0f);
}

// right- and left-face weights from the exponentials e_k = exp(z_k - max z)
__device__ __forceinline__ void cell_softmax(float e0, float e1, float e2, float wr[3], float wl[3]) {
    const float ir = fast_rcp(e0 + e1 + e2);
    wr[0] = e0 * ir; wr[1] = e1 * ir; wr[2] = e2 * ir;
    const float l0 = e2 * (1.0f / 3.0f), l2 = 3.0f * e0;
    const float il = fast_rcp(l0 + e1 + l2);
    wl[0] = l0 * il; wl[1] = e1 * il; wl[2] = l2 * il;
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

// The network's B fragments in shared memory, staged once per launch by the
// whole block (mlp_stage_forward / mlp_stage_back, called by learned_stage in
// stencil.cuh) and read at each use: register-resident fragments
// held 38 registers per thread for the whole kernel and made the step spill.
// Lane L's words sit at [.][L] as one 16-byte vector, so the warp's load of a
// vector is 512 contiguous bytes (no bank conflicts). Fragments of lane
// (g = lane/4, t = lane%4), layer l: out = act . W^T, B[k][n] = W[n][k],
// b0 = (k = 2t, 2t+1), b1 = (k = 2t+8, 2t+9), n = g.
struct MlpShared {
    uint4 w1[32];     // b0 of layer-1 n-tiles 0..3 (b1 is zero: 5 inputs + bias column)
    uint4 w2[4][32];  // layer-2 n-tile nt: (k-tile 0 b0, b1, k-tile 1 b0, b1)
    uint4 w3[32];     // layer 3 (n = 3 outputs + 5 zero rows): (k-tile 0 b0, b1, k-tile 1 b0, b1)
    float b2[32];
    float b3[8];      // 3 outputs, zero padded (columns 2t, 2t+1 for every t)
};

// the fp16 B fragments of the network backward (see mlp_stage_back)
struct MlpBackShared {
    uint4 w3[32];     // dz W3: n-tiles 0..3
    uint4 w2[4][32];  // da2 W2, n-tile nt: (k-tile 0 b0, b1, k-tile 1 b0, b1)
    uint4 w1[32];     // da1 W1: (k-tile 0 b0, b1, k-tile 1 b0, b1)
};

// The block's staged network: one of each per kernel that runs the learned
// reconstruction (a kernel that never calls these allocates neither).
__device__ __forceinline__ MlpShared& mlp_shared() {
    __shared__ MlpShared s;
    return s;
}
__device__ __forceinline__ MlpBackShared& mlp_back_shared() {
    __shared__ MlpBackShared s;
    return s;
}

// layer-1 weight of unit n for input k: inputs 0..4, the bias as input 5
__device__ __forceinline__ float mlp_w1(const float* __restrict__ P, int n, int k) {
    if (k < kMlpIn) return P[kOffW1 + n * kMlpIn + k];
    if (k == kMlpIn) return P[kOffB1 + n];
    return 0.0f;
}

// stage the inference fragments of parameters P (whole block; ends with a barrier)
__device__ inline void mlp_stage_forward(const float* __restrict__ P, MlpShared& s) {
    for (int i = threadIdx.x; i < 6 * 32; i += blockDim.x) {
        const int j = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3;
        uint32_t w[4];
        if (j == 0) {
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
                w[nt] = pack_bf16(mlp_w1(P, nt * 8 + g, 2 * t), mlp_w1(P, nt * 8 + g, 2 * t + 1));
            s.w1[lane] = make_uint4(w[0], w[1], w[2], w[3]);
        } else if (j <= 4) {
            const int n = (j - 1) * 8 + g;
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                const float* row = P + kOffW2 + n * kMlpH + kt * 16;
                w[2 * kt] = pack_bf16(row[2 * t], row[2 * t + 1]);
                w[2 * kt + 1] = pack_bf16(row[2 * t + 8], row[2 * t + 9]);
            }
            s.w2[j - 1][lane] = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                if (g < kMlpOut) {
                    const float* row = P + kOffW3 + g * kMlpH + kt * 16;
                    w[2 * kt] = pack_bf16(row[2 * t], row[2 * t + 1]);
                    w[2 * kt + 1] = pack_bf16(row[2 * t + 8], row[2 * t + 9]);
                } else {
                    w[2 * kt] = w[2 * kt + 1] = 0u;
                }
            }
            s.w3[lane] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
    for (int i = threadIdx.x; i < 40; i += blockDim.x) {
        if (i < 32) s.b2[i] = P[kOffB2 + i];
        else s.b3[i - 32] = i - 32 < kMlpOut ? P[kOffB3 + i - 32] : 0.0f;
    }
    __syncthreads();
}

// ---- 32 cells per warp iteration ----------------------------------------------
// Lane (g, t) owns one cell: row g (t = 0) / g+8 (t = 1) of m16 tile A, row g
// (t = 2) / g+8 (t = 3) of tile B. The owner holds its stencil *shifted by the
// cell value* (ds_k = s_k - s_2: the weights are shift-invariant and a face
// value is s_2 + sum_k omega_k (uhat_k - s_2), so float differences serve
// float and double states alike), computes its normalised input, and at the
// end both face corrections. The A fragments of both tiles are gathered by
// shuffles; hidden layers apply tanh to packed bf16 pairs (tanh.approx.bf16x2),
// which are exactly the next layer's A fragments.

__device__ __forceinline__ uint32_t tanh_bf16x2(uint32_t x) {
    uint32_t y;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(y) : "r"(x));
    return y;
}

// ---- warp exchanges through shared memory ------------------------------------
// Rows of the warp's 32-cell block go through a per-warp scratch area (16-byte
// aligned): row r at scr + 4 r (16 B) for fragment rows, or scr + 6 r for the
// input cotangents. An A fragment is then one ldmatrix.x4 instead of twelve
// shuffles and selects, and a lane's row of an accumulator tile one vector
// load. Every exchange begins with __syncwarp, so a lane never overwrites
// scratch that another lane of the warp is still to read.
constexpr int kWarpScratch = 128;      // floats per warp, forward
constexpr int kWarpScratchVjp = 192;   // floats per warp, backward

__device__ __forceinline__ void ldmatrix_x4(const float* row, uint32_t a[4]) {
    const uint32_t addr = static_cast<uint32_t>(__cvta_generic_to_shared(row));
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3])
                 : "r"(addr)
                 : "memory");
}

// A fragments (rows g, g+8 of tiles A and B; columns 2t, 2t+1) of the block
// whose row `myrow` holds this lane's 8 b16 values (w0..w3)
__device__ __forceinline__ void rows_to_afrags(float* scr, int myrow, uint32_t w0, uint32_t w1,
                                               uint32_t w2, uint32_t w3, uint32_t a[4]) {
    __syncwarp();
    *reinterpret_cast<uint4*>(scr + 4 * myrow) = make_uint4(w0, w1, w2, w3);
    __syncwarp();
    ldmatrix_x4(scr + 4 * (threadIdx.x & 31), a);
}

// columns 0..3 of the lane's row `myrow` from the accumulators of tiles A
// (c[0..3]: rows g, g+8) and B (d[0..3]); lanes t = 0, 1 hold columns 0..3
__device__ __forceinline__ float4 accum_row4(float* scr, int myrow, const float c[4],
                                             const float d[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __syncwarp();
    if (t < 2) {
        *reinterpret_cast<float2*>(scr + 4 * g + 2 * t) = make_float2(c[0], c[1]);
        *reinterpret_cast<float2*>(scr + 4 * (g + 8) + 2 * t) = make_float2(c[2], c[3]);
        *reinterpret_cast<float2*>(scr + 4 * (g + 16) + 2 * t) = make_float2(d[0], d[1]);
        *reinterpret_cast<float2*>(scr + 4 * (g + 24) + 2 * t) = make_float2(d[2], d[3]);
    }
    __syncwarp();
    return *reinterpret_cast<const float4*>(scr + 4 * myrow);
}

// hidden layers + output of both m16 tiles of a 32-cell block: layer-1 A
// registers a[0], a[1] (tile A, rows g and g+8) and a[2], a[3] (tile B). Each
// fragment loaded from shared memory serves both tiles, and the two tiles'
// mma chains interleave. A2x / A3x: the bf16 hidden activations
// tanh(layer-1 / layer-2 pre-activation) of tile x in A-fragment layout (the
// backward keeps them); zA, zB: the logit accumulators.
__device__ __forceinline__ void mlp_tiles(const MlpShared& s, const uint32_t a[4], uint32_t A2a[2][4],
                                          uint32_t A2b[2][4], uint32_t A3a[2][4], uint32_t A3b[2][4],
                                          float zA[4], float zB[4]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
    {
        const uint4 w = s.w1[lane];
        const uint32_t w1[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
            float d0 = 0.0f, d1 = 0.0f, d2 = 0.0f, d3 = 0.0f;
            mma_bf16(c0, c1, c2, c3, a[0], a[1], 0u, 0u, w1[nt], 0u);
            mma_bf16(d0, d1, d2, d3, a[2], a[3], 0u, 0u, w1[nt], 0u);
            A2a[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(c0, c1));
            A2a[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(c2, c3));
            A2b[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(d0, d1));
            A2b[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(d2, d3));
        }
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const uint4 w = s.w2[nt][lane];
        const float2 bb = *reinterpret_cast<const float2*>(&s.b2[nt * 8 + 2 * t]);
        float c0 = bb.x, c1 = bb.y, c2 = bb.x, c3 = bb.y;
        float d0 = bb.x, d1 = bb.y, d2 = bb.x, d3 = bb.y;
        mma_bf16(c0, c1, c2, c3, A2a[0][0], A2a[0][1], A2a[0][2], A2a[0][3], w.x, w.y);
        mma_bf16(d0, d1, d2, d3, A2b[0][0], A2b[0][1], A2b[0][2], A2b[0][3], w.x, w.y);
        mma_bf16(c0, c1, c2, c3, A2a[1][0], A2a[1][1], A2a[1][2], A2a[1][3], w.z, w.w);
        mma_bf16(d0, d1, d2, d3, A2b[1][0], A2b[1][1], A2b[1][2], A2b[1][3], w.z, w.w);
        A3a[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(c0, c1));
        A3a[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(c2, c3));
        A3b[nt >> 1][(nt & 1) * 2 + 0] = tanh_bf16x2(pack_bf16(d0, d1));
        A3b[nt >> 1][(nt & 1) * 2 + 1] = tanh_bf16x2(pack_bf16(d2, d3));
    }
    const uint4 w = s.w3[lane];
    const float2 bb = *reinterpret_cast<const float2*>(&s.b3[2 * t]);
    zA[0] = bb.x; zA[1] = bb.y; zA[2] = bb.x; zA[3] = bb.y;
    zB[0] = bb.x; zB[1] = bb.y; zB[2] = bb.x; zB[3] = bb.y;
    mma_bf16(zA[0], zA[1], zA[2], zA[3], A3a[0][0], A3a[0][1], A3a[0][2], A3a[0][3], w.x, w.y);
    mma_bf16(zB[0], zB[1], zB[2], zB[3], A3b[0][0], A3b[0][1], A3b[0][2], A3b[0][3], w.x, w.y);
    mma_bf16(zA[0], zA[1], zA[2], zA[3], A3a[1][0], A3a[1][1], A3a[1][2], A3a[1][3], w.z, w.w);
    mma_bf16(zB[0], zB[1], zB[2], zB[3], A3b[1][0], A3b[1][1], A3b[1][2], A3b[1][3], w.z, w.w);
}

// The face corrections sum_k omega_k (uhat_k - s_2) of this lane's cell (right
// face cr, left face cl) from its shifted stencil ds (ds[2] = 0), with the
// WENO-JS trust band per face. All 32 lanes must call it (shuffles) with
// finite stencils.
// scr: the warp's kWarpScratch floats of shared memory (16-byte aligned).
__device__ __forceinline__ void learned_cell32(const MlpShared& ms, const float ds[5],
                                               const LearnedParams& lp, float* scr, float& cr,
                                               float& cl) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int myrow = 16 * (t >> 1) + 8 * (t & 1) + g;
    // normalised input, its row (x0,x1) (x2,x3) (x4,1) (0,0) of the layer-1
    // A operand, and the A fragments of both tiles
    float x[5];
    mlp_normalise(ds, x, lp.norm_eps);
    uint32_t a[4];
    rows_to_afrags(scr, myrow, pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], 1.0f),
                   0u, a);
    float zA[4], zB[4];
    {
        uint32_t A2a[2][4], A2b[2][4], A3a[2][4], A3b[2][4];
        mlp_tiles(ms, a, A2a, A2b, A3a, A3b, zA, zB);
    }
    // logits of the owned row (columns 0..2 of the output tiles)
    const float4 zr = accum_row4(scr, myrow, zA, zB);
    const float z0 = zr.x, z1 = zr.y, z2 = zr.z;
    // softmax of both faces, trust band, corrections
    const float zm = fmaxf(fmaxf(z0, z1), z2);
    float wr[3], wl[3];
    cell_softmax(__expf(z0 - zm), __expf(z1 - zm), __expf(z2 - zm), wr, wl);
    float be[3], q[6], jr[3], jl[3];
    js_betas(ds, be, q);
    js_weights_pair(be, lp.eps, jr, jl);
    if (outside_band(wr, jr, lp)) { wr[0] = jr[0]; wr[1] = jr[1]; wr[2] = jr[2]; }
    if (outside_band(wl, jl, lp)) { wl[0] = jl[0]; wl[1] = jl[1]; wl[2] = jl[2]; }
    float hr[3], hl[3];
    cell_substencils(ds, hr, hl);
    cr = wr[0] * hr[0] + wr[1] * hr[1] + wr[2] * hr[2];
    cl = wl[0] * hl[0] + wl[1] * hl[1] + wl[2] * hl[2];
}

// ---- backward of the two learned face values of 32 cells (adjoint) ------------
// The forward is recomputed with the inference's own mma sequence (the same
// activations, bit for bit), keeping the bf16 hidden activations h1, h2 in
// their fragment registers. The network backward runs on the tensor cores too:
// da2 = (dz W3) * (1 - h2^2), da1 = (da2 W2) * (1 - h1^2), dx = da1 W1, as
// mma.sync m16n8k16 with fp16 operands and fp32 accumulation, the weights
// being the bf16-rounded ones of the forward (exact in fp16). Each cell's
// cotangent dz is scaled by a power of two into [1, 2) before the products
// and dx scaled back (the backward is linear and rows are independent, so the
// scaling is exact and fp16 neither overflows nor loses small cotangents).
// Roundings of the forward pass the cotangent straight through; max/min of the
// normalisation split it evenly at ties (torch/JAX convention).

__device__ __forceinline__ void mma_f16(float& d0, float& d1, float& d2, float& d3, uint32_t a0,
                                        uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                        uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d0), "+f"(d1), "+f"(d2), "+f"(d3)
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_f16(float lo, float hi) {
    __half2 v = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_lo(uint32_t x) { return __uint_as_float(x << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t x) { return __uint_as_float(x & 0xffff0000u); }

__device__ __forceinline__ float round_bf16(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

// stage the fp16 B fragments of the backward products for parameters P
// (whole block; ends with a barrier). Lane (g = lane/4, t = lane%4): B[k][n]
// with k the contracted index (rows 2t, 2t+1 and 2t+8, 2t+9), n = g; dz W3
// (k = output, 3 of 16; n = hidden, 4 n-tiles), da2 W2 (k = layer-2 unit,
// 2 k-tiles; n = layer-1 unit, 4 n-tiles), da1 W1 (k = layer-1 unit, 2
// k-tiles; n = input, 5 of 8). The weights are the forward's bf16 roundings.
__device__ inline void mlp_stage_back(const float* __restrict__ P, MlpBackShared& s) {
    for (int i = threadIdx.x; i < 6 * 32; i += blockDim.x) {
        const int j = i >> 5, lane = i & 31, g = lane >> 2, t = lane & 3;
        uint32_t w[4];
        if (j == 0) {
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int n = nt * 8 + g;
                const float w30 = 2 * t < kMlpOut ? round_bf16(P[kOffW3 + (2 * t) * kMlpH + n]) : 0.0f;
                const float w31 = 2 * t + 1 < kMlpOut ? round_bf16(P[kOffW3 + (2 * t + 1) * kMlpH + n]) : 0.0f;
                w[nt] = pack_f16(w30, w31);
            }
            s.w3[lane] = make_uint4(w[0], w[1], w[2], w[3]);
        } else if (j <= 4) {
            const int n = (j - 1) * 8 + g;
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                const int k = kt * 16 + 2 * t;
                w[2 * kt] = pack_f16(round_bf16(P[kOffW2 + k * kMlpH + n]),
                                     round_bf16(P[kOffW2 + (k + 1) * kMlpH + n]));
                w[2 * kt + 1] = pack_f16(round_bf16(P[kOffW2 + (k + 8) * kMlpH + n]),
                                         round_bf16(P[kOffW2 + (k + 9) * kMlpH + n]));
            }
            s.w2[j - 1][lane] = make_uint4(w[0], w[1], w[2], w[3]);
        } else {
            auto w1 = [&](int kk) { return g < kMlpIn ? round_bf16(P[kOffW1 + kk * kMlpIn + g]) : 0.0f; };
#pragma unroll
            for (int kt = 0; kt < 2; ++kt) {
                const int k = kt * 16 + 2 * t;
                w[2 * kt] = pack_f16(w1(k), w1(k + 1));
                w[2 * kt + 1] = pack_f16(w1(k + 8), w1(k + 9));
            }
            s.w1[lane] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
    __syncthreads();
}

// (x0, x1) * (1 - h^2) for a bf16 pair h, packed to fp16
__device__ __forceinline__ uint32_t tanh_back_f16(float x0, float x1, uint32_t h) {
    const float h0 = bf16_lo(h), h1 = bf16_hi(h);
    return pack_f16(x0 * fmaf(-h0, h0, 1.0f), x1 * fmaf(-h1, h1, 1.0f));
}

// network backward of both m16 tiles of a block: d[0], d[1] / d[2], d[3] the
// fp16 A registers of the (scaled) logit cotangents of tile A / B (rows g,
// g+8; columns 2t, 2t+1), A2x / A3x the tiles' kept activations; returns the
// input cotangents (row g: columns 2t, 2t+1 in x[0], x[1]; row g+8 in x[2],
// x[3]) of tile A in xa and of tile B in xb. Each fragment load serves both tiles.
__device__ __forceinline__ void mlp_tiles_back(const MlpBackShared& s, const uint32_t d[4],
                                               const uint32_t A2a[2][4], const uint32_t A2b[2][4],
                                               const uint32_t A3a[2][4], const uint32_t A3b[2][4],
                                               float xa[4], float xb[4]) {
    const int lane = threadIdx.x & 31;
    uint32_t D2a[2][4], D2b[2][4];
    {
        const uint4 w = s.w3[lane];
        const uint32_t w3[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
            float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
            float e0 = 0.0f, e1 = 0.0f, e2 = 0.0f, e3 = 0.0f;
            mma_f16(c0, c1, c2, c3, d[0], d[1], 0u, 0u, w3[nt], 0u);
            mma_f16(e0, e1, e2, e3, d[2], d[3], 0u, 0u, w3[nt], 0u);
            const int j = nt >> 1, q = (nt & 1) * 2;
            D2a[j][q] = tanh_back_f16(c0, c1, A3a[j][q]);
            D2a[j][q + 1] = tanh_back_f16(c2, c3, A3a[j][q + 1]);
            D2b[j][q] = tanh_back_f16(e0, e1, A3b[j][q]);
            D2b[j][q + 1] = tanh_back_f16(e2, e3, A3b[j][q + 1]);
        }
    }
    uint32_t D1a[2][4], D1b[2][4];
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
        const uint4 w = s.w2[nt][lane];
        float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
        float e0 = 0.0f, e1 = 0.0f, e2 = 0.0f, e3 = 0.0f;
        mma_f16(c0, c1, c2, c3, D2a[0][0], D2a[0][1], D2a[0][2], D2a[0][3], w.x, w.y);
        mma_f16(e0, e1, e2, e3, D2b[0][0], D2b[0][1], D2b[0][2], D2b[0][3], w.x, w.y);
        mma_f16(c0, c1, c2, c3, D2a[1][0], D2a[1][1], D2a[1][2], D2a[1][3], w.z, w.w);
        mma_f16(e0, e1, e2, e3, D2b[1][0], D2b[1][1], D2b[1][2], D2b[1][3], w.z, w.w);
        const int j = nt >> 1, q = (nt & 1) * 2;
        D1a[j][q] = tanh_back_f16(c0, c1, A2a[j][q]);
        D1a[j][q + 1] = tanh_back_f16(c2, c3, A2a[j][q + 1]);
        D1b[j][q] = tanh_back_f16(e0, e1, A2b[j][q]);
        D1b[j][q + 1] = tanh_back_f16(e2, e3, A2b[j][q + 1]);
    }
    const uint4 w = s.w1[lane];
    xa[0] = xa[1] = xa[2] = xa[3] = 0.0f;
    xb[0] = xb[1] = xb[2] = xb[3] = 0.0f;
    mma_f16(xa[0], xa[1], xa[2], xa[3], D1a[0][0], D1a[0][1], D1a[0][2], D1a[0][3], w.x, w.y);
    mma_f16(xb[0], xb[1], xb[2], xb[3], D1b[0][0], D1b[0][1], D1b[0][2], D1b[0][3], w.x, w.y);
    mma_f16(xa[0], xa[1], xa[2], xa[3], D1a[1][0], D1a[1][1], D1a[1][2], D1a[1][3], w.z, w.w);
    mma_f16(xb[0], xb[1], xb[2], xb[3], D1b[1][0], D1b[1][1], D1b[1][2], D1b[1][3], w.z, w.w);
}

// gR d(u_R)/ds + gL d(u_L)/ds of this lane's cell (right and left face values)
// with respect to its stencil s = v_{c-2..c+2}, given shifted by the cell
// value as the forward evaluates it (ds[2] = 0; the gradient of a
// shift-equivariant value does not depend on the shift). The cotangents come
// from seed(cr, cl, gR, gL), called once the forward has produced the face
// corrections cr = u_R - v_c and cl = u_L - v_c (the seeds of a flux VJP
// depend on the face values). All 32 lanes must call it (shuffles, mma) with
// finite stencils; returns dsum[5].
template <class Seed>
__device__ __forceinline__ void learned_cell_vjp32(const MlpShared& ms, const MlpBackShared& bk,
                                                   const float s[5], Seed&& seed,
                                                   const LearnedParams& lp, float* scr,
                                                   float dsum[5]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int myrow = 16 * (t >> 1) + 8 * (t & 1) + g;
    // ---- forward (as learned_cell32), keeping the activations
    float x[5];
    mlp_normalise(s, x, lp.norm_eps);
    uint32_t a[4];
    rows_to_afrags(scr, myrow, pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], 1.0f),
                   0u, a);
    uint32_t A2a[2][4], A3a[2][4], A2b[2][4], A3b[2][4];
    float zA[4], zB[4];
    mlp_tiles(ms, a, A2a, A2b, A3a, A3b, zA, zB);
    const float4 zr = accum_row4(scr, myrow, zA, zB);
    const float z0 = zr.x, z1 = zr.y, z2 = zr.z;
    // ---- per-cell part: weights, fallback, direct terms, logit cotangents
    float hr[3], hl[3];
    cell_substencils(s, hr, hl);
    float be[3], q[6], jr[3], jl[3];
    js_betas(s, be, q);
    js_weights_pair(be, lp.eps, jr, jl);
    const float zm = fmaxf(fmaxf(z0, z1), z2);
    float wr[3], wl[3];
    cell_softmax(__expf(z0 - zm), __expf(z1 - zm), __expf(z2 - zm), wr, wl);
    const bool fbr = outside_band(wr, jr, lp), fbl = outside_band(wl, jl, lp);
    const float* tr = fbr ? jr : wr;
    const float* tl = fbl ? jl : wl;
    const float uR = tr[0] * hr[0] + tr[1] * hr[1] + tr[2] * hr[2];
    const float uL = tl[0] * hl[0] + tl[1] * hl[1] + tl[2] * hl[2];
    float gR, gL;
    seed(uR, uL, gR, gL);
    // direct parts: sum_k omega_k d uhat_k / ds; 6 uhat taps, right face
    // (2,-7,11,0,0) (0,-1,5,2,0) (0,0,2,5,-1), left face mirrored
    const float cR = gR * (1.0f / 6.0f), cL = gL * (1.0f / 6.0f);
    dsum[0] = cR * (2.0f * tr[0]) - cL * tl[2];
    dsum[1] = cR * (-7.0f * tr[0] - tr[1]) + cL * (2.0f * tl[1] + 5.0f * tl[2]);
    dsum[2] = cR * (11.0f * tr[0] + 5.0f * tr[1] + 2.0f * tr[2]) +
              cL * (11.0f * tl[0] + 5.0f * tl[1] + 2.0f * tl[2]);
    dsum[3] = cR * (2.0f * tr[1] + 5.0f * tr[2]) + cL * (-7.0f * tl[0] - tl[1]);
    dsum[4] = -cR * tr[2] + cL * (2.0f * tl[0]);
    if (fbr || fbl) {
        // WENO-JS faces: d u / d beta_l = -2 omega_l (uhat_l - u) / (eps + beta_l);
        // the left face's sub-stencil k sees beta_{2-k}
        float bb[3] = {0.0f, 0.0f, 0.0f};
        if (fbr)
            for (int l = 0; l < 3; ++l) bb[l] += -2.0f * gR * jr[l] * (hr[l] - uR) / (lp.eps + be[l]);
        if (fbl)
            for (int k = 0; k < 3; ++k)
                bb[2 - k] += -2.0f * gL * jl[k] * (hl[k] - uL) / (lp.eps + be[2 - k]);
        // d beta_l / ds = 13/6 q1_l dq1_l + 1/2 q2_l dq2_l
        const float a0 = (13.0f / 6.0f) * q[0] * bb[0], c0 = 0.5f * q[1] * bb[0];
        const float a1 = (13.0f / 6.0f) * q[2] * bb[1], c1 = 0.5f * q[3] * bb[1];
        const float a2 = (13.0f / 6.0f) * q[4] * bb[2], c2 = 0.5f * q[5] * bb[2];
        dsum[0] += a0 + c0;
        dsum[1] += -2.0f * a0 - 4.0f * c0 + a1 + c1;
        dsum[2] += a0 + 3.0f * c0 - 2.0f * a1 + a2 + 3.0f * c2;
        dsum[3] += a1 - c1 - 2.0f * a2 - 4.0f * c2;
        dsum[4] += a2 + c2;
    }
    // softmax backward of the network faces into the shared logits: right
    // omega = softmax(z); left omega = softmax(z2 - ln 3, z1, z0 + ln 3)
    float dz[3] = {0.0f, 0.0f, 0.0f};
    if (!fbr) {
        const float d0 = gR * hr[0], d1 = gR * hr[1], d2 = gR * hr[2];
        const float dot = wr[0] * d0 + wr[1] * d1 + wr[2] * d2;
        dz[0] += wr[0] * (d0 - dot); dz[1] += wr[1] * (d1 - dot); dz[2] += wr[2] * (d2 - dot);
    }
    if (!fbl) {
        const float d0 = gL * hl[0], d1 = gL * hl[1], d2 = gL * hl[2];
        const float dot = wl[0] * d0 + wl[1] * d1 + wl[2] * d2;
        dz[2] += wl[0] * (d0 - dot); dz[1] += wl[1] * (d1 - dot); dz[0] += wl[2] * (d2 - dot);
    }
    // power-of-two scale of the row into [1, 2)
    const float mz = fmaxf(fmaxf(fabsf(dz[0]), fabsf(dz[1])), fabsf(dz[2]));
    int ez = static_cast<int>((__float_as_uint(mz) >> 23) & 0xffu) - 127;
    ez = mz > 0.0f ? max(-100, min(100, ez)) : 0;
    const float up = __uint_as_float(static_cast<uint32_t>(127 - ez) << 23);  // 2^-ez
    const float down = __uint_as_float(static_cast<uint32_t>(127 + ez) << 23);  // 2^ez
    // ---- network backward on the tensor cores: the A fragments of the logit
    // cotangents from the rows (dz0, dz1) (dz2, 0) (0, 0) (0, 0)
    uint32_t d[4];
    rows_to_afrags(scr, myrow, pack_f16(dz[0] * up, dz[1] * up), pack_f16(dz[2] * up, 0.0f), 0u,
                   0u, d);
    float xa[4], xb[4];
    mlp_tiles_back(bk, d, A2a, A2b, A3a, A3b, xa, xb);
    // the owned row's dx[0..5] (columns 0..5 of the input-gradient tiles, held
    // by lanes t = 0, 1, 2), through rows of 6 floats
    float dx[6];
    {
        __syncwarp();
        if (t < 3) {
            *reinterpret_cast<float2*>(scr + 6 * g + 2 * t) = make_float2(xa[0], xa[1]);
            *reinterpret_cast<float2*>(scr + 6 * (g + 8) + 2 * t) = make_float2(xa[2], xa[3]);
            *reinterpret_cast<float2*>(scr + 6 * (g + 16) + 2 * t) = make_float2(xb[0], xb[1]);
            *reinterpret_cast<float2*>(scr + 6 * (g + 24) + 2 * t) = make_float2(xb[2], xb[3]);
        }
        __syncwarp();
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float2 v = *reinterpret_cast<const float2*>(scr + 6 * myrow + 2 * k);
            dx[2 * k] = v.x;
            dx[2 * k + 1] = v.y;
        }
    }
    // ---- normalisation x = (s - mean) / (max - min + norm_eps), unscaled
    const float m = (s[0] + s[1] + s[2] + s[3] + s[4]) * 0.2f;
    float lo = fminf(fminf(fminf(s[0], s[1]), fminf(s[2], s[3])), s[4]);
    float hi = fmaxf(fmaxf(fmaxf(s[0], s[1]), fmaxf(s[2], s[3])), s[4]);
    const float inv = fast_rcp(hi - lo + lp.norm_eps);
    float sdx = 0.0f, sxd = 0.0f;
    int nhi = 0, nlo = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        dx[k] *= down;
        sdx += dx[k];
        sxd += dx[k] * (s[k] - m);
        nhi += s[k] == hi;
        nlo += s[k] == lo;
    }
    const float gr = -sxd * inv * inv;  // d/d(range)
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float dd = inv * (dx[k] - 0.2f * sdx);
        dd += gr * ((s[k] == hi ? fast_rcp(float(nhi)) : 0.0f) - (s[k] == lo ? fast_rcp(float(nlo)) : 0.0f));
        dsum[k] += dd;
    }
}

}  // namespace shk
