// Training and standalone inference kernels of the learned-weight WENO
// reconstruction (see learned.cuh for the method).
//
// Training loss over a batch of cells (stencil s_i = v_{c-2..c+2}, targets
// T_R,i / T_L,i of its right / left face, weight w_i):
//   L = 1/(2n) sum_i sum_{F in R, L} [ w_i (sum_k omega_F,k(x_i) uhat_F,k(s_i) - T_F,i)^2
//                                      + reg sum_k (omega_F,k(x_i) - d_k)^2 ]
// with x_i the normalised stencil and omega_R = softmax(z), omega_L =
// softmax(z2 - ln 3, z1, z0 + ln 3) of the one network output z(x_i). The
// second term pulls the weights toward the ideal weights d = (1, 6, 3)/10 of
// WENO-JS5 where the face error does not constrain them (on smooth data every
// sub-stencil reconstructs well, and an arbitrary choice among them can be
// unstable in time). The forward and backward passes run one cell per thread
// in fp32 (exact tanh/exp); per-block gradient sums are formed from the
// per-cell activations staged in shared memory and written to a per-block
// workspace, which a second kernel reduces in a fixed order (deterministic).
// Adam updates the fp32 master weights in place.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/shocks.h"
#include "learned.cuh"

namespace shk {

constexpr int kTrainThreads = 128;
// per-sample values staged for the weight-gradient sums
constexpr int kStage = kMlpIn + kMlpH + kMlpH + kMlpH + kMlpH + kMlpOut;  // x, h1, da1, h2, da2, dz

__global__ void __launch_bounds__(kTrainThreads) mlp_loss_grad_kernel(
    const float* __restrict__ P, const float* __restrict__ stencils, const float* __restrict__ target,
    const float* __restrict__ weight, int64_t n, float reg, float norm_eps, float* __restrict__ block_grad,
    double* __restrict__ block_loss) {
    extern __shared__ __align__(16) float sm[];
    float* Ps = sm;                              // kMlpParams
    float* S = sm + ((kMlpParams + 3) & ~3);     // kStage x kTrainThreads (column per sample)
    __shared__ double lred[kTrainThreads / 32];
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) Ps[i] = P[i];
    __syncthreads();
    const float* W1 = Ps + kOffW1;
    const float* b1 = Ps + kOffB1;
    const float* W2 = Ps + kOffW2;
    const float* b2 = Ps + kOffB2;
    const float* W3 = Ps + kOffW3;
    const float* b3 = Ps + kOffB3;
    const int tid = threadIdx.x;
    // each thread owns a strided subset of the parameter gradients
    constexpr int kOwn = (kMlpParams + kTrainThreads - 1) / kTrainThreads;
    float gacc[kOwn];
#pragma unroll
    for (int j = 0; j < kOwn; ++j) gacc[j] = 0.0f;
    double lacc = 0.0;
    const float invn = 0.5f / static_cast<float>(n);  // 2n face terms

    for (int64_t base = int64_t(blockIdx.x) * kTrainThreads; base < n;
         base += int64_t(gridDim.x) * kTrainThreads) {
        const int64_t i = base + tid;
        const bool valid = i < n;
        float s[5], x[5], h1[kMlpH], h2[kMlpH];
        float dz[3] = {0.0f, 0.0f, 0.0f};
        if (valid) {
#pragma unroll
            for (int k = 0; k < 5; ++k) s[k] = stencils[i * 5 + k];
        } else {
#pragma unroll
            for (int k = 0; k < 5; ++k) s[k] = 0.0f;
        }
        // shifted by the cell value, as the flux kernel evaluates it
        const float c = s[2];
#pragma unroll
        for (int k = 0; k < 5; ++k) s[k] -= c;
        s[2] = 0.0f;
        mlp_normalise(s, x, norm_eps);
#pragma unroll 4
        for (int a = 0; a < kMlpH; ++a) {
            float acc = b1[a];
#pragma unroll
            for (int k = 0; k < kMlpIn; ++k) acc = fmaf(W1[a * kMlpIn + k], x[k], acc);
            h1[a] = tanhf(acc);
        }
#pragma unroll 4
        for (int a = 0; a < kMlpH; ++a) {
            float acc = b2[a];
#pragma unroll 8
            for (int k = 0; k < kMlpH; ++k) acc = fmaf(W2[a * kMlpH + k], h1[k], acc);
            h2[a] = tanhf(acc);
        }
        float z[3];
#pragma unroll
        for (int o = 0; o < 3; ++o) {
            float acc = b3[o];
#pragma unroll 8
            for (int k = 0; k < kMlpH; ++k) acc = fmaf(W3[o * kMlpH + k], h2[k], acc);
            z[o] = acc;
        }
        const float zm = fmaxf(fmaxf(z[0], z[1]), z[2]);
        float wr[3], wl[3], hr[3], hl[3];
        cell_softmax(expf(z[0] - zm), expf(z[1] - zm), expf(z[2] - zm), wr, wl);
        cell_substencils(s, hr, hl);
        if (valid) {
            const float rr = (wr[0] * hr[0] + wr[1] * hr[1] + wr[2] * hr[2]) - (target[2 * i] - c);
            const float rl = (wl[0] * hl[0] + wl[1] * hl[1] + wl[2] * hl[2]) - (target[2 * i + 1] - c);
            const float wi = weight[i];
            const float gr[3] = {wr[0] - 0.1f, wr[1] - 0.6f, wr[2] - 0.3f};
            const float gl[3] = {wl[0] - 0.1f, wl[1] - 0.6f, wl[2] - 0.3f};
            lacc += static_cast<double>(wi) * (static_cast<double>(rr) * rr + static_cast<double>(rl) * rl) +
                    static_cast<double>(reg) * (gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2] +
                                                gl[0] * gl[0] + gl[1] * gl[1] + gl[2] * gl[2]);
            // dL/dv per face, dv/domega_k = uhat_k, plus the regulariser; softmax
            // backward of both faces into the shared logits
            const float dvr = 2.0f * wi * rr * invn, dvl = 2.0f * wi * rl * invn;
            const float rg = 2.0f * reg * invn;
            float dw[3], dot;
#pragma unroll
            for (int k = 0; k < 3; ++k) dw[k] = fmaf(dvr, hr[k], rg * gr[k]);
            dot = wr[0] * dw[0] + wr[1] * dw[1] + wr[2] * dw[2];
#pragma unroll
            for (int k = 0; k < 3; ++k) dz[k] = wr[k] * (dw[k] - dot);
#pragma unroll
            for (int k = 0; k < 3; ++k) dw[k] = fmaf(dvl, hl[k], rg * gl[k]);
            dot = wl[0] * dw[0] + wl[1] * dw[1] + wl[2] * dw[2];
            dz[2] += wl[0] * (dw[0] - dot);
            dz[1] += wl[1] * (dw[1] - dot);
            dz[0] += wl[2] * (dw[2] - dot);
        }
        // backward through the hidden layers
        float da2[kMlpH], da1[kMlpH];
#pragma unroll 4
        for (int k = 0; k < kMlpH; ++k) {
            const float dh = W3[0 * kMlpH + k] * dz[0] + W3[1 * kMlpH + k] * dz[1] + W3[2 * kMlpH + k] * dz[2];
            da2[k] = dh * (1.0f - h2[k] * h2[k]);
        }
#pragma unroll 4
        for (int k = 0; k < kMlpH; ++k) {
            float dh = 0.0f;
#pragma unroll 8
            for (int a = 0; a < kMlpH; ++a) dh = fmaf(W2[a * kMlpH + k], da2[a], dh);
            da1[k] = dh * (1.0f - h1[k] * h1[k]);
        }
        // stage per-sample values: S[j * T + tid]
        {
            int j = 0;
            for (int k = 0; k < kMlpIn; ++k) S[(j++) * kTrainThreads + tid] = x[k];
            for (int k = 0; k < kMlpH; ++k) S[(j++) * kTrainThreads + tid] = h1[k];
            for (int k = 0; k < kMlpH; ++k) S[(j++) * kTrainThreads + tid] = da1[k];
            for (int k = 0; k < kMlpH; ++k) S[(j++) * kTrainThreads + tid] = h2[k];
            for (int k = 0; k < kMlpH; ++k) S[(j++) * kTrainThreads + tid] = da2[k];
            for (int k = 0; k < kMlpOut; ++k) S[(j++) * kTrainThreads + tid] = dz[k];
        }
        __syncthreads();
        // parameter p owned by thread (p % T): sum over the staged samples
        constexpr int oX = 0, oH1 = kMlpIn, oDA1 = oH1 + kMlpH, oH2 = oDA1 + kMlpH,
                      oDA2 = oH2 + kMlpH, oDZ = oDA2 + kMlpH;
#pragma unroll
        for (int j = 0; j < kOwn; ++j) {
            const int p = tid + j * kTrainThreads;
            if (p >= kMlpParams) break;
            int ra, rb;  // rows of S multiplied (rb < 0: plain sum of row ra)
            if (p < kOffB1) { ra = oDA1 + p / kMlpIn; rb = oX + p % kMlpIn; }
            else if (p < kOffW2) { ra = oDA1 + (p - kOffB1); rb = -1; }
            else if (p < kOffB2) { ra = oDA2 + (p - kOffW2) / kMlpH; rb = oH1 + (p - kOffW2) % kMlpH; }
            else if (p < kOffW3) { ra = oDA2 + (p - kOffB2); rb = -1; }
            else if (p < kOffB3) { ra = oDZ + (p - kOffW3) / kMlpH; rb = oH2 + (p - kOffW3) % kMlpH; }
            else { ra = oDZ + (p - kOffB3); rb = -1; }
            const float* A = S + ra * kTrainThreads;
            float acc = 0.0f;
            if (rb < 0) {
                for (int q = 0; q < kTrainThreads; ++q) acc += A[q];
            } else {
                const float* Bv = S + rb * kTrainThreads;
                for (int q = 0; q < kTrainThreads; ++q) acc = fmaf(A[q], Bv[q], acc);
            }
            gacc[j] += acc;
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < kOwn; ++j) {
        const int p = tid + j * kTrainThreads;
        if (p < kMlpParams) block_grad[size_t(blockIdx.x) * kMlpParams + p] = gacc[j];
    }
    for (int o = 16; o > 0; o >>= 1) lacc += __shfl_xor_sync(0xffffffffu, lacc, o);
    if ((tid & 31) == 0) lred[tid >> 5] = lacc;
    __syncthreads();
    if (tid == 0) {
        double l = 0.0;
        for (int w = 0; w < kTrainThreads / 32; ++w) l += lred[w];
        block_loss[blockIdx.x] = l;
    }
}

__global__ void mlp_reduce_kernel(const float* __restrict__ block_grad, const double* __restrict__ block_loss,
                                  int nblocks, int64_t n, float* __restrict__ grad, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < kMlpParams) {
        double acc = 0.0;
        for (int b = 0; b < nblocks; ++b) acc += block_grad[size_t(b) * kMlpParams + p];
        grad[p] = static_cast<float>(acc);
    }
    if (p == 0 && loss) {
        double l = 0.0;
        for (int b = 0; b < nblocks; ++b) l += block_loss[b];
        *loss = l / (2.0 * static_cast<double>(n));
    }
}

__global__ void mlp_adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int np, float lr, float b1, float b2,
                                float eps, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// standalone learned face values (right, left) of n cell stencils
// (tensor-core path, as in the flux kernel)
__global__ void __launch_bounds__(256) learned_faces_kernel(LearnedParams lp, const float* __restrict__ stencils,
                                                            float* __restrict__ out, int64_t n) {
    __shared__ __align__(16) float scratch[(256 / 32) * kWarpScratch];
    float* scr = scratch + (threadIdx.x >> 5) * kWarpScratch;
    mlp_stage_forward(lp.mlp, mlp_shared());
    const MlpShared& ms = mlp_shared();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int myrow = 16 * (t >> 1) + 8 * (t & 1) + g;
    const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
    const int64_t wid = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int64_t blk = wid; blk * 32 < n; blk += warps) {
        const int64_t r = blk * 32 + myrow;
        const int64_t rr = r < n ? r : n - 1;
        float s[5], ds[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) s[k] = stencils[rr * 5 + k];
#pragma unroll
        for (int k = 0; k < 5; ++k) ds[k] = s[k] - s[2];
        ds[2] = 0.0f;
        float cr, cl;
        learned_cell32(ms, ds, lp, scr, cr, cl);
        if (r < n) {
            out[2 * r] = s[2] + cr;
            out[2 * r + 1] = s[2] + cl;
        }
    }
}

}  // namespace shk

using namespace shk;

namespace {
int lcheck(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libshocks: CUDA error %s\n", cudaGetErrorString(e));
        return SHK_ECUDA;
    }
    return SHK_OK;
}
int train_blocks(int64_t n) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t need = (n + kTrainThreads - 1) / kTrainThreads;
    return static_cast<int>(need < int64_t(sms) * 2 ? (need > 0 ? need : 1) : int64_t(sms) * 2);
}
}  // namespace

extern "C" {

int shk_mlp_num_params(void) { return kMlpParams; }

int64_t shk_mlp_workspace_bytes(int64_t n) {
    const int nb = train_blocks(n);
    return int64_t(nb) * kMlpParams * static_cast<int64_t>(sizeof(float)) +
           int64_t(nb) * static_cast<int64_t>(sizeof(double));
}

int shk_mlp_loss_grad_f32(const float* params, const float* stencils, const float* target,
                          const float* weight, int64_t n, float reg, float norm_eps,
                          float* grad, double* loss, void* workspace, int64_t workspace_bytes,
                          void* stream) {
    if (!params || !stencils || !target || !weight || !grad || n <= 0 || !workspace) return SHK_EINVAL;
    if (workspace_bytes < shk_mlp_workspace_bytes(n)) return SHK_EINVAL;
    const int nb = train_blocks(n);
    float* bg = static_cast<float*>(workspace);
    double* bl = reinterpret_cast<double*>(static_cast<char*>(workspace) + size_t(nb) * kMlpParams * sizeof(float));
    if (reinterpret_cast<uintptr_t>(bl) % 8) return SHK_EINVAL;
    const size_t smem = sizeof(float) * (((kMlpParams + 3) & ~3) + size_t(kStage) * kTrainThreads);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int r = lcheck(cudaFuncSetAttribute(mlp_loss_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (r) return r;
    mlp_loss_grad_kernel<<<nb, kTrainThreads, smem, st>>>(params, stencils, target, weight, n, reg,
                                                          norm_floor(norm_eps), bg, bl);
    r = lcheck(cudaGetLastError());
    if (r) return r;
    mlp_reduce_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(bg, bl, nb, n, grad, loss);
    return lcheck(cudaGetLastError());
}

int shk_mlp_adam_f32(float* params, const float* grad, float* m, float* v, float lr, float beta1,
                     float beta2, float eps, int32_t step, void* stream) {
    if (!params || !grad || !m || !v || step < 1) return SHK_EINVAL;
    const float bc1 = 1.0f - powf(beta1, static_cast<float>(step));
    const float bc2 = 1.0f - powf(beta2, static_cast<float>(step));
    mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grad, m, v, kMlpParams, lr, beta1, beta2, eps, bc1, bc2);
    return lcheck(cudaGetLastError());
}

int shk_learned_faces_f32(const shk_scheme* scheme, const float* stencils, float* out, int64_t n,
                          void* stream) {
    if (!scheme || !scheme->mlp || !stencils || !out || n <= 0) return SHK_EINVAL;
    LearnedParams lp{scheme->mlp, static_cast<float>(scheme->eps), scheme->tau, scheme->band,
                     scheme->dev, norm_floor(scheme->norm_eps)};
    const int64_t tiles = (n + 31) / 32;
    const int blocks = static_cast<int>((tiles + 7) / 8 < 4096 ? (tiles + 7) / 8 : 4096);
    learned_faces_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(lp, stencils, out, n);
    return lcheck(cudaGetLastError());
}

}  // extern "C"
