// Forward kernels: spatial operator, CFL time step, fused SSPRK33 step, batched
// persistent stepping with per-instance dt, and the C ABI around them.
//
// Reference path replaced (alexfikl/pyshocks):
//   apply_operator      src/pyshocks/schemes.py:339-346
//   periodic ghost fill src/pyshocks/scalar.py:529-540
//   numerical fluxes    src/pyshocks/scalar.py:91-132,192-278,
//                       src/pyshocks/burgers/schemes.py:98-153,230-256
//   predict_timestep    src/pyshocks/burgers/schemes.py:42-49,121-127
//   step / SSPRK33      src/pyshocks/timestepping.py:89-152,312-320
//
// Periodic boundaries are applied by circular indexing of the n interior
// cells: with stencil reach 3 and 3 ghost cells the reference's interior
// outputs equal the circular ones (its zero padding reaches ghost outputs only).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "stencil.cuh"
#ifdef SHOCKS_BOUNDS_CHECK
#include "shocks_check.h"
#endif

namespace shk {

// ---------------------------------------------------------------------------
// batched persistent stepping kernel
// ---------------------------------------------------------------------------
__device__ void finalize_step(const PlanDev& P, int64_t k) {
    const int cur = static_cast<int>(k & 1);
    for (int b = threadIdx.x; b < P.B; b += blockDim.x) {
        unsigned long long* am = P.amax + size_t(cur) * P.B + b;
        const DtState s = plan_dt(P, k, b, from_bits(*am));
        double rec = 0.0;
        if (s.active) {
            if (s.finite) {
                P.t[b] = P.t[b] + s.dt;
                rec = s.dt;
            } else {
                atomicOr(P.status, ERR_NONFINITE);
            }
        }
        if (P.dt_hist && k < P.max_steps) P.dt_hist[size_t(k) * P.B + b] = rec;
        *am = 0ull;
    }
}

template <class T, int EQ, int REC, int FLUX>
__global__ void __launch_bounds__(kThreads, REC == SHK_REC_LEARNED ? 3 : (REC == SHK_REC_WENOJS53 ? (sizeof(T) == 8 ? 3 : 4) : 1)) batched_step_kernel(PlanDev P, const T* __restrict__ uin,
                                                                T* __restrict__ uout, OpParams<T> p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ unsigned long long red[32];
    __shared__ int is_last;
    __shared__ DtState item_dt;  // the item's step, computed once per CTA
    __shared__ T item_dtdx, item_dx;
    constexpr int HL = step_halo<T>();
    using B = typename Bits<T>::type;

    Smem<T> sm;
    carve_step<T, REC>(sm, smem_raw, P.tile + 2 * HL);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    learned_stage<REC>(p.lp);
    uint32_t phase = 0;
    const int64_t k = *reinterpret_cast<volatile int64_t*>(P.step);
    const int cur = static_cast<int>(k & 1), nxt = cur ^ 1;
    bool ok = true;
    const int64_t total = P.offsets[P.B];
    const Win<const T> guin = make_win(uin, total);
    const Win<T> guout = make_win(uout, total);

    __shared__ int s_item;
    for (int item = next_item(P, 0, &s_item); item >= 0 && ok; item = next_item(P, 0, &s_item)) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        // one thread evaluates the step (double divisions: a 1/64-rate pipe on
        // this GPU) and shares it; the previous item's readers are past the
        // barrier that ended that item
        if (threadIdx.x == 0) {
            const DtState d = plan_dt(P, k, b, from_bits(P.amax[size_t(cur) * P.B + b]));
            item_dt = d;
            item_dtdx = static_cast<T>(d.dt * P.inv_dx[b]);
            item_dx = static_cast<T>(1.0 / P.inv_dx[b]);
        }
        __syncthreads();
        const DtState ds = item_dt;
        B mx = 0;
        if (!(ds.active && ds.finite)) {
            // instance finished or frozen: copy the tile through
            for (int i = threadIdx.x; i < te; i += blockDim.x) {
                const T v = guin[off + s0 + i];
                guout[off + s0 + i] = v;
                const B bb = abs_bits(wave_speed<EQ>(v, p.c));
                mx = bb > mx ? bb : mx;
            }
        } else {
            ok = load_window<T>(sm.U, uin + off, n, s0 - HL, te + 2 * HL, &bar, phase);
            if (!ok) {
                if (threadIdx.x == 0) atomicOr(P.status, ERR_TIMEOUT);
                break;
            }
            const T dtdx = item_dtdx;
            OpParams<T> pb = p;
            pb.dx = item_dx;
            mx = step_tile<T, EQ, REC, FLUX>(sm, guout + (off + s0), te, dtdx, pb, plan_bc(P, b, k),
                                             s0 - HL, n);
        }
        const B bm = block_max<B>(mx, reinterpret_cast<B*>(red));
        if (threadIdx.x == 0) atomicMax(P.amax + size_t(nxt) * P.B + b, to_double_bits<T>(bm));
        __syncthreads();
    }

    // completion: the last CTA of the step advances t, records dt, resets the
    // consumed maxima and increments the step counter (no host round trip)
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(P.done, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        finalize_step(P, k);
        __syncthreads();
        if (threadIdx.x == 0) {
            *reinterpret_cast<volatile unsigned*>(P.done) = 0u;
            atomicExch(P.sched, 0u);  // every CTA has taken its last item
            *reinterpret_cast<volatile int64_t*>(P.step) = k + 1;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// batched global Lax-Friedrichs: one launch per SSPRK33 stage
// ---------------------------------------------------------------------------
// The wave speed of the global Lax-Friedrichs flux is the maximum of |f'| over
// the whole instance, for each stage state (scalar.py:258-278 under
// timestepping.py:312-320), so the stages cannot be fused with halo
// recompute. Stage S reads a window of its input k (u, k1 or k2) and u, writes
// its output (k1, k2 or u+) and accumulates the instance maximum of |f'| of the
// output for the next stage (amax_out). Stage 1 uses the step's own maximum
// (amax[cur], which is also the CFL maximum), and every stage evaluates the
// instance's dt the same way; the last CTA of stage 3 finalises the step as
// batched_step_kernel does and clears the stage maxima. float64 states,
// periodic instances, the reference's stage formulas:
//   k1 = u + dt L(u),  k2 = 3/4 u + 1/4 (k1 + dt L(k1)),  u+ = 1/3 u + 2/3 (k2 + dt L(k2)).
template <int EQ, int STAGE>
__global__ void __launch_bounds__(kThreads) batched_lf_stage_kernel(
    PlanDev P, const double* __restrict__ u, const double* __restrict__ kin, double* __restrict__ kout,
    const unsigned long long* __restrict__ amax_in, unsigned long long* amax_out,
    unsigned long long* amax_clear, OpParams<double> p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ unsigned long long red[32];
    __shared__ int is_last;
    __shared__ DtState item_dt;
    __shared__ double item_dtdx, item_amax;
    constexpr int HL = op_halo<double>();
    Smem<double> sm;
    sm.carve(smem_raw, P.tile + 2 * HL);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const int64_t k = *reinterpret_cast<volatile int64_t*>(P.step);
    const int cur = static_cast<int>(k & 1);
    const int64_t total = P.offsets[P.B];
    const Win<const double> gu = make_win(u, total);
    const Win<double> gout = make_win(kout, total);
    // stage 1 reads the step's own maximum, stage 3 writes the next step's
    // (the parity of the device step counter picks the slot)
    const unsigned long long* ain = STAGE == 1 ? P.amax + size_t(cur) * P.B : amax_in;
    unsigned long long* aout = STAGE == 3 ? P.amax + size_t(cur ^ 1) * P.B : amax_out;
    bool ok = true;
    __shared__ int s_item;
    for (int item = next_item(P, 6, &s_item); item >= 0 && ok; item = next_item(P, 6, &s_item)) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        if (threadIdx.x == 0) {
            const DtState d = plan_dt(P, k, b, from_bits(P.amax[size_t(cur) * P.B + b]));
            item_dt = d;
            item_dtdx = d.dt * P.inv_dx[b];
            item_amax = from_bits(ain[b]);
        }
        __syncthreads();
        const DtState ds = item_dt;
        unsigned long long mx = 0;
        if (!(ds.active && ds.finite)) {
            // instance finished or frozen: every stage state is u
            for (int i = threadIdx.x; i < te; i += blockDim.x) {
                const double v = gu[off + s0 + i];
                gout[off + s0 + i] = v;
                const unsigned long long bb = abs_bits(wave_speed<EQ>(v, p.c));
                mx = bb > mx ? bb : mx;
            }
        } else {
            ok = load_window<double>(sm.U, kin + off, n, s0 - HL, te + 2 * HL, &bar, phase);
            if (!ok) {
                if (threadIdx.x == 0) atomicOr(P.status, ERR_TIMEOUT);
                break;
            }
            OpParams<double> pb = p;
            pb.hnu_amax = p.hnu * item_amax;
            face_fluxes<double, EQ, SHK_REC_WENOJS53, SHK_FLUX_LF>(sm.U, HL, HL + te, sm, pb);
            const double dtdx = item_dtdx;
            for (int i = threadIdx.x; i < te; i += blockDim.x) {
                const int w = HL + i;
                const double kk = fma(dtdx, sm.D[w - 1] - sm.D[w], sm.U[w]);  // k + dt L(k)
                double v;
                if constexpr (STAGE == 1) v = kk;
                else if constexpr (STAGE == 2) v = fma(1.0 / 4.0, kk, (3.0 / 4.0) * gu[off + s0 + i]);
                else v = fma(2.0 / 3.0, kk, (1.0 / 3.0) * gu[off + s0 + i]);
                gout[off + s0 + i] = v;
                const unsigned long long bb = abs_bits(wave_speed<EQ>(v, p.c));
                mx = bb > mx ? bb : mx;
            }
        }
        const unsigned long long bm = block_max<unsigned long long>(mx, red);
        if (threadIdx.x == 0) atomicMax(aout + b, bm);
        __syncthreads();
    }
    if constexpr (STAGE < 3) {
        finish_items(P, 6);
    } else {
        // the last CTA of the step: time, dt history, step counter, and the
        // stage maxima cleared for the next step
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            const unsigned prev = atomicAdd(P.done, 1u);
            is_last = (prev == gridDim.x - 1);
        }
        __syncthreads();
        if (is_last) {
            __threadfence();
            finalize_step(P, k);
            for (int i = threadIdx.x; i < 2 * P.B; i += blockDim.x) amax_clear[i] = 0ull;
            __syncthreads();
            if (threadIdx.x == 0) {
                *reinterpret_cast<volatile unsigned*>(P.done) = 0u;
                atomicExch(P.sched + 6, 0u);
                atomicExch(P.sched + 7, 0u);
                *reinterpret_cast<volatile int64_t*>(P.step) = k + 1;
                __threadfence();
            }
        }
    }
}

__global__ void fill_kernel(double* x, int n, double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = v;
}

// max |f'(u)| per instance into amax[cur] (plan reset / priming)
template <class T, int EQ>
__global__ void __launch_bounds__(kThreads) batched_max_kernel(PlanDev P, const T* __restrict__ u, T c,
                                                               int slot) {
    __shared__ unsigned long long red[32];
    using B = typename Bits<T>::type;
    for (int item = blockIdx.x; item < P.nitems; item += gridDim.x) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        B mx = 0;
        for (int i = threadIdx.x; i < te; i += blockDim.x) {
            const B bb = abs_bits(wave_speed<EQ>(u[off + s0 + i], c));
            mx = bb > mx ? bb : mx;
        }
        const B bm = block_max<B>(mx, reinterpret_cast<B*>(red));
        if (threadIdx.x == 0) atomicMax(P.amax + size_t(slot) * P.B + b, to_double_bits<T>(bm));
        __syncthreads();
    }
}

// deterministic FP64 reductions: per-item partials, then per-instance ordered sums
template <class T>
__global__ void __launch_bounds__(kThreads) batched_partial_kernel(PlanDev P, const T* __restrict__ u,
                                                                   int mode) {
    __shared__ double red[32];
    for (int item = blockIdx.x; item < P.nitems; item += gridDim.x) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        double acc = 0.0;
        for (int i = threadIdx.x; i < te; i += blockDim.x) {
            const double v = static_cast<double>(u[off + s0 + i]);
            if (mode == 0) acc += v;
            else if (mode == 1) acc += fabs(v);
            else if (mode == 2) acc = fma(v, v, acc);
            else acc = fmax(acc, fabs(v));
        }
        // fixed-shape tree: deterministic for a given launch shape
        if (mode == -1) {
            for (int o = 16; o > 0; o >>= 1) acc = fmax(acc, __shfl_xor_sync(0xffffffffu, acc, o));
        } else {
            acc = warp_sum(acc);
        }
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double r = red[0];
            for (int w = 1; w < (blockDim.x >> 5); ++w) r = mode == -1 ? fmax(r, red[w]) : r + red[w];
            P.partial[item] = r;
        }
        __syncthreads();
    }
}
__global__ void instance_sum_kernel(PlanDev P, const int32_t* item_first, int mode, double* out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= P.B) return;
    double r = 0.0;
    for (int i = item_first[b]; i < item_first[b + 1]; ++i)
        r = mode == -1 ? fmax(r, P.partial[i]) : r + P.partial[i];
    out[b] = r;
}

// ---------------------------------------------------------------------------
// single-instance kernels on the reference's ghosted layout (n + 2g cells)
// ---------------------------------------------------------------------------
// the boundary of a single-instance call (kernel parameter copy)
__device__ __forceinline__ BcView call_bc(const shk_boundary& b, double dx) {
    BcView v;
    v.left = b.left;
    v.right = b.right;
    v.dir = &b.dirichlet[0][0][0];
    v.dir_ss = 6;
    v.neu = &b.neumann[0][0];
    v.neu_ss = 2;
    v.dx = dx;
    return v;
}

// ghost cells of a single-instance output after a non-periodic call: the
// boundary at `stage` applied to the new interior (Neumann mirrors it), or 0
// (zero_ghosts: the operator output, whose ghost values are unspecified)
template <class T>
__global__ void bc_ghost_kernel(T* __restrict__ out, int64_t n, int g, shk_boundary b, double dx,
                                int stage, int zero_ghosts) {
    const int t = threadIdx.x;
    if (t >= 2 * g) return;
    const int side = t / g, k = t - g * side;
    const int kind = side ? b.right : b.left;
    const int64_t gidx = side ? g + n + k : g - 1 - k;  // ghosted index of ghost k
    if (kind == SHK_BC_PERIODIC) return;
    if (zero_ghosts || k >= 3) {
        out[gidx] = T(0);
    } else if (kind == SHK_BC_DIRICHLET) {
        out[gidx] = static_cast<T>(b.dirichlet[stage][side][k]);
    } else {
        const int64_t mirror = side ? g + n - 1 - k : g + k;
        out[gidx] = out[mirror] - static_cast<T>((2 * k + 1) * dx * b.neumann[stage][side]);
    }
}

template <class T, int EQ, int REC, int FLUX>
__global__ void __launch_bounds__(kThreads) apply_operator_kernel(const T* __restrict__ u, T* __restrict__ out,
                                                                  int64_t n, int g, int tile, T dx,
                                                                  const double* amax, OpParams<T> p,
                                                                  int32_t* err, shk_boundary bcp) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int HL = op_halo<T>();
    Smem<T> sm;
    sm.carve(smem_raw, tile + 2 * HL);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    learned_stage<REC>(p.lp);
    uint32_t phase = 0;
    if constexpr (FLUX == SHK_FLUX_LF) p.hnu_amax = p.hnu * static_cast<T>(*amax);
    const int64_t s0 = int64_t(blockIdx.x) * tile;
    const int te = static_cast<int>(imin64(tile, n - s0));
    if (!load_window<T>(sm.U, u + g, n, s0 - HL, te + 2 * HL, &bar, phase)) {
        if (threadIdx.x == 0 && err) atomicOr(err, ERR_TIMEOUT);
        return;
    }
    const BcView bc = call_bc(bcp, static_cast<double>(dx));
    const bool periodic = bc.periodic();
    if (!periodic) apply_bc(sm.U, s0 - HL, n, 0, te + 2 * HL, bc, 0);
    face_fluxes<T, EQ, REC, FLUX>(sm.U, HL, HL + te, sm, p);
    const Win<T> gout = make_win(out, n + 2 * g);
    for (int i = threadIdx.x; i < te; i += blockDim.x) {
        const int w = HL + i;
        // -(f[1:] - f[:-1]) / dx  (schemes.py:346)
        const T r = -((sm.D[w] - sm.D[w - 1]) * p.fscale) / dx;
        const int64_t gi = s0 + i;
        gout[g + gi] = r;
        // ghost cells of the output: periodic image of the interior output
        if (periodic) {
            if (gi < g) gout[g + n + gi] = r;
            if (gi >= n - g) gout[gi - (n - g)] = r;
        }
    }
}

template <class T, int EQ>
__global__ void max_wavespeed_kernel(const T* __restrict__ u, int64_t n, T c, unsigned long long* out) {
    __shared__ unsigned long long red[32];
    using B = typename Bits<T>::type;
    B mx = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n;
         i += int64_t(gridDim.x) * blockDim.x) {
        const B bb = abs_bits(wave_speed<EQ>(u[i], c));
        mx = bb > mx ? bb : mx;
    }
    const B bm = block_max<B>(mx, reinterpret_cast<B*>(red));
    if (threadIdx.x == 0) atomicMax(out, to_double_bits<T>(bm));
}

__global__ void finalize_dt_kernel(double* dt, double cfl, double theta) {
    const double smax = from_bits(*reinterpret_cast<unsigned long long*>(dt));
    // theta * (0.5 dx^(2-alpha) / smax)   (burgers/schemes.py:127, examples/burgers.py:162)
    *dt = theta * (cfl / smax);
}

template <class T, int EQ, int REC, int FLUX>
__global__ void __launch_bounds__(kThreads) single_step_kernel(const T* __restrict__ u, T* __restrict__ uout,
                                                               int64_t n, int g, int tile, T dtdx,
                                                               OpParams<T> p, int32_t* err,
                                                               shk_boundary bcp, double dx) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int HL = step_halo<T>();
    Smem<T> sm;
    carve_step<T, REC>(sm, smem_raw, tile + 2 * HL);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    learned_stage<REC>(p.lp);
    uint32_t phase = 0;
    const int64_t s0 = int64_t(blockIdx.x) * tile;
    const int te = static_cast<int>(imin64(tile, n - s0));
    if (!load_window<T>(sm.U, u + g, n, s0 - HL, te + 2 * HL, &bar, phase)) {
        if (threadIdx.x == 0 && err) atomicOr(err, ERR_TIMEOUT);
        return;
    }
    const BcView bc = call_bc(bcp, dx);
    const Win<T> gout = make_win(uout, n + 2 * g);
    step_tile<T, EQ, REC, FLUX>(sm, gout + (g + s0), te, dtdx, p, bc, s0 - HL, n);
    __syncthreads();
    if (!bc.periodic()) return;  // ghosts: bc_ghost_kernel after the step
    // periodic ghost image of the new state
    for (int i = threadIdx.x; i < te; i += blockDim.x) {
        const int64_t gi = s0 + i;
        const T v = gout[g + gi];
        if (gi < g) gout[g + n + gi] = v;
        if (gi >= n - g) gout[gi - (n - g)] = v;
    }
}

}  // namespace shk

// ===========================================================================
// host side
// ===========================================================================
using namespace shk;

namespace {

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

int cuda_check(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libshocks: CUDA error %s\n", cudaGetErrorString(e));
        return SHK_ECUDA;
    }
    return SHK_OK;
}
#define SHK_CUDA(call)                                  \
    do {                                                \
        int _st = cuda_check(call);                     \
        if (_st != SHK_OK) return _st;                  \
    } while (0)

// the library's tile when the caller gives none: the shapes the autotuner
// picks on the bench batches (plans that keep a dt history are tuned for
// their reverse step, whose shared memory grows with the tile)
int default_tile(const shk_scheme* s, int dtype, int max_steps) {
    if (s->rec == SHK_REC_LEARNED) return max_steps > 0 ? 1024 : 2048;
    if (s->rec == SHK_REC_WENOJS53 && s->flux == SHK_FLUX_RUSANOV) {
        if (dtype == SHK_F32) return max_steps > 0 ? 1024 : 2048;
        return max_steps > 0 ? 512 : kDefaultTile;
    }
    return kDefaultTile;
}

bool valid_scheme(const shk_scheme* s) {
    if (!s) return false;
    if (s->flux < 0 || s->flux > SHK_FLUX_EO) return false;
    if (s->rec < 0 || s->rec > SHK_REC_MUSCLS) return false;
    if (s->rec == SHK_REC_MUSCL || s->rec == SHK_REC_MUSCLS) {
        if (s->limiter < SHK_LIM_NONE || s->limiter > SHK_LIM_KOREN) return false;
        if (s->rec == SHK_REC_MUSCLS && s->limiter == SHK_LIM_KOREN) return false;  // no slope form
        if (s->limiter == SHK_LIM_MINMOD && !(s->delta >= 1.0 && s->delta <= 2.0)) return false;
        if (s->limiter == SHK_LIM_VANALBADA && s->delta != 1.0 && s->delta != 2.0) return false;
    }
    if (s->equation < 0 || s->equation > SHK_EQ_LWR) return false;
    if ((s->flux == SHK_FLUX_ESWENO) != (s->rec == SHK_REC_ESWENO32)) return false;
    if (s->rec == SHK_REC_LEARNED && (s->flux != SHK_FLUX_RUSANOV || !s->mlp)) return false;
    // the upwind and Engquist-Osher fluxes are the reference's Burgers schemes;
    // the constant and WENO-JS3 reconstructions run with Rusanov, Godunov or EO
    if ((s->flux == SHK_FLUX_GODUNOV || s->flux == SHK_FLUX_EO) &&
        (s->equation != SHK_EQ_BURGERS || s->rec == SHK_REC_LEARNED))
        return false;
    if ((s->rec == SHK_REC_CONSTANT || s->rec == SHK_REC_WENOJS32 || s->rec == SHK_REC_MUSCL ||
         s->rec == SHK_REC_MUSCLS) && s->flux == SHK_FLUX_LF)
        return false;
    return true;
}

shk_boundary periodic_boundary() {
    shk_boundary b;
    std::memset(&b, 0, sizeof(b));
    b.left = b.right = SHK_BC_PERIODIC;
    return b;
}

// both sides periodic, or each Dirichlet / Neumann
// cells a reconstruction reads on each side of a cell (the reference's
// stencil_width): the single-instance entry points need that many ghosts
int rec_reach(int rec) {
    switch (rec) {
        case SHK_REC_CONSTANT: return 1;
        case SHK_REC_WENOJS32:
        case SHK_REC_ESWENO32:
        case SHK_REC_MUSCL:
        case SHK_REC_MUSCLS: return 2;
        default: return 3;
    }
}

bool valid_boundary(const shk_boundary& b) {
    auto ok = [](int k) { return k >= SHK_BC_PERIODIC && k <= SHK_BC_NEUMANN; };
    if (!ok(b.left) || !ok(b.right)) return false;
    return (b.left == SHK_BC_PERIODIC) == (b.right == SHK_BC_PERIODIC);
}

template <class T>
OpParams<T> make_params(const shk_scheme* s) {
    OpParams<T> p;
    p.eps = static_cast<T>(s->eps);
    p.delta = static_cast<T>(s->delta);
    p.hnu = static_cast<T>(0.5 * s->nu);
    p.c = static_cast<T>(s->speed);
    p.hnu_amax = T(0);
    p.lim = s->limiter;
    p.lim_param = static_cast<T>(s->delta);
    p.atol = static_cast<T>(s->eps);
    p.dx = T(1);  // set per call / per instance
    p.lp = LearnedParams{s->mlp, static_cast<float>(s->eps), s->tau, s->band, s->dev,
                         norm_floor(s->norm_eps)};
    // FP64 Burgers-Rusanov with nu = 1 stores 4 F (see face_fluxes)
    p.fscale = (sizeof(T) == 8 && s->flux == SHK_FLUX_RUSANOV && s->rec == SHK_REC_WENOJS53 &&
                s->equation == SHK_EQ_BURGERS && s->nu == 1.0) ? T(0.25) : T(1);
    return p;
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// dispatch helpers: call F.template operator()<T, EQ, REC, FLUX>()
// Burgers with the Godunov / Engquist-Osher flux and a WENO-JS5, WENO-JS3 or
// constant reconstruction
template <class T, class F>
int dispatch_upwind(const shk_scheme* s, F&& f) {
    constexpr int EQ = SHK_EQ_BURGERS;
    if (s->flux == SHK_FLUX_GODUNOV) {
        if (s->rec == SHK_REC_MUSCL) return f.template operator()<T, EQ, SHK_REC_MUSCL, SHK_FLUX_GODUNOV>();
        if (s->rec == SHK_REC_MUSCLS) return f.template operator()<T, EQ, SHK_REC_MUSCLS, SHK_FLUX_GODUNOV>();
        if (s->rec == SHK_REC_CONSTANT) return f.template operator()<T, EQ, SHK_REC_CONSTANT, SHK_FLUX_GODUNOV>();
        if (s->rec == SHK_REC_WENOJS32) return f.template operator()<T, EQ, SHK_REC_WENOJS32, SHK_FLUX_GODUNOV>();
        return f.template operator()<T, EQ, SHK_REC_WENOJS53, SHK_FLUX_GODUNOV>();
    }
    if (s->rec == SHK_REC_MUSCL) return f.template operator()<T, EQ, SHK_REC_MUSCL, SHK_FLUX_EO>();
    if (s->rec == SHK_REC_MUSCLS) return f.template operator()<T, EQ, SHK_REC_MUSCLS, SHK_FLUX_EO>();
    if (s->rec == SHK_REC_CONSTANT) return f.template operator()<T, EQ, SHK_REC_CONSTANT, SHK_FLUX_EO>();
    if (s->rec == SHK_REC_WENOJS32) return f.template operator()<T, EQ, SHK_REC_WENOJS32, SHK_FLUX_EO>();
    return f.template operator()<T, EQ, SHK_REC_WENOJS53, SHK_FLUX_EO>();
}

template <class T, class F>
int dispatch_scheme(const shk_scheme* s, F&& f) {
    switch (s->equation) {
#define SHK_EQ_CASE(EQ)                                                                 \
    case EQ:                                                                            \
        if constexpr (EQ == SHK_EQ_BURGERS) {                                           \
            if (s->flux == SHK_FLUX_GODUNOV || s->flux == SHK_FLUX_EO)                  \
                return dispatch_upwind<T>(s, f);                                        \
        }                                                                               \
        if (s->rec == SHK_REC_CONSTANT)                                                 \
            return f.template operator()<T, EQ, SHK_REC_CONSTANT, SHK_FLUX_RUSANOV>();  \
        if (s->rec == SHK_REC_WENOJS32)                                                 \
            return f.template operator()<T, EQ, SHK_REC_WENOJS32, SHK_FLUX_RUSANOV>();  \
        if (s->rec == SHK_REC_MUSCL)                                                    \
            return f.template operator()<T, EQ, SHK_REC_MUSCL, SHK_FLUX_RUSANOV>();     \
        if (s->rec == SHK_REC_MUSCLS)                                                   \
            return f.template operator()<T, EQ, SHK_REC_MUSCLS, SHK_FLUX_RUSANOV>();    \
        if (s->rec == SHK_REC_LEARNED)                                                  \
            return f.template operator()<T, EQ, SHK_REC_LEARNED, SHK_FLUX_RUSANOV>();   \
        if (s->rec == SHK_REC_ESWENO32) return f.template operator()<T, EQ, SHK_REC_ESWENO32, SHK_FLUX_ESWENO>(); \
        if (s->flux == SHK_FLUX_LF) return f.template operator()<T, EQ, SHK_REC_WENOJS53, SHK_FLUX_LF>(); \
        return f.template operator()<T, EQ, SHK_REC_WENOJS53, SHK_FLUX_RUSANOV>();
        SHK_EQ_CASE(SHK_EQ_BURGERS)
        SHK_EQ_CASE(SHK_EQ_ADVECTION)
        SHK_EQ_CASE(SHK_EQ_LWR)
#undef SHK_EQ_CASE
    }
    return SHK_EINVAL;
}


// launch functors (namespace scope: member templates are not allowed in local classes)
struct ApplyOpLaunch {
    const double* u; double* out; int64_t n; int g; int tile; double dx; const double* amax;
    OpParams<double> p; size_t smem; int blocks; cudaStream_t st; shk_boundary bc;
    template <class T, int EQ, int REC, int FLUX> int operator()() {
        auto k = apply_operator_kernel<T, EQ, REC, FLUX>;
        SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, kThreads, smem, st>>>(u, out, n, g, tile, dx, amax, p, nullptr, bc);
        return cuda_check(cudaGetLastError());
    }
};

struct SingleStepLaunch {
    const double* u; double* uo; int64_t n; int g; int tile; double dtdx;
    OpParams<double> p; size_t smem; int blocks; cudaStream_t st; shk_boundary bc; double dx;
    template <class T, int EQ, int REC, int FLUX> int operator()() {
        if constexpr (FLUX == SHK_FLUX_LF) {
            return SHK_EUNSUPPORTED;
        } else {
            auto k = single_step_kernel<T, EQ, REC, FLUX>;
            SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<blocks, kThreads, smem, st>>>(u, uo, n, g, tile, dtdx, p, nullptr, bc, dx);
            return cuda_check(cudaGetLastError());
        }
    }
};

template <class TS>
struct BatchedStepLaunch {
    PlanDev D; const TS* uin; TS* uout; OpParams<TS> p; size_t smem; int grid; cudaStream_t st;
    template <class T, int EQ, int REC, int FLUX> int operator()() {
        if constexpr (FLUX == SHK_FLUX_LF) {
            return SHK_EUNSUPPORTED;
        } else {
            auto k = batched_step_kernel<T, EQ, REC, FLUX>;
            SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k<<<grid, kThreads, smem, st>>>(D, uin, uout, p);
            return cuda_check(cudaGetLastError());
        }
    }
};

// one global Lax-Friedrichs step of a plan: the three stage launches
struct BatchedLfLaunch {
    PlanDev D; const double* uin; double* uout; double* k1; double* k2; unsigned long long* amax_lf;
    OpParams<double> p; size_t smem; int grid; cudaStream_t st;
    template <int EQ> int run() {
        auto s1 = batched_lf_stage_kernel<EQ, 1>;
        auto s2 = batched_lf_stage_kernel<EQ, 2>;
        auto s3 = batched_lf_stage_kernel<EQ, 3>;
        for (auto k : {s1, s2, s3})
            SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int B = D.B;
        s1<<<grid, kThreads, smem, st>>>(D, uin, uin, k1, nullptr, amax_lf, amax_lf, p);
        SHK_CUDA(cudaGetLastError());
        s2<<<grid, kThreads, smem, st>>>(D, uin, k1, k2, amax_lf, amax_lf + B, amax_lf, p);
        SHK_CUDA(cudaGetLastError());
        s3<<<grid, kThreads, smem, st>>>(D, uin, k2, uout, amax_lf + B, nullptr, amax_lf, p);
        return cuda_check(cudaGetLastError());
    }
};

// resident CTAs per SM of the step kernel a scheme dispatches to, at the
// given dynamic shared memory (registers and shared memory both counted)
struct StepOccupancy {
    size_t smem; int* out;
    template <class T, int EQ, int REC, int FLUX> int operator()() {
        if constexpr (FLUX == SHK_FLUX_LF) {
            if constexpr (sizeof(T) != 8) {
                return SHK_EUNSUPPORTED;
            } else {
                auto k = batched_lf_stage_kernel<EQ, 2>;
                SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                SHK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k, kThreads, smem));
                return SHK_OK;
            }
        } else {
            auto k = batched_step_kernel<T, EQ, REC, FLUX>;
            SHK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            SHK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k, kThreads, smem));
            return SHK_OK;
        }
    }
};

}  // namespace

struct shk_plan {
    shk_scheme scheme;
    int dtype = SHK_F64;
    int B = 0, tile = 0, nitems = 0, max_steps = 0, grid = 0;
    int64_t total_cells = 0;
    double theta = 1.0;
    // device buffers
    int32_t* item_inst = nullptr;
    int32_t* item_tile = nullptr;
    int32_t* item_first = nullptr;
    int64_t* offsets = nullptr;
    double* cfl = nullptr;
    double* inv_dx = nullptr;
    double* tfinal = nullptr;
    unsigned long long* amax = nullptr;
    double* t = nullptr;
    double* dt_hist = nullptr;
    int64_t* step = nullptr;
    unsigned int* done = nullptr;
    int32_t* status = nullptr;
    double* partial = nullptr;
    double* dt_fixed = nullptr;  // prescribed steps [fixed_cap][B], active when fixed_steps > 0
    int64_t fixed_cap = 0, fixed_steps = 0;
    int bc_left = SHK_BC_PERIODIC, bc_right = SHK_BC_PERIODIC;
    double* bc_dir = nullptr;  // [B][2][3]
    double* bc_neu = nullptr;  // [B][2], or per-step [bc_steps][3][B][2]
    int64_t bc_steps = 0;      // 0: time-independent boundary data
    size_t bc_dir_cap = 0, bc_neu_cap = 0;  // doubles allocated
    int32_t* item_order = nullptr;  // [nitems] longest first
    unsigned int* sched = nullptr;  // [8] scheduling counters
    // host mirror of the number of steps launched since reset
    int64_t host_steps = 0;
    // global Lax-Friedrichs plans: stage states k1, k2 and their maxima [2][B]
    double* lf_k1 = nullptr;
    double* lf_k2 = nullptr;
    unsigned long long* amax_lf = nullptr;
    // captured two-step graph
    cudaGraphExec_t graph = nullptr;
    void* graph_a = nullptr;
    void* graph_b = nullptr;

    PlanDev dev() const {
        PlanDev P;
        P.item_inst = item_inst; P.item_tile = item_tile; P.offsets = offsets; P.cfl = cfl;
        P.inv_dx = inv_dx; P.tfinal = tfinal; P.theta = theta; P.amax = amax; P.t = t;
        P.dt_hist = dt_hist; P.step = step; P.done = done; P.status = status;
        P.partial = partial; P.B = B;
        P.dt_fixed = fixed_steps > 0 ? dt_fixed : nullptr; P.fixed_steps = fixed_steps;
        P.bc_left = bc_left; P.bc_right = bc_right; P.bc_dir = bc_dir; P.bc_neu = bc_neu; P.nitems = nitems; P.tile = tile; P.max_steps = max_steps;
        P.item_order = item_order; P.sched = sched; P.bc_steps = bc_steps;
        return P;
    }
};

namespace {
template <class T>
int launch_max(shk_plan* P, const void* u, int slot, cudaStream_t st) {
    const PlanDev D = P->dev();
    const T c = static_cast<T>(P->scheme.speed);
    const T* uu = static_cast<const T*>(u);
    switch (P->scheme.equation) {
        case SHK_EQ_BURGERS: batched_max_kernel<T, SHK_EQ_BURGERS><<<P->grid, kThreads, 0, st>>>(D, uu, c, slot); break;
        case SHK_EQ_ADVECTION: batched_max_kernel<T, SHK_EQ_ADVECTION><<<P->grid, kThreads, 0, st>>>(D, uu, c, slot); break;
        default: batched_max_kernel<T, SHK_EQ_LWR><<<P->grid, kThreads, 0, st>>>(D, uu, c, slot); break;
    }
    return cuda_check(cudaGetLastError());
}

template <class T>
int launch_step(shk_plan* P, const void* uin, void* uout, cudaStream_t st) {
    const PlanDev D = P->dev();
    if (P->scheme.flux == SHK_FLUX_LF) {
        if constexpr (sizeof(T) != 8) {
            return SHK_EUNSUPPORTED;
        } else {
            const size_t smem = Smem<double>::host_bytes(P->tile + 2 * op_halo<double>());
            BatchedLfLaunch f{D, static_cast<const double*>(uin), static_cast<double*>(uout), P->lf_k1,
                              P->lf_k2, P->amax_lf, make_params<double>(&P->scheme), smem, P->grid, st};
            switch (P->scheme.equation) {
                case SHK_EQ_BURGERS: return f.run<SHK_EQ_BURGERS>();
                case SHK_EQ_ADVECTION: return f.run<SHK_EQ_ADVECTION>();
                default: return f.run<SHK_EQ_LWR>();
            }
        }
    }
    const size_t smem = Smem<T>::step_bytes(P->tile + 2 * step_halo<T>(), P->scheme.rec);
    OpParams<T> p = make_params<T>(&P->scheme);
    BatchedStepLaunch<T> f{D, static_cast<const T*>(uin), static_cast<T*>(uout), p, smem, P->grid, st};
    return dispatch_scheme<T>(&P->scheme, f);
}
}  // namespace

namespace shk {
int plan_view(shk_plan* plan, PlanDev* dev, int* dtype, int* grid, shk_scheme* scheme,
              int64_t* total_cells, int64_t* host_steps) {
    if (!plan) return SHK_EINVAL;
    if (host_steps) *host_steps = plan->host_steps;
    *dev = plan->dev();
    *dtype = plan->dtype;
    *grid = plan->grid;
    *scheme = plan->scheme;
    *total_cells = plan->total_cells;
    return SHK_OK;
}
}  // namespace shk

extern "C" {

const char* shk_strerror(int status) {
    switch (status) {
        case SHK_OK: return "ok";
        case SHK_EINVAL: return "invalid argument";
        case SHK_ENONFINITE: return "Time step is not finite";
        case SHK_ETIMEOUT: return "bounded device wait expired";
        case SHK_ECUDA: return "CUDA runtime error";
        case SHK_ENOMEM: return "out of device memory";
        case SHK_EUNSUPPORTED: return "unsupported scheme combination";
        case SHK_ETOOLARGE: return "size exceeds the static scratch of the no-allocation entry point";
        default: return "unknown status";
    }
}

int shk_version(void) { return 1; }

int shk_max_wavespeed_f64(const shk_scheme* scheme, const double* u, int64_t n, int32_t nghosts,
                          double* amax, void* stream) {
    // only the wave speed of the equation matters here (any flux and
    // reconstruction, e.g. Lax-Friedrichs with the constant reconstruction)
    if (!scheme || scheme->equation < SHK_EQ_BURGERS || scheme->equation > SHK_EQ_LWR || !u || !amax ||
        n <= 0 || nghosts < 0)
        return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    SHK_CUDA(cudaMemsetAsync(amax, 0, sizeof(double), st));
    const int blocks = static_cast<int>(imin64((n + kThreads - 1) / kThreads, 4 * sm_count()));
    const double c = scheme->speed;
    auto* out = reinterpret_cast<unsigned long long*>(amax);
    switch (scheme->equation) {
        case SHK_EQ_BURGERS: max_wavespeed_kernel<double, SHK_EQ_BURGERS><<<blocks, kThreads, 0, st>>>(u + nghosts, n, c, out); break;
        case SHK_EQ_ADVECTION: max_wavespeed_kernel<double, SHK_EQ_ADVECTION><<<blocks, kThreads, 0, st>>>(u + nghosts, n, c, out); break;
        default: max_wavespeed_kernel<double, SHK_EQ_LWR><<<blocks, kThreads, 0, st>>>(u + nghosts, n, c, out); break;
    }
    return cuda_check(cudaGetLastError());
}

int shk_apply_operator_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                              double* out, int64_t n, int32_t nghosts, double dx,
                              const double* amax, void* stream) {
    if (!valid_scheme(scheme) || !u || !out || n < 3 || nghosts < rec_reach(scheme->rec) || !(dx > 0))
        return SHK_EINVAL;
    if (scheme->flux == SHK_FLUX_LF && !amax) return SHK_EINVAL;
    const shk_boundary b = bc ? *bc : periodic_boundary();
    if (!valid_boundary(b)) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    const int tile = 512;
    const int W = tile + 2 * op_halo<double>();
    const size_t smem = Smem<double>::host_bytes(W);
    const int blocks = static_cast<int>((n + tile - 1) / tile);
    OpParams<double> p = make_params<double>(scheme);
    p.dx = dx;
    ApplyOpLaunch f{u, out, n, nghosts, tile, dx, amax, p, smem, blocks, st, b};
    const int r = dispatch_scheme<double>(scheme, f);
    if (r != SHK_OK || (b.left == SHK_BC_PERIODIC && b.right == SHK_BC_PERIODIC)) return r;
    bc_ghost_kernel<double><<<1, 64, 0, st>>>(out, n, nghosts, b, dx, 0, 1);
    return cuda_check(cudaGetLastError());
}

int shk_apply_operator_f64(const shk_scheme* scheme, const double* u, double* out, int64_t n,
                           int32_t nghosts, double dx, const double* amax, void* stream) {
    return shk_apply_operator_bc_f64(scheme, nullptr, u, out, n, nghosts, dx, amax, stream);
}

int shk_predict_timestep_f64(const shk_scheme* scheme, const double* u, int64_t n, int32_t nghosts,
                             double cfl, double theta, double* dt, void* stream) {
    int st = shk_max_wavespeed_f64(scheme, u, n, nghosts, dt, stream);
    if (st != SHK_OK) return st;
    finalize_dt_kernel<<<1, 1, 0, as_stream(stream)>>>(dt, cfl, theta);
    return cuda_check(cudaGetLastError());
}

int shk_ssprk33_step_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                            double* u_out, int64_t n, int32_t nghosts, double dx, double dt,
                            void* stream) {
    if (!valid_scheme(scheme) || !u || !u_out || n < 3 || nghosts < rec_reach(scheme->rec) || !(dx > 0))
        return SHK_EINVAL;
    if (!std::isfinite(dt)) return SHK_ENONFINITE;
    if (scheme->flux == SHK_FLUX_LF) return SHK_EUNSUPPORTED;  // global max per stage
    const shk_boundary b = bc ? *bc : periodic_boundary();
    if (!valid_boundary(b)) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    const int tile = 512;
    const int W = tile + 2 * step_halo<double>();
    const size_t smem = Smem<double>::step_bytes(W, scheme->rec);
    const int blocks = static_cast<int>((n + tile - 1) / tile);
    OpParams<double> p = make_params<double>(scheme);
    p.dx = dx;
    SingleStepLaunch f{u, u_out, n, nghosts, tile, dt / dx, p, smem, blocks, st, b, dx};
    const int r = dispatch_scheme<double>(scheme, f);
    if (r != SHK_OK || (b.left == SHK_BC_PERIODIC && b.right == SHK_BC_PERIODIC)) return r;
    bc_ghost_kernel<double><<<1, 64, 0, st>>>(u_out, n, nghosts, b, dx, 1, 0);
    return cuda_check(cudaGetLastError());
}

int shk_ssprk33_step_f64(const shk_scheme* scheme, const double* u, double* u_out, int64_t n,
                         int32_t nghosts, double dx, double dt, void* stream) {
    return shk_ssprk33_step_bc_f64(scheme, nullptr, u, u_out, n, nghosts, dx, dt, stream);
}

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
int shk_plan_destroy(shk_plan* plan) {
    if (!plan) return SHK_OK;
    if (plan->graph) cudaGraphExecDestroy(plan->graph);
    void* ptrs[] = {plan->item_inst, plan->item_tile, plan->item_first, plan->offsets, plan->cfl,
                    plan->inv_dx, plan->tfinal, plan->amax, plan->t, plan->dt_hist, plan->step,
                    plan->done, plan->status, plan->partial, plan->dt_fixed, plan->bc_dir,
                    plan->bc_neu, plan->item_order, plan->sched, plan->lf_k1, plan->lf_k2,
                    plan->amax_lf};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete plan;
    return SHK_OK;
}

int shk_plan_create(const shk_scheme* scheme, int32_t batch, const int64_t* h_offsets,
                    const double* h_dx, const double* h_cfl, double theta,
                    const shk_plan_opts* opts, shk_plan** out) {
    if (!out) return SHK_EINVAL;
    *out = nullptr;
    if (!valid_scheme(scheme) || batch <= 0 || !h_offsets || !h_dx || !h_cfl) return SHK_EINVAL;
    const int dtype = opts ? opts->dtype : SHK_F64;
    if (dtype != SHK_F64 && dtype != SHK_F32) return SHK_EINVAL;
    // global Lax-Friedrichs: float64 stage states kept between the stage launches
    const bool lf = scheme->flux == SHK_FLUX_LF;
    if (lf && dtype != SHK_F64) return SHK_EUNSUPPORTED;
    int tile = (opts && opts->tile > 0) ? opts->tile : default_tile(scheme, dtype, opts ? opts->max_steps : 0);
    const int align = dtype == SHK_F64 ? 2 : 4;
    if (tile % align || tile < 16 || tile > 8192) return SHK_EINVAL;
    // the learned phase's warp scratch lives in the window's free arrays
    if (scheme->rec == SHK_REC_LEARNED && tile < kLearnedMinTile) return SHK_EINVAL;
    std::vector<int32_t> inst, tl, first(batch + 1, 0);
    for (int b = 0; b < batch; ++b) {
        const int64_t n = h_offsets[b + 1] - h_offsets[b];
        if (n < 3 || !(h_dx[b] > 0)) return SHK_EINVAL;
        const int64_t ntiles = (n + tile - 1) / tile;
        first[b] = static_cast<int32_t>(inst.size());
        for (int64_t j = 0; j < ntiles; ++j) {
            inst.push_back(b);
            tl.push_back(static_cast<int32_t>(j));
        }
    }
    first[batch] = static_cast<int32_t>(inst.size());
    // scheduling order: longest items first (full tiles, then partial tiles
    // by decreasing length), ties in packing order
    std::vector<int32_t> order(inst.size());
    std::vector<int64_t> len(inst.size());
    for (size_t i = 0; i < inst.size(); ++i) {
        order[i] = static_cast<int32_t>(i);
        const int64_t n = h_offsets[inst[i] + 1] - h_offsets[inst[i]];
        len[i] = std::min<int64_t>(tile, n - int64_t(tl[i]) * tile);
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return len[x] > len[y]; });
    auto* P = new (std::nothrow) shk_plan();
    if (!P) return SHK_ENOMEM;
    P->scheme = *scheme;
    P->dtype = dtype;
    P->B = batch;
    P->tile = tile;
    P->nitems = static_cast<int>(inst.size());
    P->max_steps = opts ? std::max(0, opts->max_steps) : 0;
    P->theta = theta;
    P->total_cells = h_offsets[batch] - h_offsets[0];
    std::vector<double> inv(batch), inf(batch, DBL_MAX);
    for (int b = 0; b < batch; ++b) inv[b] = 1.0 / h_dx[b];
    auto alloc = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
    bool ok = alloc((void**)&P->item_inst, sizeof(int32_t) * P->nitems) &&
              alloc((void**)&P->item_tile, sizeof(int32_t) * P->nitems) &&
              alloc((void**)&P->item_first, sizeof(int32_t) * (batch + 1)) &&
              alloc((void**)&P->offsets, sizeof(int64_t) * (batch + 1)) &&
              alloc((void**)&P->cfl, sizeof(double) * batch) &&
              alloc((void**)&P->inv_dx, sizeof(double) * batch) &&
              alloc((void**)&P->tfinal, sizeof(double) * batch) &&
              alloc((void**)&P->amax, sizeof(unsigned long long) * 2 * batch) &&
              alloc((void**)&P->t, sizeof(double) * batch) &&
              alloc((void**)&P->step, sizeof(int64_t)) && alloc((void**)&P->done, sizeof(unsigned)) &&
              alloc((void**)&P->status, sizeof(int32_t)) &&
              alloc((void**)&P->partial, sizeof(double) * P->nitems) &&
              alloc((void**)&P->item_order, sizeof(int32_t) * P->nitems) &&
              alloc((void**)&P->sched, sizeof(unsigned) * 8);
    if (ok && P->max_steps > 0)
        ok = alloc((void**)&P->dt_hist, sizeof(double) * size_t(P->max_steps) * batch);
    if (ok && lf)
        ok = alloc((void**)&P->lf_k1, sizeof(double) * size_t(P->total_cells)) &&
             alloc((void**)&P->lf_k2, sizeof(double) * size_t(P->total_cells)) &&
             alloc((void**)&P->amax_lf, sizeof(unsigned long long) * 2 * batch) &&
             cudaMemset(P->amax_lf, 0, sizeof(unsigned long long) * 2 * batch) == cudaSuccess;
    if (!ok) {
        shk_plan_destroy(P);
        return SHK_ENOMEM;
    }
    ok = cudaMemcpy(P->item_inst, inst.data(), sizeof(int32_t) * P->nitems, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->item_tile, tl.data(), sizeof(int32_t) * P->nitems, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->item_order, order.data(), sizeof(int32_t) * P->nitems, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(P->sched, 0, sizeof(unsigned) * 8) == cudaSuccess &&
         cudaMemcpy(P->item_first, first.data(), sizeof(int32_t) * (batch + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->offsets, h_offsets, sizeof(int64_t) * (batch + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->cfl, h_cfl, sizeof(double) * batch, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->inv_dx, inv.data(), sizeof(double) * batch, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(P->tfinal, inf.data(), sizeof(double) * batch, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(P->amax, 0, sizeof(unsigned long long) * 2 * batch) == cudaSuccess &&
         cudaMemset(P->t, 0, sizeof(double) * batch) == cudaSuccess &&
         cudaMemset(P->step, 0, sizeof(int64_t)) == cudaSuccess &&
         cudaMemset(P->done, 0, sizeof(unsigned)) == cudaSuccess &&
         cudaMemset(P->status, 0, sizeof(int32_t)) == cudaSuccess;
    if (!ok) {
        shk_plan_destroy(P);
        return SHK_ECUDA;
    }
    // persistent grid: resident CTAs per SM x SMs
    int per_sm = opts && opts->ctas_per_sm > 0 ? opts->ctas_per_sm : 0;
    if (per_sm == 0) {
        const size_t smem = lf ? Smem<double>::host_bytes(tile + 2 * op_halo<double>())
                               : (dtype == SHK_F64 ? Smem<double>::step_bytes(tile + 2 * step_halo<double>(), scheme->rec)
                                                   : Smem<float>::step_bytes(tile + 2 * step_halo<float>(), scheme->rec));
        int resident = 0;
        const int r = dtype == SHK_F64 ? dispatch_scheme<double>(scheme, StepOccupancy{smem, &resident})
                                       : dispatch_scheme<float>(scheme, StepOccupancy{smem, &resident});
        if (r != SHK_OK || resident < 1) {
            shk_plan_destroy(P);
            return r != SHK_OK ? r : SHK_EINVAL;  // the window does not fit one SM
        }
        per_sm = std::min(resident, 8);
    }
    P->grid = std::max(1, std::min(P->nitems, per_sm * sm_count()));
    *out = P;
    return SHK_OK;
}

int shk_plan_state(shk_plan* plan, double** t, double** dt_hist, int64_t** step_counter) {
    if (!plan) return SHK_EINVAL;
    if (t) *t = plan->t;
    if (dt_hist) *dt_hist = plan->dt_hist;
    if (step_counter) *step_counter = plan->step;
    return SHK_OK;
}

int shk_plan_copy_time(shk_plan* plan, double* t_out, void* stream) {
    if (!plan || !t_out) return SHK_EINVAL;
    return cuda_check(cudaMemcpyAsync(t_out, plan->t, sizeof(double) * plan->B,
                                      cudaMemcpyDeviceToDevice, as_stream(stream)));
}

int shk_plan_copy_dt_history(shk_plan* plan, double* out, void* stream) {
    if (!plan || !out || !plan->dt_hist) return SHK_EINVAL;
    return cuda_check(cudaMemcpyAsync(out, plan->dt_hist,
                                      sizeof(double) * size_t(plan->max_steps) * plan->B,
                                      cudaMemcpyDeviceToDevice, as_stream(stream)));
}

int shk_plan_status(shk_plan* plan, int32_t* h_status, void* stream) {
    if (!plan || !h_status) return SHK_EINVAL;
    SHK_CUDA(cudaMemcpyAsync(h_status, plan->status, sizeof(int32_t), cudaMemcpyDeviceToHost,
                             as_stream(stream)));
    SHK_CUDA(cudaStreamSynchronize(as_stream(stream)));
#ifdef SHOCKS_BOUNDS_CHECK
    // the bounds-check build also reports a recorded out-of-bounds index
    int32_t flag = 0;
    const int r = shk_check_bounds(0, &flag, nullptr, nullptr, nullptr, nullptr);
    if (r != SHK_OK) return r;
    if (flag) *h_status |= ERR_BOUNDS;
#endif
    return SHK_OK;
}


int shk_plan_reset(shk_plan* plan, const void* u, const double* t0, const double* tfinal,
                   void* stream) {
    if (!plan || !u) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    const int B = plan->B;
    SHK_CUDA(cudaMemsetAsync(plan->amax, 0, sizeof(unsigned long long) * 2 * B, st));
    if (plan->amax_lf) SHK_CUDA(cudaMemsetAsync(plan->amax_lf, 0, sizeof(unsigned long long) * 2 * B, st));
    SHK_CUDA(cudaMemsetAsync(plan->step, 0, sizeof(int64_t), st));
    SHK_CUDA(cudaMemsetAsync(plan->done, 0, sizeof(unsigned), st));
    SHK_CUDA(cudaMemsetAsync(plan->sched, 0, sizeof(unsigned) * 8, st));
    SHK_CUDA(cudaMemsetAsync(plan->status, 0, sizeof(int32_t), st));
    if (t0) SHK_CUDA(cudaMemcpyAsync(plan->t, t0, sizeof(double) * B, cudaMemcpyDeviceToDevice, st));
    else SHK_CUDA(cudaMemsetAsync(plan->t, 0, sizeof(double) * B, st));
    if (tfinal) {
        SHK_CUDA(cudaMemcpyAsync(plan->tfinal, tfinal, sizeof(double) * B, cudaMemcpyDeviceToDevice, st));
    } else {  // no final time; a kernel, so that a reset never waits on the host
        fill_kernel<<<(B + kThreads - 1) / kThreads, kThreads, 0, st>>>(plan->tfinal, B, DBL_MAX);
        SHK_CUDA(cudaGetLastError());
    }
    if (plan->dt_hist)
        SHK_CUDA(cudaMemsetAsync(plan->dt_hist, 0, sizeof(double) * size_t(plan->max_steps) * B, st));
    plan->host_steps = 0;
    return plan->dtype == SHK_F64 ? launch_max<double>(plan, u, 0, st) : launch_max<float>(plan, u, 0, st);
}

int shk_plan_step(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps, void* stream) {
    if (!plan || !u_a || !u_b || u_a == u_b || nsteps < 0) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    for (int i = 0; i < nsteps; ++i) {
        const bool even = (plan->host_steps % 2) == 0;
        void* in = even ? u_a : u_b;
        void* out = even ? u_b : u_a;
        const int r = plan->dtype == SHK_F64 ? launch_step<double>(plan, in, out, st)
                                             : launch_step<float>(plan, in, out, st);
        if (r != SHK_OK) return r;
        plan->host_steps++;
    }
    return SHK_OK;
}

int shk_plan_set_fixed_dt(shk_plan* plan, const double* dt, int32_t nsteps, void* stream) {
    if (!plan || nsteps < 0 || (nsteps > 0 && !dt)) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    if (nsteps > plan->fixed_cap) {
        SHK_CUDA(cudaStreamSynchronize(st));
        if (plan->dt_fixed) cudaFree(plan->dt_fixed);
        plan->dt_fixed = nullptr;
        plan->fixed_cap = plan->fixed_steps = 0;
        if (cudaMalloc(&plan->dt_fixed, sizeof(double) * size_t(nsteps) * plan->B) != cudaSuccess)
            return SHK_ENOMEM;
        plan->fixed_cap = nsteps;
    }
    if (nsteps > 0)
        SHK_CUDA(cudaMemcpyAsync(plan->dt_fixed, dt, sizeof(double) * size_t(nsteps) * plan->B,
                                 cudaMemcpyDefault, st));
    plan->fixed_steps = nsteps;
    // the kernels take the plan's device view by value: a captured graph is stale now
    if (plan->graph) {
        cudaGraphExecDestroy(plan->graph);
        plan->graph = nullptr;
    }
    return SHK_OK;
}

}  // extern "C"

namespace {
// boundary kinds and data for every instance: `rows` sets of [B][2][3]
// Dirichlet values / [B][2] Neumann gradients (1: time-independent; else
// steps x 3 stages)
int set_plan_boundary(shk_plan* plan, int32_t left, int32_t right, const double* dirichlet,
                      const double* neumann, int64_t rows, int64_t steps, void* stream) {
    if (!plan || rows < 1) return SHK_EINVAL;
    shk_boundary b = periodic_boundary();
    b.left = left;
    b.right = right;
    if (!valid_boundary(b)) return SHK_EINVAL;
    // the global Lax-Friedrichs speed would also span the ghost values
    if (plan->scheme.flux == SHK_FLUX_LF && left != SHK_BC_PERIODIC) return SHK_EUNSUPPORTED;
    const bool need_dir = left == SHK_BC_DIRICHLET || right == SHK_BC_DIRICHLET;
    const bool need_neu = left == SHK_BC_NEUMANN || right == SHK_BC_NEUMANN;
    if ((need_dir && !dirichlet) || (need_neu && !neumann)) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    const size_t B = static_cast<size_t>(plan->B);
    auto ensure = [&](double** buf, size_t* cap, size_t n) {
        if (*cap >= n) return true;
        if (*buf) {
            if (cudaStreamSynchronize(st) != cudaSuccess) return false;  // a step may still read it
            cudaFree(*buf);
        }
        *buf = nullptr;
        *cap = 0;
        if (cudaMalloc(reinterpret_cast<void**>(buf), sizeof(double) * n) != cudaSuccess) return false;
        *cap = n;
        return true;
    };
    const size_t ndir = 6 * B * size_t(rows), nneu = 2 * B * size_t(rows);
    if (need_dir && !ensure(&plan->bc_dir, &plan->bc_dir_cap, ndir)) return SHK_ENOMEM;
    if (need_neu && !ensure(&plan->bc_neu, &plan->bc_neu_cap, nneu)) return SHK_ENOMEM;
    if (need_dir)
        SHK_CUDA(cudaMemcpyAsync(plan->bc_dir, dirichlet, sizeof(double) * ndir, cudaMemcpyDefault, st));
    if (need_neu)
        SHK_CUDA(cudaMemcpyAsync(plan->bc_neu, neumann, sizeof(double) * nneu, cudaMemcpyDefault, st));
    plan->bc_left = left;
    plan->bc_right = right;
    plan->bc_steps = steps;
    if (plan->graph) {  // kernels take the plan's device view by value
        cudaGraphExecDestroy(plan->graph);
        plan->graph = nullptr;
    }
    return SHK_OK;
}
}  // namespace

extern "C" {

int shk_plan_set_boundary(shk_plan* plan, int32_t left, int32_t right, const double* dirichlet,
                          const double* neumann, void* stream) {
    return set_plan_boundary(plan, left, right, dirichlet, neumann, 1, 0, stream);
}

int shk_plan_set_boundary_steps(shk_plan* plan, int32_t left, int32_t right,
                                const double* dirichlet, const double* neumann, int32_t nsteps,
                                void* stream) {
    if (nsteps < 1) return SHK_EINVAL;
    return set_plan_boundary(plan, left, right, dirichlet, neumann, 3 * int64_t(nsteps), nsteps,
                             stream);
}

int shk_plan_step_graph(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps, void* stream) {
    if (!plan || !u_a || !u_b || u_a == u_b || nsteps < 0 || nsteps % 2) return SHK_EINVAL;
    if (plan->host_steps % 2) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    if (st == nullptr) return SHK_EINVAL;  // capture needs a non-default stream
    if (!plan->graph || plan->graph_a != u_a || plan->graph_b != u_b) {
        if (plan->graph) {
            cudaGraphExecDestroy(plan->graph);
            plan->graph = nullptr;
        }
        cudaGraph_t g;
        SHK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int64_t saved = plan->host_steps;
        int r = shk_plan_step(plan, u_a, u_b, 2, stream);
        plan->host_steps = saved;
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (r != SHK_OK) return r;
        SHK_CUDA(e);
        e = cudaGraphInstantiate(&plan->graph, g, 0);
        cudaGraphDestroy(g);
        SHK_CUDA(e);
        plan->graph_a = u_a;
        plan->graph_b = u_b;
    }
    for (int i = 0; i < nsteps / 2; ++i) SHK_CUDA(cudaGraphLaunch(plan->graph, st));
    plan->host_steps += nsteps;
    return SHK_OK;
}

int shk_plan_reduce(shk_plan* plan, const void* u, int32_t p, double* out, void* stream) {
    if (!plan || !u || !out || (p != 0 && p != 1 && p != 2 && p != -1)) return SHK_EINVAL;
    cudaStream_t st = as_stream(stream);
    const PlanDev D = plan->dev();
    if (plan->dtype == SHK_F64)
        batched_partial_kernel<double><<<plan->grid, kThreads, 0, st>>>(D, static_cast<const double*>(u), p);
    else
        batched_partial_kernel<float><<<plan->grid, kThreads, 0, st>>>(D, static_cast<const float*>(u), p);
    SHK_CUDA(cudaGetLastError());
    instance_sum_kernel<<<(plan->B + 127) / 128, 128, 0, st>>>(D, plan->item_first, p, out);
    return cuda_check(cudaGetLastError());
}

}  // extern "C"

// ===========================================================================
// Lax-Friedrichs operator without any device allocation
// ===========================================================================
// Some callers cannot allocate device memory of their own. The main case for
// this library is an integration as a JAX custom call: JAX reserves most of the
// GPU for its own pool up front and hands a handler only its input and output
// buffers, so a cudaMalloc in the handler competes with (or fails against)
// that pool. The regular Lax-Friedrichs path needs one scratch value (the
// instance-wide max |f'(u)|) that the caller allocates; this variant keeps its
// scratch -- one partial maximum per 512-cell tile plus the final maximum -- in
// a fixed array compiled into the library instead.
//
// The array lives in every GPU's memory from the moment the library is loaded
// on that GPU until the process exits (kNoAllocMaxTiles + 1 doubles, 32 KiB).
// All calls share it: a call overwrites every slot it reads, so nothing has to
// start at zero, but two calls that overlap on the GPU (different streams, or
// different host threads) race on it and must be serialised by the caller.
namespace {

constexpr int kNoAllocTile = 512;          // cells per tile, as shk_apply_operator_f64
constexpr int kNoAllocMaxTiles = 4096;     // => at most 2,097,152 interior cells per call

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxTiles + 1];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoAllocAddr {
    unsigned long long ctx_id = 0;  // cuCtxGetId of the context the address belongs to
    double* addr = nullptr;
};
NoAllocAddr g_noalloc_addr[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique ID of the calling thread's current CUDA context (0 if none). The
// driver functions come through the runtime's entry-point query, so the
// library does not link libcuda itself.
unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
                cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
                cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess)
            return 0;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_noalloc_scratch in the current device's context. In host
// code the symbol itself is only a host-side stand-in, so the address must come
// from cudaGetSymbolAddress with that device current. It is looked up once per
// context: a context created after cudaDeviceReset loads the module again, so
// the address of an earlier context is not reused.
int noalloc_scratch(double** out) {
    int dev = 0;
    SHK_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return SHK_EUNSUPPORTED;
    const unsigned long long id = current_context_id();  // 0 before the runtime made one current
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocAddr& slot = g_noalloc_addr[dev];
    if (!slot.addr || id == 0 || slot.ctx_id != id) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "libshocks: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return SHK_ECUDA;
        }
        slot.addr = static_cast<double*>(p);
        slot.ctx_id = current_context_id();  // the context the lookup ran in
    }
    *out = slot.addr;
    return SHK_OK;
}

// per-tile max |f'(u)| into partial[tile]
template <int EQ>
__global__ void __launch_bounds__(kThreads) noalloc_tile_max_kernel(const double* __restrict__ u, int64_t n,
                                                                    double c, double* partial) {
    __shared__ unsigned long long red[32];
    const int64_t s0 = int64_t(blockIdx.x) * kNoAllocTile;
    const int te = static_cast<int>(imin64(kNoAllocTile, n - s0));
    unsigned long long mx = 0;
    for (int i = threadIdx.x; i < te; i += blockDim.x) {
        const unsigned long long b = abs_bits(wave_speed<EQ>(u[s0 + i], c));
        mx = b > mx ? b : mx;
    }
    const unsigned long long bm = block_max<unsigned long long>(mx, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = from_bits(bm);
}

// max of the ntiles partials into partial[kNoAllocMaxTiles]
__global__ void __launch_bounds__(kThreads) noalloc_reduce_kernel(double* partial, int ntiles) {
    __shared__ unsigned long long red[32];
    unsigned long long mx = 0;
    for (int i = threadIdx.x; i < ntiles; i += blockDim.x) {
        const unsigned long long b = abs_bits(partial[i]);
        mx = b > mx ? b : mx;
    }
    const unsigned long long bm = block_max<unsigned long long>(mx, red);
    if (threadIdx.x == 0) partial[kNoAllocMaxTiles] = from_bits(bm);
}

}  // namespace

extern "C" int shk_apply_operator_lf_noalloc_f64(const shk_scheme* scheme, const double* u,
                                                 double* out, int64_t n, int32_t nghosts,
                                                 double dx, void* stream) {
    if (!valid_scheme(scheme) || scheme->flux != SHK_FLUX_LF || !u || !out || n < 3 ||
        nghosts < 3 || !(dx > 0))
        return SHK_EINVAL;
    const int64_t ntiles = (n + kNoAllocTile - 1) / kNoAllocTile;
    if (ntiles > kNoAllocMaxTiles) {
        std::fprintf(stderr,
                     "libshocks: shk_apply_operator_lf_noalloc_f64: n = %lld exceeds the static "
                     "scratch limit of %lld cells\n",
                     static_cast<long long>(n),
                     static_cast<long long>(kNoAllocMaxTiles) * kNoAllocTile);
        return SHK_ETOOLARGE;
    }
    double* scratch = nullptr;
    const int st0 = noalloc_scratch(&scratch);
    if (st0 != SHK_OK) return st0;
    cudaStream_t st = as_stream(stream);
    const double c = scheme->speed;
    const int nt = static_cast<int>(ntiles);
    switch (scheme->equation) {
        case SHK_EQ_BURGERS: noalloc_tile_max_kernel<SHK_EQ_BURGERS><<<nt, kThreads, 0, st>>>(u + nghosts, n, c, scratch); break;
        case SHK_EQ_ADVECTION: noalloc_tile_max_kernel<SHK_EQ_ADVECTION><<<nt, kThreads, 0, st>>>(u + nghosts, n, c, scratch); break;
        default: noalloc_tile_max_kernel<SHK_EQ_LWR><<<nt, kThreads, 0, st>>>(u + nghosts, n, c, scratch); break;
    }
    SHK_CUDA(cudaGetLastError());
    noalloc_reduce_kernel<<<1, kThreads, 0, st>>>(scratch, nt);
    SHK_CUDA(cudaGetLastError());
    // the operator itself is the regular one, reading the max from the scratch
    const int W = kNoAllocTile + 2 * op_halo<double>();
    const size_t smem = Smem<double>::host_bytes(W);
    OpParams<double> p = make_params<double>(scheme);
    p.dx = dx;
    ApplyOpLaunch f{u, out, n, nghosts, kNoAllocTile, dx, scratch + kNoAllocMaxTiles, p, smem, nt, st,
                    periodic_boundary()};
    return dispatch_scheme<double>(scheme, f);
}

extern "C" int64_t shk_apply_operator_lf_noalloc_max_cells(void) {
    return static_cast<int64_t>(kNoAllocMaxTiles) * kNoAllocTile;
}

// ===========================================================================
// bounds-check build (libshocks_check.so): logs and test hooks
// ===========================================================================
#ifdef SHOCKS_BOUNDS_CHECK
extern "C" int shk_check_tu_adjoint(shk::BoundsLog* out, int32_t reset);
extern "C" int shk_check_tu_ghosted(shk::BoundsLog* out, int32_t reset);

extern "C" int shk_check_bounds(int32_t reset, int32_t* flag, int32_t* block, int32_t* thread,
                                int64_t* offset, int64_t* extent) {
    SHK_CUDA(cudaDeviceSynchronize());
    shk::BoundsLog logs[3] = {};
    SHK_CUDA(shk::bounds_log_read(&logs[0], reset != 0));
    int r = shk_check_tu_adjoint(&logs[1], reset);
    if (r == SHK_OK) r = shk_check_tu_ghosted(&logs[2], reset);
    if (r != SHK_OK) return r;
    const shk::BoundsLog* hit = nullptr;
    for (const shk::BoundsLog& l : logs)
        if (!hit && l.flag) hit = &l;
    if (flag) *flag = hit ? 1 : 0;
    if (block) *block = hit ? hit->block : -1;
    if (thread) *thread = hit ? hit->thread : -1;
    if (offset) *offset = hit ? hit->offset : 0;
    if (extent) *extent = hit ? hit->extent : 0;
    return SHK_OK;
}

extern "C" int shk_check_force_timeout(uint32_t extra_bytes, int64_t wait_limit) {
    const long long lim = static_cast<long long>(wait_limit);
    SHK_CUDA(cudaMemcpyToSymbol(shk::g_test_extra_tx, &extra_bytes, sizeof(extra_bytes)));
    SHK_CUDA(cudaMemcpyToSymbol(shk::g_test_wait_limit, &lim, sizeof(lim)));
    return SHK_OK;
}
#endif
