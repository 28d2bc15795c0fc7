// Shared device templates of the forward and adjoint kernels: shared-memory
// layout, flux phases of one stage, window loader (TMA 1D bulk copies with
// bounded mbarrier waits), CFL time step, fused SSPRK33 tile and the device
// view of a batched plan. See forward.cu for the reference lines followed.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include <type_traits>

#include "device.cuh"
#include "learned.cuh"

namespace shk {

constexpr int kThreads = 256;
constexpr int kDefaultTile = 1024;
// shortest tile of a plan with the learned reconstruction: its warp scratch
// (8 warps x 128 floats forward, x 192 in the reverse step) lives in window
// arrays that the learned phase leaves free (the face-flux array D, at least
// kLearnedScratch floats, in the mixed step; 2W floats in the float step, 3W
// in the reverse step)
constexpr int kLearnedMinTile = 512;
// floats of the forward learned phase's scratch (8 warps, 16-byte alignment slack)
constexpr int kLearnedScratch = (kThreads / 32) * kWarpScratch + 4;
// length of the face-flux array D of the mixed step's layout (the learned
// phase's scratch before it takes the fluxes)
__host__ __device__ constexpr int mixed_d_len(int W) { return W > kLearnedScratch ? W : kLearnedScratch; }

// halo of a window: 9 cells are needed for three fused stages, rounded up so
// that the window start stays 16-byte aligned for cp.async.bulk
template <class T> __host__ __device__ constexpr int step_halo() { return sizeof(T) == 8 ? 10 : 12; }
template <class T> __host__ __device__ constexpr int op_halo() { return 4; }

__host__ __device__ inline int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

__host__ __device__ inline int64_t imod(int64_t a, int64_t n) {
    int64_t r = a % n;
    return r < 0 ? r + n : r;
}

// the scratch of the learned phase: the nfloats floats of shared memory from
// `region` that the layout leaves free in that phase, from a 16-byte aligned
// start
template <class PR>
__device__ __forceinline__ Win<float> learned_scratch(PR region, int nfloats) {
    float* r = reinterpret_cast<float*>(win_raw(region));
    const uintptr_t a = reinterpret_cast<uintptr_t>(r);
    float* s = reinterpret_cast<float*>((a + 15) & ~uintptr_t(15));
    return make_win(s, nfloats - static_cast<int>(s - r));
}

// ---------------------------------------------------------------------------
// shared-memory layout of one work item (window of W cells)
// ---------------------------------------------------------------------------
template <class T>
struct Smem {
    Win<T> U;   // u at the start of the step (window)
    Win<T> S;   // stage state k1 / k2
    Win<T> H;   // half differences
    Win<T> D;   // half second differences; reused for face fluxes F
    Win<T> Q;   // 13/12 (2D)^2; reused for ES-WENO omega_0
    Win<T> UL;  // ul (value at the left face of the cell)
    Win<T> UR;  // ur (value at the right face of the cell)
    Win<T> I;   // float states: stage increments (see step_tile); null for double
    Win<float> scr;  // the learned phase's warp scratch (free in that phase)
    int W;      // window length (cells) of every array

    // float states carry one more array (the stage increments)
    static constexpr int kArrays = sizeof(T) == 4 ? 8 : 7;
    __host__ static size_t host_bytes(int W) { return size_t(kArrays) * W * sizeof(T); }
    // the step tile of a double state with the learned reconstruction runs in
    // mixed precision (step_tile_mixed) on the double window and 6 float arrays
    __host__ static size_t step_bytes(int W, int rec) {
        if (sizeof(T) == 8 && rec == SHK_REC_LEARNED)
            return size_t(W) * sizeof(double) + size_t(5 * W + mixed_d_len(W)) * sizeof(float);
        if (sizeof(T) == 4 && rec == SHK_REC_WENOJS53) return size_t(6) * W * sizeof(T);
        return host_bytes(W);
    }
    // float state with WENO-JS5: the reconstruction works from the window
    // values directly, so H and Q are not needed (6 arrays)
    __device__ void carve_compact(unsigned char* base, int W) {
        T* p = reinterpret_cast<T*>(base);
        U = make_win(p, W); S = make_win(p + W, W); D = make_win(p + 2 * W, W);
        UL = make_win(p + 3 * W, W); UR = make_win(p + 4 * W, W); I = make_win(p + 5 * W, W);
        H = Q = Win<T>();
        scr = Win<float>();
        this->W = W;
    }
    // compact layout of that mixed step: U (double window), then as float
    // arrays S (2W: uf, k), I (increments), UL, UR and D (mixed_d_len(W)
    // floats: the learned phase's warp scratch before it takes the face
    // fluxes); no H, and Q aliases D (the learned reconstruction uses neither)
    __device__ void carve_mixed(unsigned char* base, int W) {
        U = make_win(reinterpret_cast<T*>(base), W);
        float* f = reinterpret_cast<float*>(base + size_t(W) * sizeof(double));
        S = win_cast<T>(make_win(f, 2 * W));
        I = win_cast<T>(make_win(f + 2 * W, W));
        UL = win_cast<T>(make_win(f + 3 * W, W));
        UR = win_cast<T>(make_win(f + 4 * W, W));
        D = win_cast<T>(make_win(f + 5 * W, W));
        scr = learned_scratch(make_win(f + 5 * W, mixed_d_len(W)), mixed_d_len(W));
        H = Win<T>();
        Q = D;
        this->W = W;
    }
    __device__ void carve(unsigned char* base, int W) {
        T* p = reinterpret_cast<T*>(base);
        U = make_win(p, W); S = make_win(p + W, W); H = make_win(p + 2 * W, W);
        D = make_win(p + 3 * W, W); Q = make_win(p + 4 * W, W);
        UL = make_win(p + 5 * W, W); UR = make_win(p + 6 * W, W);
        I = kArrays > 7 ? make_win(p + 7 * W, W) : Win<T>();
        const int hd = 2 * W * int(sizeof(T) / sizeof(float));  // H and D as floats
        scr = learned_scratch(make_win(reinterpret_cast<float*>(p + 2 * W), hd), hd);
        this->W = W;
    }
};

template <class T>
struct OpParams {
    T eps, delta, hnu, c;  // WENO eps, ES-WENO delta, nu/2, advection speed
    T hnu_amax;            // LF: nu/2 * global max |f'|
    LearnedParams lp;      // learned reconstruction (float32 state only)
    T fscale;              // face values F are stored as F / fscale (see face_fluxes)
    int lim;               // MUSCL / MUSCLS limiter (SHK_LIM_*)
    T lim_param;           // its theta / van Albada variant
    T atol;                // MUSCL slope-ratio cut
    T dx;                  // cell size (the MUSCLS van Albada variant 2 slope)
};

// shared-memory layout of a step tile (see Smem::step_bytes)
template <class T, int REC>
__device__ __forceinline__ void carve_step(Smem<T>& sm, unsigned char* base, int W) {
    if constexpr (sizeof(T) == 8 && REC == SHK_REC_LEARNED) sm.carve_mixed(base, W);
    else if constexpr (sizeof(T) == 4 && REC == SHK_REC_WENOJS53) sm.carve_compact(base, W);
    else sm.carve(base, W);
}

// ---------------------------------------------------------------------------
// Dirichlet / Neumann boundaries (scalar.py:397-511) on a window. The window
// loader fills every position circularly; for a non-periodic instance the
// three ghost cells of each side (global cells -1-k and n+k, k = 0..2) are
// then overwritten before each operator evaluation. Positions beyond the
// ghosts keep the wrapped values: they reach only ghost outputs, which the
// next overwrite replaces, never an interior output (stencil reach 3).
// ---------------------------------------------------------------------------
struct BcView {
    int left = SHK_BC_PERIODIC, right = SHK_BC_PERIODIC;
    const double* dir = nullptr;  // dir[stage * dir_ss + side * 3 + k]
    int dir_ss = 0;
    const double* neu = nullptr;  // neu[stage * neu_ss + side]
    int neu_ss = 0;
    double dx = 1.0;
    __device__ bool periodic() const { return left == SHK_BC_PERIODIC && right == SHK_BC_PERIODIC; }
};

// S: window array; g0: global cell of window position 0; [wlo, whi): the
// positions holding values of this stage. Call after a barrier; ends with one.
template <class PS>
__device__ void apply_bc(PS S, int64_t g0, int64_t n, int wlo, int whi, const BcView& bc,
                         int stage) {
    using V = elem_t<PS>;
    const int t = threadIdx.x;
    if (t < 6) {
        const int side = t / 3, k = t - 3 * side;
        const int kind = side ? bc.right : bc.left;
        const int64_t w = (side ? n + k : -1 - k) - g0;
        if (kind != SHK_BC_PERIODIC && w >= wlo && w < whi) {
            V val;
            if (kind == SHK_BC_DIRICHLET) {
                val = static_cast<V>(bc.dir[stage * bc.dir_ss + side * 3 + k]);
            } else {
                const int64_t wm = (side ? n - 1 - k : k) - g0;  // mirrored interior cell
                val = S[wm] - static_cast<V>((2 * k + 1) * bc.dx * bc.neu[stage * bc.neu_ss + side]);
            }
            S[w] = val;
        }
    }
    __syncthreads();
}

// Transpose of the ghost fill on a cotangent window z over [wlo, whi): the
// cotangent of a Dirichlet ghost vanishes (its value is data), that of a
// Neumann ghost (mirror - (2k+1) dx g) moves to its mirrored interior cell.
// One thread walks the six ghosts in order (mirrors of the two sides can
// coincide on tiny instances). Call after a barrier; ends with one.
template <class PZ>
__device__ void bc_transpose(PZ z, int64_t g0, int64_t n, int wlo, int whi, const BcView& bc) {
    using V = elem_t<PZ>;
    if (threadIdx.x == 0) {
        for (int t = 0; t < 6; ++t) {
            const int side = t / 3, k = t - 3 * side;
            const int kind = side ? bc.right : bc.left;
            const int64_t w = (side ? n + k : -1 - k) - g0;
            if (kind == SHK_BC_PERIODIC || w < wlo || w >= whi) continue;
            if (kind == SHK_BC_NEUMANN) {
                const int64_t wm = (side ? n - 1 - k : k) - g0;
                if (wm >= wlo && wm < whi) z[wm] += z[w];
            }
            z[w] = V(0);
        }
    }
    __syncthreads();
}

// zero a window array at positions outside the instance [0, n) (the circular
// loader wrapped them in): cotangents of a non-periodic instance
template <class PZ>
__device__ void zero_outside(PZ z, int64_t g0, int64_t n, int wlo, int whi) {
    using V = elem_t<PZ>;
    for (int w = wlo + threadIdx.x; w < whi; w += blockDim.x) {
        const int64_t gi = g0 + w;
        if (gi < 0 || gi >= n) z[w] = V(0);
    }
    __syncthreads();
}

// float copy of the operator parameters (the mixed-precision learned path)
template <class T>
__host__ __device__ inline OpParams<float> float_params(const OpParams<T>& p) {
    OpParams<float> f;
    f.eps = static_cast<float>(p.eps);
    f.delta = static_cast<float>(p.delta);
    f.hnu = static_cast<float>(p.hnu);
    f.c = static_cast<float>(p.c);
    f.hnu_amax = static_cast<float>(p.hnu_amax);
    f.lp = p.lp;
    f.fscale = 1.0f;
    f.lim = p.lim;
    f.lim_param = static_cast<float>(p.lim_param);
    f.atol = static_cast<float>(p.atol);
    f.dx = static_cast<float>(p.dx);
    return f;
}

// Stage the network of a learned scheme in the block's shared memory (every
// kernel that may run the learned reconstruction, before its first use; the
// whole block; ends with a barrier). BACK: also the backward's fragments.
template <int REC, bool BACK = false>
__device__ __forceinline__ void learned_stage(const LearnedParams& lp) {
    if constexpr (REC == SHK_REC_LEARNED) {
        mlp_stage_forward(lp.mlp, mlp_shared());
        if constexpr (BACK) mlp_stage_back(lp.mlp, mlp_back_shared());
    }
}


// learned reconstruction of cells [clo, chi): one cell per lane, 32 cells per
// warp iteration, both faces of a cell from one network evaluation (the
// network staged by learned_stage). A cell's
// stencil relative to v_c is formed in the state precision straight from the
// window (v_{c+o} - v_c, o = -2..2) and rounded to float; the face values are
// v_c + correction in the state precision.
// scratch: kWarpScratch floats per warp of shared memory (16-byte aligned).
template <class T, class PV, class PO>
__device__ __forceinline__ void learned_phase(PV v, int clo, int chi, PO UL, PO UR,
                                              const LearnedParams& lp, const Win<float>& scratch) {
    const MlpShared& ms = mlp_shared();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float* scr = win_span(scratch, warp * kWarpScratch, kWarpScratch);
    const int ncell = chi - clo;
    const int myrow = 16 * (t >> 1) + 8 * (t & 1) + g;  // within the 32-cell block
    for (int q = warp; q * 32 < ncell; q += nw) {
        const int r = q * 32 + myrow;
        const int c = clo + min(r, ncell - 1);
        const T vc = v[c];
        const float ds[5] = {static_cast<float>(v[c - 2] - vc), static_cast<float>(v[c - 1] - vc),
                             0.0f, static_cast<float>(v[c + 1] - vc),
                             static_cast<float>(v[c + 2] - vc)};
        float cr, cl;
        learned_cell32(ms, ds, lp, scr, cr, cl);
        if (r < ncell) {
            UR[c] = vc + static_cast<T>(cr);
            UL[c] = vc + static_cast<T>(cl);
        }
    }
}

// ---------------------------------------------------------------------------
// one evaluation of the numerical fluxes F_j (face j+1/2) for j in [lo-1, hi)
// from the stage input v (valid on [lo-3, hi+3)). Leaves F / p.fscale in sm.D
// (fscale = 1/4 for the FP64 Burgers-Rusanov flux with nu = 1, else 1).
// ---------------------------------------------------------------------------
template <class T, int EQ, int REC, int FLUX, class PV>
__device__ __forceinline__ void face_fluxes(PV v, int lo, int hi, const Smem<T>& sm,
                                            const OpParams<T>& p) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if constexpr (REC == SHK_REC_WENOJS53 && sizeof(T) == 8) {
        // FP64 (pipe-bound): unscaled differences, see weno53_cell_d.
        // phase A: d_c = v_{c+1} - v_c, c in [lo-3, hi+2)
        for (int c = lo - 3 + tid; c < hi + 2; c += nt) sm.H[c] = v[c + 1] - v[c];
        __syncthreads();
        // phase B: E_c = d_c - d_{c-1}, G_c = 13/3 E_c^2 + 4 eps, c in [lo-2, hi+2)
        const T eps4 = T(4) * p.eps;
        for (int c = lo - 2 + tid; c < hi + 2; c += nt) {
            const T e = sm.H[c] - sm.H[c - 1];
            sm.D[c] = e;
            sm.Q[c] = fma(T(13.0 / 3.0) * e, e, eps4);
        }
        __syncthreads();
#pragma unroll 2
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            T ul, ur;
            weno53_cell_d(v[c], sm.H[c - 1], sm.H[c], sm.D[c - 1], sm.D[c], sm.D[c + 1],
                          sm.Q[c - 1], sm.Q[c], sm.Q[c + 1], ul, ur);
            sm.UL[c] = ul;
            sm.UR[c] = ur;
        }
        __syncthreads();
    } else if constexpr (REC == SHK_REC_WENOJS53 && sizeof(T) == 4) {
        // float: each cell's differences straight from its five values (a few
        // more float operations, no barriers and about half the shared-memory
        // traffic of staged difference arrays)
        const float eps4 = 4.0f * p.eps;
#pragma unroll 2
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            const T vm2 = v[c - 2], vm1 = v[c - 1], v0 = v[c], vp1 = v[c + 1], vp2 = v[c + 2];
            T ul, ur;
            weno53_cell_f(v0, vm1 - vm2, v0 - vm1, vp1 - v0, vp2 - vp1, eps4, ul, ur);
            sm.UL[c] = ul;
            sm.UR[c] = ur;
        }
        __syncthreads();
    } else if constexpr (REC == SHK_REC_LEARNED) {
        // warp scratch: sm.scr (free in this phase; with tiles of at least
        // kLearnedMinTile every learned layout gives it kLearnedScratch floats
        // or more)
        learned_phase<T>(v, lo - 1, hi + 1, sm.UL, sm.UR, p.lp, sm.scr);
        __syncthreads();
    } else if constexpr (REC == SHK_REC_CONSTANT) {
        // reconstruction.py:153-163: ul = ur = u
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            sm.UL[c] = v[c];
            sm.UR[c] = v[c];
        }
        __syncthreads();
    } else if constexpr (REC == SHK_REC_MUSCL || REC == SHK_REC_MUSCLS) {
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            T ul, ur;
            if constexpr (REC == SHK_REC_MUSCL)
                muscl_cell<T>(v[c - 1], v[c], v[c + 1], p.lim, p.lim_param, p.atol, ul, ur);
            else
                muscls_cell<T>(v[c - 1], v[c], v[c + 1], p.lim, p.lim_param, p.dx, ul, ur);
            sm.UL[c] = ul;
            sm.UR[c] = ur;
        }
        __syncthreads();
    } else if constexpr (REC == SHK_REC_WENOJS32) {
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            T ul, ur;
            weno32_cell<T>(v[c - 1], v[c], v[c + 1], p.eps, ul, ur);
            sm.UL[c] = ul;
            sm.UR[c] = ur;
        }
        __syncthreads();
    } else {
        for (int c = lo - 1 + tid; c < hi + 1; c += nt) {
            T ul, ur, w0;
            esweno32_cell<T>(v[c - 1], v[c], v[c + 1], p.eps, ul, ur, w0);
            sm.UL[c] = ul;
            sm.UR[c] = ur;
            sm.Q[c] = w0;
        }
        __syncthreads();
    }
    // phase D: F_j, j in [lo-1, hi)
    for (int j = lo - 1 + tid; j < hi; j += nt) {
        T f;
        if constexpr (FLUX == SHK_FLUX_RUSANOV && EQ == SHK_EQ_BURGERS && sizeof(T) == 8) {
            if (p.fscale != T(1)) {
                // nu = 1: 4 F = L^2 + R^2 + 2a (R - L), stored with fscale = 1/4
                const T L = sm.UL[j + 1], R = sm.UR[j];
                const auto ab = abs_bits(v[j]) > abs_bits(v[j + 1]) ? abs_bits(v[j]) : abs_bits(v[j + 1]);
                f = fma(L, L, fma(R, R, twice_abs_bits(ab) * (R - L)));
            } else {
                f = rusanov_face<EQ, T>(sm.UR[j], sm.UL[j + 1], v[j], v[j + 1], p.hnu, p.c);
            }
        } else if constexpr (FLUX == SHK_FLUX_RUSANOV) {
            f = rusanov_face<EQ, T>(sm.UR[j], sm.UL[j + 1], v[j], v[j + 1], p.hnu, p.c);
        } else if constexpr (FLUX == SHK_FLUX_LF) {
            f = lf_face<EQ, T>(sm.UR[j], sm.UL[j + 1], p.hnu_amax, p.c);
        } else if constexpr (FLUX == SHK_FLUX_GODUNOV) {
            f = godunov_face<EQ, T>(sm.UR[j], sm.UL[j + 1], p.c);
        } else if constexpr (FLUX == SHK_FLUX_EO) {
            f = eo_face<EQ, T>(sm.UR[j], sm.UL[j + 1], p.c);
        } else {
            f = esweno_face<EQ, T>(sm.UR[j], sm.UL[j + 1], v[j], v[j + 1], sm.Q[j], sm.Q[j + 1],
                                   p.delta, p.c);
        }
        sm.D[j] = f;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// window loader: cells g0 .. g0+W-1 of a periodic instance (mod n) into dst.
// Uses cp.async.bulk (TMA 1D, no multicast) into the CTA's own shared memory
// when every piece is 16-byte aligned, plain coalesced loads otherwise.
// Returns false if the bulk copy did not complete within the wait limit.
// ---------------------------------------------------------------------------
template <class T>
__device__ bool load_window(Win<T> dst, const T* base, int64_t n, int64_t g0, int W,
                            uint64_t* bar, uint32_t& phase) {
    const size_t sz = sizeof(T);
    // a window no longer than its instance wraps at most once: one compare
    // instead of a 64-bit remainder per position
    const bool once = g0 >= -n && g0 + W <= 2 * n;
    auto wrap = [&](int64_t pos) -> int64_t {
        if (once) return pos < 0 ? pos + n : (pos >= n ? pos - n : pos);
        return imod(pos, n);
    };
    // order earlier generic-proxy accesses of dst before the async-proxy writes
    fence_proxy_async();
    // thread 0 decides between bulk copies and plain loads; the barrier that
    // broadcasts the decision also orders the fences before the copies
    bool bulk = false;
    if (threadIdx.x == 0) {
        bulk = (reinterpret_cast<uintptr_t>(base) % 16 == 0) &&
               (reinterpret_cast<uintptr_t>(win_raw(dst)) % 16 == 0);
        int64_t pos = g0;
        const int64_t end = g0 + W;
        int npieces = 0;
        while (pos < end && bulk) {
            const int64_t src = wrap(pos);
            const int64_t len = min(end - pos, n - src);
            if ((src * sz) % 16 || (len * sz) % 16 || ((pos - g0) * sz) % 16) bulk = false;
            pos += len;
            if (++npieces > 8) bulk = false;  // tiny instances: plain loads
        }
    }
    bulk = __syncthreads_or(bulk);
    if (!bulk) {
        for (int w = threadIdx.x; w < W; w += blockDim.x) {
            const int64_t src = wrap(g0 + w);
            if (chk_index(src, n)) dst[w] = base[src];
        }
        __syncthreads();
        return true;
    }
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, static_cast<uint32_t>(W * sz) + test_extra_tx());
        int64_t pos = g0;
        const int64_t end = g0 + W;
        while (pos < end) {
            const int64_t src = wrap(pos);
            const int64_t len = min(end - pos, n - src);
            // (bounds-check build: a piece outside the window or the instance is
            // not copied; the wait for it then expires)
            if (chk_index(src, n) && chk_index(src + len - 1, n) && win_fits(dst, pos - g0, len))
                bulk_g2s(win_raw(dst) + (pos - g0), base + src, static_cast<uint32_t>(len * sz), bar);
            pos += len;
        }
    }
    bool ok = mbar_wait_bounded(bar, phase);
    if (!ok) ok = mbar_wait_bounded(bar, phase);  // second bounded wait for copies in flight
    phase ^= 1u;
    return __syncthreads_and(ok) != 0;
}

// ---------------------------------------------------------------------------
// per-instance CFL time step (timestepping.py:139-145 with the Rusanov
// estimate of burgers/schemes.py:121-127 and the driver's theta)
// ---------------------------------------------------------------------------
struct DtState {
    double dt;
    bool active;  // t < tfinal (timestepping.py:133-134)
    bool finite;
};
__host__ __device__ inline DtState compute_dt(double smax, double cfl, double theta, double t,
                                              double tfinal) {
    DtState s;
    s.active = t < tfinal;
    double dt = theta * (cfl / smax);
    if (tfinal != INFINITY) {
        const double dtmin = tfinal - t;
        dt = (dt < dtmin ? dt : dtmin) + 1.0e-15;
    }
    s.dt = dt;
    s.finite = isfinite(dt);
    return s;
}

// ---------------------------------------------------------------------------
// What a replayed step hands to the reverse sweep (pointers to the tile's
// interior cells; null: not wanted): the stage states k1, k2 and, for the
// double WENO-JS5 step, the face values of u, k1 and k2. Their element type is
// the stage precision: float for the learned or float steps, double otherwise.
// ---------------------------------------------------------------------------
template <class S>
struct StageOut {
    Win<S> k1 = nullptr;
    Win<S> k2 = nullptr;
    Win<S> ulu = nullptr;
    Win<S> uru = nullptr;
    Win<S> ul1 = nullptr;
    Win<S> ur1 = nullptr;
    Win<S> ul2 = nullptr;  // face values of k2
    Win<S> ur2 = nullptr;
};
template <class T, int REC>
using stage_t = typename std::conditional<sizeof(T) == 8 && REC != SHK_REC_LEARNED, double, float>::type;

// the tile's interior [HL, HL + te) of a window array into out
template <class PO, class PW>
__device__ __forceinline__ void store_interior(PO out, PW w, int HL, int te) {
    using S = elem_t<PO>;
    if (out)
        for (int i = HL + threadIdx.x; i < HL + te; i += blockDim.x) out[i - HL] = static_cast<S>(w[i]);
}

// ---------------------------------------------------------------------------
// fused SSPRK33 step of one tile: window [s - HL, s + te + HL) -> u_out[s, s + te)
// returns the thread's max |f'(u_new)| bits
// ---------------------------------------------------------------------------
// Mixed precision (double state, learned reconstruction): the operator runs in
// float on the float-rounded stage states and each stage is an increment about
// the step's start state u, accumulated in float and added to u in double
// once per step:
//   k1 = u + i1,  k2 = 3/4 u + 1/4 (k1 + i2) = u + d2,  d2 = (i1 + i2) / 4,
//   u+ = 1/3 u + 2/3 (k2 + i3) = u + 2/3 (d2 + i3),
// with i_s = dt/dx (F_{j-1/2} - F_{j+1/2}) of stage s. Rounding the operator's
// inputs to float perturbs the increments only (the state itself is never
// rounded), and the learned reconstruction works in float/bfloat16 anyway;
// the double pipe then carries three operations per cell and step instead of
// the whole operator. Layout (Smem::carve_mixed, or the full double layout):
// U is the loaded double window, S holds the float window uf and the float
// stage state, I the increments.
// so (optional): the float stage states k1, k2 for a reverse step that then
// skips their recompute; gout may be null when only those are wanted (the
// last stage is skipped).
template <int EQ, int FLUX>
__device__ unsigned long long step_tile_mixed(const Smem<double>& sm, Win<double> gout, int te,
                                              double dtdx, const OpParams<double>& p,
                                              const BcView& bc, int64_t g0, int64_t n,
                                              const StageOut<float>& so = StageOut<float>()) {
    constexpr int HL = step_halo<double>();
    const int tid = threadIdx.x, nt = blockDim.x, W = sm.W;
    const OpParams<float> pf = float_params(p);
    Smem<float> fs;
    fs.U = win_cast<float>(sm.S);
    fs.S = fs.U + W;
    fs.H = win_cast<float>(sm.H);
    fs.D = win_cast<float>(sm.D);
    fs.Q = win_cast<float>(sm.Q);
    fs.UL = win_cast<float>(sm.UL);
    fs.UR = win_cast<float>(sm.UR);
    fs.I = win_cast<float>(sm.I);
    fs.scr = sm.scr;
    fs.W = W;
    const Win<float> inc = fs.I;
    const float dtf = static_cast<float>(dtdx);
    for (int i = tid; i < te + 2 * HL; i += nt) fs.U[i] = static_cast<float>(sm.U[i]);
    __syncthreads();
    if (!bc.periodic()) apply_bc(fs.U, g0, n, 0, te + 2 * HL, bc, 0);
    {
        const int lo = HL - 6, hi = HL + te + 6;
        face_fluxes<float, EQ, SHK_REC_LEARNED, FLUX>(fs.U, lo, hi, fs, pf);
        for (int i = lo + tid; i < hi; i += nt) {
            const float d = dtf * (fs.D[i - 1] - fs.D[i]);
            inc[i] = d;
            fs.S[i] = fs.U[i] + d;
        }
        __syncthreads();
        if (!bc.periodic()) apply_bc(fs.S, g0, n, lo, hi, bc, 1);
        store_interior(so.k1, fs.S, HL, te);
    }
    {
        const int lo = HL - 3, hi = HL + te + 3;
        face_fluxes<float, EQ, SHK_REC_LEARNED, FLUX>(fs.S, lo, hi, fs, pf);
        for (int i = lo + tid; i < hi; i += nt) {
            const float d = 0.25f * (inc[i] + dtf * (fs.D[i - 1] - fs.D[i]));
            inc[i] = d;
            fs.S[i] = fs.U[i] + d;
        }
        __syncthreads();
        if (!bc.periodic()) apply_bc(fs.S, g0, n, lo, hi, bc, 2);
        store_interior(so.k2, fs.S, HL, te);
    }
    unsigned long long mx = 0;
    if (!gout) return mx;
    {
        const int lo = HL, hi = HL + te;
        face_fluxes<float, EQ, SHK_REC_LEARNED, FLUX>(fs.S, lo, hi, fs, pf);
        for (int i = lo + tid; i < hi; i += nt) {
            const float d = (2.0f / 3.0f) * (inc[i] + dtf * (fs.D[i - 1] - fs.D[i]));
            const double un = sm.U[i] + static_cast<double>(d);
            gout[i - HL] = un;
            const unsigned long long b = abs_bits(wave_speed<EQ>(un, p.c));
            mx = b > mx ? b : mx;
        }
    }
    return mx;
}

// Float state, WENO-JS5 + Rusanov: each stage in one pass over the window,
// two adjacent cells per lane. A warp reconstructs the 64 cells r0 .. r0+63
// (r0 even), lane L the pair c0 = r0 + 2L, c0 + 1: its six window values come
// in three aligned 8-byte loads, and the pair shares its differences d,
// second differences E and the terms G = 13/3 E^2 + 4 eps (weno53_cell_fg).
// Each lane forms the fluxes of both its cells' right faces (the left face
// value of the next pair comes from the lane above by shuffle) and takes the
// flux of its first cell's left face from the lane below. The warp updates
// the 62 cells r0+1 .. r0+62. One barrier per stage, the same operations in
// the same order per cell as the one-cell-per-lane stage, so the same results
// bit for bit. The stages ping-pong between S (k1) and UL (k2), since a warp's
// output cells are other warps' stencil inputs.
template <int EQ>
__device__ unsigned int step_tile_f32_weno(const Smem<float>& sm, Win<float> gout, int te, float dtdx,
                                           const OpParams<float>& p, const BcView& bc, int64_t g0,
                                           int64_t n, const StageOut<float>& so) {
    constexpr int HL = step_halo<float>();
    constexpr unsigned kFull = 0xffffffffu;
    const bool np = !bc.periodic();
    if (np) apply_bc(sm.U, g0, n, 0, te + 2 * HL, bc, 0);
    dtdx *= p.fscale;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float eps4 = 4.0f * p.eps;
    const Win<float> K2 = sm.UL;
    unsigned int mx = 0;
    auto ld2 = [](const Win<float>& a, int i) {  // a[i], a[i+1]; i even
        return *reinterpret_cast<const float2*>(win_span(a, i, 2));
    };
    // stage s reads v on [lo-3, hi+3) and updates [lo, hi); pairs past hi
    // are clamped to the last even start at or below hi (their values only
    // feed unused faces), which keeps every load inside [lo-4, hi+4)
    auto stage = [&](const Win<float>& v, int lo, int hi, int s) {
        const int cmax = hi & ~1;
        for (int r0 = ((lo - 1) & ~1) + 62 * warp; r0 + 1 < hi; r0 += 62 * nw) {
            const int c0 = r0 + 2 * lane;
            const int cc = c0 < cmax ? c0 : cmax;
            const float2 wa = ld2(v, cc - 2), wb = ld2(v, cc), wc = ld2(v, cc + 2);
            const float dA = wa.y - wa.x, dB = wb.x - wa.y, dC = wb.y - wb.x, dD = wc.x - wb.y,
                        dE = wc.y - wc.x;
            const float EB = dB - dA, EC = dC - dB, ED = dD - dC, EE = dE - dD;
            const float GB = weno53_g_f(EB, eps4), GC = weno53_g_f(EC, eps4), GD = weno53_g_f(ED, eps4),
                        GE = weno53_g_f(EE, eps4);
            float ula, ura, ulb, urb;
            weno53_cell_fg(wb.x, dB, dC, EB, EC, ED, GB, GC, GD, ula, ura);
            weno53_cell_fg(wb.y, dC, dD, EC, ED, EE, GC, GD, GE, ulb, urb);
            const float uln = __shfl_down_sync(kFull, ula, 1);  // left face value of cell c0 + 2
            const float fa = rusanov_face<EQ, float>(ura, ulb, wb.x, wb.y, p.hnu, p.c);  // c0 + 1/2
            const float fb = rusanov_face<EQ, float>(urb, uln, wb.y, wc.x, p.hnu, p.c);  // c0 + 3/2
            const float fl = __shfl_up_sync(kFull, fb, 1);                               // c0 - 1/2
            const bool va = lane >= 1 && c0 >= lo && c0 < hi;
            const bool vb = lane <= 30 && c0 + 1 >= lo && c0 + 1 < hi;
            if (!(va || vb)) continue;
            const float2 u = ld2(sm.U, cc);
            const float ra = dtdx * (fl - fa), rb = dtdx * (fa - fb);
            if (s == 3) {
                const float2 inc = ld2(sm.I, cc);
                const float una = u.x + (2.0f / 3.0f) * (inc.x + ra);
                const float unb = u.y + (2.0f / 3.0f) * (inc.y + rb);
                if (va) {
                    gout[c0 - HL] = una;
                    const unsigned int bb = abs_bits(wave_speed<EQ>(una, p.c));
                    mx = bb > mx ? bb : mx;
                }
                if (vb) {
                    gout[c0 + 1 - HL] = unb;
                    const unsigned int bb = abs_bits(wave_speed<EQ>(unb, p.c));
                    mx = bb > mx ? bb : mx;
                }
                continue;
            }
            float da, db;
            if (s == 1) {
                da = ra;
                db = rb;
            } else {
                const float2 inc = ld2(sm.I, cc);
                da = 0.25f * (inc.x + ra);
                db = 0.25f * (inc.y + rb);
            }
            const Win<float>& out = s == 1 ? sm.S : K2;
            if (va && vb) {
                *reinterpret_cast<float2*>(win_span(sm.I, c0, 2)) = make_float2(da, db);
                *reinterpret_cast<float2*>(win_span(out, c0, 2)) = make_float2(u.x + da, u.y + db);
            } else if (va) {
                sm.I[c0] = da;
                out[c0] = u.x + da;
            } else {
                sm.I[c0 + 1] = db;
                out[c0 + 1] = u.y + db;
            }
        }
        __syncthreads();
    };
    stage(sm.U, HL - 6, HL + te + 6, 1);
    if (np) apply_bc(sm.S, g0, n, HL - 6, HL + te + 6, bc, 1);
    store_interior(so.k1, sm.S, HL, te);
    stage(sm.S, HL - 3, HL + te + 3, 2);
    if (np) apply_bc(K2, g0, n, HL - 3, HL + te + 3, bc, 2);
    store_interior(so.k2, K2, HL, te);
    if (!gout) return mx;
    stage(K2, HL, HL + te, 3);
    return mx;
}

// g0: global cell of window position 0 (s - HL); n: cells of the instance;
// bc: its boundary (periodic: nothing to overwrite)
// so: what the reverse sweep keeps of this step (StageOut); gout may then be
// null (the last stage is skipped)
template <class T, int EQ, int REC, int FLUX>
__device__ typename Bits<T>::type step_tile(const Smem<T>& sm, Win<T> gout, int te, T dtdx,
                                            const OpParams<T>& p, const BcView& bc = BcView(),
                                            int64_t g0 = 0, int64_t n = 0,
                                            const StageOut<stage_t<T, REC>>& so = StageOut<stage_t<T, REC>>()) {
    if constexpr (sizeof(T) == 8 && REC == SHK_REC_LEARNED)
        return step_tile_mixed<EQ, FLUX>(sm, gout, te, dtdx, p, bc, g0, n, so);
    if constexpr (sizeof(T) == 4 && REC == SHK_REC_WENOJS53 && FLUX == SHK_FLUX_RUSANOV)
        return step_tile_f32_weno<EQ>(sm, gout, te, dtdx, p, bc, g0, n, so);
    constexpr int HL = step_halo<T>();
    const int tid = threadIdx.x, nt = blockDim.x;
    const bool np = !bc.periodic();
    if (np) apply_bc(sm.U, g0, n, 0, te + 2 * HL, bc, 0);
    dtdx *= p.fscale;
    if constexpr (sizeof(T) == 4) {
        // float state: the stages as increments about u (as step_tile_mixed).
        // In float 1/3 + 2/3 rounds to 1 + 3e-8, so the textbook combination
        // would scale the mass by that every step; the increments telescope,
        // and conservation holds to rounding.
        {
            const int lo = HL - 6, hi = HL + te + 6;
            face_fluxes<T, EQ, REC, FLUX>(sm.U, lo, hi, sm, p);
            for (int i = lo + tid; i < hi; i += nt) {
                const T d = dtdx * (sm.D[i - 1] - sm.D[i]);
                sm.I[i] = d;
                sm.S[i] = sm.U[i] + d;
            }
            __syncthreads();
            if (np) apply_bc(sm.S, g0, n, lo, hi, bc, 1);
            store_interior(so.k1, sm.S, HL, te);
        }
        {
            const int lo = HL - 3, hi = HL + te + 3;
            face_fluxes<T, EQ, REC, FLUX>(sm.S, lo, hi, sm, p);
            for (int i = lo + tid; i < hi; i += nt) {
                const T d = T(0.25) * (sm.I[i] + dtdx * (sm.D[i - 1] - sm.D[i]));
                sm.I[i] = d;
                sm.S[i] = sm.U[i] + d;
            }
            __syncthreads();
            if (np) apply_bc(sm.S, g0, n, lo, hi, bc, 2);
            store_interior(so.k2, sm.S, HL, te);
        }
        using B = typename Bits<T>::type;
        B mx = 0;
        if (!gout) return mx;
        const int lo = HL, hi = HL + te;
        face_fluxes<T, EQ, REC, FLUX>(sm.S, lo, hi, sm, p);
        for (int i = lo + tid; i < hi; i += nt) {
            const T un = sm.U[i] + T(2.0 / 3.0) * (sm.I[i] + dtdx * (sm.D[i - 1] - sm.D[i]));
            gout[i - HL] = un;
            const B b = abs_bits(wave_speed<EQ>(un, p.c));
            mx = b > mx ? b : mx;
        }
        return mx;
    }
    // double state: the reference's stage formulas (timestepping.py:312-320)
    // stage 1: k1 = u + dt L(u) on [HL-6, HL+te+6)
    {
        const int lo = HL - 6, hi = HL + te + 6;
        face_fluxes<T, EQ, REC, FLUX>(sm.U, lo, hi, sm, p);
        store_interior(so.ulu, sm.UL, HL, te);
        store_interior(so.uru, sm.UR, HL, te);
        for (int i = lo + tid; i < hi; i += nt) sm.S[i] = fma(dtdx, sm.D[i - 1] - sm.D[i], sm.U[i]);
        __syncthreads();
        if (np) apply_bc(sm.S, g0, n, lo, hi, bc, 1);
        store_interior(so.k1, sm.S, HL, te);
    }
    // stage 2: k2 = 3/4 u + 1/4 (k1 + dt L(k1)) on [HL-3, HL+te+3) (in place over k1)
    {
        const int lo = HL - 3, hi = HL + te + 3;
        face_fluxes<T, EQ, REC, FLUX>(sm.S, lo, hi, sm, p);
        store_interior(so.ul1, sm.UL, HL, te);
        store_interior(so.ur1, sm.UR, HL, te);
        for (int i = lo + tid; i < hi; i += nt) {
            const T k = fma(dtdx, sm.D[i - 1] - sm.D[i], sm.S[i]);
            sm.S[i] = fma(T(1.0 / 4.0), k, T(3.0 / 4.0) * sm.U[i]);
        }
        __syncthreads();
        if (np) apply_bc(sm.S, g0, n, lo, hi, bc, 2);
        store_interior(so.k2, sm.S, HL, te);
    }
    // stage 3: u+ = 1/3 u + 2/3 (k2 + dt L(k2)) on the tile
    using B = typename Bits<T>::type;
    B mx = 0;
    if (!gout && !so.ul2) return mx;
    {
        const int lo = HL, hi = HL + te;
        face_fluxes<T, EQ, REC, FLUX>(sm.S, lo, hi, sm, p);
        store_interior(so.ul2, sm.UL, HL, te);
        store_interior(so.ur2, sm.UR, HL, te);
        if (!gout) return mx;
        for (int i = lo + tid; i < hi; i += nt) {
            const T k = fma(dtdx, sm.D[i - 1] - sm.D[i], sm.S[i]);
            const T un = fma(T(2.0 / 3.0), k, T(1.0 / 3.0) * sm.U[i]);
            gout[i - HL] = un;
            const B b = abs_bits(wave_speed<EQ>(un, p.c));
            mx = b > mx ? b : mx;
        }
    }
    return mx;
}

// device view of a batched plan (see shk_plan in forward.cu)
struct PlanDev {
    const int32_t* item_inst;
    const int32_t* item_tile;
    const int64_t* offsets;  // [B+1]
    const double* cfl;       // [B] 0.5 dx^(2-alpha)
    const double* inv_dx;    // [B]
    const double* tfinal;    // [B]
    double theta;
    unsigned long long* amax;  // [2][B] bits of max |f'(u)| (as double)
    double* t;                 // [B]
    double* dt_hist;           // [max_steps][B] or null
    int64_t* step;
    unsigned int* done;
    int32_t* status;
    double* partial;  // [nitems]
    const double* dt_fixed;  // [fixed_steps][B] prescribed steps, or null (CFL steps)
    int64_t fixed_steps;
    int bc_left, bc_right;   // SHK_BC_* of every instance
    const double* bc_dir;    // [B][2][3] Dirichlet ghost values, or [bc_steps][3][B][2][3]
    const double* bc_neu;    // [B][2] Neumann gradients, or [bc_steps][3][B][2]
    int64_t bc_steps;        // 0: time-independent data; else per-step, per-stage tables
    const int32_t* item_order;  // [nitems] items longest first (dynamic scheduling)
    unsigned int* sched;        // [8] item counters of the scheduled kernels
    int32_t B, nitems, tile, max_steps;
};

// Dynamic item scheduling. A CTA takes the next item of the plan's
// longest-first order from the counter sched[slot]; uneven items (partial
// tiles, copied-through instances) then balance over the persistent grid,
// where a fixed stride would hand some CTAs only long items. Returns the item,
// or -1 when none is left. Every caller's loop body ends with a barrier, which
// orders the read of *s_item before thread 0 overwrites it.
__device__ __forceinline__ int next_item(const PlanDev& P, int slot, int* s_item) {
    if (threadIdx.x == 0) *s_item = static_cast<int>(atomicAdd(P.sched + slot, 1u));
    __syncthreads();
    const int q = *s_item;
    return q < P.nitems ? P.item_order[q] : -1;
}

// end of a scheduled launch: the CTA that finishes last (counter
// sched[slot + 1]) resets both counters for the next launch
__device__ __forceinline__ void finish_items(const PlanDev& P, int slot) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(P.sched + slot + 1, 1u) == gridDim.x - 1) {
            atomicExch(P.sched + slot, 0u);
            atomicExch(P.sched + slot + 1, 0u);
            __threadfence();
        }
    }
}

// the boundary of instance b at step k: time-independent data (one set for
// all three stages), or the step's row of a per-step table (steps past the
// table take its last row)
__device__ __forceinline__ BcView plan_bc(const PlanDev& P, int b, int64_t k) {
    BcView v;
    v.left = P.bc_left;
    v.right = P.bc_right;
    if (!v.periodic()) {
        if (P.bc_steps > 0) {
            const int64_t kk = k < P.bc_steps ? k : P.bc_steps - 1;
            const size_t row = size_t(kk) * 3 * P.B + b;
            v.dir = P.bc_dir ? P.bc_dir + row * 6 : nullptr;
            v.dir_ss = 6 * P.B;
            v.neu = P.bc_neu ? P.bc_neu + row * 2 : nullptr;
            v.neu_ss = 2 * P.B;
        } else {
            v.dir = P.bc_dir ? P.bc_dir + size_t(b) * 6 : nullptr;
            v.neu = P.bc_neu ? P.bc_neu + size_t(b) * 2 : nullptr;
        }
        v.dx = 1.0 / P.inv_dx[b];
    }
    return v;
}

// time step k of instance b: the prescribed step when the plan has a dt table
// (a step <= 0 or past the table's end leaves the instance unchanged, a
// non-finite one is an error), else the CFL step clipped at tfinal
__device__ __forceinline__ DtState plan_dt(const PlanDev& P, int64_t k, int b, double smax) {
    if (P.dt_fixed) {
        DtState s;
        s.dt = k < P.fixed_steps ? P.dt_fixed[size_t(k) * P.B + b] : 0.0;
        s.active = !(s.dt <= 0.0);
        s.finite = isfinite(s.dt);
        return s;
    }
    return compute_dt(smax, P.cfl[b], P.theta, P.t[b], P.tfinal[b]);
}

template <class T>
__device__ __forceinline__ unsigned long long to_double_bits(typename Bits<T>::type b) {
    if constexpr (sizeof(T) == 8) return b;
    else return abs_bits(static_cast<double>(from_bits(b)));
}

// read-only view of a plan's device state (defined in forward.cu)
int plan_view(shk_plan* plan, PlanDev* dev, int* dtype, int* grid, shk_scheme* scheme,
              int64_t* total_cells, int64_t* host_steps);

}  // namespace shk
