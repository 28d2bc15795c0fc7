// Discrete adjoint of the SSPRK33 / WENO-JS5 / Rusanov step (dt frozen).
//
// Reference: adjoint_step (src/pyshocks/timestepping.py:155-215) builds the
// dense Jacobian of one step with jax.jacfwd(advance) (:174) and applies
// p <- jac.T @ p (:206), with dt re-read from the forward checkpoints
// (:200-201), i.e. not differentiated. Here the transpose Jacobian-vector
// product of one step is evaluated matrix-free, one tile per work item:
//
//   forward:  k1 = u + dt L(u)
//             k2 = 3/4 u + 1/4 (k1 + dt L(k1))
//             u+ = 1/3 u + 2/3 (k2 + dt L(k2))          (timestepping.py:318-320)
//   reverse:  k2b = 2/3 (p + dt J(k2)^T p)
//             k1b = 1/4 (k2b + dt J(k1)^T k2b)
//             ub  = 1/3 p + 3/4 k2b + k1b + dt J(u)^T k1b
//
// J(v)^T w of L(v) = -(F_{i+1/2} - F_{i-1/2})/dx is assembled from the
// derivatives of the Rusanov flux (scalar.py:248, a = max(|f'(v_i)|,
// |f'(v_{i+1})|) from cell values, scalar.py:243-246) and of the WENO-JS5
// reconstruction (weno.py:114-157,247-256), differentiated by hand in the
// product form of device.cuh. Non-differentiable points follow the JAX/torch
// conventions: d|x|/dx = 0 at 0, and max() splits the cotangent evenly at
// ties. The states k1, k2 are recomputed from u in shared memory (halo 18).
//
// Periodic boundaries are circular indexing, and cotangents live on interior
// cells only (the reference's ghost rows carry zero cotangent when J only
// involves interior cells, see pyshocks_gb300/adjoint.py).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "adjoint_math.cuh"

namespace shk {

constexpr int kAdjTile = 512;
template <class T> __host__ __device__ constexpr int adj_uhalo() { return 20; }  // 18 needed
template <class T> __host__ __device__ constexpr int adj_phalo() { return sizeof(T) == 8 ? 10 : 12; }  // 9 needed
constexpr int kAdjArrays = 24;

template <class T>
struct AdjSmem {
    Win<T> U, K1, K2, PB, CB, Z, ACC;
    Win<T> H, D, Q, UL, UR;
    Win<T> GL, GR, GA;
    Win<T> T0, T1, T2, T3, T4;
    Win<T> CLu, CRu, CL1, CR1;  // face values of u and k1 from the forward recompute
    int W;  // window length (cells) of every array

    __host__ static size_t host_bytes(int W) { return size_t(kAdjArrays) * W * sizeof(T); }
    __device__ void carve(unsigned char* base, int W) {
        T* p = reinterpret_cast<T*>(base);
        Win<T>* slots[kAdjArrays] = {&U, &K1, &K2, &PB, &CB, &Z, &ACC, &H, &D, &Q,
                                     &UL, &UR, &GL, &GR, &GA, &T0, &T1, &T2, &T3, &T4,
                                     &CLu, &CRu, &CL1, &CR1};
        for (int i = 0; i < kAdjArrays; ++i) *slots[i] = make_win(p + size_t(i) * W, W);
        this->W = W;
    }
    // forward-stage view (face_fluxes writes the face fluxes into D and the
    // face values into ul, ur: UL, UR unless given)
    __device__ Smem<T> fwd(Win<T> state_out, Win<T> ul = Win<T>(), Win<T> ur = Win<T>()) const {
        Smem<T> s;
        s.U = U; s.S = state_out; s.H = H; s.D = D; s.Q = Q;
        s.UL = ul ? ul : UL; s.UR = ur ? ur : UR;
        // the learned phase's scratch: H and D (contiguous in both layouts)
        const int hd = 2 * W * int(sizeof(T) / sizeof(float));
        s.scr = learned_scratch(make_win(reinterpret_cast<float*>(win_raw(H)), hd), hd);
        s.W = W;
        return s;
    }
};

// z_i = dt (J_L(v)^T w)_i for i in [lo, hi); v valid on [lo-6, hi+6), w on
// [lo-3, hi+3). Rusanov flux, WENO-JS5 or learned reconstruction.
// cul, cur (WENO-JS5): the face values of v on [lo-3, hi+3) as the forward's
// face pass forms them (stored by the replay, or kept by the recompute)
template <class T, int EQ, int REC, class PV, class PW, class PZ, class PC = Win<const T>>
__device__ void vjp_stage(PV v, PW w, PZ z, int lo, int hi, const AdjSmem<T>& a,
                          const OpParams<T>& p, T dtdx, PC cul = PC(), PC cur = PC()) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if constexpr (REC == SHK_REC_LEARNED) {
        static_assert(sizeof(T) == 4, "the learned VJP runs on float stage states");
        // One pass per cell: the network forward (recomputed with the
        // inference's own mma sequence) gives the cell's face values, from
        // which the flux VJP seeds of its two faces follow, then the network
        // backward. Face j+1/2 (L = ul_{j+1}, R = ur_j) seeds cell j with
        //   gR_j = fb_j (f'(R)/2 + a_j), and cell j+1 with gL = fb_j (f'(L)/2 - a_j),
        // fb_j = dt/dx (w_{j+1} - w_j), a_j = nu/2 max(|f'(v_j)|, |f'(v_{j+1})|).
        // The face values are kept for the wave-speed terms below.
        const MlpShared& ms = mlp_shared();
        const MlpBackShared& bk = mlp_back_shared();
        // warp scratch: GL, GR, GA (3W floats, unused by this branch)
        float* scr = win_span(learned_scratch(a.GL, 3 * a.W), (tid >> 5) * kWarpScratchVjp,
                              kWarpScratchVjp);
        const int lane = tid & 31, g = lane >> 2, tq = lane & 3;
        const int myrow = 16 * (tq >> 1) + 8 * (tq & 1) + g;
        const int c0 = lo - 2, ncell = hi + 2 - c0;
        for (int qb = tid >> 5; qb * 32 < ncell; qb += nt >> 5) {
            const int r = qb * 32 + myrow;
            const int c = c0 + min(r, ncell - 1);
            // the stencil relative to v_c as the forward forms it (learned_phase)
            const float vm = v[c - 1], vc = v[c], vp = v[c + 1];
            const float sc[5] = {v[c - 2] - vc, vm - vc, 0.0f, vp - vc, v[c + 2] - vc};
            const float wm = w[c - 1], wc = w[c], wp = w[c + 1];
            float ul = 0.0f, ur = 0.0f;
            auto seed = [&](float cr, float cl, float& gR, float& gL) {
                ur = vc + cr;
                ul = vc + cl;
                const float wsc = wave_speed<EQ>(vc, p.c);
                const float hp = p.hnu * absmax(wsc, wave_speed<EQ>(vp, p.c));
                const float hm = p.hnu * absmax(wave_speed<EQ>(vm, p.c), wsc);
                gR = ((wp - wc) * dtdx) * fmaf(0.5f, flux_prime<EQ>(ur, p.c), hp);
                gL = ((wc - wm) * dtdx) * fmaf(0.5f, flux_prime<EQ>(ul, p.c), -hm);
            };
            float dd[5];
            learned_cell_vjp32(ms, bk, sc, seed, p.lp, scr, dd);
            if (r < ncell) {
                a.T0[c] = dd[0]; a.T1[c] = dd[1]; a.T2[c] = dd[2]; a.T3[c] = dd[3]; a.T4[c] = dd[4];
                a.UL[c] = ul;
                a.UR[c] = ur;
            }
        }
        __syncthreads();
        for (int i = lo + tid; i < hi; i += nt) {
            T acc = (a.T0[i + 2] + a.T1[i + 1]) + a.T2[i] + (a.T3[i - 1] + a.T4[i - 2]);
            // wave-speed terms: face i-1/2 (cells i-1, i) and face i+1/2 (cells i, i+1)
            const T gam = -(((w[i] - w[i - 1]) * dtdx) * p.hnu) * (a.UL[i] - a.UR[i - 1]);
            const T gap = -(((w[i + 1] - w[i]) * dtdx) * p.hnu) * (a.UL[i + 1] - a.UR[i]);
            acc = fma(gam, damax_dx<EQ>(v[i], v[i - 1], p.c), acc);
            acc = fma(gap, damax_dx<EQ>(v[i], v[i + 1], p.c), acc);
            z[i] = acc;
        }
        __syncthreads();
        return;
    }
    for (int c = lo - 5 + tid; c < hi + 4; c += nt) a.H[c] = T(0.5) * (v[c + 1] - v[c]);
    __syncthreads();
    for (int c = lo - 4 + tid; c < hi + 4; c += nt) {
        const T d = a.H[c] - a.H[c - 1];
        a.D[c] = d;
        a.Q[c] = (T(13.0 / 3.0) * d) * d;
    }
    __syncthreads();
    const PC UL = cul;
    const PC UR = cur;
    // face j+1/2: F = 1/2 (f(L) + f(R)) - nu/2 a (L - R), L = ul_{j+1}, R = ur_j
    for (int j = lo - 3 + tid; j < hi + 2; j += nt) {
        const T fb = (w[j + 1] - w[j]) * dtdx;
        const T L = UL[j + 1], R = UR[j];
        const T ha = p.hnu * absmax(wave_speed<EQ>(v[j], p.c), wave_speed<EQ>(v[j + 1], p.c));
        a.GL[j] = fb * fma(T(0.5), flux_prime<EQ>(L, p.c), -ha);
        a.GR[j] = fb * fma(T(0.5), flux_prime<EQ>(R, p.c), ha);
        a.GA[j] = -(fb * p.hnu) * (L - R);
    }
    __syncthreads();
    for (int c = lo - 2 + tid; c < hi + 2; c += nt) {
        T t0, t1, t2, t3, t4;
        weno53_cell_vjp<T>(a.H[c - 2], a.H[c - 1], a.H[c], a.H[c + 1], a.D[c - 1], a.D[c],
                           a.D[c + 1], a.Q[c - 1], a.Q[c], a.Q[c + 1], p.eps, a.GR[c],
                           a.GL[c - 1], t0, t1, t2, t3, t4);
        a.T0[c] = t0; a.T1[c] = t1; a.T2[c] = t2; a.T3[c] = t3; a.T4[c] = t4;
    }
    __syncthreads();
    for (int i = lo + tid; i < hi; i += nt) {
        T acc = (a.T0[i + 2] + a.T1[i + 1]) + a.T2[i] + (a.T3[i - 1] + a.T4[i - 2]);
        // wave-speed terms: face i-1/2 (cells i-1, i) and face i+1/2 (cells i, i+1)
        acc = fma(a.GA[i - 1], damax_dx<EQ>(v[i], v[i - 1], p.c), acc);
        acc = fma(a.GA[i], damax_dx<EQ>(v[i], v[i + 1], p.c), acc);
        z[i] = acc;
    }
    __syncthreads();
}

// Stage storage of one replayed step: k1, k2 (learned or float steps, in
// float), plus the face values of u and k1 (double WENO-JS5 steps, in double),
// each an array of the plan's `total` cells.
template <class T, int REC>
__host__ __device__ constexpr int kStageArrays() {
    return (sizeof(T) == 8 && REC != SHK_REC_LEARNED) ? 8 : 2;
}
template <class T, int REC>
__device__ __forceinline__ StageOut<stage_t<T, REC>> stage_out(void* base, int64_t total,
                                                               int64_t at) {
    using S = stage_t<T, REC>;
    StageOut<S> so;
    if (!base) return so;
    const Win<S> b = make_win(static_cast<S*>(base), kStageArrays<T, REC>() * total) + at;
    so.k1 = b;
    so.k2 = b + total;
    if constexpr (kStageArrays<T, REC>() == 8) {
        so.ulu = b + 2 * total;
        so.uru = b + 3 * total;
        so.ul1 = b + 4 * total;
        so.ur1 = b + 5 * total;
        so.ul2 = b + 6 * total;
        so.ur2 = b + 7 * total;
    }
    return so;
}

template <class S>
__device__ __forceinline__ StageOut<const S> as_const(const StageOut<S>& so) {
    StageOut<const S> c;
    c.k1 = so.k1; c.k2 = so.k2; c.ulu = so.ulu; c.uru = so.uru; c.ul1 = so.ul1; c.ur1 = so.ur1;
    c.ul2 = so.ul2; c.ur2 = so.ur2;
    return c;
}

// window positions [lo, hi) of a stage array stored per instance cell
// (position i is cell g0 + i, periodically)
template <class PD, class PS>
__device__ __forceinline__ void load_stage(PD dst, PS src, int64_t n, int64_t g0,
                                           int lo, int hi) {
    const bool once = g0 + lo >= -n && g0 + hi <= 2 * n;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int64_t pos = g0 + i;
        dst[i] = src[once ? (pos < 0 ? pos + n : (pos >= n ? pos - n : pos)) : imod(pos, n)];
    }
}

// Adjoint step of the mixed-precision learned step (step_tile_mixed): the
// forward stages are recomputed exactly as that step computes them (float
// operator on float stage states, increments about u), the three reverse
// stages run in float on float copies of u and p, and the result
//   ub = p + 2/3 Z3 + 1/4 Z2 + Z1
// (Z_s the stage VJPs dt J^T(.) of the reverse sweep below) adds the float
// increment to the double p once. Of the double arrays only the loaded windows
// a.U and a.PB are read; af holds the float arrays (af.K1, af.K2 may overlay
// a.U, which is dead once af.U is written).
// st (optional): the instance's stored float stage states (replay with stage
// storage), which replace the recompute of k1 and k2 bit for bit.
template <int EQ>
__device__ void adjoint_tile_mixed(const AdjSmem<double>& a, const AdjSmem<float>& af, Win<double> gout,
                                   int te, double dtdx, const OpParams<double>& p,
                                   const BcView& bc = BcView(), int64_t g0 = 0, int64_t n = 0,
                                   const StageOut<const float>& st = StageOut<const float>()) {
    constexpr int HU = adj_uhalo<double>(), HP = adj_phalo<double>();
    constexpr int REC = SHK_REC_LEARNED;
    const int tid = threadIdx.x, nt = blockDim.x;
    const bool np = !bc.periodic();
    const OpParams<float> pf = float_params(p);
    const float dtf = static_cast<float>(dtdx);
    for (int i = tid; i < te + 2 * HU; i += nt) af.U[i] = static_cast<float>(a.U[i]);
    for (int i = HU - HP + tid; i < HU + te + HP; i += nt) af.PB[i] = static_cast<float>(a.PB[i]);
    __syncthreads();
    if (np) {
        apply_bc(af.U, g0, n, 0, te + 2 * HU, bc, 0);
        zero_outside(af.PB, g0, n, HU - HP, HU + te + HP);
    }
    // forward recompute: k1 on [HU-15, HU+te+15), k2 on [HU-12, HU+te+12), or
    // the stored stage states there
    if (st.k1) {
        load_stage(af.K1, st.k1, n, g0, HU - 15, HU + te + 15);
        load_stage(af.K2, st.k2, n, g0, HU - 12, HU + te + 12);
        __syncthreads();
        if (np) {
            apply_bc(af.K1, g0, n, HU - 15, HU + te + 15, bc, 1);
            apply_bc(af.K2, g0, n, HU - 12, HU + te + 12, bc, 2);
        }
    } else {
        {
            const int lo = HU - 15, hi = HU + te + 15;
            face_fluxes<float, EQ, REC, SHK_FLUX_RUSANOV>(af.U, lo, hi, af.fwd(af.K1), pf);
            for (int i = lo + tid; i < hi; i += nt) {
                const float d = dtf * (af.D[i - 1] - af.D[i]);
                af.T0[i] = d;
                af.K1[i] = af.U[i] + d;
            }
            __syncthreads();
            if (np) apply_bc(af.K1, g0, n, lo, hi, bc, 1);
        }
        {
            const int lo = HU - 12, hi = HU + te + 12;
            face_fluxes<float, EQ, REC, SHK_FLUX_RUSANOV>(af.K1, lo, hi, af.fwd(af.K2), pf);
            for (int i = lo + tid; i < hi; i += nt) {
                const float d = 0.25f * (af.T0[i] + dtf * (af.D[i - 1] - af.D[i]));
                af.K2[i] = af.U[i] + d;
            }
            __syncthreads();
            if (np) apply_bc(af.K2, g0, n, lo, hi, bc, 2);
        }
    }
    // reverse stage 3: k2b = 2/3 (p + Z3), Z3 = dt J(k2)^T p
    {
        const int lo = HU - 6, hi = HU + te + 6;
        vjp_stage<float, EQ, REC>(af.K2, af.PB, af.Z, lo, hi, af, pf, dtf);
        if (np) bc_transpose(af.Z, g0, n, lo, hi, bc);
        for (int i = lo + tid; i < hi; i += nt) af.CB[i] = (2.0f / 3.0f) * (af.PB[i] + af.Z[i]);
        for (int i = HU + tid; i < HU + te; i += nt) af.ACC[i] = (2.0f / 3.0f) * af.Z[i];
        __syncthreads();
    }
    // reverse stage 2: k1b = 1/4 (k2b + Z2), Z2 = dt J(k1)^T k2b
    {
        const int lo = HU - 3, hi = HU + te + 3;
        vjp_stage<float, EQ, REC>(af.K1, af.CB, af.Z, lo, hi, af, pf, dtf);
        if (np) bc_transpose(af.Z, g0, n, lo, hi, bc);
        for (int i = HU + tid; i < HU + te; i += nt) af.ACC[i] = fmaf(0.25f, af.Z[i], af.ACC[i]);
        for (int i = lo + tid; i < hi; i += nt) af.CB[i] = 0.25f * (af.CB[i] + af.Z[i]);
        __syncthreads();
    }
    // reverse stage 1: Z1 = dt J(u)^T k1b; ub = p + (2/3 Z3 + 1/4 Z2 + Z1)
    // (and on the ghosts of a boundary tile)
    {
        int lo = HU, hi = HU + te;
        if (np) {
            for (int i = tid; i < 3; i += nt) {  // k1b beyond its range: zero
                af.CB[HU - 6 + i] = 0.0f;
                af.CB[HU + te + 3 + i] = 0.0f;
            }
            __syncthreads();
            if (g0 + HU == 0) lo -= 3;
            if (g0 + HU + te == n) hi += 3;
        }
        vjp_stage<float, EQ, REC>(af.U, af.CB, af.Z, lo, hi, af, pf, dtf);
        if (np) bc_transpose(af.Z, g0, n, lo, hi, bc);
        for (int i = HU + tid; i < HU + te; i += nt)
            gout[i - HU] = a.PB[i] + static_cast<double>(af.ACC[i] + af.Z[i]);
    }
}

// one adjoint step of a tile: p_out[s, s+te) from u_m (window, halo 20) and
// p_next (window, halo 10/12). gout points at p_out + s.
// With a Dirichlet / Neumann boundary (bc; g0 = s - HU the global cell of
// window position 0, n the instance's cells) the forward recompute applies the
// boundary at each stage, the cotangent window is zeroed outside the instance,
// each reverse stage is followed by the boundary's transpose, and the first
// reverse stage of a boundary tile also covers the ghost cells (their
// cotangents reach the interior through the Neumann mirrors).
template <class T, int EQ, int REC>
__device__ void adjoint_tile(const AdjSmem<T>& a, Win<T> gout, int te, T dtdx, const OpParams<T>& p,
                             const BcView& bc = BcView(), int64_t g0 = 0, int64_t n = 0,
                             const StageOut<const stage_t<T, REC>>& st =
                                 StageOut<const stage_t<T, REC>>()) {
    if constexpr (sizeof(T) == 8 && REC == SHK_REC_LEARNED) {
        // full double layout: the float arrays fit from CB on (24 in 20 double ones)
        AdjSmem<float> af;
        af.carve(reinterpret_cast<unsigned char*>(win_raw(a.CB)), a.W);
        adjoint_tile_mixed<EQ>(a, af, gout, te, dtdx, p, bc, g0, n, st);
        return;
    }
    const bool np = !bc.periodic();
    // stored stage states (and, for WENO-JS5, face values) replace the forward
    // recompute bit for bit; the stored faces of a boundary instance lack its
    // ghost cells, so WENO-JS5 steps with a boundary recompute
    constexpr bool kStoreable = (sizeof(T) == 4 && REC == SHK_REC_LEARNED) ||
                                (sizeof(T) == 8 && REC == SHK_REC_WENOJS53);
    const bool stored = kStoreable && st.k1 && (REC == SHK_REC_LEARNED || !np);
    if (np) {
        constexpr int HU0 = adj_uhalo<T>(), HP0 = adj_phalo<T>();
        apply_bc(a.U, g0, n, 0, te + 2 * HU0, bc, 0);
        zero_outside(a.PB, g0, n, HU0 - HP0, HU0 + te + HP0);
    }
    constexpr int HU = adj_uhalo<T>();
    // the forward recompute's face values of u, k1 and k2 serve the reverse
    // stages (they cover [HU-16, HU+te+16), [HU-13, HU+te+13) and
    // [HU-9, HU+te+9); the stages read [HU-6, HU+te+6), k2's [HU-9, HU+te+9))
    constexpr bool kCache = REC == SHK_REC_WENOJS53;
    const int tid = threadIdx.x, nt = blockDim.x;
    const T fdt = dtdx * p.fscale;  // face fluxes are stored as F / fscale
    // forward recompute: k1 on [HU-15, HU+te+15), k2 on [HU-12, HU+te+12),
    // with the forward step's own formulas (increments about u for float)
    if constexpr (kStoreable) {
        if (stored) {
            load_stage(a.K1, st.k1, n, g0, HU - 15, HU + te + 15);
            load_stage(a.K2, st.k2, n, g0, HU - 12, HU + te + 12);
            if constexpr (kCache) {
                load_stage(a.CLu, st.ulu, n, g0, HU - 6, HU + te + 6);
                load_stage(a.CRu, st.uru, n, g0, HU - 6, HU + te + 6);
                load_stage(a.CL1, st.ul1, n, g0, HU - 6, HU + te + 6);
                load_stage(a.CR1, st.ur1, n, g0, HU - 6, HU + te + 6);
                // k2's face values in UL/UR (free: no reconstruction runs here)
                load_stage(a.UL, st.ul2, n, g0, HU - 9, HU + te + 9);
                load_stage(a.UR, st.ur2, n, g0, HU - 9, HU + te + 9);
            }
            __syncthreads();
            if (np) {
                apply_bc(a.K1, g0, n, HU - 15, HU + te + 15, bc, 1);
                apply_bc(a.K2, g0, n, HU - 12, HU + te + 12, bc, 2);
            }
        }
    }
    if (!stored) {
    {
        const int lo = HU - 15, hi = HU + te + 15;
        // WENO-JS5: the face values of u stay in CLu/CRu for reverse stage 1
        face_fluxes<T, EQ, REC, SHK_FLUX_RUSANOV>(a.U, lo, hi, kCache ? a.fwd(a.K1, a.CLu, a.CRu)
                                                                      : a.fwd(a.K1), p);
        for (int i = lo + tid; i < hi; i += nt) {
            if constexpr (sizeof(T) == 4) {
                const T d = fdt * (a.D[i - 1] - a.D[i]);
                a.T0[i] = d;
                a.K1[i] = a.U[i] + d;
            } else {
                a.K1[i] = fma(fdt, a.D[i - 1] - a.D[i], a.U[i]);
            }
        }
        __syncthreads();
        if (np) apply_bc(a.K1, g0, n, lo, hi, bc, 1);
    }
    {
        const int lo = HU - 12, hi = HU + te + 12;
        // and those of k1 in CL1/CR1 for reverse stage 2
        face_fluxes<T, EQ, REC, SHK_FLUX_RUSANOV>(a.K1, lo, hi, kCache ? a.fwd(a.K2, a.CL1, a.CR1)
                                                                       : a.fwd(a.K2), p);
        for (int i = lo + tid; i < hi; i += nt) {
            if constexpr (sizeof(T) == 4) {
                a.K2[i] = a.U[i] + T(0.25) * (a.T0[i] + fdt * (a.D[i - 1] - a.D[i]));
            } else {
                const T k = fma(fdt, a.D[i - 1] - a.D[i], a.K1[i]);
                a.K2[i] = fma(T(1.0 / 4.0), k, T(3.0 / 4.0) * a.U[i]);
            }
        }
        __syncthreads();
        if (np) apply_bc(a.K2, g0, n, lo, hi, bc, 2);
    }
    if constexpr (kCache) {
        // the face values of k2 on [HU-9, HU+te+9) as the forward's face pass
        // forms them (as the stored ones; the fluxes it also leaves in D are
        // not used)
        face_fluxes<T, EQ, REC, SHK_FLUX_RUSANOV>(a.K2, HU - 8, HU + te + 8, a.fwd(a.K2, a.UL, a.UR), p);
    }
    }
    // reverse stage 3: k2b = 2/3 (p + dt J(k2)^T p) on [HU-6, HU+te+6)
    {
        const int lo = HU - 6, hi = HU + te + 6;
        vjp_stage<T, EQ, REC>(a.K2, a.PB, a.Z, lo, hi, a, p, dtdx, kCache ? a.UL : Win<T>(),
                              kCache ? a.UR : Win<T>());
        if (np) bc_transpose(a.Z, g0, n, lo, hi, bc);
        for (int i = lo + tid; i < hi; i += nt) a.CB[i] = T(2.0 / 3.0) * (a.PB[i] + a.Z[i]);
        __syncthreads();
        for (int i = HU + tid; i < HU + te; i += nt)
            a.ACC[i] = fma(T(3.0 / 4.0), a.CB[i], T(1.0 / 3.0) * a.PB[i]);
        __syncthreads();
    }
    // reverse stage 2: k1b = 1/4 (k2b + dt J(k1)^T k2b) on [HU-3, HU+te+3)
    {
        const int lo = HU - 3, hi = HU + te + 3;
        vjp_stage<T, EQ, REC>(a.K1, a.CB, a.Z, lo, hi, a, p, dtdx, kCache ? a.CL1 : Win<T>(),
                              kCache ? a.CR1 : Win<T>());
        if (np) bc_transpose(a.Z, g0, n, lo, hi, bc);
        for (int i = lo + tid; i < hi; i += nt) a.CB[i] = T(1.0 / 4.0) * (a.CB[i] + a.Z[i]);
        __syncthreads();
    }
    // reverse stage 1: ub = 1/3 p + 3/4 k2b + k1b + dt J(u)^T k1b on the tile
    // (and on the ghosts of a boundary tile)
    {
        int lo = HU, hi = HU + te;
        if (np) {
            for (int i = tid; i < 3; i += nt) {  // k1b beyond its range: zero
                a.CB[HU - 6 + i] = T(0);
                a.CB[HU + te + 3 + i] = T(0);
            }
            __syncthreads();
            if (g0 + HU == 0) lo -= 3;
            if (g0 + HU + te == n) hi += 3;
        }
        vjp_stage<T, EQ, REC>(a.U, a.CB, a.Z, lo, hi, a, p, dtdx, kCache ? a.CLu : Win<T>(),
                              kCache ? a.CRu : Win<T>());
        if (np) bc_transpose(a.Z, g0, n, lo, hi, bc);
        for (int i = HU + tid; i < HU + te; i += nt) gout[i - HU] = a.ACC[i] + (a.CB[i] + a.Z[i]);
    }
}

// compact layout of the mixed-precision learned adjoint (22 float arrays of W):
// a.U (double, slots 0-1, dead after the float copy, then af.K1/af.K2),
// a.PB (double, slots 2-3), af.U, af.PB, then the other 16 float arrays
constexpr int kMixedAdjSlots = 22;
__device__ inline void carve_mixed(unsigned char* base, int W, AdjSmem<double>& a, AdjSmem<float>& af) {
    float* f = reinterpret_cast<float*>(base);
    a.U = win_cast<double>(make_win(f, 2 * W));
    a.PB = win_cast<double>(make_win(f + 2 * W, 2 * W));
    a.K1 = a.K2 = a.CB = a.Z = a.ACC = a.H = a.D = a.Q = a.UL = a.UR = Win<double>();
    a.GL = a.GR = a.GA = a.T0 = a.T1 = a.T2 = a.T3 = a.T4 = Win<double>();
    a.W = W;
    af.K1 = make_win(f, W);
    af.K2 = make_win(f + W, W);
    af.U = make_win(f + 4 * W, W);
    af.PB = make_win(f + 5 * W, W);
    Win<float>* rest[] = {&af.CB, &af.Z, &af.ACC, &af.H, &af.D, &af.Q, &af.UL, &af.UR,
                          &af.GL, &af.GR, &af.GA, &af.T0, &af.T1, &af.T2, &af.T3, &af.T4};
    for (int i = 0; i < 16; ++i) *rest[i] = make_win(f + (6 + i) * W, W);
    af.W = W;
}

template <class T>
__device__ __forceinline__ bool adjoint_load(const AdjSmem<T>& a, const T* um, const T* pn,
                                             int64_t n, int64_t s0, int te, uint64_t* bar,
                                             uint32_t& phase) {
    constexpr int HU = adj_uhalo<T>(), HP = adj_phalo<T>();
    if (!load_window<T>(a.U, um, n, s0 - HU, te + 2 * HU, bar, phase)) return false;
    return load_window<T>(a.PB + (HU - HP), pn, n, s0 - HP, te + 2 * HP, bar, phase);
}

template <class T, int EQ, int REC>
__global__ void __launch_bounds__(kThreads, REC == SHK_REC_LEARNED ? 2 : 1) batched_adjoint_kernel(PlanDev P, const T* __restrict__ um,
                                                                   const T* __restrict__ pnext,
                                                                   T* __restrict__ pout,
                                                                   const double* __restrict__ dt_row,
                                                                   OpParams<T> p,
                                                                   const void* stages,
                                                                   int64_t total, int64_t step) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr bool kMixed = sizeof(T) == 8 && REC == SHK_REC_LEARNED;
    AdjSmem<T> a;
    AdjSmem<float> af;
    if constexpr (kMixed) carve_mixed(smem_raw, P.tile + 2 * adj_uhalo<T>(), a, af);
    else a.carve(smem_raw, P.tile + 2 * adj_uhalo<T>());
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    learned_stage<REC, true>(p.lp);
    uint32_t phase = 0;
    const Win<const T> gpnext = make_win(pnext, total);
    const Win<T> gpout = make_win(pout, total);
    __shared__ int s_item;
    for (int item = next_item(P, 2, &s_item); item >= 0; item = next_item(P, 2, &s_item)) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        const double dt = dt_row[b];
        if (dt == 0.0) {  // no step was taken: identity
            for (int i = threadIdx.x; i < te; i += blockDim.x) gpout[off + s0 + i] = gpnext[off + s0 + i];
            __syncthreads();
            continue;
        }
        if (!adjoint_load<T>(a, um + off, pnext + off, n, s0, te, &bar, phase)) {
            if (threadIdx.x == 0) atomicOr(P.status, ERR_TIMEOUT);
            break;
        }
        const T dtdx = static_cast<T>(dt * P.inv_dx[b]);
        const BcView bc = plan_bc(P, b, step);
        const int64_t g0 = s0 - adj_uhalo<T>();
        const StageOut<const stage_t<T, REC>> st =
            as_const(stage_out<T, REC>(const_cast<void*>(stages), total, off));
        if constexpr (kMixed) adjoint_tile_mixed<EQ>(a, af, gpout + (off + s0), te, dtdx, p, bc, g0, n, st);
        else adjoint_tile<T, EQ, REC>(a, gpout + (off + s0), te, dtdx, p, bc, g0, n, st);
        __syncthreads();
    }
    finish_items(P, 2);
}

// forward step with a recorded dt (no CFL, no time update): recompute of the
// states between checkpoints
// stages (optional): the step's stage storage, kStageArrays<T, REC> arrays of
// P's cells in the stage precision (stage_arrays), for a reverse step that
// skips its forward recompute; uout may then be null.
template <class T, int EQ, int REC>
__global__ void __launch_bounds__(kThreads, REC == SHK_REC_LEARNED ? 3 : 1) replay_step_kernel(PlanDev P, const T* __restrict__ uin,
                                                               T* __restrict__ uout,
                                                               const double* __restrict__ dt_row,
                                                               OpParams<T> p, void* stages,
                                                               int64_t total, int64_t step) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int HL = step_halo<T>();
    Smem<T> sm;
    carve_step<T, REC>(sm, smem_raw, P.tile + 2 * HL);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    learned_stage<REC>(p.lp);
    uint32_t phase = 0;
    const Win<const T> guin = make_win(uin, total);
    const Win<T> guout = make_win(uout, total);
    __shared__ int s_item;
    for (int item = next_item(P, 4, &s_item); item >= 0; item = next_item(P, 4, &s_item)) {
        const int b = P.item_inst[item];
        const int64_t off = P.offsets[b];
        const int64_t n = P.offsets[b + 1] - off;
        const int64_t s0 = int64_t(P.item_tile[item]) * P.tile;
        const int te = static_cast<int>(imin64(P.tile, n - s0));
        const double dt = dt_row[b];
        if (dt == 0.0) {  // no step: the reverse step is the identity, stage states unused
            if (uout)
                for (int i = threadIdx.x; i < te; i += blockDim.x) guout[off + s0 + i] = guin[off + s0 + i];
            __syncthreads();
            continue;
        }
        if (!load_window<T>(sm.U, uin + off, n, s0 - HL, te + 2 * HL, &bar, phase)) {
            if (threadIdx.x == 0) atomicOr(P.status, ERR_TIMEOUT);
            break;
        }
        const T dtdx = static_cast<T>(dt * P.inv_dx[b]);
        step_tile<T, EQ, REC, SHK_FLUX_RUSANOV>(sm, uout ? guout + (off + s0) : Win<T>(), te, dtdx, p,
                                                plan_bc(P, b, step), s0 - HL, n,
                                                stage_out<T, REC>(stages, total, off + s0));
        __syncthreads();
    }
    finish_items(P, 4);
}

// single instance on the reference's ghosted layout (drop-in adjoint_step)
template <class T, int EQ>
__global__ void __launch_bounds__(kThreads) single_vjp_kernel(const T* __restrict__ u, const T* __restrict__ pn,
                                                              T* __restrict__ pout, int64_t n, int g,
                                                              int tile, T dtdx, OpParams<T> p,
                                                              int32_t* err, shk_boundary bcp, double dx) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    AdjSmem<T> a;
    a.carve(smem_raw, tile + 2 * adj_uhalo<T>());
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;
    const int64_t s0 = int64_t(blockIdx.x) * tile;
    const int te = static_cast<int>(imin64(tile, n - s0));
    if (!adjoint_load<T>(a, u + g, pn + g, n, s0, te, &bar, phase)) {
        if (threadIdx.x == 0 && err) atomicOr(err, ERR_TIMEOUT);
        return;
    }
    BcView bc;
    bc.left = bcp.left;
    bc.right = bcp.right;
    bc.dir = &bcp.dirichlet[0][0][0];
    bc.dir_ss = 6;
    bc.neu = &bcp.neumann[0][0];
    bc.neu_ss = 2;
    bc.dx = dx;
    const Win<T> gpout = make_win(pout, n + 2 * g);
    adjoint_tile<T, EQ, SHK_REC_WENOJS53>(a, gpout + (g + s0), te, dtdx, p, bc, s0 - adj_uhalo<T>(), n);
    // ghost cotangents are zero (interior-only adjoint)
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i < g; i += blockDim.x) {
            gpout[i] = T(0);
            gpout[g + n + i] = T(0);
        }
}

}  // namespace shk

// ===========================================================================
// host side
// ===========================================================================
using namespace shk;

namespace {

int acuda(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libshocks: CUDA error %s\n", cudaGetErrorString(e));
        return SHK_ECUDA;
    }
    return SHK_OK;
}
#define ADJ_CUDA(call)                          \
    do {                                        \
        int _st = acuda(call);                  \
        if (_st != SHK_OK) return _st;          \
    } while (0)

template <class T>
OpParams<T> adj_params(const shk_scheme* s) {
    OpParams<T> p;
    p.eps = static_cast<T>(s->eps);
    p.delta = static_cast<T>(s->delta);
    p.hnu = static_cast<T>(0.5 * s->nu);
    p.c = static_cast<T>(s->speed);
    p.hnu_amax = T(0);
    p.lp = LearnedParams{s->mlp, static_cast<float>(s->eps), s->tau, s->band, s->dev,
                         norm_floor(s->norm_eps)};
    p.fscale = (sizeof(T) == 8 && s->flux == SHK_FLUX_RUSANOV && s->rec == SHK_REC_WENOJS53 &&
                s->equation == SHK_EQ_BURGERS && s->nu == 1.0) ? T(0.25) : T(1);
    p.lim = s->limiter;
    p.lim_param = static_cast<T>(s->delta);
    p.atol = static_cast<T>(s->eps);
    p.dx = T(1);
    return p;
}

bool adjoint_supported(const shk_scheme* s) {
    return s && s->flux == SHK_FLUX_RUSANOV &&
           (s->rec == SHK_REC_WENOJS53 || (s->rec == SHK_REC_LEARNED && s->mlp)) &&
           s->equation >= 0 && s->equation <= SHK_EQ_LWR;
}

template <class T, int REC, class F>
int by_equation_rec(int eq, F&& f) {
    switch (eq) {
        case SHK_EQ_BURGERS: return f.template operator()<T, SHK_EQ_BURGERS, REC>();
        case SHK_EQ_ADVECTION: return f.template operator()<T, SHK_EQ_ADVECTION, REC>();
        case SHK_EQ_LWR: return f.template operator()<T, SHK_EQ_LWR, REC>();
    }
    return SHK_EINVAL;
}

// WENO-JS53 for both precisions, the learned reconstruction for float32 states
template <class T, class F>
int by_scheme(const shk_scheme& sch, F&& f) {
    if (sch.rec == SHK_REC_LEARNED) return by_equation_rec<T, SHK_REC_LEARNED>(sch.equation, f);
    return by_equation_rec<T, SHK_REC_WENOJS53>(sch.equation, f);
}

template <class T, class F>
int by_equation(int eq, F&& f) {
    return by_equation_rec<T, SHK_REC_WENOJS53>(eq, f);
}

template <class TS>
struct AdjLaunch {
    PlanDev D; const void* um; const void* pn; void* po; const double* dt_row; OpParams<TS> p;
    size_t smem; int grid; cudaStream_t st; const void* stages = nullptr; int64_t total = 0;
    int64_t step = 0;  // index of the forward step (its boundary data)
    template <class T, int EQ, int REC> int operator()() {
        auto k = batched_adjoint_kernel<T, EQ, REC>;
        ADJ_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kThreads, smem, st>>>(D, static_cast<const T*>(um), static_cast<const T*>(pn),
                                         static_cast<T*>(po), dt_row, p, stages, total, step);
        return acuda(cudaGetLastError());
    }
};

template <class TS>
struct ReplayLaunch {
    PlanDev D; const void* uin; void* uout; const double* dt_row; OpParams<TS> p;
    size_t smem; int grid; cudaStream_t st; void* stages = nullptr; int64_t total = 0;
    int64_t step = 0;  // index of the replayed step (its boundary data)
    template <class T, int EQ, int REC> int operator()() {
        auto k = replay_step_kernel<T, EQ, REC>;
        ADJ_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, kThreads, smem, st>>>(D, static_cast<const T*>(uin), static_cast<T*>(uout), dt_row, p,
                                         stages, total, step);
        return acuda(cudaGetLastError());
    }
};

struct SingleVjpLaunch {
    const double* u; const double* pn; double* po; int64_t n; int g; int tile; double dtdx;
    OpParams<double> p; size_t smem; int blocks; cudaStream_t st; shk_boundary bc; double dx;
    template <class T, int EQ, int REC> int operator()() {
        auto k = single_vjp_kernel<T, EQ>;
        ADJ_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<blocks, kThreads, smem, st>>>(u, pn, po, n, g, tile, dtdx, p, nullptr, bc, dx);
        return acuda(cudaGetLastError());
    }
};

}  // namespace

extern "C" {

int shk_ssprk33_vjp_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                           const double* p_next, double* p_out, int64_t n, int32_t nghosts,
                           double dx, double dt, void* stream) {
    if (!adjoint_supported(scheme) || scheme->rec != SHK_REC_WENOJS53 || !u || !p_next || !p_out || n < 3 || nghosts < 3 ||
        !(dx > 0) || !(dt >= 0))
        return SHK_EINVAL;
    shk_boundary b;
    std::memset(&b, 0, sizeof(b));
    if (bc) b = *bc;
    if (b.left < SHK_BC_PERIODIC || b.left > SHK_BC_NEUMANN || b.right < SHK_BC_PERIODIC ||
        b.right > SHK_BC_NEUMANN || ((b.left == SHK_BC_PERIODIC) != (b.right == SHK_BC_PERIODIC)))
        return SHK_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int tile = kAdjTile;
    const int W = tile + 2 * adj_uhalo<double>();
    const size_t smem = AdjSmem<double>::host_bytes(W);
    const int blocks = static_cast<int>((n + tile - 1) / tile);
    SingleVjpLaunch f{u, p_next, p_out, n, nghosts, tile, dt / dx, adj_params<double>(scheme),
                      smem, blocks, st, b, dx};
    return by_equation<double>(scheme->equation, f);
}

int shk_ssprk33_vjp_f64(const shk_scheme* scheme, const double* u, const double* p_next,
                        double* p_out, int64_t n, int32_t nghosts, double dx, double dt,
                        void* stream) {
    return shk_ssprk33_vjp_bc_f64(scheme, nullptr, u, p_next, p_out, n, nghosts, dx, dt, stream);
}

int shk_plan_forward_checkpointed(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps,
                                  void* ckpt, int32_t stride, void* stream) {
    PlanDev D;
    int dtype = 0, grid = 0;
    shk_scheme sch;
    int64_t total = 0;
    if (!plan || !u_a || !u_b || !ckpt || nsteps < 0 || stride <= 0) return SHK_EINVAL;
    int64_t hsteps = 0;
    int r = plan_view(plan, &D, &dtype, &grid, &sch, &total, &hsteps);
    if (r != SHK_OK) return r;
    // checkpoints and the dt history are indexed from the last reset
    if (!D.dt_hist || D.max_steps < nsteps || hsteps != 0) return SHK_EINVAL;
    const size_t bytes = size_t(total) * (dtype == SHK_F64 ? 8 : 4);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int k = 0; k < nsteps; ++k) {
        if (k % stride == 0) {
            // the state before step k is in u_a for even k, u_b for odd k
            const void* cur = (k % 2 == 0) ? u_a : u_b;
            ADJ_CUDA(cudaMemcpyAsync(static_cast<char*>(ckpt) + size_t(k / stride) * bytes, cur,
                                     bytes, cudaMemcpyDeviceToDevice, st));
        }
        r = shk_plan_step(plan, u_a, u_b, 1, stream);
        if (r != SHK_OK) return r;
    }
    return SHK_OK;
}

int shk_plan_adjoint(shk_plan* plan, const void* ckpt, int32_t stride, int32_t nsteps, void* seg,
                     void* p_a, void* p_b, void* stream) {
    return shk_plan_adjoint_staged(plan, ckpt, stride, nsteps, seg, nullptr, p_a, p_b, stream);
}

// bytes of stage storage per replayed step (0: the plan recomputes)
static int64_t stage_bytes(const PlanDev& D, int dtype, const shk_scheme& sch, int64_t total) {
    if (sch.rec == SHK_REC_LEARNED) return 2 * total * int64_t(sizeof(float));
    const bool periodic = D.bc_left == SHK_BC_PERIODIC && D.bc_right == SHK_BC_PERIODIC;
    if (dtype == SHK_F64 && sch.rec == SHK_REC_WENOJS53 && periodic)
        return 8 * total * int64_t(sizeof(double));
    return 0;
}

int shk_plan_adjoint_stage_bytes(shk_plan* plan, int64_t* nbytes) {
    PlanDev D;
    int dtype = 0, grid = 0;
    shk_scheme sch;
    int64_t total = 0;
    if (!plan || !nbytes) return SHK_EINVAL;
    int r = plan_view(plan, &D, &dtype, &grid, &sch, &total, nullptr);
    if (r != SHK_OK) return r;
    *nbytes = stage_bytes(D, dtype, sch, total);
    return SHK_OK;
}

int shk_plan_adjoint_staged(shk_plan* plan, const void* ckpt, int32_t stride, int32_t nsteps,
                            void* seg, void* stages, void* p_a, void* p_b, void* stream) {
    PlanDev D;
    int dtype = 0, grid = 0;
    shk_scheme sch;
    int64_t total = 0;
    if (!plan || !ckpt || !seg || !p_a || !p_b || p_a == p_b || nsteps < 0 || stride <= 0)
        return SHK_EINVAL;
    int r = plan_view(plan, &D, &dtype, &grid, &sch, &total, nullptr);
    if (r != SHK_OK) return r;
    if (!adjoint_supported(&sch)) return SHK_EUNSUPPORTED;
    const int64_t sbytes = stage_bytes(D, dtype, sch, total);
    if (stages && sbytes == 0) return SHK_EINVAL;  // this plan has no stage storage
    if (!D.dt_hist || D.max_steps < nsteps) return SHK_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t esz = dtype == SHK_F64 ? 8 : 4;
    const size_t bytes = size_t(total) * esz;
    const int W = D.tile + 2 * adj_uhalo<double>();
    const bool mixed = dtype == SHK_F64 && sch.rec == SHK_REC_LEARNED;
    const size_t asmem = mixed ? sizeof(float) * kMixedAdjSlots * size_t(W)
                               : (dtype == SHK_F64 ? AdjSmem<double>::host_bytes(W)
                                                   : AdjSmem<float>::host_bytes(W));
    {
        // the reverse step keeps ~24 windows of the tile in shared memory: plans
        // with longer tiles can step forward but not run the adjoint
        int dev0 = 0, optin = 0;
        cudaGetDevice(&dev0);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev0);
        if (asmem > static_cast<size_t>(optin)) return SHK_EUNSUPPORTED;
    }
    const size_t fsmem = dtype == SHK_F64 ? Smem<double>::step_bytes(D.tile + 2 * step_halo<double>(), sch.rec)
                                          : Smem<float>::step_bytes(D.tile + 2 * step_halo<float>(), sch.rec);
    // adjoint grid: resident CTAs for its larger shared-memory footprint
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = std::max(1, static_cast<int>((220 * 1024) / std::max<size_t>(asmem, 1)));
    const int agrid = std::max(1, std::min(D.nitems, per_sm * sms));
    auto seg_at = [&](int j) { return static_cast<char*>(seg) + size_t(j) * bytes; };
    // stage storage of segment step j
    auto stage_at = [&](int j) -> void* {
        return stages ? static_cast<char*>(stages) + size_t(j) * size_t(sbytes) : nullptr;
    };
    const int nseg = (nsteps + stride - 1) / stride;
    void* cur = p_a;
    void* nxt = p_b;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int base = sgi * stride;
        const int cnt = std::min(stride, nsteps - base);
        ADJ_CUDA(cudaMemcpyAsync(seg_at(0), static_cast<const char*>(ckpt) + size_t(sgi) * bytes,
                                 bytes, cudaMemcpyDeviceToDevice, st));
        // replay: the states u_1 .. u_{cnt-1} of the segment and, with stage
        // storage, the stage states of every step (the last step's without u_out)
        for (int j = 1; j < cnt + (stages ? 1 : 0); ++j) {
            const double* row = D.dt_hist + size_t(base + j - 1) * D.B;
            void* out = j < cnt ? seg_at(j) : nullptr;
            if (dtype == SHK_F64) {
                ReplayLaunch<double> f{D, seg_at(j - 1), out, row, adj_params<double>(&sch), fsmem, grid, st,
                                       stage_at(j - 1), total, base + j - 1};
                r = by_scheme<double>(sch, f);
            } else {
                ReplayLaunch<float> f{D, seg_at(j - 1), out, row, adj_params<float>(&sch), fsmem, grid, st,
                                      stage_at(j - 1), total, base + j - 1};
                r = by_scheme<float>(sch, f);
            }
            if (r != SHK_OK) return r;
        }
        for (int j = cnt - 1; j >= 0; --j) {
            const double* row = D.dt_hist + size_t(base + j) * D.B;
            if (dtype == SHK_F64) {
                AdjLaunch<double> f{D, seg_at(j), cur, nxt, row, adj_params<double>(&sch), asmem, agrid, st,
                                    stage_at(j), total, base + j};
                r = by_scheme<double>(sch, f);
            } else {
                AdjLaunch<float> f{D, seg_at(j), cur, nxt, row, adj_params<float>(&sch), asmem, agrid, st,
                                   stage_at(j), total, base + j};
                r = by_scheme<float>(sch, f);
            }
            if (r != SHK_OK) return r;
            std::swap(cur, nxt);
        }
    }
    return SHK_OK;
}

}  // extern "C"

#ifdef SHOCKS_BOUNDS_CHECK
// this translation unit's bounds log (read by shk_check_bounds in forward.cu)
extern "C" int shk_check_tu_adjoint(shk::BoundsLog* out, int32_t reset) {
    return acuda(shk::bounds_log_read(out, reset != 0));
}
#endif
