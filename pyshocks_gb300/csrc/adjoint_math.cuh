// Device helpers of the discrete adjoint shared by the tiled reverse step
// (adjoint.cu) and the ghosted single-instance transpose (ghosted.cu):
// derivatives of the physical flux and of the wave speed, of the Rusanov speed
// max(|s(x)|, |s(y)|) with the JAX/torch tie convention (ties split evenly,
// d|s|/ds = 0 at 0), and the hand-derived backward of the WENO-JS5
// reconstruction of one cell (both faces) in half differences.
#pragma once

#include "stencil.cuh"

namespace shk {

// f'(u) of the physical flux and s'(u) of the wave speed
template <int EQ, class T>
__device__ __forceinline__ T flux_prime(T u, T c) {
    if constexpr (EQ == SHK_EQ_BURGERS) return u;
    else if constexpr (EQ == SHK_EQ_ADVECTION) return c;
    else return fma(T(-2), u, T(1));
}
template <int EQ, class T>
__device__ __forceinline__ T speed_prime() {
    if constexpr (EQ == SHK_EQ_BURGERS) return T(1);
    else if constexpr (EQ == SHK_EQ_ADVECTION) return T(0);
    else return T(-2);
}
template <class T>
__device__ __forceinline__ T sgn(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }

// d max(|s(x)|, |s(y)|) / dx   (ties split evenly, d|s|/ds = 0 at 0)
template <int EQ, class T>
__device__ __forceinline__ T damax_dx(T x, T y, T c) {
    const T sx = wave_speed<EQ>(x, c), sy = wave_speed<EQ>(y, c);
    const auto bx = abs_bits(sx), by = abs_bits(sy);
    const T chi = bx > by ? T(1) : (bx == by ? T(0.5) : T(0));
    return chi * sgn(sx) * speed_prime<EQ, T>();
}

// Backward of the WENO-JS5 reconstruction of cell c in half differences
// (device.cuh): given the cotangents of ur (urb) and ul (ulb), the
// contributions t_o to the cotangents of v_{c+o}, o = -2..2. The face values
// themselves come from the forward's face pass; the backward recomputes the
// weights in the half-difference form.
template <class T>
__device__ __forceinline__ void weno53_cell_vjp(T Hm2, T Hm1, T H0, T Hp1, T Dm1, T D0, T Dp1,
                                                T Qm1, T Q0, T Qp1, T eps, T urb, T ulb, T& t0,
                                                T& t1, T& t2, T& t3, T& t4) {
    // forward quantities (weights in product form)
    const T h0 = fma(T(2), Hm1, Dm1);
    const T h1 = H0 + Hm1;
    const T h2 = fma(T(-2), H0, Dp1);
    const T e0 = eps + fma(h0, h0, Qm1);
    const T e1 = eps + fma(h1, h1, Q0);
    const T e2 = eps + fma(h2, h2, Qp1);
    const T s0 = e0 * e0, s1 = e1 * e1, s2 = e2 * e2;
    T P0, P1, P2;
    if constexpr (sizeof(T) == 8) {
        P0 = s1 * s2; P1 = s0 * s2; P2 = s0 * s1;
    } else {  // the forward's approximate reciprocals
        P0 = rcp_approx_f32(s0); P1 = rcp_approx_f32(s1); P2 = rcp_approx_f32(s2);
    }
    const T cr0 = fma(T(10), Hm1, T(-4) * Hm2);
    const T cr1 = fma(T(24), H0, T(12) * Hm1);
    const T cr2 = fma(T(-6), Hp1, T(24) * H0);
    const T cl0 = fma(T(-10), H0, T(4) * Hp1);
    const T cl1 = fma(T(-24), Hm1, T(-12) * H0);
    const T cl2 = fma(T(-24), Hm1, T(6) * Hm2);
    const T nr = fma(P0, cr0, fma(P1, cr1, P2 * cr2));
    const T nl = fma(P2, cl0, fma(P1, cl1, P0 * cl2));
    const T m = T(36) * P1;
    const T dr = fma(T(6), P0, fma(T(18), P2, m));
    const T dl = fma(T(6), P2, fma(T(18), P0, m));
    T gR, gL, dR, dL, ie0, ie1, ie2;
    if constexpr (sizeof(T) == 8) {
        const T r = rcp_nr(dr * dl);
        const T rl = dl * r, rr = dr * r;  // 1/dr, 1/dl
        gR = urb * rl;
        gL = ulb * rr;
        dR = nr * rl;  // ur - v
        dL = nl * rr;  // ul - v
        const T e01 = e0 * e1;
        const T q = rcp_nr(e01 * e2);
        ie0 = (e1 * e2) * q;
        ie1 = (e0 * e2) * q;
        ie2 = e01 * q;
    } else {
        const T ird = rcp_approx_f32(dr), ild = rcp_approx_f32(dl);
        gR = urb * ird;
        gL = ulb * ild;
        dR = nr * ird;
        dL = nl * ild;
        ie0 = rcp_approx_f32(e0);
        ie1 = rcp_approx_f32(e1);
        ie2 = rcp_approx_f32(e2);
    }
    // interpolation part (weights held fixed): d_k P_k / D folded with the
    // sub-stencil values 6 uhat_k
    const T g6 = T(6) * P1;
    const T rho0 = gR * P0, rho1 = gR * g6, rho2 = T(3) * gR * P2;
    const T lam0 = gL * P2, lam1 = gL * g6, lam2 = T(3) * gL * P0;
    // smoothness part: d ur / d beta_j = -2 P_j (cr_j - W_j (ur - v)) / (e_j D_R), W = (6, 36, 18);
    // the left side sees beta_j through its mirrored sub-stencil 2 - j. The
    // factor -2 is folded into the taps below (bb, bh, bd are -1/2 of the
    // cotangents of beta, h, D).
    const T x0 = fma(gR, fma(T(-6), dR, cr0), gL * fma(T(-18), dL, cl2));
    const T x1 = fma(gR, fma(T(-36), dR, cr1), gL * fma(T(-36), dL, cl1));
    const T x2 = fma(gR, fma(T(-18), dR, cr2), gL * fma(T(-6), dL, cl0));
    const T bb0 = (P0 * ie0) * x0;
    const T bb1 = (P1 * ie1) * x1;
    const T bb2 = (P2 * ie2) * x2;
    // beta_j = h_j^2 + 13/3 D_j^2 with h_j = B_j v / 2, D_j = A_j v / 2
    const T bh0 = bb0 * h0, bh1 = bb1 * h1, bh2 = bb2 * h2;
    const T bd0 = bb0 * (T(13.0 / 3.0) * Dm1);
    const T bd1 = bb1 * (T(13.0 / 3.0) * D0);
    const T bd2 = bb2 * (T(13.0 / 3.0) * Dp1);
    // taps: A_0 (1,-2,1,0,0) B_0 (1,-4,3,0,0) A_1 (0,1,-2,1,0) B_1 (0,-1,0,1,0)
    //       A_2 (0,0,1,-2,1) B_2 (0,0,3,-4,1); 6 uhat right (2,-7,11,0,0) (0,-1,5,2,0)
    //       (0,0,2,5,-1); left (0,0,11,-7,2) (0,2,5,-1,0) (-1,5,2,0,0)
    t0 = fma(T(-2), bh0 + bd0, fma(T(2), rho0, -lam2));
    t1 = fma(T(-7), rho0, -rho1) + fma(T(2), lam1, T(5) * lam2) +
         fma(T(8), bh0, fma(T(4), bd0, T(-2) * (bd1 - bh1)));
    t2 = fma(T(11), rho0 + lam0, fma(T(5), rho1 + lam1, T(2) * (rho2 + lam2))) +
         fma(T(-2), fma(T(3), bh0 + bh2, bd0 + bd2), T(4) * bd1);
    t3 = fma(T(2), rho1, T(5) * rho2) - fma(T(7), lam0, lam1) +
         fma(T(-2), bh1 + bd1, fma(T(8), bh2, T(4) * bd2));
    t4 = fma(T(-2), bh2 + bd2, fma(T(2), lam0, -rho2));
}

}  // namespace shk
