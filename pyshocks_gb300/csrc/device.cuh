// Device-side building blocks of the WENO / flux / SSPRK33 kernels (sm_103a).
//
// Arithmetic follows the reference's formulas (alexfikl/pyshocks):
//   smoothness  src/pyshocks/weno.py:114-140 with the JS53 coefficients :206-244
//   interpolants src/pyshocks/weno.py:143-157
//   weights      src/pyshocks/weno.py:247-256 (JS) and :284-296 (ES)
//   sides        src/pyshocks/reconstruction.py:351-377 (ul is the mirror of ur)
//   Rusanov      src/pyshocks/scalar.py:192-249
//   upwind       src/pyshocks/scalar.py:91-132
//   ES-WENO flux src/pyshocks/burgers/schemes.py:230-256
//   SSPRK33      src/pyshocks/timestepping.py:312-320
// reorganised to cut the FP64 instruction count (the FP64 pipe, not HBM,
// bounds this path on GB300):
//   * one set of smoothness indicators per cell serves both faces: the
//     mirrored left reconstruction sees beta_k of the right one as beta_{2-k};
//   * squares of second differences and half first differences are computed
//     once per cell and shared by the three sub-stencils of three cells;
//   * normalised weights d_k/s_k / sum_j d_j/s_j are evaluated in product form
//     d_k P_k / sum_j d_j P_j with P_k = prod_{j != k} s_j, so one reciprocal of
//     D_R * D_L serves both faces of a cell (f64 only; f32 divides per face to
//     stay clear of underflow);
//   * sub-stencil values are written as v_i + correction, so the reconstruction
//     is v_i + N/D.
// These are exact identities; results differ from the reference only by
// rounding (the oracle tests bound the difference: 1e-10 after hundreds of
// steps, measured ~4e-14).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "../../include/shocks.h"

namespace shk {

enum : int32_t {
    ERR_NONFINITE = 1,
    ERR_TIMEOUT = 2,
    ERR_BOUNDS = 4,
};

// bounded-wait iteration limit for mbarrier polls (each try_wait may suspend
// the thread for a short, hardware-defined time)
constexpr long long kWaitLimit = 1LL << 20;

// ---- window pointers ---------------------------------------------------------
// The shared-memory window arrays, the stage storage and the state arrays of
// the stencil kernels are addressed through Win<T>. In the library build a
// Win<T> is a plain T*, and the helpers below compile to pointer arithmetic.
// In the bounds-check build (-DSHOCKS_BOUNDS_CHECK, libshocks_check.so) a
// Win<T> carries the bounds of the array it points into: an index outside
// them records the first violation of the translation unit (block, thread,
// offset from the array start, array extent) in a device log and redirects
// the access to a sink word, so a faulty index is reported instead of
// touching memory it does not own. No trap, no assert.
#ifdef SHOCKS_BOUNDS_CHECK
struct BoundsLog {
    int32_t flag;
    int32_t block;
    int32_t thread;
    int32_t pad;
    int64_t offset;  // element offset of the bad access from the array start
    int64_t extent;  // elements of the array
};
static __device__ BoundsLog g_bounds_log;
static __device__ __align__(16) unsigned char g_bounds_sink[64];

static __device__ __noinline__ void bounds_fail(long long offset, long long extent) {
    if (atomicOr(&g_bounds_log.flag, 1) == 0) {
        g_bounds_log.block = static_cast<int32_t>(blockIdx.x);
        g_bounds_log.thread = static_cast<int32_t>(threadIdx.x);
        g_bounds_log.offset = offset;
        g_bounds_log.extent = extent;
    }
}

template <class T>
struct Win {
    T* p = nullptr;
    T* lo = nullptr;
    T* hi = nullptr;
    __host__ __device__ Win() {}
    __host__ __device__ Win(decltype(nullptr)) {}
    __host__ __device__ Win(T* p_, T* lo_, T* hi_) : p(p_), lo(lo_), hi(hi_) {}
    template <class U, class = typename std::enable_if<std::is_convertible<U*, T*>::value>::type>
    __host__ __device__ Win(const Win<U>& o) : p(o.p), lo(o.lo), hi(o.hi) {}
    __device__ T& operator[](long long i) const {
        T* q = p + i;
        if (q < lo || q >= hi) {
            bounds_fail(static_cast<long long>(q - lo), static_cast<long long>(hi - lo));
            return *reinterpret_cast<T*>(g_bounds_sink);
        }
        return *q;
    }
    __host__ __device__ Win operator+(long long k) const { return Win(p + k, lo, hi); }
    __host__ __device__ Win operator-(long long k) const { return Win(p - k, lo, hi); }
    __host__ __device__ explicit operator bool() const { return p != nullptr; }
};
// a window over n elements from p
template <class T>
__host__ __device__ __forceinline__ Win<T> make_win(T* p, long long n) { return Win<T>(p, p, p + n); }
// the same bytes seen as another element type
template <class U, class T>
__host__ __device__ __forceinline__ Win<U> win_cast(const Win<T>& w) {
    return Win<U>(reinterpret_cast<U*>(w.p), reinterpret_cast<U*>(w.lo), reinterpret_cast<U*>(w.hi));
}
// raw pointer to the cnt elements from w[i] once they are checked to lie in
// the array (the array start on a violation: in bounds, for instructions that
// need a real address such as ldmatrix or a bulk copy)
template <class T>
__device__ __forceinline__ T* win_span(const Win<T>& w, long long i, long long cnt) {
    T* q = w.p + i;
    if (q < w.lo || q + cnt > w.hi) {
        bounds_fail(static_cast<long long>(q - w.lo), static_cast<long long>(w.hi - w.lo));
        return w.lo;
    }
    return q;
}
// whether the cnt elements from w[i] lie in the array (logged if not)
template <class T>
__device__ __forceinline__ bool win_fits(const Win<T>& w, long long i, long long cnt) {
    const T* q = w.p + i;
    if (q < w.lo || q + cnt > w.hi) {
        bounds_fail(static_cast<long long>(q - w.lo), static_cast<long long>(w.hi - w.lo));
        return false;
    }
    return true;
}
template <class T>
__host__ __device__ __forceinline__ T* win_raw(const Win<T>& w) { return w.p; }
// index i of a length-n array (a gathered read): false and logged if outside
__device__ __forceinline__ bool chk_index(long long i, long long n) {
    if (i < 0 || i >= n) {
        bounds_fail(i, n);
        return false;
    }
    return true;
}
// host: copy (and optionally clear) this translation unit's log
static inline cudaError_t bounds_log_read(BoundsLog* out, bool reset) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_bounds_log, sizeof(BoundsLog));
    if (e == cudaSuccess && reset) {
        BoundsLog z = {};
        e = cudaMemcpyToSymbol(g_bounds_log, &z, sizeof(BoundsLog));
    }
    return e;
}
#else
template <class T>
using Win = T*;
template <class T>
__host__ __device__ __forceinline__ T* make_win(T* p, long long) { return p; }
template <class U, class T>
__host__ __device__ __forceinline__ U* win_cast(T* w) { return reinterpret_cast<U*>(w); }
template <class T>
__device__ __forceinline__ T* win_span(T* w, long long i, long long) { return w + i; }
template <class T>
__device__ __forceinline__ bool win_fits(T*, long long, long long) { return true; }
template <class T>
__host__ __device__ __forceinline__ T* win_raw(T* w) { return w; }
__device__ __forceinline__ bool chk_index(long long, long long) { return true; }
#endif
// element type of a pointer or window
template <class P>
using elem_t = typename std::remove_cv<typename std::remove_reference<decltype(std::declval<P>()[0])>::type>::type;

// ---- test hooks of the bounds-check build ----------------------------------
// libshocks_check.so can make the window loader's bounded wait run out: the
// loader then declares `extra` bytes more than its copies deliver (every copy
// lands, none stays in flight, the barrier never completes) and polls at most
// `limit` times per wait. The library build has neither.
#ifdef SHOCKS_BOUNDS_CHECK
static __device__ uint32_t g_test_extra_tx;
static __device__ long long g_test_wait_limit;
__device__ __forceinline__ uint32_t test_extra_tx() { return g_test_extra_tx; }
__device__ __forceinline__ long long wait_limit() {
    const long long l = g_test_wait_limit;
    return l > 0 ? l : kWaitLimit;
}
#else
__device__ __forceinline__ constexpr uint32_t test_extra_tx() { return 0u; }
__device__ __forceinline__ constexpr long long wait_limit() { return kWaitLimit; }
#endif

// ---- bit tricks for max-reductions on |x| (integer pipe, exact) ---------
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ unsigned int abs_bits(float x) {
    return __float_as_uint(x) & 0x7fffffffu;
}
__device__ __forceinline__ double from_bits(unsigned long long b) {
    return __longlong_as_double(static_cast<long long>(b));
}
__device__ __forceinline__ float from_bits(unsigned int b) { return __uint_as_float(b); }

template <class T> struct Bits;
template <> struct Bits<double> { using type = unsigned long long; };
template <> struct Bits<float> { using type = unsigned int; };

// 1/x to about 1 ulp in one instruction (rcp.approx.ftz.f32; subnormal inputs
// flush to zero) for float paths where a correctly rounded division buys nothing
__device__ __forceinline__ float rcp_approx_f32(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// max(|a|, |b|) without the FP pipe (NaN-free inputs)
template <class T>
__device__ __forceinline__ T absmax(T a, T b) {
    auto x = abs_bits(a), y = abs_bits(b);
    return from_bits(x > y ? x : y);
}

// ---- physical fluxes ------------------------------------------------------
// Burgers f = u^2/2 (src/pyshocks/burgers/schemes.py:37-39), f' = u
// linear advection f = c u, f' = c
// LWR traffic f = u (1 - u), f' = 1 - 2 u (examples/traffic-flow-model.py:18-24)
template <int EQ, class T>
__device__ __forceinline__ T phys_flux(T u, T c) {
    if constexpr (EQ == SHK_EQ_BURGERS) return T(0.5) * (u * u);
    else if constexpr (EQ == SHK_EQ_ADVECTION) return c * u;
    else return u * (T(1) - u);
}
// f(L) + f(R) with every product and the sum rounded separately, as the
// reference evaluates it: left to the compiler, one product could be fused
// into an FMA with the sum, and which one depends on the surrounding code
template <int EQ, class T>
__device__ __forceinline__ T phys_flux_sum(T L, T R, T c) {
    if constexpr (sizeof(T) == 8) {
        if constexpr (EQ == SHK_EQ_ADVECTION) return __dadd_rn(__dmul_rn(c, L), __dmul_rn(c, R));
        else return __dadd_rn(__dmul_rn(L, 1.0 - L), __dmul_rn(R, 1.0 - R));
    } else {
        if constexpr (EQ == SHK_EQ_ADVECTION) return __fadd_rn(__fmul_rn(c, L), __fmul_rn(c, R));
        else return __fadd_rn(__fmul_rn(L, 1.0f - L), __fmul_rn(R, 1.0f - R));
    }
}
template <int EQ, class T>
__device__ __forceinline__ T wave_speed(T u, T c) {
    if constexpr (EQ == SHK_EQ_BURGERS) return u;
    else if constexpr (EQ == SHK_EQ_ADVECTION) return c;
    else return fma(T(-2), u, T(1));
}

// Reciprocal for the FP64 pipe: the hardware approximation rcp.approx.ftz.f64
// refined by one step of the third-order (cubically convergent) reciprocal
// iteration y <- y (1 + e + e^2), e = 1 - x y: 3 DFMA instead of the full
// division sequence (two quadratic Newton-Raphson steps take 4). For normal,
// finite x it is within 1 ulp of the IEEE quotient 1/x, and equal to it for
// all but 5569 of 2^24 log-uniform samples in [1e-60, 1e60]. Subnormal inputs
// are flushed; inf gives NaN (callers stay in range).
__device__ __forceinline__ double rcp_nr(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// ---- WENO-JS 5/3 reconstruction of one cell -------------------------------
// In half differences (the form of the reverse step's weno53_cell_vjp): cell
// c, H_k = (v_{k+1}-v_k)/2 for k = c-2..c+1, D_k = H_k - H_{k-1} and
// Q_k = 13/12 (2 D_k)^2 for k = c-1..c+1;
// beta_0 = Q_{c-1} + (D_{c-1} + 2 H_{c-1})^2
// beta_1 = Q_c     + (H_c + H_{c-1})^2
// beta_2 = Q_{c+1} + (D_{c+1} - 2 H_c)^2
// which are 13/12 q1^2 + 1/4 q2^2 of src/pyshocks/weno.py:219-228; the
// weights alpha_k = d_k / (eps + beta_k)^2 (weno.py:254) in product form.
// The forward reconstruction on unscaled differences (fewer FP64
// instructions than half differences): d_k = v_{k+1} - v_k, E_k = d_k - d_{k-1}, G_k = 13/3 E_k^2 + 4 eps,
// and 4 (beta_j + eps) = G + h'^2 with h'_0 = E_{c-1} + 2 d_{c-1}, h'_1 = d_c + d_{c-1},
// h'_2 = E_{c+1} - 2 d_c. Every s_j and P_j is thus scaled by a common power
// of two, which cancels in the normalised weights. The
// corrections 6 (uhat_k - v), with the ideal weights (1, 6, 3)/10 folded in, use
// d_{c-2} = 3 d_{c-1} - h'_0 and d_{c+1} = h'_2 + 3 d_c:
//   cr0 = 2 h'_0 - d_{c-1}      cr1 = 6 d_{c-1} + 12 d_c     cr2 = 3 (d_c - h'_2)
//   cl0 = 2 h'_2 + d_c          cl1 = 6 E_c - cr1            cl2 = -3 (h'_0 + d_{c-1})
__device__ __forceinline__ void weno53_cell_d(double v, double dm1, double d0, double Em1,
                                              double E0, double Ep1, double Gm1, double G0,
                                              double Gp1, double& ul, double& ur) {
    // G_k = 13/3 E_k^2 + 4 eps (eps folded in when G is formed)
    const double h0 = fma(2.0, dm1, Em1);
    const double h1 = d0 + dm1;
    const double h2 = fma(-2.0, d0, Ep1);
    double s0 = fma(h0, h0, Gm1); s0 = s0 * s0;
    double s1 = fma(h1, h1, G0); s1 = s1 * s1;
    double s2 = fma(h2, h2, Gp1); s2 = s2 * s2;
    const double P0 = s1 * s2, P1 = s0 * s2, P2 = s0 * s1;
    const double cr0 = fma(2.0, h0, -dm1);
    const double cr1 = fma(12.0, d0, 6.0 * dm1);
    const double cr2 = 3.0 * (d0 - h2);
    const double cl0 = fma(2.0, h2, d0);
    const double cl1 = fma(6.0, E0, -cr1);
    const double cl2 = -3.0 * (h0 + dm1);
    const double nr = fma(P0, cr0, fma(P1, cr1, P2 * cr2));
    const double nl = fma(P2, cl0, fma(P1, cl1, P0 * cl2));
    const double m = 36.0 * P1;
    const double dr = fma(6.0, P0, fma(18.0, P2, m));
    const double dl = fma(6.0, P2, fma(18.0, P0, m));
    const double r = rcp_nr(dr * dl);
    ur = fma(nr * dl, r, v);
    ul = fma(nl * dr, r, v);
}

// Float variant of weno53_cell_d for the one-pass float reconstruction: the
// same unscaled differences (d_{c-1}, d_c, E_{c-1..c+1} and the terms
// G_j = 13/3 E_j^2 + 4 eps, which neighbouring cells share) and folded
// corrections, with the weights P_k = 1/s_k and the two normalisations as
// one-instruction approximate reciprocals (a product form could underflow in
// float).
__device__ __forceinline__ float weno53_g_f(float E, float eps4) {
    return fmaf((13.0f / 3.0f) * E, E, eps4);
}

__device__ __forceinline__ void weno53_cell_fg(float v, float dm1, float d0, float Em1, float E0,
                                               float Ep1, float Gm1, float G0, float Gp1,
                                               float& ul, float& ur) {
    const float h0 = fmaf(2.0f, dm1, Em1);
    const float h1 = d0 + dm1;
    const float h2 = fmaf(-2.0f, d0, Ep1);
    float s0 = fmaf(h0, h0, Gm1); s0 = s0 * s0;
    float s1 = fmaf(h1, h1, G0); s1 = s1 * s1;
    float s2 = fmaf(h2, h2, Gp1); s2 = s2 * s2;
    const float P0 = rcp_approx_f32(s0), P1 = rcp_approx_f32(s1), P2 = rcp_approx_f32(s2);
    const float cr0 = fmaf(2.0f, h0, -dm1);
    const float cr1 = fmaf(12.0f, d0, 6.0f * dm1);
    const float cr2 = 3.0f * (d0 - h2);
    const float cl0 = fmaf(2.0f, h2, d0);
    const float cl1 = fmaf(6.0f, E0, -cr1);
    const float cl2 = -3.0f * (h0 + dm1);
    const float nr = fmaf(P0, cr0, fmaf(P1, cr1, P2 * cr2));
    const float nl = fmaf(P2, cl0, fmaf(P1, cl1, P0 * cl2));
    const float m = 36.0f * P1;
    const float dr = fmaf(6.0f, P0, fmaf(18.0f, P2, m));
    const float dl = fmaf(6.0f, P2, fmaf(18.0f, P0, m));
    ur = fmaf(nr, rcp_approx_f32(dr), v);
    ul = fmaf(nl, rcp_approx_f32(dl), v);
}

// the same from the four differences d_{c-2} .. d_{c+1} of the cell's stencil
__device__ __forceinline__ void weno53_cell_f(float v, float dm2, float dm1, float d0, float dp1,
                                              float eps4, float& ul, float& ur) {
    const float Em1 = dm1 - dm2, E0 = d0 - dm1, Ep1 = dp1 - d0;
    weno53_cell_fg(v, dm1, d0, Em1, E0, Ep1, weno53_g_f(Em1, eps4), weno53_g_f(E0, eps4),
                   weno53_g_f(Ep1, eps4), ul, ur);
}

// 2|x| from the bit pattern of |x| (integer exponent increment, exact for
// normal numbers; zero and subnormals take the FP path)
__device__ __forceinline__ double twice_abs_bits(unsigned long long b) {
    return b >= (1ULL << 52) ? from_bits(b + (1ULL << 52)) : 2.0 * from_bits(b);
}

// ---- ES-WENO 3/2 reconstruction of one cell (weno.py:284-296) -----------------
// d = (1/3, 2/3); beta_0 = (v_c - v_{c-1})^2, beta_1 = (v_{c+1} - v_c)^2,
// tau = (v_{c+1} - 2 v_c + v_{c-1})^2; alpha_k = d_k (1 + tau / (eps + beta_k)).
// Returns ul, ur and omega_0 of the right side (used by the ES-WENO flux).
template <class T>
__device__ __forceinline__ void esweno32_cell(T vm1, T v, T vp1, T eps, T& ul, T& ur,
                                              T& w0) {
    const T dm = v - vm1, dp = vp1 - v;
    const T b0 = dm * dm, b1 = dp * dp;
    const T dd = dp - dm;
    const T tau = dd * dd;
    const T third = T(1) / T(3);
    const T a0 = third * (T(1) + tau / (eps + b0));
    const T a1 = (T(2) * third) * (T(1) + tau / (eps + b1));
    const T sr = a0 + a1;
    w0 = a0 / sr;
    const T w1 = a1 / sr;
    // uhat_0 = 3/2 v_c - 1/2 v_{c-1}, uhat_1 = 1/2 (v_{c+1} + v_c) (weno.py:196-198)
    ur = w0 * (T(1.5) * v - T(0.5) * vm1) + w1 * (T(0.5) * vp1 + T(0.5) * v);
    // mirror: beta_0^L = beta_1, beta_1^L = beta_0
    const T al0 = third * (T(1) + tau / (eps + b1));
    const T al1 = (T(2) * third) * (T(1) + tau / (eps + b0));
    const T sl = al0 + al1;
    ul = (al0 / sl) * (T(1.5) * v - T(0.5) * vp1) + (al1 / sl) * (T(0.5) * vm1 + T(0.5) * v);
}

// WENO-JS3 (weno.py:166-203, weights weno.py:247-256) of cell c: right face
// from v_{c-1..c+1} with beta = ((v_c - v_{c-1})^2, (v_{c+1} - v_c)^2), uhat =
// (v + dm/2, v + dp/2), d = (1/3, 2/3); left face on the mirrored stencil. The
// weights are in product form (alpha_k s_0^2 s_1^2 3): one division per face.
template <class T>
__device__ __forceinline__ void weno32_cell(T vm1, T v, T vp1, T eps, T& ul, T& ur) {
    const T dm = v - vm1, dp = vp1 - v;
    T s0 = fma(dm, dm, eps), s1 = fma(dp, dp, eps);
    s0 = s0 * s0;
    s1 = s1 * s1;
    ur = fma(T(0.5) * fma(s1, dm, T(2) * s0 * dp), T(1) / fma(T(2), s0, s1), v);
    ul = fma(T(-0.5) * fma(s0, dp, T(2) * s1 * dm), T(1) / fma(T(2), s1, s0), v);
}

// ---- MUSCL limiters (limiters.py) --------------------------------------------
// flux limiter phi(r) (evaluate(lm, r)); param: theta (minmod) or the van
// Albada variant
template <class T>
__device__ __forceinline__ T limiter_phi(int lim, T r, T param) {
    switch (lim) {
        case SHK_LIM_MINMOD: return fmax(T(0), fmin(fmin(param, param * r), (T(1) + r) / T(2)));
        case SHK_LIM_MC: return fmax(T(0), fmin(fmin(T(2), T(2) * r), (T(1) + r) / T(2)));
        case SHK_LIM_SUPERBEE: return fmax(T(0), fmax(fmin(T(1), T(2) * r), fmin(T(2), r)));
        case SHK_LIM_VANALBADA:
            return fmax(T(0), param == T(1) ? (r * r + r) / (r * r + T(1)) : T(2) * r / (r * r + T(1)));
        case SHK_LIM_VANLEER: return fmax(T(0), (r + fabs(r)) / (T(1) + fabs(r)));
        case SHK_LIM_KOREN: return fmax(T(0), fmin(fmin(T(2), T(2) * r), (T(1) + T(2) * r) / T(3)));
        default: return T(1);  // unlimited
    }
}

// phi(1/r) = phi(r)/r holds for these (limiters.py: is_symmetric)
__device__ __forceinline__ bool limiter_symmetric(int lim, double param) {
    return lim == SHK_LIM_MINMOD || lim == SHK_LIM_MC || lim == SHK_LIM_SUPERBEE ||
           lim == SHK_LIM_VANLEER || (lim == SHK_LIM_VANALBADA && param == 1.0);
}

// flux-limited MUSCL of cell c (reconstruction.py:212-245): slope ratio
// r = (v - v_{c-1}) / (v_{c+1} - v) with the atol cut of limiters.py:110-125,
// ur = v + phi(r)/2 (v_{c+1} - v), ul = v - phi(1/r)/2 (v - v_{c-1})
template <class T>
__device__ __forceinline__ void muscl_cell(T vm1, T v, T vp1, int lim, T param, T atol, T& ul,
                                           T& ur) {
    T sl = v - vm1, sr = vp1 - v;
    const T dl = sl, dr = sr;
    if (fabs(sr) < atol) {
        sl = T(0);
        sr = T(1);
    }
    const T r = sl / sr;
    const T phi_r = limiter_phi<T>(lim, r, param);
    T phi_inv;
    if (limiter_symmetric(lim, static_cast<double>(param))) {
        phi_inv = fabs(r) < atol ? T(0) : phi_r / r;
    } else {
        const T inv_r = fabs(r) < atol ? atol : T(1) / r;
        phi_inv = limiter_phi<T>(lim, inv_r, param);
    }
    ur = v + T(0.5) * phi_r * dr;
    ul = v - T(0.5) * phi_inv * dl;
}

template <class T>
__device__ __forceinline__ T minmod2(T a, T b) {
    return a * b < T(0) ? T(0) : (fabs(a) < fabs(b) ? a : b);
}

// slope-limited MUSCL of cell c (reconstruction.py:271-290 with
// limiters.py:147-155,201-209,234-245,270-278,326-339,365-375) on a uniform
// grid: du dx from the raw differences; ul, ur = v -+ (du dx) / 2
template <class T>
__device__ __forceinline__ void muscls_cell(T vm1, T v, T vp1, int lim, T param, T dx, T& ul,
                                            T& ur) {
    const T sl = v - vm1, sr = vp1 - v;
    T s;
    switch (lim) {
        case SHK_LIM_MINMOD: s = minmod2(sl, sr); break;
        case SHK_LIM_MC: s = minmod2(minmod2(sl, sr), (vp1 - vm1) / T(2)); break;
        case SHK_LIM_SUPERBEE: s = fmax(minmod2(sl, T(2) * sr), minmod2(T(2) * sl, sr)); break;
        case SHK_LIM_VANALBADA:
            // variant 2's "slope" 2 sl sr / (sl^2 + sr^2) is scale-free in the
            // reference and still multiplied by dx / 2: the face offset keeps dx
            s = sl * sr <= T(0) ? T(0)
                                : (param == T(1) ? sl * sr * (sl + sr) / (sl * sl + sr * sr)
                                                 : dx * (T(2) * sl * sr / (sl * sl + sr * sr)));
            break;
        case SHK_LIM_VANLEER: s = sl * sr <= T(0) ? T(0) : T(2) * sl * sr / (sl + sr); break;
        default: s = (vp1 + vm1) / T(2); break;  // the reference's unlimited slope (limiters.py:150)
    }
    ur = v + T(0.5) * s;
    ul = v - T(0.5) * s;
}

// ---- numerical fluxes at face j+1/2 -----------------------------------------
// R = ur_j, L = ul_{j+1}, vj, vj1 cell values.
template <int EQ, class T>
__device__ __forceinline__ T rusanov_face(T R, T L, T vj, T vj1, T hnu, T c) {
    // F = 1/2 (f(L) + f(R)) - 1/2 a nu (L - R), a = max|f'(v)| of the cells
    const T a = absmax(wave_speed<EQ>(vj, c), wave_speed<EQ>(vj1, c));
    const T diss = (hnu * a) * (L - R);
    if constexpr (EQ == SHK_EQ_BURGERS) {
        return fma(T(0.25), fma(L, L, R * R), -diss);
    } else {
        return fma(T(0.5), phys_flux_sum<EQ>(L, R, c), -diss);
    }
}

// global Lax-Friedrichs: the wave speed is the instance-wide max (scalar.py:277)
template <int EQ, class T>
__device__ __forceinline__ T lf_face(T R, T L, T hnu_amax, T c) {
    const T diss = hnu_amax * (L - R);
    if constexpr (EQ == SHK_EQ_BURGERS) {
        return fma(T(0.25), fma(L, L, R * R), -diss);
    } else {
        return fma(T(0.5), phys_flux_sum<EQ>(L, R, c), -diss);
    }
}

// ES-WENO: upwind flux with a = u (scalar.py:123-132) plus the dissipative
// g = -(mu + dw/8)(v_{j+1} - v_j), mu = sqrt(dw^2 + delta^2)/8 (burgers/schemes.py:242-251)
template <int EQ, class T>
__device__ __forceinline__ T esweno_face(T R, T L, T vj, T vj1, T w0j, T w0j1, T delta,
                                         T c) {
    const T aavg = (wave_speed<EQ>(R, c) + wave_speed<EQ>(L, c)) / T(2);
    const T fnum = aavg > T(0) ? phys_flux<EQ>(R, c) : phys_flux<EQ>(L, c);
    const T dw = w0j1 - w0j;
    const T mu = sqrt(dw * dw + delta * delta) / T(8);
    const T g = -(mu + dw / T(8)) * (vj1 - vj);
    return fnum + g;
}

// Godunov / upwind (scalar.py:91-132 with a = u, burgers/schemes.py:83-89):
// the reconstructed speeds are the reconstructed states, S = (R + L)/2
template <int EQ, class T>
__device__ __forceinline__ T godunov_face(T R, T L, T c) {
    const T aavg = (wave_speed<EQ>(R, c) + wave_speed<EQ>(L, c)) / T(2);
    return aavg > T(0) ? phys_flux<EQ>(R, c) : phys_flux<EQ>(L, c);
}

// Engquist-Osher for a convex flux with its minimum at omega = 0
// (scalar.py:287-322, burgers/schemes.py:184-196): f(max(R, 0)) + f(min(L, 0)) - f(0)
template <int EQ, class T>
__device__ __forceinline__ T eo_face(T R, T L, T c) {
    return phys_flux<EQ>(fmax(R, T(0)), c) + phys_flux<EQ>(fmin(L, T(0)), c) -
           phys_flux<EQ>(T(0), c);
}

// ---- mbarrier / bulk copy (inline PTX) -------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// bounded wait: returns false if the limit expired
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    const long long limit = wait_limit();
    for (long long it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// ---- block reductions -------------------------------------------------------
template <class U>
__device__ __forceinline__ U warp_max(U x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        U y = __shfl_xor_sync(0xffffffffu, x, o);
        x = y > x ? y : x;
    }
    return x;
}
template <class U>
__device__ __forceinline__ U block_max(U x, U* scratch /* >= 32 */) {
    x = warp_max(x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[warp] = x;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    U y = threadIdx.x < nw ? scratch[threadIdx.x] : U(0);
    if (warp == 0) y = warp_max(y);
    return y;  // valid in thread 0
}
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

}  // namespace shk
