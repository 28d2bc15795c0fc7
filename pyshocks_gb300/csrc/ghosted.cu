// The reference's SSPRK33 step on one ghosted array, forward and exact
// transpose.
//
// The drop-in adjoint_step (src/pyshocks/timestepping.py:155-215) transposes
// jax.jacfwd of advance() over the whole ghosted array of n + 2g cells
// (:174, :205-206). That Jacobian has rows for the ghost cells as well: every
// operator evaluation first overwrites the ghosts by the boundary
// (schemes.py:339-346 -> scalar.py:397-540), so the ghost *inputs* of L only
// matter through the boundary's map (periodic images, Neumann mirrors,
// Dirichlet data), but L has ghost *outputs* (the flux difference at the
// ghost cells, with the fluxes beyond the array end padded to zero,
// scalar.py:249, and the reconstruction's "same" convolutions zero-padded
// beyond the array, convolve.py:113-114), and the raw ghost values pass
// through 1/3 u + 2/3 (...) unchanged. A cotangent p with nonzero ghost
// entries -- the reference driver seeds p0 = u(T) and applies a Neumann
// adjoint boundary to p after every step (drivers/burgers-adjoint.py:203-212,
// 269-281) -- therefore reaches the interior through those ghost rows.
//
// These kernels restate that arithmetic on the ghosted array itself, one
// thread per cell, with zero padding beyond both ends:
//   fill    v -> BC(v) at the stage time (the boundary's ghost overwrite),
//   recon   ul, ur of every cell (constant, or WENO-JS5 in the product form of
//           the tiled kernels, on the zero-padded stencil),
//   flux    F_j, j = 1 .. M-1 (Rusanov a_j = max |f'| of the two cells, or the
//           global Lax-Friedrichs a = max over the whole filled array,
//           scalar.py:258-278), F_0 = F_M = 0,
//   stage   out = cu u + ck (k + dt L(BC(k))), L_i = -(F_{i+1} - F_i)/dx.
// The transpose runs the same per-stage pieces backwards:
//   k2b = 2/3 (p + Z3),  k1b = 1/4 (k2b + Z2),  ub = 1/3 p + 3/4 k2b + k1b + Z1,
// with Z_s = dt BC^T J_L(BC(k_s))^T w (w = p, k2b, k1b) over all M cells.
// max() and |.| follow the JAX convention at ties: the cotangent of the
// global maximum is shared evenly by all cells attaining it, max(x, y)
// splits evenly, d|s|/ds = 0 at 0.
//
// Memory: caller workspace (shk_ghosted_workspace_bytes), no allocation.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

#include "adjoint_math.cuh"

namespace shk {
namespace {

constexpr int kGhThreads = 256;
constexpr int kPad = 3;          // zero cells beyond each end of the array
constexpr int kGhMaxBlocks = 1024;

struct GhArgs {
    int64_t n;   // interior cells
    int64_t M;   // n + 2 g
    int g;       // ghost cells per side
    double dx;
    double eps;  // WENO epsilon
    double hnu;  // nu / 2
    double c;    // advection speed
    shk_boundary bc;
};

// ---- boundary fill (scalar.py:397-540) -------------------------------------
// value at ghosted index i of the filled stage input v: interior unchanged;
// periodic ghosts take the interior images (right ghosts the first g interior
// cells, left ghost i the cell n + i, scalar.py:529-540); Dirichlet ghosts the
// data at their centres; Neumann ghosts mirror - (2k + 1) dx g_n(t_s)
template <class PV>
__device__ __forceinline__ double gh_fill_value(const GhArgs& A, PV v, int64_t i, int stage) {
    const int64_t g = A.g, n = A.n;
    if (i >= g && i < g + n) return v[i];
    const int side = i < g ? 0 : 1;
    const int kind = side ? A.bc.right : A.bc.left;
    const int64_t k = side ? i - (g + n) : g - 1 - i;  // 0: next to the interior
    if (kind == SHK_BC_PERIODIC) return side ? v[g + k] : v[n + i];
    if (kind == SHK_BC_DIRICHLET) return A.bc.dirichlet[stage][side][k];
    const int64_t mirror = side ? g + n - 1 - k : g + k;
    return v[mirror] - static_cast<double>(2 * k + 1) * A.dx * A.bc.neumann[stage][side];
}

// vp[q], q = i + kPad: the filled array with kPad zeros on each side
__global__ void gh_fill_kernel(GhArgs A, const double* __restrict__ v_, double* __restrict__ vp_,
                               int stage) {
    const Win<const double> v = make_win(v_, A.M);
    const Win<double> vp = make_win(vp_, A.M + 2 * kPad);
    const int64_t P = A.M + 2 * kPad;
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < P;
         q += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = q - kPad;
        vp[q] = (i < 0 || i >= A.M) ? 0.0 : gh_fill_value(A, v, i, stage);
    }
}

// ---- reconstruction of every cell (reconstruction.py:153-163, 351-377) -----
template <int REC>
__global__ void gh_recon_kernel(GhArgs A, const double* __restrict__ vp_, double* __restrict__ ul_,
                                double* __restrict__ ur_) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    const Win<double> ul = make_win(ul_, A.M), ur = make_win(ur_, A.M);
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t q = i + kPad;
        if constexpr (REC == SHK_REC_CONSTANT) {
            ul[i] = vp[q];
            ur[i] = vp[q];
        } else {
            // unscaled differences of the zero-padded stencil, as face_fluxes
            const double dm2 = vp[q - 1] - vp[q - 2], dm1 = vp[q] - vp[q - 1];
            const double d0 = vp[q + 1] - vp[q], dp1 = vp[q + 2] - vp[q + 1];
            const double Em1 = dm1 - dm2, E0 = d0 - dm1, Ep1 = dp1 - d0;
            const double eps4 = 4.0 * A.eps;
            double l, r;
            weno53_cell_d(vp[q], dm1, d0, Em1, E0, Ep1, fma((13.0 / 3.0) * Em1, Em1, eps4),
                          fma((13.0 / 3.0) * E0, E0, eps4), fma((13.0 / 3.0) * Ep1, Ep1, eps4), l, r);
            ul[i] = l;
            ur[i] = r;
        }
    }
}

// ---- global max of |f'| over the filled array and the cells attaining it ---
template <int EQ>
__global__ void gh_max_kernel(GhArgs A, const double* __restrict__ vp_, unsigned long long* amax) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    __shared__ unsigned long long red[32];
    unsigned long long mx = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x) {
        const unsigned long long b = abs_bits(wave_speed<EQ>(vp[i + kPad], A.c));
        mx = b > mx ? b : mx;
    }
    const unsigned long long bm = block_max<unsigned long long>(mx, red);
    if (threadIdx.x == 0) atomicMax(amax, bm);
}
template <int EQ>
__global__ void gh_count_kernel(GhArgs A, const double* __restrict__ vp_,
                                const unsigned long long* amax, unsigned int* count) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    unsigned int cnt = 0;
    const unsigned long long m = *amax;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x)
        cnt += abs_bits(wave_speed<EQ>(vp[i + kPad], A.c)) == m ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(count, cnt);
}

// wave speed of face j (between cells j-1 and j)
template <int EQ, int FLUX>
__device__ __forceinline__ double gh_face_speed(const GhArgs& A, double vl, double vr,
                                                const unsigned long long* amax) {
    if constexpr (FLUX == SHK_FLUX_LF) return from_bits(*amax);
    else return absmax(wave_speed<EQ>(vl, A.c), wave_speed<EQ>(vr, A.c));
}

// ---- fluxes and the stage update -------------------------------------------
template <int EQ, int FLUX>
__global__ void gh_flux_kernel(GhArgs A, const double* __restrict__ vp_, const double* __restrict__ ul_,
                               const double* __restrict__ ur_, const unsigned long long* amax,
                               double* __restrict__ F_) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    const Win<const double> ul = make_win(ul_, A.M), ur = make_win(ur_, A.M);
    const Win<double> F = make_win(F_, A.M + 1);
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j <= A.M;
         j += int64_t(gridDim.x) * blockDim.x) {
        if (j == 0 || j == A.M) {
            F[j] = 0.0;  // scalar.py:249: the flux array is padded with zeros
            continue;
        }
        const double L = ul[j], R = ur[j - 1];
        const double a = gh_face_speed<EQ, FLUX>(A, vp[j - 1 + kPad], vp[j + kPad], amax);
        // F = 1/2 (f(L) + f(R)) - 1/2 a nu (L - R)   (scalar.py:248)
        F[j] = fma(0.5, phys_flux<EQ>(L, A.c) + phys_flux<EQ>(R, A.c), -((A.hnu * a) * (L - R)));
    }
}

// out = cu u + ck (k + dt L),  L_i = -(F_{i+1} - F_i) / dx  (schemes.py:346,
// timestepping.py:318-320)
__global__ void gh_stage_kernel(GhArgs A, const double* __restrict__ u_, const double* __restrict__ k_,
                                const double* __restrict__ F_, double* __restrict__ out_, double dt,
                                double cu, double ck) {
    const Win<const double> u = make_win(u_, A.M), k = make_win(k_, A.M), F = make_win(F_, A.M + 1);
    const Win<double> out = make_win(out_, A.M);
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x) {
        const double L = -(F[i + 1] - F[i]) / A.dx;
        out[i] = cu * u[i] + ck * (k[i] + dt * L);
    }
}

// L_i = -(F_{i+1} - F_i) / dx on every cell, ghosts included (schemes.py:346)
__global__ void gh_rhs_kernel(GhArgs A, const double* __restrict__ F_, double* __restrict__ out_) {
    const Win<const double> F = make_win(F_, A.M + 1);
    const Win<double> out = make_win(out_, A.M);
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x)
        out[i] = -(F[i + 1] - F[i]) / A.dx;
}

// ---- transpose of one operator evaluation ----------------------------------
// Face seeds of w (the cotangent of dt L over all M cells): fb_j = dt (w_j -
// w_{j-1}) / dx; gl[j] / gr[j-1]: cotangents of ul_j / ur_{j-1} through F_j;
// ga[j]: of F_j's wave speed.
template <int EQ, int FLUX>
__global__ void gh_seed_kernel(GhArgs A, const double* __restrict__ vp_, const double* __restrict__ ul_,
                               const double* __restrict__ ur_, const unsigned long long* amax,
                               const double* __restrict__ w_, double dt, double* __restrict__ gl_,
                               double* __restrict__ gr_, double* __restrict__ ga_) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    const Win<const double> ul = make_win(ul_, A.M), ur = make_win(ur_, A.M), w = make_win(w_, A.M);
    const Win<double> gl = make_win(gl_, A.M), gr = make_win(gr_, A.M), ga = make_win(ga_, A.M + 1);
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j <= A.M;
         j += int64_t(gridDim.x) * blockDim.x) {
        if (j == 0) {
            gl[0] = 0.0;
            ga[0] = 0.0;
            continue;
        }
        if (j == A.M) {
            gr[A.M - 1] = 0.0;
            ga[A.M] = 0.0;
            continue;
        }
        const double fb = (dt * (w[j] - w[j - 1])) / A.dx;
        const double L = ul[j], R = ur[j - 1];
        const double a = gh_face_speed<EQ, FLUX>(A, vp[j - 1 + kPad], vp[j + kPad], amax);
        gl[j] = fb * fma(0.5, flux_prime<EQ>(L, A.c), -(A.hnu * a));
        gr[j - 1] = fb * fma(0.5, flux_prime<EQ>(R, A.c), A.hnu * a);
        ga[j] = -(fb * A.hnu) * (L - R);
    }
}

// per-cell reconstruction backward: contributions t_o to the cotangents of
// v_{c-2+o} (T[o * M + c]); constant: t_2 = gl + gr
template <int REC>
__global__ void gh_recon_vjp_kernel(GhArgs A, const double* __restrict__ vp_,
                                    const double* __restrict__ gl_, const double* __restrict__ gr_,
                                    double* __restrict__ T_) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    const Win<const double> gl = make_win(gl_, A.M), gr = make_win(gr_, A.M);
    const Win<double> T = make_win(T_, 5 * A.M);
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < A.M;
         c += int64_t(gridDim.x) * blockDim.x) {
        if constexpr (REC == SHK_REC_CONSTANT) {
            T[2 * A.M + c] = gl[c] + gr[c];
        } else {
            const int64_t q = c + kPad;
            // half differences of the zero-padded stencil, as vjp_stage
            const double Hm2 = 0.5 * (vp[q - 1] - vp[q - 2]), Hm1 = 0.5 * (vp[q] - vp[q - 1]);
            const double H0 = 0.5 * (vp[q + 1] - vp[q]), Hp1 = 0.5 * (vp[q + 2] - vp[q + 1]);
            const double Dm1 = Hm1 - Hm2, D0 = H0 - Hm1, Dp1 = Hp1 - H0;
            double t0, t1, t2, t3, t4;
            weno53_cell_vjp<double>(Hm2, Hm1, H0, Hp1, Dm1, D0, Dp1, (13.0 / 3.0 * Dm1) * Dm1,
                                    (13.0 / 3.0 * D0) * D0, (13.0 / 3.0 * Dp1) * Dp1, A.eps, gr[c],
                                    gl[c], t0, t1, t2, t3, t4);
            T[c] = t0;
            T[A.M + c] = t1;
            T[2 * A.M + c] = t2;
            T[3 * A.M + c] = t3;
            T[4 * A.M + c] = t4;
        }
    }
}

// sum of the face-speed cotangents of the global Lax-Friedrichs flux: fixed
// per-block partial sums, then one ordered sum (deterministic)
__global__ void gh_sum_partial_kernel(GhArgs A, const double* __restrict__ ga_, double* __restrict__ part) {
    const Win<const double> ga = make_win(ga_, A.M + 1);
    __shared__ double red[32];
    double s = 0.0;
    for (int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; j <= A.M;
         j += int64_t(gridDim.x) * blockDim.x)
        s += ga[j];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (blockDim.x >> 5); ++w) r += red[w];
        part[blockIdx.x] = r;
    }
}
__global__ void gh_sum_final_kernel(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int b = 0; b < nparts; ++b) r += part[b];
        *out = r;
    }
}

// z_i: cotangent of the filled state at cell i (recon taps, face speeds, the
// global max), then the boundary's transpose into the raw stage input and the
// stage combination (see the file comment). mode 3: k2b = 2/3 (p + Zt),
// acc = 1/3 p; mode 2: k1b = 1/4 (k2b + Zt), acc += 3/4 k2b; mode 1:
// out = acc + (k1b + Zt).
template <int EQ, int REC, int FLUX>
__device__ double gh_z(const GhArgs& A, Win<const double> vp, Win<const double> T,
                       Win<const double> ga, const unsigned long long* amax,
                       const unsigned int* count, const double* gsum, int64_t i) {
    const int64_t M = A.M;
    double z;
    if constexpr (REC == SHK_REC_CONSTANT) {
        z = T[2 * M + i];
    } else {
        const double a0 = i + 2 < M ? T[i + 2] : 0.0;
        const double a1 = i + 1 < M ? T[M + i + 1] : 0.0;
        const double a3 = i >= 1 ? T[3 * M + i - 1] : 0.0;
        const double a4 = i >= 2 ? T[4 * M + i - 2] : 0.0;
        z = (a0 + a1) + T[2 * M + i] + (a3 + a4);
    }
    const double vi = vp[i + kPad];
    if constexpr (FLUX == SHK_FLUX_RUSANOV) {
        if (i >= 1) z = fma(ga[i], damax_dx<EQ>(vi, vp[i - 1 + kPad], A.c), z);
        if (i + 1 < M) z = fma(ga[i + 1], damax_dx<EQ>(vi, vp[i + 1 + kPad], A.c), z);
    } else {
        const double s = wave_speed<EQ>(vi, A.c);
        if (abs_bits(s) == *amax)
            z = fma(*gsum, (sgn(s) * speed_prime<EQ, double>()) / static_cast<double>(*count), z);
    }
    return z;
}

template <int EQ, int REC, int FLUX>
__global__ void gh_gather_kernel(GhArgs A, const double* __restrict__ vp_, const double* __restrict__ T_,
                                 const double* __restrict__ ga_, const unsigned long long* amax,
                                 const unsigned int* count, const double* gsum, int mode,
                                 const double* __restrict__ p_, double* __restrict__ cb_,
                                 double* __restrict__ acc_, double* __restrict__ out_) {
    const Win<const double> vp = make_win(vp_, A.M + 2 * kPad);
    const Win<const double> T = make_win(T_, 5 * A.M), ga = make_win(ga_, A.M + 1);
    const Win<const double> p = make_win(p_, A.M);
    const Win<double> cb = make_win(cb_, A.M), acc = make_win(acc_, A.M);
    const Win<double> out = make_win(out_, A.M);
    const int64_t g = A.g, n = A.n;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < A.M;
         i += int64_t(gridDim.x) * blockDim.x) {
        // the raw input's ghosts are overwritten before L reads them: zero
        double zt = 0.0;
        if (i >= g && i < g + n) {
            zt = gh_z<EQ, REC, FLUX>(A, vp, T, ga, amax, count, gsum, i);
            // transpose of the ghost fill: ghost cotangents to the interior
            // cells they were filled from
            const int64_t kl = i - g;          // left side: distance of the mirror
            const int64_t kr = g + n - 1 - i;  // right side
            if (A.bc.left == SHK_BC_PERIODIC) {
                if (kl < g) zt += gh_z<EQ, REC, FLUX>(A, vp, T, ga, amax, count, gsum, g + n + kl);
                if (i >= n && i - n < g) zt += gh_z<EQ, REC, FLUX>(A, vp, T, ga, amax, count, gsum, i - n);
            } else {
                if (A.bc.left == SHK_BC_NEUMANN && kl < g)
                    zt += gh_z<EQ, REC, FLUX>(A, vp, T, ga, amax, count, gsum, g - 1 - kl);
                if (A.bc.right == SHK_BC_NEUMANN && kr < g)
                    zt += gh_z<EQ, REC, FLUX>(A, vp, T, ga, amax, count, gsum, g + n + kr);
            }
        }
        if (mode == 3) {
            const double k2b = (2.0 / 3.0) * (p[i] + zt);
            cb[i] = k2b;
            acc[i] = fma(3.0 / 4.0, k2b, (1.0 / 3.0) * p[i]);
        } else if (mode == 2) {
            cb[i] = (1.0 / 4.0) * (cb[i] + zt);
        } else {
            out[i] = acc[i] + (cb[i] + zt);
        }
    }
}

// ---- host side ----------------------------------------------------------------

int gh_cuda(cudaError_t e) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "libshocks: CUDA error %s\n", cudaGetErrorString(e));
        return SHK_ECUDA;
    }
    return SHK_OK;
}
#define GH_CUDA(call)                       \
    do {                                    \
        const int _st = gh_cuda(call);      \
        if (_st != SHK_OK) return _st;      \
    } while (0)

// workspace carve (doubles unless noted), P = M + 2 kPad
struct GhWork {
    double* vp[3];  // filled u, k1, k2 (P each)
    double* ul[3];
    double* ur[3];  // their face values (M each)
    double* F;      // M + 1
    double* k1;
    double* k2;     // M each
    double* gl;
    double* gr;     // M each
    double* ga;     // M + 1
    double* T;      // 5 M
    double* cb;
    double* acc;    // M each
    double* part;   // kGhMaxBlocks
    double* gsum;   // 1
    unsigned long long* amax;  // 3
    unsigned int* count;       // 3
};

int64_t gh_bytes(int64_t M) {
    const int64_t P = M + 2 * kPad;
    const int64_t doubles = 3 * P + 6 * M + (M + 1) + 2 * M + 2 * M + (M + 1) + 5 * M + 2 * M +
                            kGhMaxBlocks + 1;
    return 8 * doubles + 8 * 3 + 4 * 4 + 256;
}

GhWork gh_carve(void* ws, int64_t M) {
    const int64_t P = M + 2 * kPad;
    uintptr_t a = (reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255);
    double* d = reinterpret_cast<double*>(a);
    GhWork w;
    for (int s = 0; s < 3; ++s) { w.vp[s] = d; d += P; }
    for (int s = 0; s < 3; ++s) { w.ul[s] = d; d += M; w.ur[s] = d; d += M; }
    w.F = d; d += M + 1;
    w.k1 = d; d += M;
    w.k2 = d; d += M;
    w.gl = d; d += M;
    w.gr = d; d += M;
    w.ga = d; d += M + 1;
    w.T = d; d += 5 * M;
    w.cb = d; d += M;
    w.acc = d; d += M;
    w.part = d; d += kGhMaxBlocks;
    w.gsum = d; d += 1;
    w.amax = reinterpret_cast<unsigned long long*>(d);
    w.count = reinterpret_cast<unsigned int*>(w.amax + 3);
    return w;
}

int gh_reach(int rec) { return rec == SHK_REC_CONSTANT ? 1 : 3; }

bool gh_supported(const shk_scheme* s) {
    return s && (s->rec == SHK_REC_CONSTANT || s->rec == SHK_REC_WENOJS53) &&
           (s->flux == SHK_FLUX_RUSANOV || s->flux == SHK_FLUX_LF) && s->equation >= SHK_EQ_BURGERS &&
           s->equation <= SHK_EQ_LWR;
}

int gh_args(const shk_scheme* s, const shk_boundary* bc, int64_t n, int32_t g, double dx,
            int64_t ws_bytes, const void* ws, GhArgs* A) {
    if (!gh_supported(s)) return SHK_EUNSUPPORTED;
    shk_boundary b;
    std::memset(&b, 0, sizeof(b));
    if (bc) b = *bc;
    const bool periodic = b.left == SHK_BC_PERIODIC && b.right == SHK_BC_PERIODIC;
    if (b.left < SHK_BC_PERIODIC || b.left > SHK_BC_NEUMANN || b.right < SHK_BC_PERIODIC ||
        b.right > SHK_BC_NEUMANN || (!periodic && (b.left == SHK_BC_PERIODIC || b.right == SHK_BC_PERIODIC)))
        return SHK_EINVAL;
    // ghosts: at least the reconstruction's reach; boundary data for at most 3
    if (g < gh_reach(s->rec) || (!periodic && g > 3) || n < 3 || n < g || !(dx > 0)) return SHK_EINVAL;
    if (!ws || ws_bytes < gh_bytes(n + 2 * int64_t(g))) return SHK_EINVAL;
    A->n = n;
    A->M = n + 2 * int64_t(g);
    A->g = g;
    A->dx = dx;
    A->eps = s->eps;
    A->hnu = 0.5 * s->nu;
    A->c = s->speed;
    A->bc = b;
    return SHK_OK;
}

struct GhLaunch {
    GhArgs A;
    GhWork W;
    cudaStream_t st;
    int blocks;
    int blocksP;
};

template <int EQ, int REC, int FLUX>
int gh_operator(const GhLaunch& L, const double* v, int stage) {
    // fill, reconstruct and (LF) the global max of the stage input v
    const GhArgs& A = L.A;
    const GhWork& W = L.W;
    gh_fill_kernel<<<L.blocksP, kGhThreads, 0, L.st>>>(A, v, W.vp[stage], stage);
    GH_CUDA(cudaGetLastError());
    gh_recon_kernel<REC><<<L.blocks, kGhThreads, 0, L.st>>>(A, W.vp[stage], W.ul[stage], W.ur[stage]);
    GH_CUDA(cudaGetLastError());
    if constexpr (FLUX == SHK_FLUX_LF) {
        gh_max_kernel<EQ><<<L.blocks, kGhThreads, 0, L.st>>>(A, W.vp[stage], W.amax + stage);
        GH_CUDA(cudaGetLastError());
        gh_count_kernel<EQ><<<L.blocks, kGhThreads, 0, L.st>>>(A, W.vp[stage], W.amax + stage,
                                                             W.count + stage);
        GH_CUDA(cudaGetLastError());
    }
    return SHK_OK;
}

template <int EQ, int REC, int FLUX>
int gh_stage(const GhLaunch& L, const double* u, const double* k, double* out, int stage, double dt,
             double cu, double ck) {
    int r = gh_operator<EQ, REC, FLUX>(L, k, stage);
    if (r != SHK_OK) return r;
    gh_flux_kernel<EQ, FLUX><<<L.blocks, kGhThreads, 0, L.st>>>(L.A, L.W.vp[stage], L.W.ul[stage],
                                                               L.W.ur[stage], L.W.amax + stage, L.W.F);
    GH_CUDA(cudaGetLastError());
    gh_stage_kernel<<<L.blocks, kGhThreads, 0, L.st>>>(L.A, u, k, L.W.F, out, dt, cu, ck);
    return gh_cuda(cudaGetLastError());
}

struct GhStep {
    GhLaunch L;
    const double* u;
    double* out;
    double dt;
    template <int EQ, int REC, int FLUX>
    int run() {
        GH_CUDA(cudaMemsetAsync(L.W.amax, 0, sizeof(unsigned long long) * 3 + sizeof(unsigned int) * 4, L.st));
        int r = gh_stage<EQ, REC, FLUX>(L, u, u, L.W.k1, 0, dt, 0.0, 1.0);
        if (r == SHK_OK) r = gh_stage<EQ, REC, FLUX>(L, u, L.W.k1, L.W.k2, 1, dt, 3.0 / 4.0, 1.0 / 4.0);
        if (r == SHK_OK) r = gh_stage<EQ, REC, FLUX>(L, u, L.W.k2, out, 2, dt, 1.0 / 3.0, 2.0 / 3.0);
        return r;
    }
};

struct GhRhs {
    GhLaunch L;
    const double* u;
    double* out;
    template <int EQ, int REC, int FLUX>
    int run() {
        GH_CUDA(cudaMemsetAsync(L.W.amax, 0, sizeof(unsigned long long) * 3 + sizeof(unsigned int) * 4, L.st));
        int r = gh_operator<EQ, REC, FLUX>(L, u, 0);
        if (r != SHK_OK) return r;
        gh_flux_kernel<EQ, FLUX><<<L.blocks, kGhThreads, 0, L.st>>>(L.A, L.W.vp[0], L.W.ul[0], L.W.ur[0],
                                                                   L.W.amax, L.W.F);
        GH_CUDA(cudaGetLastError());
        gh_rhs_kernel<<<L.blocks, kGhThreads, 0, L.st>>>(L.A, L.W.F, out);
        return gh_cuda(cudaGetLastError());
    }
};

struct GhVjp {
    GhLaunch L;
    const double* u;
    const double* p;
    double* out;
    double dt;
    template <int EQ, int REC, int FLUX>
    int reverse_stage(int stage, const double* w, int mode) {
        const GhArgs& A = L.A;
        const GhWork& W = L.W;
        gh_seed_kernel<EQ, FLUX><<<L.blocks, kGhThreads, 0, L.st>>>(
            A, W.vp[stage], W.ul[stage], W.ur[stage], W.amax + stage, w, dt, W.gl, W.gr, W.ga);
        GH_CUDA(cudaGetLastError());
        gh_recon_vjp_kernel<REC><<<L.blocks, kGhThreads, 0, L.st>>>(A, W.vp[stage], W.gl, W.gr, W.T);
        GH_CUDA(cudaGetLastError());
        if constexpr (FLUX == SHK_FLUX_LF) {
            gh_sum_partial_kernel<<<L.blocks, kGhThreads, 0, L.st>>>(A, W.ga, W.part);
            GH_CUDA(cudaGetLastError());
            gh_sum_final_kernel<<<1, 32, 0, L.st>>>(W.part, L.blocks, W.gsum);
            GH_CUDA(cudaGetLastError());
        }
        gh_gather_kernel<EQ, REC, FLUX><<<L.blocks, kGhThreads, 0, L.st>>>(
            A, W.vp[stage], W.T, W.ga, W.amax + stage, W.count + stage, W.gsum, mode, p, W.cb, W.acc,
            out);
        return gh_cuda(cudaGetLastError());
    }
    template <int EQ, int REC, int FLUX>
    int run() {
        GH_CUDA(cudaMemsetAsync(L.W.amax, 0, sizeof(unsigned long long) * 3 + sizeof(unsigned int) * 4, L.st));
        // forward recompute: k1, k2 and the filled states of u, k1, k2
        int r = gh_stage<EQ, REC, FLUX>(L, u, u, L.W.k1, 0, dt, 0.0, 1.0);
        if (r == SHK_OK) r = gh_stage<EQ, REC, FLUX>(L, u, L.W.k1, L.W.k2, 1, dt, 3.0 / 4.0, 1.0 / 4.0);
        if (r == SHK_OK) r = gh_operator<EQ, REC, FLUX>(L, L.W.k2, 2);
        // reverse: stage 3 at BC(k2) with w = p, stage 2 at BC(k1) with w = k2b,
        // stage 1 at BC(u) with w = k1b
        if (r == SHK_OK) r = reverse_stage<EQ, REC, FLUX>(2, p, 3);
        if (r == SHK_OK) r = reverse_stage<EQ, REC, FLUX>(1, L.W.cb, 2);
        if (r == SHK_OK) r = reverse_stage<EQ, REC, FLUX>(0, L.W.cb, 1);
        return r;
    }
};

template <class F>
int gh_dispatch(const shk_scheme& s, F& f) {
    auto by_flux = [&](auto eq, auto rec) -> int {
        constexpr int EQ = decltype(eq)::value, REC = decltype(rec)::value;
        if (s.flux == SHK_FLUX_LF) return f.template run<EQ, REC, SHK_FLUX_LF>();
        return f.template run<EQ, REC, SHK_FLUX_RUSANOV>();
    };
    auto by_rec = [&](auto eq) -> int {
        if (s.rec == SHK_REC_CONSTANT) return by_flux(eq, std::integral_constant<int, SHK_REC_CONSTANT>());
        return by_flux(eq, std::integral_constant<int, SHK_REC_WENOJS53>());
    };
    switch (s.equation) {
        case SHK_EQ_BURGERS: return by_rec(std::integral_constant<int, SHK_EQ_BURGERS>());
        case SHK_EQ_ADVECTION: return by_rec(std::integral_constant<int, SHK_EQ_ADVECTION>());
        default: return by_rec(std::integral_constant<int, SHK_EQ_LWR>());
    }
}

GhLaunch gh_launch(const GhArgs& A, void* ws, void* stream) {
    GhLaunch L;
    L.A = A;
    L.W = gh_carve(ws, A.M);
    L.st = static_cast<cudaStream_t>(stream);
    const int64_t b = (A.M + 1 + kGhThreads - 1) / kGhThreads;
    const int64_t bp = (A.M + 2 * kPad + kGhThreads - 1) / kGhThreads;
    L.blocks = static_cast<int>(b < kGhMaxBlocks ? b : kGhMaxBlocks);
    L.blocksP = static_cast<int>(bp < kGhMaxBlocks ? bp : kGhMaxBlocks);
    return L;
}

}  // namespace
}  // namespace shk

using namespace shk;

extern "C" {

int64_t shk_ghosted_workspace_bytes(int64_t n, int32_t nghosts) {
    if (n < 1 || nghosts < 0) return 0;
    return gh_bytes(n + 2 * int64_t(nghosts));
}

int shk_apply_operator_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                   double* out, int64_t n, int32_t nghosts, double dx, void* workspace,
                                   int64_t workspace_bytes, void* stream) {
    GhArgs A;
    const int r = gh_args(scheme, bc, n, nghosts, dx, workspace_bytes, workspace, &A);
    if (r != SHK_OK) return r;
    if (!u || !out || u == out) return SHK_EINVAL;
    GhRhs f{gh_launch(A, workspace, stream), u, out};
    return gh_dispatch(*scheme, f);
}

int shk_ssprk33_step_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                 double* u_out, int64_t n, int32_t nghosts, double dx, double dt,
                                 void* workspace, int64_t workspace_bytes, void* stream) {
    GhArgs A;
    const int r = gh_args(scheme, bc, n, nghosts, dx, workspace_bytes, workspace, &A);
    if (r != SHK_OK) return r;
    if (!u || !u_out || u == u_out || !(dt >= 0)) return SHK_EINVAL;
    GhStep f{gh_launch(A, workspace, stream), u, u_out, dt};
    return gh_dispatch(*scheme, f);
}

int shk_ssprk33_vjp_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                const double* p_next, double* p_out, int64_t n, int32_t nghosts,
                                double dx, double dt, void* workspace, int64_t workspace_bytes,
                                void* stream) {
    GhArgs A;
    const int r = gh_args(scheme, bc, n, nghosts, dx, workspace_bytes, workspace, &A);
    if (r != SHK_OK) return r;
    if (!u || !p_next || !p_out || p_out == p_next || p_out == u || !(dt >= 0)) return SHK_EINVAL;
    GhVjp f{gh_launch(A, workspace, stream), u, p_next, p_out, dt};
    return gh_dispatch(*scheme, f);
}

#ifdef SHOCKS_BOUNDS_CHECK
// this translation unit's bounds log (read by shk_check_bounds in forward.cu)
int shk_check_tu_ghosted(shk::BoundsLog* out, int32_t reset) {
    return gh_cuda(shk::bounds_log_read(out, reset != 0));
}
#endif

}  // extern "C"
