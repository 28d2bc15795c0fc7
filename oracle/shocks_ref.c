/*
 * C restatement of pyshocks' WENO-JS5 + Rusanov + SSPRK33 step (float64).
 *
 * THIS IS TEST INFRASTRUCTURE (the oracle) and the CPU baseline of the bench:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU legs load it. It is
 * never part of the product (pyshocks_gb300/ never links or loads it).
 *
 * It follows the reference's arithmetic per instance, on the n interior cells
 * with periodic (circular) indexing, which equals the reference's ghosted
 * evaluation for stencil reach 3 (src/pyshocks/scalar.py:529-540):
 *   smoothness   src/pyshocks/weno.py:114-140, coefficients :206-244
 *   interpolants src/pyshocks/weno.py:143-157
 *   weights      src/pyshocks/weno.py:247-256 (alpha = d/(eps+beta)^2, omega = alpha/sum)
 *   sides        src/pyshocks/reconstruction.py:351-377 (ul: own smoothness of the mirrored stencil)
 *   Rusanov      src/pyshocks/scalar.py:192-249 with the Burgers flux u^2/2
 *   operator     src/pyshocks/schemes.py:339-346
 *   SSPRK33      src/pyshocks/timestepping.py:312-320
 *   dt           src/pyshocks/burgers/schemes.py:121-127 and timestepping.py:139-142
 * Instances are independent: OpenMP threads take whole instances.
 * Build: see oracle/Makefile (no -ffast-math, no FMA contraction).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static inline int64_t wrap(int64_t i, int64_t n) {
    i %= n;
    return i < 0 ? i + n : i;
}

/* right-side WENO-JS5 value at x_{i+1/2} from taps v[0..4] = u_{i-2..i+2} */
static inline double weno5_side(const double v[5], double eps) {
    const double a0 = 13.0 / 12.0, a1 = 1.0 / 4.0;
    /* convolution taps (i+2, i+1, i, i-1, i-2) of weno.py:220-228 */
    const double q10 = v[2] - 2.0 * v[1] + v[0], q20 = 3.0 * v[2] - 4.0 * v[1] + v[0];
    const double q11 = v[3] - 2.0 * v[2] + v[1], q21 = v[3] - v[1];
    const double q12 = v[4] - 2.0 * v[3] + v[2], q22 = v[4] - 4.0 * v[3] + 3.0 * v[2];
    const double b0 = a0 * q10 * q10 + a1 * q20 * q20;
    const double b1 = a0 * q11 * q11 + a1 * q21 * q21;
    const double b2 = a0 * q12 * q12 + a1 * q22 * q22;
    const double e0 = eps + b0, e1 = eps + b1, e2 = eps + b2;
    const double al0 = 0.1 / (e0 * e0), al1 = 0.6 / (e1 * e1), al2 = 0.3 / (e2 * e2);
    const double s = al0 + al1 + al2;
    /* weno.py:231-239 */
    const double h0 = 11.0 / 6.0 * v[2] - 7.0 / 6.0 * v[1] + 2.0 / 6.0 * v[0];
    const double h1 = 2.0 / 6.0 * v[3] + 5.0 / 6.0 * v[2] - 1.0 / 6.0 * v[1];
    const double h2 = -1.0 / 6.0 * v[4] + 5.0 / 6.0 * v[3] + 2.0 / 6.0 * v[2];
    return al0 / s * h0 + al1 / s * h1 + al2 / s * h2;
}

/* L(u) = -(F_{i+1/2} - F_{i-1/2}) / dx, Burgers + Rusanov + WENO-JS5; f is n faces scratch */
void ref_apply_operator(const double* u, double* out, double* ul, double* ur, double* f,
                        int64_t n, double dx, double eps) {
    for (int64_t i = 0; i < n; ++i) {
        double v[5], w[5];
        for (int k = 0; k < 5; ++k) {
            v[k] = u[wrap(i - 2 + k, n)];
            w[k] = u[wrap(i + 2 - k, n)];
        }
        ur[i] = weno5_side(v, eps);
        ul[i] = weno5_side(w, eps); /* mirrored stencil (reconstruction.py:375) */
    }
    for (int64_t i = 0; i < n; ++i) {
        const int64_t j = wrap(i + 1, n);
        const double L = ul[j], R = ur[i];
        const double fl = L * L / 2.0, fr = R * R / 2.0;
        const double a = fmax(fabs(u[j]), fabs(u[i]));
        f[i] = 0.5 * (fl + fr) - 0.5 * a * 1.0 * (L - R);
    }
    for (int64_t i = 0; i < n; ++i) out[i] = -(f[i] - f[wrap(i - 1, n)]) / dx;
}

/* one SSPRK33 step; work holds 6 n doubles */
void ref_ssprk33(const double* u, double* out, double* work, int64_t n, double dt, double dx,
                 double eps) {
    double *k = work, *L = work + n, *ul = work + 2 * n, *ur = work + 3 * n, *f = work + 4 * n;
    ref_apply_operator(u, L, ul, ur, f, n, dx, eps);
    for (int64_t i = 0; i < n; ++i) k[i] = u[i] + dt * L[i];
    ref_apply_operator(k, L, ul, ur, f, n, dx, eps);
    for (int64_t i = 0; i < n; ++i) k[i] = 3.0 / 4.0 * u[i] + 1.0 / 4.0 * (k[i] + dt * L[i]);
    ref_apply_operator(k, L, ul, ur, f, n, dx, eps);
    for (int64_t i = 0; i < n; ++i) out[i] = 1.0 / 3.0 * u[i] + 2.0 / 3.0 * (k[i] + dt * L[i]);
}

/* batched fixed-count run (tfinal = None: dt + 1e-15 every step). u holds the
 * packed initial state on entry and the final state on exit; dts[m*B + b]
 * receives the time steps (may be NULL). Returns the thread count used. */
int ref_run_batch(double* u, const int64_t* offsets, int32_t B, const double* dx, double theta,
                  double eps, int32_t nsteps, double* dts, int32_t nthreads) {
    int used = 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
    {
#pragma omp single
        used = omp_get_num_threads();
    }
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int32_t b = 0; b < B; ++b) {
        const int64_t n = offsets[b + 1] - offsets[b];
        double* ub = u + offsets[b];
        double* tmp = (double*)malloc(sizeof(double) * 7 * (size_t)n);
        double* work = tmp + n;
        for (int32_t m = 0; m < nsteps; ++m) {
            double smax = 0.0;
            for (int64_t i = 0; i < n; ++i) smax = fmax(smax, fabs(ub[i]));
            double dt = theta * (0.5 * pow(dx[b], 1.0) / smax);
            dt = dt + 1.0e-15;
            if (dts) dts[(size_t)m * B + b] = dt;
            ref_ssprk33(ub, tmp, work, n, dt, dx[b], eps);
            memcpy(ub, tmp, sizeof(double) * (size_t)n);
        }
        free(tmp);
    }
    return used;
}
