/*
 * libshocks -- GB300 (sm_103a) kernels for the 1D scalar conservation-law hot
 * path of pyshocks: WENO-JS5 / ES-WENO3 reconstruction, Rusanov / global
 * Lax-Friedrichs / ES-WENO fluxes, SSPRK33 stepping with the CFL time step,
 * and the discrete adjoint of that step.
 *
 * C ABI: plain pointers and sizes, no C++ or torch types. All array pointers
 * are DEVICE pointers unless the name starts with `h_`. Every call is
 * asynchronous on `stream` (a cudaStream_t passed as void*; NULL = legacy
 * default stream) and returns a shk_status; a device-side status word is
 * read back with shk_plan_status().
 *
 * Reference interfaces (alexfikl/pyshocks) each entry point replaces are
 * cited beside it as src/pyshocks/<file>:<line>.
 */
#ifndef SHOCKS_H
#define SHOCKS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
typedef enum {
    SHK_OK = 0,
    SHK_EINVAL = 1,       /* bad argument (the reference raises ValueError)          */
    SHK_ENONFINITE = 2,   /* "Time step is not finite" (timestepping.py:144-145)     */
    SHK_ETIMEOUT = 3,     /* a bounded device-side wait expired                     */
    SHK_ECUDA = 4,        /* a CUDA runtime call failed                              */
    SHK_ENOMEM = 5,       /* allocation failed (plan creation only)                  */
    SHK_EUNSUPPORTED = 6, /* combination not implemented                             */
    SHK_ETOOLARGE = 7     /* size beyond the static scratch of a no-allocation call  */
} shk_status;

/* numerical flux (burgers/schemes.py:71-96,98-153,160-196,205-256);
 * SHK_FLUX_GODUNOV (upwind, scalar.py:91-132) and SHK_FLUX_EO (Engquist-Osher,
 * scalar.py:287-322, omega = 0) are Burgers fluxes */
enum { SHK_FLUX_RUSANOV = 0, SHK_FLUX_LF = 1, SHK_FLUX_ESWENO = 2, SHK_FLUX_GODUNOV = 3,
       SHK_FLUX_EO = 4 };
/* reconstruction (reconstruction.py:128-163,320-348,386-439); SHK_REC_LEARNED:
 * learned WENO weights (an MLP over the normalised stencil) */
enum { SHK_REC_WENOJS53 = 0, SHK_REC_ESWENO32 = 1, SHK_REC_LEARNED = 2, SHK_REC_CONSTANT = 3,
       SHK_REC_WENOJS32 = 4, SHK_REC_MUSCL = 5, SHK_REC_MUSCLS = 6 };
/* limiters of SHK_REC_MUSCL (flux limiter, reconstruction.py:172-245) and
 * SHK_REC_MUSCLS (slope limiter, :248-290), limiters.py:133-407; Koren has no
 * slope form */
enum { SHK_LIM_NONE = 0, SHK_LIM_MINMOD = 1, SHK_LIM_MC = 2, SHK_LIM_SUPERBEE = 3,
       SHK_LIM_VANALBADA = 4, SHK_LIM_VANLEER = 5, SHK_LIM_KOREN = 6 };
/* physical flux f(u) and wave speed f'(u) */
enum { SHK_EQ_BURGERS = 0, SHK_EQ_ADVECTION = 1, SHK_EQ_LWR = 2 };
/* state precision */
enum { SHK_F64 = 0, SHK_F32 = 1 };

/* A scheme on the hot path: the fields of the reference's frozen dataclasses
 * Rusanov(rec, alpha) / LaxFriedrichs / ESWENO32 and WENOJS53(eps) /
 * ESWENO32(eps, delta) (reconstruction.py:335-348,386-411). */
typedef struct {
    int32_t flux;      /* SHK_FLUX_*                                         */
    int32_t rec;       /* SHK_REC_*                                          */
    int32_t equation;  /* SHK_EQ_*                                           */
    int32_t limiter;   /* SHK_REC_MUSCL / MUSCLS: SHK_LIM_* (its theta or van
                        * Albada variant in delta, the slope-ratio cut atol in eps) */
    double eps;        /* WENO epsilon (WENOJS53 default 1e-12; the bench's 1e-6) */
    double delta;      /* ES-WENO delta (bound to dx^2 by burgers bind)       */
    double nu;         /* Rusanov artificial viscosity dx^(alpha-1); 1 if alpha=1 */
    double speed;      /* linear advection velocity (SHK_EQ_ADVECTION)        */
    const float* mlp;  /* SHK_REC_LEARNED: 1347 float32 parameters (device)    */
    float tau;         /* SHK_REC_LEARNED: JS weight marking a non-smooth sub-stencil */
    float band;        /* SHK_REC_LEARNED: max network weight on such sub-stencils */
    float dev;         /* SHK_REC_LEARNED: max |omega - omega_JS| per sub-stencil
                        * (>= 1: no cap)                                        */
    float norm_eps;    /* SHK_REC_LEARNED: floor of the stencil range in the network's
                        * input normalisation (s - mean) / (range + norm_eps); <= 0
                        * means 1e-12 */
} shk_scheme;

/* Boundary conditions (scalar.py:397-540). Periodic is the default of every
 * entry point. Dirichlet sets the 3 ghost cells of a side to g_d(t, x) at
 * their centres (scalar.py:419-429); Neumann mirrors the interior about the
 * boundary face, ghost k = u_mirror - (2k + 1) dx g_n(t) (scalar.py:469-495).
 * The boundary is applied before every operator evaluation, at the stage
 * times of the call: t for apply_operator; t, t + dt, t + dt/2 for an SSPRK33
 * step (timestepping.py:312-320 via schemes.py:339-346). */
enum { SHK_BC_PERIODIC = 0, SHK_BC_DIRICHLET = 1, SHK_BC_NEUMANN = 2 };
typedef struct {
    int32_t left, right;        /* SHK_BC_* of each side (periodic: both or neither) */
    double dirichlet[3][2][3];  /* g_d(t_s, x) [stage][side 0 left / 1 right][k], k = 0
                                 * the ghost next to the interior */
    double neumann[3][2];       /* g_n(t_s) [stage][side] */
} shk_boundary;

const char* shk_strerror(int status);
int shk_version(void);

/* ---- single-instance drop-ins (reference ghosted layout, n + 2g cells) -- */

/* max over the n interior cells of |f'(u)| into *amax (device double).
 * Needed by SHK_FLUX_LF (scalar.py:258-278) and by predict_timestep. */
int shk_max_wavespeed_f64(const shk_scheme* scheme, const double* u, int64_t n,
                          int32_t nghosts, double* amax, void* stream);

/* apply_operator (schemes.py:339-346 after scalar.py:529-540 periodic ghost
 * fill): out[g:n+g] = -(F[i+1/2]-F[i-1/2])/dx. Output ghost cells receive the
 * periodic image of the interior output. `amax` (device) is read for
 * SHK_FLUX_LF only (from shk_max_wavespeed_f64 on the same u); may be NULL
 * otherwise. u and out must not overlap. */
int shk_apply_operator_f64(const shk_scheme* scheme, const double* u, double* out,
                           int64_t n, int32_t nghosts, double dx, const double* amax,
                           void* stream);

/* predict_timestep with the driver's theta (burgers/schemes.py:121-127,
 * examples/burgers.py:161-162): *dt = theta * (cfl / max|f'(u_interior)|),
 * cfl = 0.5 * dx^(2 - alpha) computed by the caller. *dt is device memory. */
int shk_predict_timestep_f64(const shk_scheme* scheme, const double* u, int64_t n,
                             int32_t nghosts, double cfl, double theta, double* dt,
                             void* stream);

/* one SSPRK33 step (timestepping.py:312-320, advance() of timestepping.py:218-233)
 * of a ghosted single instance: u_out = advance(u) with the three stages fused
 * in one kernel; output ghosts receive the periodic image. */
int shk_ssprk33_step_f64(const shk_scheme* scheme, const double* u, double* u_out,
                         int64_t n, int32_t nghosts, double dx, double dt,
                         void* stream);

/* shk_apply_operator_f64 / shk_ssprk33_step_f64 with the boundary `bc`
 * (NULL: periodic) at the stage time(s) of the call. Output ghost cells:
 * apply_operator writes 0 there (the reference's values are unspecified and
 * overwritten by its next apply_boundary); the step writes the boundary at
 * t + dt (stage 1 data). */
int shk_apply_operator_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                              double* out, int64_t n, int32_t nghosts, double dx,
                              const double* amax, void* stream);
int shk_ssprk33_step_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                            double* u_out, int64_t n, int32_t nghosts, double dx, double dt,
                            void* stream);

/* ---- batched plans ----------------------------------------------------- */

/* A plan owns the device scratch of a batch: per-instance wave-speed maxima,
 * time, dt history, status word, the (instance, tile) work list, the step
 * counter and (optionally) a captured CUDA graph. Created once; every
 * per-step call allocates nothing. Layout of the state buffers it steps:
 * instance b occupies cells [h_offsets[b], h_offsets[b+1]) of a packed
 * buffer (interior cells only; periodic wrap is done by the kernels).
 * Instances whose start and length are multiples of 16 bytes are staged by
 * TMA bulk copies, others by plain loads. */
typedef struct shk_plan shk_plan;

typedef struct {
    int32_t dtype;        /* SHK_F64 / SHK_F32                                  */
    int32_t tile;         /* cells per work item (0 = the library's choice for the
                           * scheme, precision and max_steps; at least 512 with
                           * the learned reconstruction)                         */
    int32_t max_steps;    /* capacity of the dt history (0 = no history)        */
    int32_t ctas_per_sm;  /* persistent grid size per SM (0 = occupancy)         */
} shk_plan_opts;

int shk_plan_create(const shk_scheme* scheme, int32_t batch, const int64_t* h_offsets,
                    const double* h_dx, const double* h_cfl, double theta,
                    const shk_plan_opts* opts, shk_plan** out);
int shk_plan_destroy(shk_plan* plan);

/* reset the batch at time t0 (device, B doubles) with final times tfinal
 * (device, B doubles; DBL_MAX = no final time, as step() with tfinal=None,
 * timestepping.py:114-116) and prime the wave-speed maxima from u. */
int shk_plan_reset(shk_plan* plan, const void* u, const double* t0, const double* tfinal,
                   void* stream);

/* advance every active instance by `nsteps` SSPRK33 steps (the step() loop of
 * timestepping.py:128-152 with the CFL dt of burgers/schemes.py:121-127 and the
 * final-time clip + 1e-15 of timestepping.py:139-142), ping-ponging between
 * u_a and u_b (caller-owned, same layout). Step k reads the buffer holding
 * the current state; after an even number of total steps since reset the
 * state is in u_a, after an odd number in u_b. An instance with t >= tfinal is
 * copied through unchanged; a non-finite dt sets SHK_ENONFINITE in the status
 * word and freezes that instance. */
int shk_plan_step(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps, void* stream);

/* prescribe the time steps: step k of instance b takes dt[k * B + b] (dt:
 * nsteps x B doubles, device or host memory, copied into the plan on
 * `stream`) instead of the CFL step, as a stepper whose predict_timestep
 * returns a fixed step (timestepping.py:242-260, predict_timestep_from_maxit /
 * predict_maxit_from_timestep). A step <= 0, and every step past the table,
 * leaves the instance unchanged; tfinal is not consulted, so a recorded dt
 * history (shk_plan_copy_dt_history) replays exactly. nsteps = 0 returns to
 * CFL steps. Drops a captured step graph. */
int shk_plan_set_fixed_dt(shk_plan* plan, const double* dt, int32_t nsteps, void* stream);

/* time-independent Dirichlet / Neumann boundaries for every instance of the
 * plan: dirichlet [B][2][3] ghost values, neumann [B][2] gradients (device or
 * host memory, copied on `stream`; either may be NULL if no side uses it).
 * left = right = SHK_BC_PERIODIC restores periodic instances; the adjoint of
 * such a plan is the exact transpose with the boundary data as constants.
 * Drops a captured step graph. */
int shk_plan_set_boundary(shk_plan* plan, int32_t left, int32_t right, const double* dirichlet,
                          const double* neumann, void* stream);

/* time-dependent boundary data (the g(t, x) of scalar.py:397-511 at the stage
 * times t, t + dt, t + dt/2 of each step): dirichlet [nsteps][3][B][2][3],
 * neumann [nsteps][3][B][2] (device or host memory, copied on `stream`);
 * step k >= nsteps takes row nsteps - 1. The caller evaluates the data at its
 * stage times, so the tables go with prescribed steps (shk_plan_set_fixed_dt).
 * Drops a captured step graph. */
int shk_plan_set_boundary_steps(shk_plan* plan, int32_t left, int32_t right,
                                const double* dirichlet, const double* neumann, int32_t nsteps,
                                void* stream);

/* capture two steps (u_a -> u_b -> u_a) into a CUDA graph and replay it
 * nsteps/2 times (nsteps must be even). */
int shk_plan_step_graph(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps,
                        void* stream);

/* device pointers to the plan's per-instance time [B] and dt history
 * [max_steps][B] (double), and the number of steps taken since reset. */
int shk_plan_state(shk_plan* plan, double** t, double** dt_hist, int64_t** step_counter);

/* device-to-device copies of the per-instance time [B] and of the whole dt
 * history [max_steps][B] into caller buffers. */
int shk_plan_copy_time(shk_plan* plan, double* t_out, void* stream);
int shk_plan_copy_dt_history(shk_plan* plan, double* out, void* stream);

/* copy the device status word to *h_status (synchronises `stream`). */
int shk_plan_status(shk_plan* plan, int32_t* h_status, void* stream);

/* ---- host-resident batches ---------------------------------------------- */

/* A batch whose state lives in host memory, as the reference's arrays do (the
 * step() loop of timestepping.py:89-152 runs on numpy / JAX CPU arrays). The
 * stepper splits the batch by instance into `nchunks` chunks of about equal
 * cell counts (0: one per 512 Ki cells, at most 32; never more than one per
 * instance), each with its own plan and device buffers, and
 * pipelines them: host-to-device copy of chunk c+1 and device-to-host copy of
 * chunk c-1 overlap the steps of chunk c. Arguments as shk_plan_create
 * (opts->max_steps must be 0: forward only). */
typedef struct shk_host_stepper shk_host_stepper;

int shk_host_stepper_create(const shk_scheme* scheme, int32_t batch, const int64_t* h_offsets,
                            const double* h_dx, const double* h_cfl, double theta,
                            const shk_plan_opts* opts, int32_t nchunks, shk_host_stepper** out);
int shk_host_stepper_destroy(shk_host_stepper* hs);
/* number of chunks actually used (at most the number of instances) */
int shk_host_stepper_num_chunks(const shk_host_stepper* hs);

/* h_out = the packed host state h_in (plan layout, double or float as the
 * opts' dtype) advanced by `nsteps` SSPRK33 CFL steps from t = 0 with no final
 * time: the same kernels, dt and result, bit for bit, as shk_plan_reset +
 * shk_plan_step over the whole batch. h_in may equal h_out. Asynchronous with
 * respect to the host: the results are in h_out once `stream` has reached
 * the point of the call. Overlap needs pinned host buffers (cudaHostAlloc or
 * cudaHostRegister). */
int shk_host_stepper_advance(shk_host_stepper* hs, const void* h_in, void* h_out, int32_t nsteps,
                             void* stream);

/* shk_plan_set_boundary for every chunk: dirichlet [B][2][3], neumann [B][2]
 * over the whole batch (device or host memory) */
int shk_host_stepper_set_boundary(shk_host_stepper* hs, int32_t left, int32_t right,
                                  const double* dirichlet, const double* neumann, void* stream);

/* OR of the chunks' status words (synchronises `stream`) */
int shk_host_stepper_status(shk_host_stepper* hs, int32_t* h_status, void* stream);

/* ---- discrete adjoint (dt frozen, as adjoint_step: timestepping.py:155-215) -- */

/* p_out = (d advance(u) / d u)^T p_next for one SSPRK33 step of a ghosted single
 * instance (the `jac.T @ p` of timestepping.py:205-206, matrix-free). Rusanov +
 * WENO-JS53 only. Cotangents live on interior cells: ghost entries of p_next
 * are ignored and those of p_out are set to zero. */
int shk_ssprk33_vjp_f64(const shk_scheme* scheme, const double* u, const double* p_next,
                        double* p_out, int64_t n, int32_t nghosts, double dx, double dt,
                        void* stream);

/* shk_ssprk33_vjp_f64 for a step taken with a Dirichlet / Neumann boundary
 * (shk_ssprk33_step_bc_f64 with the same `bc`): the exact transpose, the
 * boundary's data entering as constants (NULL: periodic). */
int shk_ssprk33_vjp_bc_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                           const double* p_next, double* p_out, int64_t n, int32_t nghosts,
                           double dx, double dt, void* stream);

/* forward run of `nsteps` steps (as shk_plan_step) that also copies the state
 * before every step k with k % stride == 0 into ckpt[k / stride] (caller-owned,
 * ceil(nsteps/stride) packed states). The plan needs max_steps >= nsteps: the
 * dt history is the frozen dt of the adjoint (timestepping.py:200-201). */
int shk_plan_forward_checkpointed(shk_plan* plan, void* u_a, void* u_b, int32_t nsteps,
                                  void* ckpt, int32_t stride, void* stream);

/* reverse sweep of the last checkpointed forward run: p_a holds dJ/du(T) on
 * entry; after the call dJ/du(0) is in p_a if nsteps is even, else in p_b.
 * Segments of `stride` steps are recomputed from the checkpoints into `seg`
 * (caller-owned, stride packed states) with the recorded dt, then stepped
 * backwards (sqrt(nsteps) checkpointing when stride ~ sqrt(nsteps)). Rusanov +
 * WENO-JS53 only. */
/* SHK_EUNSUPPORTED when the plan's tile is too long for the reverse step's
 * shared memory (about 1140 cells in float64, 2500 in float64 with the learned
 * reconstruction, 2300 in float32). */
int shk_plan_adjoint(shk_plan* plan, const void* ckpt, int32_t stride, int32_t nsteps,
                     void* seg, void* p_a, void* p_b, void* stream);

/* shk_plan_adjoint with stage storage: the segment replay also writes what
 * each step's reverse step would recompute, and the reverse steps read it:
 * the stage states k1, k2 (float, learned reconstruction) or k1, k2 and the
 * face values of u, k1 and k2 (double, WENO-JS5 on periodic instances). `stages`
 * is caller-owned, stride x *nbytes bytes, *nbytes from
 * shk_plan_adjoint_stage_bytes (0: the plan recomputes; `stages` must then be
 * NULL). Same result, bit for bit, as shk_plan_adjoint. */
int shk_plan_adjoint_stage_bytes(shk_plan* plan, int64_t* nbytes);
int shk_plan_adjoint_staged(shk_plan* plan, const void* ckpt, int32_t stride, int32_t nsteps,
                            void* seg, void* stages, void* p_a, void* p_b, void* stream);

/* FP64 reductions over the batch (grid.py:444-506, conservation checks):
 * out[b] = sum_i u_b[i] (p = 0), sum |u_b[i]| (p = 1), sum u_b[i]^2 (p = 2) or
 * max |u_b[i]| (p = -1), accumulated in double for either state precision, in
 * a fixed order (deterministic for a given plan). */
int shk_plan_reduce(shk_plan* plan, const void* u, int32_t p, double* out, void* stream);

/* ---- the reference's ghosted step, forward and exact transpose ---------- */

/* Single instance on the reference's ghosted array of n + 2 nghosts cells, with
 * the reference's own arithmetic on the whole array: every operator evaluation
 * fills the ghosts by the boundary at its stage time (scalar.py:397-540), the
 * reconstruction sees zeros beyond the array ends (the zero-padded "same"
 * convolutions of convolve.py:113-114), the fluxes at the two array ends are
 * zero (scalar.py:249), and the ghost cells have outputs. Schemes: Rusanov
 * (any alpha, via nu) or global Lax-Friedrichs (scalar.py:258-278: the wave
 * speed is the maximum of |f'| over the whole filled array) with the
 * constant or WENO-JS5 reconstruction; Burgers, advection or LWR. nghosts >=
 * the reconstruction's stencil width (1 constant, 3 WENO-JS5), and <= 3 with a
 * Dirichlet / Neumann boundary. `workspace` is caller device memory of at
 * least shk_ghosted_workspace_bytes(n, nghosts) bytes (256-byte aligned
 * inside); nothing is allocated. */
int64_t shk_ghosted_workspace_bytes(int64_t n, int32_t nghosts);

/* apply_operator (schemes.py:339-346) on every cell, ghosts included. */
int shk_apply_operator_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                   double* out, int64_t n, int32_t nghosts, double dx, void* workspace,
                                   int64_t workspace_bytes, void* stream);

/* advance() of SSPRK33 (timestepping.py:312-320) on the raw ghosted array:
 * u_out = 1/3 u + 2/3 (k2 + dt L(k2)) on every cell, the ghosts included (the
 * raw ghost values pass through), with the boundary at t, t + dt, t + dt/2. */
int shk_ssprk33_step_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                 double* u_out, int64_t n, int32_t nghosts, double dx, double dt,
                                 void* workspace, int64_t workspace_bytes, void* stream);

/* p_out = J^T p_next with J the Jacobian of that step with respect to the whole
 * ghosted u (dt frozen): the `jac.T @ p` of adjoint_step (timestepping.py:174,
 * 205-206), matrix-free. Ghost entries of p_next reach the interior through
 * the operator's ghost rows; ghost entries of p_out are the pass-through
 * (= p_next's, the raw ghost inputs of L being overwritten by the boundary).
 * max() and |.| follow JAX's tie conventions (an even split). */
int shk_ssprk33_vjp_ghosted_f64(const shk_scheme* scheme, const shk_boundary* bc, const double* u,
                                const double* p_next, double* p_out, int64_t n, int32_t nghosts,
                                double dx, double dt, void* workspace, int64_t workspace_bytes,
                                void* stream);

/* ---- no-allocation variant --------------------------------------------- */

/* Lax-Friedrichs apply_operator for callers that cannot allocate device
 * memory. No counterpart in the reference. Same inputs, outputs and result as
 * shk_max_wavespeed_f64 followed by shk_apply_operator_f64 with
 * SHK_FLUX_LF, but the wave-speed scratch is a fixed array inside the library
 * instead of caller memory, so the call allocates nothing. Meant for hosts
 * that own the whole device memory pool, e.g. a JAX custom-call handler
 * (JAX preallocates most of the GPU and gives the handler only its operand
 * buffers).
 *  - n is limited to shk_apply_operator_lf_noalloc_max_cells() interior cells
 *    (2,097,152); larger n returns SHK_ETOOLARGE before any launch.
 *  - The first call in each CUDA context looks up the scratch address there
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *    The address is kept per context (by its cuCtxGetId), so a context created
 *    after cudaDeviceReset gets its own lookup instead of a stale address.
 *  - The scratch (32 KiB per GPU, held from library load to process exit) is
 *    shared by all calls and keeps the last call's contents; every slot a call
 *    reads is written by that call first. Calls that overlap on the GPU race on
 *    it: serialise them (one stream, or events between streams). */
int shk_apply_operator_lf_noalloc_f64(const shk_scheme* scheme, const double* u,
                                      double* out, int64_t n, int32_t nghosts, double dx,
                                      void* stream);
int64_t shk_apply_operator_lf_noalloc_max_cells(void);

/* ---- learned WENO weights: training (no reference counterpart) ---------- */

/* number of MLP parameters (1347) and the workspace a batch of n samples needs */
int shk_mlp_num_params(void);
int64_t shk_mlp_workspace_bytes(int64_t n);

/* loss 1/(2n) sum_i sum_{F = R, L} [w_i (face_F,i - target_F,i)^2
 *                                  + reg |omega_F,i - d|^2]
 * of the raw network over n cells: stencils n x 5 float32 (v_{c-2..c+2}),
 * target n x 2 (right, left face), weight n; d the WENO-JS5 ideal weights. One
 * network output z per cell gives omega_R = softmax(z) and omega_L =
 * softmax(z2 - ln 3, z1, z0 + ln 3). Also the gradient w.r.t. the parameters
 * (fp32 forward/backward, deterministic reduction); norm_eps as in
 * shk_scheme. *loss is device memory (double). */
int shk_mlp_loss_grad_f32(const float* params, const float* stencils, const float* target,
                          const float* weight, int64_t n, float reg, float norm_eps,
                          float* grad, double* loss, void* workspace, int64_t workspace_bytes,
                          void* stream);

/* one Adam step on the parameters (step >= 1 for the bias corrections) */
int shk_mlp_adam_f32(float* params, const float* grad, float* m, float* v, float lr,
                     float beta1, float beta2, float eps, int32_t step, void* stream);

/* learned face values (right, left: out is n x 2) of n cell stencils (n x 5,
 * v_{c-2..c+2}) with the tensor-core inference and the per-face WENO-JS trust
 * band of the flux kernel (scheme->mlp, eps, tau, band, dev) */
int shk_learned_faces_f32(const shk_scheme* scheme, const float* stencils, float* out,
                          int64_t n, void* stream);

/* ---- measurement ------------------------------------------------------- */

/* peak FMA throughput of the FP64 (dtype SHK_F64) or FP32 (SHK_F32) pipe of
 * the current device in flop/s (2 per FMA), from independent FMA chains on
 * every SM timed with CUDA events (synchronous; allocates a small buffer).
 * No reference counterpart: it is the roofline denominator of the FP64-bound
 * kernels. */
int shk_measure_fp_peak(int32_t dtype, int32_t iters, double* flops_per_s);

#ifdef __cplusplus
}
#endif

#endif /* SHOCKS_H */
