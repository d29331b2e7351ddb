/*
 * swampe_gb300.h -- C ABI of the GB300 time-stepping core for SWAMPE-JAX.
 *
 * The reference (imalsky/MY_SWAMPE, package my_swampe) is pure Python/JAX and
 * has no foreign-function interface; its device boundary is the jitted
 * lax.scan call inside run_model_scan (src/my_swampe/model.py:1715-1758).
 * Each entry point below replaces one piece of the path behind that call and
 * cites the reference function it stands for.  The Python package
 * my_swampe_gb300 binds these symbols with ctypes and keeps the reference's
 * run_model / run_model_scan / run_model_scan_final signatures on top.
 *
 * Conventions
 *   - Every function returns an int status: SWP_OK (0) or an SWP_ERR_* code.
 *     Nothing throws or aborts across the ABI; swp_last_error() returns the
 *     message of the last failure on that plan.
 *   - All arrays are device pointers owned by the caller; the plan owns only
 *     static geometry and scratch.  `stream` is a cudaStream_t (NULL = legacy).
 *   - Complex (Fourier) arrays -- fourier, lam, lam_y, tangent fourier, stored
 *     states, window slots -- must be 16-byte aligned (cudaMalloc and torch
 *     allocations are): the kernels move them with 16-byte accesses.  An
 *     entry point refuses a misaligned one with SWP_ERR_ARG.
 *   - A plan is not re-entrant: one host thread and one stream per plan.
 *   - Precision SWP_FP64: every array of "compute type" is double/double2.
 *     Precision SWP_FAST: compute type is float/float2 (FP32 state, FP32
 *     pointwise math; Legendre contractions in split precision on the
 *     tensor cores where available).  Geometry is always built in FP64.
 *
 * Memory layout of one truncation group (M, J, I, B members):
 *   fourier : complex[SWP_NFOURIER][M+1][B][J]   (field, zonal wavenumber m, member, latitude)
 *             fields: eta_prev, eta, delta_prev, delta, Phi_prev, Phi, U, V, A, B, C, D,
 *             E, PhiF, F, G, eta_mid, delta_mid, Phi_mid.  The *_mid carries are the
 *             Robert-Asselin-filtered lineage (the physical prev level, and the n-1
 *             base of the semi-implicit scheme).  The semi-implicit scheme never
 *             reads the unfiltered prev carries; it keeps its lagged momentum-forcing
 *             remainders Rum_lag, Rvm_lag in the eta_prev, delta_prev slots.
 *   resid   : real[5][B][J][I]   initial condition minus its band-limited part
 *   params  : double[SWP_NPAR][B]  (dt, a, omega, Phibar, taurad, taudrag, DPhieq,
 *             K6, K6Phi, RA alpha, semi-implicit si_alpha, RAW williams_alpha)
 *   member  : double[4][B]       (w_curr, w_mid, dead, updated)
 *   diag    : double[nsteps+1][5][B]  (rms^2-sum, min |u|, min Phi, max Phi, dead)
 *   hist    : real[nsteps][5][B][J][I]  (eta, delta, Phi, U, V)
 */
#ifndef SWAMPE_GB300_H
#define SWAMPE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SWP_OK 0
#define SWP_ERR_ARG 1
#define SWP_ERR_CUDA 2
#define SWP_ERR_NUMERIC 3
#define SWP_ERR_STATE 4
#define SWP_ERR_UNSUPPORTED 5

#define SWP_FP64 0
#define SWP_FAST 1

#define SWP_NFOURIER 19
#define SWP_NPAR 12
#define SWP_MAX_GROUPS 4
/* Size of the fixed device scratch used by swp_adjoint_step_noalloc (16 MiB). */
#define SWP_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)

typedef struct swp_plan swp_plan;

/* Per-group device buffers (see layout above).  Unused pointers may be NULL. */
typedef struct {
  void* fourier;
  void* resid;
  const double* params;
  double* member;
  double* diag;
  void* hist;
} swp_group_state;

/* Adjoint buffers of one group. */
typedef struct {
  void* lam;          /* complex[SWP_NFOURIER][M+1][B][J]: adjoint of the Fourier state */
  void* lam_y;        /* complex[5][M+1][B][J]: scratch for the adjoint of the step outputs */
  double* grad;       /* double[4][B]: d/d(taurad, taudrag, DPhieq, Phibar), accumulated */
} swp_group_adjoint;

/* Tangent-linear (forward-mode) buffers of one group. */
#define SWP_NTANGENT 12
typedef struct {
  void* fourier;          /* complex[SWP_NFOURIER][M+1][B][J]: tangent of the Fourier state */
  void* resid;            /* real[5][B][J][I]: tangent of the initial-condition residual     */
  const double* dparams;  /* double[SWP_NTANGENT][B]: tangents of taurad, taudrag, DPhieq,
                             Phibar, a, dt, K6, K6Phi, omega, si_alpha, alpha (the
                             Robert-Asselin coefficient), williams_alpha (RAW filter)      */
  int coef_tangents;      /* nonzero when rows a..williams_alpha may be nonzero: the step
                             then also differentiates its coefficient tables (one more
                             Legendre pass; always taken by the semi-implicit scheme) and
                             its filter weights (the primal Legendre step then runs on the
                             SIMT kernel and adds the weights' tangents times its
                             displacement to the tangent carries)                         */
  double* dweights;       /* double[2][B]: tangents of the residual weights w_curr, w_mid
                             (member[0..1] of the state), kept by the library             */
} swp_group_tangent;

/* Flags of model.py RunFlags (model.py:156-226) plus the test selector. */
typedef struct {
  int scheme;       /* 0 = modified Euler (default), 1 = explicit (expflag),
                       2 = semi-implicit leapfrog (semi_implicit=True; forward only) */
  int forcflag;
  int diffflag;
  int modalflag;
  int test;         /* 0 = forced (test=None), 1, 2                           */
  int diagnostics;  /* RMS blow-up gate and per-step diagnostics              */
  double blowup;    /* RunFlags.blowup_rms                                     */
  int t_start;      /* time index of the initial state (the run's starttime); in the
                       SWP_FAST precision the steps after the first one advance the
                       band-limited state by increments (see swp_forward)       */
  int raw_filter;   /* Robert-Asselin-Williams filter (RunFlags.raw_filter), weight
                       williams_alpha = params row 11; forward only               */
} swp_flags;

/* Create a plan for `ngroups` truncations (M[g] in {42, 63, 106}) with B[g]
 * members each; builds Gauss nodes, Legendre bases and FFT twiddles on the
 * device in FP64.  Replaces build_static/_cached_geometry (model.py:62-86,
 * 457-557) and spectral_transform.PmnHmn / gauss_legendre. */
int swp_plan_create(int ngroups, const int* M, const int* B, int precision, swp_plan** out);
int swp_plan_destroy(swp_plan* plan);
/* Grid sizes of group g (initial_conditions.spectral_params, initial_conditions.py:50-85). */
int swp_plan_dims(const swp_plan* plan, int g, int* M, int* J, int* I, int* B);
/* Message of the last failure on this plan (empty string if none). */
const char* swp_last_error(const swp_plan* plan);
/* FP64 copies of mus, w (J each) and dense Pmn, Hmn (J, M+1, M+1) for group g
 * (spectral_transform.py:80-114, 219-287).  Any pointer may be NULL. */
int swp_geometry(const swp_plan* plan, int g, double* mus, double* w, double* Pmn, double* Hmn, void* stream);

/* Two-level initial state from physical fields phys_ic[g] = real[5][B][J][I]
 * (eta, delta, Phi, U, V); fills fourier, resid and diag row 0.
 * Replaces _init_state_from_fields (model.py:694-772). */
int swp_init_state(swp_plan* plan, const swp_group_state* st, void* const* phys_ic,
                   const swp_flags* flags, void* stream);

/* Winds diagnosed from eta, delta (model.py:644-666): phys_ed[g] = real[2][B][J][I]
 * in, phys_uv[g] = real[2][B][J][I] out.  Uses st[g].fourier as scratch. */
int swp_diagnose_winds(swp_plan* plan, const swp_group_state* st, void* const* phys_ed,
                       void* const* phys_uv, void* stream);

/* Advance every group by `nsteps` steps starting at absolute time index t0
 * (the body of lax.scan over t_seq = arange(t0, t0 + nsteps), model.py:795-1194,
 * 1237-1342).  diag/hist rows are indexed from `row0`.  write_prev_last copies
 * the Fourier curr carry into the prev carry on the last step (always done for
 * the explicit scheme, which reads it).  SWP_FAST, modified Euler, t > t_start:
 * the state is band-limited, so the step is evaluated as curr + Inv(dc) with
 * dc = (sigma-1) Fwd(curr) + sigma (tendency) -- algebraically the reference's
 * Inv(sigma Fwd(curr + ...)), but the FP32 transform error then scales with
 * the increment instead of the field. */
int swp_forward(swp_plan* plan, const swp_group_state* st, const swp_flags* flags,
                int t0, int nsteps, int row0, int write_prev_last, void* stream);

/* swp_forward over [t0, t0+nsteps) that first copies the state at
 * t0 + w*ckpt_every into slot w of ckpt[g] (ceil(nsteps/ckpt_every)
 * contiguous Fourier states) -- the forward sweep of a checkpointed
 * differentiable run (diagnostics off).  Captured once into a CUDA graph per
 * argument set and replayed. */
int swp_forward_checkpointed(swp_plan* plan, const swp_group_state* st, const swp_flags* flags,
                             int t0, int nsteps, int ckpt_every, void* const* ckpt, void* stream);

/* Physical curr and RA-filtered prev fields: phys_out[g] = real[8][B][J][I]
 * (eta, delta, Phi, U, V, eta_prev, delta_prev, Phi_prev) -- the physical
 * members of the reference State (model.py:380-425). */
int swp_output_physical(swp_plan* plan, const swp_group_state* st, void* const* phys_out,
                        const swp_flags* flags, void* stream);

/* Copy of the whole Fourier state of every group into/out of `ckpt[g]`
 * (same layout as st[g].fourier).  dir = 0: state -> ckpt, 1: ckpt -> state. */
int swp_state_copy(swp_plan* plan, const swp_group_state* st, void* const* ckpt, int dir, void* stream);

/* Adjoint of one step t (modified Euler, explicit or semi-implicit leapfrog,
 * forced or unforced, diagnostics off; the RAW filter is SWP_ERR_UNSUPPORTED).
 * The semi-implicit step propagates the state's adjoint only: its parameter
 * gradients are not accumulated (take them from tangent runs).
 * On entry adj[g].lam holds the adjoint of the state after the step; primal
 * st_in[g] is the state before the step and st_out[g] the state after it.
 * On exit adj[g].lam holds the adjoint of the state before the step and
 * adj[g].grad has accumulated the parameter gradients of the step. */
int swp_adjoint_step(swp_plan* plan, const swp_group_state* st_in, const swp_group_state* st_out,
                     const swp_group_adjoint* adj, const swp_flags* flags, int t, void* stream);

/* Seed the adjoint from gradients of the physical curr fields
 * dphys[g] = real[5][B][J][I] (eta, delta, Phi, U, V): adj[g].lam is overwritten. */
int swp_adjoint_seed(swp_plan* plan, const swp_group_state* st, const swp_group_adjoint* adj,
                     void* const* dphys, void* stream);

/* Adjoint of swp_init_state: gradients of the physical initial fields
 * dic[g] = real[5][B][J][I] (eta, delta, Phi, U, V) from adj[g].lam; accumulates
 * parameter gradients of the initial forcing into adj[g].grad. */
int swp_adjoint_init(swp_plan* plan, const swp_group_state* st, const swp_group_adjoint* adj,
                     void* const* phys_ic, void* const* dic, const swp_flags* flags, void* stream);

/* Adjoint of one checkpoint window [t0, t0+nsteps): restores st[g].fourier
 * (the window's checkpoint) into slot 0 of slots[g] (nsteps+1 contiguous
 * Fourier states), recomputes the window out of place keeping every state,
 * then runs the adjoint steps backwards.  adj[g].lam: adjoint of the state at
 * t0+nsteps on entry, at t0 on exit; adj[g].grad accumulates.  The sequence
 * is captured once into a CUDA graph per (window length, buffers) and replayed.
 * Replaces reverse-mode jax.grad through lax.scan with jax.checkpoint per step
 * (model.py:1330-1334). */
int swp_adjoint_window(swp_plan* plan, const swp_group_state* st, void* const* slots,
                       const swp_group_adjoint* adj, const swp_flags* flags, int t0, int nsteps, void* stream);

/* swp_forward over [t0, t0+nsteps) that keeps every state: states[g] holds
 * nsteps+1 contiguous Fourier states (slot 0 <- st[g].fourier, slot k <- the
 * state after k steps); the final state is also copied back into st[g].fourier.
 * The forward sweep of a differentiable run when the whole trajectory fits in
 * device memory (at B=256, M=42, FP32 and 1440 steps: 154 GB), so that the
 * adjoint needs no recomputation -- what jax.grad through lax.scan stores
 * without remat (model.py:1237-1342).  Diagnostics off.  Captured once into a
 * CUDA graph per argument set and replayed. */
int swp_forward_stored(swp_plan* plan, const swp_group_state* st, const swp_flags* flags,
                       int t0, int nsteps, void* const* states, void* stream);

/* Adjoint of the steps t0+nsteps-1 down to t0 over the states kept by
 * swp_forward_stored (no recomputation).  adj[g].lam: adjoint of the state at
 * t0+nsteps on entry, at t0 on exit; adj[g].grad accumulates. */
int swp_adjoint_stored(swp_plan* plan, const swp_group_state* st, void* const* states,
                       const swp_group_adjoint* adj, const swp_flags* flags, int t0, int nsteps, void* stream);

/* Average device time (ms, CUDA events on `stream`) over nrep launches of the
 * step kernels on st (modified in place): ms_out[0] spectral (Legendre) kernel,
 * [1] grid kernel, and with adj != NULL [2] grid adjoint, [3] spectral adjoint.
 * Measurement hook for the roofline; no reference counterpart. */
int swp_time_kernels(swp_plan* plan, const swp_group_state* st, const swp_group_adjoint* adj,
                     const swp_flags* flags, int nrep, float* ms_out, void* stream);

/* Self-check of the tensor-core building blocks (no reference counterpart):
 * D[128, N] = A[128, K] . B[N, K]^T with tcgen05 kind::tf32 MMAs, FP32
 * accumulation in TMEM, read back with tcgen05.ld; split3 = 1 uses the
 * 3xTF32 split (hi*hi + hi*lo + lo*hi).  Device pointers, row-major FP32;
 * N in 16..256 (multiple of 16), K in 8..128 (multiple of 8).  Synchronises
 * the stream; SWP_ERR_NUMERIC if the MMA completion wait timed out. */
int swp_tc_selftest(const float* A, const float* B, float* D, int N, int K, int split3, void* stream);

/* Device status word of the plan (no reference counterpart): *status = 1 if a
 * bounded wait inside a tensor-core kernel ran out since the last call (the
 * affected step results are then invalid), else 0.  Synchronises the stream
 * and clears the word. */
int swp_device_status(swp_plan* plan, int* status, void* stream);

/* Which groups' modified-Euler steps run the tcgen05 Legendre kernels: bit g
 * set for group g (so 1 or 0 for a one-group plan).  FP32 plans use them for
 * every group (M = 42, 63, 106), unless SWP_NO_TC=1 was set when the plan was
 * created or the autotuner chose the SIMT kernel for the group.  No reference
 * counterpart. */
int swp_plan_uses_tensor_cores(const swp_plan* plan);

/* Autotuner of the plan's Legendre kernels and tile shapes (no reference
 * counterpart): for every group, the candidates are the tensor-core kernels
 * (FP32 plans: a fixed tile of 8 members) and each member tile
 * MT in {1, 2, 4, 8} (<= B) of the SIMT kernels that fits in shared memory.
 * Each is timed -- nrep launches of the step's Legendre kernel and of its
 * adjoint on the caller's buffers st / adj, which it overwrites (pass scratch
 * copies) -- and the fastest is kept for the plan's later calls (captured
 * graphs are dropped).  chosen_mt[g] (may be NULL) receives the choice: 0 for
 * the tensor-core kernels, else the SIMT tile (which the steps without a
 * tensor-core form keep using either way). */
int swp_plan_autotune(swp_plan* plan, const swp_group_state* st, const swp_group_adjoint* adj,
                      const swp_flags* flags, int nrep, int* chosen_mt, void* stream);

/* Tile shapes of group g: member tile of the SIMT Legendre kernels and
 * latitude rows per CTA of the grid step kernel. */
int swp_plan_tiles(const swp_plan* plan, int g, int* mt, int* jb);

/* Set the Legendre kernel of group g -- e.g. a previously tuned choice: mt = 1,
 * 2, 4 or 8 runs its modified-Euler steps on the SIMT kernels with that member
 * tile (SWP_ERR_ARG if it does not fit in shared memory), mt = 0 on the
 * tensor-core kernels (SWP_ERR_ARG if the group cannot run them). */
int swp_plan_set_tile(swp_plan* plan, int g, int mt);

/* Allocation-free swp_adjoint_step (no counterpart in the reference, which has
 * no C interface): identical arguments and results, except that adj[g].lam_y
 * is ignored and the step's scratch lives in a fixed device array of
 * SWP_NOALLOC_SCRATCH_BYTES (16 MiB) that every device loading the library
 * holds until exit.  For callers that cannot call cudaMalloc where they run
 * the adjoint (inside another framework's custom call or callback that owns
 * the allocator, hard-latency loops, embedded users of the C ABI).  Calls no
 * cudaMalloc/cudaFree.  The plan must need at most that much scratch
 * (5*(M+1)*B*J complex values per group, 256-byte aligned), else SWP_ERR_ARG.
 * The first call on a device resolves the array's device address
 * (cudaGetSymbolAddress) and caches it for the process -- make that first
 * call before any stream capture, and do not cudaDeviceReset that device
 * afterwards (the cached address would be stale).  All calls share the array:
 * calls that overlap on the GPU (other streams, other plans, other threads)
 * race on it.  Nothing in it needs to start at zero: each call overwrites the
 * part it reads.  The argument checks are those of swp_adjoint_step (lam_y
 * aside): a missing lam or Fourier buffer is SWP_ERR_ARG, a RAW-filtered,
 * test 1 or diagnostics run SWP_ERR_UNSUPPORTED. */
int swp_adjoint_step_noalloc(swp_plan* plan, const swp_group_state* st_in, const swp_group_state* st_out,
                             const swp_group_adjoint* adj, const swp_flags* flags, int t, void* stream);

/* Forward-mode derivative (tangent-linear model) of the run: the directional
 * derivative of the state along tangents of the physical ICs and of taurad,
 * taudrag, DPhieq, Phibar -- what jax.jvp / jax.jacfwd through run_model_scan
 * give the reference (autodiff_utils.py:27-89 fwd_grad; the retrieval's
 * forward-mode gradients), along the ICs and the per-member parameters of
 * dparams.  Modified Euler, explicit or semi-implicit scheme, classic or RAW
 * filter, diagnostics off, test 0 or 2.
 *   swp_tangent_init: after swp_init_state on the same ICs, the tangent state
 *     from dphys_ic[g] = real[5][B][J][I] (tangents of eta, delta, Phi, U, V).
 *   swp_tangent_forward: advances the primal state st and its tangent together
 *     by nsteps steps from t0 (replaces swp_forward for that window).
 *   swp_tangent_output: tangents of the physical fields of swp_output_physical. */
int swp_tangent_init(swp_plan* plan, const swp_group_state* st, const swp_group_tangent* tan,
                     void* const* phys_ic, void* const* dphys_ic, const swp_flags* flags, void* stream);
int swp_tangent_forward(swp_plan* plan, const swp_group_state* st, const swp_group_tangent* tan,
                        const swp_flags* flags, int t0, int nsteps, void* stream);
int swp_tangent_output(swp_plan* plan, const swp_group_state* st, const swp_group_tangent* tan,
                       void* const* dphys_out, const swp_flags* flags, void* stream);

/* Schedule of a plan with several groups: on = 1 runs each group's step chain
 * on its own stream, forked from and joined to the caller's stream (parallel
 * branches of the captured graphs), so that the latency-bound kernels of one
 * group overlap those of another; 0 (default) launches all groups together.
 * Splitting one ensemble into two groups of equal size and running them
 * concurrently is the faster schedule on GB300.  Results do not depend on it. */
int swp_plan_set_concurrency(swp_plan* plan, int on);

/* Poll limit of the bounded mbarrier waits inside the tensor-core kernels
 * (no reference counterpart; default SWP_WAIT_LIMIT_DEFAULT).  A test hook for
 * the failure path: with max_polls = 0 every such wait gives up at once, and
 * each CTA then sets the plan's device error word, waits (bounded, with the
 * fixed drain limit) for the copies and MMAs it issued, frees its TMEM and
 * returns without writing its outputs -- what swp_device_status then reports,
 * reached without hanging or faulting the GPU.  Captured graphs are dropped
 * when the limit changes. */
#define SWP_WAIT_LIMIT_DEFAULT (1u << 22)
int swp_plan_set_wait_limit(swp_plan* plan, unsigned int max_polls);

/* ---------------------------------------------------------------- emission
 * The retrieval's emission stage on ensembles of terminal Phi fields
 * (retrieval/scripts/pipeline.py:690-1000), FP64 like the reference's.  These
 * entries take no plan: every array is a device pointer, fields are
 * real[B][J][I] (latitude-major pixels, the model's grid), and a status of
 * SWP_ERR_ARG means a null pointer, a size below 1 or a bad configuration.
 * Non-finite inputs give all-NaN outputs per member, as the reference's guards. */
#define SWP_EMISSION_MAX_BANDS 8
typedef struct {
  int temp_mode;          /* 0 "geopotential": T = (Phibar + Phi) / R_d;
                             1 "linear": T = T_ref + Phi / phi_to_T_scale; then max(T, Tmin)
                             (pipeline.py:696-714 phi_to_temperature)                       */
  double R_d, T_ref, phi_to_T_scale, Tmin;
  int model;              /* 0 "bolometric": T^4; 1 "planck": sum_k w_k / (expm1(x_k) + 1e-30),
                             x_k = h c / (lambda_k kB T) clipped to [0, x_clip]
                             (pipeline.py:716-754 temperature_to_intensity)                 */
  int nbands;             /* planck: wavelengths used, 1..SWP_EMISSION_MAX_BANDS            */
  double wavelengths[SWP_EMISSION_MAX_BANDS];   /* m                                        */
  double band_weights[SWP_EMISSION_MAX_BANDS];  /* summing to 1 (one band: weight 1)        */
  double x_clip;
} swp_emission_cfg;

/* One pass of the emission maps per member.  input selects what `in` holds
 * (0 Phi, 1 T, 2 intensity) and stage what `out` receives (0 T, 1 intensity,
 * 2 the weighted relative intensity sqrt(w_j) I / I_mean that the projector
 * multiplies, I_mean the w-weighted mean over the finite pixels); input <= stage.
 * Phibar: double[B] (geopotential mode); w_lat: double[J] Gauss weights
 * (stage 2); ok: int[B] or NULL, set at stage 2 to whether the map passed the
 * guards of intensity_map_to_y_dense (pipeline.py:821-837). */
int swp_emission_map(const double* in, const double* Phibar, int B, int J, int I, const double* w_lat,
                     const swp_emission_cfg* cfg, int input, int stage, double* out, int* ok, void* stream);
/* y[b] = projector . rhs[b], divided by its first coefficient, all NaN unless
 * ok[b], y0 and every coefficient pass the guards (pipeline.py:838-846
 * intensity_map_to_y_dense).  projector: double[ncoef][npix], the weighted
 * ridge least-squares inverse of the Ylm design matrix (pipeline.py:808-819). */
int swp_emission_project(const double* rhs, const int* ok, int B, int npix, const double* projector, int ncoef,
                         double* y, void* stream);
/* The planet's light curve, linear in its map: lc[b][t] = amplitude[b]
 * sum_c design[t][c] y[b][c] (pipeline.py:983-994, amplitude = planet_fpfs;
 * design = the light-curve model's flux for unit coefficient vectors;
 * amplitude NULL = 1). */
int swp_phase_curve_linear(const double* y, const double* design, const double* amplitude, int B, int ncoef,
                           int ntimes, double* lc, void* stream);
/* The simplified phase-curve projection of the reference's parity test
 * (unit_tests/test_parity_reference_regression.py:67-82): flux[b][k] = sum over
 * pixels of Phi max(cos(lambda_i - phase_k), 0) sqrt(1 - mu_j^2), lambda_i =
 * -pi + 2 pi i / I, divided by mean_k |flux| when positive.  mus: double[J]. */
int swp_phase_curve_simple(const double* phi, int B, int J, int I, const double* mus, const double* phases,
                           int nphase, double* flux, void* stream);

#ifdef __cplusplus
}
#endif
#endif
