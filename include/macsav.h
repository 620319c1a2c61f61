/*
 * macsav.h -- C ABI of the GB300 (sm_103a) MAC mr-SAV stage library.
 *
 * Drop-in boundary for the no-slip MAC hot path of HaifengWang1031/MAC-mr-SAV-RK.
 * Every entry point names the reference interface it replaces (paths are
 * relative to that project's root).  Conventions:
 *   - All array arguments are DEVICE pointers to float64 data unless stated.
 *   - A "packed velocity" is the reference's free vector
 *     [u[:,1:-1].ravel(), v[1:-1,:].ravel()] of length size=(nx-1)ny+nx(ny-1)
 *     (solver/mac/grid.py:52-65); cells are (ny, nx) row-major, length np=nx*ny.
 *   - Multi-column data is column-blocked: column k starts at k*size (or k*np).
 *     (The reference stores (size, c) row-major; the Python layer transposes.)
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *     stream-ordered; entry points that return scalars synchronise the stream.
 *   - Return value: MACSAV_OK or an error code; macsav_plan_error() gives the
 *     message.  Codes map to the reference's exception types (see below).
 *   - No entry point falls back to the CPU.
 */
#ifndef MACSAV_H
#define MACSAV_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MACSAV_OK 0
#define MACSAV_ERR_VALUE 1        /* ValueError: invalid argument / RHS / shifts */
#define MACSAV_ERR_CUDA 2         /* CUDA runtime failure */
#define MACSAV_ERR_CG 3           /* RuntimeError("Pressure Schur CG failed with info=N") */
#define MACSAV_ERR_STOKES_GATE 4  /* RuntimeError("Stokes residual=..., divergence=...") */
#define MACSAV_ERR_STAGE_GATE 5   /* RuntimeError("SAV stage residuals ...") */
#define MACSAV_ERR_NEG_ENERGY 6   /* RuntimeError("Negative Stokes response energy") */
#define MACSAV_ERR_SCALAR 7       /* RuntimeError from the frozen SAV scalar map */
#define MACSAV_ERR_UNSUPPORTED 8  /* grid size outside what the plan supports */

/* precision of the Stokes solve */
#define MACSAV_FP64 0        /* FP64 throughout (parity path) */
#define MACSAV_FP32_MIXED 1  /* FP32 transforms/stencils, FP64 reductions + FP64 defect correction */

/* transform kinds for macsav_transform */
#define MACSAV_DCT2 0
#define MACSAV_DST2 1
#define MACSAV_DST1 2

#define MACSAV_MAX_COLUMNS 4

typedef struct macsav_plan macsav_plan;

/* Result of one Stokes solve (StokesResult, solver/mac/stokes.py:32-37, plus
 * the TensorStokes counters of solver/mac/tensor_stokes.py:169-174,340-344). */
typedef struct {
  double residual;        /* max|defect| / (1 + max|f|) */
  double divergence_inf;  /* max|D u| */
  double max_velocity;    /* max|u| (gate scale) */
  int iterations[MACSAV_MAX_COLUMNS];
  int refinements;        /* defect-correction sweeps (FP32_MIXED), 0 for FP64 */
} macsav_stokes_info;

/* Replaces TensorStokes.__init__ (solver/mac/tensor_stokes.py:128-174) and the
 * MACGrid/MACOperators set-up it relies on (solver/mac/grid.py:9-34,
 * solver/mac/operators.py:11-31): builds eigenvalue/twiddle tables and owns
 * the device work buffers for up to max_columns right-hand sides. */
int macsav_plan_create(macsav_plan** plan, int nx, int ny, double lx, double ly, int precision,
                       double tolerance, double krylov_tolerance, int max_iterations, int max_columns);
void macsav_plan_destroy(macsav_plan* plan);
/* Message of the last failing call on this plan (or of a failed create when plan==NULL). */
const char* macsav_plan_error(const macsav_plan* plan);
/* Kernel launches issued through this plan so far. */
long long macsav_plan_launches(const macsav_plan* plan);

/* y = K x (MACOperators.K, solver/mac/operators.py:16-18; MACNavierStokes.apply_K,
 * solver/mac_ns.py:47-48).  x, y: packed velocities, `columns` columns. */
int macsav_apply_K(macsav_plan* plan, const double* x, double* y, int columns, void* stream);
/* p = D x (MACOperators.D, operators.py:19-29; packed_divergence[_vector],
 * solver/mac/kernels.py:46-87). */
int macsav_apply_D(macsav_plan* plan, const double* x, double* p, int columns, void* stream);
/* x = D^T p = -G p (packed_divergence_transpose[_vector], kernels.py:89-132;
 * MACNavierStokes.apply_G is the negative, solver/mac_ns.py:50-51). */
int macsav_apply_Dt(macsav_plan* plan, const double* p, double* x, int columns, void* stream);
/* n = N(x): skew-symmetric dual-cell convection on the packed vector
 * (kernels.convection, solver/mac/kernels.py:6-35, via MACNavierStokes.nonlinear,
 * solver/mac_ns.py:22-25). */
int macsav_convection(macsav_plan* plan, const double* x, double* n, int columns, void* stream);

/* Orthonormal DCT-II / DST-II / DST-I (or inverse) along each row of a
 * (rows, n) row-major array (_transform_axis, solver/mac/tensor_stokes.py:58-82,
 * scipy.fft norm="ortho").  Runs the same FFT machinery as the solver. */
int macsav_transform(macsav_plan* plan, int kind, int inverse, int rows, int n, const double* in,
                     double* out, void* stream);

/* FP32 form of macsav_transform: the same orthonormal transforms along each
 * row of a (rows, n) row-major FP32 array, computed by
 *   MACSAV_TRANSFORM_FFT  the shared-memory FFT kernels of the solver (FP32);
 *   MACSAV_TRANSFORM_TC3  a transform-matrix product on the tcgen05 tensor
 *                         cores, operands split into 2 BF16 pieces, 3 products
 *                         (relative error about 1e-5);
 *   MACSAV_TRANSFORM_TC6  the same with 3 BF16 pieces, 6 products (FP32 accuracy);
 *   MACSAV_TRANSFORM_AUTO the autotuner's choice for this (kind, direction,
 *                         rows, n), measured on first use.
 * The tensor-core forms take n <= 512 (MACSAV_ERR_UNSUPPORTED beyond).  The
 * reference applies these transforms with scipy.fft (_transform_axis,
 * solver/mac/tensor_stokes.py:58-82); synchronises `stream`. */
#define MACSAV_TRANSFORM_FFT 0
#define MACSAV_TRANSFORM_TC3 1
#define MACSAV_TRANSFORM_TC6 2
#define MACSAV_TRANSFORM_AUTO 3
int macsav_transform32(macsav_plan* plan, int kind, int inverse, int rows, int n, int method, const float* in,
                       float* out, void* stream);
/* The autotuner: times the FFT and the TC6 form for this (kind, direction,
 * rows, n) (10 launches each after a warm-up, CUDA events on `stream`),
 * keeps the faster one as the plan's choice for MACSAV_TRANSFORM_AUTO and
 * returns it with both average times (ms; ms_tensor = -1 when n > 512). */
int macsav_transform32_autotune(macsav_plan* plan, int kind, int inverse, int rows, int n, int* method,
                                double* ms_fft, double* ms_tensor, void* stream);

/* Shifted Stokes solve (mass I + viscosity K) u - D^T p = f, D u = 0 by
 * DST/DCT velocity inverses inside a pressure Schur PCG
 * (TensorStokes.solve, solver/mac/tensor_stokes.py:245-364).
 * rhs, velocity: packed, `columns` columns; pressure: cells, mean-zero per column.
 * Returns MACSAV_ERR_VALUE for invalid shifts or a non-finite RHS,
 * MACSAV_ERR_CG when PCG does not converge in max_iterations, and
 * MACSAV_ERR_STOKES_GATE when residual > tolerance or
 * divergence > tolerance*(1+max|u|); info is filled in every case. */
int macsav_stokes_solve(macsav_plan* plan, const double* rhs, int columns, double mass, double viscosity,
                        double* velocity, double* pressure, macsav_stokes_info* info, void* stream);

/* The two spectral operators of the Stokes solve, applied on their own in the
 * plan's precision (FP32 transforms for MACSAV_FP32_MIXED plans, inputs and
 * outputs FP64 either way); `columns` columns, at most the plan's maximum.
 * macsav_velocity_inverse: out = (mass I + viscosity K)^{-1} values, packed
 * velocities (TensorStokes._velocity_inverse, solver/mac/tensor_stokes.py:200-215).
 * macsav_schur_precondition: out = mass (D D^T)^+ p + viscosity p on the
 * mean-zero part of the cell columns p, mean zero (the preconditioner of the
 * pressure Schur CG, tensor_stokes.py:217-243,281-287).
 * Both return MACSAV_ERR_VALUE for invalid shifts or column counts. */
int macsav_velocity_inverse(macsav_plan* plan, const double* values, double* out, int columns, double mass,
                            double viscosity, void* stream);
int macsav_schur_precondition(macsav_plan* plan, const double* pressure, double* out, int columns, double mass,
                              double viscosity, void* stream);

/* out = sum_k coeffs[k] * fields[k] accumulated in the order given
 * (MACNavierStokes.combine, solver/mac_ns.py:40-45).  coeffs is a HOST array,
 * fields a HOST array of device pointers, n elements each. */
int macsav_combine(macsav_plan* plan, int nterms, const double* coeffs, const double* const* fields, double* out,
                   long long n, void* stream);
/* Host scalar results (synchronising):
 * inner = hx*hy*dot(a,b) (MACGrid.inner, solver/mac/grid.py:67-68);
 * max_abs = max|a| with NaN propagation (MACNavierStokes.max_abs, solver/mac_ns.py:66-67). */
int macsav_inner(macsav_plan* plan, const double* a, const double* b, long long n, double* result, void* stream);
int macsav_max_abs(macsav_plan* plan, const double* a, long long n, double* result, void* stream);

/* Plan-free form of macsav_inner + macsav_max_abs that takes no device memory
 * (no counterpart in the reference, which has no device memory to manage).
 * It is for callers that hold no plan and may not allocate: an error handler
 * after the device ran out of memory, or a monitor of a state's size and
 * finiteness while the solver owns the memory.  result[0] = weight*dot(a,b)
 * (weight*sum(a) when b is NULL), result[1] = max|a| with NaN propagation; a,b
 * device, result HOST; synchronises `stream`.  Its scratch is a fixed
 * 64 KiB device array of the library, so n <= MACSAV_STATIC_REDUCE_MAX_N
 * (larger n: MACSAV_ERR_UNSUPPORTED, before any device work; NULL a/result or
 * n < 0: MACSAV_ERR_VALUE).  The first call on each device finds the array's
 * address (this may load the module) and clears its completion counter:
 * make it outside any stream capture.  The address is kept per device
 * context: after cudaDeviceReset (or any new context on the device) the next
 * call repeats that set-up, and is again a first call.  Calls share that
 * array, so calls that overlap on the device race: order them (e.g. one
 * stream). */
#define MACSAV_STATIC_REDUCE_MAX_N 16777216LL
int macsav_inner_max_static(const double* a, const double* b, long long n, double weight, double* result,
                            void* stream);

/* MACGrid.unpack (direction 0: packed -> u (ny, nx+1), v (ny+1, nx), zero
 * normal wall faces) and MACGrid.pack (direction 1: u, v -> packed)
 * (solver/mac/grid.py:52-65), on device arrays, so host states cross the bus
 * as plain copies. */
int macsav_layout(macsav_plan* plan, int direction, double* packed, double* u, double* v, void* stream);

/* *mapped = 1 when the first and last byte of [p, p + bytes) are page-locked
 * host memory that the current device dereferences at the same address (the
 * pinned memory of cudaHostAlloc under unified addressing), else 0; never
 * an error for ordinary pageable or foreign pointers.  A caller that knows
 * the range lies in one allocation may then pass p to macsav_layout as u or
 * v: the pack kernel reads, and the unpack kernel writes, the host arrays
 * over the host link directly, with no staging copy (the host arrays of
 * MACGrid.pack / unpack, solver/mac/grid.py:52-65).  NULL mapped or
 * bytes < 0: MACSAV_ERR_VALUE. */
int macsav_host_mapped(const void* p, long long bytes, int* mapped);

/* Copies `count` vectors in one kernel on `stream`: src[k] -> dst[k], n[k]
 * doubles each (max_n >= every n[k] sizes the grid).  The arrays src, dst, n
 * and every src[k], dst[k] must be device-accessible: device memory, or
 * pinned host memory that the device maps (macsav_host_mapped), which the
 * kernel then reads or writes over the host link.  This is the ensemble's
 * host boundary: all members' packed velocities in or out in one launch
 * instead of one copy per member (no reference counterpart: the reference
 * steps one model at a time).  count < 0, max_n < 0 or NULL arrays:
 * MACSAV_ERR_VALUE; count == 0: MACSAV_OK, nothing launched. */
int macsav_copy_vectors(int count, const double* const* src, double* const* dst, const long long* n, long long max_n,
                        void* stream);

/* MACNavierStokes.diagnostics (solver/mac_ns.py:95-107) of a packed velocity x
 * with scalar r: out[0..7] = kinetic, modified_energy, divergence_inf,
 * h1_seminorm_squared, r, angular_momentum, power, dissipation.  force may be
 * NULL (zero body force). */
int macsav_diagnostics(macsav_plan* plan, const double* x, double r, double nu, const double* force,
                       double* out, void* stream);

/* time schemes for macsav_step (make_scheme names, solver/schemes/registry.py:24-41) */
#define MACSAV_SDIRK2_MRSAV 0
#define MACSAV_SDIRK3_MRSAV 1
#define MACSAV_IMEX_EULER_MRSAV 2
#define MACSAV_SDIRK2 3
#define MACSAV_SDIRK3 4
#define MACSAV_IMEX_EULER 5

/* stage status codes (records[i].status) */
#define MACSAV_STAGE_OK 0
#define MACSAV_STAGE_STOKES_RHS 1    /* ValueError("Invalid Stokes RHS") */
#define MACSAV_STAGE_CG 2            /* RuntimeError("Pressure Schur CG failed with info=N") */
#define MACSAV_STAGE_STOKES_GATE 3   /* RuntimeError("Stokes residual=..., divergence=...") */
#define MACSAV_STAGE_NEG_ENERGY 4    /* RuntimeError("Negative Stokes response energy") */
#define MACSAV_STAGE_SAV_INPUT 5     /* ValueError("Invalid frozen SAV scalar inputs") */
#define MACSAV_STAGE_SAV_DENOM 6     /* RuntimeError("Invalid frozen SAV scalar denominator") */
#define MACSAV_STAGE_SAV_NONFINITE 7 /* RuntimeError("Nonfinite frozen SAV correction") */
#define MACSAV_STAGE_GATE 8          /* RuntimeError("SAV stage residuals ..., divergence ...") */

/* One stage record: the fields of solver/core.py:15-26 (Stage) that are
 * scalars, plus the Stokes solve's own outcome and CG iterations. */
typedef struct {
  double r, residual, scalar_residual, divergence_inf, continuity_residual;
  double correction_predictor, frozen_factor, corrections[2];
  double stokes_residual, stokes_divergence, max_velocity, max_pressure;
  int n_corrections, iterations[2], cg_info, status;
} macsav_stage_record;

/* One whole time step of `scheme` on the device: replaces Scheme.step for
 * SDIRK2MRSAV (solver/schemes/sdirk2_mrsav.py:61-75), SDIRK3MRSAV
 * (sdirk3_mrsav.py:18-65), IMEXEulerMRSAV (imex_euler_mrsav.py:20-52) and the
 * plain SDIRK2 / SDIRK3 / IMEXEuler (sdirk2.py:20-43, sdirk3.py:34-57,
 * imex_euler.py:13-32) over MACNavierStokes (solver/mac_ns.py:12-107).
 *   x0: packed velocity at t; r0: SAV scalar; forces: NULL for zero body
 *   force, else n_nodes packed vectors f(t + c_j dt) back to back (nodes: SDIRK3
 *   c = 0, 1/4, 4/5, 1; SDIRK2 c = 0, 1-1/sqrt(2); Euler c = 0).
 *   x1: packed velocity at t+dt; embedded (NULL = skip): the embedded velocity;
 *   pressures (NULL = skip): the stage pressures pi_i, n_stages x np;
 *   records: HOST array of n_stages; r1: HOST scalar.
 * Returns MACSAV_OK, or the code of the first failing stage (records[i].status
 * tells which check failed; MACSAV_ERR_VALUE / _CG / _STOKES_GATE /
 * _NEG_ENERGY / _SCALAR / _STAGE_GATE).  Synchronises the stream. */
int macsav_step(macsav_plan* plan, int scheme, double t, double dt, double nu, double gamma, const double* x0,
                double r0, const double* forces, double* x1, double* embedded, double* pressures,
                macsav_stage_record* records, double* r1, void* stream);

/* macsav_step split in two, so that many plans (an ensemble of cavities, one
 * plan each) can have their steps in flight at once: _enqueue issues the step
 * on the plan's own stream (in graph mode without any host wait) and returns;
 * _finish waits for it and fills records / r1 as macsav_step does.  One step
 * per plan may be in flight.  Arguments as for macsav_step (the reference's
 * Scheme.step, see above); there the ensemble is a loop over models. */
int macsav_step_enqueue(macsav_plan* plan, int scheme, double t, double dt, double nu, double gamma,
                        const double* x0, double r0, const double* forces, double* x1, double* embedded,
                        double* pressures, void* stream);
int macsav_step_finish(macsav_plan* plan, macsav_stage_record* records, double* r1);

/* ---- learned preconditioner (no reference counterpart: the reference's
 * pressure CG uses the spectral preconditioner only, tensor_stokes.py:313-321).
 * A bias-free 4-level U-Net (channels c0..c3, default 16/32/64/64; BF16
 * activations, FP32 accumulation) maps a unit-RMS pressure residual to a
 * correction of the spectral preconditioner: z = M r + s(r) net(r / rms(r)),
 * s(r) = rms(r) (r.Mr)/(r.r), projected to mean zero, inside flexible CG
 * (Polak-Ribiere beta) in the FP32 inner solves.  A column whose learned
 * attempt has not converged after learned_max_iterations (or turned
 * non-finite) restarts plain PCG from zero, and the FP64 defect correction
 * and closing gates accept or reject the result as before.  Grids need nx, ny
 * multiples of 8.  Inputs/outputs of the network calls are device FP32
 * [batch][ny][nx]; parameters are host FP32 in layer order, each layer
 * [c_out][c_in][k][k]. */
typedef struct macsav_unet macsav_unet;
int macsav_unet_create(macsav_unet** net, const int* channels /* 4 values or NULL */);
void macsav_unet_destroy(macsav_unet* net);
const char* macsav_unet_error(const macsav_unet* net);
long long macsav_unet_num_params(const macsav_unet* net);
int macsav_unet_set_params(macsav_unet* net, const float* params);
int macsav_unet_get_params(const macsav_unet* net, float* params);
int macsav_unet_forward(macsav_unet* net, const float* in, int batch, int ny, int nx, float* out, void* stream);
/* Forward 3x3 convolutions with 16/32/64 output channels on the tcgen05
 * tensor cores (implicit GEMM, BF16 operands, FP32 accumulation in tensor
 * memory; enable = 1, the default) or on the CUDA-core kernels (0). */
int macsav_unet_set_tensor_cores(macsav_unet* net, int enable);
/* loss = mean((net(in) - target)^2); grads = d loss / d params (host). */
int macsav_unet_gradients(macsav_unet* net, const float* in, const float* target, int batch, int ny, int nx,
                          double* loss, float* grads, void* stream);
/* One Adam step (beta 0.9 / 0.999) on that loss; *loss (host, may be NULL) is
 * the loss before the step. */
int macsav_unet_train_step(macsav_unet* net, const float* in, const float* target, int batch, int ny, int nx,
                           float lr, double* loss, void* stream);
/* Attach (net != NULL) or detach the learned preconditioner of an FP32_MIXED
 * plan.  The plan keeps a pointer: destroy the plan (or detach) first. */
int macsav_plan_set_preconditioner(macsav_plan* plan, macsav_unet* net, int learned_max_iterations);
/* Where the attached network is evaluated.  every_iteration = 0 (the
 * default): only in the first CG iteration of the first FP32 inner solve of
 * each Stokes solve, i.e. it shapes the first search direction of the solve
 * of the stage's own right-hand side, and the remaining iterations are
 * flexible CG with the spectral preconditioner; 1: in every iteration of
 * every inner solve.  restriction f = 1, 2, 4 or 8: the network sees the residual
 * averaged over f x f cells (nx / f, ny / f multiples of 8) and its output is
 * prolonged bilinearly to the cells, which makes one evaluation f^2 times
 * cheaper.  No reference counterpart (see macsav_unet above). */
int macsav_plan_set_learned_placement(macsav_plan* plan, int every_iteration, int restriction);
/* Per-column CG counters since the start of the last macsav_stokes_solve:
 * iterations of every inner solve, those run with the network, and plain-PCG
 * restarts. */
int macsav_plan_cg_counters(macsav_plan* plan, int columns, int* iterations, int* learned_iterations,
                            int* fallbacks);
/* One-column FP64 solve that logs, for every PCG iteration k, the residual
 * r_k, the spectrally preconditioned residual M r_k and the iterate p_k
 * (device arrays of max_pairs x np doubles; `iterates` has max_pairs + 1 rows,
 * the last row after the loop holds the converged iterate).  The exact error
 * of iterate k, p* - p_k, solves S e = r_k: these are the training pairs of
 * the learned preconditioner. */
int macsav_stokes_log(macsav_plan* plan, const double* rhs, double mass, double viscosity, int max_pairs,
                      double* residuals, double* preconditioned, double* iterates, int* pairs, void* stream);

/* After a step that produced an embedded velocity (macsav_step, or
 * macsav_step_finish): out[0] = <x1 - emb, x1 - emb>_h, out[1] = <x0, x0>_h,
 * out[2] = <x1, x1>_h (inner = hx*hy*dot, solver/mac/grid.py:67-68) and
 * out[3] = 1 if emb has a non-finite entry, else 0.  These are the inner
 * products of the adaptive controller's embedded error (controller.py:112-123),
 * formed on the device inside the step, so an adaptive attempt costs one
 * device round trip.  Reads host memory only. */
int macsav_step_embedded_norms(macsav_plan* plan, double* out);

/* Embedded-error step control of the device-resident adaptive run: the
 * reference's IController / PIController (solver/adaptivity/controller.py:14-70)
 * with its scaled error (controller.py:112-123).  proportional <= 0 selects
 * the elementary (I) controller; the PI factor is
 * safety err^(-proportional/order) err_prev^(integral/order). */
typedef struct {
  double atol, rtol, safety, min_factor, max_factor, min_step, max_step, error_floor;
  double proportional, integral;
  int order, max_rejections, max_steps, pad;
} macsav_step_control;

/* One attempt of the device-resident adaptive run.  reason: 0 accepted,
 * 1 scaled error above 1, 2 non-finite error, 3 non-finite trial state,
 * 4 a stage check failed (its status in stage_status). */
typedef struct {
  double t, step, error, factor;
  int accepted, reason, stage_status, pad;
} macsav_adaptive_attempt;

/* Outcome: status 0 complete, 1 failed; reason (failed): the last
 * attempt's reason after too many rejections or a step below min_step
 * following a rejection, 5 the next step below min_step, 6 the maximum
 * number of accepted steps reached.  next_step: the step the controller
 * proposes after the last attempt. */
typedef struct {
  double t, r, next_step;
  int status, reason, accepted_steps, attempted_steps;
} macsav_adaptive_result;

/* The adaptive integration of an autonomous cavity (no body force) from
 * (t0, x0, r0) over a span T with first step dt0, entirely on the device:
 * each attempt (one fused step with its embedded error), the accept/reject
 * decision, the retry with a smaller step and the next step's proposal run
 * inside one CUDA graph launch (a conditional WHILE node over attempts), and
 * the host reads the outcome once at the end.  The reference's driver
 * (integrate_adaptive, solver/adaptivity/controller.py:126-398) makes the same
 * decisions on the host after every attempt.  x0, x_final: device packed
 * velocities (may alias).  history: host array for up to history_cap
 * attempts (may be NULL).  Single-cavity plans; schemes with an embedded
 * velocity (sdirk2[_mrsav], sdirk3[_mrsav]).  Synchronises. */
int macsav_integrate_adaptive(macsav_plan* plan, int scheme, double t0, double T, double dt0, double nu,
                              double gamma, const double* x0, double r0, const macsav_step_control* control,
                              double* x_final, macsav_adaptive_result* result, macsav_adaptive_attempt* history,
                              int history_cap, void* stream);

/* ---- channel MAC: periodic x, no-slip walls in y (the reference's solver/channel/ package).
 * Packed free vector (grid.py:64-77): u faces (j, i), i < nx, then the v faces
 * of the interior rows; cells (j, i).  All arithmetic FP64, device pointers,
 * column-blocked multi-RHS data as for the cavity. */
typedef struct macsav_channel macsav_channel;
/* ChannelGrid(nx, ny, lx, ly) with FFTStokes(tolerance, cache_size)
 * (fft_stokes.py:48-58); nx <= 2048. */
int macsav_channel_create(macsav_channel** ch, int nx, int ny, double lx, double ly, double tolerance,
                          int cache_size);
void macsav_channel_destroy(macsav_channel* ch);
const char* macsav_channel_error(const macsav_channel* ch);
/* which: 0 K (operators.py:15-18), 1 D, 2 G = -D^T (operators.py:19-25),
 * 3 skew convection (kernels.py:9-41). */
int macsav_channel_apply(macsav_channel* ch, int which, const double* in, double* out, int columns, void* stream);
/* out = sum_k coeffs[k] fields[k] in the order given (model.py:57-61); host
 * coeffs, host array of device field pointers, nterms <= 8. */
int macsav_channel_combine(macsav_channel* ch, int nterms, const double* coeffs, const double* const* fields,
                           double* out, long long n, void* stream);
/* result[0] = hx*hy*dot(a, b) (0 when b is NULL), result[1] = max|a| with NaN
 * propagation (grid.py:79-80, model.py:81-82); host result, synchronises. */
int macsav_channel_reduce(macsav_channel* ch, const double* a, const double* b, long long n, double* result,
                          void* stream);
/* flow rate through each x column: hy * sum_j u[j, i] (model.py:94-96), nx device values. */
int macsav_channel_flow_rates(macsav_channel* ch, const double* velocity, double* out, void* stream);
/* FFTStokes.solve (fft_stokes.py:94-137): orthonormal real FFTs along x, one
 * banded saddle solve per x mode (factors cached per (mass, viscosity),
 * least recently used evicted), inverse FFTs, pressure mean removed, FP64
 * closing checks.  *factorized = 1 when this call factored a new shift.
 * Errors: MACSAV_ERR_VALUE (shifts, RHS), MACSAV_ERR_CG (a singular band
 * factor), MACSAV_ERR_STOKES_GATE ("Channel FFT residual=..., divergence=...").
 * Synchronises. */
int macsav_channel_solve(macsav_channel* ch, const double* rhs, int columns, double mass, double viscosity,
                         double* velocity, double* pressure, double* residual, double* divergence, int* factorized,
                         void* stream);

/* ---- ensembles of equal-shape cavities in one plan (no reference
 * counterpart: the reference steps one model at a time).  A plan created for
 * `members` cavities (1..32) of the same grid steps all of them with one
 * launch per kernel: every stage kernel covers all members, the Stokes solve
 * treats their 2 x members right-hand sides as columns with per-member
 * shifts, and every member keeps its own viscosity, SAV scalar, records and
 * gates.  Each member's result is bitwise the single-cavity step's. */
int macsav_plan_create_members(macsav_plan** plan, int nx, int ny, double lx, double ly, int precision,
                               double tolerance, double krylov_tolerance, int max_iterations, int members);
int macsav_plan_members(const macsav_plan* plan);
/* nus, r0: host arrays of `members` values; x0, x1, embedded: device
 * [members][size]; forces: device [members][stages][size] or NULL;
 * pressures: device [members][stages][np]. */
int macsav_step_members_enqueue(macsav_plan* plan, int scheme, double t, double dt, const double* nus, double gamma,
                                const double* x0, const double* r0, const double* forces, double* x1,
                                double* embedded, double* pressures, void* stream);
/* records: host [members][stages]; r1: host [members].  Returns the first
 * failing member's code (its records carry the status). */
int macsav_step_members_finish(macsav_plan* plan, macsav_stage_record* records, double* r1);

/* Process-wide switch (no reference counterpart): launch the solver and step
 * kernels with programmatic dependent launch (default 1), so each kernel's
 * launch and ramp-up overlap the tail of the previous one; 0 launches them in
 * plain stream order.  Affects steps captured after the call. */
int macsav_set_programmatic_launch(int enable);

/* Measurement helper (no reference counterpart: it times this library's own
 * kernels for the roofline): average device milliseconds of `reps`
 * back-to-back launches of one transform pass over the velocity blocks with two
 * right-hand sides, and the pass's algorithmic bytes per launch.
 * pass 0: FP32 column pass, 1: FP32 forward row pass, 2: FP32 inverse row pass
 * (these need a MACSAV_FP32_MIXED plan), 3: FP64 column pass, 4, 5, 6: the
 * FP32 pressure-block column, forward row and inverse row passes (the Schur
 * preconditioner's); pass + 10 s forces launch shape s on every block: 1 one
 * radix-8 butterfly per thread and pass, 2 twice the threads per line, 3 half
 * the threads per line with two butterflies each (0: the plan's own choice;
 * FP32 passes only).  Synchronises. */
int macsav_time_pass(macsav_plan* plan, int pass, int reps, double* ms, double* bytes, void* stream);

/* FP32_MIXED only (no reference counterpart: the reference solves in FP64):
 * number of FP64 defect-correction sweeps after the first FP32 solve
 * (default 2) and the relative Krylov tolerance of each FP32 inner solve
 * (default 1e-4).  The closing FP64 gates are unchanged, so too few sweeps
 * surface as the reference's Stokes-gate error, never as a silent loss. */
int macsav_plan_set_refinement(macsav_plan* plan, int corrections, double inner_krylov_tolerance);
/* Krylov tolerance of the first FP32 solve of each FP32_MIXED Stokes solve
 * (the one that starts from zero); the correction sweeps keep the inner
 * tolerance above.  0 (the default) means the inner tolerance.  A tighter
 * first solve leaves a smaller defect, so fewer sweeps reach the gates; like
 * the sweep count, a bad choice surfaces as the Stokes-gate error. */
int macsav_plan_set_first_solve_tolerance(macsav_plan* plan, double first_krylov_tolerance);
/* Launch shape of the plan's FP32 power-of-two transform passes (no reference
 * counterpart: a tuning control): 0 each pass's own choice (the default),
 * 1 one radix-8 butterfly per thread and Stockham pass, 2 twice the threads
 * per line, 3 half the threads per line with two butterflies each (lengths
 * 1024 to 4096; others fall back to 1).  Every shape computes the same bits;
 * only the time differs.  Affects launches and captures after the call. */
int macsav_plan_set_launch_shape(macsav_plan* plan, int shape);
/* Launch-shape autotuner (no reference counterpart; FP32_MIXED plans): for
 * each of six pass kinds (velocity forward rows, columns, inverse rows, then
 * the pressure block's) times the plan's rule and the three shapes above,
 * `reps` launches each from a captured graph on `stream`'s device, and keeps
 * the fastest (another shape replaces the rule only when 2 % faster).
 * chosen (6 ints, or NULL) receives the kept shapes in that order
 * (0 = the rule).  Results do not change; graphs captured before are
 * dropped.  Synchronises. */
int macsav_plan_autotune_launch_shapes(macsav_plan* plan, int reps, int* chosen, void* stream);

/* Run macsav_step as one captured CUDA graph per (scheme, force, embedded)
 * (the pressure CG loop becomes a conditional WHILE node).  Default: off. */
int macsav_plan_set_graph(macsav_plan* plan, int enable);

#ifdef __cplusplus
}
#endif
#endif /* MACSAV_H */
