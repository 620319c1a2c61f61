// extern "C" entry points (declared in include/macsav.h).
#include <cmath>
#include <cstdio>
#include <string>

#include "step.cuh"

struct macsav_plan {
  macsav::Plan p;
};

struct macsav_unet {
  macsav::UNet net;
  macsav::NetWork work;  // training / stand-alone forward workspace
};

namespace macsav {
int solve_fp64(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
               cudaStream_t s);
int solve_mixed(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
                cudaStream_t s, int* sweeps);
int op_apply(Plan* P, int which, const double* in, double* out, int cols, cudaStream_t s);
int op_layout(Plan* P, int direction, double* packed, double* u, double* v, cudaStream_t s);
int op_copy_vectors(int count, const double* const* src, double* const* dst, const long long* n, long long max_n,
                    cudaStream_t s);
int op_combine(Plan* P, int nterms, const double* coeffs, const double* const* fields, double* out, long long n,
               cudaStream_t s);
int op_dot_max(Plan* P, const double* a, const double* b, long long n, double* result, cudaStream_t s);
int op_diagnostics(Plan* P, const double* x, double r, double nu, const double* force, double* out,
                   cudaStream_t s);
int op_transform(Plan* P, int kind, int inverse, int rows, int n, const double* in, double* out, cudaStream_t s);
int time_pass(Plan* P, int pass, int reps, cudaStream_t s, double* ms, double* bytes);
int autotune_shapes(Plan* P, int reps, cudaStream_t user, int* chosen);
int op_velocity_inverse(Plan* P, const double* in, double* out, int cols, cudaStream_t s);
int op_schur_precondition(Plan* P, const double* in, double* out, int cols, cudaStream_t s);
int op_transform32(Plan* P, int kind, int inverse, int rows, int n, int method, const float* in, float* out,
                   cudaStream_t s);
int op_transform32_autotune(Plan* P, int kind, int inverse, int rows, int n, int* method, double* ms_fft,
                            double* ms_tensor, cudaStream_t s);
void reset_cg_counters(Plan* P, int cols, cudaStream_t s);
}  // namespace macsav

using macsav::Plan;

static thread_local std::string g_create_error;

static int fail(Plan* P, int code, const std::string& msg) {
  P->err = msg;
  return code;
}

static int cuda_status(Plan* P) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(P, MACSAV_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  return MACSAV_OK;
}

extern "C" {

static int create_plan(macsav_plan** out, int nx, int ny, double lx, double ly, int precision, double tolerance,
                       double krylov_tolerance, int max_iterations, int max_columns, int members);

int macsav_plan_create(macsav_plan** out, int nx, int ny, double lx, double ly, int precision, double tolerance,
                       double krylov_tolerance, int max_iterations, int max_columns) {
  if (max_columns < 1 || max_columns > MACSAV_MAX_COLUMNS) {
    g_create_error = "max_columns must be in 1..4";
    if (out) *out = nullptr;
    return MACSAV_ERR_VALUE;
  }
  return create_plan(out, nx, ny, lx, ly, precision, tolerance, krylov_tolerance, max_iterations, max_columns, 1);
}

int macsav_plan_create_members(macsav_plan** out, int nx, int ny, double lx, double ly, int precision,
                               double tolerance, double krylov_tolerance, int max_iterations, int members) {
  if (members < 1 || members > macsav::kMaxMembers) {
    g_create_error = "members must be in 1..32";
    if (out) *out = nullptr;
    return MACSAV_ERR_VALUE;
  }
  return create_plan(out, nx, ny, lx, ly, precision, tolerance, krylov_tolerance, max_iterations, 2 * members,
                     members);
}

static int create_plan(macsav_plan** out, int nx, int ny, double lx, double ly, int precision, double tolerance,
                       double krylov_tolerance, int max_iterations, int max_columns, int members) {
  if (!out) return MACSAV_ERR_VALUE;
  *out = nullptr;
  // solver/mac/grid.py:15-19 and solver/mac/tensor_stokes.py:137-143
  if (nx < 3 || ny < 3 || !std::isfinite(lx) || !std::isfinite(ly) || lx <= 0 || ly <= 0) {
    g_create_error = "Require nx,ny >= 3 and positive finite domain lengths";
    return MACSAV_ERR_VALUE;
  }
  if (!(tolerance > 0) || !(krylov_tolerance > 0) || !std::isfinite(tolerance) || !std::isfinite(krylov_tolerance) ||
      max_iterations < 1) {
    g_create_error = "Invalid solver controls";
    return MACSAV_ERR_VALUE;
  }
  if (precision != MACSAV_FP64 && precision != MACSAV_FP32_MIXED) {
    g_create_error = "precision must be MACSAV_FP64 or MACSAV_FP32_MIXED";
    return MACSAV_ERR_VALUE;
  }
  macsav_plan* h = new macsav_plan();
  Plan& p = h->p;
  macsav::GridDev& g = p.g;
  g.nx = nx;
  g.ny = ny;
  g.nu = (nx - 1) * ny;
  g.nv = nx * (ny - 1);
  g.size = g.nu + g.nv;
  g.np = nx * ny;
  g.hx = lx / nx;
  g.hy = ly / ny;
  g.ihx = 1.0 / g.hx;
  g.ihy = 1.0 / g.hy;
  g.ihx2 = 1.0 / (g.hx * g.hx);
  g.ihy2 = 1.0 / (g.hy * g.hy);
  p.lx = lx;
  p.ly = ly;
  p.precision = precision;
  p.tol = tolerance;
  p.ktol = krylov_tolerance;
  p.maxit = max_iterations;
  p.maxcols = max_columns;
  p.members = members;
  const int rc = macsav::plan_build(&p);
  if (rc != MACSAV_OK) {
    g_create_error = p.err;
    delete h;
    return rc;
  }
  *out = h;
  return MACSAV_OK;
}

void macsav_plan_destroy(macsav_plan* plan) {
  if (!plan) return;
  macsav::plan_free(&plan->p);
  delete plan;
}

const char* macsav_plan_error(const macsav_plan* plan) {
  return plan ? plan->p.err.c_str() : g_create_error.c_str();
}

long long macsav_plan_launches(const macsav_plan* plan) { return plan ? plan->p.launches : 0; }

static int apply(macsav_plan* plan, int which, const double* in, double* out, int columns, void* stream) {
  if (!plan || !in || !out) return MACSAV_ERR_VALUE;
  if (columns < 1) return fail(&plan->p, MACSAV_ERR_VALUE, "columns must be >= 1");
  const int rc = macsav::op_apply(&plan->p, which, in, out, columns, static_cast<cudaStream_t>(stream));
  return rc != MACSAV_OK ? cuda_status(&plan->p) : MACSAV_OK;
}
int macsav_apply_K(macsav_plan* plan, const double* x, double* y, int columns, void* stream) {
  return apply(plan, 0, x, y, columns, stream);
}
int macsav_apply_D(macsav_plan* plan, const double* x, double* p, int columns, void* stream) {
  return apply(plan, 1, x, p, columns, stream);
}
int macsav_apply_Dt(macsav_plan* plan, const double* p, double* x, int columns, void* stream) {
  return apply(plan, 2, p, x, columns, stream);
}
int macsav_convection(macsav_plan* plan, const double* x, double* n, int columns, void* stream) {
  return apply(plan, 3, x, n, columns, stream);
}

int macsav_transform(macsav_plan* plan, int kind, int inverse, int rows, int n, const double* in, double* out,
                     void* stream) {
  if (!plan || !in || !out) return MACSAV_ERR_VALUE;
  return macsav::op_transform(&plan->p, kind, inverse, rows, n, in, out, static_cast<cudaStream_t>(stream));
}

static int spectral_op(macsav_plan* plan, int which, const double* in, double* out, int columns, double mass,
                       double viscosity, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // tensor_stokes.py:246-251
  if (!std::isfinite(mass) || !std::isfinite(viscosity) || std::fmin(mass, viscosity) < 0 || mass + viscosity <= 0)
    return fail(P, MACSAV_ERR_VALUE, "Require mass,viscosity >= 0 and nonzero total");
  if (!in || !out || columns < 1 || columns > P->maxcols || columns > MACSAV_MAX_COLUMNS)
    return fail(P, MACSAV_ERR_VALUE, "columns must be in 1..the plan's maximum");
  double shift[2 * MACSAV_MAX_COLUMNS];
  for (int c = 0; c < columns; ++c) {
    shift[2 * c] = mass;
    shift[2 * c + 1] = viscosity;
  }
  cudaMemcpyAsync(P->shift, shift, sizeof(double) * 2 * columns, cudaMemcpyHostToDevice, s);
  const int rc = which == 0 ? macsav::op_velocity_inverse(P, in, out, columns, s)
                            : macsav::op_schur_precondition(P, in, out, columns, s);
  return rc == MACSAV_OK ? cuda_status(P) : rc;
}

int macsav_velocity_inverse(macsav_plan* plan, const double* values, double* out, int columns, double mass,
                            double viscosity, void* stream) {
  return spectral_op(plan, 0, values, out, columns, mass, viscosity, stream);
}

int macsav_schur_precondition(macsav_plan* plan, const double* pressure, double* out, int columns, double mass,
                              double viscosity, void* stream) {
  return spectral_op(plan, 1, pressure, out, columns, mass, viscosity, stream);
}

int macsav_stokes_solve(macsav_plan* plan, const double* rhs, int columns, double mass, double viscosity,
                        double* velocity, double* pressure, macsav_stokes_info* info, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (info) *info = macsav_stokes_info{};
  // tensor_stokes.py:246-251
  if (!std::isfinite(mass) || !std::isfinite(viscosity) || std::fmin(mass, viscosity) < 0 || mass + viscosity <= 0)
    return fail(P, MACSAV_ERR_VALUE, "Require mass,viscosity >= 0 and nonzero total");
  if (!rhs || !velocity || !pressure || columns < 1 || columns > P->maxcols || columns > MACSAV_MAX_COLUMNS)
    return fail(P, MACSAV_ERR_VALUE, "Invalid Stokes RHS");
  double shift[2 * MACSAV_MAX_COLUMNS];
  for (int c = 0; c < columns; ++c) {
    shift[2 * c] = mass;
    shift[2 * c + 1] = viscosity;
  }
  cudaMemcpyAsync(P->shift, shift, sizeof(double) * 2 * columns, cudaMemcpyHostToDevice, s);
  macsav::reset_cg_counters(P, columns, s);
  int sweeps = 0;
  int rc = P->precision == MACSAV_FP64
               ? macsav::solve_fp64(P, rhs, columns, mass, viscosity, velocity, pressure, s)
               : macsav::solve_mixed(P, rhs, columns, mass, viscosity, velocity, pressure, s, &sweeps);
  if (rc != MACSAV_OK) return rc;
  cudaMemcpyAsync(P->h_cg, P->cg, sizeof(macsav::CGScalars) * columns, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(P->h_checks, P->checks, sizeof(macsav::SolveChecks) * columns, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return cuda_status(P);
  if ((rc = cuda_status(P)) != MACSAV_OK) return rc;
  double maxdef = 0, maxf = 0, maxu = 0, maxdiv = 0;
  bool bad_rhs = false, bad_sol = false;
  for (int c = 0; c < columns; ++c) {
    const macsav::SolveChecks& k = P->h_checks[c];
    auto mx = [](double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); };
    maxdef = mx(maxdef, k.max_defect);
    maxf = mx(maxf, k.max_force);
    maxu = mx(maxu, k.max_velocity);
    maxdiv = mx(maxdiv, k.max_div);
    bad_rhs |= k.nonfinite_force != 0;
    bad_sol |= k.nonfinite_solution != 0;
  }
  const double residual = maxdef / (1.0 + maxf);
  if (info) {
    info->residual = residual;
    info->divergence_inf = maxdiv;
    info->max_velocity = maxu;
    info->refinements = sweeps;
    for (int c = 0; c < columns; ++c) info->iterations[c] = P->h_cg[c].iters;
  }
  if (bad_rhs) return fail(P, MACSAV_ERR_VALUE, "Invalid Stokes RHS");
  for (int c = 0; c < columns; ++c)
    if (P->h_cg[c].info != 0) {
      char buf[96];
      std::snprintf(buf, sizeof buf, "Pressure Schur CG failed with info=%d", P->h_cg[c].info);
      return fail(P, MACSAV_ERR_CG, buf);
    }
  if (bad_sol || residual > P->tol || maxdiv > P->tol * (1.0 + maxu)) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "Stokes residual=%.3e, divergence=%.3e", residual, maxdiv);
    return fail(P, MACSAV_ERR_STOKES_GATE, buf);
  }
  return MACSAV_OK;
}

int macsav_combine(macsav_plan* plan, int nterms, const double* coeffs, const double* const* fields, double* out,
                   long long n, void* stream) {
  if (!plan || !coeffs || !fields || !out) return MACSAV_ERR_VALUE;
  return macsav::op_combine(&plan->p, nterms, coeffs, fields, out, n, static_cast<cudaStream_t>(stream));
}

int macsav_inner(macsav_plan* plan, const double* a, const double* b, long long n, double* result, void* stream) {
  if (!plan || !a || !b || !result) return MACSAV_ERR_VALUE;
  double r[2];
  const int rc = macsav::op_dot_max(&plan->p, a, b, n, r, static_cast<cudaStream_t>(stream));
  *result = plan->p.g.hx * plan->p.g.hy * r[0];
  return rc;
}

int macsav_max_abs(macsav_plan* plan, const double* a, long long n, double* result, void* stream) {
  if (!plan || !a || !result) return MACSAV_ERR_VALUE;
  double r[2];
  const int rc = macsav::op_dot_max(&plan->p, a, nullptr, n, r, static_cast<cudaStream_t>(stream));
  *result = r[1];
  return rc;
}

int macsav_layout(macsav_plan* plan, int direction, double* packed, double* u, double* v, void* stream) {
  if (!plan || !packed || !u || !v || direction < 0 || direction > 1) return MACSAV_ERR_VALUE;
  const int rc = macsav::op_layout(&plan->p, direction, packed, u, v, static_cast<cudaStream_t>(stream));
  return rc == MACSAV_OK ? MACSAV_OK : cuda_status(&plan->p);
}

int macsav_host_mapped(const void* p, long long bytes, int* mapped) {
  if (!mapped || bytes < 0) return MACSAV_ERR_VALUE;
  *mapped = 0;
  if (!p || bytes == 0) return MACSAV_OK;
  const char* ends[2] = {static_cast<const char*>(p), static_cast<const char*>(p) + (bytes - 1)};
  for (const char* q : ends) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, q) != cudaSuccess) {
      (void)cudaGetLastError();
      return MACSAV_OK;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer != q || at.hostPointer != q) return MACSAV_OK;
  }
  *mapped = 1;
  return MACSAV_OK;
}

int macsav_copy_vectors(int count, const double* const* src, double* const* dst, const long long* n, long long max_n,
                        void* stream) {
  if (count < 0 || max_n < 0 || (count > 0 && (!src || !dst || !n))) return MACSAV_ERR_VALUE;
  if (count == 0 || max_n == 0) return MACSAV_OK;
  return macsav::op_copy_vectors(count, src, dst, n, max_n, static_cast<cudaStream_t>(stream));
}

int macsav_diagnostics(macsav_plan* plan, const double* x, double r, double nu, const double* force, double* out,
                       void* stream) {
  if (!plan || !x || !out) return MACSAV_ERR_VALUE;
  return macsav::op_diagnostics(&plan->p, x, r, nu, force, out, static_cast<cudaStream_t>(stream));
}

static int stage_status_code(Plan* P, int st) {
  switch (st) {
    case macsav::ST_OK: return MACSAV_OK;
    case macsav::ST_STOKES_RHS: return fail(P, MACSAV_ERR_VALUE, "Invalid Stokes RHS");
    case macsav::ST_CG: return fail(P, MACSAV_ERR_CG, "Pressure Schur CG failed");
    case macsav::ST_STOKES_GATE: return fail(P, MACSAV_ERR_STOKES_GATE, "Stokes gate");
    case macsav::ST_NEG_ENERGY: return fail(P, MACSAV_ERR_NEG_ENERGY, "Negative Stokes response energy");
    case macsav::ST_SAV_INPUT: return fail(P, MACSAV_ERR_VALUE, "Invalid frozen SAV scalar inputs");
    case macsav::ST_SAV_DENOM: return fail(P, MACSAV_ERR_SCALAR, "Invalid frozen SAV scalar denominator");
    case macsav::ST_SAV_NONFINITE: return fail(P, MACSAV_ERR_SCALAR, "Nonfinite frozen SAV correction");
    case macsav::ST_STAGE_GATE: return fail(P, MACSAV_ERR_STAGE_GATE, "stage gate");
    default: return st == MACSAV_ERR_CUDA ? cuda_status(P) : st;
  }
}

int macsav_step(macsav_plan* plan, int scheme, double t, double dt, double nu, double gamma, const double* x0,
                double r0, const double* forces, double* x1, double* embedded, double* pressures,
                macsav_stage_record* records, double* r1, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (scheme < 0 || scheme > MACSAV_IMEX_EULER) return fail(P, MACSAV_ERR_VALUE, "Unknown scheme");
  if (!std::isfinite(dt) || dt <= 0) return fail(P, MACSAV_ERR_VALUE, "Invalid step size");
  if (!std::isfinite(nu) || nu <= 0) return fail(P, MACSAV_ERR_VALUE, "nu must be positive and finite");
  if (!std::isfinite(gamma) || gamma < 0) return fail(P, MACSAV_ERR_VALUE, "gamma must be finite and nonnegative");
  if (!x0 || !records || P->maxcols < 2) return fail(P, MACSAV_ERR_VALUE, "invalid step buffers");
  const int st = macsav::run_step(P, scheme, t, dt, nu, gamma, x0, r0, forces, x1, embedded, pressures, records, r1,
                                  static_cast<cudaStream_t>(stream));
  return stage_status_code(P, st);
}

int macsav_integrate_adaptive(macsav_plan* plan, int scheme, double t0, double T, double dt0, double nu,
                              double gamma, const double* x0, double r0, const macsav_step_control* control,
                              double* x_final, macsav_adaptive_result* result, macsav_adaptive_attempt* history,
                              int history_cap, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (scheme < 0 || scheme > MACSAV_IMEX_EULER) return fail(P, MACSAV_ERR_VALUE, "Unknown scheme");
  if (!control || !result || !x0 || !x_final || history_cap < 0 || P->maxcols < 2)
    return fail(P, MACSAV_ERR_VALUE, "invalid adaptive-run arguments");
  if (!std::isfinite(nu) || nu <= 0) return fail(P, MACSAV_ERR_VALUE, "nu must be positive and finite");
  if (!std::isfinite(gamma) || gamma < 0) return fail(P, MACSAV_ERR_VALUE, "gamma must be finite and nonnegative");
  if (!std::isfinite(t0) || !std::isfinite(T) || !std::isfinite(dt0) || T <= 0 || dt0 <= 0)
    return fail(P, MACSAV_ERR_VALUE, "T and initial_step must be finite and positive");
  const macsav_step_control& c = *control;
  // controller.py:14-70 (validation)
  if (!(c.atol >= 0 && c.rtol >= 0 && c.atol + c.rtol > 0) || !(c.safety > 0 && c.safety < 1) ||
      !(c.min_factor > 0 && c.min_factor < 1 && c.max_factor > 1) || !(c.min_step > 0 && c.min_step <= c.max_step) ||
      c.max_rejections < 0 || c.max_steps < 1 || c.order < 2 || !(c.error_floor > 0 && c.error_floor < 1) ||
      (c.proportional > 0 && !(c.proportional > c.integral && c.integral >= 0)))
    return fail(P, MACSAV_ERR_VALUE, "invalid step control");
  if (dt0 < c.min_step) return fail(P, MACSAV_ERR_VALUE, "initial_step is below min_step");
  const int st = macsav::run_adaptive_device(P, scheme, t0, T, dt0, nu, gamma, x0, r0, c, x_final, result, history,
                                             history_cap, static_cast<cudaStream_t>(stream));
  return st == MACSAV_ERR_CUDA ? cuda_status(P) : st;
}

int macsav_step_enqueue(macsav_plan* plan, int scheme, double t, double dt, double nu, double gamma,
                        const double* x0, double r0, const double* forces, double* x1, double* embedded,
                        double* pressures, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (scheme < 0 || scheme > MACSAV_IMEX_EULER) return fail(P, MACSAV_ERR_VALUE, "Unknown scheme");
  if (!std::isfinite(dt) || dt <= 0) return fail(P, MACSAV_ERR_VALUE, "Invalid step size");
  if (!std::isfinite(nu) || nu <= 0) return fail(P, MACSAV_ERR_VALUE, "nu must be positive and finite");
  if (!std::isfinite(gamma) || gamma < 0) return fail(P, MACSAV_ERR_VALUE, "gamma must be finite and nonnegative");
  if (!x0 || P->maxcols < 2) return fail(P, MACSAV_ERR_VALUE, "invalid step buffers");
  const int rc = macsav::enqueue_step_async(P, scheme, t, dt, nu, gamma, x0, r0, forces, x1, embedded, pressures,
                                            static_cast<cudaStream_t>(stream));
  return rc == MACSAV_ERR_CUDA ? cuda_status(P) : rc;
}

int macsav_step_members_enqueue(macsav_plan* plan, int scheme, double t, double dt, const double* nus, double gamma,
                                const double* x0, const double* r0, const double* forces, double* x1,
                                double* embedded, double* pressures, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (scheme < 0 || scheme > MACSAV_IMEX_EULER) return fail(P, MACSAV_ERR_VALUE, "Unknown scheme");
  if (!std::isfinite(dt) || dt <= 0) return fail(P, MACSAV_ERR_VALUE, "Invalid step size");
  if (!std::isfinite(gamma) || gamma < 0) return fail(P, MACSAV_ERR_VALUE, "gamma must be finite and nonnegative");
  if (!nus || !r0 || !x0) return fail(P, MACSAV_ERR_VALUE, "invalid step buffers");
  for (int m = 0; m < P->members; ++m)
    if (!std::isfinite(nus[m]) || nus[m] <= 0) return fail(P, MACSAV_ERR_VALUE, "nu must be positive and finite");
  const int rc = macsav::enqueue_members(P, scheme, t, dt, nus, gamma, x0, r0, forces, x1, embedded, pressures,
                                         static_cast<cudaStream_t>(stream));
  return rc == MACSAV_ERR_CUDA ? cuda_status(P) : rc;
}

int macsav_step_members_finish(macsav_plan* plan, macsav_stage_record* records, double* r1) {
  if (!plan || !records) return MACSAV_ERR_VALUE;
  return stage_status_code(&plan->p, macsav::finish_members(&plan->p, records, r1));
}

int macsav_plan_members(const macsav_plan* plan) { return plan ? plan->p.members : 0; }

int macsav_step_finish(macsav_plan* plan, macsav_stage_record* records, double* r1) {
  if (!plan || !records) return MACSAV_ERR_VALUE;
  return stage_status_code(&plan->p, macsav::finish_step(&plan->p, records, r1));
}

// ------------------------------------------------ learned preconditioner ---
static int net_fail(macsav_unet* net, int code, const char* msg) {
  net->net.err = msg;
  return code;
}

int macsav_unet_create(macsav_unet** out, const int* channels) {
  if (!out) return MACSAV_ERR_VALUE;
  *out = nullptr;
  macsav_unet* h = new macsav_unet();
  const int rc = macsav::unet_init(&h->net, channels);
  if (rc != MACSAV_OK) {
    g_create_error = h->net.err.empty() ? std::string("U-Net allocation failed") : h->net.err;
    macsav::unet_free(&h->net);
    delete h;
    return rc;
  }
  *out = h;
  return MACSAV_OK;
}

void macsav_unet_destroy(macsav_unet* net) {
  if (!net) return;
  cudaDeviceSynchronize();
  macsav::net_work_free(&net->work);
  macsav::unet_free(&net->net);
  delete net;
}

const char* macsav_unet_error(const macsav_unet* net) { return net ? net->net.err.c_str() : g_create_error.c_str(); }

long long macsav_unet_num_params(const macsav_unet* net) { return net ? net->net.nparams : 0; }

int macsav_unet_set_params(macsav_unet* net, const float* params) {
  if (!net || !params) return MACSAV_ERR_VALUE;
  macsav::UNet& N = net->net;
  if (cudaMemcpy(N.w32, params, sizeof(float) * N.nparams, cudaMemcpyHostToDevice) != cudaSuccess)
    return net_fail(net, MACSAV_ERR_CUDA, "parameter upload failed");
  cudaMemset(N.m1, 0, sizeof(float) * N.nparams);
  cudaMemset(N.m2, 0, sizeof(float) * N.nparams);
  cudaMemset(N.grad, 0, sizeof(float) * N.nparams);
  N.adam_t = 0;
  macsav::unet_sync_bf16(&N, nullptr);
  return cudaDeviceSynchronize() == cudaSuccess ? MACSAV_OK : net_fail(net, MACSAV_ERR_CUDA, "parameter upload failed");
}

int macsav_unet_get_params(const macsav_unet* net, float* params) {
  if (!net || !params) return MACSAV_ERR_VALUE;
  return cudaMemcpy(params, net->net.w32, sizeof(float) * net->net.nparams, cudaMemcpyDeviceToHost) == cudaSuccess
             ? MACSAV_OK
             : MACSAV_ERR_CUDA;
}

int macsav_unet_set_tensor_cores(macsav_unet* net, int enable) {
  if (!net) return MACSAV_ERR_VALUE;
  net->net.tensor_cores = enable != 0;
  return MACSAV_OK;
}

int macsav_unet_forward(macsav_unet* net, const float* in, int batch, int ny, int nx, float* out, void* stream) {
  if (!net || !in || !out) return MACSAV_ERR_VALUE;
  int rc = macsav::net_work_ensure(&net->net, &net->work, batch, ny, nx, net->work.grad);
  if (rc != MACSAV_OK) return net_fail(net, rc, "U-Net needs batch >= 1 and ny, nx multiples of 8");
  rc = macsav::unet_forward(&net->net, &net->work, in, nullptr, batch, ny, nx, out, nullptr,
                            static_cast<cudaStream_t>(stream));
  if (rc != MACSAV_OK) return net_fail(net, rc, "U-Net forward failed");
  if (net->net.tensor_cores) {  // a tensor-core wait that ran out is reported here
    int flag = 0;
    cudaMemcpyAsync(&flag, net->net.tc_err, sizeof(int), cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream));
    if (cudaStreamSynchronize(static_cast<cudaStream_t>(stream)) != cudaSuccess) return MACSAV_ERR_CUDA;
    if (flag) return net_fail(net, MACSAV_ERR_CUDA, "tensor-core convolution wait ran out");
  }
  return MACSAV_OK;
}

static int net_backward(macsav_unet* net, const float* in, const float* target, int batch, int ny, int nx,
                        cudaStream_t s) {
  int rc = macsav::net_work_ensure(&net->net, &net->work, batch, ny, nx, true);
  if (rc != MACSAV_OK) return net_fail(net, rc, "U-Net needs batch >= 1 and ny, nx multiples of 8");
  cudaMemsetAsync(net->net.loss, 0, sizeof(double), s);
  rc = macsav::unet_backward(&net->net, &net->work, in, target, batch, ny, nx, s);
  return rc == MACSAV_OK ? MACSAV_OK : net_fail(net, rc, "U-Net backward failed");
}

int macsav_unet_gradients(macsav_unet* net, const float* in, const float* target, int batch, int ny, int nx,
                          double* loss, float* grads, void* stream) {
  if (!net || !in || !target || !loss || !grads) return MACSAV_ERR_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  macsav::UNet& N = net->net;
  cudaMemsetAsync(N.grad, 0, sizeof(float) * N.nparams, s);
  int rc = net_backward(net, in, target, batch, ny, nx, s);
  if (rc != MACSAV_OK) return rc;
  cudaMemcpyAsync(grads, N.grad, sizeof(float) * N.nparams, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(loss, N.loss, sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaMemsetAsync(N.grad, 0, sizeof(float) * N.nparams, s);
  return cudaStreamSynchronize(s) == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

int macsav_unet_train_step(macsav_unet* net, const float* in, const float* target, int batch, int ny, int nx,
                           float lr, double* loss, void* stream) {
  if (!net || !in || !target || !(lr > 0)) return MACSAV_ERR_VALUE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = net_backward(net, in, target, batch, ny, nx, s);
  if (rc != MACSAV_OK) return rc;
  if ((rc = macsav::unet_adam(&net->net, lr, s)) != MACSAV_OK) return net_fail(net, rc, "Adam step failed");
  if (loss) {
    cudaMemcpyAsync(loss, net->net.loss, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return MACSAV_ERR_CUDA;
  }
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// The plan's buffers for a network that works on the cells restricted by f:
// the network workspace (batch = the plan's columns), the full-resolution
// output, the previous residual and the scales, and the restricted input and
// output when f > 1.
static int net_buffers(Plan* P, macsav::UNet* net, int f) {
  const int ny = P->g.ny, nx = P->g.nx;
  if (ny % f || nx % f)
    return fail(P, MACSAV_ERR_UNSUPPORTED, "the restriction factor must divide nx and ny");
  const int rc = macsav::net_work_ensure(net, &P->netw, P->maxcols, ny / f, nx / f, false);
  if (rc == MACSAV_ERR_UNSUPPORTED)
    return fail(P, rc, "the learned preconditioner needs nx / f and ny / f multiples of 8 (f: restriction)");
  if (rc != MACSAV_OK) return cuda_status(P);
  const size_t cells = size_t(P->maxcols) * P->g.np;
  if (!P->net_out) {
    if (cudaMalloc(&P->net_out, cells * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&P->net_rold, cells * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&P->net_scale, 2 * macsav::kMaxCols * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&P->net_wacc0, size_t(P->maxcols) * P->g.size * sizeof(float)) != cudaSuccess)
      return cuda_status(P);
    cudaMemset(P->net_rold, 0, cells * sizeof(float));
  }
  if (f > 1 && !P->net_cin) {
    // sized for the finest restriction (f = 2) so a later change of f reuses them
    const size_t coarse = size_t(P->maxcols) * (ny / 2) * (nx / 2);
    if (cudaMalloc(&P->net_cin, coarse * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&P->net_cout, coarse * sizeof(float)) != cudaSuccess)
      return cuda_status(P);
  }
  return MACSAV_OK;
}

int macsav_plan_set_preconditioner(macsav_plan* plan, macsav_unet* net, int learned_max_iterations) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  cudaDeviceSynchronize();
  for (auto& kv : P->st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old preconditioner
  P->st.graphs.clear();
  if (!net) {
    P->net = nullptr;
    return MACSAV_OK;
  }
  if (P->precision != MACSAV_FP32_MIXED)
    return fail(P, MACSAV_ERR_UNSUPPORTED, "the learned preconditioner runs in the FP32 inner solves (FP32_MIXED)");
  if (learned_max_iterations < 1 || learned_max_iterations > 1000)
    return fail(P, MACSAV_ERR_VALUE, "learned_max_iterations must be in 1..1000");
  const int rc = net_buffers(P, &net->net, P->net_restrict);
  if (rc != MACSAV_OK) return rc;
  P->net = &net->net;
  P->net_maxit = learned_max_iterations;
  return cudaDeviceSynchronize() == cudaSuccess ? MACSAV_OK : cuda_status(P);
}

int macsav_plan_set_learned_placement(macsav_plan* plan, int every_iteration, int restriction) {
  if (!plan) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (restriction != 1 && restriction != 2 && restriction != 4 && restriction != 8)
    return fail(P, MACSAV_ERR_VALUE, "restriction must be 1, 2, 4 or 8");
  cudaDeviceSynchronize();
  for (auto& kv : P->st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old placement
  P->st.graphs.clear();
  if (P->net) {
    const int rc = net_buffers(P, P->net, restriction);
    if (rc != MACSAV_OK) return rc;
  }
  P->net_every = every_iteration ? 1 : 0;
  P->net_restrict = restriction;
  return MACSAV_OK;
}

int macsav_plan_cg_counters(macsav_plan* plan, int columns, int* iterations, int* learned_iterations,
                            int* fallbacks) {
  if (!plan || columns < 1 || columns > plan->p.maxcols) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (cudaMemcpy(P->h_cg, P->cg, sizeof(macsav::CGScalars) * columns, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_status(P);
  for (int c = 0; c < columns; ++c) {
    if (iterations) iterations[c] = P->h_cg[c].cum_iters;
    if (learned_iterations) learned_iterations[c] = P->h_cg[c].cum_net_iters;
    if (fallbacks) fallbacks[c] = P->h_cg[c].cum_fallbacks;
  }
  return MACSAV_OK;
}

int macsav_stokes_log(macsav_plan* plan, const double* rhs, double mass, double viscosity, int max_pairs,
                      double* residuals, double* preconditioned, double* iterates, int* pairs, void* stream) {
  if (!plan || !rhs || !residuals || !preconditioned || !iterates || !pairs || max_pairs < 1) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  if (P->precision != MACSAV_FP64) return fail(P, MACSAV_ERR_UNSUPPORTED, "the CG log needs an FP64 plan");
  P->log_r = residuals;
  P->log_z = preconditioned;
  P->log_x = iterates;
  P->log_cap = max_pairs;
  P->log_n = 0;
  macsav_stokes_info info;
  double* vel = nullptr;
  double* pres = nullptr;
  int rc = MACSAV_OK;
  if (cudaMalloc(&vel, sizeof(double) * P->g.size) != cudaSuccess ||
      cudaMalloc(&pres, sizeof(double) * P->g.np) != cudaSuccess)
    rc = cuda_status(P);
  if (rc == MACSAV_OK) rc = macsav_stokes_solve(plan, rhs, 1, mass, viscosity, vel, pres, &info, stream);
  cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  *pairs = P->log_n;
  P->log_cap = 0;
  P->log_n = 0;
  P->log_r = P->log_z = P->log_x = nullptr;
  cudaFree(vel);
  cudaFree(pres);
  return rc;
}

int macsav_step_embedded_norms(macsav_plan* plan, double* out) {
  if (!plan || !out) return MACSAV_ERR_VALUE;
  const macsav::StepBuffers& B = plan->p.st;
  if (!B.h_enorm || !B.have_enorm || B.pending_stages > 0)
    return fail(&plan->p, MACSAV_ERR_VALUE, "no finished step with an embedded velocity");
  for (int k = 0; k < 4; ++k) out[k] = B.h_enorm[k];
  return MACSAV_OK;
}

int macsav_set_programmatic_launch(int enable) {
  macsav::g_launch_pdl = enable != 0;
  return MACSAV_OK;
}

int macsav_time_pass(macsav_plan* plan, int pass, int reps, double* ms, double* bytes, void* stream) {
  if (!plan || !ms || !bytes) return MACSAV_ERR_VALUE;
  const int rc = macsav::time_pass(&plan->p, pass, reps, static_cast<cudaStream_t>(stream), ms, bytes);
  return rc == MACSAV_ERR_CUDA ? cuda_status(&plan->p) : rc;
}

int macsav_plan_set_refinement(macsav_plan* plan, int corrections, double inner_krylov_tolerance) {
  if (!plan) return MACSAV_ERR_VALUE;
  if (corrections < 0 || corrections > 8 || !(inner_krylov_tolerance > 0) || !(inner_krylov_tolerance < 1))
    return fail(&plan->p, MACSAV_ERR_VALUE, "corrections must be in 0..8 and 0 < inner tolerance < 1");
  Plan* P = &plan->p;
  if (P->precision == MACSAV_FP32_MIXED && corrections + 1 > P->pieces) {
    // one velocity and pressure piece per FP32 solve of a Stokes solve
    cudaDeviceSynchronize();
    cudaFree(P->wacc32);
    cudaFree(P->xpieces);
    P->wacc32 = nullptr;
    P->xpieces = nullptr;
    P->pieces = 0;
    const size_t C = size_t(P->maxcols), n = size_t(corrections + 1);
    if (cudaMalloc(&P->wacc32, sizeof(float) * P->g.size * C * n) != cudaSuccess ||
        cudaMalloc(&P->xpieces, sizeof(float) * P->g.np * C * n) != cudaSuccess)
      return cuda_status(P);
    P->pieces = corrections + 1;
  }
  plan->p.corrections = corrections;
  plan->p.inner_ktol = inner_krylov_tolerance;
  for (auto& kv : plan->p.st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old sweep count
  plan->p.st.graphs.clear();
  return MACSAV_OK;
}

int macsav_plan_set_first_solve_tolerance(macsav_plan* plan, double first_krylov_tolerance) {
  if (!plan) return MACSAV_ERR_VALUE;
  if (!(first_krylov_tolerance >= 0) || !(first_krylov_tolerance < 1))
    return fail(&plan->p, MACSAV_ERR_VALUE, "0 <= first-solve tolerance < 1");
  plan->p.first_ktol = first_krylov_tolerance;
  for (auto& kv : plan->p.st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old tolerance
  plan->p.st.graphs.clear();
  return MACSAV_OK;
}

int macsav_plan_autotune_launch_shapes(macsav_plan* plan, int reps, int* chosen, void* stream) {
  if (!plan) return MACSAV_ERR_VALUE;
  if (plan->p.precision != MACSAV_FP32_MIXED || reps < 1 || reps > 1000)
    return fail(&plan->p, MACSAV_ERR_VALUE, "autotune: an FP32_MIXED plan and 1 <= reps <= 1000");
  const int rc = macsav::autotune_shapes(&plan->p, reps, static_cast<cudaStream_t>(stream), chosen);
  for (auto& kv : plan->p.st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old shapes
  plan->p.st.graphs.clear();
  return rc == MACSAV_ERR_CUDA ? cuda_status(&plan->p) : rc;
}

int macsav_plan_set_launch_shape(macsav_plan* plan, int shape) {
  if (!plan || shape < 0 || shape > 3) return MACSAV_ERR_VALUE;
  for (macsav::TBlockDev<float>* B : {&plan->p.t32.u, &plan->p.t32.v, &plan->p.t32.p})
    B->shape[0] = B->shape[1] = B->shape[2] = shape;
  for (auto& kv : plan->p.st.graphs) cudaGraphExecDestroy(kv.exec);  // captured with the old shapes
  plan->p.st.graphs.clear();
  return MACSAV_OK;
}

int macsav_plan_set_graph(macsav_plan* plan, int enable) {
  if (!plan) return MACSAV_ERR_VALUE;
  plan->p.use_graph = enable ? 1 : 0;
  return MACSAV_OK;
}

}  // extern "C"

int macsav_transform32(macsav_plan* plan, int kind, int inverse, int rows, int n, int method, const float* in,
                       float* out, void* stream) {
  if (!plan || !in || !out) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  const int rc = macsav::op_transform32(P, kind, inverse, rows, n, method, in, out, static_cast<cudaStream_t>(stream));
  return rc == MACSAV_ERR_CUDA ? cuda_status(P) : rc;
}

int macsav_transform32_autotune(macsav_plan* plan, int kind, int inverse, int rows, int n, int* method,
                                double* ms_fft, double* ms_tensor, void* stream) {
  if (!plan || !method || !ms_fft || !ms_tensor) return MACSAV_ERR_VALUE;
  Plan* P = &plan->p;
  const int rc = macsav::op_transform32_autotune(P, kind, inverse, rows, n, method, ms_fft, ms_tensor,
                                                 static_cast<cudaStream_t>(stream));
  return rc == MACSAV_ERR_CUDA ? cuda_status(P) : rc;
}
