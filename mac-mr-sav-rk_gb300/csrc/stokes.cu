// Shifted Stokes solve by DST/DCT velocity inverses inside a pressure Schur PCG.
//
// Restates TensorStokes.solve (solver/mac/tensor_stokes.py:245-364) and the
// SciPy 1.18.1 conjugate-gradient loop it calls (x0 = 0; stop when
// ||r||_2 < rtol ||b||_2, tested before every update; the iteration count is
// the number of updates; info = maxiter when the loop is exhausted).
//
// Device data per right-hand-side column c: b (pressure RHS), x (pressure),
// r (residual), z (preconditioned residual), p (search direction), q (S p).
// Every Krylov scalar lives on the device (CGScalars); each kernel of the
// loop is predicated on the column's `active` flag, so the host only needs the
// flags to know when to stop launching.
#include <cmath>
#include <cstdio>

#include "solver.cuh"

namespace macsav {

constexpr int kRedMax = 1024;  // cap on blocks of grid-stride reduction kernels

inline int red_blocks(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : (b > kRedMax ? kRedMax : b));
}

// ------------------------------------------------------------ CG kernels ---
template <typename T, typename WIn>
__global__ void __launch_bounds__(kThreads) k_pressure_rhs(GridDev g, const WIn* w, long long ws, T* b, long long cs,
                                                           double* partial) {
  __shared__ double red[64];
  const int c = blockIdx.y;
  double acc[1] = {0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.np; idx += gridDim.x * blockDim.x) {
    const int j = idx / g.nx, i = idx - j * g.nx;
    const T v = T(-D_at(w + c * ws, g, j, i));
    b[c * cs + idx] = v;
    acc[0] += double(v);
  }
  block_sum<1>(acc, red);
  if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = acc[0];
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_start(int np, T* b, T* x, T* r, long long cs, const CGScalars* cg,
                                                       double* partial) {
  __shared__ double red[64];
  const int c = blockIdx.y;
  const double mean = cg[c].mean_b;
  double s[1] = {0.0}, m[1] = {0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
    const long long i = c * cs + idx;
    const T v = T(double(b[i]) - mean);
    b[i] = v;
    r[i] = v;
    x[i] = T(0);
    s[0] += double(v) * double(v);
    m[0] = nanmax(m[0], fabs(double(v)));
  }
  block_sum<1>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0) {
    partial[(c * gridDim.x + blockIdx.x) * 2] = s[0];
    partial[(c * gridDim.x + blockIdx.x) * 2 + 1] = m[0];
  }
}

template <typename T, typename WIn>
__global__ void __launch_bounds__(kThreads) k_div_q(GridDev g, const WIn* w, long long ws, T* q, const T* z, const T* p,
                                                    long long cs, const CGScalars* cg, const int* active,
                                                    double* partial) {
  const int c = blockIdx.y;
  if (!active[c]) return;
  __shared__ double red[96];
  const bool first = cg[c].iters == 0;
  const T beta = T(cg[c].beta);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.np; idx += gridDim.x * blockDim.x) {
    const int j = idx / g.nx, i = idx - j * g.nx;
    const long long k = c * cs + idx;
    const T qv = T(D_at(w + c * ws, g, j, i));
    q[k] = qv;
    const T pd = first ? z[k] : T(z[k] + beta * p[k]);
    acc[0] += double(pd) * double(qv);
    acc[1] += double(qv);
    acc[2] += double(pd);
  }
  block_sum<3>(acc, red);
  if (threadIdx.x == 0) {
    double* o = partial + (c * gridDim.x + blockIdx.x) * 3;
    o[0] = acc[0];
    o[1] = acc[1];
    o[2] = acc[2];
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_update(int np, T* x, T* r, T* p, const T* z, const T* q,
                                                        long long cs, const CGScalars* cg, const int* active,
                                                        double* partial) {
  const int c = blockIdx.y;
  if (!active[c]) return;
  __shared__ double red[64];
  const bool first = cg[c].iters == 0;
  const T beta = T(cg[c].beta), alpha = T(cg[c].alpha), mq = T(cg[c].mean_q);
  double acc[1] = {0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
    const long long k = c * cs + idx;
    const T pd = first ? z[k] : T(z[k] + beta * p[k]);
    p[k] = pd;
    x[k] = x[k] + alpha * pd;
    const T rv = r[k] - alpha * (q[k] - mq);
    r[k] = rv;
    acc[0] += double(rv) * double(rv);
  }
  block_sum<1>(acc, red);
  if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = acc[0];
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_sum_cells(int np, const T* x, long long cs, double* partial) {
  __shared__ double red[64];
  const int c = blockIdx.y;
  double acc[1] = {0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x)
    acc[0] += double(x[c * cs + idx]);
  block_sum<1>(acc, red);
  if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = acc[0];
}

// out = x - mean (mean kept in cg[c].mean_q after the loop); partial sum of out.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_center_cells(int np, const T* x, long long xs, double* out,
                                                           long long os, const CGScalars* cg, double* partial) {
  __shared__ double red[64];
  const int c = blockIdx.y;
  const double mean = cg[c].mean_q;
  double acc[1] = {0.0};
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
    const double v = double(x[c * xs + idx]) - mean;
    out[c * os + idx] = v;
    acc[0] += v;
  }
  block_sum<1>(acc, red);
  if (partial && threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = acc[0];
}

// Closing checks (tensor_stokes.py:329-351): defect = m u + k K u - D^T p - f.
// Partial slots: max|defect|, max|f|, max|u|, max|D u|, nonfinite f, nonfinite u/p.
__global__ void __launch_bounds__(kThreads) k_stokes_check(GridDev g, const double* vel, const double* pres,
                                                           const double* f, long long vs, long long ps, double mass,
                                                           double visc, double* partial) {
  __shared__ double red[6 * 32];
  const int c = blockIdx.y;
  const double* u = vel + c * vs;
  const double* pp = pres + c * ps;
  const double* ff = f + c * vs;
  double m[6] = {0, 0, 0, 0, 0, 0};
  const int n = g.size > g.np ? g.size : g.np;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (idx < g.size) {
      const double fe = ff[idx], ue = u[idx];
      const double d = mass * ue + visc * K_at(u, g, idx) - Dt_at(pp, g, idx) - fe;
      m[0] = nanmax(m[0], fabs(d));
      m[1] = nanmax(m[1], fabs(fe));
      m[2] = nanmax(m[2], fabs(ue));
      if (!isfinite(fe)) m[4] = 1.0;
      if (!isfinite(ue)) m[5] = 1.0;
    }
    if (idx < g.np) {
      const int j = idx / g.nx, i = idx - j * g.nx;
      m[3] = nanmax(m[3], fabs(D_at(u, g, j, i)));
      if (!isfinite(pp[idx])) m[5] = 1.0;
    }
  }
  block_max<6>(m, red);
  if (threadIdx.x == 0)
    for (int k = 0; k < 6; ++k) partial[(c * gridDim.x + blockIdx.x) * 6 + k] = m[k];
}

// ----------------------------------------------------------- scalar logic ---
enum ScalarOp : int { OP_MEAN_B, OP_START, OP_RHO, OP_ALPHA, OP_CHECK, OP_MEAN_X, OP_CHECKS };

// One block per column: reduce the K-slot partials of `nb` blocks in a fixed
// order (sums; maxima for OP_START slot 1 and every OP_CHECKS slot), then
// thread 0 updates the column's scalars.
__global__ void __launch_bounds__(kThreads) k_scalar(int op, const double* partial, int nb, int K, CGScalars* cgs,
                                                     int* active, int np, double ktol, int maxit,
                                                     SolveChecks* checks) {
  __shared__ double red[6 * 32];
  const int c = blockIdx.x;
  CGScalars& cg = cgs[c];
  const bool gated = op == OP_RHO || op == OP_ALPHA || op == OP_CHECK;
  if (gated && !active[c]) return;
  double s[6] = {0, 0, 0, 0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const double* o = partial + (size_t(c) * nb + b) * K;
    for (int k = 0; k < K && k < 6; ++k) {
      s[k] += o[k];
      m[k] = nanmax(m[k], o[k]);
    }
  }
  block_sum<6>(s, red);
  block_max<6>(m, red);
  if (threadIdx.x != 0) return;
  switch (op) {
    case OP_MEAN_B:
      cg.mean_b = s[0] / np;
      break;
    case OP_START: {
      cg.bnorm = sqrt(s[0]);
      cg.max_b = m[1];
      cg.atol = ktol * cg.bnorm;  // _get_atol_rtol: max(atol=0, rtol*||b||)
      cg.iters = 0;
      cg.info = 0;
      cg.rho_prev = 0;
      cg.beta = 0;
      cg.rr = s[0];
      // zero RHS (tensor_stokes.py:309-311) or already converged: no update
      const bool go = (cg.max_b != 0.0) && !(sqrt(cg.rr) < cg.atol) && (cg.bnorm == cg.bnorm);
      active[c] = go ? 1 : 0;
      break;
    }
    case OP_RHO:
      cg.rho = s[0];
      cg.beta = cg.iters > 0 ? cg.rho / cg.rho_prev : 0.0;
      break;
    case OP_ALPHA:
      cg.mean_q = s[1] / np;
      cg.pq = s[0] - s[1] * s[2] / np;  // p . (q - mean(q))
      cg.alpha = cg.rho / cg.pq;
      break;
    case OP_CHECK:
      cg.rr = s[0];
      cg.iters += 1;
      cg.rho_prev = cg.rho;
      if (sqrt(cg.rr) < cg.atol) {
        active[c] = 0;
      } else if (cg.iters >= maxit || !(cg.rr == cg.rr)) {
        active[c] = 0;
        cg.info = maxit;
      }
      break;
    case OP_MEAN_X:
      cg.mean_q = s[0] / np;
      break;
    case OP_CHECKS:
      checks[c].max_defect = m[0];
      checks[c].max_force = m[1];
      checks[c].max_velocity = m[2];
      checks[c].max_div = m[3];
      checks[c].nonfinite_force = m[4] != 0.0;
      checks[c].nonfinite_solution = m[5] != 0.0;
      break;
  }
}

static inline void scalar(Plan* P, int op, int nb, int K, int cols, cudaStream_t s) {
  k_scalar<<<cols, kThreads, 0, s>>>(op, P->partial, nb, K, P->cg, P->active, P->g.np, P->ktol, P->maxit,
                                     P->checks);
  ++P->launches;
}

// ----------------------------------------------------------------- solve ---
// Velocity inverse (m I + k K)^{-1} of `src` rows into packed `dst`.
template <typename T, class Src, typename Out>
static void velocity_inverse(Plan* P, const Launcher<T>& L, Src src, Out* dst, long long dstride, int cols,
                             const int* active) {
  const GridDev& g = P->g;
  L.row_forward_uv(src, cols, active);
  L.column_uv(cols, active, P->shift);
  DstPacked<T, Out> d{dst, dstride, g.nu, g.nx - 1, g.nx};
  L.row_inverse_uv(d, cols, active, nullptr);
}

// PCG on S p = b for `cols` columns (SciPy cg semantics, see file header).
// On entry w holds (mI+kK)^{-1} f in T; on exit x holds the pressure iterate,
// P->cg the per-column counters, P->h_cg their host copy.
template <typename T>
static void schur_pcg(Plan* P, const Launcher<T>& L, T* w, T* cells, int cols, cudaStream_t s) {
  const GridDev& g = P->g;
  const long long np = g.np, sz = g.size;
  T* b = cells;
  T* x = cells + 1 * np * cols;
  T* r = cells + 2 * np * cols;
  T* z = cells + 3 * np * cols;
  T* pd = cells + 4 * np * cols;
  T* q = cells + 5 * np * cols;
  const int rb = red_blocks(np);
  k_pressure_rhs<T, T><<<dim3(rb, cols), kThreads, 0, s>>>(g, w, sz, b, np, P->partial);
  ++P->launches;
  scalar(P, OP_MEAN_B, rb, 1, cols, s);
  k_cg_start<T><<<dim3(rb, cols), kThreads, 0, s>>>(g.np, b, x, r, np, P->cg, P->partial);
  ++P->launches;
  scalar(P, OP_START, rb, 2, cols, s);
  cudaMemcpyAsync(P->h_active, P->active, sizeof(int) * cols, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  const int nbp = L.groups_row_p();
  const T ihx = T(g.ihx), ihy = T(g.ihy);
  for (int it = 0; it < P->maxit; ++it) {
    bool any = false;
    for (int c = 0; c < cols; ++c) any |= P->h_active[c] != 0;
    if (!any) break;
    // z = M r = IDCT(g * DCT(r)), rho = r . z
    L.row_forward_p(SrcCells<T, T>{r, np, g.nx}, cols, P->active);
    L.column_p(cols, P->active, P->shift, T(P->pthr));
    L.row_inverse_p(DstCellsDot<T>{z, r, np, g.nx}, cols, P->active, P->partial);
    scalar(P, OP_RHO, nbp, 2, cols, s);
    // q = S pdir = D (mI+kK)^{-1} D^T pdir,  pdir = z + beta p
    velocity_inverse<T>(P, L, SrcLift<T, double, T>{nullptr, 0, z, pd, P->cg, np, g.nx, g.nu, ihx, ihy}, w, sz,
                        cols, P->active);
    k_div_q<T, T><<<dim3(rb, cols), kThreads, 0, s>>>(g, w, sz, q, z, pd, np, P->cg, P->active, P->partial);
    ++P->launches;
    scalar(P, OP_ALPHA, rb, 3, cols, s);
    k_cg_update<T><<<dim3(rb, cols), kThreads, 0, s>>>(g.np, x, r, pd, z, q, np, P->cg, P->active, P->partial);
    ++P->launches;
    scalar(P, OP_CHECK, rb, 1, cols, s);
    cudaMemcpyAsync(P->h_active, P->active, sizeof(int) * cols, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
  }
}

// Mean-zero pressure (tensor_stokes.py:324-327: the mean is removed twice).
template <typename T>
static void finish_pressure(Plan* P, const T* x, double* pres, int cols, cudaStream_t s) {
  const long long np = P->g.np;
  const int rb = red_blocks(np);
  k_sum_cells<T><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, x, np, P->partial);
  scalar(P, OP_MEAN_X, rb, 1, cols, s);
  k_center_cells<T><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, x, np, pres, np, P->cg, P->partial);
  scalar(P, OP_MEAN_X, rb, 1, cols, s);
  k_center_cells<double><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, pres, np, pres, np, P->cg, nullptr);
  P->launches += 3;
}

static void closing_checks(Plan* P, const double* f, const double* vel, const double* pres, int cols, double mass,
                           double visc, cudaStream_t s) {
  const long long n = P->g.size > P->g.np ? P->g.size : P->g.np;
  const int rb = red_blocks(n);
  k_stokes_check<<<dim3(rb, cols), kThreads, 0, s>>>(P->g, vel, pres, f, P->g.size, P->g.np, mass, visc,
                                                     P->partial);
  ++P->launches;
  scalar(P, OP_CHECKS, rb, 6, cols, s);
}

// FP64 solve: TensorStokes.solve with every vector in double.
int solve_fp64(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
               cudaStream_t s) {
  const GridDev& g = P->g;
  Launcher<double> L{P->t64, s, &P->launches};
  const long long sz = g.size;
  velocity_inverse<double>(P, L, SrcPacked<double, double>{f, sz, g.nu, g.nx - 1, g.nx}, P->w, sz, cols, nullptr);
  schur_pcg<double>(P, L, P->w, P->cells, cols, s);
  finish_pressure<double>(P, P->cells + 1LL * g.np * cols, pres, cols, s);
  // u = (mI + kK)^{-1} (f + D^T p)
  velocity_inverse<double>(
      P, L, SrcLift<double, double, double>{f, sz, pres, nullptr, P->cg, (long long)g.np, g.nx, g.nu, g.ihx, g.ihy},
      vel, sz, cols, nullptr);
  closing_checks(P, f, vel, pres, cols, mass, visc, s);
  return MACSAV_OK;
}

// FP32 transforms with FP64 defect correction (filled in below).
int solve_mixed(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
                cudaStream_t s, int* sweeps) {
  (void)f; (void)cols; (void)mass; (void)visc; (void)vel; (void)pres; (void)s; (void)sweeps;
  P->err = "FP32_MIXED solve not built yet";
  return MACSAV_ERR_UNSUPPORTED;
}

}  // namespace macsav
