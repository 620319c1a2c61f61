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
                                                           const double* f, long long vs, long long ps,
                                                           const double* shift, double* partial) {
  __shared__ double red[6 * 32];
  const int c = blockIdx.y;
  const double mass = shift[2 * c], visc = shift[2 * c + 1];
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

// One block for all columns: reduce the K-slot partials of `nb` blocks per
// column in a fixed order (sums, and maxima for OP_START slot 1 and every
// OP_CHECKS slot), then thread 0 updates the column's scalars.  Under graph
// capture (cond != 0) OP_START and OP_CHECK also set the CG while-loop
// condition to "some column still active".
__global__ void __launch_bounds__(kThreads) k_scalar(int op, const double* partial, int nb, int K, int cols,
                                                     CGScalars* cgs, int* active, int np, double ktol, int maxit,
                                                     SolveChecks* checks, int use_cond,
                                                     cudaGraphConditionalHandle cond) {
  __shared__ double red[6 * 32];
  const bool gated = op == OP_RHO || op == OP_ALPHA || op == OP_CHECK;
  int any = 0;
  for (int c = 0; c < cols; ++c) {
    CGScalars& cg = cgs[c];
    if (gated && !active[c]) continue;  // uniform across the block
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
    if (threadIdx.x == 0) {
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
      any |= active[c];
    }
    __syncthreads();
  }
  if (use_cond && threadIdx.x == 0 && (op == OP_START || op == OP_CHECK)) {
    int a = 0;
    for (int c = 0; c < cols; ++c) a |= active[c];
    cudaGraphSetConditional(cond, a ? 1u : 0u);
  }
}

static inline void scalar(Plan* P, const Exec& X, int op, int nb, int K, int cols, cudaStream_t s) {
  k_scalar<<<1, kThreads, 0, s>>>(op, P->partial, nb, K, cols, P->cg, P->active, P->g.np, P->ktol, P->maxit,
                                  P->checks, X.graph ? 1 : 0, X.cond);
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

// One PCG iteration for every active column (all kernels predicated).
template <typename T>
static void cg_iteration(Plan* P, const Exec& X, const Launcher<T>& L, T* w, T* cells, int cols) {
  const GridDev& g = P->g;
  const long long np = g.np, sz = g.size;
  T* x = cells + 1 * np * cols;
  T* r = cells + 2 * np * cols;
  T* z = cells + 3 * np * cols;
  T* pd = cells + 4 * np * cols;
  T* q = cells + 5 * np * cols;
  const int rb = red_blocks(np);
  const cudaStream_t s = L.s;
  // z = M r = IDCT(g * DCT(r)), rho = r . z
  L.row_forward_p(SrcCells<T, T>{r, np, g.nx}, cols, P->active);
  L.column_p(cols, P->active, P->shift, T(P->pthr));
  L.row_inverse_p(DstCellsDot<T>{z, r, np, g.nx}, cols, P->active, P->partial);
  scalar(P, X, OP_RHO, L.groups_row_p(), 2, cols, s);
  // q = S pdir = D (mI+kK)^{-1} D^T pdir,  pdir = z + beta p
  velocity_inverse<T>(P, L, SrcLift<T, double, T>{nullptr, 0, z, pd, P->cg, np, g.nx, g.nu, T(g.ihx), T(g.ihy)}, w,
                      sz, cols, P->active);
  k_div_q<T, T><<<dim3(rb, cols), kThreads, 0, s>>>(g, w, sz, q, z, pd, np, P->cg, P->active, P->partial);
  scalar(P, X, OP_ALPHA, rb, 3, cols, s);
  k_cg_update<T><<<dim3(rb, cols), kThreads, 0, s>>>(g.np, x, r, pd, z, q, np, P->cg, P->active, P->partial);
  scalar(P, X, OP_CHECK, rb, 1, cols, s);
  P->launches += 2;
}

// PCG on S p = b for `cols` columns (SciPy cg semantics, see file header).
// On entry w holds (mI+kK)^{-1} f in T; on exit x holds the pressure iterate
// and P->cg the per-column counters.
template <typename T>
static int schur_pcg(Plan* P, Exec& X, const Launcher<T>& L, T* w, T* cells, int cols) {
  const GridDev& g = P->g;
  const long long np = g.np, sz = g.size;
  T* b = cells;
  T* x = cells + 1 * np * cols;
  T* r = cells + 2 * np * cols;
  const int rb = red_blocks(np);
  const cudaStream_t s = X.s;
  k_pressure_rhs<T, T><<<dim3(rb, cols), kThreads, 0, s>>>(g, w, sz, b, np, P->partial);
  scalar(P, X, OP_MEAN_B, rb, 1, cols, s);
  k_cg_start<T><<<dim3(rb, cols), kThreads, 0, s>>>(g.np, b, x, r, np, P->cg, P->partial);
  P->launches += 2;
  if (!X.graph) {
    scalar(P, X, OP_START, rb, 2, cols, s);
    for (int it = 0; it < P->maxit; ++it) {
      cudaMemcpyAsync(P->h_active, P->active, sizeof(int) * cols, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return MACSAV_ERR_CUDA;
      bool any = false;
      for (int c = 0; c < cols; ++c) any |= P->h_active[c] != 0;
      if (!any) break;
      cg_iteration<T>(P, X, L, w, cells, cols);
    }
    return MACSAV_OK;
  }
  // graph mode: conditional WHILE node, body = one iteration
  cudaStreamCaptureStatus st;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  if (cudaStreamGetCaptureInfo(s, &st, nullptr, &graph, &deps, nullptr, &ndeps) != cudaSuccess ||
      st != cudaStreamCaptureStatusActive)
    return MACSAV_ERR_CUDA;
  if (cudaGraphConditionalHandleCreate(&X.cond, graph, 0, cudaGraphCondAssignDefault) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  scalar(P, X, OP_START, rb, 2, cols, s);  // sets the loop condition
  if (cudaStreamGetCaptureInfo(s, &st, nullptr, &graph, &deps, nullptr, &ndeps) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = X.cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(X.side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  Launcher<T> Ls{L.t, X.side, L.counter};
  Exec Xs = X;
  Xs.s = X.side;
  cg_iteration<T>(P, Xs, Ls, w, cells, cols);
  cudaGraph_t captured;
  if (cudaStreamEndCapture(X.side, &captured) != cudaSuccess) return MACSAV_ERR_CUDA;
  return MACSAV_OK;
}

// Mean-zero pressure (tensor_stokes.py:324-327: the mean is removed twice).
template <typename T>
static void finish_pressure(Plan* P, const Exec& X, const T* x, double* pres, int cols) {
  const long long np = P->g.np;
  const int rb = red_blocks(np);
  const cudaStream_t s = X.s;
  k_sum_cells<T><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, x, np, P->partial);
  scalar(P, X, OP_MEAN_X, rb, 1, cols, s);
  k_center_cells<T><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, x, np, pres, np, P->cg, P->partial);
  scalar(P, X, OP_MEAN_X, rb, 1, cols, s);
  k_center_cells<double><<<dim3(rb, cols), kThreads, 0, s>>>(P->g.np, pres, np, pres, np, P->cg, nullptr);
  P->launches += 3;
}

static void closing_checks(Plan* P, const Exec& X, const double* f, const double* vel, const double* pres, int cols,
                           const double* shift) {
  const long long n = P->g.size > P->g.np ? P->g.size : P->g.np;
  const int rb = red_blocks(n);
  k_stokes_check<<<dim3(rb, cols), kThreads, 0, X.s>>>(P->g, vel, pres, f, P->g.size, P->g.np, shift, P->partial);
  ++P->launches;
  scalar(P, X, OP_CHECKS, rb, 6, cols, X.s);
}

// FP64 solve: TensorStokes.solve with every vector in double.  Shifts are
// read from P->shift (device), so the same enqueue serves the stand-alone
// solve and the captured stage.
int enqueue_solve_fp64(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres) {
  const GridDev& g = P->g;
  Launcher<double> L{P->t64, X.s, &P->launches};
  const long long sz = g.size;
  velocity_inverse<double>(P, L, SrcPacked<double, double>{f, sz, g.nu, g.nx - 1, g.nx}, P->w, sz, cols, nullptr);
  int rc = schur_pcg<double>(P, X, L, P->w, P->cells, cols);
  if (rc != MACSAV_OK) return rc;
  finish_pressure<double>(P, X, P->cells + 1LL * g.np * cols, pres, cols);
  // u = (mI + kK)^{-1} (f + D^T p)
  velocity_inverse<double>(
      P, L, SrcLift<double, double, double>{f, sz, pres, nullptr, P->cg, (long long)g.np, g.nx, g.nu, g.ihx, g.ihy},
      vel, sz, cols, nullptr);
  closing_checks(P, X, f, vel, pres, cols, P->shift);
  return MACSAV_OK;
}

int solve_fp64(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
               cudaStream_t s) {
  (void)mass;
  (void)visc;
  Exec X{s, false, nullptr, 0};
  return enqueue_solve_fp64(P, X, f, cols, vel, pres);
}

int enqueue_solve_mixed(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres) {
  (void)X; (void)f; (void)cols; (void)vel; (void)pres;
  P->err = "FP32_MIXED solve not built yet";
  return MACSAV_ERR_UNSUPPORTED;
}

// FP32 transforms with FP64 defect correction (filled in below).
int solve_mixed(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
                cudaStream_t s, int* sweeps) {
  (void)f; (void)cols; (void)mass; (void)visc; (void)vel; (void)pres; (void)s; (void)sweeps;
  P->err = "FP32_MIXED solve not built yet";
  return MACSAV_ERR_UNSUPPORTED;
}

}  // namespace macsav
