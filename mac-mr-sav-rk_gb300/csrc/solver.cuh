// Device functors, the Krylov scalar logic and the transform launchers.
#pragma once
#include <algorithm>

#include "fftp.cuh"
#include "plan.cuh"

namespace macsav {

// CG scalars in the working type (FP32 kernels read the float copies, so
// they issue no FP64 conversion).
template <typename T> __device__ __forceinline__ T cg_beta(const CGScalars& g) {
  if constexpr (sizeof(T) == 4) return g.beta_t; else return g.beta;
}
template <typename T> __device__ __forceinline__ T cg_alpha(const CGScalars& g) {
  if constexpr (sizeof(T) == 4) return g.alpha_t; else return g.alpha;
}
template <typename T> __device__ __forceinline__ T cg_mean_q(const CGScalars& g) {
  if constexpr (sizeof(T) == 4) return g.mean_q_t; else return g.mean_q;
}
template <typename T> __device__ __forceinline__ T cg_mean_b(const CGScalars& g) {
  if constexpr (sizeof(T) == 4) return g.mean_b_t; else return g.mean_b;
}

// ------------------------------------------------------------ row sources ---
// Packed velocity rows: block 0 = u rows (length nx-1), block 1 = v rows (nx).
template <typename T, typename In>
struct SrcPacked {
  const In* x;
  long long cstride;
  int off1, n0, n1;
  __device__ T operator()(int b, int c, int row, int n) const {
    const In* base = x + c * cstride;
    return b == 0 ? load_as<T>(base + (long long)row * n0 + n) : load_as<T>(base + off1 + (long long)row * n1 + n);
  }
};

// Cell rows (ny, nx).
template <typename T, typename In>
struct SrcCells {
  const In* x;
  long long cstride;
  int nx;
  __device__ T operator()(int, int c, int row, int n) const { return load_as<T>(x + c * cstride + (long long)row * nx + n); }
};

// r = b - mean(b) for the first CG iteration of a fused start (the source of
// the preconditioner's row pass, which reads every element once, also
// stores r).
template <typename T>
struct SrcCellsStart {
  const T* b;
  T* r;
  const CGScalars* cg;
  long long cstride;
  int nx;
  __device__ T operator()(int, int c, int row, int n) const {
    const long long k = c * cstride + (long long)row * nx + n;
    const T v = b[k] - cg_mean_b<T>(cg[c]);
    r[k] = v;
    return v;
  }
};

// f + D^T P with P = p1 (+ beta p2 after the first CG iteration), on u/v rows.
template <typename T, typename FIn, typename PIn>
struct SrcLift {
  const FIn* f;  // may be null
  long long fstride;
  const PIn* p1;
  const PIn* p2;  // may be null
  const CGScalars* cg;
  long long pstride;
  int nx, nu;
  T ihx, ihy;
  __device__ T operator()(int bk, int c, int row, int n) const {
    const PIn* a = p1 + c * pstride;
    const long long l = (long long)row * nx + n;
    const long long l2 = bk == 0 ? l + 1 : l + nx;
    T v0 = load_as<T>(a + l), v1 = load_as<T>(a + l2);
    if (p2 && cg[c].iters > 0) {
      const PIn* b = p2 + c * pstride;
      const T beta = cg_beta<T>(cg[c]);
      v0 = v0 + beta * load_as<T>(b + l);
      v1 = v1 + beta * load_as<T>(b + l2);
    }
    T v = (v0 - v1) * (bk == 0 ? ihx : ihy);
    if (f) v += load_as<T>(f + c * fstride + (bk == 0 ? (long long)row * (nx - 1) + n : nu + l));
    return v;
  }
};

// --------------------------------------------------------------- row sinks ---
// Two-phase sinks: aux = load(...) is issued for a batch, then store(...).
template <typename T, typename Out>
struct DstPacked {
  using aux_t = int;
  Out* x;
  long long cstride;
  int off1, n0, n1;
  __device__ aux_t load(int, int, int, int) const { return 0; }
  __device__ void store(int b, int c, int row, int n, T v, aux_t, Acc<T> (&)[2]) const {
    Out* base = x + c * cstride;
    if (b == 0) base[(long long)row * n0 + n] = Out(v);
    else base[off1 + (long long)row * n1 + n] = Out(v);
  }
};

template <typename T, typename Out>
struct DstCells {
  using aux_t = int;
  Out* x;
  long long cstride;
  int nx;
  __device__ aux_t load(int, int, int, int) const { return 0; }
  __device__ void store(int, int c, int row, int n, T v, aux_t, Acc<T> (&)[2]) const {
    x[c * cstride + (long long)row * nx + n] = Out(v);
  }
};

// z = value; acc[0] += r . z
template <typename T>
struct DstCellsDot {
  using aux_t = T;
  T* z;
  const T* r;
  long long cstride;
  int nx;
  __device__ aux_t load(int, int c, int row, int n) const { return r[c * cstride + (long long)row * nx + n]; }
  __device__ void store(int, int c, int row, int n, T v, aux_t rv, Acc<T> (&acc)[2]) const {
    z[c * cstride + (long long)row * nx + n] = v;
    acc[0].add(rv * v);
  }
};

// ------------------------------------------------------- Krylov scalars ---
enum ScalarOp : int { OP_MEAN_B, OP_START, OP_RHO, OP_ALPHA, OP_CHECK, OP_MEAN_X, OP_CHECKS, OP_FCG, OP_START_RHS };

// Block-wide fold of the K-slot partials of `nb` blocks per column in a
// fixed order, then thread 0 updates each column's scalars.  Sum slots hold
// Red<T>::P partials (double, or a double-float pair for FP32 data, so no
// FP64 instruction is issued for FP32 data until the final scalars); max
// slots hold abs_key integers.  Under graph capture OP_START and OP_CHECK also
// set the CG while-loop condition to "some column active".
template <typename T>
struct CGFin {
  int op;
  const double* partial;
  int nb, K, cols;
  CGScalars* cg;
  int* active;
  int np;
  double ktol;
  int maxit;
  SolveChecks* checks;
  int use_cond;
  cudaGraphConditionalHandle cond;
  int use_net, net_maxit;
  double inv_np;

  __device__ int maxmask() const {
    return op == OP_START ? 0x2 : (op == OP_CHECKS ? 0x3f : (op == OP_START_RHS ? 0x4 : 0));
  }

  // One warp per (column, slot) folds that slot's nb block partials (lane
  // stride, then a shuffle tree: a fixed order), so all columns and slots are
  // folded at once with a single block barrier; then one thread per column
  // forms its scalars.
  __device__ void operator()() const {
    using R = Red<T>;
    __shared__ double vals[kMaxCols][6];
    const bool gated = op == OP_RHO || op == OP_ALPHA || op == OP_CHECK || op == OP_FCG;
    const int mm = maxmask();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int pr = wid; pr < cols * K; pr += nw) {
      const int c = pr / K, k = pr - c * K;
      if (gated && !active[c]) continue;  // uniform across the warp
      const double* o = partial + size_t(c) * nb * K + k;
      // the lane's partials are loaded kFold at a time before they are
      // combined (in the same order as one by one, so the same bits): the
      // last block then waits for one L2 round trip per kFold partials, not
      // per partial
      constexpr int kFold = 8;
      if ((mm >> k) & 1) {
        unsigned long long m = 0ull;
        int b = lane;
        for (; b + (kFold - 1) * 32 < nb; b += kFold * 32) {
          unsigned long long t[kFold];
#pragma unroll
          for (int u = 0; u < kFold; ++u)
            t[u] = (unsigned long long)__ldcg(reinterpret_cast<const long long*>(o + size_t(b + 32 * u) * K));
#pragma unroll
          for (int u = 0; u < kFold; ++u) m = max(m, t[u]);
        }
        for (; b < nb; b += 32)
          m = max(m, (unsigned long long)__ldcg(reinterpret_cast<const long long*>(o + size_t(b) * K)));
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, off));
        if (lane == 0) vals[c][k] = key_value(m);
      } else {
        typename R::P v = R::zero();
        int b = lane;
        for (; b + (kFold - 1) * 32 < nb; b += kFold * 32) {
          typename R::P t[kFold];
#pragma unroll
          for (int u = 0; u < kFold; ++u) t[u] = R::load(o + size_t(b + 32 * u) * K);
#pragma unroll
          for (int u = 0; u < kFold; ++u) v = R::add(v, t[u]);
        }
        for (; b < nb; b += 32) v = R::add(v, R::load(o + size_t(b) * K));
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v = R::add(v, R::shfl_down(v, off));
        if (lane == 0) vals[c][k] = R::value(v);
      }
    }
    __syncthreads();
    if (threadIdx.x < cols) {
      const int c = threadIdx.x;
      if (!(gated && !active[c])) update(c, vals[c], vals[c]);
    }
    if (use_cond && (op == OP_START || op == OP_CHECK || op == OP_START_RHS)) {
      __syncthreads();
      if (threadIdx.x == 0) {
        int a = 0;
        for (int c = 0; c < cols; ++c) a |= active[c];
        cudaGraphSetConditional(cond, a ? 1u : 0u);
      }
    }
  }

  // CG start from ||b||^2 = rr (bnorm and max_b set)
  __device__ void start(int c, CGScalars& g, double rr) const {
    g.atol = ktol * g.bnorm;  // _get_atol_rtol: max(atol=0, rtol*||b||)
    g.atol2 = g.atol * g.atol;
    g.iters = 0;
    g.info = 0;
    g.rho_prev = 0;
    g.beta = 0;
    g.beta_t = 0.0f;
    g.rr = rr;
    g.net_on = use_net;
    g.restart = 0;
    // zero RHS (tensor_stokes.py:309-311) or already converged: no update
    const bool go = (g.max_b != 0.0) && !(sqrt(g.rr) < g.atol) && (g.bnorm == g.bnorm);
    active[c] = go ? 1 : 0;
  }

  // s[k] / m[k]: the folded sum / maximum of slot k (one array, per maxmask)
  __device__ void update(int c, const double* s, const double* m) const {
    CGScalars& g = cg[c];
    switch (op) {
      case OP_MEAN_B:
        g.mean_b = s[0] * inv_np;
        g.mean_b_t = float(g.mean_b);
        break;
      case OP_START_RHS:  // fused pressure right-hand side and start (FP32 inner solves):
        // sums of b and b^2 and max|b| of the uncentred b; ||b - mean|| from them
        g.mean_b = s[0] * inv_np;
        g.mean_b_t = float(g.mean_b);
        g.bnorm = sqrt(fmax(s[1] - s[0] * g.mean_b, 0.0));
        g.max_b = m[2];
        start(c, g, g.bnorm * g.bnorm);
        break;
      case OP_START: {
        g.bnorm = sqrt(s[0]);
        g.max_b = m[1];
        start(c, g, s[0]);
        break;
      }
      case OP_RHO:
        g.rho = s[0];
        g.beta = g.iters > 0 ? g.rho / g.rho_prev : 0.0;
        g.beta_t = float(g.beta);
        break;
      case OP_ALPHA:
        g.mean_q = s[1] * inv_np;
        g.pq = s[0] - s[1] * s[2] * inv_np;  // p . (q - mean(q))
        g.alpha = g.rho / g.pq;
        g.alpha_t = float(g.alpha);
        g.mean_q_t = float(g.mean_q);
        break;
      case OP_CHECK:
        g.rr = s[0];
        g.iters += 1;
        g.cum_iters += 1;
        if (g.net_on) g.cum_net_iters += 1;
        g.rho_prev = g.rho;
        if (g.rr < g.atol2) {  // ||r|| < atol without the FP64 square root
          active[c] = 0;
        } else if (g.net_on && (g.iters >= net_maxit || !(g.rr == g.rr))) {
          // the learned attempt did not converge: plain PCG from zero
          g.net_on = 0;
          g.restart = 1;
          g.cum_fallbacks += 1;
          g.iters = 0;
          g.rho_prev = 0;
          g.beta = 0;
          g.beta_t = 0.0f;
          g.rr = g.bnorm * g.bnorm;
        } else if (g.iters >= maxit || !(g.rr == g.rr)) {
          active[c] = 0;
          g.info = maxit;
        }
        break;
      case OP_FCG: {
        // z = M r + net(r): mean of z, rho = r.(z - mean), Polak-Ribiere beta
        // (r - r_old).(z - mean) / rho_prev (flexible CG)
        g.mean_z = s[0] * inv_np;
        g.mean_z_t = float(g.mean_z);
        g.rho = s[1] - g.mean_z * s[3];
        const double rzo = s[2] - g.mean_z * s[4];
        g.beta = g.iters > 0 ? (g.rho - rzo) / g.rho_prev : 0.0;
        g.beta_t = float(g.beta);
        g.restart = 0;
        break;
      }
      case OP_MEAN_X:
        g.mean_q = s[0] * inv_np;
        g.mean_q_t = float(g.mean_q);
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
};

template <typename T>
inline CGFin<T> make_fin(const Plan* P, const Exec& X, int op, int nb, int K, int cols) {
  return CGFin<T>{op, X.partial ? X.partial : P->partial, nb, K, cols, P->cg, P->active, P->g.np,
                  X.ktol > 0 ? X.ktol : P->ktol, P->maxit, P->checks, X.graph ? 1 : 0, X.cond,
                  X.net && P->net ? 1 : 0, P->net_maxit, 1.0 / P->g.np};
}

// ------------------------------------------------------------- launching ---
constexpr int kVmax = 8;

template <typename T>
inline RowArgs<T> row_args(const TBlockDev<T>& a, const TBlockDev<T>* b, const int* active) {
  RowArgs<T> r;
  r.blk[0] = a;
  r.blk[0].groups = (a.rows + 2 * a.px - 1) / (2 * a.px);
  r.nblk = 1;
  if (b) {
    r.blk[1] = *b;
    r.blk[1].groups = (b->rows + 2 * b->px - 1) / (2 * b->px);
    r.nblk = 2;
  }
  r.active = active;
  return r;
}

template <typename T>
inline ColArgs<T> col_args(const TBlockDev<T>& a, const TBlockDev<T>* b, const int* active, int mode,
                           const double* shift, T thr) {
  ColArgs<T> r;
  r.blk[0] = a;
  r.blk[0].groups = (a.cols + a.wy - 1) / a.wy;
  r.nblk = 1;
  if (b) {
    r.blk[1] = *b;
    r.blk[1].groups = (b->cols + b->wy - 1) / b->wy;
    r.nblk = 2;
  }
  r.active = active;
  r.mode = mode;
  r.shift = shift;
  r.thr = thr;
  return r;
}

template <typename T>
inline int total_groups(const RowArgs<T>& a) { return a.blk[0].groups + (a.nblk > 1 ? a.blk[1].groups : 0); }
template <typename T>
inline int total_groups(const ColArgs<T>& a) { return a.blk[0].groups + (a.nblk > 1 ? a.blk[1].groups : 0); }

// Opt in to more than the default 48 KB of shared memory per CTA.  The
// default covers static plus dynamic bytes, and the finishers' static arrays
// take a few KB, so the opt-in starts well below 48 KB of dynamic memory.
template <class K>
inline void set_smem(K kernel, size_t bytes) {
  if (bytes > 40 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
}

// Row pairs per CTA of a specialised row pass (at least 64 threads per CTA).
template <typename T>
inline int p2_pairs(const TBlockDev<T>& B) {
  const int G = B.fx.L / kE;
  return std::max(B.px, std::max(1, 64 / G));
}
template <typename T>
inline bool row_p2(const TBlockDev<T>& B) { return B.fx.nstages > 0 && is_p2_length(B.fx.L); }
template <typename T>
inline bool col_p2(const TBlockDev<T>& B) { return B.fy.nstages > 0 && is_p2_length(B.fy.L); }

template <typename T>
struct Launcher {
  const Transforms<T>& t;
  cudaStream_t s;
  long long* counter;
  // Optional fork stream: the u- and v-block passes are independent, so they
  // run concurrently (s2 joins and leaves through events; graph-capturable).
  cudaStream_t s2 = nullptr;
  cudaEvent_t ef = nullptr, ej = nullptr;

  template <class F>
  void two_blocks(F launch_one) const {
    if (s2) {
      cudaEventRecord(ef, s);
      cudaStreamWaitEvent(s2, ef, 0);
      launch_one(0, s);
      launch_one(1, s2);
      cudaEventRecord(ej, s2);
      cudaStreamWaitEvent(s, ej, 0);
    } else {
      launch_one(0, s);
      launch_one(1, s);
    }
  }

  // number of CTAs along x of a row pass over one block
  int row_grid(const TBlockDev<T>& B) const {
    const int P = row_p2(B) ? p2_pairs(B) : B.px;
    return (B.rows + 2 * P - 1) / (2 * P);
  }

  // One specialised pass over block B (bk: 0 = u or the only block, 1 = v) on stream st.
  template <class Src>
  void row_forward_p2(const TBlockDev<T>& B, int bk, cudaStream_t st, Src src, int cols, const int* active) const {
    const int P = p2_pairs(B);
    const int shape = p2_shape<T>(B, B.fx.L, P, B.shape[0]);
    const bool split = shape == P2_SPLIT;
    const int G = p2_tpl(B.fx.L, shape);
    TBlockDev<T> Bl = B;
    Bl.tpl = G;
    const size_t sm = p2_smem<T>(B.fx.L, P);
#define MACSAV_RF(LL, GG)                                                      \
  {                                                                            \
    auto k = k_row_forward_p2<T, LL, Src, GG>;                                 \
    set_smem(k, sm);                                                           \
    launch_k(k, dim3(row_grid(B), cols), P * G, sm, st, Bl, active, src, bk);  \
  }
#define MACSAV_RF1(LL) MACSAV_RF(LL, LL / kE)
    if (!split) {
      MACSAV_P2_SWITCH(B.fx.L, MACSAV_RF1)
    } else {
      MACSAV_SPLIT_SWITCH(B.fx.L, MACSAV_RF)
    }
#undef MACSAV_RF1
#undef MACSAV_RF
    ++*counter;
  }
  template <class Dst, class Fin>
  void row_inverse_p2(const TBlockDev<T>& B, int bk, cudaStream_t st, Dst dst, int cols, const int* active,
                      double* partial, Fin fin, unsigned int* done) const {
    const int P = p2_pairs(B);
    const int shape = p2_shape<T>(B, B.fx.L, P, B.shape[2]);
    const bool split = shape == P2_SPLIT;
    const int G = p2_tpl(B.fx.L, shape);
    TBlockDev<T> Bl = B;
    Bl.tpl = G;
    const size_t sm = p2_smem<T>(B.fx.L, P);
#define MACSAV_RI(LL, GG)                                                                            \
  {                                                                                                  \
    auto k = k_row_inverse_p2<T, LL, Dst, Fin, GG>;                                                  \
    set_smem(k, sm);                                                                                 \
    launch_k(k, dim3(row_grid(B), cols), P * G, sm, st, Bl, active, dst, bk, partial, fin, done);  \
  }
#define MACSAV_RI1(LL) MACSAV_RI(LL, LL / kE)
    if (!split) {
      MACSAV_P2_SWITCH(B.fx.L, MACSAV_RI1)
    } else {
      MACSAV_SPLIT_SWITCH(B.fx.L, MACSAV_RI)
    }
#undef MACSAV_RI1
#undef MACSAV_RI
    ++*counter;
  }
  void column_p2(const TBlockDev<T>& B, cudaStream_t st, int cols, const int* active, int mode, const double* shift,
                 T thr) const {
    const int NL = B.wy / 2;
    const int shape = p2_shape<T>(B, B.fy.L, NL, B.shape[1]);
    const bool split = shape == P2_SPLIT;
    const int G = p2_tpl(B.fy.L, shape);
    TBlockDev<T> Bl = B;
    Bl.tpl = G;
    const size_t sm = p2_smem<T>(B.fy.L, NL);
    const int grid = (B.cols + B.wy - 1) / B.wy;
#define MACSAV_CO(LL, GG)                                                              \
  {                                                                                    \
    auto k = k_column_p2<T, LL, GG>;                                                   \
    set_smem(k, sm);                                                                   \
    launch_k(k, dim3(grid, cols), NL * G, sm, st, Bl, active, mode, shift, thr);      \
  }
#define MACSAV_CO1(LL) MACSAV_CO(LL, LL / kE)
    if (!split) {
      MACSAV_P2_SWITCH(B.fy.L, MACSAV_CO1)
    } else {
      MACSAV_SPLIT_SWITCH(B.fy.L, MACSAV_CO)
    }
#undef MACSAV_CO1
#undef MACSAV_CO
    ++*counter;
  }

  template <class Src>
  void row_forward(const TBlockDev<T>& a, const TBlockDev<T>* b, size_t smem, Src src, int cols,
                   const int* active) const {
    if (row_p2(a) && (!b || row_p2(*b))) {
      auto one = [&](int bk, cudaStream_t st) { row_forward_p2(bk ? *b : a, bk, st, src, cols, active); };
      if (b) two_blocks(one);
      else one(0, s);
      return;
    }
    RowArgs<T> r = row_args(a, b, active);
    auto k = k_row_forward<T, kVmax, Src>;
    set_smem(k, smem);
    launch_k(k, dim3(total_groups(r), cols), kFFTThreads, smem, s, r, src);
    ++*counter;
  }
  template <class Dst, class Fin>
  void row_inverse(const TBlockDev<T>& a, const TBlockDev<T>* b, size_t smem, Dst dst, int cols, const int* active,
                   double* partial, Fin fin, unsigned int* done) const {
    if (row_p2(a) && (!b || row_p2(*b)) && (!partial || !b)) {
      auto one = [&](int bk, cudaStream_t st) {
        row_inverse_p2(bk ? *b : a, bk, st, dst, cols, active, partial, fin, done);
      };
      if (b) two_blocks(one);
      else one(0, s);
      return;
    }
    RowArgs<T> r = row_args(a, b, active);
    auto k = k_row_inverse<T, kVmax, Dst, Fin>;
    set_smem(k, smem);
    launch_k(k, dim3(total_groups(r), cols), kFFTThreads, smem, s, r, dst, partial, fin, done);
    ++*counter;
  }
  void column(const TBlockDev<T>& a, const TBlockDev<T>* b, size_t smem, int cols, const int* active, int mode,
              const double* shift, T thr) const {
    if (col_p2(a) && (!b || col_p2(*b))) {
      auto one = [&](int bk, cudaStream_t st) { column_p2(bk ? *b : a, st, cols, active, mode, shift, thr); };
      if (b) two_blocks(one);
      else one(0, s);
      return;
    }
    ColArgs<T> r = col_args(a, b, active, mode, shift, thr);
    auto k = k_column<T, kVmax>;
    set_smem(k, smem);
    launch_k(k, dim3(total_groups(r), cols), kFFTThreads, smem, s, r);
    ++*counter;
  }

  // Velocity inverse (forward rows, column weights, inverse rows) of both
  // blocks.  With a fork stream and specialised passes the u chain runs on s
  // and the v chain on s2, forked and joined once, so neither waits for the
  // other between its passes.
  // `pre_v(stream)` launches independent work at the head of the v chain
  // (or before the passes when there is no fork).
  struct NoPre {
    void operator()(cudaStream_t) const {}
  };
  template <class Src, class Dst, class Pre = NoPre>
  void velocity_solve(Src src, Dst dst, int cols, const int* active, const double* shift, Pre pre_v = Pre{}) const {
    const bool p2 = row_p2(t.u) && row_p2(t.v) && col_p2(t.u) && col_p2(t.v);
    if (!p2 || !s2) {
      pre_v(s);
      row_forward_uv(src, cols, active);
      column_uv(cols, active, shift);
      row_inverse_uv(dst, cols, active);
      return;
    }
    cudaEventRecord(ef, s);
    cudaStreamWaitEvent(s2, ef, 0);
    pre_v(s2);
    for (int bk = 0; bk < 2; ++bk) {
      const TBlockDev<T>& B = bk ? t.v : t.u;
      const cudaStream_t st = bk ? s2 : s;
      row_forward_p2(B, bk, st, src, cols, active);
      column_p2(B, st, cols, active, W_HELMHOLTZ, shift, T(0));
      row_inverse_p2(B, bk, st, dst, cols, active, nullptr, NoFin{}, nullptr);
    }
    cudaEventRecord(ej, s2);
    cudaStreamWaitEvent(s, ej, 0);
  }

  template <class Src>
  void row_forward_uv(Src src, int cols, const int* active) const {
    row_forward(t.u, &t.v, t.smem_row_uv, src, cols, active);
  }
  template <class Dst>
  void row_inverse_uv(Dst dst, int cols, const int* active) const {
    row_inverse(t.u, &t.v, t.smem_row_uv, dst, cols, active, nullptr, NoFin{}, nullptr);
  }
  void column_uv(int cols, const int* active, const double* shift) const {
    column(t.u, &t.v, t.smem_col_uv, cols, active, W_HELMHOLTZ, shift, T(0));
  }
  template <class Src>
  void row_forward_p(Src src, int cols, const int* active) const {
    row_forward(t.p, nullptr, t.smem_row_p, src, cols, active);
  }
  template <class Dst, class Fin>
  void row_inverse_p(Dst dst, int cols, const int* active, double* partial, Fin fin, unsigned int* done) const {
    row_inverse(t.p, nullptr, t.smem_row_p, dst, cols, active, partial, fin, done);
  }
  void column_p(int cols, const int* active, const double* shift, T thr) const {
    column(t.p, nullptr, t.smem_col_p, cols, active, W_POISSON, shift, thr);
  }
  int groups_row_p() const {
    if (row_p2(t.p)) return row_grid(t.p);
    return (t.p.rows + 2 * t.p.px - 1) / (2 * t.p.px);
  }
};

}  // namespace macsav
