// Shifted Stokes solve by DST/DCT velocity inverses inside a pressure Schur PCG.
//
// Restates TensorStokes.solve (solver/mac/tensor_stokes.py:245-364) and the
// SciPy 1.18.1 conjugate-gradient loop it calls (x0 = 0; stop when
// ||r||_2 < rtol ||b||_2, tested before every update; the iteration count is
// the number of updates; info = maxiter when the loop is exhausted).
//
// Device data per right-hand-side column c: b (pressure RHS), x (pressure),
// r (residual), z (preconditioned residual), p (search direction), q (S p).
// Every Krylov scalar lives on the device (CGScalars).  Each reduction kernel
// writes per-block partials and its last block folds them in a fixed order
// and updates the scalars (no separate scalar launches).  Each kernel of the
// loop is predicated on the column's `active` flag, so the host (or a CUDA
// graph conditional node) only needs the flags to know when to stop.
#include <cmath>
#include <cstdio>
#include <type_traits>

#include "solver.cuh"

namespace macsav {

// Blocks of a grid-stride reduction kernel: enough to fill every SM twice,
// no more (each block costs a block-level reduction, and the last block folds
// one partial per block).
static int g_red_cap = 304;
inline int red_blocks(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : (b > g_red_cap ? g_red_cap : b));
}
// Light kernels without a block reduction take one element (or one 16-byte
// vector) per thread: the whole range in flight at once, up to full occupancy.
inline int flat_blocks(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}
#ifndef MACSAV_RED_PER_SM
#define MACSAV_RED_PER_SM 2
#endif
void set_reduction_cap(int sms) { g_red_cap = sms > 0 ? MACSAV_RED_PER_SM * sms : 304; }

// ------------------------------------------------------------ CG kernels ---
// abs_key of a T value (as the key of the same value in double).
template <typename T>
__device__ __forceinline__ unsigned long long abs_key_t(T v) {
  if constexpr (sizeof(T) == 4) return abs_key(f2d_bits(v));
  else return abs_key(v);
}

// b = rd - D w (rd: continuity defect of a correction solve, may be null);
// last block: mean of b (OP_MEAN_B).
template <typename T, typename WIn>
__global__ void __launch_bounds__(kThreads) k_pressure_rhs(GridDev g, const WIn* w, long long ws, T* b, long long cs,
                                                           const float* rd, double* partial, CGFin<T> fin,
                                                           unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const T ihx = T(g.ihx), ihy = T(g.ihy);
  Acc<T> acc[1];
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.np; idx += gridDim.x * blockDim.x) {
    const int j = idx / g.nx, i = idx - j * g.nx;
    T v = -D_atT<T>(w + c * ws, g, j, i, ihx, ihy);
    if (rd) v += load_as<T>(rd + c * (long long)g.np + idx);
    b[c * cs + idx] = v;
    acc[0].add(v);
  }
  write_sums<T, 1>(acc, partial, 1);
  last_block_finish(fin, done);
}

// b -= mean; x = 0; r = b; last block: ||b||, max|b| and the start (OP_START).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_start(int np, T* b, T* x, T* r, long long cs, const CGScalars* cg,
                                                       double* partial, CGFin<T> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const T mean = cg_mean_b<T>(cg[c]);
  Acc<T> s[1];
  T mt = T(0);
  bool bad = false;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
    const long long i = c * cs + idx;
    const T v = b[i] - mean;
    b[i] = v;
    r[i] = v;
    x[i] = T(0);
    s[0].add(v * v);
    const T av = v < T(0) ? -v : v;
    bad |= !(av == av);
    mt = av > mt ? av : mt;
  }
  unsigned long long key[1] = {bad ? 0x7ff8000000000000ull : abs_key_t<T>(mt)};
  write_sums<T, 1>(s, partial, 2);
  write_keys<1>(key, partial, 2, 1);
  last_block_finish(fin, done);
}

// Fused start of an FP32 inner solve: b = rd - D w (stored uncentred);
// last block: mean, ||b - mean|| and max|b| and the CG start (OP_START_RHS).
// The first iteration's preconditioner pass forms r = b - mean (SrcCellsStart),
// so no separate start kernel runs.
template <typename T, typename WIn>
__global__ void __launch_bounds__(kThreads) k_pressure_rhs_start(GridDev g, const WIn* w, long long ws, T* b, T* x,
                                                                 long long cs, const float* rd, double* partial,
                                                                 CGFin<T> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const T ihx = T(g.ihx), ihy = T(g.ihy);
  Acc<T> acc[2];
  T mt = T(0);
  bool bad = false;
  auto take = [&](T v) {
    acc[0].add(v);
    acc[1].add(v * v);
    const T av = v < T(0) ? -v : v;
    bad |= !(av == av);
    mt = av > mt ? av : mt;
  };
  bool vec = false;
  if constexpr (sizeof(T) == 4 && sizeof(WIn) == 4) {
    // FP32: four cells of a row per thread (16-byte vectors of b, x, rd)
    vec = (g.nx & 3) == 0 && (cs & 3) == 0;
    if (vec) {
      const long long stride = (long long)gridDim.x * blockDim.x;
      float4* b4 = reinterpret_cast<float4*>(b + c * cs);
      float4* x4 = reinterpret_cast<float4*>(x + c * cs);
      const float4* r4 = rd ? reinterpret_cast<const float4*>(rd + c * (long long)g.np) : nullptr;
      for (long long i4 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i4 < (g.np >> 2); i4 += stride) {
        const int e = int(i4 << 2), j = e / g.nx, i0 = e - j * g.nx;
        const float4 d = D_at4(w + c * ws, g, j, i0, ihx, ihy);
        float4 v = make_float4(-d.x, -d.y, -d.z, -d.w);
        if (r4) {
          const float4 rr = r4[i4];
          v = make_float4(v.x + rr.x, v.y + rr.y, v.z + rr.z, v.w + rr.w);
        }
        b4[i4] = v;
        x4[i4] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // x0 = 0 (also the answer of a column that never starts)
        take(v.x);
        take(v.y);
        take(v.z);
        take(v.w);
      }
    }
  }
  if (!vec) {
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.np; idx += gridDim.x * blockDim.x) {
      const int j = idx / g.nx, i = idx - j * g.nx;
      T v = -D_atT<T>(w + c * ws, g, j, i, ihx, ihy);
      if (rd) v += load_as<T>(rd + c * (long long)g.np + idx);
      b[c * cs + idx] = v;
      x[c * cs + idx] = T(0);  // x0 = 0 (also the answer of a column that never starts)
      take(v);
    }
  }
  unsigned long long key[1] = {bad ? 0x7ff8000000000000ull : abs_key_t<T>(mt)};
  write_sums<T, 2>(acc, partial, 3);
  write_keys<1>(key, partial, 3, 2);
  last_block_finish(fin, done);
}

// D w at the four cells (j, i0..i0+3) of one row (nx a multiple of 4), in the
// operation order of D_atT: the five u faces and eight v faces they touch are
// loaded together.
__device__ __forceinline__ float4 D_at4(const float* w, const GridDev& g, int j, int i0, float ihx, float ihy) {
  const float* u = w + (long long)j * (g.nx - 1);
  const float* vn = w + g.nu + (long long)j * g.nx;
  const float* vs = vn - g.nx;
  float ul[5], n4[4], s4[4];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    const int i = i0 - 1 + t;
    ul[t] = (i >= 0 && i < g.nx - 1) ? u[i] : 0.0f;
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    n4[t] = j < g.ny - 1 ? vn[i0 + t] : 0.0f;
    s4[t] = j > 0 ? vs[i0 + t] : 0.0f;
  }
  float r[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = i0 + t;
    float v = 0.0f;
    if (i < g.nx - 1) v += ul[t + 1] * ihx;
    if (i > 0) v -= ul[t] * ihx;
    if (j < g.ny - 1) v += n4[t] * ihy;
    if (j > 0) v -= s4[t] * ihy;
    r[t] = v;
  }
  return make_float4(r[0], r[1], r[2], r[3]);
}

// q = D w; last block: alpha from p.q, sum q, sum p (OP_ALPHA), p = z + beta p.
template <typename T, typename WIn>
__global__ void __launch_bounds__(kThreads) k_div_q(GridDev g, const WIn* w, long long ws, T* q, const T* z, const T* p,
                                                    long long cs, const CGScalars* cg, const int* active,
                                                    double* partial, CGFin<T> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  Acc<T> a[3];
  if (active[c]) {
    const bool first = cg[c].iters == 0;
    const T beta = cg_beta<T>(cg[c]);
    const T ihx = T(g.ihx), ihy = T(g.ihy);
    bool vec = false;
    if constexpr (sizeof(T) == 4 && sizeof(WIn) == 4) {
      // FP32: four cells of a row per thread (16-byte vectors of q, z, p)
      vec = (g.nx & 3) == 0 && (cs & 3) == 0;
      if (vec) {
        const long long stride = (long long)gridDim.x * blockDim.x;
        float4* q4 = reinterpret_cast<float4*>(q + c * cs);
        const float4* z4 = reinterpret_cast<const float4*>(z + c * cs);
        const float4* p4 = reinterpret_cast<const float4*>(p + c * cs);
        for (long long i4 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i4 < (g.np >> 2); i4 += stride) {
          const int e = int(i4 << 2), j = e / g.nx, i0 = e - j * g.nx;
          const float4 qv = D_at4(w + c * ws, g, j, i0, ihx, ihy);
          q4[i4] = qv;
          const float4 zz = z4[i4];
          float4 pd = zz;
          if (!first) {
            const float4 pp = p4[i4];
            pd = make_float4(zz.x + beta * pp.x, zz.y + beta * pp.y, zz.z + beta * pp.z, zz.w + beta * pp.w);
          }
          a[0].add(pd.x * qv.x);
          a[1].add(qv.x);
          a[2].add(pd.x);
          a[0].add(pd.y * qv.y);
          a[1].add(qv.y);
          a[2].add(pd.y);
          a[0].add(pd.z * qv.z);
          a[1].add(qv.z);
          a[2].add(pd.z);
          a[0].add(pd.w * qv.w);
          a[1].add(qv.w);
          a[2].add(pd.w);
        }
      }
    }
    if (!vec) {
      for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < g.np; idx += gridDim.x * blockDim.x) {
        const int j = idx / g.nx, i = idx - j * g.nx;
        const long long k = c * cs + idx;
        const T qv = D_atT<T>(w + c * ws, g, j, i, ihx, ihy);
        q[k] = qv;
        const T pd = first ? z[k] : T(z[k] + beta * p[k]);
        a[0].add(pd * qv);
        a[1].add(qv);
        a[2].add(pd);
      }
    }
  }
  write_sums<T, 3>(a, partial, 3);
  last_block_finish(fin, done);
}

// p = z + beta p; x += alpha p; r -= alpha (q - mean q); last block: ||r||
// and the convergence test (OP_CHECK).  r_old (flexible CG) keeps the old r.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_cg_update(int np, T* x, T* r, T* p, const T* z, const T* q, T* r_old,
                                                        long long cs, const CGScalars* cg, const int* active,
                                                        double* partial, CGFin<T> fin, unsigned int* done,
                                                        const T* wv, T* wacc, long long vsz) {
  pdl_wait();
  const int c = blockIdx.y;
  Acc<T> acc[1];
  if (active[c]) {
    const bool first = cg[c].iters == 0;
    const T beta = cg_beta<T>(cg[c]), alpha = cg_alpha<T>(cg[c]), mq = cg_mean_q<T>(cg[c]);
    const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    bool vec = false;
    if constexpr (sizeof(T) == 4) {
      // FP32: 16-byte vectors of four cells (the same arithmetic per cell),
      // four times the bytes in flight per load of these streaming loops
      vec = (np & 3) == 0 && (cs & 3) == 0;
      if (vec) {
        float4* x4 = reinterpret_cast<float4*>(x + c * cs);
        float4* r4 = reinterpret_cast<float4*>(r + c * cs);
        float4* p4 = reinterpret_cast<float4*>(p + c * cs);
        const float4* z4 = reinterpret_cast<const float4*>(z + c * cs);
        const float4* q4 = reinterpret_cast<const float4*>(q + c * cs);
        float4* o4 = r_old ? reinterpret_cast<float4*>(r_old + c * cs) : nullptr;
        for (long long i = t0; i < (np >> 2); i += stride) {
          const float4 zz = z4[i], qq = q4[i], ro = r4[i], xx = x4[i];
          float4 pd = zz;
          if (!first) {
            const float4 pp = p4[i];
            pd = make_float4(zz.x + beta * pp.x, zz.y + beta * pp.y, zz.z + beta * pp.z, zz.w + beta * pp.w);
          }
          p4[i] = pd;
          x4[i] = make_float4(xx.x + alpha * pd.x, xx.y + alpha * pd.y, xx.z + alpha * pd.z, xx.w + alpha * pd.w);
          if (o4) o4[i] = ro;
          const float4 rv = make_float4(ro.x - alpha * (qq.x - mq), ro.y - alpha * (qq.y - mq),
                                        ro.z - alpha * (qq.z - mq), ro.w - alpha * (qq.w - mq));
          r4[i] = rv;
          acc[0].add(rv.x * rv.x);
          acc[0].add(rv.y * rv.y);
          acc[0].add(rv.z * rv.z);
          acc[0].add(rv.w * rv.w);
        }
      }
    }
    if (!vec) {
      for (long long idx = t0; idx < np; idx += stride) {
        const long long k = c * cs + idx;
        const T pd = first ? z[k] : T(z[k] + beta * p[k]);
        p[k] = pd;
        x[k] = x[k] + alpha * pd;
        const T ro = r[k];
        if (r_old) r_old[k] = ro;
        const T rv = ro - alpha * (q[k] - mq);
        r[k] = rv;
        acc[0].add(rv * rv);
      }
    }
    // the velocity follows x: wacc += alpha (mI+kK)^{-1} D^T pdir (wv holds
    // that velocity for this iteration's direction)
    if (wacc) {
      if constexpr (sizeof(T) == 4) {
        if ((vsz & 3) == 0) {
          float4* a4 = reinterpret_cast<float4*>(wacc + c * vsz);
          const float4* w4 = reinterpret_cast<const float4*>(wv + c * vsz);
          for (long long i = t0; i < (vsz >> 2); i += stride) {
            const float4 a = a4[i], w = w4[i];
            a4[i] = make_float4(a.x + alpha * w.x, a.y + alpha * w.y, a.z + alpha * w.z, a.w + alpha * w.w);
          }
        } else {
          for (long long i = t0; i < vsz; i += stride) wacc[c * vsz + i] += alpha * wv[c * vsz + i];
        }
      } else {
        for (long long i = t0; i < vsz; i += stride) wacc[c * vsz + i] += alpha * wv[c * vsz + i];
      }
    }
  }
  write_sums<T, 1>(acc, partial, 1);
  last_block_finish(fin, done);
}

// ------------------------------------------- learned preconditioner (FCG) ---
// Columns whose learned attempt failed restart plain PCG from zero: x = 0,
// r = b, and the accumulated velocity back to its start (mI+kK)^{-1} ru,
// kept in wacc0 (sz elements per column).
__global__ void __launch_bounds__(kThreads) k_fcg_restart(int np, const float* b, float* x, float* r, long long cs,
                                                          const CGScalars* cg, float* wacc, const float* wacc0,
                                                          long long sz) {
  pdl_wait();
  const int c = blockIdx.y;
  if (!cg[c].restart) return;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) {
    const long long k = c * cs + idx;
    x[k] = 0.0f;
    r[k] = b[k];
  }
  if (wacc && wacc0)
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < sz;
         idx += (long long)gridDim.x * blockDim.x)
      wacc[c * sz + idx] = wacc0[c * sz + idx];
}

// Network input scale 1/rms(r) and output scale rms(r) rho/rr (rho = r.Mr of
// the spectral preconditioner): the network sees unit-RMS residuals and
// answers in units of the spectral preconditioner's Rayleigh quotient.
// Columns without the network get 0 (a zero correction).
__global__ void k_net_scales(const CGScalars* cg, const int* active, int cols, int np, float* scale) {
  pdl_wait();
  const int c = threadIdx.x;
  if (c >= cols) return;
  const CGScalars& g = cg[c];
  const bool on = active[c] && g.net_on && g.rr > 0.0 && g.rho > 0.0;
  const double rms = on ? sqrt(g.rr / np) : 0.0;
  scale[c] = on ? float(1.0 / rms) : 0.0f;
  scale[cols + c] = on ? float(rms * g.rho / g.rr) : 0.0f;
}

// z += net output (add null: z unchanged); partial sums of z, r.z, r_old.z,
// r, r_old (OP_FCG).
__global__ void __launch_bounds__(kThreads) k_fcg_z(int np, float* z, const float* add, const float* r,
                                                    const float* r_old, long long cs, const CGScalars* cg,
                                                    const int* active, double* partial, CGFin<float> fin,
                                                    unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  Acc<float> a[5];
  auto take = [&](float zn, float rv, float ro) {
    a[0].add(zn);
    a[1].add(rv * zn);
    a[2].add(ro * zn);
    a[3].add(rv);
    a[4].add(ro);
  };
  if (active[c]) {
    const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if ((np & 3) == 0 && (cs & 3) == 0) {  // 16-byte vectors of four cells
      float4* z4 = reinterpret_cast<float4*>(z + c * cs);
      const float4* a4 = add ? reinterpret_cast<const float4*>(add + c * cs) : nullptr;
      const float4* r4 = reinterpret_cast<const float4*>(r + c * cs);
      const float4* o4 = reinterpret_cast<const float4*>(r_old + c * cs);
      for (long long i = t0; i < (np >> 2); i += stride) {
        float4 zn = z4[i];
        if (a4) {
          const float4 ad = a4[i];
          zn = make_float4(zn.x + ad.x, zn.y + ad.y, zn.z + ad.z, zn.w + ad.w);
          z4[i] = zn;
        }
        const float4 rv = r4[i], ro = o4[i];
        take(zn.x, rv.x, ro.x);
        take(zn.y, rv.y, ro.y);
        take(zn.z, rv.z, ro.z);
        take(zn.w, rv.w, ro.w);
      }
    } else {
      for (long long idx = t0; idx < np; idx += stride) {
        const long long k = c * cs + idx;
        const float zn = add ? z[k] + add[k] : z[k];
        z[k] = zn;
        take(zn, r[k], r_old[k]);
      }
    }
  }
  write_sums<float, 5>(a, partial, 5);
  last_block_finish(fin, done);
}

// z -= mean(z): the mean-zero projection of the flexible preconditioner.
__global__ void __launch_bounds__(kThreads) k_fcg_center(int np, float* z, long long cs, const CGScalars* cg,
                                                         const int* active) {
  pdl_wait();
  const int c = blockIdx.y;
  if (!active[c]) return;
  const float m = cg[c].mean_z_t;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x) z[c * cs + idx] -= m;
}

// Restricted network input: the mean of each f x f block of cells of r, times
// the column's input scale.  One thread per coarse cell and column.
__global__ void __launch_bounds__(kThreads) k_net_restrict(int ny, int nx, int f, const float* r, long long cs,
                                                           const float* scale, float* out) {
  pdl_wait();
  const int c = blockIdx.y;
  const int nyc = ny / f, nxc = nx / f;
  const float w = scale[c] / float(f * f);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nyc * nxc; idx += gridDim.x * blockDim.x) {
    const int jc = idx / nxc, ic = idx - jc * nxc;
    const float* src = r + c * cs + (long long)(jc * f) * nx + ic * f;
    float acc = 0.0f;
    for (int a = 0; a < f; ++a)
      for (int b = 0; b < f; ++b) acc += src[(long long)a * nx + b];
    out[(long long)c * nyc * nxc + idx] = w * acc;
  }
}

// Bilinear prolongation of the restricted network output to the cells: cell
// (j, i) sits at coarse position ((j + 1/2)/f - 1/2, (i + 1/2)/f - 1/2);
// beyond the outermost coarse centres the value is held constant.
__global__ void __launch_bounds__(kThreads) k_net_prolong(int ny, int nx, int f, const float* in, float* out,
                                                          long long cs) {
  pdl_wait();
  const int c = blockIdx.y;
  const int nyc = ny / f, nxc = nx / f;
  const float* src = in + (long long)c * nyc * nxc;
  const float inv = 1.0f / float(f);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < ny * nx; idx += gridDim.x * blockDim.x) {
    const int j = idx / nx, i = idx - j * nx;
    const float yc = fminf(fmaxf((j + 0.5f) * inv - 0.5f, 0.0f), float(nyc - 1));
    const float xc = fminf(fmaxf((i + 0.5f) * inv - 0.5f, 0.0f), float(nxc - 1));
    const int j0 = min(int(yc), nyc - 1), i0 = min(int(xc), nxc - 1);
    const int j1 = min(j0 + 1, nyc - 1), i1 = min(i0 + 1, nxc - 1);
    const float ty = yc - float(j0), tx = xc - float(i0);
    const float a = src[j0 * nxc + i0] + tx * (src[j0 * nxc + i1] - src[j0 * nxc + i0]);
    const float b = src[j1 * nxc + i0] + tx * (src[j1 * nxc + i1] - src[j1 * nxc + i0]);
    out[c * cs + idx] = a + ty * (b - a);
  }
}

__global__ void k_reset_counters(CGScalars* cg, int cols) {
  pdl_wait();
  const int c = threadIdx.x;
  if (c < cols) {
    cg[c].cum_iters = 0;
    cg[c].cum_net_iters = 0;
    cg[c].cum_fallbacks = 0;
  }
}

void reset_cg_counters(Plan* P, int cols, cudaStream_t s) {
  launch_k(k_reset_counters, 1, 32, 0, s, P->cg, cols);
  ++P->launches;
}

// out = x - mean (the mean held in cg[c].mean_q when `center`); partial sum
// of out; last block: the new mean (OP_MEAN_X).  FP64 output.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_center_cells(int np, const T* x, long long xs, double* out,
                                                           long long os, const CGScalars* cg, int center,
                                                           double* partial, CGFin<double> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const double mean = center ? cg[c].mean_q : 0.0;
  Acc<double> acc[1];
  const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  bool vec = false;
  if constexpr (sizeof(T) == 8) {  // pairs on 16-byte vectors
    vec = (np & 1) == 0 && (xs & 1) == 0 && (os & 1) == 0 &&
          ((reinterpret_cast<unsigned long long>(x) | reinterpret_cast<unsigned long long>(out)) & 15) == 0;
    if (vec) {
      const double2* x2 = reinterpret_cast<const double2*>(x + c * xs);
      double2* o2 = out ? reinterpret_cast<double2*>(out + c * os) : nullptr;
      for (long long i = t0; i < (np >> 1); i += stride) {
        const double2 xv = x2[i];
        const double2 v = make_double2(xv.x - mean, xv.y - mean);
        if (o2) o2[i] = v;
        acc[0].add(v.x);
        acc[0].add(v.y);
      }
    }
  }
  if (!vec) {
    for (long long idx = t0; idx < np; idx += stride) {
      const double v = double(x[c * xs + idx]) - mean;
      if (out) out[c * os + idx] = v;
      acc[0].add(v);
    }
  }
  write_sums<double, 1>(acc, partial, 1);
  last_block_finish(fin, done);
}

__global__ void __launch_bounds__(kThreads) k_shift_cells(int np, double* out, long long os, const CGScalars* cg) {
  pdl_wait();
  const int c = blockIdx.y;
  const double mean = cg[c].mean_q;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < np; idx += gridDim.x * blockDim.x)
    out[c * os + idx] -= mean;
}

// Closing checks (tensor_stokes.py:329-351): defect = m u + k K u - D^T p - f.
// Key slots: max|defect|, max|f|, max|u|, max|D u|, nonfinite f, nonfinite u/p.
__global__ void __launch_bounds__(kThreads) k_stokes_check(GridDev g, const double* vel, const double* pres,
                                                           const double* f, long long vs, long long ps,
                                                           const double* shift, double* partial,
                                                           CGFin<double> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const double mass = shift[2 * c], visc = shift[2 * c + 1];
  const double* u = vel + c * vs;
  const double* pp = pres + c * ps;
  const double* ff = f + c * vs;
  unsigned long long m[6] = {0, 0, 0, 0, 0, 0};
  constexpr unsigned long long kInf = 0x7ff0000000000000ull;
  const int n = g.size > g.np ? g.size : g.np;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (idx < g.size) {
      const double fe = ff[idx], ue = u[idx];
      const double d = mass * ue + visc * K_at(u, g, idx) - Dt_at(pp, g, idx) - fe;
      const unsigned long long kf = abs_key(fe), ku = abs_key(ue);
      m[0] = max(m[0], abs_key(d));
      m[1] = max(m[1], kf);
      m[2] = max(m[2], ku);
      if (kf >= kInf) m[4] = 1;
      if (ku >= kInf) m[5] = 1;
    }
    if (idx < g.np) {
      const int j = idx / g.nx, i = idx - j * g.nx;
      m[3] = max(m[3], abs_key(D_at(u, g, j, i)));
      if (abs_key(pp[idx]) >= kInf) m[5] = 1;
    }
  }
  write_keys<6>(m, partial, 6, 0);
  last_block_finish(fin, done);
}

// ----------------------------------------------------------------- solve ---
// Velocity inverse (m I + k K)^{-1} of `src` rows into packed `dst`.
template <typename T, class Src, typename Out>
static void velocity_inverse(Plan* P, const Launcher<T>& L, Src src, Out* dst, long long dstride, int cols,
                             const int* active) {
  const GridDev& g = P->g;
  L.velocity_solve(src, DstPacked<T, Out>{dst, dstride, g.nu, g.nx - 1, g.nx}, cols, active, P->shift);
}

// One PCG iteration for every active column (all kernels predicated).  With
// the learned preconditioner (X.net, FP32 only) beta is the Polak-Ribiere form
// of flexible CG and, in iterations that evaluate the network (eval_net),
// z = M r + net(r), projected to mean zero; otherwise z = M r.
template <typename T>
static void cg_iteration(Plan* P, const Exec& X, const Launcher<T>& L, T* w, T* cells, int cols, T* wacc,
                         bool fused_first = false, bool eval_net = true) {
  const GridDev& g = P->g;
  const long long np = g.np, sz = g.size;
  T* b = cells;
  T* x = cells + 1 * np * cols;
  T* r = cells + 2 * np * cols;
  T* z = cells + 3 * np * cols;
  T* pd = cells + 4 * np * cols;
  T* q = cells + 5 * np * cols;
  const int rb = red_blocks(np);
  const cudaStream_t s = L.s;
  T* r_old = nullptr;
  bool net = false;
  if constexpr (std::is_same<T, float>::value) {
    net = X.net && P->net;
    if (net) {
      r_old = P->net_rold;
      launch_k(k_fcg_restart, dim3(rb, cols), kThreads, 0, s, g.np, b, x, r, np, P->cg, wacc,
               static_cast<const float*>(P->net_wacc0), sz);
      ++P->launches;
    }
  }
  (void)b;
  // z = M r = IDCT(g * DCT(r)); last block: rho = r . z, beta
  if (fused_first) L.row_forward_p(SrcCellsStart<T>{b, r, P->cg, np, g.nx}, cols, P->active);
  else L.row_forward_p(SrcCells<T, T>{r, np, g.nx}, cols, P->active);
  L.column_p(cols, P->active, P->shift, T(P->pthr));
  L.row_inverse_p(DstCellsDot<T>{z, r, np, g.nx}, cols, P->active, P->partial,
                  make_fin<T>(P, X, OP_RHO, L.groups_row_p(), 2, cols), P->done_counter);
  if constexpr (std::is_same<T, float>::value) {
    if (net) {
      const float* add = nullptr;
      if (eval_net) {
        launch_k(k_net_scales, 1, 32, 0, s, P->cg, P->active, cols, g.np, P->net_scale);
        ++P->launches;
        const int f = P->net_restrict;
        const long long net_before = P->net->launches;
        if (f == 1) {
          unet_forward(P->net, &P->netw, r, P->net_scale, cols, g.ny, g.nx, P->net_out, P->net_scale + cols, s);
        } else {
          const int npc = (g.ny / f) * (g.nx / f);
          launch_k(k_net_restrict, dim3(red_blocks(npc), cols), kThreads, 0, s, g.ny, g.nx, f,
                   static_cast<const float*>(r), np, static_cast<const float*>(P->net_scale), P->net_cin);
          unet_forward(P->net, &P->netw, P->net_cin, nullptr, cols, g.ny / f, g.nx / f, P->net_cout,
                       P->net_scale + cols, s);
          launch_k(k_net_prolong, dim3(rb, cols), kThreads, 0, s, g.ny, g.nx, f,
                   static_cast<const float*>(P->net_cout), P->net_out, np);
          P->launches += 2;
        }
        P->launches += P->net->launches - net_before;  // the network's own kernels count as the plan's
        add = P->net_out;
      }
      launch_k(k_fcg_z, dim3(rb, cols), kThreads, 0, s, g.np, z, add, r, r_old, np, P->cg, P->active, P->partial,
                                                  make_fin<float>(P, X, OP_FCG, rb, 5, cols), P->done_counter);
      ++P->launches;
      // the network's output is projected to mean zero; M r alone already is
      // (the preconditioner's Poisson inverse drops the zero mode), as in plain PCG
      if (eval_net) {
        launch_k(k_fcg_center, dim3(rb, cols), kThreads, 0, s, g.np, z, np, P->cg, P->active);
        ++P->launches;
      }
    }
  }
  // q = S pdir = D (mI+kK)^{-1} D^T pdir,  pdir = z + beta p
  velocity_inverse<T>(P, L, SrcLift<T, double, T>{nullptr, 0, z, pd, P->cg, np, g.nx, g.nu, T(g.ihx), T(g.ihy)}, w,
                      sz, cols, P->active);
  launch_k(k_div_q<T, T>, dim3(rb, cols), kThreads, 0, s, g, w, sz, q, z, pd, np, P->cg, P->active, P->partial,
                                                    make_fin<T>(P, X, OP_ALPHA, rb, 3, cols), P->done_counter);
  launch_k(k_cg_update<T>, dim3(rb, cols), kThreads, 0, s, g.np, x, r, pd, z, q, r_old, np, P->cg, P->active, P->partial,
                                                     make_fin<T>(P, X, OP_CHECK, rb, 1, cols), P->done_counter,
                                                     static_cast<const T*>(w), wacc, sz);
  P->launches += 2;
}

// PCG on S p = b for `cols` columns (SciPy cg semantics, see file header).
// On entry w holds (mI+kK)^{-1} f in T; on exit x holds the pressure iterate
// and P->cg the per-column counters.
template <typename T>
static int schur_pcg(Plan* P, Exec& X, const Launcher<T>& L, T* w, T* cells, int cols, const float* rd = nullptr,
                     T* wacc = nullptr) {
  const GridDev& g = P->g;
  const long long np = g.np, sz = g.size;
  T* b = cells;
  T* x = cells + 1 * np * cols;
  T* r = cells + 2 * np * cols;
  const int rb = red_blocks(np);
  const cudaStream_t s = X.s;
  const T* w0 = static_cast<const T*>(wacc ? wacc : w);
  // FP32 inner solves with an accumulated velocity start in one kernel; the
  // FP64 path keeps the reference's centring then start (SciPy semantics)
  const bool fused = std::is_same<T, float>::value && wacc != nullptr;
  if (X.graph) {
    cudaStreamCaptureStatus st;
    cudaGraph_t graph;
    if (cudaStreamGetCaptureInfo(s, &st, nullptr, &graph, nullptr, nullptr, nullptr) != cudaSuccess ||
        st != cudaStreamCaptureStatusActive)
      return MACSAV_ERR_CUDA;
    if (cudaGraphConditionalHandleCreate(&X.cond, graph, 0, cudaGraphCondAssignDefault) != cudaSuccess)
      return MACSAV_ERR_CUDA;
  }
  if (fused) {
    launch_k(k_pressure_rhs_start<T, T>, dim3(rb, cols), kThreads, 0, s, g, w0, sz, b, x, np, rd, P->partial,
             make_fin<T>(P, X, OP_START_RHS, rb, 3, cols), P->done_counter);
  } else {
    launch_k(k_pressure_rhs<T, T>, dim3(rb, cols), kThreads, 0, s, g, w0, sz, b, np, rd, P->partial,
             make_fin<T>(P, X, OP_MEAN_B, rb, 1, cols), P->done_counter);
  }
  ++P->launches;
  if (!X.graph) {
    if (!fused) {
      launch_k(k_cg_start<T>, dim3(rb, cols), kThreads, 0, s, g.np, b, x, r, np, P->cg, P->partial,
               make_fin<T>(P, X, OP_START, rb, 2, cols), P->done_counter);
      ++P->launches;
    }
    const int limit = P->maxit + (X.net && P->net ? P->net_maxit : 0);
    for (int it = 0; it < limit; ++it) {
      cudaMemcpyAsync(P->h_active, P->active, sizeof(int) * cols, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return MACSAV_ERR_CUDA;
      bool any = false;
      for (int c = 0; c < cols; ++c) any |= P->h_active[c] != 0;
      if (!any) break;
      bool log = false;
      if constexpr (std::is_same<T, double>::value) {
        // residual / iterate / preconditioned residual log (column 0)
        log = P->log_cap > 0 && P->log_n < P->log_cap;
        if (log) {
          cudaMemcpyAsync(P->log_r + P->log_n * np, cells + 2 * np * cols, sizeof(double) * np,
                          cudaMemcpyDeviceToDevice, s);
          cudaMemcpyAsync(P->log_x + P->log_n * np, cells + 1 * np * cols, sizeof(double) * np,
                          cudaMemcpyDeviceToDevice, s);
        }
      }
      cg_iteration<T>(P, X, L, w, cells, cols, wacc, fused && it == 0, P->net_every || it == 0);
      if constexpr (std::is_same<T, double>::value) {
        if (log) {
          cudaMemcpyAsync(P->log_z + P->log_n * np, cells + 3 * np * cols, sizeof(double) * np,
                          cudaMemcpyDeviceToDevice, s);
          ++P->log_n;
        }
      }
    }
    if constexpr (std::is_same<T, double>::value) {
      if (P->log_cap > 0)  // the converged iterate closes the log
        cudaMemcpyAsync(P->log_x + P->log_n * np, cells + 1 * np * cols, sizeof(double) * np,
                        cudaMemcpyDeviceToDevice, s);
    }
    return MACSAV_OK;
  }
  // graph mode: conditional WHILE node, body = one iteration
  cudaStreamCaptureStatus st;
  cudaGraph_t graph;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  // the start kernel's last block sets the loop condition
  if (!fused) {
    launch_k(k_cg_start<T>, dim3(rb, cols), kThreads, 0, s, g.np, b, x, r, np, P->cg, P->partial,
             make_fin<T>(P, X, OP_START, rb, 2, cols), P->done_counter);
    ++P->launches;
  }
  // The first iteration outside the loop: its kernels are predicated on the
  // columns' flags like the loop body's (a column that is already converged,
  // e.g. a zero right-hand side, does nothing), its convergence check sets
  // the loop condition, and nearly every solve needs it, so one conditional
  // body launch per solve is saved.
  cg_iteration<T>(P, X, L, w, cells, cols, wacc, fused);
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
  Launcher<T> Ls{L.t, X.side, L.counter, P->aux[1], P->evf[1], P->evj[1]};
  Exec Xs = X;
  Xs.s = X.side;
  cg_iteration<T>(P, Xs, Ls, w, cells, cols, wacc, false, P->net_every != 0);
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
  double* part = X.partial ? X.partial : P->partial;
  unsigned int* done = X.counter ? X.counter : P->done_counter;
  launch_k(k_center_cells<T>, dim3(rb, cols), kThreads, 0, s, P->g.np, x, np, nullptr, np, P->cg, 0, part,
                                                        make_fin<double>(P, X, OP_MEAN_X, rb, 1, cols), done);
  launch_k(k_center_cells<T>, dim3(rb, cols), kThreads, 0, s, P->g.np, x, np, pres, np, P->cg, 1, part,
                                                        make_fin<double>(P, X, OP_MEAN_X, rb, 1, cols), done);
  launch_k(k_shift_cells, dim3(flat_blocks(np), cols), kThreads, 0, s, P->g.np, pres, np, P->cg);
  P->launches += 3;
}

// ------------------------------------------- double-float defect groups ---
// The defect kernels below walk the packed velocity and the cells in groups
// of four consecutive elements per thread (16-byte loads and stores of the
// float pieces and pairs where the arrays allow it, one division per group,
// the left and right neighbours of a face from the group's registers).
//
// Double-float coefficients of m u + k K u - D^T p and of D: m, k/hx^2,
// k/hy^2, 1/hx, 1/hy (FP64 products rounded to double-float), formed once
// per block.
struct OpCoef {
  df32 m, kx, ky, gx, gy;
};
__device__ __forceinline__ OpCoef op_coef(const GridDev& g, const double* shift, int c) {
  __shared__ OpCoef sc;
  if (threadIdx.x == 0) {
    const double m = shift[2 * c], k = shift[2 * c + 1];
    sc = OpCoef{d2df(m), d2df(k * g.ihx2), d2df(k * g.ihy2), d2df(g.ihx), d2df(g.ihy)};
  }
  __syncthreads();
  return sc;
}

// s + c: a running double-float sum.  Each product of double-floats enters
// as p = a.hi b.hi and its low part (the FMA error of p plus the cross terms,
// rounded once: about 2^-48 of the product), the sum of p into s by an
// error-free two-sum whose error joins c.  Each term then carries an error
// of about 2^-48 of its own size, as a chain of double-float operations.
struct DFSum {
  float s, c;
  __device__ __forceinline__ void add(float p, float pe) {
    const df32 t = df_two_sum(s, p);
    s = t.hi;
    c += t.lo + pe;
  }
  __device__ __forceinline__ void add_mul(df32 a, df32 b) {
    const float p = a.hi * b.hi;
    add(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p))));
  }
  __device__ __forceinline__ void add_mul(df32 a, float b) {
    const float p = a.hi * b;
    add(p, fmaf(a.lo, b, fmaf(a.hi, b, -p)));
  }
  __device__ __forceinline__ df32 value() const {
    const float h = s + c;
    return {h, c - (h - s)};
  }
};

// prev - (m u + k K u - D^T p) at one face: l, r, s, n its neighbours in x
// and y (wall values already applied), xa - xb the pressure difference across
// it.  The stencil differences are exact two-sums, so the error is relative
// to the terms m u, k K u and D^T p, not to the neighbours.
__device__ __forceinline__ df32 face_defect(const OpCoef& C, df32 prev, float cc, float l, float r, float s,
                                            float n, float xa, float xb, bool ublk) {
  const df32 ex = df_add(df_two_sum(cc, -l), df_two_sum(cc, -r));
  const df32 ey = df_add(df_two_sum(cc, -s), df_two_sum(cc, -n));
  DFSum a{prev.hi, prev.lo};
  a.add_mul(df_neg(C.m), cc);
  a.add_mul(df_neg(C.kx), ex);
  a.add_mul(df_neg(C.ky), ey);
  a.add_mul(ublk ? C.gx : C.gy, df_two_sum(xa, -xb));
  return a.value();
}

// prev - D u at one cell from its four faces.
__device__ __forceinline__ df32 cell_defect(const OpCoef& C, df32 prev, float ue, float uw, float vn, float vs) {
  DFSum a{prev.hi, prev.lo};
  a.add_mul(df_neg(C.gx), df_two_sum(ue, -uw));
  a.add_mul(df_neg(C.gy), df_two_sum(vn, -vs));
  return a.value();
}

// Four consecutive floats from p[i..i+3] (cnt of them valid, the rest 0):
// one 16-byte load when vec and the group is whole.
__device__ __forceinline__ void load4(const float* p, long long i, int cnt, bool vec, float (&v)[4]) {
  if (vec && cnt == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p + i);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = e < cnt ? p[i + e] : 0.0f;
  }
}
__device__ __forceinline__ void store4(float* p, long long i, int cnt, bool vec, const float (&v)[4]) {
  if (vec && cnt == 4) {
    *reinterpret_cast<float4*>(p + i) = make_float4(v[0], v[1], v[2], v[3]);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (e < cnt) p[i + e] = v[e];
  }
}
__device__ __forceinline__ void load4d(const double* p, long long i, int cnt, bool vec, double (&v)[4]) {
  if (vec && cnt == 4) {
    const double2 a = *reinterpret_cast<const double2*>(p + i), b = *reinterpret_cast<const double2*>(p + i + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = e < cnt ? p[i + e] : 0.0;
  }
}

// The defects of faces i0 .. i0 + cnt - 1 of one column (uc: its velocity
// piece, xc: its pressure piece, prev: the defect before the piece).
__device__ __forceinline__ void face_group(const GridDev& g, const OpCoef& C, const float* uc, const float* xc,
                                           int i0, int cnt, bool vec, const df32 (&prev)[4], df32 (&out)[4]) {
  float u[4];
  load4(uc, i0, cnt, vec, u);
  const float left = i0 > 0 ? uc[i0 - 1] : 0.0f;
  const float right = i0 + 4 < g.size ? uc[i0 + 4] : 0.0f;
  bool isu = i0 < g.nu;
  int j, q;
  if (isu) {
    j = i0 / (g.nx - 1);
    q = i0 - j * (g.nx - 1);
  } else {
    j = (i0 - g.nu) / g.nx;
    q = i0 - g.nu - j * g.nx;
  }
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = i0 + e;
    if (e > 0) {
      if (i == g.nu) {
        isu = false;
        j = 0;
        q = 0;
      } else if (++q == (isu ? g.nx - 1 : g.nx)) {
        q = 0;
        ++j;
      }
    }
    if (e < cnt) {
      const float cc = u[e];
      const float lv = e > 0 ? u[e - 1] : left, rv = e < 3 ? u[e + 1] : right;
      float l, r, s, n, xa, xb;
      const int lc = j * g.nx + q;
      if (isu) {
        // K_at's wall rows: beyond a normal wall 0, beyond a tangential wall -u
        const int w = g.nx - 1;
        l = q > 0 ? lv : 0.0f;
        r = q < w - 1 ? rv : 0.0f;
        s = j > 0 ? uc[i - w] : -cc;
        n = j < g.ny - 1 ? uc[i + w] : -cc;
        xa = xc[lc];
        xb = xc[lc + 1];
      } else {
        l = q > 0 ? lv : -cc;
        r = q < g.nx - 1 ? rv : -cc;
        s = j > 0 ? uc[i - g.nx] : 0.0f;
        n = j < g.ny - 2 ? uc[i + g.nx] : 0.0f;
        xa = xc[lc];
        xb = xc[lc + g.nx];
      }
      out[e] = face_defect(C, prev[e], cc, l, r, s, n, xa, xb, isu);
    }
  }
}

// The divergence defects of cells i0 .. i0 + cnt - 1 of one column.
__device__ __forceinline__ void cell_group(const GridDev& g, const OpCoef& C, const float* uc, int i0, int cnt,
                                           const df32 (&prev)[4], df32 (&out)[4]) {
  int j = i0 / g.nx, q = i0 - j * g.nx;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    if (e > 0 && ++q == g.nx) {
      q = 0;
      ++j;
    }
    if (e < cnt) {
      const float* ur = uc + j * (g.nx - 1);
      const float ue = q < g.nx - 1 ? ur[q] : 0.0f, uw = q > 0 ? ur[q - 1] : 0.0f;
      const float vn = j < g.ny - 1 ? uc[g.nu + j * g.nx + q] : 0.0f;
      const float vs = j > 0 ? uc[g.nu + (j - 1) * g.nx + q] : 0.0f;
      out[e] = cell_defect(C, prev[e], ue, uw, vn, vs);
    }
  }
}

// Closing checks of an FP32-bulk solve (tensor_stokes.py:329-351, the same
// key slots as k_stokes_check): the final defect m u + k K u - D^T p - f and
// divergence D u of the FP64 fields are the defect pairs before the last
// sweep minus what the last sweep's float solve (u, x) adds, formed as in
// k_defect_update (double-float, about 48 bits; the fields' FP64 sums of the
// pieces round at 1e-16 of their size, far below the 1e-9 gates), so the
// check needs no FP64 arithmetic.  max|f|, max|u| and the finiteness of
// f, u and p are read from the FP64 arrays themselves.  f_prev: the Stokes
// right-hand side when the last sweep was the first solve, else null (the
// pairs hold the defect).
__global__ void __launch_bounds__(kThreads, 4) k_stokes_check_df(GridDev g, const double* f_prev, const float* u,
                                                              const float* x, const float* ru_hi, const float* ru_lo,
                                                              const float* rd_hi, const float* rd_lo,
                                                              const double* vel, const double* pres, const double* f,
                                                              const double* shift, int vec, double* partial,
                                                              CGFin<double> fin, unsigned int* done) {
  pdl_wait();
  const int c = blockIdx.y;
  const OpCoef C = op_coef(g, shift, c);
  const long long su = c * (long long)g.size, sp = c * (long long)g.np;
  const float* uc = u + su;
  const float* xc = x + sp;
  const bool first = f_prev != nullptr;  // then f_prev is f
  unsigned long long m[6] = {0, 0, 0, 0, 0, 0};
  constexpr unsigned long long kInf = 0x7ff0000000000000ull;
  const int ngf = (g.size + 3) / 4, ngc = (g.np + 3) / 4, ng = ngf > ngc ? ngf : ngc;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    if (t < ngf) {
      const int i0 = 4 * t, cnt = min(4, g.size - i0);
      df32 prev[4], d[4];
      {
        // the FP64 fields' maxima and finiteness first, so that their values
        // are dead before the defect arithmetic
        double fv[4], vv[4];
        load4d(f + su, i0, cnt, vec, fv);
        load4d(vel + su, i0, cnt, vec, vv);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (e < cnt) {
            const unsigned long long kf = abs_key(fv[e]), ku = abs_key(vv[e]);
            m[1] = max(m[1], kf);
            m[2] = max(m[2], ku);
            if (kf >= kInf) m[4] = 1;
            if (ku >= kInf) m[5] = 1;
          }
          if (first) prev[e] = d2df(fv[e]);
        }
      }
      if (!first) {
        float hi[4], lo[4];
        load4(ru_hi + su, i0, cnt, vec, hi);
        load4(ru_lo + su, i0, cnt, vec, lo);
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{hi[e], lo[e]};
      }
      face_group(g, C, uc, xc, i0, cnt, vec, prev, d);
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (e < cnt) m[0] = max(m[0], abs_key(f2d_bits(d[e].hi)));
    }
    if (t < ngc) {
      const int i0 = 4 * t, cnt = min(4, g.np - i0);
      double pv[4];
      load4d(pres + sp, i0, cnt, vec, pv);
      df32 prev[4], d[4];
      if (first) {
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{0.0f, 0.0f};
      } else {
        float hi[4], lo[4];
        load4(rd_hi + sp, i0, cnt, vec, hi);
        load4(rd_lo + sp, i0, cnt, vec, lo);
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{hi[e], lo[e]};
      }
      cell_group(g, C, uc, i0, cnt, prev, d);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (e < cnt) {
          m[3] = max(m[3], abs_key(f2d_bits(d[e].hi)));
          if (abs_key(pv[e]) >= kInf) m[5] = 1;
        }
      }
    }
  }
  write_keys<6>(m, partial, 6, 0);
  last_block_finish(fin, done);
}

// 16-byte group loads in the defect kernels: every column's face and cell
// ranges start on a 16-byte boundary (sizes multiples of four, aligned bases).
static int defect_vec(const GridDev& g, std::initializer_list<const void*> ptrs) {
  if (g.size % 4 || g.np % 4) return 0;
  for (const void* p : ptrs)
    if (reinterpret_cast<uintptr_t>(p) % 16) return 0;
  return 1;
}

static void closing_checks(Plan* P, const Exec& X, const double* f, const double* vel, const double* pres, int cols,
                           const double* shift) {
  const GridDev& g = P->g;
  const long long n = g.size > g.np ? g.size : g.np;
  const int rb = red_blocks(n);
  double* part = X.partial ? X.partial : P->partial;
  unsigned int* done = X.counter ? X.counter : P->done_counter;
  if (P->precision == MACSAV_FP32_MIXED) {
    // from the defect pairs and the last sweep's pieces (enqueue_solve_mixed)
    const int last = P->corrections;
    const long long sz = g.size, np = g.np;
    const float* ru_hi = reinterpret_cast<const float*>(P->w);
    const float* rd_hi = reinterpret_cast<const float*>(P->cells);
    const float* u = static_cast<const float*>(P->wacc32 + last * sz * cols);
    const float* x = static_cast<const float*>(P->xpieces + last * np * cols);
    const int vec = defect_vec(g, {u, x, ru_hi, rd_hi, f, vel, pres});
    // four times the reduction blocks: the groups' loads in flight fill the SMs
    const int nb = std::min(4 * rb, flat_blocks((n + 3) / 4));
    launch_k(k_stokes_check_df, dim3(nb, cols), kThreads, 0, X.s, g, last == 0 ? f : nullptr, u, x, ru_hi,
             ru_hi + sz * cols, rd_hi, rd_hi + np * cols, vel, pres, f, shift, vec, part,
             make_fin<double>(P, X, OP_CHECKS, nb, 6, cols), done);
  } else {
    launch_k(k_stokes_check, dim3(rb, cols), kThreads, 0, X.s, g, vel, pres, f, g.size, g.np, shift, part,
             make_fin<double>(P, X, OP_CHECKS, rb, 6, cols), done);
  }
  ++P->launches;
}

// The closing work a solve enqueued with close = false left out: for the
// mixed path the pressure centring (signalling `centred` once pres is final)
// and for both the FP64 closing checks.  The step runs it on its side stream.
int enqueue_close(Plan* P, Exec& X, const double* f, const double* vel, double* pres, int cols, cudaEvent_t centred) {
  if (P->precision != MACSAV_FP64) finish_pressure<double>(P, X, pres, pres, cols);
  if (centred) cudaEventRecord(centred, X.s);
  closing_checks(P, X, f, vel, pres, cols, P->shift);
  return MACSAV_OK;
}

// FP64 solve: TensorStokes.solve with every vector in double.  Shifts are
// read from P->shift (device), so the same enqueue serves the stand-alone
// solve and the captured stage.
int enqueue_solve_fp64(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres, bool close) {
  const GridDev& g = P->g;
  Launcher<double> L{P->t64, X.s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
  const long long sz = g.size;
  // u = (mI + kK)^{-1} (f + D^T p) (tensor_stokes.py:331-336), accumulated
  // alongside p inside the CG: vel starts as (mI+kK)^{-1} f and each update
  // adds alpha (mI+kK)^{-1} D^T pdir, the velocity the iteration computed for
  // its direction.  The same vector as the reference's closing inverse, to
  // rounding (D^T of the pressure mean is zero, so the centring does not
  // enter), without its three transform passes.
  velocity_inverse<double>(P, L, SrcPacked<double, double>{f, sz, g.nu, g.nx - 1, g.nx}, vel, sz, cols, nullptr);
  int rc = schur_pcg<double>(P, X, L, P->w, P->cells, cols, nullptr, vel);
  if (rc != MACSAV_OK) return rc;
  finish_pressure<double>(P, X, P->cells + 1LL * g.np * cols, pres, cols);
  if (close) closing_checks(P, X, f, vel, pres, cols, P->shift);
  return MACSAV_OK;
}

int solve_fp64(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
               cudaStream_t s) {
  (void)mass;
  (void)visc;
  Exec X{s, false, nullptr, 0, 0.0};
  return enqueue_solve_fp64(P, X, f, cols, vel, pres, true);
}

// ------------------------------------------------- FP32 + FP64 correction ---
// Defect for the next correction sweep, updated from the last FP32 solve:
// with the accumulated solution (vel, pres) = sum of the solves' (u_k, x_k),
// the momentum defect f - (m vel + k K vel - D^T pres) after solve k is the
// one after solve k-1 minus (m u_k + k K u_k - D^T x_k), and the continuity
// defect -D vel is the last one minus D u_k (both start from f and 0).  u_k
// and x_k are exactly the floats added to the FP64 fields, so the update needs
// no FP64 input but f once: it runs in double-float arithmetic on the FP32
// pipe (about 48 bits, no FP64 instruction) and keeps each defect as a float
// pair (hi, lo) in place.  The next FP32 solve reads the hi parts, the float
// nearest to the defect; the pairs keep the cancellation between f and the
// operator (the defect is 1e-4 .. 1e-9 of f) exact to far below that
// rounding.  The closing FP64 check of the solve measures the true defect of
// (vel, pres) in FP64.  GB300 runs FP64 at about 1/70 of FP32, and the FP64
// form of this kernel read the FP64 fields and issued about 20 FP64
// operations per face.
//   f: the Stokes right-hand side (first sweep) or null (the pairs hold the
//   previous defect); u, x: the last solve's velocity and pressure (float).
__global__ void __launch_bounds__(kThreads, 4) k_defect_update(GridDev g, const double* f, const float* u,
                                                            const float* x, const double* shift, int vec,
                                                            float* ru_hi, float* ru_lo, float* rd_hi, float* rd_lo) {
  pdl_wait();
  const int c = blockIdx.y;
  const OpCoef C = op_coef(g, shift, c);
  const long long su = c * (long long)g.size, sp = c * (long long)g.np;
  const float* uc = u + su;
  const float* xc = x + sp;
  const int ngf = (g.size + 3) / 4, ngc = (g.np + 3) / 4, ng = ngf > ngc ? ngf : ngc;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    if (t < ngf) {
      const int i0 = 4 * t, cnt = min(4, g.size - i0);
      df32 prev[4], d[4];
      if (f) {
        double fv[4];
        load4d(f + su, i0, cnt, vec, fv);
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = d2df(fv[e]);
      } else {
        float hi[4], lo[4];
        load4(ru_hi + su, i0, cnt, vec, hi);
        load4(ru_lo + su, i0, cnt, vec, lo);
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{hi[e], lo[e]};
      }
      face_group(g, C, uc, xc, i0, cnt, vec, prev, d);
      float hi[4], lo[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        hi[e] = d[e].hi;
        lo[e] = d[e].lo;
      }
      store4(ru_hi + su, i0, cnt, vec, hi);
      store4(ru_lo + su, i0, cnt, vec, lo);
    }
    if (t < ngc) {
      const int i0 = 4 * t, cnt = min(4, g.np - i0);
      df32 prev[4], d[4];
      if (f) {
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{0.0f, 0.0f};
      } else {
        float hi[4], lo[4];
        load4(rd_hi + sp, i0, cnt, vec, hi);
        load4(rd_lo + sp, i0, cnt, vec, lo);
#pragma unroll
        for (int e = 0; e < 4; ++e) prev[e] = df32{hi[e], lo[e]};
      }
      cell_group(g, C, uc, i0, cnt, prev, d);
      float hi[4], lo[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        hi[e] = d[e].hi;
        lo[e] = d[e].lo;
      }
      store4(rd_hi + sp, i0, cnt, vec, hi);
      store4(rd_lo + sp, i0, cnt, vec, lo);
    }
  }
}

// vel = sum of the pieces' double(u) and pres = sum of double(x), in sweep
// order (FP64 adds, the same rounding as adding each sweep's piece to the
// FP64 fields as it comes): the closing accumulation of an FP32-bulk solve.
__global__ void __launch_bounds__(kThreads) k_sum_pieces(const float* u, double* vel, long long sz, const float* x,
                                                         double* pres, long long np, int cols, int pieces) {
  pdl_wait();
  const int c = blockIdx.y;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long us = sz * cols, xs = np * cols;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  // four elements per thread (16-byte float loads, two 16-byte double stores)
  auto sum4 = [&](const float* src, long long ps, double* dst, long long n, long long base) {
    const bool aligned = ((reinterpret_cast<unsigned long long>(src) | reinterpret_cast<unsigned long long>(dst)) & 15) == 0;
    if (aligned && (n & 3) == 0 && (ps & 3) == 0) {
      for (long long i4 = t0; i4 < (n >> 2); i4 += stride) {
        const long long k = base + (i4 << 2);
        float4 f = *reinterpret_cast<const float4*>(src + k);
        double v0 = f2d_bits(f.x), v1 = f2d_bits(f.y), v2 = f2d_bits(f.z), v3 = f2d_bits(f.w);
        for (int q = 1; q < pieces; ++q) {
          f = *reinterpret_cast<const float4*>(src + q * ps + k);
          v0 += f2d_bits(f.x);
          v1 += f2d_bits(f.y);
          v2 += f2d_bits(f.z);
          v3 += f2d_bits(f.w);
        }
        reinterpret_cast<double2*>(dst + k)[0] = make_double2(v0, v1);
        reinterpret_cast<double2*>(dst + k)[1] = make_double2(v2, v3);
      }
    } else {
      for (long long i = t0; i < n; i += stride) {
        const long long k = base + i;
        double v = f2d_bits(src[k]);
        for (int q = 1; q < pieces; ++q) v += f2d_bits(src[q * ps + k]);
        dst[k] = v;
      }
    }
  };
  sum4(u, us, vel, sz, c * sz);
  sum4(x, xs, pres, np, c * np);
}

// One FP32 Stokes solve of (f, 0) or of the defect (ru, rd): transforms,
// stencils and Krylov vectors in float, reductions in double.  Its velocity
// and pressure become the sweep's pieces (wacc32 and xpieces slot `sweep`).
//
// Plain PCG: the velocity is accumulated inside the CG, u = (mI+kK)^{-1} ru
// + sum_k alpha_k (mI+kK)^{-1} D^T pdir_k, from the velocity each iteration
// computes anyway (k_cg_update), so no closing velocity inverse
// (mI+kK)^{-1}(ru + D^T x) is needed; one kernel adds u and x to the FP64
// fields.  The same vector in exact arithmetic; in float it differs at
// rounding level, which the FP64 defect correction absorbs like any other
// inner-solve error.  The learned preconditioner (flexible CG, whose columns
// may restart) runs in the first inner solve of a Stokes solve only (add = 0:
// its right-hand side is the stage's own, a smooth field; the correction
// sweeps solve for rounding-level defects), or in all of them with the
// every-iteration placement.  A column that restarts from zero also takes its
// accumulated velocity back to the start, kept in net_wacc0.
static int inner_solve32(Plan* P, Exec& X, const double* f, const float* ru, const float* rd, int cols, int sweep) {
  const GridDev& g = P->g;
  Launcher<float> L{P->t32, X.s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
  const long long sz = g.size, np = g.np;
  float* w = P->w32;
  const bool net = P->net != nullptr && (P->net_every || sweep == 0);
  float* wacc = P->wacc32 + sweep * sz * cols;
  if (f) velocity_inverse<float>(P, L, SrcPacked<float, double>{f, sz, g.nu, g.nx - 1, g.nx}, wacc, sz, cols, nullptr);
  else velocity_inverse<float>(P, L, SrcPacked<float, float>{ru, sz, g.nu, g.nx - 1, g.nx}, wacc, sz, cols, nullptr);
  if (net) cudaMemcpyAsync(P->net_wacc0, wacc, sizeof(float) * size_t(sz) * cols, cudaMemcpyDeviceToDevice, X.s);
  const double keep = X.ktol;
  const int keep_net = X.net;
  X.ktol = (sweep == 0 && P->first_ktol > 0.0) ? P->first_ktol : P->inner_ktol;
  X.net = net ? 1 : 0;
  int rc = schur_pcg<float>(P, X, L, w, P->cells32, cols, rd, wacc);
  X.ktol = keep;
  X.net = keep_net;
  if (rc != MACSAV_OK) return rc;
  const float* x = P->cells32 + 1 * np * cols;
  cudaMemcpyAsync(P->xpieces + sweep * np * cols, x, sizeof(float) * size_t(np) * cols, cudaMemcpyDeviceToDevice, X.s);
  return MACSAV_OK;
}

// TensorStokes.solve with FP32 bulk: an FP32 solve, then `corrections`
// defect-correction sweeps whose defects are formed from the FP64 fields in
// double-float arithmetic, so the result satisfies the same FP64 residual and
// divergence gates (checked in FP64) as the FP64 path.
int enqueue_solve_mixed(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres, bool close) {
  const GridDev& g = P->g;
  const long long sz = g.size, np = g.np;
  // the defect pairs live in the FP64 work buffers, unused on this path
  float* ru_hi = reinterpret_cast<float*>(P->w);
  float* ru_lo = ru_hi + sz * cols;
  float* rd_hi = reinterpret_cast<float*>(P->cells);
  float* rd_lo = rd_hi + np * cols;
  for (int sweep = 0; sweep <= P->corrections; ++sweep) {
    if (sweep > 0) {
      // no block reduction: four times the reduction kernels' blocks fill the
      // SMs (a few elements per thread keep its set-up amortised)
      const float* u = static_cast<const float*>(P->wacc32 + (sweep - 1) * sz * cols);
      const float* x = static_cast<const float*>(P->xpieces + (sweep - 1) * np * cols);
      const long long n4 = ((sz > np ? sz : np) + 3) / 4;
      launch_k(k_defect_update, dim3(std::min(4 * red_blocks(4 * n4), flat_blocks(n4)), cols), kThreads, 0, X.s, g,
               sweep == 1 ? f : nullptr, u, x, P->shift, defect_vec(g, {u, x, ru_hi, rd_hi, f}), ru_hi, ru_lo, rd_hi,
               rd_lo);
      ++P->launches;
    }
    int rc = inner_solve32(P, X, sweep == 0 ? f : nullptr, ru_hi, sweep == 0 ? nullptr : rd_hi, cols, sweep);
    if (rc != MACSAV_OK) return rc;
  }
  launch_k(k_sum_pieces, dim3(flat_blocks(sz / 4 + 1), cols), kThreads, 0, X.s, static_cast<const float*>(P->wacc32),
           vel, sz,
           static_cast<const float*>(P->xpieces), pres, np, cols, P->corrections + 1);
  ++P->launches;
  // mean-zero pressure and the FP64 closing checks, as in the FP64 path
  if (close) {
    finish_pressure<double>(P, X, pres, pres, cols);
    closing_checks(P, X, f, vel, pres, cols, P->shift);
  }
  return MACSAV_OK;
}

// Average device milliseconds of `reps` launches of transform pass `base`
// (two right-hand sides; the velocity passes over the u and v blocks
// concurrently), replayed from a captured graph on a stream of its own
// ordered after `user`, with the FP32 transforms t32 (the plan's, or a copy
// with other launch shapes):
//   0: FP32 velocity column pass; 1: FP32 velocity forward row pass (FP64
//   packed input); 2: FP32 velocity inverse row pass; 3: FP64 velocity column
//   pass; 4: FP32 pressure column pass; 5: FP32 pressure forward row pass
//   (FP64 cells in); 6: FP32 pressure inverse row pass (FP64 cells out).
static int time_pass_t(Plan* P, const Transforms<float>& t32, int base, int reps, cudaStream_t user, double* ms) {
  const GridDev& g = P->g;
  const int cols = 2;
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return MACSAV_ERR_CUDA;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, user);
  cudaStreamWaitEvent(s, a, 0);
  const double shift[4] = {1.0, 1e-6, 1.0, 1e-6};
  cudaMemcpyAsync(P->shift, shift, sizeof shift, cudaMemcpyHostToDevice, s);
  const long long np = g.np;
  auto run = [&]() {
    const Launcher<float> L{t32, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
    if (base == 0) L.column_uv(cols, nullptr, P->shift);
    else if (base == 1) L.row_forward_uv(SrcPacked<float, double>{P->w, g.size, g.nu, g.nx - 1, g.nx}, cols, nullptr);
    else if (base == 2) L.row_inverse_uv(DstPacked<float, float>{P->w32, g.size, g.nu, g.nx - 1, g.nx}, cols, nullptr);
    else if (base == 3)
      Launcher<double>{P->t64, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]}.column_uv(cols, nullptr, P->shift);
    else if (base == 4) L.column_p(cols, nullptr, P->shift, float(P->pthr));
    else if (base == 5) L.row_forward_p(SrcCells<float, double>{P->w, np, g.nx}, cols, nullptr);
    else L.row_inverse_p(DstCells<float, double>{P->w, np, g.nx}, cols, nullptr, nullptr, NoFin{}, nullptr);
  };
  run();  // warm-up
  // the reps are captured into one graph and replayed, as the pass runs
  // inside the captured step (u and v blocks concurrently, no host gaps)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    for (int k = 0; k < reps; ++k) run();
    e = cudaStreamEndCapture(s, &graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);  // warm
  if (e == cudaSuccess) {
    cudaEventRecord(a, s);
    e = cudaGraphLaunch(exec, s);
    cudaEventRecord(b, s);
  }
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0;
  if (e == cudaSuccess) cudaEventElapsedTime(&t, a, b);
  cudaStreamSynchronize(s);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamDestroy(s);
  *ms = double(t) / reps;
  return e == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// macsav_time_pass: pass % 10 is the pass of time_pass_t, pass / 10 the
// launch shape forced on every block (0 the plan's own, 1 plain, 2 doubled,
// 3 split: P2Shape, where the pass allows it); also the pass's algorithmic
// bytes per launch (each element of its input read once and output written
// once).
int time_pass(Plan* P, int pass, int reps, cudaStream_t user, double* ms, double* bytes) {
  const int base = pass % 10, shape = pass / 10;
  if (P->maxcols < 2 || reps < 1 || pass < 0 || base > 6 || shape > 3) return MACSAV_ERR_VALUE;
  if (base != 3 && P->precision != MACSAV_FP32_MIXED) return MACSAV_ERR_VALUE;
  if (base == 3 && shape != 0) return MACSAV_ERR_VALUE;
  Transforms<float> t32 = P->t32;
  if (shape)
    for (TBlockDev<float>* B : {&t32.u, &t32.v, &t32.p}) B->shape[0] = B->shape[1] = B->shape[2] = shape;
  const int rc = time_pass_t(P, t32, base, reps, user, ms);
  const double n = double(base >= 4 ? P->g.np : P->g.size) * 2;
  const double per[7] = {2 * 4, 8 + 4, 4 + 4, 2 * 8, 2 * 4, 8 + 4, 4 + 8};
  *bytes = per[base] * n;
  return rc;
}

// Launch-shape autotuner of the FP32 power-of-two passes.  For each of the
// six pass kinds (velocity forward rows, columns, inverse rows; the same for
// the pressure block) it times the block's rule (P2_AUTO) and the plain,
// doubled and split shapes on every block of that kind, `reps` launches each
// from a captured graph, and keeps the fastest; another shape replaces the
// rule only when at least 2 % faster, so timing noise does not flip it.
// Every shape computes the same bits, so the choice changes time only.
// chosen[k] (if not null): the kept shape per kind, in the order above.
int autotune_shapes(Plan* P, int reps, cudaStream_t user, int* chosen) {
  if (P->precision != MACSAV_FP32_MIXED || P->maxcols < 2 || reps < 1) return MACSAV_ERR_VALUE;
  struct Kind {
    int base, idx;
    bool vel;
  };
  const Kind kinds[6] = {{1, 0, true}, {0, 1, true}, {2, 2, true}, {5, 0, false}, {4, 1, false}, {6, 2, false}};
  for (int k = 0; k < 6; ++k) {
    const Kind& K = kinds[k];
    double best = 0.0;
    int keep = P2_AUTO;
    for (int sh = P2_AUTO; sh <= P2_SPLIT; ++sh) {
      Transforms<float> t = P->t32;
      if (K.vel) {
        t.u.shape[K.idx] = sh;
        t.v.shape[K.idx] = sh;
      } else {
        t.p.shape[K.idx] = sh;
      }
      double ms = 0.0;
      const int rc = time_pass_t(P, t, K.base, reps, user, &ms);
      if (rc != MACSAV_OK) return rc;
      if (sh == P2_AUTO) best = ms;
      else if (ms < 0.98 * best) {
        best = ms;
        keep = sh;
      }
    }
    if (K.vel) {
      P->t32.u.shape[K.idx] = keep;
      P->t32.v.shape[K.idx] = keep;
    } else {
      P->t32.p.shape[K.idx] = keep;
    }
    if (chosen) chosen[k] = keep;
  }
  return MACSAV_OK;
}

// (m I + k K)^{-1} of `cols` packed velocity columns in the plan's precision
// (TensorStokes._velocity_inverse, solver/mac/tensor_stokes.py:200-215).
int op_velocity_inverse(Plan* P, const double* in, double* out, int cols, cudaStream_t s) {
  const GridDev& g = P->g;
  if (P->precision == MACSAV_FP64) {
    const Launcher<double> L{P->t64, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
    velocity_inverse(P, L, SrcPacked<double, double>{in, g.size, g.nu, g.nx - 1, g.nx}, out, g.size, cols, nullptr);
  } else {
    const Launcher<float> L{P->t32, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
    velocity_inverse(P, L, SrcPacked<float, double>{in, g.size, g.nu, g.nx - 1, g.nx}, out, g.size, cols, nullptr);
  }
  return MACSAV_OK;
}

// m (D D^T)^+ p + k p on the mean-zero part of `cols` cell columns, mean
// zero out (the pressure Schur preconditioner, tensor_stokes.py:217-243,281-287).
int op_schur_precondition(Plan* P, const double* in, double* out, int cols, cudaStream_t s) {
  const GridDev& g = P->g;
  const long long np = g.np;
  if (P->precision == MACSAV_FP64) {
    const Launcher<double> L{P->t64, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
    L.row_forward_p(SrcCells<double, double>{in, np, g.nx}, cols, nullptr);
    L.column_p(cols, nullptr, P->shift, P->pthr);
    L.row_inverse_p(DstCells<double, double>{out, np, g.nx}, cols, nullptr, nullptr, NoFin{}, nullptr);
  } else {
    const Launcher<float> L{P->t32, s, &P->launches, P->aux[0], P->evf[0], P->evj[0]};
    L.row_forward_p(SrcCells<float, double>{in, np, g.nx}, cols, nullptr);
    L.column_p(cols, nullptr, P->shift, float(P->pthr));
    L.row_inverse_p(DstCells<float, double>{out, np, g.nx}, cols, nullptr, nullptr, NoFin{}, nullptr);
  }
  return MACSAV_OK;
}

int solve_mixed(Plan* P, const double* f, int cols, double mass, double visc, double* vel, double* pres,
                cudaStream_t s, int* sweeps) {
  (void)mass;
  (void)visc;
  Exec X{s, false, nullptr, 0, 0.0};
  *sweeps = P->corrections;
  return enqueue_solve_mixed(P, X, f, cols, vel, pres, true);
}

}  // namespace macsav
