// Shared device/host helpers for the MAC mr-SAV CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/macsav.h"

#define MACSAV_HD __host__ __device__ __forceinline__

namespace macsav {

template <typename T>
struct cplx {
  T x, y;
};

template <typename T>
MACSAV_HD cplx<T> mk(T a, T b) { cplx<T> r; r.x = a; r.y = b; return r; }
template <typename T>
MACSAV_HD cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.x + b.x, a.y + b.y); }
template <typename T>
MACSAV_HD cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.x - b.x, a.y - b.y); }
template <typename T>
MACSAV_HD cplx<T> cmul(cplx<T> a, cplx<T> b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <typename T>
MACSAV_HD cplx<T> cmulc(cplx<T> a, cplx<T> b) { return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
template <typename T>
MACSAV_HD cplx<T> cscale(cplx<T> a, T s) { return mk(a.x * s, a.y * s); }
template <typename T>
MACSAV_HD cplx<T> conjg(cplx<T> a) { return mk(a.x, -a.y); }
// multiply by -i (sign=-1) or +i (sign=+1)
template <typename T>
MACSAV_HD cplx<T> mul_i(cplx<T> a, int sign) { return sign > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x); }

// Error word bits written by device code and converted to exceptions on the host.
enum ErrorBits : int {
  ERR_NONFINITE = 1 << 0,
  ERR_CG_MAXITER = 1 << 1,
  ERR_STOKES_GATE = 1 << 2,
  ERR_STAGE_GATE = 1 << 3,
  ERR_NEG_ENERGY = 1 << 4,
  ERR_SCALAR = 1 << 5,
};

// Division by a runtime-constant divisor d >= 1 for 0 <= n < 2^31 with one
// multiply-high (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994): q = (umulhi(n, m) + n) >> s, m = floor(2^32 (2^s - d) / d) + 1.
struct FastDiv {
  unsigned int d, m, s;
  FastDiv() : d(1), m(1), s(0) {}
  explicit FastDiv(unsigned int div) : d(div) {
    s = 0;
    while ((1ull << s) < d) ++s;
    m = (unsigned int)((((1ull << s) - d) << 32) / d + 1);
  }
  __device__ __forceinline__ int div(int n) const {
    return int((__umulhi((unsigned int)n, m) + (unsigned int)n) >> s);
  }
  __device__ __forceinline__ int mod(int n, int q) const { return n - q * int(d); }
};

constexpr int kThreads = 256;     // element-wise and reduction kernels
constexpr int kFFTThreads = 512;  // transform passes (shared-memory FFTs)

// Element type of a 16-byte vector of T.
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

// Per-thread accumulator for inner products: plain double for FP64 data;
// for FP32 data the products are summed in float with Neumaier compensation
// (error independent of the number of terms), and the block and grid sums
// are then formed in double.
template <typename T> struct Acc {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct Acc<float> {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return double(s) + double(c); }
};

// ---- deterministic block reductions in double --------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
// Maximum that propagates NaN (fmax would drop it), as numpy.max does.
__device__ __forceinline__ double nanmax(double a, double b) {
  return (a != a) ? a : ((b != b) ? b : fmax(a, b));
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = nanmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Sums NV values over the block; result valid in thread 0.  Fixed tree order,
// so the result is bitwise reproducible for a given launch shape.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* scratch /* >= 32*NV */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nw ? scratch[k * 32 + lane] : 0.0;
      v[k] = warp_sum(s);
    }
  }
  __syncthreads();
}
template <int NV>
__device__ __forceinline__ void block_max(double (&v)[NV], double* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_max(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = lane < nw ? scratch[k * 32 + lane] : 0.0;
      v[k] = warp_max(s);
    }
  }
  __syncthreads();
}


// Grid-wide "last block finishes" step: every block calls this once after
// writing its partials; the block that arrives last (all partials visible)
// runs fin() with all its threads and resets the counter for the next kernel.
template <class Fin>
__device__ __forceinline__ void last_block_finish(const Fin& fin, unsigned int* counter) {
  __shared__ int is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int total = gridDim.x * gridDim.y * gridDim.z;
    is_last = (atomicAdd(counter, 1u) == total - 1) ? 1 : 0;
  }
  __syncthreads();
  if (is_last) {
    __threadfence();
    fin();
    if (threadIdx.x == 0) *counter = 0u;
  }
}

struct NoFin {
  __device__ void operator()() const {}
};

}  // namespace macsav
