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

// ---- double-float arithmetic on the FP32 pipe ------------------------------
// GB300 runs FP64 at a small fraction of FP32, so every reduction of FP32 data
// is carried as an unevaluated sum hi + lo of two floats (Knuth's TwoSum,
// Dekker's fast renormalisation): ~48-bit significands without FP64 issue.
struct df32 {
  float hi, lo;
};
__device__ __forceinline__ df32 df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  const df32 s = df_two_sum(a.hi, b.hi);
  const float e = s.lo + (a.lo + b.lo);
  const float h = s.hi + e;
  return {h, e - (h - s.hi)};
}
__device__ __forceinline__ double df_value(df32 a) { return double(a.hi) + double(a.lo); }
__device__ __forceinline__ df32 df_neg(df32 a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df32 df_sub(df32 a, df32 b) { return df_add(a, df_neg(b)); }
// Product of two double-floats (Dekker's product with an FMA for the exact
// low part of hi*hi), renormalised.
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float h = p + e;
  return {h, e - (h - p)};
}

// Conversions between double and float without the FP64 pipe: the binary64
// fields are re-packed with integer instructions, rounding to nearest even.
// Values beyond the float range saturate to +-inf; binary32 subnormals flush
// to zero (the magnitudes seen here are far from both ends).
__device__ __forceinline__ float d2f_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const int e = int((b >> 52) & 0x7ff);
  unsigned long long m = b & 0xfffffffffffffull;
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));  // inf / nan
  const int ef = e - 1023 + 127;
  if (ef <= 0) return __uint_as_float(sign);  // zero, subnormal, underflow
  unsigned int mf = (unsigned int)(m >> 29);
  const unsigned int rem = (unsigned int)(m & 0x1fffffffu);
  unsigned int bits = ((unsigned int)ef << 23) | mf;
  if (rem > 0x10000000u || (rem == 0x10000000u && (mf & 1u))) ++bits;  // carries into the exponent correctly
  if (ef >= 255 || bits >= 0x7f800000u) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | bits);
}
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  const unsigned int e = (b >> 23) & 0xffu;
  const unsigned long long m = b & 0x7fffffu;
  if (e == 0) return __longlong_as_double((long long)sign);  // zero (subnormals flush)
  if (e == 0xff) return __longlong_as_double((long long)(sign | 0x7ff0000000000000ull | (m << 29)));
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e - 127 + 1023) << 52) | (m << 29)));
}
// A double as a double-float hi + lo without the FP64 pipe: hi is x rounded
// to float (d2f_bits), lo the rest x - hi (exact in binary64, at most 30
// significant bits) rounded to float, so hi + lo carries about 48 bits.
// Zero, subnormal, infinite and NaN inputs, and parts beyond the float range,
// give lo = 0 (hi carries the special value).
__device__ __forceinline__ df32 d2df(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const float hi = d2f_bits(x);
  const int e = int((b >> 52) & 0x7ff);
  const unsigned int hb = __float_as_uint(hi);
  const int he = int((hb >> 23) & 0xffu);
  const int se = e - 1075 + 127;  // biased float exponent of 2^(e - 1075)
  if (e == 0 || e == 0x7ff || he == 0 || he == 0xff || se + 64 <= 0 || se >= 255) return {hi, 0.0f};
  const long long m = (long long)((b & 0xfffffffffffffull) | (1ull << 52));  // |x| = m 2^(e-1075)
  const long long hm = (long long)((hb & 0x7fffffu) | 0x800000u);              // |hi| = hm 2^(he-150)
  const int sh = he - e + 925;  // 29, or 30 when the rounding carried into the exponent
  const int r = int(m - (hm << sh));  // |r| <= 2^29
  // r 2^(e-1075) as a float, scaled in two steps when 2^(e-1075) is below
  // the normal float range (|x| below about 2^-75)
  const float lo = se > 0 ? float(r) * __uint_as_float((unsigned int)se << 23)
                          : (float(r) * __uint_as_float((unsigned int)(se + 64) << 23)) * 5.421010862427522e-20f;
  return {hi, (b >> 63) ? -lo : lo};
}

// Load a double into T without touching the FP64 pipe when T is float.
template <typename T>
__device__ __forceinline__ T load_as(const double* p) {
  if constexpr (sizeof(T) == 4) return d2f_bits(*p);
  else return *p;
}
template <typename T>
__device__ __forceinline__ T load_as(const float* p) { return T(*p); }

// |x| of a double as an ordered integer key: the maximum key is the maximum
// |x|, and NaN keys exceed every finite or infinite one (so NaN propagates).
__device__ __forceinline__ unsigned long long abs_key(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ double key_value(unsigned long long k) { return __longlong_as_double((long long)k); }

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
  __device__ __forceinline__ df32 pair() const { return df_two_sum(s, c); }
  __device__ __forceinline__ double value() const { return df_value(pair()); }
};

// Reduction traits: the partial type of FP64 data is double, of FP32 data a
// double-float pair (stored in the same 8 bytes as a float2).
template <typename T> struct Red;
template <> struct Red<double> {
  using P = double;
  __device__ __forceinline__ static P from(const Acc<double>& a) { return a.s; }
  __device__ __forceinline__ static P add(P a, P b) { return a + b; }
  __device__ __forceinline__ static P shfl_down(P v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
  __device__ __forceinline__ static P zero() { return 0.0; }
  __device__ __forceinline__ static double value(P p) { return p; }
  __device__ __forceinline__ static P load(const double* p) { return __ldcg(p); }
  __device__ __forceinline__ static void store(double* p, P v) { *p = v; }
};
template <> struct Red<float> {
  using P = df32;
  __device__ __forceinline__ static P from(const Acc<float>& a) { return a.pair(); }
  __device__ __forceinline__ static P add(P a, P b) { return df_add(a, b); }
  __device__ __forceinline__ static P shfl_down(P v, int o) {
    return {__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
  }
  __device__ __forceinline__ static P zero() { return {0.0f, 0.0f}; }
  __device__ __forceinline__ static double value(P p) { return df_value(p); }
  __device__ __forceinline__ static P load(const double* p) {
    const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
    return {f.x, f.y};
  }
  __device__ __forceinline__ static void store(double* p, P v) { *reinterpret_cast<float2*>(p) = make_float2(v.hi, v.lo); }
};

// Block sum of NV partials (result in thread 0), fixed tree order.
template <typename T, int NV>
__device__ __forceinline__ void block_sum_p(typename Red<T>::P (&v)[NV], typename Red<T>::P* scratch /* >= 32*NV */) {
  using R = Red<T>;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] = R::add(v[k], R::shfl_down(v[k], o));
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      v[k] = lane < nw ? scratch[k * 32 + lane] : R::zero();
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] = R::add(v[k], R::shfl_down(v[k], o));
    }
  }
  __syncthreads();
}

// Block maximum of NV integer keys (abs_key of doubles), result in thread 0.
template <int NV>
__device__ __forceinline__ void block_max_key(unsigned long long (&v)[NV], unsigned long long* scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] = max(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * 32 + wid] = v[k];
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      v[k] = lane < nw ? scratch[k * 32 + lane] : 0ull;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] = max(v[k], __shfl_down_sync(0xffffffffu, v[k], o));
    }
  }
  __syncthreads();
}

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


// Block partial of NV sums (Red<T>) written to partial[(c*gridDim.x+b)*K + k].
template <typename T, int NV>
__device__ __forceinline__ void write_sums(const Acc<T> (&acc)[NV], double* partial, int K) {
  using R = Red<T>;
  __shared__ typename R::P red[NV * 32];
  typename R::P v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = R::from(acc[k]);
  block_sum_p<T, NV>(v, red);
  if (threadIdx.x == 0) {
    double* o = partial + (size_t(blockIdx.y) * gridDim.x + blockIdx.x) * K;
#pragma unroll
    for (int k = 0; k < NV; ++k) R::store(o + k, v[k]);
  }
}

// Block maximum of NV abs_key values written to slots off..off+NV-1.
template <int NV>
__device__ __forceinline__ void write_keys(unsigned long long (&key)[NV], double* partial, int K, int off) {
  __shared__ unsigned long long redk[NV * 32];
  block_max_key<NV>(key, redk);
  if (threadIdx.x == 0) {
    double* o = partial + (size_t(blockIdx.y) * gridDim.x + blockIdx.x) * K + off;
#pragma unroll
    for (int k = 0; k < NV; ++k) reinterpret_cast<unsigned long long*>(o)[k] = key[k];
  }
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

// Programmatic dependent launch.  Kernels started with launch_k may be
// launched while the previous kernel of their stream drains; such a kernel
// calls pdl_wait() first, which returns once the previous grid has completed
// and its writes are visible (a no-op for a kernel launched without the
// attribute).  No kernel triggers its dependents early: measured on GB300, an
// early trigger let waiting blocks of the next kernel take SM slots and
// slowed the step by 8-19%, while the plain form gains the launch latency.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool g_launch_pdl = true;  // launch_k uses the programmatic-serialization attribute

template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_launch_pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

struct NoFin {
  __device__ void operator()() const {}
};

}  // namespace macsav
