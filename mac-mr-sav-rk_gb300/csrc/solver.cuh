// Device functors, CG kernels and the templated Stokes solve core.
#pragma once
#include "plan.cuh"

namespace macsav {

// ------------------------------------------------------------ row sources ---
// Packed velocity rows: block 0 = u rows (length nx-1), block 1 = v rows (nx).
template <typename T, typename In>
struct SrcPacked {
  const In* x;
  long long cstride;
  int off1, n0, n1;
  __device__ T operator()(int b, int c, int row, int n) const {
    const In* base = x + c * cstride;
    return b == 0 ? T(base[(long long)row * n0 + n]) : T(base[off1 + (long long)row * n1 + n]);
  }
};

// Cell rows (ny, nx).
template <typename T, typename In>
struct SrcCells {
  const In* x;
  long long cstride;
  int nx;
  __device__ T operator()(int, int c, int row, int n) const { return T(x[c * cstride + (long long)row * nx + n]); }
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
  __device__ T P(const PIn* a, const PIn* b, T beta, long long i) const {
    return b ? T(a[i]) + beta * T(b[i]) : T(a[i]);
  }
  __device__ T operator()(int bk, int c, int row, int n) const {
    const PIn* a = p1 + c * pstride;
    const PIn* b = nullptr;
    T beta = T(0);
    if (p2 && cg[c].iters > 0) {
      b = p2 + c * pstride;
      beta = T(cg[c].beta);
    }
    const long long l = (long long)row * nx + n;
    T v;
    long long fi;
    if (bk == 0) {
      v = (P(a, b, beta, l) - P(a, b, beta, l + 1)) * ihx;
      fi = (long long)row * (nx - 1) + n;
    } else {
      v = (P(a, b, beta, l) - P(a, b, beta, l + nx)) * ihy;
      fi = nu + l;
    }
    if (f) v += T(f[c * fstride + fi]);
    return v;
  }
};

// --------------------------------------------------------------- row sinks ---
template <typename T, typename Out>
struct DstPacked {
  Out* x;
  long long cstride;
  int off1, n0, n1;
  __device__ void operator()(int b, int c, int row, int n, T v, double (&)[2]) const {
    Out* base = x + c * cstride;
    if (b == 0) base[(long long)row * n0 + n] = Out(v);
    else base[off1 + (long long)row * n1 + n] = Out(v);
  }
};

template <typename T, typename Out>
struct DstCells {
  Out* x;
  long long cstride;
  int nx;
  __device__ void operator()(int, int c, int row, int n, T v, double (&)[2]) const {
    x[c * cstride + (long long)row * nx + n] = Out(v);
  }
};

// z = value; acc[0] += r . z
template <typename T>
struct DstCellsDot {
  T* z;
  const T* r;
  long long cstride;
  int nx;
  __device__ void operator()(int, int c, int row, int n, T v, double (&acc)[2]) const {
    const long long i = c * cstride + (long long)row * nx + n;
    z[i] = v;
    acc[0] += double(r[i]) * double(v);
  }
};

// ------------------------------------------------------------- launching ---
template <typename T>
struct Launcher {
  const Transforms<T>& t;
  cudaStream_t s;
  long long* counter;

  template <class Src>
  void row_forward_uv(Src src, int cols, const int* active) const;
  template <class Dst>
  void row_inverse_uv(Dst dst, int cols, const int* active, double* partial) const;
  void column_uv(int cols, const int* active, const double* shift) const;
  template <class Src>
  void row_forward_p(Src src, int cols, const int* active) const;
  template <class Dst>
  void row_inverse_p(Dst dst, int cols, const int* active, double* partial) const;
  void column_p(int cols, const int* active, const double* shift, T thr) const;
  int groups_row_p() const { return (t.p.rows + 2 * t.p.px - 1) / (2 * t.p.px); }
};

constexpr int kVmax = 16;

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

template <class K>
inline void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
}

template <typename T>
template <class Src>
void Launcher<T>::row_forward_uv(Src src, int cols, const int* active) const {
  RowArgs<T> a = row_args(t.u, &t.v, active);
  auto k = k_row_forward<T, kVmax, Src>;
  set_smem(k, t.smem_row_uv);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_row_uv, s>>>(a, src);
  ++*counter;
}
template <typename T>
template <class Dst>
void Launcher<T>::row_inverse_uv(Dst dst, int cols, const int* active, double* partial) const {
  RowArgs<T> a = row_args(t.u, &t.v, active);
  auto k = k_row_inverse<T, kVmax, Dst>;
  set_smem(k, t.smem_row_uv);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_row_uv, s>>>(a, dst, partial);
  ++*counter;
}
template <typename T>
void Launcher<T>::column_uv(int cols, const int* active, const double* shift) const {
  ColArgs<T> a = col_args(t.u, &t.v, active, W_HELMHOLTZ, shift, T(0));
  auto k = k_column<T, kVmax>;
  set_smem(k, t.smem_col_uv);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_col_uv, s>>>(a);
  ++*counter;
}
template <typename T>
template <class Src>
void Launcher<T>::row_forward_p(Src src, int cols, const int* active) const {
  RowArgs<T> a = row_args(t.p, (const TBlockDev<T>*)nullptr, active);
  auto k = k_row_forward<T, kVmax, Src>;
  set_smem(k, t.smem_row_p);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_row_p, s>>>(a, src);
  ++*counter;
}
template <typename T>
template <class Dst>
void Launcher<T>::row_inverse_p(Dst dst, int cols, const int* active, double* partial) const {
  RowArgs<T> a = row_args(t.p, (const TBlockDev<T>*)nullptr, active);
  auto k = k_row_inverse<T, kVmax, Dst>;
  set_smem(k, t.smem_row_p);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_row_p, s>>>(a, dst, partial);
  ++*counter;
}
template <typename T>
void Launcher<T>::column_p(int cols, const int* active, const double* shift, T thr) const {
  ColArgs<T> a = col_args(t.p, (const TBlockDev<T>*)nullptr, active, W_POISSON, shift, thr);
  auto k = k_column<T, kVmax>;
  set_smem(k, t.smem_col_p);
  k<<<dim3(total_groups(a), cols), kThreads, t.smem_col_p, s>>>(a);
  ++*counter;
}

}  // namespace macsav
