// Separable DST-I / DST-II / DCT-II block transforms of MAC fields.
//
// A "block" is one 2-D array (the u faces, the v faces or the cells) whose
// x-lines (rows, contiguous) and y-lines (columns) are transformed with the
// real trigonometric transform that diagonalises the 1-D second difference
// with the block's boundary conditions (the bases of the reference's
// solver/mac/tensor_stokes.py:156-168).  A shifted inverse or Poisson
// pseudo-inverse is done in three passes:
//
//   row pass   : forward x-transform of every row  -> spectral buffer H
//   column pass: forward y-transform, multiply by the spectral weight
//                w(ky,kx), inverse y-transform of every column of H (in place)
//   row pass   : inverse x-transform of every row of H -> result
//
// so the only column-strided pass runs on the padded, aligned H buffer.
// All transforms work on two real lines packed into one complex FFT:
//   DCT-II   : Makhoul reordering, FFT of length N;
//   DST-II   : DCT-II of (-1)^n x, coefficient j is the DST coefficient N-1-j
//              (the eigenvalue tables are stored in this internal order);
//   DST-I    : odd extension of length 2(N+1).
// Forward transforms are unnormalised; inverses carry the normalisation, so
// inverse(forward(x)) = x and spectral weights are the plain eigen-weights.
#pragma once
#include "fft.cuh"

namespace macsav {

enum Kind : int { KIND_DCT2 = 0, KIND_DST2 = 1, KIND_DST1 = 2 };
enum WeightMode : int { W_HELMHOLTZ = 0, W_POISSON = 1 };

template <typename T>
struct TBlockDev {
  int rows, cols;    // y extent (number of rows), x extent (row length)
  int kx, ky;        // transform kind along x (rows) and along y (columns)
  FFTPlan fx, fy;
  const cplx<T>* twx;  // exp(-2 pi i m / Lx)
  const cplx<T>* twy;
  const cplx<T>* qx;   // exp(-i pi k / (2 N)) for DCT kinds
  const cplx<T>* qy;
  const T* eigx;       // eigenvalues in internal order
  const T* eigy;
  T* H;                // spectral buffer of column 0
  long long hstride;   // elements between RHS columns
  int pitch;           // row pitch of H (elements)
  int lsx, lsy;        // shared-memory line strides (complex elements)
  int px;              // row pairs per CTA in row passes
  int wy;              // columns per CTA in the column pass (even)
  int groups;          // CTAs of this block in the current pass
};

__device__ __forceinline__ int makhoul_pos(int n, int N) { return (n & 1) ? N - 1 - (n >> 1) : (n >> 1); }

// ---------------------------------------------------------------- packing ---
template <typename T>
__device__ __forceinline__ void put_real(cplx<T>* z, int kind, int N, int n, int part, T val) {
  // part 0 -> real component (line a), 1 -> imaginary component (line b)
  if (kind == KIND_DST1) {
    const int M = N + 1;
    T* p = reinterpret_cast<T*>(z + n + 1) + part;
    T* m = reinterpret_cast<T*>(z + 2 * M - 1 - n) + part;
    *p = val;
    *m = -val;
  } else {
    if (kind == KIND_DST2 && (n & 1)) val = -val;
    reinterpret_cast<T*>(z + makhoul_pos(n, N))[part] = val;
  }
}

template <typename T>
__device__ __forceinline__ void put_pair(cplx<T>* z, int kind, int N, int n, T va, T vb) {
  if (kind == KIND_DST1) {
    const int M = N + 1;
    z[n + 1] = mk(va, vb);
    z[2 * M - 1 - n] = mk(-va, -vb);
  } else {
    if (kind == KIND_DST2 && (n & 1)) { va = -va; vb = -vb; }
    z[makhoul_pos(n, N)] = mk(va, vb);
  }
}

template <typename T>
__device__ __forceinline__ void zero_dst1_ends(cplx<T>* z, int N) {
  z[0] = mk(T(0), T(0));
  z[N + 1] = mk(T(0), T(0));
}

// Forward post-processing: unnormalised coefficient k of lines a and b.
template <typename T>
__device__ __forceinline__ void coef_forward(const cplx<T>* z, int kind, int N, int k,
                                             const cplx<T>* __restrict__ q, T& ya, T& yb) {
  if (kind == KIND_DST1) {
    const cplx<T> Z = z[k + 1];
    ya = -Z.y * T(0.5);
    yb = Z.x * T(0.5);
  } else {
    const cplx<T> Zk = z[k], Zm = conjg(z[k == 0 ? 0 : N - k]);
    const cplx<T> qk = q[k];
    ya = cmul(qk, Zk + Zm).x;
    yb = cmul(qk, Zk - Zm).y;
  }
}

// Inverse pre-processing for DCT kinds: Z_k = V^a_k + i V^b_k with
// V_k = 1/2 conj(q_k) (y_k - i y_{N-k}), y_N = 0.
template <typename T>
__device__ __forceinline__ cplx<T> pre_inverse(T yak, T yam, T ybk, T ybm, cplx<T> qk) {
  const cplx<T> va = cmulc(mk(yak, -yam), qk);
  const cplx<T> vb = cmulc(mk(ybk, -ybm), qk);
  return mk(T(0.5) * (va.x - vb.y), T(0.5) * (va.y + vb.x));
}

// Inverse post-processing: real value n of line a (part 0) or b (part 1),
// after an unscaled inverse FFT (DCT kinds) or a forward FFT (DST-I).
template <typename T>
__device__ __forceinline__ T value_inverse(const cplx<T>* z, int kind, int N, int n, int part) {
  if (kind == KIND_DST1) {
    const cplx<T> Z = z[n + 1];
    const T s = T(1) / T(N + 1);
    return part == 0 ? -Z.y * s : Z.x * s;
  }
  const cplx<T> Z = z[makhoul_pos(n, N)];
  T v = (part == 0 ? Z.x : Z.y) / T(N);
  if (kind == KIND_DST2 && (n & 1)) v = -v;
  return v;
}

__device__ __forceinline__ int inverse_sign(int kind) { return kind == KIND_DST1 ? -1 : 1; }

// Spectral weight of mode (ky, kx).
template <typename T>
__device__ __forceinline__ T spectral_weight(int mode, T mass, T visc, T thr, T ey, T ex) {
  const T lam = ey + ex;
  if (mode == W_HELMHOLTZ) return T(1) / (mass + visc * lam);
  return lam > thr ? mass / lam + visc : T(0);
}

// ============================================================ row passes ====
template <typename T>
struct RowArgs {
  TBlockDev<T> blk[2];
  int nblk;
  const int* active;  // per RHS column (nullptr: all active)
};

__device__ __forceinline__ int pick_block(int nblk, int g0, int& g) {
  g = blockIdx.x;
  if (nblk > 1 && g >= g0) { g -= g0; return 1; }
  return 0;
}

// Forward x-transform of rows: src(blk, col, row, n) -> H.
template <typename T, int VMAX, class Src>
__global__ void __launch_bounds__(kThreads) k_row_forward(RowArgs<T> a, Src src) {
  const int c = blockIdx.y;
  if (a.active && !a.active[c]) return;
  int g;
  const int b = pick_block(a.nblk, a.blk[0].groups, g);
  const TBlockDev<T>& B = a.blk[b];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  const int N = B.cols, P = B.px, LS = B.lsx;
  const int row0 = g * 2 * P;
  const int npairs = min(P, (B.rows - row0 + 1) / 2);
  for (int e = threadIdx.x; e < npairs * N; e += blockDim.x) {
    const int q = e / N, n = e - q * N;
    const int ra = row0 + 2 * q, rb = ra + 1;
    const T va = src(b, c, ra, n);
    const T vb = rb < B.rows ? src(b, c, rb, n) : T(0);
    put_pair(z + q * LS, B.kx, N, n, va, vb);
  }
  if (B.kx == KIND_DST1)
    for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
  __syncthreads();
  fft_lines<T, VMAX>(z, z + P * LS, B.fx, LS, npairs, B.twx, -1);
  T* H = B.H + c * B.hstride;
  for (int e = threadIdx.x; e < npairs * N; e += blockDim.x) {
    const int q = e / N, k = e - q * N;
    const int ra = row0 + 2 * q, rb = ra + 1;
    T ya, yb;
    coef_forward(z + q * LS, B.kx, N, k, B.qx, ya, yb);
    H[(long long)ra * B.pitch + k] = ya;
    if (rb < B.rows) H[(long long)rb * B.pitch + k] = yb;
  }
}

// Inverse x-transform of rows: H -> dst(blk, col, row, n, value, acc).
// Dst may accumulate up to 2 double sums per thread (block-reduced into
// partial[c * gridDim.x * 2 + blockIdx.x * 2 + k]).
template <typename T, int VMAX, class Dst>
__global__ void __launch_bounds__(kThreads) k_row_inverse(RowArgs<T> a, Dst dst, double* partial) {
  const int c = blockIdx.y;
  if (a.active && !a.active[c]) return;
  int g;
  const int b = pick_block(a.nblk, a.blk[0].groups, g);
  const TBlockDev<T>& B = a.blk[b];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  __shared__ double red[64];
  const int N = B.cols, P = B.px, LS = B.lsx;
  const int row0 = g * 2 * P;
  const int npairs = min(P, (B.rows - row0 + 1) / 2);
  const T* H = B.H + c * B.hstride;
  if (B.kx == KIND_DST1) {
    for (int e = threadIdx.x; e < npairs * N; e += blockDim.x) {
      const int q = e / N, k = e - q * N;
      const int ra = row0 + 2 * q, rb = ra + 1;
      const T va = H[(long long)ra * B.pitch + k];
      const T vb = rb < B.rows ? H[(long long)rb * B.pitch + k] : T(0);
      put_pair(z + q * LS, KIND_DST1, N, k, va, vb);
    }
    for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
  } else {
    for (int e = threadIdx.x; e < npairs * N; e += blockDim.x) {
      const int q = e / N, k = e - q * N;
      const int ra = row0 + 2 * q, rb = ra + 1;
      const int m = N - k;  // partner; y_N = 0
      const T yak = H[(long long)ra * B.pitch + k];
      const T yam = k ? H[(long long)ra * B.pitch + m] : T(0);
      T ybk = T(0), ybm = T(0);
      if (rb < B.rows) {
        ybk = H[(long long)rb * B.pitch + k];
        ybm = k ? H[(long long)rb * B.pitch + m] : T(0);
      }
      z[q * LS + k] = pre_inverse(yak, yam, ybk, ybm, B.qx[k]);
    }
  }
  __syncthreads();
  fft_lines<T, VMAX>(z, z + P * LS, B.fx, LS, npairs, B.twx, inverse_sign(B.kx));
  double acc[2] = {0.0, 0.0};
  for (int e = threadIdx.x; e < npairs * N; e += blockDim.x) {
    const int q = e / N, n = e - q * N;
    const int ra = row0 + 2 * q, rb = ra + 1;
    dst(b, c, ra, n, value_inverse(z + q * LS, B.kx, N, n, 0), acc);
    if (rb < B.rows) dst(b, c, rb, n, value_inverse(z + q * LS, B.kx, N, n, 1), acc);
  }
  if (partial) {
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
      const int slot = (c * gridDim.x + blockIdx.x) * 2;
      partial[slot] = acc[0];
      partial[slot + 1] = acc[1];
    }
  }
}

// ============================================================ column pass ===
template <typename T>
struct ColArgs {
  TBlockDev<T> blk[2];
  int nblk;
  const int* active;
  int mode;                 // WeightMode
  const double* shift;      // per RHS column: (mass, viscosity)
  T thr;                    // Poisson zero-mode threshold
};

template <typename T, int VMAX>
__global__ void __launch_bounds__(kThreads) k_column(ColArgs<T> a) {
  const int c = blockIdx.y;
  if (a.active && !a.active[c]) return;
  int g;
  const int b = pick_block(a.nblk, a.blk[0].groups, g);
  const TBlockDev<T>& B = a.blk[b];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  const int N = B.rows, W = B.wy, LS = B.lsy, kind = B.ky;
  const int col0 = g * W;
  const int ncols = min(W, B.cols - col0);
  const int nl = (ncols + 1) / 2;
  T* H = B.H + c * B.hstride;
  const T mass = T(a.shift[2 * c]), visc = T(a.shift[2 * c + 1]);
  // load the strip, two columns per complex line
  for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
    const int n = e / W, j = e - n * W;
    if (j < 2 * nl) {
      const T v = j < ncols ? H[(long long)n * B.pitch + col0 + j] : T(0);
      put_real(z + (j >> 1) * LS, kind, N, n, j & 1, v);
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < nl; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
  __syncthreads();
  fft_lines<T, VMAX>(z, z + W / 2 * LS, B.fy, LS, nl, B.twy, -1);
  // forward post-processing, spectral weight, inverse pre-processing (in place)
  if (kind == KIND_DST1) {
    for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
      const int q = e / N, k = e - q * N;
      cplx<T>* zl = z + q * LS;
      const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
      const T ey = B.eigy[k];
      const T wa = spectral_weight<T>(a.mode, mass, visc, a.thr, ey, B.eigx[ca]);
      const T wb = spectral_weight<T>(a.mode, mass, visc, a.thr, ey, B.eigx[cb]);
      const cplx<T> Z = zl[k + 1];
      const T sa = -Z.y * T(0.5) * wa, sb = Z.x * T(0.5) * wb;
      zl[k + 1] = mk(sa, sb);
      zl[2 * (N + 1) - 1 - k] = mk(-sa, -sb);
      if (k == 0) {
        zl[0] = mk(T(0), T(0));
        zl[N + 1] = mk(T(0), T(0));
      }
    }
  } else {
    const int half = N / 2 + 1;
    for (int e = threadIdx.x; e < nl * half; e += blockDim.x) {
      const int q = e / half, k = e - q * half;
      cplx<T>* zl = z + q * LS;
      const int m = k == 0 ? 0 : N - k;
      const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
      const cplx<T> Zk = zl[k], Zm = zl[m];
      const cplx<T> qk = B.qy[k], qm = B.qy[m];
      T yak = cmul(qk, Zk + conjg(Zm)).x, ybk = cmul(qk, Zk - conjg(Zm)).y;
      T yam = cmul(qm, Zm + conjg(Zk)).x, ybm = cmul(qm, Zm - conjg(Zk)).y;
      const T eyk = B.eigy[k], eym = B.eigy[m], exa = B.eigx[ca], exb = B.eigx[cb];
      yak *= spectral_weight<T>(a.mode, mass, visc, a.thr, eyk, exa);
      ybk *= spectral_weight<T>(a.mode, mass, visc, a.thr, eyk, exb);
      yam *= spectral_weight<T>(a.mode, mass, visc, a.thr, eym, exa);
      ybm *= spectral_weight<T>(a.mode, mass, visc, a.thr, eym, exb);
      if (k == 0) {
        zl[0] = pre_inverse(yak, T(0), ybk, T(0), qk);
      } else {
        zl[k] = pre_inverse(yak, yam, ybk, ybm, qk);
        if (m != k) zl[m] = pre_inverse(yam, yak, ybm, ybk, qm);
      }
    }
  }
  __syncthreads();
  fft_lines<T, VMAX>(z, z + W / 2 * LS, B.fy, LS, nl, B.twy, inverse_sign(kind));
  for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
    const int n = e / W, j = e - n * W;
    if (j < ncols) H[(long long)n * B.pitch + col0 + j] = value_inverse(z + (j >> 1) * LS, kind, N, n, j & 1);
  }
}

}  // namespace macsav
