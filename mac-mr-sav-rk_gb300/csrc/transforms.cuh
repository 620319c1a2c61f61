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
// Launch shape of a power-of-two transform pass (p2_shape, fftp.cuh).
enum P2Shape : int { P2_AUTO = 0, P2_PLAIN = 1, P2_DOUBLED = 2, P2_SPLIT = 3 };

template <typename T>
struct TBlockDev {
  int rows, cols;    // y extent (number of rows), x extent (row length)
  int kx, ky;        // transform kind along x (rows) and along y (columns)
  FFTPlan fx, fy;
  const cplx<T>* twx;  // exp(-2 pi i m / Lx)
  const cplx<T>* twy;
  const cplx<T>* twpx;  // the same twiddles in Stockham-pass order (power-of-two Lx, fftp.cuh)
  const cplx<T>* twpy;
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
  int tpl;             // threads per line of a specialised pass (set per launch)
  int shape[3];        // launch shapes of the forward row, column and inverse row passes (P2Shape, fftp.cuh)
  FastDiv fcols, frows, fw, fvpr, fhalf;  // divisors of the element loops
  T sx, sy;            // inverse normalisation of the x / y transforms
};

__device__ __forceinline__ int makhoul_pos(int n, int N) { return (n & 1) ? N - 1 - (n >> 1) : (n >> 1); }

// ---------------------------------------------------------------- packing ---
// Element k of a shared line sits at z[ix(k)]: the identity for the generic
// kernels, a bank swizzle for the power-of-two kernels (fftp.cuh).
struct IdIx {
  __device__ __forceinline__ int operator()(int i) const { return i; }
};

template <typename T, class Ix = IdIx>
__device__ __forceinline__ void put_real(cplx<T>* z, int kind, int N, int n, int part, T val, Ix ix = Ix{}) {
  // part 0 -> real component (line a), 1 -> imaginary component (line b)
  if (kind == KIND_DST1) {
    const int M = N + 1;
    T* p = reinterpret_cast<T*>(z + ix(n + 1)) + part;
    T* m = reinterpret_cast<T*>(z + ix(2 * M - 1 - n)) + part;
    *p = val;
    *m = -val;
  } else {
    if (kind == KIND_DST2 && (n & 1)) val = -val;
    reinterpret_cast<T*>(z + ix(makhoul_pos(n, N)))[part] = val;
  }
}

template <typename T, class Ix = IdIx>
__device__ __forceinline__ void put_pair(cplx<T>* z, int kind, int N, int n, T va, T vb, Ix ix = Ix{}) {
  if (kind == KIND_DST1) {
    const int M = N + 1;
    z[ix(n + 1)] = mk(va, vb);
    z[ix(2 * M - 1 - n)] = mk(-va, -vb);
  } else {
    if (kind == KIND_DST2 && (n & 1)) { va = -va; vb = -vb; }
    z[ix(makhoul_pos(n, N))] = mk(va, vb);
  }
}

template <typename T, class Ix = IdIx>
__device__ __forceinline__ void zero_dst1_ends(cplx<T>* z, int N, Ix ix = Ix{}) {
  z[ix(0)] = mk(T(0), T(0));
  z[ix(N + 1)] = mk(T(0), T(0));
}

// Forward post-processing: unnormalised coefficient k of lines a and b.
template <typename T, class Ix = IdIx>
__device__ __forceinline__ void coef_forward(const cplx<T>* z, int kind, int N, int k,
                                             const cplx<T>* __restrict__ q, T& ya, T& yb, Ix ix = Ix{}) {
  if (kind == KIND_DST1) {
    const cplx<T> Z = z[ix(k + 1)];
    ya = -Z.y * T(0.5);
    yb = Z.x * T(0.5);
  } else {
    const cplx<T> Zk = z[ix(k)], Zm = conjg(z[ix(k == 0 ? 0 : N - k)]);
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
// after an unscaled inverse FFT (DCT kinds) or a forward FFT (DST-I); `scale`
// is the normalisation 1/N (DCT kinds) or 1/(N+1) (DST-I), precomputed.
template <typename T, class Ix = IdIx>
__device__ __forceinline__ T value_inverse(const cplx<T>* z, int kind, int N, int n, int part, T scale,
                                           Ix ix = Ix{}) {
  if (kind == KIND_DST1) {
    const cplx<T> Z = z[ix(n + 1)];
    return part == 0 ? -Z.y * scale : Z.x * scale;
  }
  const cplx<T> Z = z[ix(makhoul_pos(n, N))];
  T v = (part == 0 ? Z.x : Z.y) * scale;
  if (kind == KIND_DST2 && (n & 1)) v = -v;
  return v;
}

__device__ __forceinline__ int inverse_sign(int kind) { return kind == KIND_DST1 ? -1 : 1; }

// Spectral weight of mode (ky, kx).  The FP32 path (an inexact inner solve
// under FP64 defect correction) uses the hardware reciprocal; FP64 divides.
template <typename T>
__device__ __forceinline__ T recip(T x) {
  if constexpr (sizeof(T) == 4) return __frcp_rn(x);
  else return T(1) / x;
}
template <typename T>
__device__ __forceinline__ T spectral_weight(int mode, T mass, T visc, T thr, T ey, T ex) {
  const T lam = ey + ex;
  if (mode == W_HELMHOLTZ) return recip(mass + visc * lam);
  return lam > thr ? mass * recip(lam) + visc : T(0);
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

constexpr int kStage = 4;  // independent global loads in flight per thread

// Forward x-transform of rows: src(blk, col, row, n) -> H.
template <typename T, int VMAX, class Src>
__global__ void __launch_bounds__(kFFTThreads, sizeof(T) == 4 ? 2 : 1) k_row_forward(RowArgs<T> a, Src src) {
  pdl_wait();
  const int c = blockIdx.y;
  if (a.active && !a.active[c]) return;
  int g;
  const int b = pick_block(a.nblk, a.blk[0].groups, g);
  const TBlockDev<T>& B = a.blk[b];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  const int N = B.cols, P = B.px, LS = B.lsx, rows = B.rows, kind = B.kx;
  const int row0 = g * 2 * P;
  const int npairs = min(P, (rows - row0 + 1) / 2);
  const int total = npairs * N;
  for (int base = threadIdx.x; base < total; base += kStage * blockDim.x) {
    T va[kStage], vb[kStage];
#pragma unroll
    for (int u = 0; u < kStage; ++u) {
      const int e = base + u * blockDim.x;
      va[u] = T(0);
      vb[u] = T(0);
      if (e < total) {
        const int q = B.fcols.div(e), n = e - q * N, ra = row0 + 2 * q;
        va[u] = src(b, c, ra, n);
        if (ra + 1 < rows) vb[u] = src(b, c, ra + 1, n);
      }
    }
#pragma unroll
    for (int u = 0; u < kStage; ++u) {
      const int e = base + u * blockDim.x;
      if (e < total) {
        const int q = B.fcols.div(e), n = e - q * N;
        put_pair(z + q * LS, kind, N, n, va[u], vb[u]);
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
  __syncthreads();
  fft_lines<T, VMAX>(z, z + P * LS, B.fx, LS, npairs, B.twx, -1);
  T* H = B.H + c * B.hstride;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int q = B.fcols.div(e), k = e - q * N;
    const int ra = row0 + 2 * q;
    T ya, yb;
    coef_forward(z + q * LS, kind, N, k, B.qx, ya, yb);
    H[(long long)ra * B.pitch + k] = ya;
    if (ra + 1 < rows) H[(long long)ra * B.pitch + B.pitch + k] = yb;
  }
}

// Inverse x-transform of rows: H -> dst.  Dst has a two-phase interface so
// its global loads can be issued together: aux = dst.load(b, c, row, n), then
// dst.store(b, c, row, n, value, aux, acc) with acc two per-thread sums.  When
// `partial` is set, the sums are block-reduced into
// partial[(c * gridDim.x + blockIdx.x) * 2 + k] and the last block runs fin().
template <typename T, int VMAX, class Dst, class Fin>
__global__ void __launch_bounds__(kFFTThreads, sizeof(T) == 4 ? 2 : 1) k_row_inverse(RowArgs<T> a, Dst dst, double* partial, Fin fin,
                                                             unsigned int* counter) {
  pdl_wait();
  const int c = blockIdx.y;
  const bool live = !a.active || a.active[c];
  Acc<T> acc[2];
  if (live) {
    int g;
    const int b = pick_block(a.nblk, a.blk[0].groups, g);
    const TBlockDev<T>& B = a.blk[b];
    extern __shared__ __align__(16) unsigned char smraw[];
    cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
    const int N = B.cols, P = B.px, LS = B.lsx, rows = B.rows, kind = B.kx;
    const int row0 = g * 2 * P;
    const int npairs = min(P, (rows - row0 + 1) / 2);
    const int total = npairs * N;
    const T* H = B.H + c * B.hstride;
    const long long pitch = B.pitch;
    for (int base = threadIdx.x; base < total; base += kStage * blockDim.x) {
      T yak[kStage], yam[kStage], ybk[kStage], ybm[kStage];
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        yak[u] = yam[u] = ybk[u] = ybm[u] = T(0);
        if (e < total) {
          const int q = B.fcols.div(e), k = e - q * N, ra = row0 + 2 * q;
          const T* ha = H + ra * pitch;
          const bool hb = ra + 1 < rows;
          yak[u] = ha[k];
          if (hb) ybk[u] = ha[pitch + k];
          if (kind != KIND_DST1 && k) {
            yam[u] = ha[N - k];
            if (hb) ybm[u] = ha[pitch + N - k];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        if (e < total) {
          const int q = B.fcols.div(e), k = e - q * N;
          if (kind == KIND_DST1) put_pair(z + q * LS, KIND_DST1, N, k, yak[u], ybk[u]);
          else z[q * LS + k] = pre_inverse(yak[u], yam[u], ybk[u], ybm[u], B.qx[k]);
        }
      }
    }
    if (kind == KIND_DST1)
      for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
    __syncthreads();
    fft_lines<T, VMAX>(z, z + P * LS, B.fx, LS, npairs, B.twx, inverse_sign(kind));
    for (int base = threadIdx.x; base < total; base += kStage * blockDim.x) {
      typename Dst::aux_t xa[kStage], xb[kStage];
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        if (e < total) {
          const int q = B.fcols.div(e), n = e - q * N, ra = row0 + 2 * q;
          xa[u] = dst.load(b, c, ra, n);
          if (ra + 1 < rows) xb[u] = dst.load(b, c, ra + 1, n);
        }
      }
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        if (e < total) {
          const int q = B.fcols.div(e), n = e - q * N, ra = row0 + 2 * q;
          dst.store(b, c, ra, n, value_inverse(z + q * LS, kind, N, n, 0, B.sx), xa[u], acc);
          if (ra + 1 < rows) dst.store(b, c, ra + 1, n, value_inverse(z + q * LS, kind, N, n, 1, B.sx), xb[u], acc);
        }
      }
    }
  }
  if (partial) {
    write_sums<T, 2>(acc, partial, 2);
    last_block_finish(fin, counter);
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

// Column strips of W columns (W a multiple of the 16-byte vector width, the
// strip start 16-byte aligned; H's row padding is zero, so full-width vector
// loads past the last column read zeros).
template <typename T, int VMAX>
__global__ void __launch_bounds__(kFFTThreads, sizeof(T) == 4 ? 2 : 1) k_column(ColArgs<T> a) {
  pdl_wait();
  const int c = blockIdx.y;
  if (a.active && !a.active[c]) return;
  int g;
  const int b = pick_block(a.nblk, a.blk[0].groups, g);
  const TBlockDev<T>& B = a.blk[b];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  using vec_t = typename Vec16<T>::type;
  constexpr int V = Vec16<T>::n;
  const int N = B.rows, W = B.wy, LS = B.lsy, kind = B.ky;
  const int col0 = g * W;
  const int ncols = min(W, B.cols - col0);
  const int nl = (ncols + 1) / 2;
  T* H = B.H + c * B.hstride;
  const long long pitch = B.pitch;
  const T mass = T(a.shift[2 * c]), visc = T(a.shift[2 * c + 1]);
  const bool vec = (W % V) == 0;
  const int vpr = W / V, totv = N * vpr;
  if (!vec) {  // narrow strips (W < 16 bytes): scalar loads
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
      const int n = B.fw.div(e), j = e - n * W;
      if (j < 2 * nl) put_real(z + (j >> 1) * LS, kind, N, n, j & 1, j < ncols ? H[n * pitch + col0 + j] : T(0));
    }
  }
  // load the strip (16-byte vectors), two columns per complex line
  for (int base = threadIdx.x; vec && base < totv; base += kStage * blockDim.x) {
    vec_t v[kStage];
#pragma unroll
    for (int u = 0; u < kStage; ++u) {
      const int e = base + u * blockDim.x;
      if (e < totv) {
        const int n = B.fvpr.div(e), jv = e - n * vpr;
        v[u] = *reinterpret_cast<const vec_t*>(H + n * pitch + col0 + jv * V);
      }
    }
#pragma unroll
    for (int u = 0; u < kStage; ++u) {
      const int e = base + u * blockDim.x;
      if (e < totv) {
        const int n = B.fvpr.div(e), jv = e - n * vpr;
        const T* comp = reinterpret_cast<const T*>(&v[u]);
#pragma unroll
        for (int k = 0; k < V; ++k) {
          const int j = jv * V + k;
          if (j < 2 * nl) put_real(z + (j >> 1) * LS, kind, N, n, j & 1, j < ncols ? comp[k] : T(0));
        }
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < nl; q += blockDim.x) zero_dst1_ends(z + q * LS, N);
  __syncthreads();
  fft_lines<T, VMAX>(z, z + W / 2 * LS, B.fy, LS, nl, B.twy, -1);
  // forward post-processing, spectral weight, inverse pre-processing (in place)
  if (kind == KIND_DST1) {
    for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
      const int q = B.frows.div(e), k = e - q * N;
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
      const int q = B.fhalf.div(e), k = e - q * half;
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
  if (vec && ncols == W) {
    for (int e = threadIdx.x; e < totv; e += blockDim.x) {
      const int n = B.fvpr.div(e), jv = e - n * vpr;
      vec_t v;
      T* comp = reinterpret_cast<T*>(&v);
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const int j = jv * V + k;
        comp[k] = value_inverse(z + (j >> 1) * LS, kind, N, n, j & 1, B.sy);
      }
      *reinterpret_cast<vec_t*>(H + n * pitch + col0 + jv * V) = v;
    }
  } else {
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
      const int n = B.fw.div(e), j = e - n * W;
      if (j < ncols) H[n * pitch + col0 + j] = value_inverse(z + (j >> 1) * LS, kind, N, n, j & 1, B.sy);
    }
  }
}

}  // namespace macsav
