// Power-of-two transform passes with compile-time FFT length.
//
// For L = 2^k in [64, 4096] every pass kernel is specialised on L: each line
// is transformed by G = L/8 threads, each owning one radix-8 butterfly per
// Stockham pass (register-resident 8-point DFTs, the last pass radix 2 or 4
// when log2 L is not a multiple of 3), so log8(L) passes with all index
// arithmetic folded to shifts and masks.  A CTA holds NL = blockDim.x / tpl
// lines (tpl = G or 2G threads per line, below).  Packing, spectral weights
// and the post/pre-processing are the same as in the generic kernels
// (transforms.cuh).
//
// Shared lines are stored bank-swizzled (SwIx below).  Each launch picks a
// shape (threads per line, p2_shape below; TBlockDev::tpl carries it).
// Measured on GB300 (512^2 sdirk3_mrsav step): the swizzle takes the FP64
// step from 11.54 to 11.13 ms.  A ping-pong buffer pair (one barrier per
// pass) and a shared copy of the twiddle table gave nothing on top and are
// not used.
#pragma once
#include "transforms.cuh"

namespace macsav {

constexpr int kE = 8;  // elements per thread per line

// Launch shape of a pass of length L over `lines` lines per CTA:
//   P2_PLAIN    G = L/8 threads per line, one radix-8 butterfly per pass;
//   P2_DOUBLED  2G threads per line; the packing and unpacking loops, the
//               longer dependent chains of these latency-bound passes, run on
//               twice the warps while the extra threads only join the FFT
//               barriers (the CTA stays within kFFTThreads);
//   P2_SPLIT    G/2 threads per line, two radix-8 butterflies per thread and
//               pass (FP32, L from 1024 to 4096).
// P2_AUTO picks by block: split for FP32 L >= 2048, doubled for FP32 blocks
// of at most 512 x 512, plain otherwise.  Measured on GB300 (two right-hand
// sides, u and v concurrently): at 1024^2 the split DST-I column pass of the
// v block (L = 2048) takes 32.5 us against 39.7 us plain (two waves of
// 512-thread CTAs at 44 registers become one of 256-thread CTAs), and the
// velocity row-inverse pair 22.3 against 25.9 us; the split L = 1024 column
// pass of the u block, already one wave, 27.2 against 26.4 us; at 512^2 the
// doubled threads took the FP32 step from 4.74 to 4.63 ms (with the
// swizzle) and the split L = 1024 column pass is twice as slow.  Which
// thread computes a butterfly does not change its arithmetic: every shape
// gives the same bits.
// (P2Shape: transforms.cuh, beside TBlockDev::shape)

template <typename T>
inline int p2_shape(const TBlockDev<T>& B, int L, int lines, int shape) {
  const int G = L / kE;
  const bool can_split = sizeof(T) == 4 && L >= 1024 && L <= 4096;
  const bool can_double = 2 * G * lines <= kFFTThreads;
  if (shape == P2_AUTO) {
    if (can_split && L >= 2048) return P2_SPLIT;
    if (sizeof(T) == 4 && (long long)B.rows * B.cols <= 512LL * 512 && can_double) return P2_DOUBLED;
    return P2_PLAIN;
  }
  if ((shape == P2_SPLIT && !can_split) || (shape == P2_DOUBLED && !can_double)) return P2_PLAIN;
  return shape;
}

// Threads per line of a resolved shape.
inline int p2_tpl(int L, int shape) {
  return shape == P2_SPLIT ? L / 16 : (shape == P2_DOUBLED ? L / 4 : L / 8);
}

// Shared bytes of a CTA holding `lines` lines of length L.
template <typename T>
inline size_t p2_smem(int L, int lines) {
  return size_t(lines) * size_t(L) * sizeof(cplx<T>);
}

// Bank swizzle of element i of a shared line (a bijection on each aligned
// group of 128 elements).  The first Stockham pass writes each thread's 8
// outputs contiguously (thread stride 8 elements) and the second writes
// groups of 8 that are 64 elements apart; unswizzled, those stores are
// 8-way and 2-way bank conflicts for 8-byte elements (8-way for 16-byte
// ones).  XOR-ing bits 0-2 with bits 3-5 and bit 3 with bit 6 makes every
// pass's loads and stores conflict-free (16 threads of 8 bytes or 8 threads
// of 16 bytes per shared-memory wavefront).
// Bits 3-6 of i XOR-ed into bits 0-3: a GF(2)-linear map, so for bit-disjoint
// a and b (a + b = a ^ b) swz(a + b) = swz(a) ^ swz(b), and swz(b) = b when b
// is a multiple of 128.  The Stockham passes use this to fold the compile-time
// part of every shared address into a constant (an immediate offset where the
// constant is a multiple of 128, one XOR otherwise).
__host__ __device__ constexpr int swz(int i) { return i ^ ((i >> 3) & 15); }
struct SwIx {
  __device__ __forceinline__ int operator()(int i) const { return swz(i); }
};

// swz(b + C) for b bit-disjoint from the constant C (C's lowest set bit above b).
template <int STEP>
__device__ __forceinline__ int swz_plus(int sb, int c) {
  if constexpr (STEP % 128 == 0) return sb + c;
  else return sb ^ swz(c);
}

template <typename T, int SIGN>
__device__ __forceinline__ cplx<T> tw_at(const cplx<T>* __restrict__ tw, int m) {
  cplx<T> w;
  if constexpr (sizeof(T) == 4) {
    const float2 f = __ldg(reinterpret_cast<const float2*>(tw) + m);
    w = mk(T(f.x), T(f.y));
  } else {
    const double2 d = __ldg(reinterpret_cast<const double2*>(tw) + m);
    w = mk(T(d.x), T(d.y));
  }
  return SIGN < 0 ? w : conjg(w);
}

template <typename T, int SIGN>
__device__ __forceinline__ void dft4s(cplx<T>& a, cplx<T>& b, cplx<T>& c, cplx<T>& d) {
  const cplx<T> s0 = a + c, d0 = a - c, s1 = b + d, d1 = mul_i(b - d, SIGN);
  a = s0 + s1;
  c = s0 - s1;
  b = d0 + d1;
  d = d0 - d1;
}

// R-point DFT (R = 2, 4, 8) of v in place, natural output order.
template <typename T, int R, int SIGN>
__device__ __forceinline__ void dftR(cplx<T> (&v)[R]) {
  if constexpr (R == 2) {
    const cplx<T> t = v[0] - v[1];
    v[0] = v[0] + v[1];
    v[1] = t;
  } else if constexpr (R == 4) {
    dft4s<T, SIGN>(v[0], v[1], v[2], v[3]);
  } else {
    // X_{2m} = DFT4(x_k + x_{k+4}), X_{2m+1} = DFT4((x_k - x_{k+4}) W8^k)
    const T h = T(0.70710678118654752440);
    cplx<T> a0 = v[0] + v[4], a1 = v[1] + v[5], a2 = v[2] + v[6], a3 = v[3] + v[7];
    cplx<T> b0 = v[0] - v[4], b1 = v[1] - v[5], b2 = v[2] - v[6], b3 = v[3] - v[7];
    if constexpr (SIGN < 0) {
      b1 = mk(h * (b1.x + b1.y), h * (b1.y - b1.x));   // * (1 - i)/sqrt2
      b3 = mk(h * (b3.y - b3.x), -h * (b3.x + b3.y));  // * (-1 - i)/sqrt2
    } else {
      b1 = mk(h * (b1.x - b1.y), h * (b1.x + b1.y));   // * (1 + i)/sqrt2
      b3 = mk(-h * (b3.x + b3.y), h * (b3.x - b3.y));  // * (-1 + i)/sqrt2
    }
    b2 = mul_i(b2, SIGN);
    dft4s<T, SIGN>(a0, a1, a2, a3);
    dft4s<T, SIGN>(b0, b1, b2, b3);
    v[0] = a0; v[2] = a1; v[4] = a2; v[6] = a3;
    v[1] = b0; v[3] = b1; v[5] = b2; v[7] = b3;
  }
}

// Stockham passes on one (swizzled) line z by its first G threads (L/8, or
// L/16 for the split launches, whose threads own two radix-8 butterflies per
// pass); thread t < G owns butterflies j = t + q G, threads t >= G (doubled
// launches) only join the barriers.  Every thread of the CTA must call this
// (two block barriers per pass).  Which thread computes a butterfly does not
// change its arithmetic, so every G gives the same bits.
// tw: the twiddles in pass order (TBlockDev::twpx / twpy, plan.cu's
// pass_twiddles); OFF is this pass's offset in that table.
template <typename T, int L, int NS, int SIGN, int G = L / kE, int OFF = 0>
__device__ __forceinline__ void fft_p2(cplx<T>* z, int t, const cplx<T>* __restrict__ tw) {
  constexpr int R = (L / NS >= kE) ? kE : L / NS;
  constexpr int NB = (L / R) / G;
  constexpr int STRIDE = L / R;
  static_assert(NB * G == L / R, "threads per line must divide the butterflies of every pass");
  const SwIx ix;
  cplx<T> v[NB][R];
  const bool own = t < G;
  if (own) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      // j < STRIDE and r * STRIDE share no bits, so swz(j + r STRIDE) folds
      const int j = t + q * G;
      const int k = j & (NS - 1);
      const int sj = ix(j);
#pragma unroll
      for (int r = 0; r < R; ++r) v[q][r] = z[swz_plus<STRIDE>(sj, r * STRIDE)];
      if constexpr (NS > 1) {
        const cplx<T>* twk = tw + OFF + k;  // row r - 1 of this pass's table at (r - 1) NS
#pragma unroll
        for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], tw_at<T, SIGN>(twk, (r - 1) * NS));
      }
      dftR<T, R, SIGN>(v[q]);
    }
  }
  __syncthreads();
  if (own) {
#pragma unroll
    for (int q = 0; q < NB; ++q) {
      const int j = t + q * G;
      const int k = j & (NS - 1);
      // (j - k) R is a multiple of NS R and k < NS: r * NS shares no bits
      const int sb = ix((j - k) * R + k);
#pragma unroll
      for (int r = 0; r < R; ++r) z[swz_plus<NS>(sb, r * NS)] = v[q][r];
    }
  }
  __syncthreads();
  if constexpr (NS * R < L) fft_p2<T, L, NS * R, SIGN, G, OFF + (NS > 1 ? (R - 1) * NS : 0)>(z, t, tw);
}

// ------------------------------------------------------------ row passes ---
// One block (u, v or p) per launch; NL = blockDim.x / B.tpl line pairs per CTA.
template <typename T, int L, class Src, int GT = L / kE>
__global__ void __launch_bounds__(kFFTThreads) k_row_forward_p2(TBlockDev<T> B, const int* active, Src src, int bk) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  const int TPL = B.tpl;
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  const int NL = blockDim.x / TPL;
  const cplx<T>* tw = B.twpx;
  const int N = B.cols, rows = B.rows, kind = B.kx;
  const int row0 = blockIdx.x * 2 * NL;
  const int npairs = min(NL, (rows - row0 + 1) / 2);
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
        va[u] = src(bk, c, ra, n);
        if (ra + 1 < rows) vb[u] = src(bk, c, ra + 1, n);
      }
    }
#pragma unroll
    for (int u = 0; u < kStage; ++u) {
      const int e = base + u * blockDim.x;
      if (e < total) {
        const int q = B.fcols.div(e), n = e - q * N;
        put_pair(z + q * L, kind, N, n, va[u], vb[u], SwIx{});
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * L, N, SwIx{});
  __syncthreads();
  fft_p2<T, L, 1, -1, GT>(z + (threadIdx.x / TPL) * L, threadIdx.x % TPL, tw);
  T* H = B.H + c * B.hstride;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int q = B.fcols.div(e), k = e - q * N;
    const int ra = row0 + 2 * q;
    T ya, yb;
    coef_forward(z + q * L, kind, N, k, B.qx, ya, yb, SwIx{});
    H[(long long)ra * B.pitch + k] = ya;
    if (ra + 1 < rows) H[(long long)ra * B.pitch + B.pitch + k] = yb;
  }
}

template <typename T, int L, class Dst, class Fin, int GT = L / kE>
__global__ void __launch_bounds__(kFFTThreads) k_row_inverse_p2(TBlockDev<T> B, const int* active, Dst dst, int bk,
                                                                double* partial, Fin fin, unsigned int* counter) {
  pdl_wait();
  const int c = blockIdx.y;
  const int TPL = B.tpl;
  const bool live = !active || active[c];
  Acc<T> acc[2];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  if (live) {
    const int NL = blockDim.x / TPL;
    const cplx<T>* tw = B.twpx;
    const int N = B.cols, rows = B.rows, kind = B.kx;
    const int row0 = blockIdx.x * 2 * NL;
    const int npairs = min(NL, (rows - row0 + 1) / 2);
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
          if (kind == KIND_DST1) put_pair(z + q * L, KIND_DST1, N, k, yak[u], ybk[u], SwIx{});
          else z[q * L + SwIx{}(k)] = pre_inverse(yak[u], yam[u], ybk[u], ybm[u], B.qx[k]);
        }
      }
    }
    if (kind == KIND_DST1)
      for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * L, N, SwIx{});
      __syncthreads();
    cplx<T>* za = z + (threadIdx.x / TPL) * L;
    if (kind == KIND_DST1) fft_p2<T, L, 1, -1, GT>(za, threadIdx.x % TPL, tw);
    else fft_p2<T, L, 1, 1, GT>(za, threadIdx.x % TPL, tw);
      for (int base = threadIdx.x; base < total; base += kStage * blockDim.x) {
      typename Dst::aux_t xa[kStage], xb[kStage];
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        if (e < total) {
          const int q = B.fcols.div(e), n = e - q * N, ra = row0 + 2 * q;
          xa[u] = dst.load(bk, c, ra, n);
          if (ra + 1 < rows) xb[u] = dst.load(bk, c, ra + 1, n);
        }
      }
#pragma unroll
      for (int u = 0; u < kStage; ++u) {
        const int e = base + u * blockDim.x;
        if (e < total) {
          const int q = B.fcols.div(e), n = e - q * N, ra = row0 + 2 * q;
          dst.store(bk, c, ra, n, value_inverse(z + q * L, kind, N, n, 0, B.sx, SwIx{}), xa[u], acc);
          if (ra + 1 < rows) dst.store(bk, c, ra + 1, n, value_inverse(z + q * L, kind, N, n, 1, B.sx, SwIx{}), xb[u], acc);
        }
      }
    }
  }
  if (partial) {
    write_sums<T, 2>(acc, partial, 2);
    last_block_finish(fin, counter);
  }
}

// ----------------------------------------------------------- column pass ---
// NL = blockDim.x / B.tpl complex lines = W = 2 NL columns per CTA; GT
// threads per line compute the FFTs (L/8, or L/16 for the split launch).
template <typename T, int L, int GT = L / kE>
__global__ void __launch_bounds__(kFFTThreads) k_column_p2(TBlockDev<T> B, const int* active, int mode,
                                                          const double* shift, T thr) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  const int TPL = B.tpl;
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  using vec_t = typename Vec16<T>::type;
  constexpr int V = Vec16<T>::n;
  const int NL = blockDim.x / TPL;
  const cplx<T>* tw = B.twpy;
  const int W = 2 * NL;
  const int N = B.rows, kind = B.ky;
  const int col0 = blockIdx.x * W;
  const int ncols = min(W, B.cols - col0);
  const int nl = (ncols + 1) / 2;
  T* H = B.H + c * B.hstride;
  const long long pitch = B.pitch;
  const T mass = T(shift[2 * c]), visc = T(shift[2 * c + 1]);
  const bool vec = (W % V) == 0;
  const int vpr = W / V, totv = N * vpr;
  if (!vec) {
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
      const int n = B.fw.div(e), j = e - n * W;
      if (j < 2 * nl) put_real(z + (j >> 1) * L, kind, N, n, j & 1, j < ncols ? H[n * pitch + col0 + j] : T(0), SwIx{});
    }
  }
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
        // columns (2h, 2h + 1) of the vector are the real and imaginary parts of one line
#pragma unroll
        for (int h = 0; h < V / 2; ++h) {
          const int j = jv * V + 2 * h;
          if (j < 2 * nl)
            put_pair(z + (j >> 1) * L, kind, N, n, j < ncols ? comp[2 * h] : T(0),
                     j + 1 < ncols ? comp[2 * h + 1] : T(0), SwIx{});
        }
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < nl; q += blockDim.x) zero_dst1_ends(z + q * L, N, SwIx{});
  __syncthreads();
  const int line = threadIdx.x / TPL, t = threadIdx.x % TPL;
  fft_p2<T, L, 1, -1, GT>(z + line * L, t, tw);
  // spectral weights: a thread takes one wavenumber k for every line of the
  // CTA (the y tables read once per k, the lines' x eigenvalues broadcast)
  if (kind == KIND_DST1) {
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const T ey = B.eigy[k];
      for (int q = 0; q < nl; ++q) {
        cplx<T>* y = z + q * L;
        const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
        const T wa = spectral_weight<T>(mode, mass, visc, thr, ey, B.eigx[ca]);
        const T wb = spectral_weight<T>(mode, mass, visc, thr, ey, B.eigx[cb]);
        const SwIx ix;
        const cplx<T> Z = y[ix(k + 1)];
        const T sa = -Z.y * T(0.5) * wa, sb = Z.x * T(0.5) * wb;
        y[ix(k + 1)] = mk(sa, sb);
        y[ix(2 * (N + 1) - 1 - k)] = mk(-sa, -sb);
        if (k == 0) {
          y[ix(0)] = mk(T(0), T(0));
          y[ix(N + 1)] = mk(T(0), T(0));
        }
      }
    }
  } else {
    const int half = N / 2 + 1;
    for (int k = threadIdx.x; k < half; k += blockDim.x) {
      const int m = k == 0 ? 0 : N - k;
      const cplx<T> qk = B.qy[k], qm = B.qy[m];
      const T eyk = B.eigy[k], eym = B.eigy[m];
      for (int q = 0; q < nl; ++q) {
        const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
        cplx<T>* y = z + q * L;
        const SwIx ix;
        const cplx<T> Zk = y[ix(k)], Zm = y[ix(m)];
        T yak = cmul(qk, Zk + conjg(Zm)).x, ybk = cmul(qk, Zk - conjg(Zm)).y;
        T yam = cmul(qm, Zm + conjg(Zk)).x, ybm = cmul(qm, Zm - conjg(Zk)).y;
        const T exa = B.eigx[ca], exb = B.eigx[cb];
        yak *= spectral_weight<T>(mode, mass, visc, thr, eyk, exa);
        ybk *= spectral_weight<T>(mode, mass, visc, thr, eyk, exb);
        yam *= spectral_weight<T>(mode, mass, visc, thr, eym, exa);
        ybm *= spectral_weight<T>(mode, mass, visc, thr, eym, exb);
        if (k == 0) {
          y[ix(0)] = pre_inverse(yak, T(0), ybk, T(0), qk);
        } else {
          y[ix(k)] = pre_inverse(yak, yam, ybk, ybm, qk);
          if (m != k) y[ix(m)] = pre_inverse(yam, yak, ybm, ybk, qm);
        }
      }
    }
  }
  __syncthreads();
  if (kind == KIND_DST1) fft_p2<T, L, 1, -1, GT>(z + line * L, t, tw);
  else fft_p2<T, L, 1, 1, GT>(z + line * L, t, tw);
  if (vec && ncols == W) {
    for (int e = threadIdx.x; e < totv; e += blockDim.x) {
      const int n = B.fvpr.div(e), jv = e - n * vpr;
      vec_t v;
      T* comp = reinterpret_cast<T*>(&v);
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const int j = jv * V + k;
        comp[k] = value_inverse(z + (j >> 1) * L, kind, N, n, j & 1, B.sy, SwIx{});
      }
      *reinterpret_cast<vec_t*>(H + n * pitch + col0 + jv * V) = v;
    }
  } else {
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
      const int n = B.fw.div(e), j = e - n * W;
      if (j < ncols) H[n * pitch + col0 + j] = value_inverse(z + (j >> 1) * L, kind, N, n, j & 1, B.sy, SwIx{});
    }
  }
}

// ---------------------------------------------------------------- dispatch ---
inline bool is_p2_length(int L) { return L >= 64 && L <= 4096 && (L & (L - 1)) == 0; }

#define MACSAV_P2_SWITCH(L, CALL) \
  switch (L) {                    \
    case 64: CALL(64); break;     \
    case 128: CALL(128); break;   \
    case 256: CALL(256); break;   \
    case 512: CALL(512); break;   \
    case 1024: CALL(1024); break; \
    case 2048: CALL(2048); break; \
    case 4096: CALL(4096); break; \
    default: break;               \
  }

// The split launches (p2_split), FP32 only: CALL(L, threads per line).
#define MACSAV_SPLIT_SWITCH(L, CALL)                 \
  if constexpr (sizeof(T) == 4) {                    \
    switch (L) {                                     \
      case 1024: CALL(1024, 64); break;              \
      case 2048: CALL(2048, 128); break;             \
      case 4096: CALL(4096, 256); break;             \
      default: break;                                \
    }                                                \
  }

}  // namespace macsav
