// Power-of-two transform passes with compile-time FFT length.
//
// For L = 2^k in [64, 4096] every pass kernel is specialised on L: each line
// is transformed by G = L/8 threads, each owning one radix-8 butterfly per
// Stockham pass (register-resident 8-point DFTs, the last pass radix 2 or 4
// when log2 L is not a multiple of 3), so log8(L) passes with all index
// arithmetic folded to shifts and masks.  A CTA holds NL = blockDim.x / G
// lines.  Packing, spectral weights and the post/pre-processing are the same
// as in the generic kernels (transforms.cuh).
#pragma once
#include "transforms.cuh"

namespace macsav {

constexpr int kE = 8;  // elements per thread per line

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

// Stockham passes on one line z (stride 1) by the G = L/8 threads of the
// line; thread t owns butterflies j = t + q G.  Every thread of the CTA must
// call this (it synchronises the block twice per pass).
template <typename T, int L, int NS, int SIGN>
__device__ __forceinline__ void fft_p2(cplx<T>* z, int t, const cplx<T>* __restrict__ tw) {
  constexpr int R = (L / NS >= kE) ? kE : L / NS;
  constexpr int G = L / kE;
  constexpr int NB = kE / R;
  constexpr int STRIDE = L / R;
  constexpr int TWS = L / (NS * R);
  cplx<T> v[NB][R];
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = t + q * G;
    const int k = j & (NS - 1);
#pragma unroll
    for (int r = 0; r < R; ++r) v[q][r] = z[j + r * STRIDE];
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[q][r] = cmul(v[q][r], tw_at<T, SIGN>(tw, r * k * TWS));
    }
    dftR<T, R, SIGN>(v[q]);
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    const int j = t + q * G;
    const int k = j & (NS - 1);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) z[base + r * NS] = v[q][r];
  }
  __syncthreads();
  if constexpr (NS * R < L) fft_p2<T, L, NS * R, SIGN>(z, t, tw);
}

// ------------------------------------------------------------ row passes ---
// One block (u, v or p) per launch; NL = blockDim.x / (L/8) line pairs per CTA.
template <typename T, int L, class Src>
__global__ void __launch_bounds__(kFFTThreads) k_row_forward_p2(TBlockDev<T> B, const int* active, Src src, int bk) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  constexpr int G = L / kE;
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  const int NL = blockDim.x / G;
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
        put_pair(z + q * L, kind, N, n, va[u], vb[u]);
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * L, N);
  __syncthreads();
  fft_p2<T, L, 1, -1>(z + (threadIdx.x / G) * L, threadIdx.x % G, B.twx);
  T* H = B.H + c * B.hstride;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int q = B.fcols.div(e), k = e - q * N;
    const int ra = row0 + 2 * q;
    T ya, yb;
    coef_forward(z + q * L, kind, N, k, B.qx, ya, yb);
    H[(long long)ra * B.pitch + k] = ya;
    if (ra + 1 < rows) H[(long long)ra * B.pitch + B.pitch + k] = yb;
  }
}

template <typename T, int L, class Dst, class Fin>
__global__ void __launch_bounds__(kFFTThreads) k_row_inverse_p2(TBlockDev<T> B, const int* active, Dst dst, int bk,
                                                                double* partial, Fin fin, unsigned int* counter) {
  pdl_wait();
  const int c = blockIdx.y;
  constexpr int G = L / kE;
  const bool live = !active || active[c];
  Acc<T> acc[2];
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  if (live) {
    const int NL = blockDim.x / G;
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
          if (kind == KIND_DST1) put_pair(z + q * L, KIND_DST1, N, k, yak[u], ybk[u]);
          else z[q * L + k] = pre_inverse(yak[u], yam[u], ybk[u], ybm[u], B.qx[k]);
        }
      }
    }
    if (kind == KIND_DST1)
      for (int q = threadIdx.x; q < npairs; q += blockDim.x) zero_dst1_ends(z + q * L, N);
    __syncthreads();
    if (kind == KIND_DST1) fft_p2<T, L, 1, -1>(z + (threadIdx.x / G) * L, threadIdx.x % G, B.twx);
    else fft_p2<T, L, 1, 1>(z + (threadIdx.x / G) * L, threadIdx.x % G, B.twx);
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
          dst.store(bk, c, ra, n, value_inverse(z + q * L, kind, N, n, 0, B.sx), xa[u], acc);
          if (ra + 1 < rows) dst.store(bk, c, ra + 1, n, value_inverse(z + q * L, kind, N, n, 1, B.sx), xb[u], acc);
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
// NL = blockDim.x / (L/8) complex lines = W = 2 NL columns per CTA.
template <typename T, int L>
__global__ void __launch_bounds__(kFFTThreads) k_column_p2(TBlockDev<T> B, const int* active, int mode,
                                                          const double* shift, T thr) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  constexpr int G = L / kE;
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* z = reinterpret_cast<cplx<T>*>(smraw);
  using vec_t = typename Vec16<T>::type;
  constexpr int V = Vec16<T>::n;
  const int NL = blockDim.x / G;
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
      if (j < 2 * nl) put_real(z + (j >> 1) * L, kind, N, n, j & 1, j < ncols ? H[n * pitch + col0 + j] : T(0));
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
#pragma unroll
        for (int k = 0; k < V; ++k) {
          const int j = jv * V + k;
          if (j < 2 * nl) put_real(z + (j >> 1) * L, kind, N, n, j & 1, j < ncols ? comp[k] : T(0));
        }
      }
    }
  }
  if (kind == KIND_DST1)
    for (int q = threadIdx.x; q < nl; q += blockDim.x) zero_dst1_ends(z + q * L, N);
  __syncthreads();
  cplx<T>* zl = z + (threadIdx.x / G) * L;
  const int t = threadIdx.x % G;
  fft_p2<T, L, 1, -1>(zl, t, B.twy);
  if (kind == KIND_DST1) {
    for (int e = threadIdx.x; e < nl * N; e += blockDim.x) {
      const int q = B.frows.div(e), k = e - q * N;
      cplx<T>* y = z + q * L;
      const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
      const T ey = B.eigy[k];
      const T wa = spectral_weight<T>(mode, mass, visc, thr, ey, B.eigx[ca]);
      const T wb = spectral_weight<T>(mode, mass, visc, thr, ey, B.eigx[cb]);
      const cplx<T> Z = y[k + 1];
      const T sa = -Z.y * T(0.5) * wa, sb = Z.x * T(0.5) * wb;
      y[k + 1] = mk(sa, sb);
      y[2 * (N + 1) - 1 - k] = mk(-sa, -sb);
      if (k == 0) {
        y[0] = mk(T(0), T(0));
        y[N + 1] = mk(T(0), T(0));
      }
    }
  } else {
    const int half = N / 2 + 1;
    for (int e = threadIdx.x; e < nl * half; e += blockDim.x) {
      const int q = B.fhalf.div(e), k = e - q * half;
      cplx<T>* y = z + q * L;
      const int m = k == 0 ? 0 : N - k;
      const int ca = col0 + 2 * q, cb = min(ca + 1, B.cols - 1);
      const cplx<T> Zk = y[k], Zm = y[m];
      const cplx<T> qk = B.qy[k], qm = B.qy[m];
      T yak = cmul(qk, Zk + conjg(Zm)).x, ybk = cmul(qk, Zk - conjg(Zm)).y;
      T yam = cmul(qm, Zm + conjg(Zk)).x, ybm = cmul(qm, Zm - conjg(Zk)).y;
      const T eyk = B.eigy[k], eym = B.eigy[m], exa = B.eigx[ca], exb = B.eigx[cb];
      yak *= spectral_weight<T>(mode, mass, visc, thr, eyk, exa);
      ybk *= spectral_weight<T>(mode, mass, visc, thr, eyk, exb);
      yam *= spectral_weight<T>(mode, mass, visc, thr, eym, exa);
      ybm *= spectral_weight<T>(mode, mass, visc, thr, eym, exb);
      if (k == 0) {
        y[0] = pre_inverse(yak, T(0), ybk, T(0), qk);
      } else {
        y[k] = pre_inverse(yak, yam, ybk, ybm, qk);
        if (m != k) y[m] = pre_inverse(yam, yak, ybm, ybk, qm);
      }
    }
  }
  __syncthreads();
  if (kind == KIND_DST1) fft_p2<T, L, 1, -1>(zl, t, B.twy);
  else fft_p2<T, L, 1, 1>(zl, t, B.twy);
  if (vec && ncols == W) {
    for (int e = threadIdx.x; e < totv; e += blockDim.x) {
      const int n = B.fvpr.div(e), jv = e - n * vpr;
      vec_t v;
      T* comp = reinterpret_cast<T*>(&v);
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const int j = jv * V + k;
        comp[k] = value_inverse(z + (j >> 1) * L, kind, N, n, j & 1, B.sy);
      }
      *reinterpret_cast<vec_t*>(H + n * pitch + col0 + jv * V) = v;
    }
  } else {
    for (int e = threadIdx.x; e < N * W; e += blockDim.x) {
      const int n = B.fw.div(e), j = e - n * W;
      if (j < ncols) H[n * pitch + col0 + j] = value_inverse(z + (j >> 1) * L, kind, N, n, j & 1, B.sy);
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

}  // namespace macsav
