// Warp-line column pass (FP32, columns of 512 or 1024 FFT points).
//
// The column pass of the velocity and Poisson inverses (forward y-transform,
// spectral weight, inverse y-transform of every column of the spectral
// buffer H; solver/mac/tensor_stokes.py:104-111,200-243) with one complex
// line (two real columns, a + i b) per warp:
//
//   * a CTA of kWLines warps stages a strip of 2 kWLines columns of H in
//     shared memory with coalesced 16-byte loads, one line region of L
//     complex values per warp, and writes the strip back the same way: the
//     only CTA-wide barriers of the pass;
//   * each warp transforms its line in registers.  L = 32 R; lane l holds
//     points l + 32 r (r < R).  An R-point DFT per lane, the twiddles
//     exp(-2 pi i l k2 / L), one transpose through the line's own shared
//     region and a 32-point DFT (split radix-2 for R = 16) leave lane l
//     holding frequencies l + 32 r, which is again the input distribution,
//     so the inverse transform starts from the registers the weights were
//     applied in.  Pairing frequency k with L - k goes through the line's
//     region (one store and one load per point); nothing waits on another
//     warp;
//   * DCT-II / DST-II lines of N = L points use the Makhoul order and the
//     post- and pre-processing of the shared-memory passes (transforms.cuh);
//   * DST-I lines of N = L - 1 points use an FFT of length L = N + 1 in place
//     of the odd extension of length 2 (N + 1): with x_0 = x_L = 0,
//     y_j = sin(pi j / L) (x_j + x_{L-j}) + (x_j - x_{L-j}) / 2 has the DFT Y
//     with -Im Y_k = F_{2k} and Re Y_k = F_{2k+1} - F_{2k-1} (F_{-1} = -F_1),
//     F_k = sum_j x_j sin(pi j k / L) the DST-I, so the odd coefficients are
//     a prefix sum of Re Y (a warp scan per register plus a running carry).
//     Both real lines of a warp share one FFT and are separated with the
//     partner L - k.  The DST-I is its own inverse up to 2 / L.
//
// Compared with the shared-memory radix-8 passes (fftp.cuh: two CTA barriers
// per Stockham pass, about 165 instructions per real element at 1024^2) this
// issues a third of the instructions and no CTA barrier inside the
// transforms.
#pragma once
#include "fftp.cuh"

namespace macsav {

constexpr int kWLines = 8;  // warps (complex lines) per CTA
constexpr int kWThreads = 32 * kWLines;

// Shared bytes of a warp-line CTA with lines of L points (a two-point pad per
// line keeps the strip's stores and loads at two wavefronts per warp).
inline size_t wline_smem(int L) { return size_t(kWLines) * size_t(L + 2) * sizeof(float2); }

// cos(2 pi m / 32)
__host__ __device__ constexpr float cos32q(int m) {  // m in [0, 8]
  return m == 0 ? 1.0f
       : m == 1 ? 0.980785280403230449f
       : m == 2 ? 0.923879532511286756f
       : m == 3 ? 0.831469612302545237f
       : m == 4 ? 0.707106781186547524f
       : m == 5 ? 0.555570233019602225f
       : m == 6 ? 0.382683432365089772f
       : m == 7 ? 0.195090322016128268f
                : 0.0f;
}
__host__ __device__ constexpr float cos32(int m) {
  return (m & 31) <= 8 ? cos32q(m & 31)
       : (m & 31) <= 16 ? -cos32q(16 - (m & 31))
       : (m & 31) <= 24 ? -cos32q((m & 31) - 16)
                        : cos32q(32 - (m & 31));
}

// a * exp(SIGN 2 pi i m / 32)
template <int SIGN>
__device__ __forceinline__ cplx<float> tw32(cplx<float> a, int m) {
  m &= 31;
  if (m == 0) return a;
  if (m == 8) return mul_i(a, SIGN);
  if (m == 16) return mk(-a.x, -a.y);
  if (m == 24) return mul_i(a, -SIGN);
  return cmul(a, mk(cos32(m), float(SIGN) * cos32(m - 8)));
}

// In-register DFT of R = 2, 4, 8, 16 or 32 points, natural order in and out
// (R = 4 Q: Q-point DFTs of the four residues, twiddles, 4-point DFTs).
template <int R, int SIGN>
__device__ __forceinline__ void dft_reg(cplx<float> (&v)[R]) {
  if constexpr (R <= 8) {
    dftR<float, R, SIGN>(v);
  } else {
    constexpr int P = 4, Q = R / 4;
    cplx<float> a[P][Q];
#pragma unroll
    for (int p = 0; p < P; ++p) {
#pragma unroll
      for (int q = 0; q < Q; ++q) a[p][q] = v[P * q + p];
      dft_reg<Q, SIGN>(a[p]);
#pragma unroll
      for (int k1 = 1; k1 < Q; ++k1) a[p][k1] = tw32<SIGN>(a[p][k1], p * k1 * (32 / R));
    }
#pragma unroll
    for (int k1 = 0; k1 < Q; ++k1) {
      cplx<float> b[P];
#pragma unroll
      for (int p = 0; p < P; ++p) b[p] = a[p][k1];
      dft_reg<P, SIGN>(b);
#pragma unroll
      for (int k2 = 0; k2 < P; ++k2) v[k1 + Q * k2] = b[k2];
    }
  }
}

__device__ __forceinline__ cplx<float> ld_c(const float2* p) {
  const float2 a = *p;
  return mk(a.x, a.y);
}
__device__ __forceinline__ void st_c(float2* p, cplx<float> a) { *p = make_float2(a.x, a.y); }

// Unnormalised DFT of L = 32 R points of one line held by a warp: v[r] is
// point lane + 32 r on entry and frequency lane + 32 r on exit.  s is the
// line's shared region (L values; the caller has finished reading it),
// twc[32 k2 + lane] = exp(-2 pi i lane k2 / L).
template <int R, int SIGN>
__device__ __forceinline__ void warp_fft(cplx<float> (&v)[R], float2* s, const float2* __restrict__ twc, int lane) {
  static_assert(R == 16 || R == 32, "warp-line FFT of 512 or 1024 points");
  // Y[n1 = lane][k2] = sum_n2 x[lane + 32 n2] W_R^{n2 k2}, times W_L^{lane k2}
  dft_reg<R, SIGN>(v);
#pragma unroll
  for (int k2 = 1; k2 < R; ++k2) {
    const float2 t = __ldg(twc + 32 * k2 + lane);
    v[k2] = cmul(v[k2], mk(t.x, SIGN < 0 ? t.y : -t.y));
  }
  // transpose: row n1 at n1 R, column k2 stored at k2 ^ (n1 mod R), so both
  // the row stores and the column loads are conflict-free
  __syncwarp();
#pragma unroll
  for (int k2 = 0; k2 < R; ++k2) st_c(s + lane * R + (k2 ^ (lane & (R - 1))), v[k2]);
  __syncwarp();
  // X[k2 + R k1] = sum_n1 Y[n1][k2] W_32^{n1 k1}
  if constexpr (R == 32) {
#pragma unroll
    for (int n1 = 0; n1 < 32; ++n1) v[n1] = ld_c(s + n1 * 32 + (lane ^ n1));
  } else {
    // lane = k2 + 16 h computes k1 = 2 k1' + h: a 16-point DFT of
    // (Y[n1] + (-1)^h Y[n1 + 16]) W_32^{h n1}
    const int k2 = lane & 15;
    const bool h = lane >= 16;
#pragma unroll
    for (int n1 = 0; n1 < 16; ++n1) {
      const cplx<float> a = ld_c(s + n1 * 16 + (k2 ^ n1)), b = ld_c(s + (n1 + 16) * 16 + (k2 ^ n1));
      v[n1] = h ? tw32<SIGN>(a - b, n1) : a + b;
    }
  }
  dft_reg<R, SIGN>(v);
}

// Two real DST-I lines from the DFT of their packed y (a + i b): writes
// F_{2k} to e[r] and F_{2k+1} to o[r] for k = lane + 32 r, r < R / 2.
template <int R>
__device__ __forceinline__ void dst1_post(const cplx<float> (&v)[R], float2* s, int lane, cplx<float> (&e)[R / 2],
                                          cplx<float> (&o)[R / 2]) {
  constexpr int L = 32 * R;
  __syncwarp();
#pragma unroll
  for (int r = 0; r < R; ++r) st_c(s + lane + 32 * r, v[r]);
  __syncwarp();
  float carry_a = 0.f, carry_b = 0.f, c0a = 0.f, c0b = 0.f;
#pragma unroll
  for (int r = 0; r < R / 2; ++r) {
    const int k = lane + 32 * r;
    const cplx<float> yk = v[r], ym = ld_c(s + ((L - k) & (L - 1)));
    // Y^a_k = (Y_k + conj Y_{L-k}) / 2, Y^b_k = (Y_k - conj Y_{L-k}) / (2 i)
    float ca = 0.5f * (yk.x + ym.x), cb = 0.5f * (yk.y + ym.y);
    e[r] = mk(-0.5f * (yk.y - ym.y), 0.5f * (yk.x - ym.x));
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const float ta = __shfl_up_sync(0xffffffffu, ca, off), tb = __shfl_up_sync(0xffffffffu, cb, off);
      if (lane >= off) {
        ca += ta;
        cb += tb;
      }
    }
    ca += carry_a;
    cb += carry_b;
    if (r == 0) {
      c0a = __shfl_sync(0xffffffffu, ca, 0);
      c0b = __shfl_sync(0xffffffffu, cb, 0);
    }
    carry_a = __shfl_sync(0xffffffffu, ca, 31);
    carry_b = __shfl_sync(0xffffffffu, cb, 31);
    o[r] = mk(ca - 0.5f * c0a, cb - 0.5f * c0b);
  }
}

// y_j = sin(pi j / L) (x_j + x_{L-j}) + (x_j - x_{L-j}) / 2 for j = lane + 32 r,
// from the line's region in natural order (s[0] = 0 stands for x_0 and x_L).
template <int R>
__device__ __forceinline__ void dst1_pre(cplx<float> (&v)[R], const float2* s, const float2* __restrict__ twy,
                                         int lane) {
  constexpr int L = 32 * R;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int j = lane + 32 * r;
    const cplx<float> xj = ld_c(s + j), xm = ld_c(s + ((L - j) & (L - 1)));
    const float sj = -__ldg(twy + j).y;  // twy[j] = exp(-i pi j / L)
    v[r] = mk(sj * (xj.x + xm.x) + 0.5f * (xj.x - xm.x), sj * (xj.y + xm.y) + 0.5f * (xj.y - xm.y));
  }
}

// One CTA: columns col0 .. col0 + 2 kWLines - 1 of right-hand side blockIdx.y.
// ODD: DST-I columns (N = L - 1), else DCT-II / DST-II (N = L).
template <int R, bool ODD>
__global__ void __launch_bounds__(kWThreads, 2) k_column_w(TBlockDev<float> B, const int* active, int mode,
                                                           const double* shift, float thr) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  constexpr int L = 32 * R;
  constexpr int LS = L + 2;
  constexpr int PER = (4 * L + kWThreads - 1) / kWThreads;  // 16-byte vectors per thread
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* S = reinterpret_cast<float2*>(smraw);
  const int N = B.rows;
  const int col0 = blockIdx.x * 2 * kWLines;
  float* H = B.H + c * B.hstride;
  const long long pitch = B.pitch;
  const int t = threadIdx.x;
  const bool dst2 = !ODD && B.ky == KIND_DST2;
  // ---- strip -> line regions (row n of column col0 + 4q + i: line 2q + i/2, part i%2)
  {
    float4 x[PER];
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = t + u * kWThreads, n = e >> 2, q = e & 3;
      x[u] = n < N ? *reinterpret_cast<const float4*>(H + n * pitch + col0 + 4 * q) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = t + u * kWThreads, n = e >> 2, q = e & 3;
      if (n < N) {
        const int cb = col0 + 4 * q;
        float4 a = x[u];
        if (cb >= B.cols) a.x = 0.f;  // padding columns of H read as zero
        if (cb + 1 >= B.cols) a.y = 0.f;
        if (cb + 2 >= B.cols) a.z = 0.f;
        if (cb + 3 >= B.cols) a.w = 0.f;
        const int pos = ODD ? n + 1 : makhoul_pos(n, N);
        const float sg = (dst2 && (n & 1)) ? -1.f : 1.f;
        S[(2 * q) * LS + pos] = make_float2(sg * a.x, sg * a.y);
        S[(2 * q + 1) * LS + pos] = make_float2(sg * a.z, sg * a.w);
      }
    }
    if (ODD && t < kWLines) S[t * LS] = make_float2(0.f, 0.f);
  }
  __syncthreads();
  const int lane = t & 31, l = t >> 5;
  const int ca = col0 + 2 * l;
  if (ca < B.cols) {
    float2* s = S + l * LS;
    const float2* twc = reinterpret_cast<const float2*>(B.twcy);
    const float mass = float(shift[2 * c]), visc = float(shift[2 * c + 1]);
    const float exa = B.eigx[ca], exb = B.eigx[min(ca + 1, B.cols - 1)];
    cplx<float> v[R];
    if constexpr (!ODD) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = ld_c(s + lane + 32 * r);
      warp_fft<R, -1>(v, s, twc, lane);
      // coefficients of k and N - k, weights, inverse pre-processing
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R; ++r) st_c(s + lane + 32 * r, v[r]);
      __syncwarp();
      const float2* qy = reinterpret_cast<const float2*>(B.qy);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = lane + 32 * r, m = (L - k) & (L - 1);
        const cplx<float> vk = v[r], vm = ld_c(s + m);
        const float2 q2 = __ldg(qy + k);
        const cplx<float> qk = mk(q2.x, q2.y), qm = mk(-q2.y, -q2.x);  // q_{N-k} = -i conj(q_k)
        float yak = cmul(qk, vk + conjg(vm)).x, ybk = cmul(qk, vk - conjg(vm)).y;
        float yam = cmul(qm, vm + conjg(vk)).x, ybm = cmul(qm, vm - conjg(vk)).y;
        const float eyk = __ldg(B.eigy + k), eym = __ldg(B.eigy + m);
        yak *= spectral_weight<float>(mode, mass, visc, thr, eyk, exa);
        ybk *= spectral_weight<float>(mode, mass, visc, thr, eyk, exb);
        yam *= spectral_weight<float>(mode, mass, visc, thr, eym, exa);
        ybm *= spectral_weight<float>(mode, mass, visc, thr, eym, exb);
        v[r] = k == 0 ? pre_inverse(yak, 0.f, ybk, 0.f, qk) : pre_inverse(yak, yam, ybk, ybm, qk);
      }
      warp_fft<R, 1>(v, s, twc, lane);
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R; ++r) st_c(s + lane + 32 * r, v[r]);  // Makhoul order, as staged
    } else {
      const float2* twy = reinterpret_cast<const float2*>(B.twy);
      cplx<float> fe[R / 2], fo[R / 2];
      dst1_pre<R>(v, s, twy, lane);
      warp_fft<R, -1>(v, s, twc, lane);
      dst1_post<R>(v, s, lane, fe, fo);
      // weights: F_{2k} is coefficient 2k - 1, F_{2k+1} coefficient 2k
#pragma unroll
      for (int r = 0; r < R / 2; ++r) {
        const int k = lane + 32 * r;
        const float eyo = __ldg(B.eigy + 2 * k);
        const float eye = k ? __ldg(B.eigy + 2 * k - 1) : 0.f;
        fe[r] = k ? mk(fe[r].x * spectral_weight<float>(mode, mass, visc, thr, eye, exa),
                       fe[r].y * spectral_weight<float>(mode, mass, visc, thr, eye, exb))
                  : mk(0.f, 0.f);
        fo[r] = mk(fo[r].x * spectral_weight<float>(mode, mass, visc, thr, eyo, exa),
                   fo[r].y * spectral_weight<float>(mode, mass, visc, thr, eyo, exb));
      }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R / 2; ++r) {
        const int k = lane + 32 * r;
        *reinterpret_cast<float4*>(s + 2 * k) = make_float4(fe[r].x, fe[r].y, fo[r].x, fo[r].y);
      }
      __syncwarp();
      dst1_pre<R>(v, s, twy, lane);
      warp_fft<R, -1>(v, s, twc, lane);
      dst1_post<R>(v, s, lane, fe, fo);
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R / 2; ++r) {
        const int k = lane + 32 * r;
        *reinterpret_cast<float4*>(s + 2 * k) = make_float4(fe[r].x, fe[r].y, fo[r].x, fo[r].y);
      }
    }
  }
  __syncthreads();
  // ---- line regions -> strip (normalisation 1/N, or 2/L for DST-I)
  {
    const float sc = ODD ? 2.f * B.sy : B.sy;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int e = t + u * kWThreads, n = e >> 2, q = e & 3;
      if (n < N) {
        const int pos = ODD ? n + 1 : makhoul_pos(n, N);
        const float sg = (dst2 && (n & 1)) ? -sc : sc;
        const float2 a = S[(2 * q) * LS + pos], b = S[(2 * q + 1) * LS + pos];
        const int cb = col0 + 4 * q;
        float4 y = make_float4(sg * a.x, sg * a.y, sg * b.x, sg * b.y);
        if (cb >= B.cols) y.x = 0.f;  // the padding stays zero
        if (cb + 1 >= B.cols) y.y = 0.f;
        if (cb + 2 >= B.cols) y.z = 0.f;
        if (cb + 3 >= B.cols) y.w = 0.f;
        *reinterpret_cast<float4*>(H + n * pitch + cb) = y;
      }
    }
  }
}

// ============================================================ row passes ===
// One pair of rows (a = 2q, b = 2q + 1, packed a + i b) per warp and no CTA
// barrier: the sources are read and the sinks written with lanes along the
// row (coalesced), the reordering (Makhoul order, the DST-I index shift) and
// the pairing of k with L - k go through the warp's own line region.
constexpr int kWRowLines = 4;  // warps (row pairs) per CTA

inline size_t wrow_smem(int L) { return size_t(kWRowLines) * size_t(L + 2) * sizeof(float2); }

template <int R, bool ODD, class Src>
__global__ void __launch_bounds__(32 * kWRowLines) k_row_forward_w(TBlockDev<float> B, const int* active, Src src,
                                                                   int bk) {
  pdl_wait();
  const int c = blockIdx.y;
  if (active && !active[c]) return;
  constexpr int L = 32 * R;
  constexpr int LS = L + 2;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ra = 2 * (blockIdx.x * kWRowLines + w), rows = B.rows, N = B.cols;
  if (ra >= rows) return;  // the whole warp: no CTA barrier follows
  const bool hb = ra + 1 < rows;
  float2* s = reinterpret_cast<float2*>(smraw) + w * LS;
  const float2* twc = reinterpret_cast<const float2*>(B.twcx);
  float* Ha = B.H + c * B.hstride + (long long)ra * B.pitch;
  cplx<float> v[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int n = lane + 32 * r;
    float a = 0.f, b = 0.f;
    if (n < N) {
      a = src(bk, c, ra, n);
      if (hb) b = src(bk, c, ra + 1, n);
    }
    v[r] = mk(a, b);
  }
  if constexpr (!ODD) {
    const bool dst2 = B.kx == KIND_DST2;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int n = lane + 32 * r;
      st_c(s + makhoul_pos(n, N), (dst2 && (n & 1)) ? mk(-v[r].x, -v[r].y) : v[r]);
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = ld_c(s + lane + 32 * r);
    warp_fft<R, -1>(v, s, twc, lane);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R; ++r) st_c(s + lane + 32 * r, v[r]);
    __syncwarp();
    const float2* qx = reinterpret_cast<const float2*>(B.qx);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = lane + 32 * r;
      const cplx<float> vk = v[r], vm = ld_c(s + ((L - k) & (L - 1)));
      const float2 q2 = __ldg(qx + k);
      const cplx<float> qk = mk(q2.x, q2.y);
      Ha[k] = cmul(qk, vk + conjg(vm)).x;
      if (hb) Ha[B.pitch + k] = cmul(qk, vk - conjg(vm)).y;
    }
  } else {
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int n = lane + 32 * r;
      if (n < N) st_c(s + n + 1, v[r]);
    }
    if (lane == 0) s[0] = make_float2(0.f, 0.f);
    __syncwarp();
    cplx<float> fe[R / 2], fo[R / 2];
    dst1_pre<R>(v, s, reinterpret_cast<const float2*>(B.twx), lane);
    warp_fft<R, -1>(v, s, twc, lane);
    dst1_post<R>(v, s, lane, fe, fo);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < R / 2; ++r) {
      const int k = lane + 32 * r;
      *reinterpret_cast<float4*>(s + 2 * k) = make_float4(fe[r].x, fe[r].y, fo[r].x, fo[r].y);
    }
    __syncwarp();
    // coefficient j is F_{j + 1}
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int j = lane + 32 * r;
      if (j < N) {
        const float2 F = s[j + 1];
        Ha[j] = F.x;
        if (hb) Ha[B.pitch + j] = F.y;
      }
    }
  }
}

template <int R, bool ODD, class Dst, class Fin>
__global__ void __launch_bounds__(32 * kWRowLines) k_row_inverse_w(TBlockDev<float> B, const int* active, Dst dst,
                                                                   int bk, double* partial, Fin fin,
                                                                   unsigned int* counter) {
  pdl_wait();
  const int c = blockIdx.y;
  const bool live = !active || active[c];
  Acc<float> acc[2];
  constexpr int L = 32 * R;
  constexpr int LS = L + 2;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int ra = 2 * (blockIdx.x * kWRowLines + w), rows = B.rows, N = B.cols;
  if (live && ra < rows) {
    const bool hb = ra + 1 < rows;
    float2* s = reinterpret_cast<float2*>(smraw) + w * LS;
    const float2* twc = reinterpret_cast<const float2*>(B.twcx);
    const float* Ha = B.H + c * B.hstride + (long long)ra * B.pitch;
    const float* Hb = Ha + B.pitch;
    cplx<float> v[R];
    float sc = B.sx;
    if constexpr (!ODD) {
      const float2* qx = reinterpret_cast<const float2*>(B.qx);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = lane + 32 * r, m = (L - k) & (L - 1);
        const float yak = Ha[k], yam = k ? Ha[m] : 0.f;
        const float ybk = hb ? Hb[k] : 0.f, ybm = (hb && k) ? Hb[m] : 0.f;
        const float2 q2 = __ldg(qx + k);
        v[r] = pre_inverse(yak, yam, ybk, ybm, mk(q2.x, q2.y));
      }
      warp_fft<R, 1>(v, s, twc, lane);
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R; ++r) st_c(s + lane + 32 * r, v[r]);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int j = lane + 32 * r;
        if (j < N) s[j + 1] = make_float2(Ha[j], hb ? Hb[j] : 0.f);
      }
      if (lane == 0) s[0] = make_float2(0.f, 0.f);
      __syncwarp();
      cplx<float> fe[R / 2], fo[R / 2];
      dst1_pre<R>(v, s, reinterpret_cast<const float2*>(B.twx), lane);
      warp_fft<R, -1>(v, s, twc, lane);
      dst1_post<R>(v, s, lane, fe, fo);
      __syncwarp();
#pragma unroll
      for (int r = 0; r < R / 2; ++r) {
        const int k = lane + 32 * r;
        *reinterpret_cast<float4*>(s + 2 * k) = make_float4(fe[r].x, fe[r].y, fo[r].x, fo[r].y);
      }
      sc = 2.f * B.sx;
    }
    __syncwarp();
    const bool dst2 = !ODD && B.kx == KIND_DST2;
    typename Dst::aux_t xa[R], xb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int n = lane + 32 * r;
      if (n < N) {
        xa[r] = dst.load(bk, c, ra, n);
        if (hb) xb[r] = dst.load(bk, c, ra + 1, n);
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int n = lane + 32 * r;
      if (n < N) {
        const float2 z = s[ODD ? n + 1 : makhoul_pos(n, N)];
        const float sg = (dst2 && (n & 1)) ? -sc : sc;
        dst.store(bk, c, ra, n, z.x * sg, xa[r], acc);
        if (hb) dst.store(bk, c, ra + 1, n, z.y * sg, xb[r], acc);
      }
    }
  }
  if (partial) {
    write_sums<float, 2>(acc, partial, 2);
    last_block_finish(fin, counter);
  }
}

}  // namespace macsav
