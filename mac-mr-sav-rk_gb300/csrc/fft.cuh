// Shared-memory complex FFTs for batches of lines, used by the trig transforms.
//
// A CTA holds `nl` complex lines of length L (stride LS) in shared memory and
// transforms all of them together.  Lengths whose factors are all in {2,3,4}
// use an in-place mixed-radix Stockham autosort FFT: every stage reads all its
// butterfly inputs into registers, synchronises, then writes the outputs (one
// buffer, no ping-pong).  Other lengths (the small odd grids of the unit
// tests) use a direct O(L^2) DFT through a second shared buffer.
//
// Twiddles come from a table tw[m] = exp(-2 pi i m / L) computed on the host in
// double precision and rounded to T; the inverse direction conjugates them.
#pragma once
#include "common.cuh"

namespace macsav {

constexpr int kMaxStages = 14;

// Radix plan of one FFT length (host fills, passed by value to kernels),
// with the stage divisors pre-inverted (FastDiv) so no butterfly divides.
struct FFTPlan {
  int L;
  int nstages;       // 0 => direct DFT
  int radix[kMaxStages];
  FastDiv ns[kMaxStages];   // Ns, the product of the earlier radices
  FastDiv nbf[kMaxStages];  // L / radix
};

template <typename T>
__device__ __forceinline__ cplx<T> twiddle(const cplx<T>* __restrict__ tw, int m, int sign) {
  cplx<T> w = tw[m];
  return sign < 0 ? w : conjg(w);
}

template <typename T, int R>
__device__ __forceinline__ void dft_small(cplx<T> (&v)[R], int sign) {
  if constexpr (R == 2) {
    cplx<T> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else if constexpr (R == 3) {
    // exp(sign*2*pi*i/3) = -1/2 + sign*i*sqrt(3)/2
    const T h = T(0.5), s3 = T(0.86602540378443864676);
    cplx<T> a = v[0], b = v[1], c = v[2];
    cplx<T> sum = b + c, dif = b - c;
    v[0] = a + sum;
    cplx<T> m = mk(a.x - h * sum.x, a.y - h * sum.y);
    cplx<T> r = mul_i(cscale(dif, s3), sign);  // sign*i*s3*(b-c)
    v[1] = m + r;
    v[2] = m - r;
  } else if constexpr (R == 4) {
    cplx<T> a = v[0], b = v[1], c = v[2], d = v[3];
    cplx<T> s0 = a + c, d0 = a - c, s1 = b + d, d1 = mul_i(b - d, sign);
    v[0] = s0 + s1;
    v[2] = s0 - s1;
    v[1] = d0 + d1;
    v[3] = d0 - d1;
  }
}

// One Stockham stage of radix R over all lines, in place.  MAXB bounds the
// butterflies a thread owns (host guarantees nl*L/R <= MAXB*blockDim.x).
template <typename T, int R, int MAXB>
__device__ __forceinline__ void stockham_stage(cplx<T>* buf, int L, int LS, int nl, int Ns, const FastDiv& fns,
                                               const FastDiv& fnbf, const cplx<T>* __restrict__ tw, int sign) {
  const int nbf = L / R;
  const int total = nl * nbf;
  const int step = L / (Ns * R);
  cplx<T> v[MAXB][R];
  int dst[MAXB];
#pragma unroll
  for (int q = 0; q < MAXB; ++q) {
    const int b = threadIdx.x + q * blockDim.x;
    dst[q] = -1;
    if (b < total) {
      const int line = fnbf.div(b);
      const int j = b - line * nbf;
      const cplx<T>* in = buf + line * LS;
      const int jq = fns.div(j);
      const int k = j - jq * Ns;
      v[q][0] = in[j];
#pragma unroll
      for (int r = 1; r < R; ++r) v[q][r] = cmul(in[j + r * nbf], twiddle(tw, r * k * step, sign));
      dft_small<T, R>(v[q], sign);
      dst[q] = line * LS + jq * Ns * R + k;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < MAXB; ++q) {
    if (dst[q] >= 0) {
#pragma unroll
      for (int r = 0; r < R; ++r) buf[dst[q] + r * Ns] = v[q][r];
    }
  }
  __syncthreads();
}

// Direct DFT (small, awkward lengths): buf -> tmp -> buf.
template <typename T>
__device__ void direct_dft(cplx<T>* buf, cplx<T>* tmp, int L, int LS, int nl,
                           const cplx<T>* __restrict__ tw, int sign) {
  const int total = nl * L;
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / L, k = b - line * L;
    const cplx<T>* in = buf + line * LS;
    cplx<T> acc = mk(T(0), T(0));
    int m = 0;
    for (int n = 0; n < L; ++n) {
      acc = acc + cmul(in[n], twiddle(tw, m, sign));
      m += k;
      if (m >= L) m -= L;
    }
    tmp[line * LS + k] = acc;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / L, k = b - line * L;
    buf[line * LS + k] = tmp[line * LS + k];
  }
  __syncthreads();
}

// Complex FFT (sign -1) or unscaled inverse (sign +1) of nl lines in place.
// Requires a __syncthreads() between the writes that filled buf and this call.
template <typename T, int VMAX>
__device__ void fft_lines(cplx<T>* buf, cplx<T>* tmp, const FFTPlan& plan, int LS, int nl,
                          const cplx<T>* __restrict__ tw, int sign) {
  const int L = plan.L;
  if (plan.nstages == 0) {
    direct_dft(buf, tmp, L, LS, nl, tw, sign);
    return;
  }
  int Ns = 1;
  for (int s = 0; s < plan.nstages; ++s) {
    const int R = plan.radix[s];
    if (R == 4) stockham_stage<T, 4, (VMAX + 3) / 4>(buf, L, LS, nl, Ns, plan.ns[s], plan.nbf[s], tw, sign);
    else if (R == 2) stockham_stage<T, 2, (VMAX + 1) / 2>(buf, L, LS, nl, Ns, plan.ns[s], plan.nbf[s], tw, sign);
    else stockham_stage<T, 3, (VMAX + 2) / 3>(buf, L, LS, nl, Ns, plan.ns[s], plan.nbf[s], tw, sign);
    Ns *= R;
  }
}

}  // namespace macsav
