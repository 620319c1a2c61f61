// Channel MAC (periodic x, stationary no-slip walls in y) on the GPU: the
// operators, the skew convection and the FFT Stokes backend of the reference
// (solver/channel/operators.py, kernels.py, fft_stokes.py).
//
// Packed free vector (solver/channel/grid.py:64-77): u faces (j, i), j < ny,
// i < nx (the periodic duplicate u[:, nx] = u[:, 0] is not stored) at j*nx+i,
// then v faces of the interior rows J = 1..ny-1 at n_u + (J-1)*nx + i.
//
// FFT Stokes (fft_stokes.py:34-137): an orthonormal real FFT along x of every
// row (two real rows per complex FFT, shared-memory FFT of fft.cuh), then for
// each x mode m one solve of the banded saddle system in the interleaved
// unknown order [u_j, p_j, v_j] (bandwidth 3):
//   hu u - conj(d) p = fu,  hv v - Dy^T p = fv,  -d u - Dy v = 0,
//   d = (exp(i theta) - 1)/hx (-2/hx at the Nyquist mode), lambda =
//   4 sin^2(theta/2)/hx^2, hu = (m + k lambda) I + k Ly(ny, half-cell wall),
//   hv = (m + k lambda) I + k Ly(ny-1, Dirichlet)
// by banded LU with partial pivoting (the elimination of LAPACK's gbtf2 /
// gbtrs, one thread per mode for the factors, one per (mode, column) for the
// solves); mode 0 is a tridiagonal solve for u with v = 0 and p from the
// cumulative sum of fv (mean removed); then the inverse FFTs and the FP64
// closing checks.  Factors are cached per (mass, viscosity) like the
// reference; all arithmetic is FP64.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fft.cuh"

namespace macsav {

FFTPlan make_fft_plan(int L);

namespace {

using cd = cplx<double>;
constexpr int kKL = 3, kKU = 3, kLD = 2 * kKL + kKU + 1;  // band storage rows
constexpr int kChThreads = 256;
constexpr int kChFactorThreads = 8;  // threads per CTA of the per-mode band factorisations

struct ChanGrid {
  int nx, ny, nu, nv, size, np, nm;  // nm = nx/2 + 1 x modes
  double hx, hy, ihx, ihy, ihx2, ihy2;
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
// u at (j, i) with periodic i; v at physical face row J (0 and ny are walls)
__device__ __forceinline__ double cu_(const double* x, const ChanGrid& g, int j, int i) {
  return x[j * g.nx + wrap(i, g.nx)];
}
__device__ __forceinline__ double cv_(const double* x, const ChanGrid& g, int J, int i) {
  return (J <= 0 || J >= g.ny) ? 0.0 : x[g.nu + (J - 1) * g.nx + wrap(i, g.nx)];
}

// (K x)_e (operators.py:11-18): periodic second difference in x; in y the
// half-cell tangential wall rows for u and the Dirichlet rows for v.
__device__ double ch_K(const double* x, const ChanGrid& g, int e) {
  if (e < g.nu) {
    const int j = e / g.nx, i = e - j * g.nx;
    const double c = x[e];
    const double l = cu_(x, g, j, i - 1), r = cu_(x, g, j, i + 1);
    const double s = j > 0 ? x[e - g.nx] : -c, n = j < g.ny - 1 ? x[e + g.nx] : -c;
    return (2.0 * c - l - r) * g.ihx2 + (2.0 * c - s - n) * g.ihy2;
  }
  const int f = e - g.nu, k = f / g.nx, i = f - k * g.nx;
  const double c = x[e];
  const double l = x[g.nu + k * g.nx + wrap(i - 1, g.nx)], r = x[g.nu + k * g.nx + wrap(i + 1, g.nx)];
  const double s = k > 0 ? x[e - g.nx] : 0.0, n = k < g.ny - 2 ? x[e + g.nx] : 0.0;
  return (2.0 * c - l - r) * g.ihx2 + (2.0 * c - s - n) * g.ihy2;
}
// (D x) at cell (j, i) (operators.py:19-23)
__device__ double ch_D(const double* x, const ChanGrid& g, int j, int i) {
  return (cu_(x, g, j, i + 1) - cu_(x, g, j, i)) * g.ihx + (cv_(x, g, j + 1, i) - cv_(x, g, j, i)) * g.ihy;
}
// (G p)_e = -(D^T p)_e (operators.py:25)
__device__ double ch_G(const double* p, const ChanGrid& g, int e) {
  if (e < g.nu) {
    const int j = e / g.nx, i = e - j * g.nx;
    return (p[j * g.nx + i] - p[j * g.nx + wrap(i - 1, g.nx)]) * g.ihx;
  }
  const int f = e - g.nu, k = f / g.nx, i = f - k * g.nx;
  return (p[(k + 1) * g.nx + i] - p[k * g.nx + i]) * g.ihy;
}
// Skew dual-cell convection (kernels.py:9-41)
__device__ double ch_conv(const double* x, const ChanGrid& g, int e) {
  if (e < g.nu) {
    const int j = e / g.nx, i = e - j * g.nx;
    const double uc = x[e], ue = cu_(x, g, j, i + 1), uw = cu_(x, g, j, i - 1);
    const double east = 0.5 * (uc + ue), west = 0.5 * (uc + uw);
    const double north = 0.5 * (cv_(x, g, j + 1, i - 1) + cv_(x, g, j + 1, i));
    const double south = 0.5 * (cv_(x, g, j, i - 1) + cv_(x, g, j, i));
    const double un = j < g.ny - 1 ? x[e + g.nx] : -uc, us = j > 0 ? x[e - g.nx] : -uc;
    double r = (east * east - west * west) * g.ihx;
    r += (north * 0.5 * (uc + un) - south * 0.5 * (uc + us)) * g.ihy;
    r -= 0.5 * uc * ((east - west) * g.ihx + (north - south) * g.ihy);
    return r;
  }
  const int f = e - g.nu, J = f / g.nx + 1, i = f - (J - 1) * g.nx;
  const double vc = x[e];
  const double east = 0.5 * (cu_(x, g, J - 1, i + 1) + cu_(x, g, J, i + 1));
  const double west = 0.5 * (cu_(x, g, J - 1, i) + cu_(x, g, J, i));
  const double vn = cv_(x, g, J + 1, i), vs = cv_(x, g, J - 1, i);
  const double north = 0.5 * (vc + vn), south = 0.5 * (vc + vs);
  double r = (east * 0.5 * (vc + cv_(x, g, J, i + 1)) - west * 0.5 * (vc + cv_(x, g, J, i - 1))) * g.ihx;
  r += (north * north - south * south) * g.ihy;
  r -= 0.5 * vc * ((east - west) * g.ihx + (north - south) * g.ihy);
  return r;
}

// which: 0 K, 1 D (velocity -> cells), 2 G (cells -> velocity), 3 convection
__global__ void k_ch_apply(ChanGrid g, int which, const double* in, double* out) {
  const int c = blockIdx.y;
  const int n = which == 1 ? g.np : g.size;
  const long long is = which == 2 ? g.np : g.size, os = which == 1 ? g.np : g.size;
  const double* x = in + c * is;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    double v;
    if (which == 0) v = ch_K(x, g, e);
    else if (which == 1) v = ch_D(x, g, e / g.nx, e - (e / g.nx) * g.nx);
    else if (which == 2) v = ch_G(x, g, e);
    else v = ch_conv(x, g, e);
    out[c * os + e] = v;
  }
}

// out = sum_k a_k f_k over n values, accumulated in the order given
struct ChTerms {
  const double* f[8];
  double a[8];
  int n;
};
__global__ void k_ch_combine(ChTerms t, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < t.n; ++k) s += t.a[k] * t.f[k][i];
    out[i] = s;
  }
}

// Per-block partial sums / maxima for dot(a,b) and max|a| (abs keys).
__global__ void k_ch_dot(const double* a, const double* b, long long n, double* partial) {
  __shared__ double red[32];
  __shared__ unsigned long long redk[32];
  double s[1] = {0.0};
  unsigned long long m[1] = {0ull};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double av = a[i];
    if (b) s[0] += av * b[i];
    m[0] = max(m[0], abs_key(av));
  }
  block_sum<1>(s, red);
  block_max_key<1>(m, redk);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = s[0];
    reinterpret_cast<unsigned long long*>(partial)[2 * blockIdx.x + 1] = m[0];
  }
}
__global__ void k_ch_dot_fold(const double* partial, int nb, double* out) {
  __shared__ double red[32];
  __shared__ unsigned long long redk[32];
  double s[1] = {0.0};
  unsigned long long m[1] = {0ull};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    s[0] += partial[2 * b];
    m[0] = max(m[0], reinterpret_cast<const unsigned long long*>(partial)[2 * b + 1]);
  }
  block_sum<1>(s, red);
  block_max_key<1>(m, redk);
  if (threadIdx.x == 0) {
    out[0] = s[0];
    out[1] = key_value(m[0]);
  }
}

// flow rate through each x column of u faces: hy * sum_j u[j, i] (model.py:94-96)
__global__ void k_ch_flow(ChanGrid g, const double* x, double* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nx; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < g.ny; ++j) s += x[j * g.nx + i];
    out[i] = g.hy * s;
  }
}

// ------------------------------------------------------------ real FFTs ---
// rows of length nx, two real rows per complex line; spectral layout
// [column][row][nm] complex (orthonormal scaling).
__global__ void k_ch_rfft(const double* in, long long cstride, int rows, int nx, int nm, cd* out,
                          long long ostride, FFTPlan plan, const cd* tw, double scale, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cd* buf = reinterpret_cast<cd*>(smraw);
  cd* tmp = buf + nl * nx;
  const int c = blockIdx.y;
  const int pair0 = blockIdx.x * nl;
  const int npairs = (rows + 1) / 2;
  const double* x = in + c * cstride;
  for (int e = threadIdx.x; e < nl * nx; e += blockDim.x) {
    const int q = e / nx, i = e - q * nx, pr = pair0 + q;
    const int ra = 2 * pr, rb = 2 * pr + 1;
    const double a = (pr < npairs && ra < rows) ? x[(long long)ra * nx + i] : 0.0;
    const double b = (pr < npairs && rb < rows) ? x[(long long)rb * nx + i] : 0.0;
    buf[e] = mk(a, b);
  }
  __syncthreads();
  fft_lines<double, 8>(buf, tmp, plan, nx, nl, tw, -1);
  cd* o = out + c * ostride;
  for (int e = threadIdx.x; e < nl * nm; e += blockDim.x) {
    const int q = e / nm, k = e - q * nm, pr = pair0 + q;
    if (pr >= npairs) continue;
    const cd zk = buf[q * nx + k], zm = buf[q * nx + (k == 0 ? 0 : nx - k)];
    const cd cz = conjg(zm);
    // A = (Z_k + conj Z_{N-k}) / 2, B = (Z_k - conj Z_{N-k}) / (2i)
    const cd A = mk(0.5 * (zk.x + cz.x) * scale, 0.5 * (zk.y + cz.y) * scale);
    const cd B = mk(0.5 * (zk.y - cz.y) * scale, -0.5 * (zk.x - cz.x) * scale);
    const int ra = 2 * pr, rb = 2 * pr + 1;
    o[(long long)ra * nm + k] = A;
    if (rb < rows) o[(long long)rb * nm + k] = B;
  }
}

// inverse of k_ch_rfft (numpy irfft semantics: the imaginary parts of the
// mode-0 and Nyquist coefficients are ignored)
__global__ void k_ch_irfft(const cd* in, long long istride, int rows, int nx, int nm, double* out, long long cstride,
                           FFTPlan plan, const cd* tw, double scale, int nl) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cd* buf = reinterpret_cast<cd*>(smraw);
  cd* tmp = buf + nl * nx;
  const int c = blockIdx.y;
  const int pair0 = blockIdx.x * nl;
  const int npairs = (rows + 1) / 2;
  const cd* s = in + c * istride;
  const bool even = (nx % 2) == 0;
  for (int e = threadIdx.x; e < nl * nx; e += blockDim.x) {
    const int q = e / nx, k = e - q * nx, pr = pair0 + q;
    const int ra = 2 * pr, rb = 2 * pr + 1;
    cd A = mk(0.0, 0.0), B = mk(0.0, 0.0);
    const int kk = k < nm ? k : nx - k;
    if (pr < npairs) {
      A = s[(long long)ra * nm + kk];
      if (rb < rows) B = s[(long long)rb * nm + kk];
    }
    if (kk == 0 || (even && kk == nx / 2)) {
      A.y = 0.0;
      B.y = 0.0;
    }
    if (k >= nm) {  // Hermitian half: Z_k = conj(A_{N-k}) + i conj(B_{N-k})
      A = conjg(A);
      B = conjg(B);
    }
    buf[e] = mk(A.x - B.y, A.y + B.x);  // A + i B
  }
  __syncthreads();
  fft_lines<double, 8>(buf, tmp, plan, nx, nl, tw, +1);
  double* x = out + c * cstride;
  for (int e = threadIdx.x; e < nl * nx; e += blockDim.x) {
    const int q = e / nx, i = e - q * nx, pr = pair0 + q;
    if (pr >= npairs) continue;
    const int ra = 2 * pr, rb = 2 * pr + 1;
    x[(long long)ra * nx + i] = buf[e].x * scale;
    if (rb < rows) x[(long long)rb * nx + i] = buf[e].y * scale;
  }
}

// ---------------------------------------------------------- mode solves ---
struct ModeCoef {
  cd d;
  double lam;
};
__device__ ModeCoef mode_coef(const ChanGrid& g, int m) {
  const double kPi = 3.14159265358979323846264338327950288;
  const double theta = 2.0 * kPi * m / g.nx;
  ModeCoef r;
  if ((g.nx % 2) == 0 && m == g.nx / 2) r.d = mk(-2.0 * g.ihx, 0.0);
  else r.d = mk((cos(theta) - 1.0) * g.ihx, sin(theta) * g.ihx);
  const double sh = sin(0.5 * theta);
  r.lam = 4.0 * sh * sh * g.ihx2;
  return r;
}

// Band element (i, j) of the factor of mode m1 + 1 (LAPACK band layout:
// column j holds rows j-KU-KL .. j+KL at offsets 0 .. LD-1).  The modes are
// interleaved (element e of every mode contiguous, nmodes apart), so the
// threads of a warp, one mode each, read and write coalesced.
__device__ __forceinline__ long long band_index(int i, int j, int nmodes, int m1) {
  return ((long long)j * kLD + (kKL + kKU + i - j)) * nmodes + m1;
}

// Assemble and factor the saddle system of every mode m >= 1 (one thread per
// mode); mode 0 stores the Thomas factors of hu0 = m I + k Ly(ny, wall).
__global__ void k_ch_factor(ChanGrid g, double mass, double visc, cd* lu, int* piv, double* zero, int* status) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= g.nm) return;
  const int ny = g.ny;
  const double iy2 = g.ihy2;
  if (m == 0) {
    // Thomas: diag a_j = mass + visc*wall_j/hy^2, off = -visc/hy^2
    double* cp = zero;        // modified super-diagonal
    double* dn = zero + ny;   // pivots
    const double off = -visc * iy2;
    for (int j = 0; j < ny; ++j) {
      const double a = mass + visc * ((j == 0 || j == ny - 1) ? 3.0 : 2.0) * iy2;
      const double den = j == 0 ? a : a - off * cp[j - 1];
      dn[j] = den;
      cp[j] = off / den;
      if (!(den != 0.0)) status[0] = 1;
    }
    return;
  }
  const int n = 3 * ny - 1;
  const int nmodes = g.nm - 1, m1 = m - 1;
  auto band = [&](int i, int j) -> cd& { return lu[band_index(i, j, nmodes, m1)]; };
  for (long long e = 0; e < (long long)n * kLD; ++e) lu[e * nmodes + m1] = mk(0.0, 0.0);
  const ModeCoef mc = mode_coef(g, m);
  const double a0 = mass + visc * mc.lam;
  const cd d = mc.d, dc = conjg(d);
  for (int j = 0; j < ny; ++j) {
    const int ru = 3 * j, rp = 3 * j + 1, rv = 3 * j + 2;
    // u_j momentum: hu, -conj(d) p_j
    band(ru, ru) = mk(a0 + visc * ((j == 0 || j == ny - 1) ? 3.0 : 2.0) * iy2, 0.0);
    if (j > 0) band(ru, ru - 3) = mk(-visc * iy2, 0.0);
    if (j < ny - 1) band(ru, ru + 3) = mk(-visc * iy2, 0.0);
    band(ru, rp) = mk(-dc.x, -dc.y);
    // continuity j (negated): -d u_j - (v_j - v_{j-1})/hy
    band(rp, ru) = mk(-d.x, -d.y);
    if (j < ny - 1) band(rp, rv) = mk(-g.ihy, 0.0);
    if (j > 0) band(rp, rv - 3) = mk(g.ihy, 0.0);
    // v_j momentum (face j+1): hv, -(p_j - p_{j+1})/hy
    if (j < ny - 1) {
      band(rv, rv) = mk(a0 + 2.0 * visc * iy2, 0.0);
      if (j > 0) band(rv, rv - 3) = mk(-visc * iy2, 0.0);
      if (j < ny - 2) band(rv, rv + 3) = mk(-visc * iy2, 0.0);
      band(rv, rp) = mk(-g.ihy, 0.0);
      band(rv, rp + 3) = mk(g.ihy, 0.0);
    }
  }
  // banded LU with partial pivoting (the elimination order of gbtf2)
  int ju = 0;
  for (int k = 0; k < n; ++k) {
    const int km = min(kKL, n - 1 - k);
    int p = 0;
    double best = -1.0;
    for (int r = 0; r <= km; ++r) {
      const cd v = band(k + r, k);
      const double a = fabs(v.x) + fabs(v.y);  // |re| + |im|, as izamax
      if (a > best) {
        best = a;
        p = r;
      }
    }
    piv[(long long)k * nmodes + m1] = k + p;
    if (!(best > 0.0)) {
      status[0] = 2;
      continue;
    }
    ju = max(ju, min(k + kKU + p, n - 1));
    if (p != 0)
      for (int j = k; j <= ju; ++j) {
        const cd t = band(k, j);
        band(k, j) = band(k + p, j);
        band(k + p, j) = t;
      }
    const cd piv_v = band(k, k);
    const double den = piv_v.x * piv_v.x + piv_v.y * piv_v.y;
    const cd inv = mk(piv_v.x / den, -piv_v.y / den);
    for (int r = 1; r <= km; ++r) band(k + r, k) = cmul(band(k + r, k), inv);
    for (int j = k + 1; j <= ju; ++j) {
      const cd akj = band(k, j);
      if (akj.x == 0.0 && akj.y == 0.0) continue;
      for (int r = 1; r <= km; ++r) {
        cd& t = band(k + r, j);
        t = t - cmul(band(k + r, k), akj);
      }
    }
  }
  // the solve multiplies by 1/U(k,k): store the reciprocal pivots
  for (int k = 0; k < n; ++k) {
    const cd d = band(k, k);
    const double den = d.x * d.x + d.y * d.y;
    band(k, k) = mk(d.x / den, -d.y / den);
  }
}

// Partitioned (spike) substitution: one warp per (mode >= 1, column).  The
// n = 3 ny - 1 steps of each sweep are split into 32 chunks, one per lane.
// A sweep step is an affine map of its register window (forward: the 4
// pending entries; back: the last 6 unknowns), so a lane (1) runs its chunk
// on the unit windows and on the zero window with the chunk's inputs, which
// gives the chunk's map W_out = T W_in + t; (2) the lanes pass the windows
// along (W_in of chunk c+1 = T_c W_in(c) + t_c, 31 shuffle steps); (3) each
// lane reruns its chunk from its true window.  The dependent chain per lane
// is about 2 n / 32 + 31 steps instead of 2 n.  Mode 0 runs on one extra
// warp per column (ch_mode0_warp).
// Mode 0 of column c by one warp: hu0 u = fu by Thomas, v = 0, and
// p_{j+1} = p_j + hy fv_j with the mean removed.  The three recurrences are
// affine in their carried value (y_j = a_j y_{j-1} + b_j), so each lane
// composes its chunk's map, the lanes pass the carried value along (31
// shuffle steps), and each lane reruns its chunk from the true value.
__device__ __forceinline__ void ch_mode0_warp(const ChanGrid& g, const cd* __restrict__ fu, const cd* __restrict__ fv,
                                              long long fstride, const double* __restrict__ zero, cd* __restrict__ uo,
                                              cd* __restrict__ vo, cd* __restrict__ po, long long vstride,
                                              long long pstride, double visc, int c, int lane) {
  const int ny = g.ny, nm = g.nm;
  const cd* fuc = fu + c * fstride;
  const cd* fvc = fv + c * fstride;
  cd* uc = uo + c * vstride;
  cd* vc = vo + c * vstride;
  cd* pc = po + c * pstride;
  const double* cp = zero;
  const double* dn = zero + ny;
  const double off = -visc * g.ihy2;
  const cd z0 = mk(0.0, 0.0);
  const int S = (ny + 31) / 32;
  const int j0 = min(lane * S, ny), j1 = min(j0 + S, ny);
  // carry v across lanes: lane it+1 receives lane it's map applied to its carry
  auto pass = [&](double a, cd b, cd first) -> cd {  // returns this lane's incoming carry
    cd v = first;
    for (int it = 0; it < 31; ++it) {
      const cd cand = mk(a * v.x + b.x, a * v.y + b.y);
      const double re = __shfl_sync(0xffffffffu, cand.x, it), im = __shfl_sync(0xffffffffu, cand.y, it);
      if (lane == it + 1) v = mk(re, im);
    }
    return v;
  };
  // forward Thomas: y_j = (f_j - off y_{j-1}) / dn_j  (y_{-1} = 0)
  double A = 1.0;
  cd B = z0;
  for (int j = j0; j < j1; ++j) {
    const double a = -off / dn[j];
    const cd f = fuc[(long long)j * nm];
    const cd b = mk(f.x / dn[j], f.y / dn[j]);
    A = a * A;
    B = mk(a * B.x + b.x, a * B.y + b.y);
  }
  cd yin = pass(A, B, z0);
  for (int j = j0; j < j1; ++j) {
    const cd f = fuc[(long long)j * nm];
    yin = mk((f.x - off * yin.x) / dn[j], (f.y - off * yin.y) / dn[j]);
    uc[(long long)j * nm] = yin;
  }
  __syncwarp();
  // back: u_j = y_j - cp_j u_{j+1} (u_{ny} = 0 reproduces u_{ny-1} = y_{ny-1});
  // chunks from the top: lane l covers j = ny-1-l S down to ny-(l+1) S
  const int bt = ny - 1 - min(lane * S, ny), bb = max(ny - (lane + 1) * S, 0);
  A = 1.0;
  B = z0;
  for (int j = bt; j >= bb; --j) {
    const double a = j < ny - 1 ? -cp[j] : 0.0;
    const cd yj = uc[(long long)j * nm];
    A = a * A;
    B = mk(a * B.x + yj.x, a * B.y + yj.y);
  }
  cd uin = pass(A, B, z0);
  __syncwarp();  // every lane has read its y before any overwrites them
  for (int j = bt; j >= bb; --j) {
    const cd yj = uc[(long long)j * nm];
    uin = j < ny - 1 ? mk(yj.x - cp[j] * uin.x, yj.y - cp[j] * uin.y) : yj;
    uc[(long long)j * nm] = uin;
  }
  for (int k = lane; k < ny - 1; k += 32) vc[(long long)k * nm] = z0;
  // pressure: p_0 = 0, p_j = p_{j-1} + hy fv_{j-1}; then the mean removed
  cd P = z0;
  for (int j = j0; j < j1; ++j)
    if (j > 0) {
      const cd f = fvc[(long long)(j - 1) * nm];
      P = mk(P.x + g.hy * f.x, P.y + g.hy * f.y);
    }
  cd pin = pass(1.0, P, z0);
  cd sum = z0;
  for (int j = j0; j < j1; ++j) {
    if (j > 0) {
      const cd f = fvc[(long long)(j - 1) * nm];
      pin = mk(pin.x + g.hy * f.x, pin.y + g.hy * f.y);
    }
    pc[(long long)j * nm] = pin;
    sum = sum + pin;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sum.x += __shfl_xor_sync(0xffffffffu, sum.x, o);
    sum.y += __shfl_xor_sync(0xffffffffu, sum.y, o);
  }
  const cd mean = mk(sum.x / ny, sum.y / ny);
  for (int j = j0; j < j1; ++j) pc[(long long)j * nm] = pc[(long long)j * nm] - mean;
}

// One warp per CTA: the kernel is warp-synchronous (shuffles only), and
// with 8-warp CTAs the 514 warps of a 512-mode, two-column solve packed into
// 65 CTAs, so 65 of GB300's 152 SMs did all the FP64 work (ncu: FP64 pipe 86%
// busy on the active SMs, 36% over the GPU).  Single-warp CTAs spread the
// recurrences over every SM (3-4 warps each).
constexpr int kSpikeThreads = 32;
__global__ void __launch_bounds__(kSpikeThreads) k_ch_solve_spike(
    ChanGrid g, const cd* __restrict__ fu, const cd* __restrict__ fv, long long fstride, const cd* __restrict__ lu,
    const int* __restrict__ piv, const double* __restrict__ zero, cd* __restrict__ uo, cd* __restrict__ vo,
    cd* __restrict__ po, long long vstride, long long pstride, cd* __restrict__ work, int cols, double visc) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nm = g.nm, ny = g.ny, nmodes = nm - 1;
  if (warp < cols) {
    ch_mode0_warp(g, fu, fv, fstride, zero, uo, vo, po, vstride, pstride, visc, warp, lane);
    return;
  }
  const int wm = warp - cols;
  if (wm >= nmodes * cols) return;  // whole warp
  const int c = wm / nmodes, m1 = wm - c * nmodes, m = m1 + 1;
  const cd z0 = mk(0.0, 0.0), one = mk(1.0, 0.0);
  const cd* fuc = fu + c * fstride;
  const cd* fvc = fv + c * fstride;
  cd* uc = uo + c * vstride;
  cd* vc = vo + c * vstride;
  cd* pc = po + c * pstride;
  const int n = 3 * ny - 1;
  const long long wstride = (long long)cols * nmodes;
  cd* y = work + (long long)c * nmodes + m1;
  const long long cstep = (long long)kLD * nmodes;
  const cd* lum = lu + m1;
  const int* pvm = piv + m1;
  const int oL1 = 7 * nmodes, oL2 = 8 * nmodes, oL3 = 9 * nmodes, oD = 6 * nmodes;
  const long long fj = nm;
  auto rhs = [&](int k) -> cd {  // entry k < n of the interleaved right-hand side
    const int j = k / 3, r = k - 3 * j;
    return r == 0 ? fuc[(long long)j * fj + m] : (r == 1 ? z0 : fvc[(long long)j * fj + m]);
  };
  const int S = (n + 31) / 32;
  // ---- forward: window (w0..w3) = b[k..k+3] before step k -------------------
  const int f0 = min(lane * S, n), f1 = min(f0 + S, n);
  // one forward step of NV windows; the last one (if aff) takes b[k+4]
  auto fwd = [&](auto& W, int nv, int k, bool aff, cd* out) {
    const cd* col = lum + k * cstep;
    const int p = pvm[(long long)k * nmodes] - k;
    const cd l1 = k + 1 < n ? col[oL1] : z0, l2 = k + 2 < n ? col[oL2] : z0, l3 = k + 3 < n ? col[oL3] : z0;
    const cd bn = (aff && k + 4 < n) ? rhs(k + 4) : z0;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      if (v >= nv) break;
      cd w0 = W[v][0], w1 = W[v][1], w2 = W[v][2], w3 = W[v][3];
      if (p == 1) { const cd tmp = w0; w0 = w1; w1 = tmp; }
      else if (p == 2) { const cd tmp = w0; w0 = w2; w2 = tmp; }
      else if (p == 3) { const cd tmp = w0; w0 = w3; w3 = tmp; }
      if (out && v == nv - 1) *out = w0;
      if (k + 1 < n) w1 = w1 - cmul(l1, w0);
      if (k + 2 < n) w2 = w2 - cmul(l2, w0);
      if (k + 3 < n) w3 = w3 - cmul(l3, w0);
      W[v][0] = w1;
      W[v][1] = w2;
      W[v][2] = w3;
      W[v][3] = (aff && v == nv - 1) ? bn : z0;
    }
  };
  cd T[5][4];  // columns 0..3: responses to the unit windows; 4: the affine part
#pragma unroll
  for (int v = 0; v < 5; ++v)
#pragma unroll
    for (int i = 0; i < 4; ++i) T[v][i] = (v == i) ? one : z0;
  for (int k = f0; k < f1; ++k) fwd(T, 5, k, true, nullptr);
  // pass the windows along the chunks
  cd win[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) win[i] = (lane == 0 && i < n) ? rhs(i) : z0;
  for (int it = 0; it < 31; ++it) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      cd cand = T[4][i];
#pragma unroll
      for (int j = 0; j < 4; ++j) cand = cand + cmul(T[j][i], win[j]);
      const double re = __shfl_sync(0xffffffffu, cand.x, it), im = __shfl_sync(0xffffffffu, cand.y, it);
      if (lane == it + 1) win[i] = mk(re, im);
    }
  }
  {
    cd W1[1][4] = {{win[0], win[1], win[2], win[3]}};
    for (int k = f0; k < f1; ++k) {
      cd yk;
      fwd(W1, 1, k, true, &yk);
      y[(long long)k * wstride] = yk;
    }
  }
  __syncwarp();
  // ---- back: window (x1..x6) = x[k+1..k+6] before step k (descending) -------
  const int bt = n - 1 - min(lane * S, n), bb = max(n - (lane + 1) * S, 0);  // chunk k = bt .. bb
  auto bwd = [&](auto& X, int nv, int k, bool aff, cd* out) {
    const cd* col = lum + k * cstep;
    cd a[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) a[i] = k + 1 + i < n ? col[(15 + 9 * i) * nmodes] : z0;
    const cd rp = col[oD];
    const cd yk = aff ? y[(long long)k * wstride] : z0;
#pragma unroll
    for (int v = 0; v < 7; ++v) {
      if (v >= nv) break;
      cd sacc = (aff && v == nv - 1) ? yk : z0;
      if (k + 6 < n) sacc = sacc - cmul(a[5], X[v][5]);
      if (k + 5 < n) sacc = sacc - cmul(a[4], X[v][4]);
      if (k + 4 < n) sacc = sacc - cmul(a[3], X[v][3]);
      if (k + 3 < n) sacc = sacc - cmul(a[2], X[v][2]);
      if (k + 2 < n) sacc = sacc - cmul(a[1], X[v][1]);
      if (k + 1 < n) sacc = sacc - cmul(a[0], X[v][0]);
      const cd xk = cmul(sacc, rp);
      if (out && v == nv - 1) *out = xk;
      X[v][5] = X[v][4];
      X[v][4] = X[v][3];
      X[v][3] = X[v][2];
      X[v][2] = X[v][1];
      X[v][1] = X[v][0];
      X[v][0] = xk;
    }
  };
  // the chunk's map in two batches (registers): unit windows 0..3, then 4, 5 and the affine part
  cd R[7][6];
  {
    cd XA[4][6];
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int i = 0; i < 6; ++i) XA[v][i] = (v == i) ? one : z0;
    for (int k = bt; k >= bb; --k) bwd(XA, 4, k, false, nullptr);
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int i = 0; i < 6; ++i) R[v][i] = XA[v][i];
  }
  {
    cd XB[3][6];
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int i = 0; i < 6; ++i) XB[v][i] = (v < 2 && v + 4 == i) ? one : z0;
    for (int k = bt; k >= bb; --k) bwd(XB, 3, k, true, nullptr);
#pragma unroll
    for (int v = 0; v < 3; ++v)
#pragma unroll
      for (int i = 0; i < 6; ++i) R[4 + v][i] = XB[v][i];
  }
  cd xin[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) xin[i] = z0;  // above the top chunk: x[n..n+5] = 0
  for (int it = 0; it < 31; ++it) {
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      cd cand = R[6][i];
#pragma unroll
      for (int j = 0; j < 6; ++j) cand = cand + cmul(R[j][i], xin[j]);
      const double re = __shfl_sync(0xffffffffu, cand.x, it), im = __shfl_sync(0xffffffffu, cand.y, it);
      if (lane == it + 1) xin[i] = mk(re, im);
    }
  }
  {
    cd X1[1][6] = {{xin[0], xin[1], xin[2], xin[3], xin[4], xin[5]}};
    for (int k = bt; k >= bb; --k) {
      cd xk;
      bwd(X1, 1, k, true, &xk);
      const int j = k / 3, r = k - 3 * j;
      const long long o = (long long)j * fj + m;
      if (r == 0) uc[o] = xk;
      else if (r == 1) pc[o] = xk;
      else vc[o] = xk;
    }
  }
}

// pressure -= mean over all cells, per column (fft_stokes.py:122), in two
// launches over (kChCenterBlocks, column): block sums, then every block folds
// the column's block sums in the same fixed order and shifts its part.
constexpr int kChCenterBlocks = 128;
__global__ void k_ch_center_sums(const double* p, int np, double* partial) {
  __shared__ double red[32];
  const int c = blockIdx.y;
  double s[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
    s[0] += p[(long long)c * np + i];
  block_sum<1>(s, red);
  if (threadIdx.x == 0) partial[c * gridDim.x + blockIdx.x] = s[0];
}
__global__ void k_ch_center_shift(double* p, int np, const double* partial) {
  __shared__ double mean;
  const int c = blockIdx.y;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < gridDim.x; ++b) t += partial[c * gridDim.x + b];
    mean = t / np;
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x)
    p[(long long)c * np + i] -= mean;
}

// Closing checks (fft_stokes.py:124-131): max|defect|, max|f|, max|u|,
// max|D u|, non-finite velocity/pressure; abs keys folded per column.
__global__ void k_ch_check(ChanGrid g, const double* vel, const double* pres, const double* f, double mass,
                           double visc, unsigned long long* keys) {
  constexpr unsigned long long kInf = 0x7ff0000000000000ull;
  __shared__ unsigned long long redk[5 * 32];
  const int c = blockIdx.y;
  const double* u = vel + (long long)c * g.size;
  const double* p = pres + (long long)c * g.np;
  const double* ff = f + (long long)c * g.size;
  unsigned long long m[5] = {0, 0, 0, 0, 0};
  const int n = g.size > g.np ? g.size : g.np;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    if (e < g.size) {
      const double d = mass * u[e] + visc * ch_K(u, g, e) + ch_G(p, g, e) - ff[e];
      m[0] = max(m[0], abs_key(d));
      m[1] = max(m[1], abs_key(ff[e]));
      const unsigned long long ku = abs_key(u[e]);
      m[2] = max(m[2], ku);
      if (ku >= kInf) m[4] = 1;
    }
    if (e < g.np) {
      const int j = e / g.nx, i = e - j * g.nx;
      m[3] = max(m[3], abs_key(ch_D(u, g, j, i)));
      if (abs_key(p[e]) >= kInf) m[4] = 1;
    }
  }
  block_max_key<5>(m, redk);
  if (threadIdx.x == 0)
    for (int k = 0; k < 5; ++k) atomicMax(keys + c * 5 + k, m[k]);
}

}  // namespace

struct Channel {
  ChanGrid g;
  double lx, ly, tol;
  int cache_size;
  std::string err;
  FFTPlan plan;
  cd* tw = nullptr;
  int nl = 1;
  size_t smem = 0;
  // factor cache: (mass, visc) -> slot
  struct Slot {
    double mass, visc;
    cd* lu;
    int* piv;
    double* zero;
    long long last_use;
  };
  std::vector<Slot> slots;
  long long clock = 0;
  int* status = nullptr;
  int* h_status = nullptr;
  // per-solve buffers (maxcols columns)
  int maxcols = 0;
  cd *fspec = nullptr, *uspec = nullptr, *pspec = nullptr, *work = nullptr;
  unsigned long long* keys = nullptr;
  unsigned long long* h_keys = nullptr;
  double* partial = nullptr;
  double* h_red = nullptr;
  double* d_red = nullptr;
};

}  // namespace macsav

using macsav::Channel;
using macsav::cd;

struct macsav_channel {
  Channel ch;
};

namespace {

int ch_fail(Channel* C, int code, const char* msg) {
  C->err = msg;
  return code;
}
int ch_cuda(Channel* C) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    C->err = std::string("CUDA: ") + cudaGetErrorString(e);
    return MACSAV_ERR_CUDA;
  }
  return MACSAV_OK;
}
int ch_grid_blocks(long long n) {
  long long b = (n + macsav::kChThreads - 1) / macsav::kChThreads;
  return int(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

int ensure_buffers(Channel* C, int cols) {
  if (cols <= C->maxcols) return MACSAV_OK;
  cudaFree(C->fspec);
  cudaFree(C->uspec);
  cudaFree(C->pspec);
  cudaFree(C->work);
  cudaFree(C->keys);
  cudaFreeHost(C->h_keys);
  const auto& g = C->g;
  const size_t rows = size_t(2 * g.ny - 1);
  if (cudaMalloc(&C->fspec, sizeof(cd) * rows * g.nm * cols) != cudaSuccess ||
      cudaMalloc(&C->uspec, sizeof(cd) * rows * g.nm * cols) != cudaSuccess ||
      cudaMalloc(&C->pspec, sizeof(cd) * size_t(g.ny) * g.nm * cols) != cudaSuccess ||
      cudaMalloc(&C->work, sizeof(cd) * size_t(3 * g.ny - 1) * g.nm * cols) != cudaSuccess ||
      cudaMalloc(&C->keys, sizeof(unsigned long long) * 5 * cols) != cudaSuccess ||
      cudaMallocHost(&C->h_keys, sizeof(unsigned long long) * 5 * cols) != cudaSuccess)
    return ch_cuda(C);
  C->maxcols = cols;
  return MACSAV_OK;
}

void launch_fft(Channel* C, bool inverse, const void* in, long long istride, int rows, void* out, long long ostride,
                int cols, cudaStream_t s) {
  const auto& g = C->g;
  const int npairs = (rows + 1) / 2;
  const dim3 grid((npairs + C->nl - 1) / C->nl, cols);
  const double scale = 1.0 / std::sqrt(double(g.nx));
  if (!inverse)
    macsav::k_ch_rfft<<<grid, macsav::kChThreads, C->smem, s>>>(static_cast<const double*>(in), istride, rows, g.nx,
                                                               g.nm, static_cast<cd*>(out), ostride, C->plan, C->tw,
                                                               scale, C->nl);
  else
    macsav::k_ch_irfft<<<grid, macsav::kChThreads, C->smem, s>>>(static_cast<const cd*>(in), istride, rows, g.nx,
                                                                g.nm, static_cast<double*>(out), ostride, C->plan,
                                                                C->tw, scale, C->nl);
}

}  // namespace

extern "C" {

int macsav_channel_create(macsav_channel** out, int nx, int ny, double lx, double ly, double tolerance,
                          int cache_size) {
  if (!out) return MACSAV_ERR_VALUE;
  *out = nullptr;
  if (nx < 3 || ny < 3 || !std::isfinite(lx) || !std::isfinite(ly) || lx <= 0 || ly <= 0) return MACSAV_ERR_VALUE;
  if (cache_size < 1 || !(tolerance > 0) || !std::isfinite(tolerance)) return MACSAV_ERR_VALUE;
  if (nx > 2048) return MACSAV_ERR_UNSUPPORTED;
  macsav_channel* h = new macsav_channel();
  Channel& C = h->ch;
  auto& g = C.g;
  g.nx = nx;
  g.ny = ny;
  g.nu = nx * ny;
  g.nv = nx * (ny - 1);
  g.size = g.nu + g.nv;
  g.np = nx * ny;
  g.nm = nx / 2 + 1;
  g.hx = lx / nx;
  g.hy = ly / ny;
  g.ihx = 1.0 / g.hx;
  g.ihy = 1.0 / g.hy;
  g.ihx2 = g.ihx * g.ihx;
  g.ihy2 = g.ihy * g.ihy;
  C.lx = lx;
  C.ly = ly;
  C.tol = tolerance;
  C.cache_size = cache_size;
  C.plan = macsav::make_fft_plan(nx);
  std::vector<cd> tw(nx);
  const double kPi = 3.14159265358979323846264338327950288;
  for (int m = 0; m < nx; ++m) tw[m] = macsav::mk(std::cos(2 * kPi * m / nx), -std::sin(2 * kPi * m / nx));
  C.nl = std::max(1, 2048 / nx);
  C.smem = size_t(2) * C.nl * nx * sizeof(cd);
  int rc = MACSAV_OK;
  if (cudaMalloc(&C.tw, sizeof(cd) * nx) != cudaSuccess ||
      cudaMemcpy(C.tw, tw.data(), sizeof(cd) * nx, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMalloc(&C.status, sizeof(int)) != cudaSuccess || cudaMallocHost(&C.h_status, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&C.partial, sizeof(double) * 2 * 1024) != cudaSuccess ||
      cudaMalloc(&C.d_red, sizeof(double) * 2) != cudaSuccess ||
      cudaMallocHost(&C.h_red, sizeof(double) * 2) != cudaSuccess)
    rc = MACSAV_ERR_CUDA;
  if (rc == MACSAV_OK && C.smem > 48 * 1024) {
    cudaFuncSetAttribute(macsav::k_ch_rfft, cudaFuncAttributeMaxDynamicSharedMemorySize, int(C.smem));
    cudaFuncSetAttribute(macsav::k_ch_irfft, cudaFuncAttributeMaxDynamicSharedMemorySize, int(C.smem));
  }
  if (rc == MACSAV_OK) rc = ensure_buffers(&C, 2);
  if (rc != MACSAV_OK) {
    macsav_channel_destroy(h);
    return MACSAV_ERR_CUDA;
  }
  *out = h;
  return MACSAV_OK;
}

void macsav_channel_destroy(macsav_channel* h) {
  if (!h) return;
  Channel& C = h->ch;
  cudaDeviceSynchronize();
  for (auto& s : C.slots) {
    cudaFree(s.lu);
    cudaFree(s.piv);
    cudaFree(s.zero);
  }
  cudaFree(C.tw);
  cudaFree(C.status);
  cudaFreeHost(C.h_status);
  cudaFree(C.fspec);
  cudaFree(C.uspec);
  cudaFree(C.pspec);
  cudaFree(C.work);
  cudaFree(C.keys);
  cudaFreeHost(C.h_keys);
  cudaFree(C.partial);
  cudaFree(C.d_red);
  cudaFreeHost(C.h_red);
  delete h;
}

const char* macsav_channel_error(const macsav_channel* h) { return h ? h->ch.err.c_str() : ""; }

int macsav_channel_apply(macsav_channel* h, int which, const double* in, double* out, int cols, void* stream) {
  if (!h || !in || !out || which < 0 || which > 3 || cols < 1) return MACSAV_ERR_VALUE;
  Channel& C = h->ch;
  const int n = which == 1 ? C.g.np : C.g.size;
  macsav::k_ch_apply<<<dim3(ch_grid_blocks(n), cols), macsav::kChThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      C.g, which, in, out);
  return ch_cuda(&C);
}

int macsav_channel_combine(macsav_channel* h, int nterms, const double* coeffs, const double* const* fields,
                           double* out, long long n, void* stream) {
  if (!h || nterms < 1 || nterms > 8 || !coeffs || !fields || !out || n < 0) return MACSAV_ERR_VALUE;
  macsav::ChTerms t;
  t.n = nterms;
  for (int k = 0; k < nterms; ++k) {
    t.f[k] = fields[k];
    t.a[k] = coeffs[k];
  }
  macsav::k_ch_combine<<<ch_grid_blocks(n), macsav::kChThreads, 0, static_cast<cudaStream_t>(stream)>>>(t, out, n);
  return ch_cuda(&h->ch);
}

int macsav_channel_reduce(macsav_channel* h, const double* a, const double* b, long long n, double* result,
                          void* stream) {
  if (!h || !a || !result || n < 0) return MACSAV_ERR_VALUE;
  Channel& C = h->ch;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = ch_grid_blocks(n);
  macsav::k_ch_dot<<<nb, macsav::kChThreads, 0, s>>>(a, b, n, C.partial);
  macsav::k_ch_dot_fold<<<1, macsav::kChThreads, 0, s>>>(C.partial, nb, C.d_red);
  cudaMemcpyAsync(C.h_red, C.d_red, sizeof(double) * 2, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return ch_cuda(&C);
  result[0] = C.h_red[0] * C.g.hx * C.g.hy;
  result[1] = C.h_red[1];
  return ch_cuda(&C);
}

int macsav_channel_flow_rates(macsav_channel* h, const double* x, double* out, void* stream) {
  if (!h || !x || !out) return MACSAV_ERR_VALUE;
  macsav::k_ch_flow<<<ch_grid_blocks(h->ch.g.nx), macsav::kChThreads, 0, static_cast<cudaStream_t>(stream)>>>(h->ch.g,
                                                                                                            x, out);
  return ch_cuda(&h->ch);
}

int macsav_channel_solve(macsav_channel* h, const double* rhs, int cols, double mass, double viscosity, double* vel,
                         double* pres, double* residual, double* divergence, int* factorized, void* stream) {
  if (!h) return MACSAV_ERR_VALUE;
  Channel& C = h->ch;
  const auto& g = C.g;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!std::isfinite(mass) || !std::isfinite(viscosity) || std::fmin(mass, viscosity) < 0 || mass + viscosity <= 0)
    return ch_fail(&C, MACSAV_ERR_VALUE, "Require nonnegative mass/viscosity with nonzero total");
  if (!rhs || !vel || !pres || cols < 1) return ch_fail(&C, MACSAV_ERR_VALUE, "Invalid channel FFT RHS");
  int rc = ensure_buffers(&C, cols);
  if (rc != MACSAV_OK) return rc;
  if (factorized) *factorized = 0;
  // factor cache (fft_stokes.py:64-92): least recently used slot is evicted
  Channel::Slot* slot = nullptr;
  for (auto& sl : C.slots)
    if (sl.mass == mass && sl.visc == viscosity) slot = &sl;
  if (!slot) {
    Channel::Slot fresh{mass, viscosity, nullptr, nullptr, nullptr, 0};
    if (int(C.slots.size()) >= C.cache_size) {
      size_t old = 0;
      for (size_t k = 1; k < C.slots.size(); ++k)
        if (C.slots[k].last_use < C.slots[old].last_use) old = k;
      fresh.lu = C.slots[old].lu;
      fresh.piv = C.slots[old].piv;
      fresh.zero = C.slots[old].zero;
      C.slots.erase(C.slots.begin() + old);
    } else {
      const long long n = 3LL * g.ny - 1;
      const long long nmodes = std::max(1, g.nm - 1);
      if (cudaMalloc(&fresh.lu, sizeof(cd) * n * macsav::kLD * nmodes) != cudaSuccess ||
          cudaMalloc(&fresh.piv, sizeof(int) * n * nmodes) != cudaSuccess ||
          cudaMalloc(&fresh.zero, sizeof(double) * 2 * g.ny) != cudaSuccess)
        return ch_cuda(&C);
    }
    cudaMemsetAsync(C.status, 0, sizeof(int), s);
    const int tpb = macsav::kChFactorThreads;
    macsav::k_ch_factor<<<(g.nm + tpb - 1) / tpb, tpb, 0, s>>>(g, mass, viscosity, fresh.lu, fresh.piv, fresh.zero,
                                                              C.status);
    cudaMemcpyAsync(C.h_status, C.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return ch_cuda(&C);
    if (C.h_status[0] != 0) {
      cudaFree(fresh.lu);
      cudaFree(fresh.piv);
      cudaFree(fresh.zero);
      return ch_fail(&C, MACSAV_ERR_CG, "Channel band factorization failed");
    }
    C.slots.push_back(fresh);
    slot = &C.slots.back();
    if (factorized) *factorized = 1;
  }
  slot->last_use = ++C.clock;
  const int rows = 2 * g.ny - 1;
  const long long fstride = (long long)rows * g.nm;
  // forward FFTs of the loads (u rows then v rows: one (2ny-1) x nx matrix)
  launch_fft(&C, false, rhs, g.size, rows, C.fspec, fstride, cols, s);
  // mode solves into u/v spectra (uspec: u rows then v rows) and pspec
  // one warp per (mode >= 1, column) in the partitioned form, plus one warp
  // per column for mode 0
  const long long threads = 32LL * (cols + (long long)(g.nm - 1) * cols);
  const int tpb = macsav::kSpikeThreads;
  macsav::k_ch_solve_spike<<<int((threads + tpb - 1) / tpb), tpb, 0, s>>>(
      g, C.fspec, C.fspec + (long long)g.ny * g.nm, fstride, slot->lu, slot->piv, slot->zero, C.uspec,
      C.uspec + (long long)g.ny * g.nm, C.pspec, fstride, (long long)g.ny * g.nm, C.work, cols, viscosity);
  launch_fft(&C, true, C.uspec, fstride, rows, vel, g.size, cols, s);
  launch_fft(&C, true, C.pspec, (long long)g.ny * g.nm, g.ny, pres, g.np, cols, s);
  {
    const int nbc = std::max(1, std::min(macsav::kChCenterBlocks, 2048 / cols));  // C.partial holds 2048 sums
    macsav::k_ch_center_sums<<<dim3(nbc, cols), macsav::kChThreads, 0, s>>>(pres, g.np, C.partial);
    macsav::k_ch_center_shift<<<dim3(nbc, cols), macsav::kChThreads, 0, s>>>(pres, g.np, C.partial);
  }
  cudaMemsetAsync(C.keys, 0, sizeof(unsigned long long) * 5 * cols, s);
  const int n = g.size > g.np ? g.size : g.np;
  macsav::k_ch_check<<<dim3(ch_grid_blocks(n), cols), macsav::kChThreads, 0, s>>>(g, vel, pres, rhs, mass,
                                                                                  viscosity, C.keys);
  cudaMemcpyAsync(C.h_keys, C.keys, sizeof(unsigned long long) * 5 * cols, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return ch_cuda(&C);
  if ((rc = ch_cuda(&C)) != MACSAV_OK) return rc;
  double maxdef = 0, maxf = 0, maxu = 0, maxdiv = 0;
  bool bad = false;
  auto mx = [](double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); };
  for (int c = 0; c < cols; ++c) {
    const unsigned long long* k = C.h_keys + 5 * c;
    double v[4];
    for (int q = 0; q < 4; ++q) std::memcpy(&v[q], &k[q], sizeof(double));
    maxdef = mx(maxdef, v[0]);
    maxf = mx(maxf, v[1]);
    maxu = mx(maxu, v[2]);
    maxdiv = mx(maxdiv, v[3]);
    bad |= k[4] != 0;
  }
  const double res = maxdef / (1.0 + maxf);
  if (residual) *residual = res;
  if (divergence) *divergence = maxdiv;
  if (bad || !(res <= C.tol) || !(maxdiv <= C.tol * (1.0 + maxu))) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "Channel FFT residual=%.3e, divergence=%.3e", res, maxdiv);
    return ch_fail(&C, MACSAV_ERR_STOKES_GATE, buf);
  }
  return MACSAV_OK;
}

}  // extern "C"
