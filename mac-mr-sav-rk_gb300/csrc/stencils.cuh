// Matrix-free MAC stencils on packed vectors (walls eliminated).
//
// Packed velocity: u faces (j, i), j < ny, i < nx-1, at j*(nx-1)+i, then v
// faces (j, i), j < ny-1, i < nx, at n_u + j*nx + i (the reference's
// solver/mac/grid.py:52-65).  Cells (j, i) at j*nx+i.
#pragma once
#include "common.cuh"

namespace macsav {

struct GridDev {
  int nx, ny, nu, nv, size, np;
  double hx, hy, ihx, ihy, ihx2, ihy2;
};

// Full-array accessors of a packed vector: u at face column I in [0, nx],
// v at face row J in [0, ny]; normal wall faces are zero.
template <typename In>
__device__ __forceinline__ double U(const In* x, const GridDev& g, int j, int I) {
  return (I <= 0 || I >= g.nx) ? 0.0 : double(x[j * (g.nx - 1) + I - 1]);
}
template <typename In>
__device__ __forceinline__ double V(const In* x, const GridDev& g, int J, int i) {
  return (J <= 0 || J >= g.ny) ? 0.0 : double(x[g.nu + (J - 1) * g.nx + i]);
}

// (K x)_e for packed index e (solver/mac/operators.py:6-18): positive 5-point
// Laplacian, tangential half-cell wall rows have diagonal 3/h^2.
template <typename In>
__device__ __forceinline__ double K_at(const In* x, const GridDev& g, int e) {
  if (e < g.nu) {
    const int w = g.nx - 1, j = e / w, i = e - j * w;
    const double c = double(x[e]);
    const double l = i > 0 ? double(x[e - 1]) : 0.0, r = i < w - 1 ? double(x[e + 1]) : 0.0;
    const double s = j > 0 ? double(x[e - w]) : -c, n = j < g.ny - 1 ? double(x[e + w]) : -c;
    return (2.0 * c - l - r) * g.ihx2 + (2.0 * c - s - n) * g.ihy2;
  }
  const int f = e - g.nu, j = f / g.nx, i = f - j * g.nx;
  const double c = double(x[e]);
  const double l = i > 0 ? double(x[e - 1]) : -c, r = i < g.nx - 1 ? double(x[e + 1]) : -c;
  const double s = j > 0 ? double(x[e - g.nx]) : 0.0, n = j < g.ny - 2 ? double(x[e + g.nx]) : 0.0;
  return (2.0 * c - l - r) * g.ihx2 + (2.0 * c - s - n) * g.ihy2;
}

// (D x) at cell (j, i) (kernels.py:46-87).
template <typename In>
__device__ __forceinline__ double D_at(const In* x, const GridDev& g, int j, int i) {
  double v = 0.0;
  if (i < g.nx - 1) v += double(x[j * (g.nx - 1) + i]) * g.ihx;
  if (i > 0) v -= double(x[j * (g.nx - 1) + i - 1]) * g.ihx;
  if (j < g.ny - 1) v += double(x[g.nu + j * g.nx + i]) * g.ihy;
  if (j > 0) v -= double(x[g.nu + (j - 1) * g.nx + i]) * g.ihy;
  return v;
}

// (D x) at cell (j, i) computed in T (the FP32 path stays off the FP64 units).
template <typename T, typename In>
__device__ __forceinline__ T D_atT(const In* x, const GridDev& g, int j, int i, T ihx, T ihy) {
  T v = T(0);
  if (i < g.nx - 1) v += T(x[j * (g.nx - 1) + i]) * ihx;
  if (i > 0) v -= T(x[j * (g.nx - 1) + i - 1]) * ihx;
  if (j < g.ny - 1) v += T(x[g.nu + j * g.nx + i]) * ihy;
  if (j > 0) v -= T(x[g.nu + (j - 1) * g.nx + i]) * ihy;
  return v;
}

// (D^T p) at packed face e (kernels.py:89-132).
template <typename In>
__device__ __forceinline__ double Dt_at(const In* p, const GridDev& g, int e) {
  if (e < g.nu) {
    const int w = g.nx - 1, j = e / w, i = e - j * w;
    const int l = j * g.nx + i;
    return (double(p[l]) - double(p[l + 1])) * g.ihx;
  }
  const int f = e - g.nu, j = f / g.nx, i = f - j * g.nx;
  const int l = j * g.nx + i;
  return (double(p[l]) - double(p[l + g.nx])) * g.ihy;
}

// Skew-symmetric dual-cell convection at packed face e (kernels.py:6-35).
__device__ __forceinline__ double conv_at(const double* x, const GridDev& g, int e) {
  if (e < g.nu) {
    const int w = g.nx - 1, j = e / w, I = e - j * w + 1;
    const double uc = U(x, g, j, I);
    const double ue = U(x, g, j, I + 1), uw = U(x, g, j, I - 1);
    const double un = j < g.ny - 1 ? U(x, g, j + 1, I) : -uc;
    const double us = j > 0 ? U(x, g, j - 1, I) : -uc;
    const double fe = 0.5 * (uc + ue), fw = 0.5 * (uc + uw);
    const double fn = 0.5 * (V(x, g, j + 1, I - 1) + V(x, g, j + 1, I));
    const double fs = 0.5 * (V(x, g, j, I - 1) + V(x, g, j, I));
    double r = (fe * fe - fw * fw) * g.ihx + (fn * 0.5 * (uc + un) - fs * 0.5 * (uc + us)) * g.ihy;
    r -= 0.5 * uc * ((fe - fw) * g.ihx + (fn - fs) * g.ihy);
    return r;
  }
  const int f = e - g.nu, J = f / g.nx + 1, i = f - (J - 1) * g.nx;
  const double vc = V(x, g, J, i);
  const double vn = V(x, g, J + 1, i), vs = V(x, g, J - 1, i);
  const double ve = i < g.nx - 1 ? V(x, g, J, i + 1) : -vc;
  const double vw = i > 0 ? V(x, g, J, i - 1) : -vc;
  const double ge = 0.5 * (U(x, g, J - 1, i + 1) + U(x, g, J, i + 1));
  const double gw = 0.5 * (U(x, g, J - 1, i) + U(x, g, J, i));
  const double gn = 0.5 * (vc + vn), gs = 0.5 * (vc + vs);
  double r = (ge * 0.5 * (vc + ve) - gw * 0.5 * (vc + vw)) * g.ihx + (gn * gn - gs * gs) * g.ihy;
  r -= 0.5 * vc * ((ge - gw) * g.ihx + (gn - gs) * g.ihy);
  return r;
}

// The same convection in double-float arithmetic on the FP32 pipe (about 48
// bits; no FP64 instruction but the final hi + lo).  The FP32-bulk form uses
// it: GB300 runs FP64 at about 1/70 of FP32, and conv_at issues about 35 FP64
// operations per face.
__device__ __forceinline__ df32 df_half(df32 a) { return {0.5f * a.hi, 0.5f * a.lo}; }
__device__ __forceinline__ df32 U_df(const double* x, const GridDev& g, int j, int I) {
  return (I <= 0 || I >= g.nx) ? df32{0.0f, 0.0f} : d2df(x[j * (g.nx - 1) + I - 1]);
}
__device__ __forceinline__ df32 V_df(const double* x, const GridDev& g, int J, int i) {
  return (J <= 0 || J >= g.ny) ? df32{0.0f, 0.0f} : d2df(x[g.nu + (J - 1) * g.nx + i]);
}
__device__ __forceinline__ double conv_at_df(const double* x, const GridDev& g, int e, df32 ihx, df32 ihy) {
  df32 r;
  if (e < g.nu) {
    const int w = g.nx - 1, j = e / w, I = e - j * w + 1;
    const df32 uc = U_df(x, g, j, I);
    const df32 ue = U_df(x, g, j, I + 1), uw = U_df(x, g, j, I - 1);
    const df32 un = j < g.ny - 1 ? U_df(x, g, j + 1, I) : df_neg(uc);
    const df32 us = j > 0 ? U_df(x, g, j - 1, I) : df_neg(uc);
    const df32 fe = df_half(df_add(uc, ue)), fw = df_half(df_add(uc, uw));
    const df32 fn = df_half(df_add(V_df(x, g, j + 1, I - 1), V_df(x, g, j + 1, I)));
    const df32 fs = df_half(df_add(V_df(x, g, j, I - 1), V_df(x, g, j, I)));
    r = df_add(df_mul(df_sub(df_mul(fe, fe), df_mul(fw, fw)), ihx),
               df_mul(df_sub(df_mul(fn, df_half(df_add(uc, un))), df_mul(fs, df_half(df_add(uc, us)))), ihy));
    r = df_sub(r, df_mul(df_half(uc), df_add(df_mul(df_sub(fe, fw), ihx), df_mul(df_sub(fn, fs), ihy))));
  } else {
    const int f = e - g.nu, J = f / g.nx + 1, i = f - (J - 1) * g.nx;
    const df32 vc = V_df(x, g, J, i);
    const df32 vn = V_df(x, g, J + 1, i), vs = V_df(x, g, J - 1, i);
    const df32 ve = i < g.nx - 1 ? V_df(x, g, J, i + 1) : df_neg(vc);
    const df32 vw = i > 0 ? V_df(x, g, J, i - 1) : df_neg(vc);
    const df32 ge = df_half(df_add(U_df(x, g, J - 1, i + 1), U_df(x, g, J, i + 1)));
    const df32 gw = df_half(df_add(U_df(x, g, J - 1, i), U_df(x, g, J, i)));
    const df32 gn = df_half(df_add(vc, vn)), gs = df_half(df_add(vc, vs));
    r = df_add(df_mul(df_sub(df_mul(ge, df_half(df_add(vc, ve))), df_mul(gw, df_half(df_add(vc, vw)))), ihx),
               df_mul(df_sub(df_mul(gn, gn), df_mul(gs, gs)), ihy));
    r = df_sub(r, df_mul(df_half(vc), df_add(df_mul(df_sub(ge, gw), ihx), df_mul(df_sub(gn, gs), ihy))));
  }
  return f2d_bits(r.hi) + f2d_bits(r.lo);
}

}  // namespace macsav
