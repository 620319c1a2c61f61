// Whole mr-SAV / plain IMEX-SDIRK time step on the device.
//
// Restates SDIRK2MRSAV (solver/schemes/sdirk2_mrsav.py:15-75), SDIRK3MRSAV
// (solver/schemes/sdirk3_mrsav.py:11-65), IMEXEulerMRSAV
// (solver/schemes/imex_euler_mrsav.py:11-53) and the plain SDIRK2 / SDIRK3 /
// IMEXEuler schemes (sdirk2.py:17-43, sdirk3.py:31-57, imex_euler.py:10-32)
// over the MAC model seam (solver/mac_ns.py:12-107).  Every scalar of a stage
// (alpha, beta, the frozen-factor map Phi, the residuals and gates) is
// computed on the device, so a whole step is one stream of launches (or one
// CUDA graph) with a single read-back of the stage records at the end.
//
// Coefficients that depend on dt, nu and gamma are written by the host into a
// device table before each step; kernels read them by index, so a captured
// graph stays valid when dt changes.
#include <cmath>
#include <cstring>
#include <vector>

#include "step.cuh"

namespace macsav {

int enqueue_solve_fp64(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres, bool close);
int enqueue_solve_mixed(Plan* P, Exec& X, const double* f, int cols, double* vel, double* pres, bool close);
int enqueue_close(Plan* P, Exec& X, const double* f, const double* vel, double* pres, int cols, cudaEvent_t centred);

namespace {

constexpr double kEta = 1.0 - 0.70710678118654752440;    // sdirk2.py:14, 1 - 1/sqrt(2)
constexpr double kDelta = -0.70710678118654752440;       // sdirk2.py:15, -1/sqrt(2)
const double kD3[4][4] = {{1. / 4, 0, 0, 0}, {3. / 10, 1. / 4, 0, 0}, {-31. / 220, 1. / 11, 1. / 4, 0},
                          {31. / 198, 5. / 132, -4. / 9, 1. / 4}};                       // sdirk3.py:8-9
const double kDH3[4][4] = {{1. / 4, 0, 0, 0}, {-33. / 50, 121. / 100, 0, 0}, {239. / 400, -71. / 100, 5. / 16, 0},
                           {-1. / 48, -17. / 66, 235. / 528, -1. / 6}};                  // sdirk3.py:10-12

// ------------------------------------------------------------- kernels ---
// Every kernel serves all M members of the plan at once (an ensemble of
// equal-shape cavities, M = 1 for a single cavity): member m is blockIdx.y
// (or blockIdx.x for the one-block scalar kernels) and reads its copy of each
// array at base + m * stride (MemberStrides), its coefficient table at coef +
// m * kCoefStride, its stage records at recs + m * kRecStride and its block
// partials at partial + m * kPartStride.
constexpr int kCoefStride = 256;
constexpr int kRecStride = 4;  // stage records per member
constexpr long long kPartStride = 16384;  // per-member partial region (doubles)
constexpr long long kPartNu = 8192;       // <N,U> partials within the region
constexpr long long kPartEmb = 4096;      // embedded-error partials within the region

// out[k] = sum_t coef[idx[k][t]] * src[k][t]  for two outputs (rhs and the
// convection combination); partial slots: max|out0|, max|out1|, sum out1^2.
__global__ void __launch_bounds__(kThreads) k_combine2(CombineArgs a, const double* coef, long long n,
                                                       double* partial) {
  pdl_wait();
  __shared__ double red[6 * 32];
  __shared__ unsigned long long redk[2 * 32];
  const int mem = blockIdx.y;
  coef += mem * kCoefStride;
  partial += mem * kPartStride;
  unsigned long long m[2] = {0ull, 0ull};  // abs_key maxima: integer pipe, NaN propagates
  double s[1] = {0.0};
  // pairs of elements on 16-byte vectors when every array allows (the same
  // arithmetic per element, twice the bytes per load of this streaming loop)
  bool vec = (n & 1) == 0 && (a.ostr & 1) == 0;
  for (int o = 0; o < a.nout && vec; ++o) {
    vec = (reinterpret_cast<unsigned long long>(a.out[o]) & 15) == 0;
    for (int t = 0; t < a.nterm[o]; ++t)
      if (a.src[o][t]) vec = vec && (a.sstr[o][t] & 1) == 0 && (reinterpret_cast<unsigned long long>(a.src[o][t]) & 15) == 0;
  }
  const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (vec) {
    for (long long i2 = t0; i2 < (n >> 1); i2 += stride) {
      for (int o = 0; o < a.nout; ++o) {
        double a0 = 0.0, a1 = 0.0;
        for (int t = 0; t < a.nterm[o]; ++t) {
          const double* src = a.src[o][t];
          if (src) {
            const double cf = coef[a.idx[o][t]];
            const double2 v = reinterpret_cast<const double2*>(src + mem * a.sstr[o][t])[i2];
            a0 += cf * v.x;
            a1 += cf * v.y;
          }
        }
        reinterpret_cast<double2*>(a.out[o] + mem * a.ostr)[i2] = make_double2(a0, a1);
        m[o] = max(m[o], max(abs_key(a0), abs_key(a1)));
        if (o == 1) {
          s[0] += a0 * a0;
          s[0] += a1 * a1;
        }
      }
    }
  } else {
    for (long long i = t0; i < n; i += stride) {
      for (int o = 0; o < a.nout; ++o) {
        double acc = 0.0;
        for (int t = 0; t < a.nterm[o]; ++t) {
          const double* src = a.src[o][t];
          if (src) acc += coef[a.idx[o][t]] * src[mem * a.sstr[o][t] + i];
        }
        a.out[o][mem * a.ostr + i] = acc;
        m[o] = max(m[o], abs_key(acc));
        if (o == 1) s[0] += acc * acc;
      }
    }
  }
  block_max_key<2>(m, redk);
  block_sum<1>(s, red);
  if (threadIdx.x == 0) {
    unsigned long long* o = reinterpret_cast<unsigned long long*>(partial + blockIdx.x * 3);
    o[0] = m[0];
    o[1] = m[1];
    partial[blockIdx.x * 3 + 2] = s[0];
  }
}

// Partial sums of <N,V>, <N,W>, <W,W> with V, W the two Stokes columns.
__global__ void __launch_bounds__(kThreads) k_dots3(const double* N, const double* V, long long n, long long vstr,
                                                    double* partial) {
  pdl_wait();
  __shared__ double red[6 * 32];
  const int mem = blockIdx.y;
  N += mem * vstr;
  V += mem * vstr;
  const double* W = V + n;
  partial += mem * kPartStride;
  double s[3] = {0, 0, 0};
  const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const bool vec = (n & 1) == 0 && ((reinterpret_cast<unsigned long long>(N) | reinterpret_cast<unsigned long long>(V)) & 15) == 0;
  if (vec) {  // pairs on 16-byte vectors
    const double2* N2 = reinterpret_cast<const double2*>(N);
    const double2* V2 = reinterpret_cast<const double2*>(V);
    const double2* W2 = reinterpret_cast<const double2*>(W);
    for (long long i = t0; i < (n >> 1); i += stride) {
      const double2 nv = N2[i], v = V2[i], w = W2[i];
      s[0] += nv.x * v.x;
      s[1] += nv.x * w.x;
      s[2] += w.x * w.x;
      s[0] += nv.y * v.y;
      s[1] += nv.y * w.y;
      s[2] += w.y * w.y;
    }
  } else {
    for (long long i = t0; i < n; i += stride) {
      const double nv = N[i], w = W[i];
      s[0] += nv * V[i];
      s[1] += nv * w;
      s[2] += w * w;
    }
  }
  block_sum<3>(s, red);
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) partial[blockIdx.x * 3 + k] = s[k];
}

// Member strides (elements) of the step arrays.
struct MemberStrides {
  long long X, KU, NN, F, VW, PI, PS;
};

// U = V - dt*coupling*W ; pi = piV/dt - coupling*piW ; partial <N,U>.
// Plain schemes (sav == 0): U = V, pi = piV/dt.
__global__ void __launch_bounds__(kThreads) k_recombine(GridDev g, const double* VW, const double* PI,
                                                        const double* N, double* U, double* pi, const StageRec* rec,
                                                        const double* coef, int dt_idx, int sav, double* partial,
                                                        MemberStrides ms) {
  pdl_wait();
  __shared__ double red[64];
  const int mem = blockIdx.y;
  VW += mem * ms.VW;
  PI += mem * ms.PI;
  N += mem * ms.F;
  U += mem * ms.X;
  pi += mem * ms.PS;
  rec += mem * kRecStride;
  coef += mem * kCoefStride;
  partial += mem * kPartStride;
  const double dt = coef[dt_idx];
  const double cpl = sav ? rec->coupling : 0.0;
  const double resp = dt * cpl;
  double s[1] = {0.0};
  const long long stride = (long long)gridDim.x * blockDim.x, t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const unsigned long long ptrs = reinterpret_cast<unsigned long long>(VW) | reinterpret_cast<unsigned long long>(PI) |
                                  reinterpret_cast<unsigned long long>(N) | reinterpret_cast<unsigned long long>(U) |
                                  reinterpret_cast<unsigned long long>(pi);
  if ((g.size & 1) == 0 && (g.np & 1) == 0 && (ptrs & 15) == 0) {  // pairs on 16-byte vectors
    const double2* V2 = reinterpret_cast<const double2*>(VW);
    const double2* W2 = reinterpret_cast<const double2*>(VW + g.size);
    const double2* N2 = reinterpret_cast<const double2*>(N);
    double2* U2 = reinterpret_cast<double2*>(U);
    for (long long i = t0; i < (g.size >> 1); i += stride) {
      const double2 v = V2[i];
      double2 u = v;
      if (sav) {
        const double2 w = W2[i], nn = N2[i];
        u = make_double2(v.x - resp * w.x, v.y - resp * w.y);
        s[0] += nn.x * u.x;
        s[0] += nn.y * u.y;
      }
      U2[i] = u;
    }
    const double2* P2 = reinterpret_cast<const double2*>(PI);
    const double2* Q2 = reinterpret_cast<const double2*>(PI + g.np);
    double2* pi2 = reinterpret_cast<double2*>(pi);
    for (long long i = t0; i < (g.np >> 1); i += stride) {
      const double2 a = P2[i];
      if (sav) {
        const double2 b = Q2[i];
        pi2[i] = make_double2(a.x / dt - cpl * b.x, a.y / dt - cpl * b.y);
      } else {
        pi2[i] = make_double2(a.x / dt, a.y / dt);
      }
    }
  } else {
    const int n = g.size > g.np ? g.size : g.np;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      if (i < g.size) {
        const double u = sav ? VW[i] - resp * VW[g.size + i] : VW[i];
        U[i] = u;
        if (sav) s[0] += N[i] * u;
      }
      if (i < g.np) pi[i] = sav ? PI[i] / dt - cpl * PI[g.np + i] : PI[i] / dt;
    }
  }
  block_sum<1>(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

// KU and the stage momentum defect (sdirk3_mrsav.py:107-110):
// defect = U + kappa K U + dt G pi - rhs + dt*coupling*N,  G = -D^T.
// Partial slots: max|defect|, max|U|, max|D U|, max|pi|.
__global__ void __launch_bounds__(kThreads) k_stage_defect(GridDev g, const double* U, const double* pi,
                                                           const double* rhs, double* KU, const StageRec* rec,
                                                           const double* coef, int dt_idx, int kappa_idx, int sav,
                                                           double* partial, MemberStrides ms) {
  pdl_wait();
  __shared__ unsigned long long redk[4 * 32];
  const int mem = blockIdx.y;
  U += mem * ms.X;
  pi += mem * ms.PS;
  rhs += mem * ms.F;
  const double* N = rhs + g.size;
  KU += mem * ms.KU;
  rec += mem * kRecStride;
  coef += mem * kCoefStride;
  partial += mem * kPartStride;
  const double dt = coef[dt_idx], kappa = coef[kappa_idx];
  const double dtc = sav ? dt * rec->coupling : 0.0;
  unsigned long long m[4] = {0, 0, 0, 0};  // abs_key maxima
  const int n = g.size > g.np ? g.size : g.np;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i < g.size) {
      const double u = U[i];
      const double ku = K_at(U, g, i);
      KU[i] = ku;
      double d = u + kappa * ku;
      d = d - dt * Dt_at(pi, g, i);
      d = d - rhs[i];
      if (sav) d = d + dtc * N[i];
      m[0] = max(m[0], abs_key(d));
      m[1] = max(m[1], abs_key(u));
    }
    if (i < g.np) {
      const int j = i / g.nx, k = i - j * g.nx;
      m[2] = max(m[2], abs_key(D_at(U, g, j, k)));
      m[3] = max(m[3], abs_key(pi[i]));
    }
  }
  block_max_key<4>(m, redk);
  if (threadIdx.x == 0) {
    unsigned long long* o = reinterpret_cast<unsigned long long*>(partial + blockIdx.x * 4);
    for (int k = 0; k < 4; ++k) o[k] = m[k];
  }
}

// Skew convection of every member's stage velocity (kernels.py:6-35); DF:
// in double-float arithmetic on the FP32 pipe (the FP32-bulk form; the FP64
// path keeps conv_at in FP64).
template <bool DF>
__global__ void k_conv_members(GridDev g, const double* x, long long xstr, double* out, long long ostr) {
  pdl_wait();
  const int mem = blockIdx.y;
  x += mem * xstr;
  out += mem * ostr;
  if constexpr (DF) {
    const df32 ihx = d2df(g.ihx), ihy = d2df(g.ihy);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.size; e += gridDim.x * blockDim.x)
      out[e] = conv_at_df(x, g, e, ihx, ihy);
  } else {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.size; e += gridDim.x * blockDim.x)
      out[e] = conv_at(x, g, e);
  }
}

__device__ double fold_sum(const double* partial, int nb, int K, int k, double* red) {
  double s[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s[0] += partial[b * K + k];
  block_sum<1>(s, red);
  return s[0];
}
// Maximum of abs_key partials (slot k of K per block), as a double.
__device__ double fold_max(const double* partial, int nb, int K, int k, double* red) {
  unsigned long long* redk = reinterpret_cast<unsigned long long*>(red);
  unsigned long long m[1] = {0ull};
  const unsigned long long* p = reinterpret_cast<const unsigned long long*>(partial);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) m[0] = max(m[0], p[b * K + k]);
  block_max_key<1>(m, redk);
  return key_value(m[0]);
}

// Stokes outcome of the stage: residual / divergence over the member's
// columns (tensor_stokes.py:338-351) and the iteration counts; thread = member.
__global__ void k_stage_stokes(const SolveChecks* checks, const CGScalars* cg, int cols, int members, double tol,
                               StageRec* recs_i) {
  pdl_wait();
  const int mem = threadIdx.x;
  if (mem >= members) return;
  StageRec* rec = recs_i + mem * kRecStride;
  double md = 0, mf = 0, mu = 0, mdiv = 0;
  int bad_rhs = 0, bad_sol = 0, info = 0;
  for (int k = 0; k < cols; ++k) {
    const int c = mem * cols + k;
    md = nanmax(md, checks[c].max_defect);
    mf = nanmax(mf, checks[c].max_force);
    mu = nanmax(mu, checks[c].max_velocity);
    mdiv = nanmax(mdiv, checks[c].max_div);
    bad_rhs |= checks[c].nonfinite_force;
    bad_sol |= checks[c].nonfinite_solution;
    rec->iters[k] = cg[c].iters;
    if (!info && cg[c].info) info = cg[c].info;
  }
  const double res = md / (1.0 + mf);
  rec->stokes_residual = res;
  rec->stokes_divergence = mdiv;
  rec->cg_info = info;
  if (rec->status) return;
  if (bad_rhs) rec->status = ST_STOKES_RHS;
  else if (info) rec->status = ST_CG;
  else if (bad_sol || res > tol || mdiv > tol * (1.0 + mu)) rec->status = ST_STOKES_GATE;
}

// The frozen SAV scalar map for one stage (scalar_correction.py:29-52 and the
// alpha/beta guard of sdirk3_mrsav.py:92-100); one block per member.
__global__ void __launch_bounds__(kThreads) k_stage_sav(const double* partial, int nb, StageRec* recs, int stage,
                                                        const double* coef, SavIdx ix, double area) {
  pdl_wait();
  __shared__ double red[64];
  const int mem = blockIdx.x;
  partial += mem * kPartStride;
  recs += mem * kRecStride;
  coef += mem * kCoefStride;
  const double nv = fold_sum(partial, nb, 3, 0, red);
  const double nw = fold_sum(partial, nb, 3, 1, red);
  const double ww = fold_sum(partial, nb, 3, 2, red);
  if (threadIdx.x != 0) return;
  StageRec& R = recs[stage];
  const double dt = coef[ix.dt], d = coef[ix.d], r0 = coef[ix.r0];
  // predictor and scalar right-hand side from earlier stages' r (r_0 = r0)
  auto rval = [&](int k) { return k == 0 ? r0 : recs[k - 1].r; };
  const double predictor = rval(ix.pred);
  double srhs = 0.0;
  for (int t = 0; t < ix.nsr; ++t) srhs += coef[ix.sr_coef[t]] * rval(ix.sr_r[t]);
  R.scalar_rhs = srhs;
  R.predictor = predictor;
  const double alpha = area * nv;  // + lifting work, zero for MAC
  double beta = area * nw;
  R.alpha = alpha;
  // statuses set before the Stokes solve stop here; the solve's own status
  // (k_stage_stokes, on the side stream) may still be unset, so this kernel
  // records its failures in sav_status and k_stage_close merges them
  if (R.status) return;
  if (beta < 0.0) {
    const double scale = sqrt(area * R.nn * area * ww);  // Momentum.cauchy_scale
    if (beta < -1e-12 * (1.0 + scale)) {
      R.sav_status = ST_NEG_ENERGY;
      return;
    }
  }
  beta = beta > 0.0 ? beta : 0.0;
  R.beta = beta;
  const int order = ix.order;
  if (!isfinite(predictor) || !isfinite(dt) || !isfinite(d) || !isfinite(srhs) || !isfinite(alpha) ||
      !isfinite(beta) || dt <= 0 || d <= 0) {
    R.sav_status = ST_SAV_INPUT;
    return;
  }
  double z = predictor, c = 1.0;
  const int count = order == 3 ? 2 : 1;
  for (int it = 0; it < count; ++it) {
    c = order == 1 ? 1.0 : (order == 2 ? 1.0 + z : 1.0 + z + z * z);
    const double resp = dt * dt * c * c * beta;
    const double den = d + resp;
    if (!isfinite(den) || den <= 0) {
      R.sav_status = ST_SAV_DENOM;
      return;
    }
    z = (srhs - dt * c * alpha + resp) / den;
    if (!isfinite(z)) {
      R.sav_status = ST_SAV_NONFINITE;
      return;
    }
    R.corr[it] = z;
  }
  R.n_corr = count;
  R.factor = c;
  R.r = z;
  R.coupling = c * (1.0 - z);
}

// Closing scalar checks of the stage (sdirk3_mrsav.py:105-114); one block per
// member.  gate: 1 = the stage defect gate (mr-SAV schemes, IMEX Euler);
// 0 = none (plain SDIRK2/3 report the Stokes residual, sdirk3.py:52-55).
__global__ void __launch_bounds__(kThreads) k_stage_close(const double* partial, int nbd, int nbn, StageRec* recs,
                                                          int stage, const double* coef, SavIdx ix, double area,
                                                          int sav, int gate) {
  pdl_wait();
  __shared__ double red[64];
  const int mem = blockIdx.x;
  partial += mem * kPartStride;
  recs += mem * kRecStride;
  coef += mem * kCoefStride;
  const double maxdef = fold_max(partial, nbd, 4, 0, red);
  const double maxu = fold_max(partial, nbd, 4, 1, red);
  const double maxdiv = fold_max(partial, nbd, 4, 2, red);
  const double maxpi = fold_max(partial, nbd, 4, 3, red);
  const double nu_dot = sav ? fold_sum(partial + kPartNu, nbn, 1, 0, red) : 0.0;
  if (threadIdx.x != 0) return;
  StageRec& R = recs[stage];
  if (!R.status && R.sav_status) R.status = R.sav_status;  // a Stokes failure comes first
  const double dt = coef[ix.dt];
  R.max_velocity = maxu;
  R.divergence = maxdiv;
  R.max_pressure = maxpi;
  double denom = 1.0 + R.max_rhs;
  if (sav) {
    const double scalar = coef[ix.d] * R.r - R.scalar_rhs + dt * R.factor * (area * nu_dot);
    R.scalar_residual = fabs(scalar) / (1.0 + fabs(R.scalar_rhs) + fabs(R.r));
    denom += dt * fabs(R.coupling) * R.max_conv;
  } else {
    R.scalar_residual = 0.0;
  }
  R.residual = gate ? maxdef / denom : R.stokes_residual;
  if (R.status || !gate) return;
  const bool finite = isfinite(R.residual) && isfinite(R.scalar_residual) && isfinite(maxdiv) && isfinite(maxu) &&
                      isfinite(maxpi);
  if (!finite || R.residual > 1e-8 || R.scalar_residual > 1e-8 || maxdiv > 1e-8 * (1.0 + maxu))
    R.status = ST_STAGE_GATE;
}

// one block per member
__global__ void k_fold_combine(const double* partial, int nb, StageRec* recs_i) {
  pdl_wait();
  __shared__ double red[64];
  const int mem = blockIdx.x;
  partial += mem * kPartStride;
  const double m0 = fold_max(partial, nb, 3, 0, red);
  const double m1 = fold_max(partial, nb, 3, 1, red);
  const double s2 = fold_sum(partial, nb, 3, 2, red);
  if (threadIdx.x == 0) {
    StageRec* rec = recs_i + mem * kRecStride;
    rec->max_rhs = m0;
    rec->max_conv = m1;
    rec->nn = s2;
  }
}

// shifts of every member's Stokes columns: mass 1, viscosity kappa (member's table)
__global__ void k_set_shift(double* shift, const double* coef, int kappa_idx, int cols, int total) {
  pdl_wait();
  const int c = threadIdx.x;
  if (c < total) {
    shift[2 * c] = 1.0;
    shift[2 * c + 1] = coef[(c / cols) * kCoefStride + kappa_idx];
  }
}

// Embedded-error inner products of a step (controller.py:112-123 needs
// <x1-emb, x1-emb>, <x0, x0>, <x1, x1> with the grid weight hx*hy) and a
// non-finite flag of emb, folded per member by the last block into
// out[4m .. 4m+3].
struct EmbFin {
  const double* partial;
  int nb, members;
  double w;
  double* out;
  __device__ void operator()() const {
    __shared__ double red[3 * 32];
    for (int mem = 0; mem < members; ++mem) {
      const double* p = partial + mem * kPartStride;
      double s[3] = {0.0, 0.0, 0.0};
      int bad = 0;
      for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        for (int k = 0; k < 3; ++k) s[k] += __ldcg(p + b * 4 + k);
        bad |= __ldcg(p + b * 4 + 3) != 0.0;
      }
      bad = __syncthreads_or(bad);
      block_sum<3>(s, red);
      if (threadIdx.x == 0) {
        out[4 * mem + 0] = w * s[0];
        out[4 * mem + 1] = w * s[1];
        out[4 * mem + 2] = w * s[2];
        out[4 * mem + 3] = bad ? 1.0 : 0.0;
      }
      __syncthreads();
    }
  }
};
__global__ void __launch_bounds__(kThreads) k_emb_norms(const double* X, long long xstr, long long last,
                                                        const double* emb, long long n, double* partial, EmbFin fin,
                                                        unsigned int* done) {
  pdl_wait();
  __shared__ double red[3 * 32];
  constexpr unsigned long long kInf = 0x7ff0000000000000ull;
  const int mem = blockIdx.y;
  const double* x0 = X + mem * xstr;
  const double* x1 = x0 + last;
  emb += mem * n;
  double* part = partial + mem * kPartStride;
  double s[3] = {0.0, 0.0, 0.0};
  int bad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = x0[i], b = x1[i], e = emb[i];
    const double d = b - e;
    s[0] += d * d;
    s[1] += a * a;
    s[2] += b * b;
    bad |= abs_key(e) >= kInf;
  }
  bad = __syncthreads_or(bad);
  block_sum<3>(s, red);
  if (threadIdx.x == 0) {
    double* o = part + blockIdx.x * 4;
    o[0] = s[0];
    o[1] = s[1];
    o[2] = s[2];
    o[3] = bad ? 1.0 : 0.0;
  }
  last_block_finish(fin, done);
}

__global__ void k_clear_recs(StageRec* recs, int n) {
  pdl_wait();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    StageRec z;
    memset(&z, 0, sizeof(z));
    recs[i] = z;
  }
}

// ---------------------------------------------- device-resident adaptive run ---
// State of an adaptive run on the device: the accepted time, SAV scalar and
// proposed step, the attempt in flight and the counters.  status: 0 running,
// 1 complete, 2 failed.
struct AdaptState {
  double t, end, dt, r, prev_err;  // prev_err < 0: no accepted attempt yet
  double h;                        // step of the attempt in flight
  int last, copy, accepted, attempts, rejections, status, reason, hist_cap, max_attempts;
};

// Step-factor arithmetic of the reference's controllers (controller.py:14-70).
__device__ double adapt_elementary(const macsav_step_control& c, double err) {
  if (err == 0.0) return c.max_factor;
  return fmin(fmax(c.safety * pow(err, -1.0 / c.order), c.min_factor), c.max_factor);
}
__device__ double adapt_grow(const macsav_step_control& c, double err, double prev) {
  if (c.proportional <= 0.0 || prev < 0.0) return adapt_elementary(c, err);
  const double f = c.safety * pow(fmax(err, c.error_floor), -c.proportional / c.order) *
                   pow(fmax(prev, c.error_floor), c.integral / c.order);
  return fmin(fmax(f, c.min_factor), c.max_factor);
}

// Head of an attempt: h = min(dt, end - t) and the step's coefficient table
// for h (every slot is c0 + c1 h; the SAV scalar's slot is the accepted r).
__global__ void k_adapt_begin(AdaptState* st, const double* c0, const double* c1, int ncoef, int r0_idx,
                              double* coef) {
  pdl_wait();
  const double rem = st->end - st->t;
  const double h = fmin(st->dt, rem);
  for (int i = threadIdx.x; i < ncoef; i += blockDim.x) coef[i] = i == r0_idx ? st->r : c0[i] + c1[i] * h;
  if (threadIdx.x == 0) {
    st->h = h;
    st->last = h == rem;
  }
}

// Decision on the attempt (the reference driver's loop body,
// controller.py:244-327): the scaled embedded error, accept or reject, the
// next step, the history record, and the WHILE node's condition.
__global__ void k_adapt_control(AdaptState* st, const macsav_step_control* ctl, const double* enorm,
                                const StageRec* recs, int nstages, int sav, macsav_adaptive_attempt* hist,
                                cudaGraphConditionalHandle cond) {
  pdl_wait();
  if (threadIdx.x != 0) return;
  const macsav_step_control c = *ctl;
  const double h = st->h;
  int stage_status = 0;
  for (int i = 0; i < nstages; ++i)
    if (recs[i].status && !stage_status) stage_status = recs[i].status;
  const double r1 = sav ? recs[nstages - 1].r : 0.0;
  double err = INFINITY;
  int reason = 0;
  if (stage_status) {
    reason = 4;
  } else {
    const double d = enorm[0], o = enorm[1], n = enorm[2];
    if (enorm[3] != 0.0 || !isfinite(n) || !isfinite(r1)) {
      reason = 3;
    } else {
      if (isfinite(d) && d >= 0.0 && isfinite(o) && o >= 0.0 && n >= 0.0)
        err = sqrt(d) / (c.atol + c.rtol * fmax(sqrt(o), sqrt(n)));
      reason = !isfinite(err) ? 2 : (err > 1.0 ? 1 : 0);
    }
  }
  const double factor = reason ? fmin(adapt_elementary(c, err), 0.8) : adapt_grow(c, err, st->prev_err);
  if (st->attempts < st->hist_cap) {
    macsav_adaptive_attempt a;
    a.t = st->t;
    a.step = h;
    a.error = err;
    a.factor = factor;
    a.accepted = reason == 0;
    a.reason = reason;
    a.stage_status = stage_status;
    a.pad = 0;
    hist[st->attempts] = a;
  }
  ++st->attempts;
  st->copy = 0;
  if (reason) {
    ++st->rejections;
    st->dt = h * factor;
    if (st->rejections > c.max_rejections || st->dt < c.min_step) {
      st->status = 2;
      st->reason = reason;
    }
  } else {
    st->rejections = 0;
    st->prev_err = err;
    st->t = st->last ? st->end : st->t + h;
    st->r = r1;
    ++st->accepted;
    st->dt = fmin(h * factor, c.max_step);
    st->copy = 1;
    if (!(st->t < st->end)) st->status = 1;
  }
  if (st->status == 0) {  // the checks at the head of the reference's loop, for the next attempt
    const double rem = st->end - st->t, hn = fmin(st->dt, rem);
    if (st->accepted >= c.max_steps) {
      st->status = 2;
      st->reason = 6;
    } else if (hn < c.min_step && hn != rem) {
      st->status = 2;
      st->reason = 5;
    } else if (st->attempts >= st->max_attempts) {
      st->status = 2;
      st->reason = reason ? reason : 6;
    }
  }
  cudaGraphSetConditional(cond, st->status == 0 ? 1u : 0u);
}

// An accepted attempt's velocity becomes the next attempt's start.
__global__ void __launch_bounds__(kThreads) k_adapt_accept(const AdaptState* st, double* X, long long src,
                                                           long long n) {
  pdl_wait();
  if (!st->copy) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    X[i] = X[src + i];
}

}  // namespace

// --------------------------------------------------------------- host side ---
static int red_nb(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

// Member-major step buffers: member m's block of each array at base + m * stride.
int step_buffers(Plan* P) {
  if (P->st.X) return MACSAV_OK;
  const size_t sz = P->g.size, np = P->g.np, M = size_t(P->members);
  StepBuffers& B = P->st;
  const size_t per = sz * (5 + 4 + 4 + 2 + 2 + 4 + 1) + np * (2 + 4) + kCoefStride;
  void* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * per * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  B.base = d;
  double* p = static_cast<double*>(d);
  B.X = p; p += 5 * sz * M;
  B.KU = p; p += 4 * sz * M;
  B.NN = p; p += 4 * sz * M;
  B.F = p; p += 2 * sz * M;
  B.VW = p; p += 2 * sz * M;
  B.FORCE = p; p += 4 * sz * M;
  B.EMB = p; p += sz * M;
  B.PI = p; p += 2 * np * M;
  B.PS = p; p += 4 * np * M;
  B.coef = p;
  if (cudaMalloc(&B.recs, sizeof(StageRec) * kRecStride * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMallocHost(&B.h_recs, sizeof(StageRec) * kRecStride * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMallocHost(&B.h_coef, sizeof(double) * kCoefStride * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMalloc(&B.enorm, sizeof(double) * 4 * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMallocHost(&B.h_enorm, sizeof(double) * 4 * M) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&B.side, cudaStreamNonBlocking) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaStreamCreateWithFlags(&B.loop, cudaStreamNonBlocking) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaEventCreateWithFlags(&B.ev_in, cudaEventDisableTiming) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaEventCreateWithFlags(&B.ev_out, cudaEventDisableTiming) != cudaSuccess) return MACSAV_ERR_CUDA;
  return MACSAV_OK;
}

void step_free(Plan* P) {
  StepBuffers& B = P->st;
  for (auto& kv : B.graphs) cudaGraphExecDestroy(kv.exec);
  B.graphs.clear();
  cudaFree(B.base);
  cudaFree(B.recs);
  cudaFreeHost(B.h_recs);
  cudaFreeHost(B.h_coef);
  cudaFree(B.enorm);
  cudaFreeHost(B.h_enorm);
  if (B.stream) cudaStreamDestroy(B.stream);
  if (B.side) cudaStreamDestroy(B.side);
  if (B.loop) cudaStreamDestroy(B.loop);
  cudaFree(B.adapt);
  if (B.ev_in) cudaEventDestroy(B.ev_in);
  if (B.ev_out) cudaEventDestroy(B.ev_out);
  B = StepBuffers{};
}

int scheme_stages(int scheme) {
  switch (scheme) {
    case MACSAV_SDIRK2_MRSAV: case MACSAV_SDIRK2: return 2;
    case MACSAV_SDIRK3_MRSAV: case MACSAV_SDIRK3: return 4;
    case MACSAV_IMEX_EULER_MRSAV: case MACSAV_IMEX_EULER: return 1;
  }
  return 0;
}
static bool scheme_sav(int scheme) {
  return scheme == MACSAV_SDIRK2_MRSAV || scheme == MACSAV_SDIRK3_MRSAV || scheme == MACSAV_IMEX_EULER_MRSAV;
}

// Host-built stage program: which vectors each combine reads, with which
// coefficient slots, plus the slot values for the current (dt, nu, gamma).
struct StageProgram {
  CombineArgs comb[4];
  SavIdx sav[4];
  int kappa[4];
  int dt_idx, r0_idx;
  int need_conv[5];    // convection at node j needed
  int emb_terms;
  int emb_idx[4];
  int emb_node[4];
  int nstages;
};

static void build_program(Plan* P, int scheme, bool has_force, double dt, double nu, double gamma, double r0,
                          StageProgram& G, double* coef) {
  StepBuffers& B = P->st;
  const long long sz = P->g.size;
  int nc = 0;
  auto slot = [&](double v) { coef[nc] = v; return nc++; };
  std::memset(&G, 0, sizeof(G));
  G.nstages = scheme_stages(scheme);
  G.dt_idx = slot(dt);
  G.r0_idx = slot(r0);
  auto U = [&](int k) { return B.X + k * sz; };
  auto KU = [&](int k) { return B.KU + k * sz; };
  auto NN = [&](int k) { return B.NN + k * sz; };
  auto FF = [&](int k) { return has_force ? B.FORCE + k * sz : (const double*)nullptr; };
  const bool sav = scheme_sav(scheme);
  // member stride of a source: stage velocities hold 5 vectors per member,
  // K U, N and the forces 4
  auto mstride = [&](const double* src) { return (src >= B.X && src < B.X + 5 * sz * P->members) ? 5 * sz : 4 * sz; };
  for (int i = 0; i < G.nstages; ++i) {
    CombineArgs& c = G.comb[i];
    c.nout = 2;
    c.out[0] = B.F;
    c.out[1] = B.F + sz;
    c.ostr = (sav ? 2 : 1) * sz;
    auto add = [&](int o, const double* src, double v) {
      const int t = c.nterm[o]++;
      c.src[o][t] = src;
      c.sstr[o][t] = src ? mstride(src) : 0;
      c.idx[o][t] = slot(v);
    };
    SavIdx& s = G.sav[i];
    if (scheme == MACSAV_SDIRK3_MRSAV || scheme == MACSAV_SDIRK3) {
      // rhs = U_i + dt*sum_j DHAT[i,j] f_j - nu*dt*sum_{j<i} D[i,j] K U_{j+1}   (sdirk3_mrsav.py:85-88)
      add(0, U(i), 1.0);
      for (int j = 0; j <= i; ++j) add(0, FF(j), dt * kDH3[i][j]);
      for (int j = 0; j < i; ++j) add(0, KU(j), -nu * dt * kD3[i][j]);
      for (int j = 0; j <= i; ++j) add(1, NN(j), kDH3[i][j]);
      if (scheme == MACSAV_SDIRK3) {  // plain: convection moves into the rhs (sdirk3.py:44-46)
        for (int j = 0; j <= i; ++j) add(0, NN(j), -dt * kDH3[i][j]);
      }
      G.kappa[i] = slot(nu * dt * kD3[i][i]);
      s.d = slot(1.0 + gamma * dt * kD3[i][i]);
      s.order = 3;
      s.pred = i;  // scalars[-1]
      s.nsr = 0;
      s.sr_r[s.nsr] = i;
      s.sr_coef[s.nsr++] = slot(1.0);
      for (int j = 0; j < i; ++j) {
        s.sr_r[s.nsr] = j + 1;
        s.sr_coef[s.nsr++] = slot(-gamma * dt * kD3[i][j]);
      }
    } else if (scheme == MACSAV_SDIRK2_MRSAV || scheme == MACSAV_SDIRK2) {
      const bool plain = scheme == MACSAV_SDIRK2;
      if (i == 0) {  // sdirk2_mrsav.py:215-216
        add(0, U(0), 1.0);
        add(0, FF(0), kEta * dt);
        add(1, NN(0), kEta);
        if (plain) add(0, NN(0), -kEta * dt);  // sdirk2.py:32
        s.pred = 0;
        s.nsr = 1;
        s.sr_r[0] = 0;
        s.sr_coef[0] = slot(1.0);
      } else {  // sdirk2_mrsav.py:218-221
        add(0, U(1), 1.0);
        add(0, KU(0), -nu * dt * (1 - 2 * kEta));
        add(0, FF(0), -dt);
        add(0, FF(1), dt * (1 - kDelta));
        add(1, NN(0), -1.0);
        add(1, NN(1), 1 - kDelta);
        if (plain) {  // sdirk2.py:36-37
          add(0, NN(0), dt);
          add(0, NN(1), -dt * (1 - kDelta));
        }
        s.pred = 1;
        s.nsr = 1;
        s.sr_r[0] = 1;
        s.sr_coef[0] = slot(1 - gamma * dt * (1 - 2 * kEta));
      }
      G.kappa[i] = slot(nu * kEta * dt);
      s.d = slot(1.0 + gamma * kEta * dt);
      s.order = 2;
    } else {  // IMEX Euler (imex_euler_mrsav.py:57-58, imex_euler.py:19)
      add(0, U(0), 1.0);
      add(0, FF(0), dt);
      add(1, NN(0), 1.0);
      if (scheme == MACSAV_IMEX_EULER) add(0, NN(0), -dt);
      G.kappa[i] = slot(nu * dt);
      s.d = slot(1.0 + gamma * dt);
      s.order = 1;
      s.pred = 0;
      s.nsr = 1;
      s.sr_r[0] = 0;
      s.sr_coef[0] = slot(1.0);
    }
    s.dt = G.dt_idx;
    s.r0 = G.r0_idx;
    (void)sav;
  }
  // convection needed at nodes 0..nstages-1
  for (int j = 0; j < G.nstages; ++j) G.need_conv[j] = 1;
  // embedded velocity (sdirk3.py:16-19; sdirk2_mrsav.py:222)
  if (G.nstages == 4) {
    const double w[4] = {2. / 3, -128. / 99, 50. / 33, 1. / 9};
    G.emb_terms = 4;
    for (int k = 0; k < 4; ++k) {
      G.emb_idx[k] = slot(w[k]);
      G.emb_node[k] = k;
    }
  } else if (G.nstages == 2) {
    G.emb_terms = 2;
    G.emb_idx[0] = slot(1.0 - 1.0 / kEta);
    G.emb_node[0] = 0;
    G.emb_idx[1] = slot(1.0 / kEta);
    G.emb_node[1] = 1;
  }
}

// Enqueue one whole step of all members on X.s reading U_0 from B.X (and
// forces from B.FORCE), writing U_n to B.X + n*size, stage pressures to B.PS
// and records to B.recs (member-major layouts, see step_buffers).
static int enqueue_step(Plan* P, Exec& X, int scheme, const StageProgram& G, bool want_emb) {
  StepBuffers& B = P->st;
  const GridDev& g = P->g;
  const long long sz = g.size, np = g.np;
  const int M = P->members;
  const cudaStream_t s = X.s;
  const int nbs = red_nb(sz), nbn = red_nb(sz > np ? sz : np);
  const bool sav = scheme_sav(scheme);
  const int cols = sav ? 2 : 1;
  const double area = g.hx * g.hy;
  const MemberStrides ms{5 * sz, 4 * sz, 4 * sz, cols * sz, cols * sz, cols * np, 4 * np};
  launch_k(k_clear_recs, 1, 128, 0, s, B.recs, kRecStride * M);
  // N(U_0)
  auto conv = P->precision == MACSAV_FP64 ? k_conv_members<false> : k_conv_members<true>;
  launch_k(conv, dim3(red_nb(sz), M), kThreads, 0, s, g, B.X, ms.X, B.NN, ms.NN);
  P->launches += 2;
  for (int i = 0; i < G.nstages; ++i) {
    StageRec* rec = B.recs + i;
    double* U = B.X + (i + 1) * sz;
    CombineArgs ca = G.comb[i];
    if (!sav) ca.nout = 1;
    launch_k(k_combine2, dim3(nbs, M), kThreads, 0, s, ca, B.coef, sz, P->partial);
    launch_k(k_fold_combine, M, kThreads, 0, s, P->partial, nbs, rec);
    launch_k(k_set_shift, 1, kMaxCols, 0, s, P->shift, B.coef, G.kappa[i], cols, cols * M);
    P->launches += 3;
    const bool fp64 = P->precision == MACSAV_FP64;
    int rc = fp64 ? enqueue_solve_fp64(P, X, B.F, cols * M, B.VW, B.PI, false)
                  : enqueue_solve_mixed(P, X, B.F, cols * M, B.VW, B.PI, false);
    if (rc != MACSAV_OK) return rc;
    // The solve's closing work (pressure centring on the mixed path, the
    // FP64 Stokes check and its stage record) on the side stream, with its
    // own partials and counter, beside the SAV algebra below: the velocity
    // is final here, the centred pressure is first needed by k_recombine
    // and the check's record by k_stage_close.  Single-cavity plans only:
    // a batched plan already fills the GPU, and with many plans in flight
    // (ensembles) the extra streams cost more than they hide (measured on
    // GB300: single cavity 512^2 -1.6% step time, 256-member ensemble +9%).
    const bool overlap = M == 1;
    {
      const cudaStream_t side = overlap ? P->aux[2] : s;
      if (overlap) {
        cudaEventRecord(P->evf[2], s);
        cudaStreamWaitEvent(side, P->evf[2], 0);
      }
      Exec Xc = X;
      Xc.s = side;
      Xc.partial = P->partial2;
      Xc.counter = P->done_counter + 8;
      enqueue_close(P, Xc, B.F, B.VW, B.PI, cols * M, fp64 || !overlap ? nullptr : P->evj[2]);
      launch_k(k_stage_stokes, 1, kMaxMembers, 0, side, P->checks, P->cg, cols, M, P->tol, rec);
      ++P->launches;
      if (overlap) cudaEventRecord(P->evc, side);
    }
    if (sav) {
      launch_k(k_dots3, dim3(nbs, M), kThreads, 0, s, B.F + sz, B.VW, sz, ms.F, P->partial);
      launch_k(k_stage_sav, M, kThreads, 0, s, P->partial, nbs, B.recs, i, B.coef, G.sav[i], area);
      P->launches += 2;
    }
    if (overlap && !fp64) cudaStreamWaitEvent(s, P->evj[2], 0);  // centred pressure
    double* pi = B.PS + i * np;
    launch_k(k_recombine, dim3(nbn, M), kThreads, 0, s, g, B.VW, B.PI, B.F + sz, U, pi, rec, B.coef, G.dt_idx, sav ? 1 : 0,
                                                   P->partial + kPartNu, ms);
    launch_k(k_stage_defect, dim3(nbn, M), kThreads, 0, s, g, U, pi, B.F, B.KU + i * sz, rec, B.coef, G.dt_idx,
                                                      G.kappa[i], sav ? 1 : 0, P->partial, ms);
    if (overlap) cudaStreamWaitEvent(s, P->evc, 0);  // Stokes check and its record
    const int gate = (scheme == MACSAV_SDIRK2 || scheme == MACSAV_SDIRK3) ? 0 : 1;
    launch_k(k_stage_close, M, kThreads, 0, s, P->partial, nbn, nbn, B.recs, i, B.coef, G.sav[i], area, sav ? 1 : 0, gate);
    P->launches += 3;
    if (i + 1 < G.nstages) {
      launch_k(conv, dim3(red_nb(sz), M), kThreads, 0, s, g, U, ms.X, B.NN + (i + 1) * sz, ms.NN);
      ++P->launches;
    }
  }
  if (want_emb && G.emb_terms) {
    CombineArgs e;
    std::memset(&e, 0, sizeof(e));
    e.nout = 1;
    e.out[0] = B.EMB;
    e.ostr = sz;
    e.nterm[0] = G.emb_terms;
    for (int k = 0; k < G.emb_terms; ++k) {
      e.src[0][k] = B.X + G.emb_node[k] * sz;
      e.sstr[0][k] = ms.X;
      e.idx[0][k] = G.emb_idx[k];
    }
    launch_k(k_combine2, dim3(nbs, M), kThreads, 0, s, e, B.coef, sz, P->partial);
    ++P->launches;
    // the adaptive controller's inner products, so an attempt needs no more
    // device round trips than the step itself
    launch_k(k_emb_norms, dim3(nbs, M), kThreads, 0, s, B.X, ms.X, G.nstages * sz, B.EMB, sz, P->partial + kPartEmb,
                                                   EmbFin{P->partial + kPartEmb, nbs, M, g.hx * g.hy, B.enorm},
                                                   P->done_counter);
    ++P->launches;
  }
  return MACSAV_OK;
}

// Enqueue one step of all members (no host wait in graph mode); finish_members
// waits for it and folds the stage records.
int enqueue_members(Plan* P, int scheme, double t, double dt, const double* nus, double gamma, const double* x0,
                    const double* r0, const double* forces, double* x1, double* embedded, double* pressures,
                    cudaStream_t user) {
  (void)t;
  int rc = step_buffers(P);
  if (rc != MACSAV_OK) return rc;
  StepBuffers& B = P->st;
  const long long sz = P->g.size, np = P->g.np;
  const int M = P->members;
  StageProgram G;
  for (int m = 0; m < M; ++m)  // the same program; per-member coefficient values
    build_program(P, scheme, forces != nullptr, dt, nus[m], gamma, r0[m], G, B.h_coef + m * kCoefStride);
  const int n = G.nstages;
  // inputs onto the plan's stream
  cudaEventRecord(B.ev_in, user);
  cudaStreamWaitEvent(B.stream, B.ev_in, 0);
  const cudaStream_t s = B.stream;
  const size_t d8 = sizeof(double);
  cudaMemcpyAsync(B.coef, B.h_coef, d8 * kCoefStride * M, cudaMemcpyHostToDevice, s);
  cudaMemcpy2DAsync(B.X, d8 * 5 * sz, x0, d8 * sz, d8 * sz, M, cudaMemcpyDeviceToDevice, s);
  if (forces) cudaMemcpy2DAsync(B.FORCE, d8 * 4 * sz, forces, d8 * n * sz, d8 * n * sz, M, cudaMemcpyDeviceToDevice, s);
  const bool want_emb = embedded != nullptr;
  if (!P->use_graph) {
    Exec X{s, false, nullptr, 0, 0.0};
    rc = enqueue_step(P, X, scheme, G, want_emb);
    if (rc != MACSAV_OK) return rc;
  } else {
    const int key = scheme * 4 + (forces ? 1 : 0) + (want_emb ? 2 : 0);
    cudaGraphExec_t exec = nullptr;
    for (auto& kv : B.graphs)
      if (kv.key == key) exec = kv.exec;
    if (!exec) {
      Exec X{s, true, B.side, 0, 0.0};
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return MACSAV_ERR_CUDA;
      rc = enqueue_step(P, X, scheme, G, want_emb);
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamEndCapture(s, &graph);
      if (rc != MACSAV_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        P->err = std::string("graph capture failed: ") + cudaGetErrorString(e);
        return MACSAV_ERR_CUDA;
      }
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        P->err = std::string("graph instantiate failed: ") + cudaGetErrorString(e);
        return MACSAV_ERR_CUDA;
      }
      B.graphs.push_back(GraphEntry{key, exec});
    }
    if (cudaGraphLaunch(exec, s) != cudaSuccess) return MACSAV_ERR_CUDA;
  }
  if (x1) cudaMemcpy2DAsync(x1, d8 * sz, B.X + n * sz, d8 * 5 * sz, d8 * sz, M, cudaMemcpyDeviceToDevice, s);
  if (want_emb && G.emb_terms) cudaMemcpyAsync(embedded, B.EMB, d8 * sz * M, cudaMemcpyDeviceToDevice, s);
  if (pressures)
    cudaMemcpy2DAsync(pressures, d8 * n * np, B.PS, d8 * 4 * np, d8 * n * np, M, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(B.h_recs, B.recs, sizeof(StageRec) * kRecStride * M, cudaMemcpyDeviceToHost, s);
  B.have_enorm = want_emb && G.emb_terms;
  if (B.have_enorm) cudaMemcpyAsync(B.h_enorm, B.enorm, d8 * 4 * M, cudaMemcpyDeviceToHost, s);
  cudaEventRecord(B.ev_out, s);
  cudaStreamWaitEvent(user, B.ev_out, 0);
  B.pending_scheme = scheme;
  B.pending_stages = n;
  return MACSAV_OK;
}

// records: [M][stages] host array; r1: M host values.  Returns the first
// failing member's stage status (ST_OK when all passed).
int finish_members(Plan* P, macsav_stage_record* records, double* r1) {
  StepBuffers& B = P->st;
  const int scheme = B.pending_scheme, n = B.pending_stages, M = P->members;
  if (n <= 0) {
    P->err = "no step enqueued";
    return MACSAV_ERR_VALUE;
  }
  B.pending_stages = 0;
  if (cudaEventSynchronize(B.ev_out) != cudaSuccess) return MACSAV_ERR_CUDA;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    P->err = std::string("CUDA: ") + cudaGetErrorString(e);
    return MACSAV_ERR_CUDA;
  }
  int status = MACSAV_OK;
  const bool sav = scheme_sav(scheme);
  for (int m = 0; m < M; ++m) {
    for (int i = 0; i < n; ++i) {
      const StageRec& R = B.h_recs[m * kRecStride + i];
      macsav_stage_record& o = records[m * n + i];
      std::memset(&o, 0, sizeof(o));
      o.r = R.r;
      o.residual = R.residual;
      o.scalar_residual = R.scalar_residual;
      o.divergence_inf = R.divergence;
      o.continuity_residual = R.divergence;
      o.correction_predictor = sav ? R.predictor : NAN;
      o.frozen_factor = sav ? R.factor : NAN;
      o.n_corrections = sav ? R.n_corr : 0;
      o.corrections[0] = R.corr[0];
      o.corrections[1] = R.corr[1];
      o.iterations[0] = R.iters[0];
      o.iterations[1] = R.iters[1];
      o.stokes_residual = R.stokes_residual;
      o.stokes_divergence = R.stokes_divergence;
      o.max_velocity = R.max_velocity;
      o.max_pressure = R.max_pressure;
      o.cg_info = R.cg_info;
      o.status = R.status;
      if (status == MACSAV_OK && R.status) status = R.status;
    }
    if (r1) r1[m] = sav ? B.h_recs[m * kRecStride + n - 1].r : 0.0;
  }
  return status;
}

int enqueue_step_async(Plan* P, int scheme, double t, double dt, double nu, double gamma, const double* x0,
                       double r0, const double* forces, double* x1, double* embedded, double* pressures,
                       cudaStream_t user) {
  if (P->members != 1) {
    P->err = "a plan with several members steps through macsav_step_members";
    return MACSAV_ERR_VALUE;
  }
  return enqueue_members(P, scheme, t, dt, &nu, gamma, x0, &r0, forces, x1, embedded, pressures, user);
}

int finish_step(Plan* P, macsav_stage_record* records, double* r1) { return finish_members(P, records, r1); }

// Device-resident adaptive run (see macsav_integrate_adaptive).  The step
// program is affine in dt, so its coefficient table is c0 + c1 dt with
// (c0, c1) from two host builds; the attempt loop is one conditional WHILE
// node whose body is [table for the attempt's step, the fused step with its
// embedded-error inner products, the decision, the copy of an accepted
// velocity], captured once per scheme.
constexpr int kAdaptHistory = 65536;  // attempts kept on the device
int run_adaptive_device(Plan* P, int scheme, double t0, double T, double dt0, double nu, double gamma,
                        const double* x0, double r0, const macsav_step_control& ctl, double* x_final,
                        macsav_adaptive_result* res, macsav_adaptive_attempt* hist, int hist_cap,
                        cudaStream_t user) {
  if (P->members != 1) {
    P->err = "the device-resident adaptive run takes single-cavity plans";
    return MACSAV_ERR_VALUE;
  }
  const int n = scheme_stages(scheme);
  if (n < 2) {
    P->err = "the scheme has no embedded velocity";
    return MACSAV_ERR_VALUE;
  }
  int rc = step_buffers(P);
  if (rc != MACSAV_OK) return rc;
  StepBuffers& B = P->st;
  const long long sz = P->g.size;
  StageProgram G, G1;
  std::vector<double> c(2 * kCoefStride, 0.0), one(kCoefStride, 0.0);
  build_program(P, scheme, false, 0.0, nu, gamma, r0, G, c.data());
  build_program(P, scheme, false, 1.0, nu, gamma, r0, G1, one.data());
  for (int i = 0; i < kCoefStride; ++i) c[kCoefStride + i] = one[i] - c[i];
  const size_t state_off = 2 * kCoefStride * sizeof(double);
  const size_t hist_off = (state_off + sizeof(AdaptState) + sizeof(macsav_step_control) + 255) / 256 * 256;
  if (!B.adapt && cudaMalloc(&B.adapt, hist_off + sizeof(macsav_adaptive_attempt) * kAdaptHistory) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  char* base = static_cast<char*>(B.adapt);
  double* dc0 = reinterpret_cast<double*>(base);
  AdaptState* dst = reinterpret_cast<AdaptState*>(base + state_off);
  macsav_step_control* dctl = reinterpret_cast<macsav_step_control*>(dst + 1);
  macsav_adaptive_attempt* dh = reinterpret_cast<macsav_adaptive_attempt*>(base + hist_off);
  AdaptState s0;
  std::memset(&s0, 0, sizeof(s0));
  s0.t = t0;
  s0.end = t0 + T;
  s0.dt = std::fmin(dt0, ctl.max_step);
  s0.r = r0;
  s0.prev_err = -1.0;
  s0.hist_cap = kAdaptHistory;
  const double cap_attempts = double(ctl.max_steps) * (double(ctl.max_rejections) + 1.0) + 1.0;
  s0.max_attempts = cap_attempts > 2e9 ? 2000000000 : int(cap_attempts);
  const cudaStream_t s = B.stream;
  cudaEventRecord(B.ev_in, user);
  cudaStreamWaitEvent(s, B.ev_in, 0);
  cudaMemcpyAsync(dc0, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dst, &s0, sizeof(s0), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(B.X, x0, sizeof(double) * sz, cudaMemcpyDeviceToDevice, s);
  const int key = 1000 + scheme;
  cudaGraphExec_t exec = nullptr;
  for (auto& kv : B.graphs)
    if (kv.key == key) exec = kv.exec;
  if (!exec) {
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed) != cudaSuccess) return MACSAV_ERR_CUDA;
    cudaStreamCaptureStatus st;
    cudaGraph_t cap;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraphConditionalHandle cond;
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node;
    bool ok = cudaStreamGetCaptureInfo(s, &st, nullptr, &cap, &deps, nullptr, &ndeps) == cudaSuccess &&
              cudaGraphConditionalHandleCreate(&cond, cap, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = cond;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      ok = cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &cp) == cudaSuccess &&
           cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies) == cudaSuccess;
    }
    if (ok) {
      ok = cudaStreamBeginCaptureToGraph(B.loop, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                         cudaStreamCaptureModeRelaxed) == cudaSuccess;
      if (ok) {
        launch_k(k_adapt_begin, 1, kThreads, 0, B.loop, dst, static_cast<const double*>(dc0),
                 static_cast<const double*>(dc0 + kCoefStride), kCoefStride, G.r0_idx, B.coef);
        Exec X{B.loop, true, B.side, 0, 0.0};
        rc = enqueue_step(P, X, scheme, G, true);
        launch_k(k_adapt_control, 1, 32, 0, B.loop, dst, static_cast<const macsav_step_control*>(dctl),
                 static_cast<const double*>(B.enorm),
                 static_cast<const StageRec*>(B.recs), n, scheme_sav(scheme) ? 1 : 0, dh, cond);
        launch_k(k_adapt_accept, red_nb(sz), kThreads, 0, B.loop, static_cast<const AdaptState*>(dst), B.X, n * sz, sz);
        P->launches += 3;
        cudaGraph_t body;
        ok = cudaStreamEndCapture(B.loop, &body) == cudaSuccess && rc == MACSAV_OK;
      }
    }
    const cudaError_t e = cudaStreamEndCapture(s, &graph);
    if (!ok || e != cudaSuccess || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      P->err = "adaptive loop capture failed";
      return rc != MACSAV_OK ? rc : MACSAV_ERR_CUDA;
    }
    cudaGraphDestroy(graph);
    B.graphs.push_back(GraphEntry{key, exec});
  }
  if (cudaGraphLaunch(exec, s) != cudaSuccess) return MACSAV_ERR_CUDA;
  cudaMemcpyAsync(x_final, B.X, sizeof(double) * sz, cudaMemcpyDeviceToDevice, s);
  AdaptState out;
  cudaMemcpyAsync(&out, dst, sizeof(out), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return MACSAV_ERR_CUDA;
  const int nh = std::min(std::min(hist_cap, out.attempts), kAdaptHistory);
  if (hist && nh > 0 && cudaMemcpy(hist, dh, sizeof(macsav_adaptive_attempt) * nh, cudaMemcpyDeviceToHost) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  cudaEventRecord(B.ev_out, s);
  cudaStreamWaitEvent(user, B.ev_out, 0);
  res->t = out.t;
  res->r = out.r;
  res->next_step = out.dt;
  res->status = out.status == 1 ? 0 : 1;
  res->reason = out.status == 1 ? 0 : out.reason;
  res->accepted_steps = out.accepted;
  res->attempted_steps = out.attempts;
  return MACSAV_OK;
}

int run_step(Plan* P, int scheme, double t, double dt, double nu, double gamma, const double* x0, double r0,
             const double* forces, double* x1, double* embedded, double* pressures, macsav_stage_record* records,
             double* r1, cudaStream_t user) {
  const int rc = enqueue_step_async(P, scheme, t, dt, nu, gamma, x0, r0, forces, x1, embedded, pressures, user);
  if (rc != MACSAV_OK) return rc;
  return finish_step(P, records, r1);
}

}  // namespace macsav
