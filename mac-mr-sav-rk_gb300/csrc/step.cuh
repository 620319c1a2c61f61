// Internal declarations of the device time step (step.cu).
#pragma once
#include "plan.cuh"

namespace macsav {

constexpr int kMaxCombine = 12;

// Two outputs, each a sum of coef[idx] * src (null src = zero term); member
// m reads src + m * sstr and writes out + m * ostr.
struct CombineArgs {
  int nout;
  int nterm[2];
  double* out[2];
  long long ostr;
  const double* src[2][kMaxCombine];
  long long sstr[2][kMaxCombine];
  int idx[2][kMaxCombine];
};

// Coefficient-table slots of one stage's scalar update.
struct SavIdx {
  int dt, d, order, pred, nsr, r0;
  int sr_r[4];      // which r_k enters the scalar rhs (0 = the step's r0)
  int sr_coef[4];   // coefficient slots
};

void launch_convection(Plan* P, const double* x, double* out, cudaStream_t s);
int run_step(Plan* P, int scheme, double t, double dt, double nu, double gamma, const double* x0, double r0,
             const double* forces, double* x1, double* embedded, double* pressures, macsav_stage_record* records,
             double* r1, cudaStream_t user);
int enqueue_step_async(Plan* P, int scheme, double t, double dt, double nu, double gamma, const double* x0,
                       double r0, const double* forces, double* x1, double* embedded, double* pressures,
                       cudaStream_t user);
int finish_step(Plan* P, macsav_stage_record* records, double* r1);
// The same for all P->members equal-shape members at once: nus and r0 are host
// arrays of M values; x0, x1, embedded are [M][size], forces [M][stages][size],
// pressures [M][stages][np] (device); records [M][stages] and r1 [M] (host).
int enqueue_members(Plan* P, int scheme, double t, double dt, const double* nus, double gamma, const double* x0,
                    const double* r0, const double* forces, double* x1, double* embedded, double* pressures,
                    cudaStream_t user);
int finish_members(Plan* P, macsav_stage_record* records, double* r1);
int scheme_stages(int scheme);
void step_free(Plan* P);
int run_adaptive_device(Plan* P, int scheme, double t0, double T, double dt0, double nu, double gamma,
                        const double* x0, double r0, const macsav_step_control& ctl, double* x_final,
                        macsav_adaptive_result* res, macsav_adaptive_attempt* hist, int hist_cap,
                        cudaStream_t user);

}  // namespace macsav
