// Host-side plan: grid, transform descriptors, device work buffers.
#pragma once
#include <string>
#include <vector>

#include "stencils.cuh"
#include "transforms.cuh"

namespace macsav {

// Per-RHS-column Krylov scalars (device resident, mirrored to pinned memory).
struct CGScalars {
  double bnorm, atol, rho, rho_prev, alpha, beta, pq, rr, mean_q, mean_b, max_b;
  int active, iters, info, pad;
};

// Results of the closing checks of one solve (device resident).
struct SolveChecks {
  double max_defect, max_force, max_velocity, max_div;
  int nonfinite_force, nonfinite_solution, pad0, pad1;
};

template <typename T>
struct Transforms {
  TBlockDev<T> u, v, p;
  std::vector<void*> allocations;
  T* H = nullptr;
  size_t smem_row_uv = 0, smem_col_uv = 0, smem_row_p = 0, smem_col_p = 0;
};

struct Plan {
  GridDev g;
  double lx, ly;
  int precision;  // MACSAV_FP64 or MACSAV_FP32_MIXED
  double tol, ktol;
  int maxit, maxcols;
  int num_sms;
  std::string err;
  Transforms<double> t64;
  Transforms<float> t32;
  double pthr;  // Poisson zero-mode threshold

  // work buffers (column-blocked, maxcols columns)
  double* w = nullptr;      // packed velocity scratch
  double* vel = nullptr;    // packed velocity scratch 2
  double* cells = nullptr;  // 6 cell-sized vectors per column: b x r z p q
  float* cells32 = nullptr; // float CG vectors (mixed path)
  float* w32 = nullptr;
  double* partial = nullptr;
  size_t partial_len = 0;
  CGScalars* cg = nullptr;
  SolveChecks* checks = nullptr;
  int* active = nullptr;
  double* shift = nullptr;
  int* errword = nullptr;
  // pinned host mirrors
  CGScalars* h_cg = nullptr;
  SolveChecks* h_checks = nullptr;
  int* h_active = nullptr;
  int* h_err = nullptr;
  cudaEvent_t done = nullptr;

  // counters of kernel launches issued by this plan (for reporting)
  long long launches = 0;
};

int plan_build(Plan* p);
void plan_free(Plan* p);

}  // namespace macsav
