// Host-side plan: grid, transform descriptors, device work buffers.
#pragma once
#include <string>
#include <vector>

#include "stencils.cuh"
#include "transforms.cuh"
#include "unet.cuh"

namespace macsav {

constexpr int kMaxCols = 64;     // Stokes right-hand-side columns of one plan
constexpr int kMaxMembers = 32;  // members of one plan (2 columns each)

// Per-RHS-column Krylov scalars (device resident, mirrored to pinned memory).
struct CGScalars {
  double bnorm, atol, atol2, rho, rho_prev, alpha, beta, pq, rr, mean_q, mean_b, max_b, mean_z;
  float alpha_t, beta_t, mean_q_t, mean_b_t, mean_z_t, pad_t;  // the same scalars rounded once for FP32 kernels
  int active, iters, info;
  // learned preconditioner (flexible CG): on for this column, restart pending
  // (plain PCG from zero after the learned attempt failed), and counters that
  // accumulate over the solves since the last reset
  int net_on, restart, cum_iters, cum_net_iters, cum_fallbacks;
};

// Results of the closing checks of one solve (device resident).
struct SolveChecks {
  double max_defect, max_force, max_velocity, max_div;
  int nonfinite_force, nonfinite_solution, pad0, pad1;
};

// Detailed status of one device stage (mapped to exceptions by the host).
enum StageStatus : int {
  ST_OK = 0,
  ST_STOKES_RHS = 1,     // ValueError("Invalid Stokes RHS")
  ST_CG = 2,             // RuntimeError("Pressure Schur CG failed with info=N")
  ST_STOKES_GATE = 3,    // RuntimeError("Stokes residual=..., divergence=...")
  ST_NEG_ENERGY = 4,     // RuntimeError("Negative Stokes response energy")
  ST_SAV_INPUT = 5,      // ValueError("Invalid frozen SAV scalar inputs")
  ST_SAV_DENOM = 6,      // RuntimeError("Invalid frozen SAV scalar denominator")
  ST_SAV_NONFINITE = 7,  // RuntimeError("Nonfinite frozen SAV correction")
  ST_STAGE_GATE = 8,     // RuntimeError("SAV stage residuals ...")
};

// Device record of one stage (folded into macsav_stage_record).
struct StageRec {
  double r, residual, scalar_residual, divergence, predictor, factor, corr[2];
  double stokes_residual, stokes_divergence, alpha, beta, coupling, scalar_rhs;
  double max_rhs, max_conv, nn, max_velocity, max_pressure;
  int n_corr, status, iters[2], cg_info;
  int sav_status;  // SAV failure of the stage, merged into status by k_stage_close
};

struct GraphEntry {
  int key;
  cudaGraphExec_t exec;
};

// Buffers of the device time step, allocated at the first step call.
struct StepBuffers {
  void* base = nullptr;
  double *X = nullptr, *KU = nullptr, *NN = nullptr, *F = nullptr, *VW = nullptr, *FORCE = nullptr,
         *EMB = nullptr, *PI = nullptr, *PS = nullptr, *coef = nullptr;
  StageRec* recs = nullptr;
  StageRec* h_recs = nullptr;
  double* h_coef = nullptr;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  std::vector<GraphEntry> graphs;
  int pending_scheme = 0, pending_stages = 0;  // an enqueued step awaiting finish_step
  double* enorm = nullptr;    // embedded-error inner products of the last step (device)
  double* h_enorm = nullptr;  // and their pinned host copy
  bool have_enorm = false;
  void* adapt = nullptr;            // device-resident adaptive run: coefficient recipe, state, history
  cudaStream_t loop = nullptr;      // capture stream of its attempt loop's body
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
  int members = 1;  // equal-shape cavities stepped together (2 Stokes columns each)
  // FP32_MIXED: inner FP32 Krylov tolerance and defect-correction sweeps
  double inner_ktol = 1e-4;
  double first_ktol = 0.0;  // tolerance of a Stokes solve's first FP32 solve (0: inner_ktol)
  int corrections = 2;
  int num_sms;
  std::string err;
  Transforms<double> t64;
  Transforms<float> t32;
  double pthr;  // Poisson zero-mode threshold

  // work buffers (column-blocked, maxcols columns)
  double* w = nullptr;      // packed velocity scratch
  double* cells = nullptr;  // 6 cell-sized vectors per column: b x r z p q
  float* cells32 = nullptr; // float CG vectors (mixed path)
  float* w32 = nullptr;
  // mixed path: the velocity and pressure of each FP32 inner solve of a
  // Stokes solve (velocity accumulated inside its CG), one piece per sweep,
  // summed into the FP64 fields once at the end
  float* wacc32 = nullptr;   // [pieces][maxcols][size]
  float* xpieces = nullptr;  // [pieces][maxcols][np]
  int pieces = 0;
  double* partial = nullptr;
  size_t partial_len = 0;
  CGScalars* cg = nullptr;
  SolveChecks* checks = nullptr;
  int* active = nullptr;
  double* shift = nullptr;
  int* errword = nullptr;
  unsigned int* done_counter = nullptr;  // last-block counter of reductions
  // fork streams/events: [0] concurrent u/v passes of the main stream, [1] the
  // same inside the CG body, [2] a stage's closing work (pressure centring and
  // the Stokes check), which runs beside the stage's SAV algebra and uses
  // partial2 and done_counter[8] for its reductions
  cudaStream_t aux[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t evf[3] = {nullptr, nullptr, nullptr}, evj[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t evc = nullptr;
  double* partial2 = nullptr;
  // pinned host mirrors
  CGScalars* h_cg = nullptr;
  SolveChecks* h_checks = nullptr;
  int* h_active = nullptr;
  int* h_err = nullptr;
  cudaEvent_t done = nullptr;

  // device time step
  StepBuffers st;
  int use_graph = 0;

  // counters of kernel launches issued by this plan (for reporting)
  long long launches = 0;

  // learned correction of the pressure preconditioner (FP32_MIXED inner
  // solves); the network is owned by the caller, the buffers by the plan
  UNet* net = nullptr;
  NetWork netw;
  float* net_out = nullptr;    // network output, [maxcols][np]
  float* net_rold = nullptr;   // previous residual (Polak-Ribiere beta), [maxcols][np]
  float* net_wacc0 = nullptr;  // start of the accumulated velocity, for restarts, [maxcols][size]
  float* net_scale = nullptr;  // per-column input and output scales, [2][maxcols]
  int net_maxit = 20;          // learned iterations before the plain-PCG restart
  // placement: every_iter = 0 evaluates the network only in the first CG
  // iteration of the first inner solve of each Stokes solve (its first search
  // direction); 1 in every iteration of every inner solve.  The network works
  // on the residual restricted by `restrict_f` (1, 2 or 4: f x f cell means)
  // and its output is prolonged bilinearly back to the cells.
  int net_every = 0;
  int net_restrict = 1;
  float* net_cin = nullptr;    // restricted network input,  [maxcols][np / f^2]
  float* net_cout = nullptr;   // restricted network output, [maxcols][np / f^2]

  // FP32 row transforms of macsav_transform32: tensor-core matrices, FFT
  // line blocks and the autotuner's choices (tgemm.cu)
  struct Transform32Cache* tcache = nullptr;

  // residual / preconditioned residual / iterate log of eager FP64 solves
  double* log_r = nullptr;
  double* log_z = nullptr;
  double* log_x = nullptr;
  int log_cap = 0, log_n = 0;
};

// Execution context of one enqueue: eager (the host drives the CG loop on the
// device flags) or graph capture (the CG loop becomes a conditional WHILE
// node whose body is one iteration).
struct Exec {
  cudaStream_t s;
  bool graph;
  cudaStream_t side;  // body capture stream (graph mode)
  cudaGraphConditionalHandle cond;
  double ktol;        // Krylov tolerance of the solve being enqueued (0: the plan's)
  int net = 0;        // use the plan's learned preconditioner (flexible CG)
  double* partial = nullptr;       // reduction partials (null: the plan's)
  unsigned int* counter = nullptr; // last-block counter (null: the plan's)
};

int plan_build(Plan* p);
void plan_free(Plan* p);

}  // namespace macsav
