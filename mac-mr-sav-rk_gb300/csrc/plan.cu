// Plan construction: FFT radix plans, twiddle/eigenvalue tables, launch shapes
// and device work buffers.  Tables are computed on the host in double
// precision (std::cos/std::sin) and rounded to the working type.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "plan.cuh"

namespace macsav {

static const double kPi = 3.14159265358979323846264338327950288;

FFTPlan make_fft_plan(int L) {
  FFTPlan f{};
  f.L = L;
  int m = L, ns = 0;
  while (m % 4 == 0 && ns < kMaxStages) { f.radix[ns++] = 4; m /= 4; }
  while (m % 2 == 0 && ns < kMaxStages) { f.radix[ns++] = 2; m /= 2; }
  while (m % 3 == 0 && ns < kMaxStages) { f.radix[ns++] = 3; m /= 3; }
  f.nstages = (m == 1) ? ns : 0;  // 0: direct DFT
  int prod = 1;
  for (int s = 0; s < f.nstages; ++s) {
    f.ns[s] = FastDiv(prod);
    f.nbf[s] = FastDiv(L / f.radix[s]);
    prod *= f.radix[s];
  }
  return f;
}

int fft_length(int kind, int n) { return kind == KIND_DST1 ? 2 * (n + 1) : n; }

// Eigenvalues of the 1-D second difference in the internal coefficient order
// (solver/mac/tensor_stokes.py:31-38; DST-II is stored reversed, see transforms.cuh).
std::vector<double> internal_eigenvalues(int kind, int n, double h) {
  std::vector<double> e(n);
  for (int j = 0; j < n; ++j) {
    double theta;
    if (kind == KIND_DCT2) theta = kPi * j / n;
    else if (kind == KIND_DST1) theta = kPi * (j + 1) / (n + 1);
    else theta = kPi * (n - j) / n;  // DST-II coefficient n-1-j has theta = pi (n-j)/n
    e[j] = (2.0 - 2.0 * std::cos(theta)) / (h * h);
  }
  return e;
}

static int pick_pairs(int L, int rows, int sms) {
  int P = std::max(1, std::min(4096 / L, (rows + 1) / 2));
  while (P > 1 && (rows + 2 * P - 1) / (2 * P) < 2 * sms) P /= 2;
  return P;
}

// Columns per CTA of the column pass (a power of two): at most 4096 complex
// values in shared memory, and at least 32 bytes of each row per CTA (one
// full DRAM sector) when that fits, then narrower only while there are too
// few CTAs.
static int pick_strip(int L, int cols, int sms, int elem_bytes) {
  int W = 2;
  while (W < 32 && (W * 2 / 2) * L <= 4096 && W * 2 * L / 2 <= 4096) W *= 2;
  const int wmin = std::min(W, std::max(2, 16 / elem_bytes));
  while (W > wmin && (cols + W - 1) / W < 2 * sms) W /= 2;
  return W;
}

// The twiddles of a power-of-two length L = tw.size() in the order the
// Stockham passes of fft_p2 read them: for each pass with NS > 1 (radix R,
// TWS = L / (NS R)), rows r = 1 .. R-1 of NS entries tw[r k TWS], k = 0 ..
// NS-1.  A butterfly's seven twiddles are then one per-thread base plus
// compile-time offsets, and a warp's loads of one r are consecutive.  The
// values are the table's own, so the transforms' bits do not change.  Empty
// for other lengths (the generic passes read tw itself).
template <typename T>
static std::vector<cplx<T>> pass_twiddles(const std::vector<cplx<T>>& tw) {
  const int L = int(tw.size());
  std::vector<cplx<T>> out;
  if (L < 64 || L > 4096 || (L & (L - 1))) return out;  // the power-of-two passes' lengths
  for (int NS = 1; NS < L;) {
    const int R = L / NS >= 8 ? 8 : L / NS, TWS = L / (NS * R);
    if (NS > 1)
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < NS; ++k) out.push_back(tw[size_t(r) * k * TWS]);
    NS *= R;
  }
  return out;
}

template <typename T>
static cudaError_t build_block(TBlockDev<T>& B, int rows, int cols, int kx, int ky, double hx, double hy,
                               int sms, std::vector<void*>& allocs) {
  B.rows = rows;
  B.cols = cols;
  B.kx = kx;
  B.ky = ky;
  const int Lx = fft_length(kx, cols), Ly = fft_length(ky, rows);
  B.fx = make_fft_plan(Lx);
  B.fy = make_fft_plan(Ly);
  B.lsx = Lx;
  B.lsy = Ly;
  B.pitch = (cols + 31) / 32 * 32;
  B.px = pick_pairs(Lx, rows, sms);
  B.wy = pick_strip(Ly, cols, sms, int(sizeof(T)));
  B.tpl = Lx / 8;  // each specialised launch sets its own
  B.shape[0] = B.shape[1] = B.shape[2] = 0;  // P2_AUTO: each pass picks its launch shape
  B.fcols = FastDiv(cols);
  B.frows = FastDiv(rows);
  B.fw = FastDiv(B.wy);
  B.fvpr = FastDiv(std::max(1, B.wy / int(16 / sizeof(T))));
  B.fhalf = FastDiv(rows / 2 + 1);
  B.sx = T(kx == KIND_DST1 ? 1.0 / (cols + 1) : 1.0 / cols);
  B.sy = T(ky == KIND_DST1 ? 1.0 / (rows + 1) : 1.0 / rows);
  // host tables
  std::vector<cplx<T>> twx(Lx), twy(Ly), qx(cols), qy(rows);
  for (int m = 0; m < Lx; ++m) twx[m] = mk(T(std::cos(2 * kPi * m / Lx)), T(-std::sin(2 * kPi * m / Lx)));
  for (int m = 0; m < Ly; ++m) twy[m] = mk(T(std::cos(2 * kPi * m / Ly)), T(-std::sin(2 * kPi * m / Ly)));
  const std::vector<cplx<T>> twpx = pass_twiddles(twx), twpy = pass_twiddles(twy);
  for (int k = 0; k < cols; ++k) qx[k] = mk(T(std::cos(kPi * k / (2.0 * cols))), T(-std::sin(kPi * k / (2.0 * cols))));
  for (int k = 0; k < rows; ++k) qy[k] = mk(T(std::cos(kPi * k / (2.0 * rows))), T(-std::sin(kPi * k / (2.0 * rows))));
  std::vector<double> ex = internal_eigenvalues(kx, cols, hx), ey = internal_eigenvalues(ky, rows, hy);
  std::vector<T> exT(ex.begin(), ex.end()), eyT(ey.begin(), ey.end());
  // every table starts on a 16-byte boundary (the kernels read the complex
  // tables as 8- or 16-byte vectors, and an FP32 eigenvalue table of odd
  // length would leave a following table 4 bytes off)
  auto up16 = [](size_t n) { return (n + 15) / 16 * 16; };
  const size_t bytes = up16(sizeof(cplx<T>) * Lx) + up16(sizeof(cplx<T>) * Ly) + up16(sizeof(cplx<T>) * cols) +
                       up16(sizeof(cplx<T>) * rows) + up16(sizeof(T) * cols) + up16(sizeof(T) * rows) +
                       up16(sizeof(cplx<T>) * twpx.size()) + up16(sizeof(cplx<T>) * twpy.size());
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, bytes);
  if (e != cudaSuccess) return e;
  allocs.push_back(d);
  char* p = static_cast<char*>(d);
  auto put = [&](const void* src, size_t n) {
    void* dst = p;
    if (n) cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice);
    p += up16(n);
    return dst;
  };
  B.twx = static_cast<const cplx<T>*>(put(twx.data(), sizeof(cplx<T>) * Lx));
  B.twy = static_cast<const cplx<T>*>(put(twy.data(), sizeof(cplx<T>) * Ly));
  B.qx = static_cast<const cplx<T>*>(put(qx.data(), sizeof(cplx<T>) * cols));
  B.qy = static_cast<const cplx<T>*>(put(qy.data(), sizeof(cplx<T>) * rows));
  B.eigx = static_cast<const T*>(put(exT.data(), sizeof(T) * cols));
  B.eigy = static_cast<const T*>(put(eyT.data(), sizeof(T) * rows));
  B.twpx = twpx.empty() ? nullptr : static_cast<const cplx<T>*>(put(twpx.data(), sizeof(cplx<T>) * twpx.size()));
  B.twpy = twpy.empty() ? nullptr : static_cast<const cplx<T>*>(put(twpy.data(), sizeof(cplx<T>) * twpy.size()));
  return cudaGetLastError();
}

// A block used only for x-line transforms (the 1-D transform entry).
template <typename T>
cudaError_t build_line_block(TBlockDev<T>& B, int rows, int cols, int kx, int sms, std::vector<void*>& allocs) {
  return build_block(B, rows, cols, kx, KIND_DCT2, 1.0, 1.0, sms, allocs);
}
template cudaError_t build_line_block<double>(TBlockDev<double>&, int, int, int, int, std::vector<void*>&);
template cudaError_t build_line_block<float>(TBlockDev<float>&, int, int, int, int, std::vector<void*>&);

template <typename T>
size_t row_smem(const TBlockDev<T>& B) {
  return size_t(B.px) * B.lsx * sizeof(cplx<T>) * (B.fx.nstages == 0 ? 2 : 1);
}
template <typename T>
size_t col_smem(const TBlockDev<T>& B) {
  return size_t(B.wy / 2) * B.lsy * sizeof(cplx<T>) * (B.fy.nstages == 0 ? 2 : 1);
}
template size_t row_smem<double>(const TBlockDev<double>&);
template size_t row_smem<float>(const TBlockDev<float>&);
template size_t col_smem<double>(const TBlockDev<double>&);
template size_t col_smem<float>(const TBlockDev<float>&);

template <typename T>
static cudaError_t build_transforms(Transforms<T>& t, const Plan& pl) {
  const GridDev& g = pl.g;
  cudaError_t e;
  if ((e = build_block(t.u, g.ny, g.nx - 1, KIND_DST1, KIND_DST2, g.hx, g.hy, pl.num_sms, t.allocations))) return e;
  if ((e = build_block(t.v, g.ny - 1, g.nx, KIND_DST2, KIND_DST1, g.hx, g.hy, pl.num_sms, t.allocations))) return e;
  if ((e = build_block(t.p, g.ny, g.nx, KIND_DCT2, KIND_DCT2, g.hx, g.hy, pl.num_sms, t.allocations))) return e;
  const size_t hu = size_t(t.u.rows) * t.u.pitch, hv = size_t(t.v.rows) * t.v.pitch, hp = size_t(t.p.rows) * t.p.pitch;
  const size_t per_col = hu + hv + hp;
  void* d = nullptr;
  if ((e = cudaMalloc(&d, sizeof(T) * per_col * pl.maxcols))) return e;
  t.allocations.push_back(d);
  if ((e = cudaMemset(d, 0, sizeof(T) * per_col * pl.maxcols))) return e;  // padding stays zero
  t.H = static_cast<T*>(d);
  t.u.H = t.H;
  t.v.H = t.H + hu;
  t.p.H = t.H + hu + hv;
  t.u.hstride = t.v.hstride = t.p.hstride = (long long)per_col;
  t.smem_row_uv = std::max(row_smem(t.u), row_smem(t.v));
  t.smem_col_uv = std::max(col_smem(t.u), col_smem(t.v));
  t.smem_row_p = row_smem(t.p);
  t.smem_col_p = col_smem(t.p);
  return cudaSuccess;
}

template <typename T>
static void free_transforms(Transforms<T>& t) {
  for (void* p : t.allocations) cudaFree(p);
  t.allocations.clear();
  t.H = nullptr;
}

void set_reduction_cap(int sms);

int plan_build(Plan* p) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) { p->err = std::string("CUDA: ") + cudaGetErrorString(e); return MACSAV_ERR_CUDA; }
  set_reduction_cap(p->num_sms);
  GridDev& g = p->g;
  const int largest = std::max(fft_length(KIND_DST1, g.nx - 1), fft_length(KIND_DST1, g.ny - 1));
  if (largest > 4096) { p->err = "grid too large: FFT length above 4096"; return MACSAV_ERR_UNSUPPORTED; }
  for (int L : {2 * g.nx, 2 * g.ny, g.nx, g.ny})
    if (make_fft_plan(L).nstages == 0 && L > 512) {
      p->err = "grid size needs an FFT length with a prime factor above 3 (> 512)";
      return MACSAV_ERR_UNSUPPORTED;
    }
  if ((e = build_transforms(p->t64, *p))) goto fail;
  if (p->precision == MACSAV_FP32_MIXED)
    if ((e = build_transforms(p->t32, *p))) goto fail;
  {
    const int C = p->maxcols;
    const size_t size = g.size, np = g.np;
    if ((e = cudaMalloc(&p->w, sizeof(double) * size * C))) goto fail;
    if ((e = cudaMalloc(&p->cells, sizeof(double) * np * C * 6))) goto fail;
    if (p->precision == MACSAV_FP32_MIXED) {
      if ((e = cudaMalloc(&p->cells32, sizeof(float) * np * C * 6))) goto fail;
      if ((e = cudaMalloc(&p->w32, sizeof(float) * size * C))) goto fail;
      p->pieces = p->corrections + 1;
      if ((e = cudaMalloc(&p->wacc32, sizeof(float) * size * C * p->pieces))) goto fail;
      if ((e = cudaMalloc(&p->xpieces, sizeof(float) * np * C * p->pieces))) goto fail;
    }
    p->partial_len = size_t(C) * 8 * 4096;
    if ((e = cudaMalloc(&p->partial, sizeof(double) * p->partial_len))) goto fail;
    if ((e = cudaMalloc(&p->partial2, sizeof(double) * p->partial_len))) goto fail;
    if ((e = cudaMalloc(&p->cg, sizeof(CGScalars) * C))) goto fail;
    if ((e = cudaMalloc(&p->checks, sizeof(SolveChecks) * C))) goto fail;
    if ((e = cudaMalloc(&p->active, sizeof(int) * C))) goto fail;
    if ((e = cudaMalloc(&p->shift, sizeof(double) * 2 * C))) goto fail;
    if ((e = cudaMalloc(&p->errword, sizeof(int)))) goto fail;
    if ((e = cudaMalloc(&p->done_counter, sizeof(unsigned int) * 16))) goto fail;
    if ((e = cudaMemset(p->done_counter, 0, sizeof(unsigned int) * 16))) goto fail;
    if ((e = cudaMallocHost(&p->h_cg, sizeof(CGScalars) * C))) goto fail;
    if ((e = cudaMallocHost(&p->h_checks, sizeof(SolveChecks) * C))) goto fail;
    if ((e = cudaMallocHost(&p->h_active, sizeof(int) * C))) goto fail;
    if ((e = cudaMallocHost(&p->h_err, sizeof(int)))) goto fail;
    if ((e = cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming))) goto fail;
    for (int k = 0; k < 3; ++k) {
      if ((e = cudaStreamCreateWithFlags(&p->aux[k], cudaStreamNonBlocking))) goto fail;
      if ((e = cudaEventCreateWithFlags(&p->evf[k], cudaEventDisableTiming))) goto fail;
      if ((e = cudaEventCreateWithFlags(&p->evj[k], cudaEventDisableTiming))) goto fail;
    }
    if ((e = cudaEventCreateWithFlags(&p->evc, cudaEventDisableTiming))) goto fail;
  }
  // Poisson zero-mode threshold: 100 eps max(lambda) (tensor_stokes.py:165-168)
  {
    std::vector<double> ex = internal_eigenvalues(KIND_DCT2, g.nx, g.hx), ey = internal_eigenvalues(KIND_DCT2, g.ny, g.hy);
    double mx = 0;
    for (double a : ey)
      for (double b : ex) mx = std::max(mx, a + b);
    p->pthr = 100.0 * 2.220446049250313e-16 * mx;
  }
  return MACSAV_OK;
fail:
  p->err = std::string("CUDA: ") + cudaGetErrorString(e);
  plan_free(p);
  return MACSAV_ERR_CUDA;
}

void step_free(Plan* P);

void free_transform32_cache(Plan* P);

void plan_free(Plan* p) {
  step_free(p);
  free_transform32_cache(p);
  free_transforms(p->t64);
  free_transforms(p->t32);
  cudaFree(p->w); cudaFree(p->cells); cudaFree(p->cells32); cudaFree(p->w32); cudaFree(p->wacc32);
  cudaFree(p->xpieces);
  cudaFree(p->partial); cudaFree(p->partial2); cudaFree(p->cg); cudaFree(p->checks); cudaFree(p->active); cudaFree(p->shift);
  cudaFree(p->errword);
  cudaFree(p->done_counter);
  cudaFree(p->net_out); cudaFree(p->net_rold); cudaFree(p->net_scale);
  cudaFree(p->net_cin); cudaFree(p->net_cout); cudaFree(p->net_wacc0);
  net_work_free(&p->netw);
  p->done_counter = nullptr;
  cudaFreeHost(p->h_cg); cudaFreeHost(p->h_checks); cudaFreeHost(p->h_active); cudaFreeHost(p->h_err);
  if (p->done) cudaEventDestroy(p->done);
  for (int k = 0; k < 3; ++k) {
    if (p->aux[k]) cudaStreamDestroy(p->aux[k]);
    if (p->evf[k]) cudaEventDestroy(p->evf[k]);
    if (p->evj[k]) cudaEventDestroy(p->evj[k]);
    p->aux[k] = nullptr;
    p->evf[k] = p->evj[k] = nullptr;
  }
  if (p->evc) cudaEventDestroy(p->evc);
  p->evc = nullptr;
  p->w = p->cells = p->partial = p->partial2 = p->shift = nullptr;
  p->cells32 = p->w32 = p->wacc32 = p->xpieces = nullptr;
  p->pieces = 0;
  p->cg = nullptr; p->checks = nullptr; p->active = p->errword = nullptr;
  p->h_cg = nullptr; p->h_checks = nullptr; p->h_active = p->h_err = nullptr;
  p->done = nullptr;
}

}  // namespace macsav
