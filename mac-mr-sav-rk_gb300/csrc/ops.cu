// Stand-alone operators of the MAC model seam: K, D, D^T, convection,
// combine / inner / max_abs reductions, diagnostics and the 1-D transform
// entry used to check the FFT machinery against scipy.fft.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "solver.cuh"

namespace macsav {

constexpr int kOpsRedMax = 1024;

inline int op_blocks(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : b);
}
inline int op_red_blocks(long long n) {
  long long b = (n + kThreads - 1) / kThreads;
  return int(b < 1 ? 1 : (b > kOpsRedMax ? kOpsRedMax : b));
}

__global__ void k_apply_K(GridDev g, const double* x, double* y) {
  const int c = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < g.size) y[(long long)c * g.size + e] = K_at(x + (long long)c * g.size, g, e);
}
__global__ void k_apply_D(GridDev g, const double* x, double* p) {
  const int c = blockIdx.y;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < g.np) {
    const int j = idx / g.nx, i = idx - j * g.nx;
    p[(long long)c * g.np + idx] = D_at(x + (long long)c * g.size, g, j, i);
  }
}
__global__ void k_apply_Dt(GridDev g, const double* p, double* x) {
  const int c = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < g.size) x[(long long)c * g.size + e] = Dt_at(p + (long long)c * g.np, g, e);
}
__global__ void k_convection(GridDev g, const double* x, double* n) {
  const int c = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < g.size) n[(long long)c * g.size + e] = conv_at(x + (long long)c * g.size, g, e);
}

constexpr int kMaxTerms = 16;
struct Terms {
  const double* f[kMaxTerms];
  double a[kMaxTerms];
  int n;
};
// out = sum_k a_k f_k, accumulated left to right (solver/mac_ns.py:40-45).
__global__ void k_combine(Terms t, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < t.n; ++k) s += t.a[k] * t.f[k][i];
    out[i] = s;
  }
}

// slot 0: dot(a,b) (or sum a when b null); slot 1: max|a|
__global__ void k_dot_max(const double* a, const double* b, long long n, double* partial) {
  __shared__ double red[64];
  double s[1] = {0.0}, m[1] = {0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double av = a[i];
    s[0] += b ? av * b[i] : av;
    m[0] = nanmax(m[0], fabs(av));
  }
  block_sum<1>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0) {
    partial[blockIdx.x * 2] = s[0];
    partial[blockIdx.x * 2 + 1] = m[0];
  }
}
__global__ void k_fold(const double* partial, int nb, double* out) {
  __shared__ double red[64];
  double s[1] = {0.0}, m[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    s[0] += partial[2 * b];
    m[0] = nanmax(m[0], partial[2 * b + 1]);
  }
  block_sum<1>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0) {
    out[0] = s[0];
    out[1] = m[0];
  }
}

// Diagnostics partials: kinetic <x,x>, h1 <x,Kx>, max|Dx|, angular, power <f,x>.
__global__ void k_diag(GridDev g, double lx, double ly, const double* x, const double* f, double* partial) {
  __shared__ double red[6 * 32];
  double s[4] = {0, 0, 0, 0}, m[1] = {0.0};
  const int n = g.size > g.np ? g.size : g.np;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (idx < g.size) {
      const double xe = x[idx];
      s[0] += xe * xe;
      s[1] += xe * K_at(x, g, idx);
      if (f) s[3] += f[idx] * xe;
    }
    if (idx < g.np) {
      const int j = idx / g.nx, i = idx - j * g.nx;
      m[0] = nanmax(m[0], fabs(D_at(x, g, j, i)));
      // angular momentum about the centre with cell-centred velocities (mac_ns.py:84-93)
      const double cu = 0.5 * (U(x, g, j, i) + U(x, g, j, i + 1));
      const double cv = 0.5 * (V(x, g, j, i) + V(x, g, j + 1, i));
      const double xc = (i + 0.5) * g.hx - 0.5 * lx, yc = (j + 0.5) * g.hy - 0.5 * ly;
      s[2] += xc * cv - yc * cu;
    }
  }
  block_sum<4>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0)
    for (int k = 0; k < 5; ++k) partial[blockIdx.x * 5 + k] = k < 4 ? s[k] : m[0];
}
__global__ void k_diag_fold(const double* partial, int nb, double area, double r, double nu, double* out) {
  __shared__ double red[6 * 32];
  double s[4] = {0, 0, 0, 0}, m[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    for (int k = 0; k < 4; ++k) s[k] += partial[b * 5 + k];
    m[0] = nanmax(m[0], partial[b * 5 + 4]);
  }
  block_sum<4>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0) {
    const double kinetic = 0.5 * area * s[0], h1 = area * s[1];
    out[0] = kinetic;
    out[1] = kinetic + 0.5 * (r - 1) * (r - 1);
    out[2] = m[0];
    out[3] = h1;
    out[4] = r;
    out[5] = area * s[2];
    out[6] = area * s[3];
    out[7] = nu * h1;
  }
}

// ----- 1-D ortho transform along rows (test entry) -----
// forward unnormalised -> ortho scale, with DST-II re-reversed.
__global__ void k_ortho_out(const double* H, int pitch, double* out, int rows, int n, int kind) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
  if (k >= n || row >= rows) return;
  const double v = H[(long long)row * pitch + k];
  if (kind == KIND_DST1) {
    out[(long long)row * n + k] = v * sqrt(2.0 / (n + 1));
  } else {
    const double s = k == 0 ? sqrt(1.0 / (4.0 * n)) : sqrt(1.0 / (2.0 * n));
    const int dst = kind == KIND_DST2 ? n - 1 - k : k;
    out[(long long)row * n + dst] = v * s;
  }
}
// ortho coefficients -> internal unnormalised coefficients in H
__global__ void k_ortho_in(const double* in, double* H, int pitch, int rows, int n, int kind) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
  if (k >= n || row >= rows) return;
  double v;
  if (kind == KIND_DST1) {
    v = in[(long long)row * n + k] / sqrt(2.0 / (n + 1));
  } else {
    const double s = k == 0 ? sqrt(1.0 / (4.0 * n)) : sqrt(1.0 / (2.0 * n));
    const int src = kind == KIND_DST2 ? n - 1 - k : k;
    v = in[(long long)row * n + src] / s;
  }
  H[(long long)row * pitch + k] = v;
}


// ------------------------------------------------------------ host entries ---
template <typename T>
cudaError_t build_line_block(TBlockDev<T>& B, int rows, int cols, int kx, int sms, std::vector<void*>& allocs);

int op_apply(Plan* P, int which, const double* in, double* out, int cols, cudaStream_t s) {
  const GridDev& g = P->g;
  if (which == 0) k_apply_K<<<dim3(op_blocks(g.size), cols), kThreads, 0, s>>>(g, in, out);
  else if (which == 1) k_apply_D<<<dim3(op_blocks(g.np), cols), kThreads, 0, s>>>(g, in, out);
  else if (which == 2) k_apply_Dt<<<dim3(op_blocks(g.size), cols), kThreads, 0, s>>>(g, in, out);
  else k_convection<<<dim3(op_blocks(g.size), cols), kThreads, 0, s>>>(g, in, out);
  ++P->launches;
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// Packed free vector <-> full face arrays u (ny, nx+1) and v (ny+1, nx)
// (MACGrid.pack / unpack, solver/mac/grid.py:52-65); unpack writes the zero
// normal wall faces.
__global__ void k_unpack(GridDev g, const double* x, double* u, double* v) {
  const int nU = g.ny * (g.nx + 1), nV = (g.ny + 1) * g.nx;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nU + nV; e += gridDim.x * blockDim.x) {
    if (e < nU) {
      const int j = e / (g.nx + 1), I = e - j * (g.nx + 1);
      u[e] = (I == 0 || I == g.nx) ? 0.0 : x[j * (g.nx - 1) + I - 1];
    } else {
      const int f = e - nU, J = f / g.nx, i = f - J * g.nx;
      v[f] = (J == 0 || J == g.ny) ? 0.0 : x[g.nu + (J - 1) * g.nx + i];
    }
  }
}
__global__ void k_pack(GridDev g, const double* u, const double* v, double* x) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.size; e += gridDim.x * blockDim.x) {
    if (e < g.nu) {
      const int j = e / (g.nx - 1), i = e - j * (g.nx - 1);
      x[e] = u[j * (g.nx + 1) + i + 1];
    } else {
      const int f = e - g.nu, k = f / g.nx, i = f - k * g.nx;
      x[e] = v[(k + 1) * g.nx + i];
    }
  }
}

int op_layout(Plan* P, int direction, double* packed, double* u, double* v, cudaStream_t s) {
  const GridDev& g = P->g;
  if (direction == 0) k_unpack<<<op_blocks(g.ny * (g.nx + 1) + (g.ny + 1) * g.nx), kThreads, 0, s>>>(g, packed, u, v);
  else k_pack<<<op_blocks(g.size), kThreads, 0, s>>>(g, u, v, packed);
  ++P->launches;
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// Copies `count` vectors, src[k] -> dst[k] (n[k] doubles each), in one
// launch: blockIdx.y strides over the vectors, blockIdx.x and the threads over
// each vector's elements.  The ensemble's host boundary: src or dst are then
// pinned host arrays that the device maps, read or written over the host link.
__global__ void __launch_bounds__(kThreads) k_copy_vectors(int count, const double* const* src, double* const* dst,
                                                           const long long* n) {
  for (int k = blockIdx.y; k < count; k += gridDim.y) {
    const double* s = src[k];
    double* d = dst[k];
    const long long m = n[k];
    for (long long i = blockIdx.x * (long long)kThreads + threadIdx.x; i < m; i += (long long)gridDim.x * kThreads)
      d[i] = s[i];
  }
}

int op_copy_vectors(int count, const double* const* src, double* const* dst, const long long* n, long long max_n,
                    cudaStream_t s) {
  const long long per = (max_n + 8LL * kThreads - 1) / (8LL * kThreads);  // about 8 elements per thread
  const dim3 grid(unsigned(std::min<long long>(std::max<long long>(per, 1), 1024)), unsigned(std::min(count, 65535)));
  k_copy_vectors<<<grid, kThreads, 0, s>>>(count, src, dst, n);
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

void launch_convection(Plan* P, const double* x, double* out, cudaStream_t s) {
  k_convection<<<dim3(op_blocks(P->g.size), 1), kThreads, 0, s>>>(P->g, x, out);
  ++P->launches;
}

int op_combine(Plan* P, int nterms, const double* coeffs, const double* const* fields, double* out, long long n,
               cudaStream_t s) {
  if (nterms < 1 || nterms > kMaxTerms) {
    P->err = "combine: 1..16 terms";
    return MACSAV_ERR_VALUE;
  }
  Terms t;
  t.n = nterms;
  for (int k = 0; k < nterms; ++k) {
    t.f[k] = fields[k];
    t.a[k] = coeffs[k];
  }
  const int nb = int(std::min<long long>(op_blocks(n), 4LL * P->num_sms * 8));
  k_combine<<<nb, kThreads, 0, s>>>(t, out, n);
  ++P->launches;
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// result[0] = dot (or sum), result[1] = max|a|; synchronises.
int op_dot_max(Plan* P, const double* a, const double* b, long long n, double* result, cudaStream_t s) {
  const int nb = op_red_blocks(n);
  k_dot_max<<<nb, kThreads, 0, s>>>(a, b, n, P->partial);
  k_fold<<<1, kThreads, 0, s>>>(P->partial, nb, P->partial + 2 * kOpsRedMax);
  P->launches += 2;
  cudaMemcpyAsync(result, P->partial + 2 * kOpsRedMax, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

int op_diagnostics(Plan* P, const double* x, double r, double nu, const double* force, double* out,
                   cudaStream_t s) {
  const GridDev& g = P->g;
  const int nb = op_red_blocks(g.size > g.np ? g.size : g.np);
  k_diag<<<nb, kThreads, 0, s>>>(g, P->lx, P->ly, x, force, P->partial);
  k_diag_fold<<<1, kThreads, 0, s>>>(P->partial, nb, g.hx * g.hy, r, nu, P->partial + 5 * kOpsRedMax);
  P->launches += 2;
  cudaMemcpyAsync(out, P->partial + 5 * kOpsRedMax, 8 * sizeof(double), cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

int op_transform(Plan* P, int kind, int inverse, int rows, int n, const double* in, double* out, cudaStream_t s) {
  if (kind < 0 || kind > 2 || rows < 1 || n < 2) {
    P->err = "transform: invalid kind or shape";
    return MACSAV_ERR_VALUE;
  }
  std::vector<void*> allocs;
  TBlockDev<double> B;
  cudaError_t e = build_line_block<double>(B, rows, n, kind, P->num_sms, allocs);
  double* H = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&H, sizeof(double) * size_t(rows) * B.pitch);
  if (e == cudaSuccess) {
    B.H = H;
    B.hstride = 0;
    RowArgs<double> a = row_args(B, (const TBlockDev<double>*)nullptr, nullptr);
    const size_t sm = size_t(B.px) * B.lsx * sizeof(cplx<double>) * (B.fx.nstages == 0 ? 2 : 1);
    const dim3 og((n + kThreads - 1) / kThreads, rows);
    if (!inverse) {
      auto k = k_row_forward<double, kVmax, SrcCells<double, double>>;
      set_smem(k, sm);
      k<<<dim3(total_groups(a), 1), kFFTThreads, sm, s>>>(a, SrcCells<double, double>{in, 0, n});
      k_ortho_out<<<og, kThreads, 0, s>>>(H, B.pitch, out, rows, n, kind);
    } else {
      k_ortho_in<<<og, kThreads, 0, s>>>(in, H, B.pitch, rows, n, kind);
      auto k = k_row_inverse<double, kVmax, DstCells<double, double>, NoFin>;
      set_smem(k, sm);
      k<<<dim3(total_groups(a), 1), kFFTThreads, sm, s>>>(a, DstCells<double, double>{out, 0, n}, nullptr, NoFin{},
                                                          nullptr);
    }
    P->launches += 2;
    e = cudaStreamSynchronize(s);
  }
  cudaFree(H);
  for (void* p : allocs) cudaFree(p);
  if (e != cudaSuccess) {
    P->err = std::string("CUDA: ") + cudaGetErrorString(e);
    return MACSAV_ERR_CUDA;
  }
  return MACSAV_OK;
}

}  // namespace macsav
