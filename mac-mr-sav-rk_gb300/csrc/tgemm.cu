// Orthonormal DCT-II / DST-II / DST-I along the rows of a (rows, n) FP32
// array as a transform-matrix product on the tcgen05 tensor cores, and the
// per-size choice between it and the shared-memory FFT.
//
// out[r][j] = sum_k in[r][k] B[j][k], with B = T (forward) or T^T (inverse)
// for the orthonormal n x n transform matrix T (the scipy.fft norm="ortho"
// transforms the reference applies along each axis, solver/mac/
// tensor_stokes.py:58-82).  BF16 operands lose FP32 accuracy, so both
// operands are split into S BF16 pieces (x = x0 + x1 + x2, each piece the
// BF16 rounding of what the previous ones left) and the products of pieces
// (i, j) with i + j < S are accumulated in FP32 in tensor memory:
//   S = 2: 3 products, about 16 mantissa bits (relative error ~1e-5);
//   S = 3: 6 products, about 24 bits, the accuracy of an FP32 FFT.
//
// A CTA owns 128 rows and NT outputs (32 <= NT <= 256, chosen so that the
// launch keeps about two CTAs per SM busy; one TMEM accumulator of NT
// columns) and walks K = n in chunks of 32 (two K=16 MMAs per product),
// double-buffered: while the MMAs of chunk c run, all 128 threads stage
// chunk c + 1 (A: coalesced row loads split into BF16 pieces; B: the
// transform pieces, stored in global memory already in the shared-memory
// layout, copied with 16-byte vectors).  Shared-memory operands use the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes): A [k/8][row/8],
// B [k/8][j/8].  One elected thread issues the MMAs and commits them to the
// buffer's mbarrier; the epilogue reads the accumulator with tcgen05.ld (warp
// w owns TMEM lanes 32w..32w+31 = rows).  Waits are bounded: a wait that runs
// out sets *err, waits (bounded) once more for MMAs in flight, frees its
// tensor memory and returns.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "solver.cuh"
#include "../../include/macsav.h"

namespace macsav {

namespace {

constexpr int kTgM = 128;        // rows per CTA
constexpr int kTgK = 32;         // K per chunk
constexpr int kTgMaxN = 256;     // outputs per CTA (one accumulator)
constexpr long long kTgSpin = 1LL << 22;
constexpr int kMaxTensorTransform = 512;  // largest n the tensor-core form takes

__device__ __forceinline__ uint32_t tg_smem(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// no-swizzle K-major matrix descriptor (version 1, base offset 0)
__device__ __forceinline__ uint64_t tg_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;
  return d;
}
__device__ __forceinline__ bool tg_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < kTgSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Element offset of (row, k) in a K-major no-swizzle chunk of `rows8` row
// groups: [k/8][row/8][row%8][k%8].
__device__ __forceinline__ int tg_off(int row, int k, int rows8) {
  return (((k >> 3) * rows8 + (row >> 3)) << 6) + ((row & 7) << 3) + (k & 7);
}

// smem: [2 stages][S pieces A: 128 x 32][S pieces B: NT x 32], BF16.
template <int S>
__global__ void __launch_bounds__(128) k_tgemm(const float* __restrict__ in, float* __restrict__ out, int rows, int n,
                                                int nt, const __nv_bfloat16* __restrict__ bpieces, int nchunks,
                                                int* err) {
  extern __shared__ __align__(1024) unsigned char tg_sm[];
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row0 = blockIdx.x * kTgM, n0 = blockIdx.y * nt;
  const int a_elems = kTgM * kTgK, b_elems = nt * kTgK;
  const int stage_elems = S * (a_elems + b_elems);
  __nv_bfloat16* sm = reinterpret_cast<__nv_bfloat16*>(tg_sm);
  uint32_t cols = 32;
  while (int(cols) < nt) cols <<= 1;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tg_smem(&tmem_slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    failed = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tg_smem(&mbar[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tg_smem(&mbar[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  // instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M = 128, N = nt
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(nt >> 3) << 17) | (uint32_t(kTgM >> 4) << 24);
  const uint32_t a_lbo = (kTgM / 8) * 128, b_lbo = uint32_t(nt / 8) * 128, sbo = 128;
  const long long chunk_b = (long long)S * b_elems;  // elements of one chunk's B pieces in global memory
  const __nv_bfloat16* btile = bpieces + (long long)blockIdx.y * nchunks * chunk_b;

  auto stage = [&](int c, int buf) {
    __nv_bfloat16* A = sm + buf * stage_elems;
    __nv_bfloat16* Bs = A + S * a_elems;
    const int k = c * kTgK + lane;
    // A: each warp stages 32 rows, one row per step, lanes along k (coalesced)
    for (int rr = 0; rr < 32; ++rr) {
      const int row = warp * 32 + rr, r = row0 + row;
      float x = (r < rows && k < n) ? __ldg(in + (long long)r * n + k) : 0.0f;
      const int o = tg_off(row, lane, kTgM / 8);
#pragma unroll
      for (int p = 0; p < S; ++p) {
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        A[p * a_elems + o] = h;
        x -= __bfloat162float(h);
      }
    }
    // B: pieces stored in the chunk layout; 16-byte copies
    const uint4* src = reinterpret_cast<const uint4*>(btile + (long long)c * chunk_b);
    uint4* dst = reinterpret_cast<uint4*>(Bs);
    for (int e = tid; e < int(chunk_b / 8); e += 128) dst[e] = __ldg(src + e);
  };

  stage(0, 0);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  for (int c = 0; c < nchunks; ++c) {
    const int buf = c & 1;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t abase = tg_smem(sm + buf * stage_elems);
      const uint32_t bbase = abase + uint32_t(S * a_elems) * 2;
      int q = 0;
#pragma unroll
      for (int kk = 0; kk < kTgK / 16; ++kk) {
#pragma unroll
        for (int i = 0; i < S; ++i) {
#pragma unroll
          for (int j = 0; j < S - i; ++j) {
            const uint64_t ad = tg_desc(abase + uint32_t(i * a_elems) * 2 + 2 * kk * a_lbo, a_lbo, sbo);
            const uint64_t bd = tg_desc(bbase + uint32_t(j * b_elems) * 2 + 2 * kk * b_lbo, b_lbo, sbo);
            const uint32_t acc = (c > 0 || q > 0) ? 1u : 0u;
            asm volatile(
                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            ++q;
          }
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       tg_smem(&mbar[buf]))
                   : "memory");
    }
    if (c + 1 < nchunks) {
      const int nb = (c + 1) & 1;
      // the MMAs of chunk c - 1 read buffer nb: wait for them before restaging it
      if (c >= 1 && !tg_wait(tg_smem(&mbar[nb]), uint32_t(((c - 1) >> 1) & 1))) failed = 1;
      stage(c + 1, nb);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (failed) break;
  }
  const int last = nchunks - 1;
  const uint32_t last_bar = tg_smem(&mbar[last & 1]), last_par = uint32_t((last >> 1) & 1);
  if (!failed && !tg_wait(last_bar, last_par)) failed = 1;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  __syncthreads();
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
    tg_wait(last_bar, last_par);  // bounded: lets MMAs still in flight finish
  } else {
    const int r = row0 + warp * 32 + lane;
    for (int c0 = 0; c0 < nt; c0 += 16) {
      uint32_t v[16];
      const uint32_t addr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (r < rows) {
        float* o = out + (long long)r * n + n0 + c0;
        const int lim = min(16, n - n0 - c0);
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j < lim) o[j] = __uint_as_float(v[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols));
  }
}

// BF16 rounding (nearest, ties to even) of a float, on the host.
float host_bf16_round(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return x;
  const uint32_t lsb = (u >> 16) & 1u;
  u = (u + 0x7fffu + lsb) & 0xffff0000u;
  float y;
  std::memcpy(&y, &u, 4);
  return y;
}
uint16_t host_bf16_bits(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return uint16_t(u >> 16);
}

// Orthonormal transform matrix entry T[j][k] (scipy.fft norm="ortho").
double ortho_entry(int kind, int n, int j, int k) {
  const double pi = 3.14159265358979323846;
  if (kind == KIND_DCT2) {
    const double f = j == 0 ? std::sqrt(1.0 / (4.0 * n)) : std::sqrt(1.0 / (2.0 * n));
    return 2.0 * f * std::cos(pi * j * (2.0 * k + 1.0) / (2.0 * n));
  }
  if (kind == KIND_DST2) {
    const double f = j == n - 1 ? std::sqrt(1.0 / (4.0 * n)) : std::sqrt(1.0 / (2.0 * n));
    return 2.0 * f * std::sin(pi * (j + 1.0) * (2.0 * k + 1.0) / (2.0 * n));
  }
  return std::sqrt(2.0 / (n + 1.0)) * std::sin(pi * (j + 1.0) * (k + 1.0) / (n + 1.0));
}

}  // namespace

// One size's tensor-core transform: the B pieces in the chunk layout.
struct TGemmPlan {
  int kind = 0, inverse = 0, n = 0, split = 0, nt = 0, ntiles = 0, nchunks = 0;
  __nv_bfloat16* pieces = nullptr;
};

// nt: the outputs per CTA (a multiple of 16, 32..256), chosen by the caller
// so that the launch has enough CTAs for the rows it transforms.
static int tgemm_build(TGemmPlan& G, int kind, int inverse, int n, int split, int nt) {
  G.kind = kind;
  G.inverse = inverse;
  G.n = n;
  G.split = split;
  const int n16 = (n + 15) / 16 * 16;
  G.ntiles = (n16 + nt - 1) / nt;
  G.nt = ((n16 + G.ntiles - 1) / G.ntiles + 15) / 16 * 16;
  G.nchunks = (n + kTgK - 1) / kTgK;
  const long long per_chunk = (long long)split * G.nt * kTgK;
  std::vector<uint16_t> host(size_t(G.ntiles) * G.nchunks * per_chunk, 0);
  for (int t = 0; t < G.ntiles; ++t)
    for (int c = 0; c < G.nchunks; ++c)
      for (int jj = 0; jj < G.nt; ++jj)
        for (int kk = 0; kk < kTgK; ++kk) {
          const int j = t * G.nt + jj, k = c * kTgK + kk;
          if (j >= n || k >= n) continue;
          double rest = inverse ? ortho_entry(kind, n, k, j) : ortho_entry(kind, n, j, k);
          for (int p = 0; p < split; ++p) {
            const float h = host_bf16_round(float(rest));
            const long long base = ((long long)(t * G.nchunks + c) * split + p) * G.nt * kTgK;
            const int off = (((kk >> 3) * (G.nt / 8) + (jj >> 3)) << 6) + ((jj & 7) << 3) + (kk & 7);
            host[size_t(base + off)] = host_bf16_bits(h);
            rest -= double(h);
          }
        }
  if (cudaMalloc(&G.pieces, host.size() * sizeof(uint16_t)) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMemcpy(G.pieces, host.data(), host.size() * sizeof(uint16_t), cudaMemcpyHostToDevice) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  return MACSAV_OK;
}

static size_t tgemm_smem(int split, int nt) {
  return size_t(2) * split * (kTgM * kTgK + nt * kTgK) * sizeof(__nv_bfloat16);
}

static int tgemm_run(const TGemmPlan& G, const float* in, float* out, int rows, int* err, cudaStream_t s) {
  const size_t sm = tgemm_smem(G.split, G.nt);
  const dim3 grid((rows + kTgM - 1) / kTgM, G.ntiles);
  if (G.split == 2) {
    cudaFuncSetAttribute(k_tgemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_tgemm<2><<<grid, 128, sm, s>>>(in, out, rows, G.n, G.nt, G.pieces, G.nchunks, err);
  } else {
    cudaFuncSetAttribute(k_tgemm<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
    k_tgemm<3><<<grid, 128, sm, s>>>(in, out, rows, G.n, G.nt, G.pieces, G.nchunks, err);
  }
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// ---------------------------------------------- FFT path (FP32, rows) ---
template <typename T>
cudaError_t build_line_block(TBlockDev<T>& B, int rows, int cols, int kx, int sms, std::vector<void*>& allocs);

__global__ void k_ortho_out32(const float* H, int pitch, float* out, int rows, int n, int kind) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
  if (k >= n || row >= rows) return;
  const float v = H[(long long)row * pitch + k];
  if (kind == KIND_DST1) {
    out[(long long)row * n + k] = v * sqrtf(2.0f / (n + 1));
  } else {
    const float sc = k == 0 ? sqrtf(1.0f / (4.0f * n)) : sqrtf(1.0f / (2.0f * n));
    out[(long long)row * n + (kind == KIND_DST2 ? n - 1 - k : k)] = v * sc;
  }
}
__global__ void k_ortho_in32(const float* in, float* H, int pitch, int rows, int n, int kind) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, row = blockIdx.y;
  if (k >= n || row >= rows) return;
  float v;
  if (kind == KIND_DST1) {
    v = in[(long long)row * n + k] * sqrtf((n + 1) / 2.0f);
  } else {
    const float sc = k == 0 ? sqrtf(4.0f * n) : sqrtf(2.0f * n);
    v = in[(long long)row * n + (kind == KIND_DST2 ? n - 1 - k : k)] * sc;
  }
  H[(long long)row * pitch + k] = v;
}

struct FFTLine32 {
  TBlockDev<float> B;
  float* H = nullptr;
  std::vector<void*> allocs;
  int rows = 0, n = 0, kind = 0;
};

static int fft32_build(FFTLine32& F, int kind, int rows, int n, int sms) {
  F.kind = kind;
  F.rows = rows;
  F.n = n;
  cudaError_t e = build_line_block<float>(F.B, rows, n, kind, sms, F.allocs);
  if (e == cudaSuccess) e = cudaMalloc(&F.H, sizeof(float) * size_t(rows) * F.B.pitch);
  if (e != cudaSuccess) return MACSAV_ERR_CUDA;
  F.B.H = F.H;
  F.B.hstride = 0;
  return MACSAV_OK;
}

static int fft32_run(const FFTLine32& F, int inverse, const float* in, float* out, cudaStream_t s) {
  RowArgs<float> a = row_args(F.B, (const TBlockDev<float>*)nullptr, nullptr);
  const size_t sm = size_t(F.B.px) * F.B.lsx * sizeof(cplx<float>) * (F.B.fx.nstages == 0 ? 2 : 1);
  const dim3 og((F.n + kThreads - 1) / kThreads, F.rows);
  if (!inverse) {
    auto k = k_row_forward<float, kVmax, SrcCells<float, float>>;
    set_smem(k, sm);
    k<<<dim3(total_groups(a), 1), kFFTThreads, sm, s>>>(a, SrcCells<float, float>{in, 0, F.n});
    k_ortho_out32<<<og, kThreads, 0, s>>>(F.H, F.B.pitch, out, F.rows, F.n, F.kind);
  } else {
    k_ortho_in32<<<og, kThreads, 0, s>>>(in, F.H, F.B.pitch, F.rows, F.n, F.kind);
    auto k = k_row_inverse<float, kVmax, DstCells<float, float>, NoFin>;
    set_smem(k, sm);
    k<<<dim3(total_groups(a), 1), kFFTThreads, sm, s>>>(a, DstCells<float, float>{out, 0, F.n}, nullptr, NoFin{},
                                                        nullptr);
  }
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// ------------------------------------------------ per-plan cache, autotune ---
struct Transform32Cache {
  std::map<std::tuple<int, int, int, int, int>, TGemmPlan> gemm;  // (kind, inverse, n, split, nt)
  std::map<std::tuple<int, int, int>, FFTLine32*> fft;            // (kind, rows, n)
  std::map<std::tuple<int, int, int, int>, int> choice;           // (kind, inverse, rows, n) -> method
  int* err = nullptr;
  ~Transform32Cache() {
    for (auto& kv : gemm) cudaFree(kv.second.pieces);
    for (auto& kv : fft) {
      cudaFree(kv.second->H);
      for (void* p : kv.second->allocs) cudaFree(p);
      delete kv.second;
    }
    cudaFree(err);
  }
};

static Transform32Cache& cache_of(Plan* P) {
  if (!P->tcache) P->tcache = new Transform32Cache();
  return *P->tcache;
}

void free_transform32_cache(Plan* P) {
  delete P->tcache;
  P->tcache = nullptr;
}

static int run_method(Plan* P, int kind, int inverse, int rows, int n, int method, const float* in, float* out,
                      cudaStream_t s) {
  Transform32Cache& C = cache_of(P);
  if (!C.err) {
    if (cudaMalloc(&C.err, sizeof(int)) != cudaSuccess || cudaMemset(C.err, 0, sizeof(int)) != cudaSuccess)
      return MACSAV_ERR_CUDA;
  }
  if (method == MACSAV_TRANSFORM_FFT) {
    auto key = std::make_tuple(kind, rows, n);
    auto it = C.fft.find(key);
    if (it == C.fft.end()) {
      FFTLine32* F = new FFTLine32();
      const int rc = fft32_build(*F, kind, rows, n, P->num_sms);
      if (rc != MACSAV_OK) {
        cudaFree(F->H);
        for (void* p : F->allocs) cudaFree(p);
        delete F;
        return rc;
      }
      it = C.fft.emplace(key, F).first;
    }
    P->launches += 2;
    return fft32_run(*it->second, inverse, in, out, s);
  }
  const int split = method == MACSAV_TRANSFORM_TC3 ? 2 : 3;
  // outputs per CTA: as many as keep about two CTAs per SM busy, 32..256
  const int row_tiles = (rows + kTgM - 1) / kTgM;
  const int want_tiles = (2 * P->num_sms + row_tiles - 1) / row_tiles;
  const int n16 = (n + 15) / 16 * 16;
  int nt = ((n16 + want_tiles - 1) / want_tiles + 15) / 16 * 16;
  nt = nt < 32 ? 32 : (nt > kTgMaxN ? kTgMaxN : nt);
  auto key = std::make_tuple(kind, inverse, n, split, nt);
  auto it = C.gemm.find(key);
  if (it == C.gemm.end()) {
    TGemmPlan G;
    const int rc = tgemm_build(G, kind, inverse, n, split, nt);
    if (rc != MACSAV_OK) {
      cudaFree(G.pieces);
      return rc;
    }
    it = C.gemm.emplace(key, G).first;
  }
  ++P->launches;
  return tgemm_run(it->second, in, out, rows, C.err, s);
}

int op_transform32_autotune(Plan* P, int kind, int inverse, int rows, int n, int* method, double* ms_fft,
                            double* ms_tensor, cudaStream_t s);

int op_transform32(Plan* P, int kind, int inverse, int rows, int n, int method, const float* in, float* out,
                   cudaStream_t s) {
  if (kind < 0 || kind > 2 || rows < 1 || n < 2 || method < 0 || method > MACSAV_TRANSFORM_AUTO) {
    P->err = "transform32: invalid kind, shape or method";
    return MACSAV_ERR_VALUE;
  }
  if (method == MACSAV_TRANSFORM_AUTO) {
    // the autotuner's choice for this size, measured on first use
    auto& choice = cache_of(P).choice;
    auto it = choice.find(std::make_tuple(kind, inverse, rows, n));
    if (it != choice.end()) {
      method = it->second;
    } else {
      int chosen = MACSAV_TRANSFORM_FFT;
      double a = 0, b = 0;
      const int rc = op_transform32_autotune(P, kind, inverse, rows, n, &chosen, &a, &b, s);
      if (rc != MACSAV_OK) return rc;
      method = chosen;
    }
  }
  if (method != MACSAV_TRANSFORM_FFT && n > kMaxTensorTransform) {
    P->err = "transform32: the tensor-core form takes n <= 512";
    return MACSAV_ERR_UNSUPPORTED;
  }
  int rc = run_method(P, kind, inverse, rows, n, method, in, out, s);
  if (rc != MACSAV_OK) return rc;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MACSAV_ERR_CUDA;
  int h_err = 0;
  cudaMemcpy(&h_err, cache_of(P).err, sizeof(int), cudaMemcpyDeviceToHost);
  if (h_err) {
    P->err = "transform32: a tensor-core wait ran out";
    cudaMemset(cache_of(P).err, 0, sizeof(int));
    return MACSAV_ERR_CUDA;
  }
  return MACSAV_OK;
}

// Average device time of `reps` launches of one method, after a warm-up.
static int time_method(Plan* P, int kind, int inverse, int rows, int n, int method, const float* in, float* out,
                       int reps, cudaStream_t s, double* ms) {
  int rc = run_method(P, kind, inverse, rows, n, method, in, out, s);
  if (rc != MACSAV_OK) return rc;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s);
  for (int k = 0; k < reps && rc == MACSAV_OK; ++k) rc = run_method(P, kind, inverse, rows, n, method, in, out, s);
  cudaEventRecord(b, s);
  cudaEventSynchronize(b);
  float t = 0;
  cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = double(t) / reps;
  return rc;
}

int op_transform32_autotune(Plan* P, int kind, int inverse, int rows, int n, int* method, double* ms_fft,
                            double* ms_tensor, cudaStream_t s) {
  if (kind < 0 || kind > 2 || rows < 1 || n < 2) {
    P->err = "transform32: invalid kind or shape";
    return MACSAV_ERR_VALUE;
  }
  Transform32Cache& C = cache_of(P);
  auto key = std::make_tuple(kind, inverse, rows, n);
  float *in = nullptr, *out = nullptr;
  const size_t bytes = sizeof(float) * size_t(rows) * n;
  if (cudaMalloc(&in, bytes) != cudaSuccess || cudaMalloc(&out, bytes) != cudaSuccess) {
    cudaFree(in);
    return MACSAV_ERR_CUDA;
  }
  cudaMemsetAsync(in, 0, bytes, s);
  *ms_fft = *ms_tensor = -1.0;
  int rc = time_method(P, kind, inverse, rows, n, MACSAV_TRANSFORM_FFT, in, out, 10, s, ms_fft);
  int best = MACSAV_TRANSFORM_FFT;
  if (rc == MACSAV_OK && n <= kMaxTensorTransform) {
    rc = time_method(P, kind, inverse, rows, n, MACSAV_TRANSFORM_TC6, in, out, 10, s, ms_tensor);
    if (rc == MACSAV_OK && *ms_tensor < *ms_fft) best = MACSAV_TRANSFORM_TC6;
  }
  cudaStreamSynchronize(s);
  cudaFree(in);
  cudaFree(out);
  if (rc != MACSAV_OK) return rc;
  C.choice[key] = best;
  *method = best;
  return MACSAV_OK;
}

}  // namespace macsav
