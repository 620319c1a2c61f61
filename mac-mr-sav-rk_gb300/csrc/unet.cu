// U-Net kernels: BF16 activations, FP32 accumulation, forward and backward
// (layout and architecture in unet.cuh).  Convolutions are direct: a CTA
// stages a 16x16 pixel tile (plus halo) of 8 input channels and their weights
// in shared memory and each thread accumulates 16 output channels of one
// pixel.  The data gradient is the same kernel on the flipped, transposed
// weights; the weight gradient reduces tile products and adds them atomically.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "unet.cuh"
#include "common.cuh"
#include "../../include/macsav.h"

namespace macsav {

namespace {

constexpr int kTile = 16;
constexpr int kCT = 16;  // output channels per CTA
constexpr int kCI = 8;   // input channels per shared-memory chunk
constexpr int kWO = 8, kWI = 8;  // weight-gradient CTA: output x input channels

__device__ __forceinline__ float bf2f(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ __nv_bfloat16 f2bf(float v) { return __float2bfloat16_rn(v); }

struct ConvArgs {
  const __nv_bfloat16* xa;  // forward input channels [0, ca)   [B][ca][H][W]
  const __nv_bfloat16* xb;  // forward input channels [ca, ca+cb) [B][cb][H][W]
  int ca, cb, co;
  const float* dy;          // backward: masked output gradient [B][co][H][W]
  const __nv_bfloat16* w;   // [co][ca+cb][ks*ks]
  const __nv_bfloat16* wp;  // the tensor-core operand copy of w (k_conv3_tc), per chunk
  __nv_bfloat16* yb;        // forward output (BF16) or
  float* yf;                // forward output (FP32)
  float* ga;                // backward: input gradient of channels [0, ca)
  float* gb;                // backward: input gradient of channels [ca, ca+cb)
  const float* out_scale;   // forward: per-sample output factor (or null)
  int relu, B, H, W;
  int tc_group;             // k_conv3_tc: input-channel chunks staged together (shared memory per group)
};

// FWD: out[o](p) = sum_i sum_k w[o][i][k] x[i](p + d_k)
// BWD: gx[i](p) = sum_o sum_k w[o][i][k] dy[o](p - d_k)   (d_k: tap offset)
template <int KS, bool BWD>
__global__ void __launch_bounds__(256) k_conv(ConvArgs q) {
  pdl_wait();
  constexpr int R = KS / 2, KK = KS * KS, SW = kTile + 2 * R;
  __shared__ float xs[kCI][SW][SW];
  __shared__ __align__(16) float wsh[kCI][KK][kCT];
  const int cin = BWD ? q.co : q.ca + q.cb;
  const int cout = BWD ? q.ca + q.cb : q.co;
  const int ntile_o = (cout + kCT - 1) / kCT;
  const int b = blockIdx.z / ntile_o, o0 = (blockIdx.z - b * ntile_o) * kCT;
  const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
  const int H = q.H, W = q.W;
  const long long HW = (long long)H * W;
  float acc[kCT];
#pragma unroll
  for (int o = 0; o < kCT; ++o) acc[o] = 0.f;
  for (int i0 = 0; i0 < cin; i0 += kCI) {
    __syncthreads();
    for (int e = threadIdx.x; e < kCI * SW * SW; e += blockDim.x) {
      const int ci = e / (SW * SW), rem = e - ci * SW * SW, yy = rem / SW, xx = rem - yy * SW;
      const int i = i0 + ci, gy = y0 + yy - R, gx = x0 + xx - R;
      float v = 0.f;
      if (i < cin && gy >= 0 && gy < H && gx >= 0 && gx < W) {
        const long long off = (long long)gy * W + gx;
        if (BWD) v = q.dy[((long long)b * cin + i) * HW + off];
        else v = i < q.ca ? bf2f(q.xa[((long long)b * q.ca + i) * HW + off])
                          : bf2f(q.xb[((long long)b * q.cb + (i - q.ca)) * HW + off]);
      }
      xs[ci][yy][xx] = v;
    }
    for (int e = threadIdx.x; e < kCI * KK * kCT; e += blockDim.x) {
      const int ci = e / (KK * kCT), rem = e - ci * KK * kCT, k = rem / kCT, o = rem - k * kCT;
      const int i = i0 + ci, oo = o0 + o;
      float v = 0.f;
      if (i < cin && oo < cout)
        v = BWD ? bf2f(q.w[((long long)i * cout + oo) * KK + (KK - 1 - k)])
                : bf2f(q.w[((long long)oo * cin + i) * KK + k]);
      wsh[ci][k][o] = v;
    }
    __syncthreads();
#pragma unroll 2
    for (int ci = 0; ci < kCI; ++ci) {
#pragma unroll
      for (int k = 0; k < KK; ++k) {
        const float xv = xs[ci][ty + k / KS][tx + k % KS];
        const float4* wp = reinterpret_cast<const float4*>(&wsh[ci][k][0]);
#pragma unroll
        for (int o4 = 0; o4 < kCT / 4; ++o4) {
          const float4 w4 = wp[o4];
          acc[4 * o4 + 0] = fmaf(w4.x, xv, acc[4 * o4 + 0]);
          acc[4 * o4 + 1] = fmaf(w4.y, xv, acc[4 * o4 + 1]);
          acc[4 * o4 + 2] = fmaf(w4.z, xv, acc[4 * o4 + 2]);
          acc[4 * o4 + 3] = fmaf(w4.w, xv, acc[4 * o4 + 3]);
        }
      }
    }
  }
  const int gx = x0 + tx, gy = y0 + ty;
  if (gx >= W || gy >= H) return;
  const long long off = (long long)gy * W + gx;
#pragma unroll
  for (int o = 0; o < kCT; ++o) {
    const int oo = o0 + o;
    if (oo >= cout) break;
    float v = acc[o];
    if (BWD) {
      if (oo < q.ca) q.ga[((long long)b * q.ca + oo) * HW + off] = v;
      else q.gb[((long long)b * q.cb + (oo - q.ca)) * HW + off] = v;
    } else {
      if (q.relu) v = fmaxf(v, 0.f);
      if (q.out_scale) v *= q.out_scale[b];
      if (q.yf) q.yf[((long long)b * cout + oo) * HW + off] = v;
      else q.yb[((long long)b * cout + oo) * HW + off] = f2bf(v);
    }
  }
}

// ------------------------------------------- tcgen05 implicit-GEMM conv ---
// Forward 3x3 convolution on the 5th-generation tensor cores (tcgen05.mma,
// kind::f16 with BF16 A and B, FP32 accumulation in tensor memory) as nine
// shifted GEMMs per 16-channel chunk: D[128 px, co] += A_t[128 px, 16 ci] .
// B_t[co, 16 ci]^T for the taps t, with no im2col.  A CTA of 128 threads owns
// a 16x8 pixel tile (rows y0.., columns x0..) of one image and all co (16, 32
// or 64).  Per chunk its threads stage the 18x10 halo of 16 channels in shared
// memory as [channel group of 8][halo pixel][8 channels], so that for tap
// (dy, dx) the operand A_t is the no-swizzle K-major core-matrix layout
// starting at halo pixel (dy, dx): 8 consecutive pixels of a tile row form a
// core matrix (16 B rows), SBO = 10 pixels * 16 B = 160 B steps one tile row,
// LBO = 180 pixels * 16 B = 2880 B steps to the next 8 channels.  B_t is
// staged as [tap][co/8][2][8 rows x 16 B] (SBO 256 B, LBO 128 B).  The chunks
// are staged in groups (as many as the opt-in shared memory holds, all of
// this network's layers in one group): every load of a group is in flight
// together, then one elected thread issues the group's 9 x chunks MMAs and
// commits them to one mbarrier, and all threads wait (bounded) before the
// tiles are reused, so a deep layer pays one load latency and one wait
// instead of one per chunk.  The epilogue reads accumulator
// rows with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile pixels),
// applies ReLU and stores BF16.  On a wait that runs out the kernel sets
// *err, waits (bounded) once more, frees its tensor memory and returns.
constexpr int kTcC = 16;                          // input channels per chunk (K of one MMA)
constexpr int kTcHx = 10, kTcHy = 18;             // halo columns / rows
constexpr int kTcHalo = kTcHx * kTcHy;            // 180 halo pixels
constexpr uint32_t kTcALBO = kTcHalo * 16;        // 2880: next 8 channels
constexpr uint32_t kTcASBO = kTcHx * 16;          // 160: next tile row
constexpr uint32_t kTcBLBO = 128, kTcBSBO = 256;  // B: next 8 channels / next 8 rows
constexpr size_t kTcSmemHalo = size_t(2) * kTcHalo * 16;  // 5760
constexpr long long kTcSpin = 1LL << 22;          // mbarrier poll limit

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// no-swizzle K-major shared-memory matrix descriptor (version 1, base offset 0)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFF);
  d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
  d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
  d |= uint64_t(1) << 46;
  return d;
}
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < kTcSpin; ++it) {
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

__global__ void __launch_bounds__(128, 5) k_conv3_tc(ConvArgs q, int* err) {
  pdl_wait();
  extern __shared__ __align__(1024) unsigned char tcsm[];
  __shared__ __align__(8) unsigned long long mbar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = q.co, cin = q.ca + q.cb, nchunks = (cin + kTcC - 1) / kTcC;
  const int H = q.H, W = q.W;
  const long long HW = (long long)H * W;
  const int b = blockIdx.z, x0 = blockIdx.x * 8, y0 = blockIdx.y * 16;
  // tensor-memory columns: the accumulator's N (a power of two, at least 32),
  // so that more CTAs of a small layer fit an SM's 512 columns
  const uint32_t kCols = N <= 32 ? 32u : 64u;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    failed = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t mb = smem_u32(&mbar);
  // instruction descriptor: FP32 accumulator, BF16 A and B, K-major, M=128, N
  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(128 >> 4) << 24);
  const uint32_t btap = uint32_t(N >> 3) * kTcBSBO;  // bytes of one tap's B tile
  // the chunks of a group are all staged (every load of the group in flight
  // at once), then all their MMAs issued under one commit and one wait
  const int per_chunk = int(kTcSmemHalo) + 9 * int(btap);
  const int group = q.tc_group;
  uint32_t phase = 0;
  const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
  for (int g0 = 0; g0 < nchunks; g0 += group) {
    const int gn = min(group, nchunks - g0);
    for (int cc = 0; cc < gn; ++cc) {
      const int ch = g0 + cc;
      const int ci0 = ch * kTcC;
      __nv_bfloat16* halo = reinterpret_cast<__nv_bfloat16*>(tcsm + cc * per_chunk);
      unsigned char* Bs = tcsm + cc * per_chunk + kTcSmemHalo;
      // halo [c/8][pixel][c%8] of the chunk's channels (zero outside the image /
      // cin), in two halves whose loads are all issued before their stores
      constexpr int kHaloPer = (kTcC * kTcHalo + 127) / 128, kHalf = (kHaloPer + 1) / 2;
  #pragma unroll
      for (int h0 = 0; h0 < kHaloPer; h0 += kHalf) {
        __nv_bfloat16 hv[kHalf];
  #pragma unroll
        for (int k = 0; k < kHalf; ++k) {
          const int e = tid + (h0 + k) * 128;
          const int c = e / kTcHalo, pix = e - c * kTcHalo, hy = pix / kTcHx, hx = pix - hy * kTcHx;
          const int ci = ci0 + c, gy = y0 + hy - 1, gx = x0 + hx - 1;
          hv[k] = zero;
          if (h0 + k < kHaloPer && e < kTcC * kTcHalo && ci < cin && gy >= 0 && gy < H && gx >= 0 && gx < W) {
            const long long off = (long long)gy * W + gx;
            hv[k] = ci < q.ca ? __ldg(q.xa + ((long long)b * q.ca + ci) * HW + off)
                              : __ldg(q.xb + ((long long)b * q.cb + (ci - q.ca)) * HW + off);
          }
        }
  #pragma unroll
        for (int k = 0; k < kHalf; ++k) {
          const int e = tid + (h0 + k) * 128;
          if (h0 + k < kHaloPer && e < kTcC * kTcHalo) {
            const int c = e / kTcHalo, pix = e - c * kTcHalo;
            halo[((c >> 3) * kTcHalo + pix) * 8 + (c & 7)] = hv[k];
          }
        }
      }
      // B_t[co][c] = w[co][ci0 + c][t]: the chunk's operand copy, already in
      // the [tap][co/8][2][8 rows][8 channels] layout, 16 bytes per copy
      {
        const uint4* src = reinterpret_cast<const uint4*>(q.wp) + (long long)ch * 9 * N * 2;
        uint4* dst = reinterpret_cast<uint4*>(Bs);
        for (int e = tid; e < 9 * N * 2; e += 128) dst[e] = __ldg(src + e);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int cc = 0; cc < gn; ++cc) {
        const uint32_t halo_s = smem_u32(tcsm + cc * per_chunk), b_s = halo_s + uint32_t(kTcSmemHalo);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
          const uint32_t a_start = halo_s + uint32_t((t / 3) * kTcHx + (t % 3)) * 16;
          const uint64_t ad = tc_desc(a_start, kTcALBO, kTcASBO);
          const uint64_t bd = tc_desc(b_s + t * btap, kTcBLBO, kTcBSBO);
          const uint32_t acc = (g0 + cc > 0 || t > 0) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
                   : "memory");
    }
    if (!tc_wait(mb, phase)) failed = 1;
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (failed) break;
  }
  if (failed) {
    if (tid == 0) atomicExch(err, 1);
    tc_wait(mb, phase);  // bounded: lets an MMA still in flight finish
  } else {
    // epilogue: lane p = tile pixel (row p/8, column p%8), columns are co
    const int p = warp * 32 + lane;
    const int gy = y0 + (p >> 3), gx = x0 + (p & 7);
    const bool inside = gy < H && gx < W;
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (inside) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float v = __uint_as_float(r[j]);
          if (q.relu) v = fmaxf(v, 0.f);
          if (q.out_scale) v *= q.out_scale[b];
          q.yb[((long long)b * N + c0 + j) * HW + (long long)gy * W + gx] = f2bf(v);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols));
  }
}

// dw[o][i][k] += sum_b sum_p dy[b][o](p) x[b][i](p + d_k); each CTA covers
// kWO x kWI channel pairs and a stride of pixel tiles.
template <int KS>
__global__ void __launch_bounds__(256) k_conv_wgrad(ConvArgs q, int tiles_x, int tiles_y, float* dw) {
  constexpr int R = KS / 2, KK = KS * KS, SW = kTile + 2 * R;
  constexpr int E = kWO * kWI * KK;
  constexpr int PER = (E + 255) / 256;
  __shared__ float xs[kWI][SW][SW];
  __shared__ float ds[kWO][kTile][kTile];
  const int cin = q.ca + q.cb, cout = q.co;
  const int nti = (cin + kWI - 1) / kWI;
  const int o0 = (blockIdx.x / nti) * kWO, i0 = (blockIdx.x - (blockIdx.x / nti) * nti) * kWI;
  const int H = q.H, W = q.W;
  const long long HW = (long long)H * W;
  const int per_img = tiles_x * tiles_y, ntiles = per_img * q.B;
  float acc[PER];
#pragma unroll
  for (int r = 0; r < PER; ++r) acc[r] = 0.f;
  for (int t = blockIdx.y; t < ntiles; t += gridDim.y) {
    const int b = t / per_img, tt = t - b * per_img;
    const int y0 = (tt / tiles_x) * kTile, x0 = (tt - (tt / tiles_x) * tiles_x) * kTile;
    __syncthreads();
    for (int e = threadIdx.x; e < kWI * SW * SW; e += blockDim.x) {
      const int ci = e / (SW * SW), rem = e - ci * SW * SW, yy = rem / SW, xx = rem - yy * SW;
      const int i = i0 + ci, gy = y0 + yy - R, gx = x0 + xx - R;
      float v = 0.f;
      if (i < cin && gy >= 0 && gy < H && gx >= 0 && gx < W) {
        const long long off = (long long)gy * W + gx;
        v = i < q.ca ? bf2f(q.xa[((long long)b * q.ca + i) * HW + off])
                     : bf2f(q.xb[((long long)b * q.cb + (i - q.ca)) * HW + off]);
      }
      xs[ci][yy][xx] = v;
    }
    for (int e = threadIdx.x; e < kWO * kTile * kTile; e += blockDim.x) {
      const int co = e / (kTile * kTile), rem = e - co * kTile * kTile, yy = rem / kTile, xx = rem - yy * kTile;
      const int o = o0 + co, gy = y0 + yy, gx = x0 + xx;
      float v = 0.f;
      if (o < cout && gy < H && gx < W) v = q.dy[((long long)b * cout + o) * HW + (long long)gy * W + gx];
      ds[co][yy][xx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PER; ++r) {
      const int e = threadIdx.x + r * 256;
      if (e < E) {
        const int o = e / (kWI * KK), rem = e - o * kWI * KK, i = rem / KK, k = rem - i * KK;
        const int ky = k / KS, kx = k - ky * KS;
        float s = 0.f;
        for (int py = 0; py < kTile; ++py)
#pragma unroll 4
          for (int px = 0; px < kTile; ++px) s = fmaf(ds[o][py][px], xs[i][py + ky][px + kx], s);
        acc[r] += s;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const int e = threadIdx.x + r * 256;
    if (e < E) {
      const int o = e / (kWI * KK), rem = e - o * kWI * KK, i = rem / KK, k = rem - i * KK;
      if (o0 + o < cout && i0 + i < cin) atomicAdd(&dw[((long long)(o0 + o) * cin + (i0 + i)) * KK + k], acc[r]);
    }
  }
}

__global__ void k_to_bf16(const float* in, const float* scale, long long hw, int batch, __nv_bfloat16* out) {
  pdl_wait();
  const long long n = hw * batch;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int b = int(e / hw);
    out[e] = f2bf(scale ? in[e] * scale[b] : in[e]);
  }
}

// 2x2 average pool of [planes][H][W] to [planes][H/2][W/2]
__global__ void k_pool(const __nv_bfloat16* x, __nv_bfloat16* y, long long planes, int H, int W) {
  pdl_wait();
  const int h = H / 2, w = W / 2;
  const long long n = planes * h * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pl = e / ((long long)h * w);
    const int rem = int(e - pl * h * w), yy = rem / w, xx = rem - yy * w;
    const __nv_bfloat16* s = x + pl * H * W + (long long)(2 * yy) * W + 2 * xx;
    y[e] = f2bf(0.25f * (bf2f(s[0]) + bf2f(s[1]) + bf2f(s[W]) + bf2f(s[W + 1])));
  }
}
// gx[fine] += 0.25 gy[coarse]
__global__ void k_pool_bwd(const float* gy, float* gx, long long planes, int H, int W) {
  const long long n = planes * H * W;
  const int h = H / 2, w = W / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pl = e / ((long long)H * W);
    const int rem = int(e - pl * H * W), yy = rem / W, xx = rem - yy * W;
    gx[e] += 0.25f * gy[pl * h * w + (long long)(yy / 2) * w + xx / 2];
  }
}
// nearest 2x upsample of [planes][h][w] to [planes][2h][2w]
__global__ void k_up(const __nv_bfloat16* x, __nv_bfloat16* y, long long planes, int H, int W) {
  pdl_wait();
  const long long n = planes * H * W;
  const int h = H / 2, w = W / 2;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pl = e / ((long long)H * W);
    const int rem = int(e - pl * H * W), yy = rem / W, xx = rem - yy * W;
    y[e] = x[pl * h * w + (long long)(yy / 2) * w + xx / 2];
  }
}
// gx[coarse] = sum of the four fine gradients
__global__ void k_up_bwd(const float* gy, float* gx, long long planes, int H, int W) {
  const int h = H / 2, w = W / 2;
  const long long n = planes * h * w;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pl = e / ((long long)h * w);
    const int rem = int(e - pl * h * w), yy = rem / w, xx = rem - yy * w;
    const float* s = gy + pl * H * W + (long long)(2 * yy) * W + 2 * xx;
    gx[e] = s[0] + s[1] + s[W] + s[W + 1];
  }
}
// g = 0 where the ReLU output was not positive
__global__ void k_relu_mask(float* g, const __nv_bfloat16* y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    if (!(bf2f(y[e]) > 0.f)) g[e] = 0.f;
}
// loss += sum (y - t)^2 / n; gy = 2 (y - t) / n
__global__ void k_mse(const float* y, const float* t, float* gy, long long n, double* loss) {
  __shared__ float red[32];
  float s = 0.f;
  const float inv = 1.0f / float(n);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float d = y[e] - t[e];
    gy[e] = 2.f * d * inv;
    s += d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < int(blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) atomicAdd(loss, double(s) / double(n));
  }
}
__global__ void k_adam(float* w, float* g, float* m1, float* m2, __nv_bfloat16* wb, long long n, float lr, float b1,
                       float b2, float c1, float c2, float eps) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gv = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * gv;
    const float v = b2 * m2[e] + (1.f - b2) * gv * gv;
    m1[e] = a;
    m2[e] = v;
    const float wn = w[e] - lr * (a / c1) / (sqrtf(v / c2) + eps);
    w[e] = wn;
    wb[e] = f2bf(wn);
    g[e] = 0.f;
  }
}
// The tensor-core operand copy of one 3x3 layer: element e of chunk ch, tap
// t, row group rg, channel group kg, row r8, channel c8 is
// w[row = 8 rg + r8][ci = 16 ch + 8 kg + c8][t] (zero beyond cin).
__global__ void k_pack_w3(const __nv_bfloat16* w, __nv_bfloat16* wp, int co, int cin, long long total) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c8 = int(e & 7), r8 = int((e >> 3) & 7), kg = int((e >> 6) & 1);
    long long rest = e >> 7;
    const int rg = int(rest % (co / 8));
    rest /= (co / 8);
    const int t = int(rest % 9), ch = int(rest / 9);
    const int row = rg * 8 + r8, ci = ch * 16 + kg * 8 + c8;
    wp[e] = ci < cin ? w[((long long)row * cin + ci) * 9 + t] : __float2bfloat16_rn(0.f);
  }
}

__global__ void k_sync_bf16(const float* w, __nv_bfloat16* wb, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    wb[e] = f2bf(w[e]);
}

inline int grid1(long long n) {
  long long b = (n + 255) / 256;
  return int(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

// Buffer table of one workspace: forward BF16 activations, then (when sized
// for training) FP32 gradients of the same shapes.
struct Bufs {
  __nv_bfloat16 *x0, *a[kNetLevels], *e[kNetLevels], *p[kNetLevels - 1], *u[kNetLevels - 1], *d[kNetLevels - 1];
  float *y, *gy, *ga[kNetLevels], *ge[kNetLevels], *gp[kNetLevels - 1], *gu[kNetLevels - 1], *gd[kNetLevels - 1];
};

size_t layout(const UNet* N, int B, int ny, int nx, bool grad, char* base, Bufs* out) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char* {
    char* p = base ? base + off : nullptr;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  long long pix[kNetLevels];
  for (int l = 0; l < kNetLevels; ++l) pix[l] = (long long)B * (ny >> l) * (nx >> l);
  const int* c = N->ch;
  auto cu = [&](int l) { return l == kNetLevels - 2 ? c[kNetLevels - 1] : c[l + 1]; };
  Bufs b{};
  const size_t h2 = sizeof(__nv_bfloat16), f4 = sizeof(float);
  b.x0 = reinterpret_cast<__nv_bfloat16*>(take(pix[0] * h2));
  for (int l = 0; l < kNetLevels; ++l) {
    b.a[l] = reinterpret_cast<__nv_bfloat16*>(take(c[l] * pix[l] * h2));
    b.e[l] = reinterpret_cast<__nv_bfloat16*>(take(c[l] * pix[l] * h2));
  }
  for (int l = 0; l + 1 < kNetLevels; ++l) {
    b.p[l] = reinterpret_cast<__nv_bfloat16*>(take(c[l] * pix[l + 1] * h2));
    b.u[l] = reinterpret_cast<__nv_bfloat16*>(take(cu(l) * pix[l] * h2));
    b.d[l] = reinterpret_cast<__nv_bfloat16*>(take(c[l] * pix[l] * h2));
  }
  if (grad) {
    b.y = reinterpret_cast<float*>(take(pix[0] * f4));
    b.gy = reinterpret_cast<float*>(take(pix[0] * f4));
    for (int l = 0; l < kNetLevels; ++l) {
      b.ga[l] = reinterpret_cast<float*>(take(c[l] * pix[l] * f4));
      b.ge[l] = reinterpret_cast<float*>(take(c[l] * pix[l] * f4));
    }
    for (int l = 0; l + 1 < kNetLevels; ++l) {
      b.gp[l] = reinterpret_cast<float*>(take(c[l] * pix[l + 1] * f4));
      b.gu[l] = reinterpret_cast<float*>(take(cu(l) * pix[l] * f4));
      b.gd[l] = reinterpret_cast<float*>(take(c[l] * pix[l] * f4));
    }
  }
  if (out) *out = b;
  return off;
}

void conv_fwd(UNet* N, int li, const __nv_bfloat16* xa, const __nv_bfloat16* xb, __nv_bfloat16* yb, float* yf,
              const float* oscale, int B, int H, int W, cudaStream_t s) {
  const ConvLayer& L = N->layer[li];
  ConvArgs q{};
  q.xa = xa;
  q.xb = xb;
  q.ca = L.ca;
  q.cb = L.cb;
  q.co = L.co;
  q.w = N->wb + L.w_off;
  q.wp = L.p_off >= 0 ? N->wpack + L.p_off : nullptr;
  q.yb = yb;
  q.yf = yf;
  q.out_scale = oscale;
  q.relu = L.relu;
  q.B = B;
  q.H = H;
  q.W = W;
  if (N->tensor_cores && L.ks == 3 && yb && L.p_off >= 0) {
    const dim3 tgrid((W + 7) / 8, (H + 15) / 16, B);
    // as many input-channel chunks per group as the opt-in shared memory holds
    static int smem_max = 0;
    if (!smem_max) {
      int dev = 0, optin = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      smem_max = optin - 2048;  // room for the kernel's static shared memory
      cudaFuncSetAttribute(k_conv3_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max);
    }
    const int cin = L.ca + L.cb, nchunks = (cin + kTcC - 1) / kTcC;
    const int per_chunk = int(kTcSmemHalo) + 9 * (L.co / 8) * int(kTcBSBO);
    q.tc_group = std::max(1, std::min(nchunks, smem_max / per_chunk));
    launch_k(k_conv3_tc, tgrid, 128, size_t(q.tc_group) * per_chunk, s, q, N->tc_err);
    ++N->launches;
    return;
  }
  const dim3 grid((W + kTile - 1) / kTile, (H + kTile - 1) / kTile, B * ((L.co + kCT - 1) / kCT));
  if (L.ks == 3) launch_k(k_conv<3, false>, grid, 256, 0, s, q);
  else launch_k(k_conv<1, false>, grid, 256, 0, s, q);
  ++N->launches;
}

// Backward of layer li: dy (FP32, already ReLU-masked) -> input gradients
// ga/gb (skipped when both are null) and weight gradients (added to N->grad).
void conv_bwd(UNet* N, int li, const float* dy, const __nv_bfloat16* xa, const __nv_bfloat16* xb, float* ga,
              float* gb, int B, int H, int W, cudaStream_t s) {
  const ConvLayer& L = N->layer[li];
  ConvArgs q{};
  q.xa = xa;
  q.xb = xb;
  q.ca = L.ca;
  q.cb = L.cb;
  q.co = L.co;
  q.dy = dy;
  q.w = N->wb + L.w_off;
  q.ga = ga;
  q.gb = gb;
  q.B = B;
  q.H = H;
  q.W = W;
  const int cin = L.ca + L.cb;
  if (ga || gb) {
    const dim3 grid((W + kTile - 1) / kTile, (H + kTile - 1) / kTile, B * ((cin + kCT - 1) / kCT));
    if (L.ks == 3) k_conv<3, true><<<grid, 256, 0, s>>>(q);
    else k_conv<1, true><<<grid, 256, 0, s>>>(q);
    ++N->launches;
  }
  const int tx = (W + kTile - 1) / kTile, ty = (H + kTile - 1) / kTile;
  const int pairs = ((L.co + kWO - 1) / kWO) * ((cin + kWI - 1) / kWI);
  const int ntiles = tx * ty * B;
  const dim3 grid(pairs, ntiles < 64 ? ntiles : 64);
  if (L.ks == 3) k_conv_wgrad<3><<<grid, 256, 0, s>>>(q, tx, ty, N->grad + L.w_off);
  else k_conv_wgrad<1><<<grid, 256, 0, s>>>(q, tx, ty, N->grad + L.w_off);
  ++N->launches;
}

void forward_into(UNet* N, const Bufs& b, const float* in, const float* in_scale, int B, int ny, int nx, float* out,
                  const float* out_scale, cudaStream_t s) {
  const int* c = N->ch;
  int H[kNetLevels], W[kNetLevels];
  for (int l = 0; l < kNetLevels; ++l) {
    H[l] = ny >> l;
    W[l] = nx >> l;
  }
  const long long hw0 = (long long)ny * nx;
  launch_k(k_to_bf16, grid1(hw0 * B), 256, 0, s, in, in_scale, hw0, B, b.x0);
  ++N->launches;
  // encoder and bottom: layers 2l (from x0 or the pooled level above) and 2l+1
  for (int l = 0; l < kNetLevels; ++l) {
    const __nv_bfloat16* src = l == 0 ? b.x0 : b.p[l - 1];
    conv_fwd(N, 2 * l, src, nullptr, b.a[l], nullptr, nullptr, B, H[l], W[l], s);
    conv_fwd(N, 2 * l + 1, b.a[l], nullptr, b.e[l], nullptr, nullptr, B, H[l], W[l], s);
    if (l + 1 < kNetLevels) {
      const long long planes = (long long)B * c[l];
      launch_k(k_pool, grid1(planes * H[l + 1] * W[l + 1]), 256, 0, s, b.e[l], b.p[l], planes, H[l], W[l]);
      ++N->launches;
    }
  }
  // decoder: layers 8 (level 2), 9 (level 1), 10 (level 0)
  for (int l = kNetLevels - 2; l >= 0; --l) {
    const __nv_bfloat16* below = l == kNetLevels - 2 ? b.e[kNetLevels - 1] : b.d[l + 1];
    const int cbelow = l == kNetLevels - 2 ? c[kNetLevels - 1] : c[l + 1];
    const long long planes = (long long)B * cbelow;
    launch_k(k_up, grid1(planes * H[l] * W[l]), 256, 0, s, below, b.u[l], planes, H[l], W[l]);
    ++N->launches;
    conv_fwd(N, 2 * kNetLevels + (kNetLevels - 2 - l), b.u[l], b.e[l], b.d[l], nullptr, nullptr, B, H[l], W[l], s);
  }
  conv_fwd(N, kNetLayers - 1, b.d[0], nullptr, nullptr, out, out_scale, B, ny, nx, s);
}

}  // namespace

int unet_init(UNet* N, const int* channels) {
  if (channels)
    for (int l = 0; l < kNetLevels; ++l) {
      if (channels[l] < 1 || channels[l] > 256) {
        N->err = "U-Net channels must be in 1..256";
        return MACSAV_ERR_VALUE;
      }
      N->ch[l] = channels[l];
    }
  const int* c = N->ch;
  long long off = 0;
  long long poff = 0;
  auto add = [&](int idx, int ca, int cb, int co, int ks, int relu) {
    const bool tc = ks == 3 && (co == 16 || co == 32 || co == 64);
    N->layer[idx] = ConvLayer{ca, cb, co, ks, relu, off, tc ? poff : -1};
    off += (long long)co * (ca + cb) * ks * ks;
    if (tc) poff += (long long)((ca + cb + 15) / 16) * 9 * co * 16;
  };
  add(0, 1, 0, c[0], 3, 1);
  add(1, c[0], 0, c[0], 3, 1);
  for (int l = 1; l < kNetLevels; ++l) {
    add(2 * l, c[l - 1], 0, c[l], 3, 1);
    add(2 * l + 1, c[l], 0, c[l], 3, 1);
  }
  // decoder: level 2 reads the bottom (c3), levels 1 and 0 the decoder below
  add(8, c[3], c[2], c[2], 3, 1);
  add(9, c[2], c[1], c[1], 3, 1);
  add(10, c[1], c[0], c[0], 3, 1);
  add(11, c[0], 0, 1, 1, 0);
  N->nparams = off;
  N->npack = poff;
  const size_t n = size_t(off);
  if (cudaMalloc(&N->wpack, size_t(poff) * sizeof(__nv_bfloat16)) != cudaSuccess) return MACSAV_ERR_CUDA;
  cudaMemset(N->wpack, 0, size_t(poff) * sizeof(__nv_bfloat16));
  if (cudaMalloc(&N->w32, n * sizeof(float)) != cudaSuccess || cudaMalloc(&N->grad, n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&N->m1, n * sizeof(float)) != cudaSuccess || cudaMalloc(&N->m2, n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&N->wb, n * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc(&N->loss, sizeof(double)) != cudaSuccess || cudaMalloc(&N->tc_err, sizeof(int)) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  cudaMemset(N->tc_err, 0, sizeof(int));
  cudaMemset(N->w32, 0, n * sizeof(float));
  cudaMemset(N->grad, 0, n * sizeof(float));
  cudaMemset(N->m1, 0, n * sizeof(float));
  cudaMemset(N->m2, 0, n * sizeof(float));
  cudaMemset(N->wb, 0, n * sizeof(__nv_bfloat16));
  cudaMemset(N->loss, 0, sizeof(double));
  return cudaDeviceSynchronize() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

void unet_free(UNet* N) {
  cudaFree(N->w32);
  cudaFree(N->grad);
  cudaFree(N->m1);
  cudaFree(N->m2);
  cudaFree(N->wb);
  cudaFree(N->wpack);
  N->wpack = nullptr;
  cudaFree(N->loss);
  cudaFree(N->tc_err);
  N->tc_err = nullptr;
  N->w32 = N->grad = N->m1 = N->m2 = nullptr;
  N->wb = nullptr;
  N->loss = nullptr;
}

int net_work_ensure(const UNet* N, NetWork* W, int batch, int ny, int nx, bool grad) {
  if (batch < 1 || ny < 8 || nx < 8 || ny % 8 || nx % 8) return MACSAV_ERR_UNSUPPORTED;
  if (W->base && W->batch == batch && W->ny == ny && W->nx == nx && (W->grad || !grad)) return MACSAV_OK;
  net_work_free(W);
  const size_t bytes = layout(N, batch, ny, nx, grad, nullptr, nullptr);
  if (cudaMalloc(&W->base, bytes) != cudaSuccess) {
    W->base = nullptr;
    return MACSAV_ERR_CUDA;
  }
  W->bytes = bytes;
  W->batch = batch;
  W->ny = ny;
  W->nx = nx;
  W->grad = grad;
  return MACSAV_OK;
}

void net_work_free(NetWork* W) {
  if (W->base) cudaFree(W->base);
  W->base = nullptr;
  W->bytes = 0;
  W->batch = W->ny = W->nx = 0;
}

int unet_forward(UNet* N, NetWork* W, const float* in, const float* in_scale, int batch, int ny, int nx, float* out,
                 const float* out_scale, cudaStream_t s) {
  if (!W->base || batch < 1 || batch > W->batch || W->ny != ny || W->nx != nx) return MACSAV_ERR_VALUE;
  Bufs b;
  layout(N, W->batch, ny, nx, W->grad, W->base, &b);  // buffers sized for W->batch >= batch
  forward_into(N, b, in, in_scale, batch, ny, nx, out, out_scale, s);
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

int unet_backward(UNet* N, NetWork* W, const float* in, const float* target, int batch, int ny, int nx,
                  cudaStream_t s) {
  if (!W->base || !W->grad || batch < 1 || batch > W->batch || W->ny != ny || W->nx != nx) return MACSAV_ERR_VALUE;
  Bufs b;
  layout(N, W->batch, ny, nx, true, W->base, &b);
  forward_into(N, b, in, nullptr, batch, ny, nx, b.y, nullptr, s);
  const int* c = N->ch;
  int H[kNetLevels], Wd[kNetLevels];
  for (int l = 0; l < kNetLevels; ++l) {
    H[l] = ny >> l;
    Wd[l] = nx >> l;
  }
  const long long pix0 = (long long)batch * ny * nx;
  k_mse<<<grid1(pix0), 256, 0, s>>>(b.y, target, b.gy, pix0, N->loss);
  ++N->launches;
  auto mask = [&](float* g, const __nv_bfloat16* y, long long n) {
    k_relu_mask<<<grid1(n), 256, 0, s>>>(g, y, n);
    ++N->launches;
  };
  auto npx = [&](int l) { return (long long)batch * H[l] * Wd[l]; };
  // output layer (no ReLU)
  conv_bwd(N, kNetLayers - 1, b.gy, b.d[0], nullptr, b.gd[0], nullptr, batch, ny, nx, s);
  // decoder, level 0 up to level 2
  for (int l = 0; l <= kNetLevels - 2; ++l) {
    mask(b.gd[l], b.d[l], c[l] * npx(l));
    const int li = 2 * kNetLevels + (kNetLevels - 2 - l);
    conv_bwd(N, li, b.gd[l], b.u[l], b.e[l], b.gu[l], b.ge[l], batch, H[l], Wd[l], s);
    const bool bottom = l == kNetLevels - 2;
    const int cbelow = bottom ? c[kNetLevels - 1] : c[l + 1];
    float* gbelow = bottom ? b.ge[kNetLevels - 1] : b.gd[l + 1];
    const long long planes = (long long)batch * cbelow;
    k_up_bwd<<<grid1(planes * H[l + 1] * Wd[l + 1]), 256, 0, s>>>(b.gu[l], gbelow, planes, H[l], Wd[l]);
    ++N->launches;
  }
  // bottom and encoder, level 3 up to level 0
  for (int l = kNetLevels - 1; l >= 0; --l) {
    mask(b.ge[l], b.e[l], c[l] * npx(l));
    conv_bwd(N, 2 * l + 1, b.ge[l], b.a[l], nullptr, b.ga[l], nullptr, batch, H[l], Wd[l], s);
    mask(b.ga[l], b.a[l], c[l] * npx(l));
    const __nv_bfloat16* src = l == 0 ? b.x0 : b.p[l - 1];
    conv_bwd(N, 2 * l, b.ga[l], src, nullptr, l == 0 ? nullptr : b.gp[l - 1], nullptr, batch, H[l], Wd[l], s);
    if (l > 0) {
      const long long planes = (long long)batch * c[l - 1];
      k_pool_bwd<<<grid1(planes * H[l - 1] * Wd[l - 1]), 256, 0, s>>>(b.gp[l - 1], b.ge[l - 1], planes, H[l - 1],
                                                                        Wd[l - 1]);
      ++N->launches;
    }
  }
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

// Refresh the tensor-core operand copies from the BF16 weights.
static void pack_weights(UNet* N, cudaStream_t s) {
  for (int li = 0; li < kNetLayers; ++li) {
    const ConvLayer& L = N->layer[li];
    if (L.p_off < 0) continue;
    const int cin = L.ca + L.cb;
    const long long total = (long long)((cin + 15) / 16) * 9 * L.co * 16;
    k_pack_w3<<<grid1(total), 256, 0, s>>>(N->wb + L.w_off, N->wpack + L.p_off, L.co, cin, total);
    ++N->launches;
  }
}

int unet_adam(UNet* N, float lr, cudaStream_t s) {
  const double b1 = 0.9, b2 = 0.999;
  N->adam_t += 1;
  const double c1 = 1.0 - std::pow(b1, double(N->adam_t)), c2 = 1.0 - std::pow(b2, double(N->adam_t));
  k_adam<<<grid1(N->nparams), 256, 0, s>>>(N->w32, N->grad, N->m1, N->m2, N->wb, N->nparams, lr, float(b1), float(b2),
                                           float(c1), float(c2), 1e-8f);
  ++N->launches;
  pack_weights(N, s);
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

int unet_sync_bf16(UNet* N, cudaStream_t s) {
  k_sync_bf16<<<grid1(N->nparams), 256, 0, s>>>(N->w32, N->wb, N->nparams);
  ++N->launches;
  pack_weights(N, s);
  return cudaGetLastError() == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}

}  // namespace macsav
