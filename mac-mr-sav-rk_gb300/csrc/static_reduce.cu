// Plan-free inner product / max-abs reduction whose scratch is a fixed-size
// file-scope device array, so a call takes no device memory of its own.
//
// Who needs it: callers that may not allocate device memory and hold no plan
// (a plan's buffers come from cudaMalloc at create time).  Two cases: an error
// handler that runs after the device has reported out-of-memory, where creating
// a plan would fail in turn, and a monitor that checks the size and finiteness
// of a packed state between steps while the solver's plans own the rest of the
// memory it was given.  The arithmetic is that of macsav_inner / macsav_max_abs
// (hx*hy*dot and max|a| with NaN propagation); only the summation order differs,
// so the dot product agrees with them to rounding and the maximum exactly.
//
// Scratch: kSRDoubles doubles (64 KiB + 32 B) in one static __device__ array:
//   [0, 2*kSRBlocks)             per-block partials (sum, max), written before
//                                they are read in every call;
//   [2*kSRBlocks, 2*kSRBlocks+2) the folded result, copied to the host;
//   [2*kSRBlocks+2]              the completion counter (an unsigned int in the
//                                low word of that slot).  It must be zero when a
//                                call starts: set-up clears it, and the block
//                                that finishes a call sets it back to zero.
// A block reduces one chunk of kSRChunk elements, so n is limited to
// kSRBlocks*kSRChunk = 16,777,216 elements (MACSAV_STATIC_REDUCE_MAX_N); the
// largest packed velocity of the 2048x1024 cavity is 4,191,232.
//
// Set-up: the first call on each device (the device current on the calling
// thread) looks up the array's device address with cudaGetSymbolAddress and
// clears the counter with cudaMemsetAsync on the caller's stream.  The lookup
// may load the module, so make that first call outside any stream capture.
// The address belongs to the device's context: a call that finds a different
// context current (after cudaDeviceReset, or after the primary context was
// released and made again) repeats the set-up for the new context, so it never
// hands the kernel an address of a context that is gone.  Such a call is again
// a first call, to be made outside any stream capture.
//
// Calls share the one array per device: two calls whose kernels overlap (on
// different streams, or from different threads without ordering) race on the
// partials, the counter and the result.  Order them, e.g. on one stream.
#include <cuda.h>

#include <mutex>

#include "common.cuh"
#include "../../include/macsav.h"

namespace macsav {
namespace {

constexpr int kSRThreads = 256;
constexpr int kSRPerThread = 16;
constexpr int kSRChunk = kSRThreads * kSRPerThread;  // 4096 elements per block
constexpr int kSRBlocks = 4096;
constexpr int kSRResult = 2 * kSRBlocks;
constexpr int kSRCounter = kSRResult + 2;
constexpr int kSRDoubles = kSRResult + 4;
constexpr int kSRMaxDevices = 64;
static_assert((long long)kSRBlocks * kSRChunk == MACSAV_STATIC_REDUCE_MAX_N, "limit and scratch size disagree");

static __device__ __align__(256) double g_reduce_scratch[kSRDoubles];

// scratch = the address of g_reduce_scratch on the launching device.
__global__ void __launch_bounds__(kSRThreads) k_inner_max_static(const double* a, const double* b, long long n,
                                                                 double weight, double* scratch) {
  __shared__ double red[64];
  double s[1] = {0.0}, m[1] = {0.0};
  const long long base = (long long)blockIdx.x * kSRChunk + threadIdx.x;
#pragma unroll 4
  for (int k = 0; k < kSRPerThread; ++k) {
    const long long i = base + (long long)k * kSRThreads;
    if (i < n) {
      const double av = a[i];
      s[0] += b ? av * b[i] : av;
      m[0] = nanmax(m[0], fabs(av));
    }
  }
  block_sum<1>(s, red);
  block_max<1>(m, red);
  if (threadIdx.x == 0) {
    scratch[2 * blockIdx.x] = s[0];
    scratch[2 * blockIdx.x + 1] = m[0];
  }
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kSRCounter);
  last_block_finish(
      [&] {
        double fs[1] = {0.0}, fm[1] = {0.0};
        for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
          fs[0] += __ldcg(scratch + 2 * q);
          fm[0] = nanmax(fm[0], __ldcg(scratch + 2 * q + 1));
        }
        block_sum<1>(fs, red);
        block_max<1>(fm, red);
        if (threadIdx.x == 0) {
          scratch[kSRResult] = weight * fs[0];
          scratch[kSRResult + 1] = fm[0];
        }
      },
      counter);
}

std::mutex g_setup_lock;
double* g_scratch_ptr[kSRMaxDevices] = {};
unsigned long long g_scratch_ctx[kSRMaxDevices] = {};  // context id the address belongs to

// The driver's id of the context current on this thread (0 when none is
// current yet).  The two driver entry points are looked up through the
// runtime once, so the library does not link the driver library itself.
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<GetCurrent>(f1);
      get_id = reinterpret_cast<GetId>(f2);
    }
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch on the current device; set-up on the first
// use in each context of that device.
int scratch_for_current_device(double** out, cudaStream_t s) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return MACSAV_ERR_CUDA;
  if (dev < 0 || dev >= kSRMaxDevices) return MACSAV_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> hold(g_setup_lock);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    double* ptr = nullptr;
    if (cudaGetSymbolAddress((void**)&ptr, g_reduce_scratch) != cudaSuccess || !ptr) return MACSAV_ERR_CUDA;
    if (cudaMemsetAsync(ptr + kSRCounter, 0, sizeof(double), s) != cudaSuccess) return MACSAV_ERR_CUDA;
    g_scratch_ptr[dev] = ptr;
    g_scratch_ctx[dev] = current_context_id();  // the lookup made the context current if none was
  }
  *out = g_scratch_ptr[dev];
  return MACSAV_OK;
}

}  // namespace
}  // namespace macsav

extern "C" int macsav_inner_max_static(const double* a, const double* b, long long n, double weight,
                                       double* result, void* stream) {
  using namespace macsav;
  if (!a || !result || n < 0) return MACSAV_ERR_VALUE;
  if (n > MACSAV_STATIC_REDUCE_MAX_N) return MACSAV_ERR_UNSUPPORTED;  // checked before any device work
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch, s);
  if (rc != MACSAV_OK) return rc;
  const int blocks = n == 0 ? 1 : int((n + kSRChunk - 1) / kSRChunk);
  k_inner_max_static<<<blocks, kSRThreads, 0, s>>>(a, b, n, weight, scratch);
  if (cudaGetLastError() != cudaSuccess) return MACSAV_ERR_CUDA;
  if (cudaMemcpyAsync(result, scratch + kSRResult, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return MACSAV_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? MACSAV_OK : MACSAV_ERR_CUDA;
}
