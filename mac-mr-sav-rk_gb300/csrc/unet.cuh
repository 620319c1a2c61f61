// Small convolutional network used as a learned correction to the spectral
// pressure preconditioner (flexible CG in the FP32 inner Stokes solves).
//
// Architecture (4 levels, channels c0..c3, bias-free, ReLU, zero padding):
//   encoder   level l: conv3x3 -> conv3x3 (c_l), 2x2 average pool to level l+1
//   bottom    level 3: conv3x3 -> conv3x3 (c3)
//   decoder   level l: nearest 2x upsample of the level below, concatenated
//             with the encoder output of level l, conv3x3 (c_l)
//   output    conv1x1 (c0 -> 1), no ReLU, FP32
// Without biases every layer is positively homogeneous, so the network is
// too: net(a r) = a net(r) for a > 0.  Activations are stored in BF16,
// products are accumulated in FP32, activation gradients are FP32, and the
// weights have an FP32 master copy (Adam) and a BF16 copy read by the kernels.
// Inputs and outputs are [batch][ny][nx] FP32 with per-sample scales.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

namespace macsav {

constexpr int kNetLevels = 4;
constexpr int kNetLayers = 12;

struct ConvLayer {
  int ca, cb, co, ks, relu;
  long long w_off;  // offset of the layer's [co][ca+cb][ks*ks] weights in the parameter vector
  long long p_off;  // offset of its tensor-core operand copy in UNet::wpack (-1: none)
};

struct UNet {
  int ch[kNetLevels] = {16, 32, 64, 64};
  ConvLayer layer[kNetLayers];
  long long nparams = 0;
  float* w32 = nullptr;                 // master weights
  __nv_bfloat16* wb = nullptr;          // BF16 copy read by the kernels
  // BF16 weights of the 3x3 layers in the shared-memory operand layout of
  // the tensor-core convolution, per 16-channel chunk [chunk][tap][co/8][2][8][8],
  // refreshed whenever the weights change, so a CTA stages them with
  // contiguous 16-byte copies
  __nv_bfloat16* wpack = nullptr;
  long long npack = 0;
  float* grad = nullptr;                // weight gradients
  float *m1 = nullptr, *m2 = nullptr;   // Adam moments
  long long adam_t = 0;
  double* loss = nullptr;               // device loss accumulator
  bool tensor_cores = true;             // forward 3x3 convolutions on tcgen05 (k_conv3_tc)
  int* tc_err = nullptr;                // set when a tensor-core wait ran out
  std::string err;
  long long launches = 0;
};

// Activation workspace for one (batch, ny, nx); a plan keeps its own, so a
// captured graph never sees it move.
struct NetWork {
  int batch = 0, ny = 0, nx = 0;
  bool grad = false;
  char* base = nullptr;
  size_t bytes = 0;
};

int unet_init(UNet* N, const int* channels);
void unet_free(UNet* N);
int net_work_ensure(const UNet* N, NetWork* W, int batch, int ny, int nx, bool grad);
void net_work_free(NetWork* W);

// out[b] = out_scale[b] * net(in_scale[b] * in[b]) for b < batch (null scale:
// 1).  ny and nx must be multiples of 8; W must be sized for (batch, ny, nx).
int unet_forward(UNet* N, NetWork* W, const float* in, const float* in_scale, int batch, int ny, int nx, float* out,
                 const float* out_scale, cudaStream_t s);
// Forward and backward of the mean squared error against `target`: adds the
// weight gradients to N->grad and the loss to N->loss (both device).
int unet_backward(UNet* N, NetWork* W, const float* in, const float* target, int batch, int ny, int nx,
                  cudaStream_t s);
// One Adam step with N->grad, then clears N->grad and refreshes the BF16 copy.
int unet_adam(UNet* N, float lr, cudaStream_t s);
int unet_sync_bf16(UNet* N, cudaStream_t s);

}  // namespace macsav
