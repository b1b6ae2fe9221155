// Added form 3, the learned part: a 16 -> 64 -> 64 -> 3 FP32 MLP (ReLU,
// softmax cross-entropy) that maps per-matrix features to the lowest
// factorization precision (FP64 / FP32 / BF16) whose refinement converges.
// Hand-written training and inference kernels:
//   mlp_forward_kernel   one thread per sample, weights in shared memory;
//                        stores the activations a training step needs
//   mlp_param_grad_kernel one thread per parameter, summing over the batch
//                        in sample order (deterministic, no atomics)
//   mlp_adam_kernel      Adam update
// Parameters live in one flat FP32 vector:
//   W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]   (row-major, in x out)
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/elgb300.h"
#include "driver.h"

namespace elgb {

namespace {

constexpr int kIn = 16, kH = 64, kOut = 3;
constexpr int oW1 = 0, ob1 = oW1 + kIn * kH, oW2 = ob1 + kH, ob2 = oW2 + kH * kH,
              oW3 = ob2 + kH, ob3 = oW3 + kH * kOut, kParams = ob3 + kOut;

// Per-sample forward pass.  With `act` non-null the step's activations are
// stored: act[s] = {z1[64], z2[64], h2[64]... } laid out as
//   Z1 (B x 64), H1 (B x 64), Z2 (B x 64), H2 (B x 64), P (B x 3)
__global__ void mlp_forward_kernel(const float* __restrict__ params, const float* __restrict__ X,
                                   int B, float* __restrict__ probs, int* __restrict__ argmax,
                                   float* __restrict__ act, const int* __restrict__ labels,
                                   float* __restrict__ loss_per_sample) {
  __shared__ float sp[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) sp[i] = params[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  float x[kIn], h1[kH], h2[kH];
#pragma unroll
  for (int i = 0; i < kIn; ++i) x[i] = X[(long)s * kIn + i];
  for (int j = 0; j < kH; ++j) {
    float z = sp[ob1 + j];
#pragma unroll
    for (int i = 0; i < kIn; ++i) z = fmaf(x[i], sp[oW1 + i * kH + j], z);
    h1[j] = z > 0.f ? z : 0.f;
    if (act) {
      act[(long)s * kH + j] = z;                       // Z1
      act[(long)B * kH + (long)s * kH + j] = h1[j];    // H1
    }
  }
  for (int j = 0; j < kH; ++j) {
    float z = sp[ob2 + j];
    for (int i = 0; i < kH; ++i) z = fmaf(h1[i], sp[oW2 + i * kH + j], z);
    h2[j] = z > 0.f ? z : 0.f;
    if (act) {
      act[2L * B * kH + (long)s * kH + j] = z;         // Z2
      act[3L * B * kH + (long)s * kH + j] = h2[j];     // H2
    }
  }
  float lg[kOut];
  float mx = -INFINITY;
#pragma unroll
  for (int k = 0; k < kOut; ++k) {
    float z = sp[ob3 + k];
    for (int i = 0; i < kH; ++i) z = fmaf(h2[i], sp[oW3 + i * kOut + k], z);
    lg[k] = z;
    mx = fmaxf(mx, z);
  }
  float den = 0.f;
#pragma unroll
  for (int k = 0; k < kOut; ++k) den += expf(lg[k] - mx);
  int best = 0;
#pragma unroll
  for (int k = 0; k < kOut; ++k) {
    const float p = expf(lg[k] - mx) / den;
    if (probs) probs[(long)s * kOut + k] = p;
    if (act) act[4L * B * kH + (long)s * kOut + k] = p;
    if (lg[k] > lg[best]) best = k;
  }
  if (argmax) argmax[s] = best;
  if (labels && loss_per_sample) {
    const int y = labels[s];
    loss_per_sample[s] = -(lg[y] - mx - logf(den));
  }
}

// Backward through the layers for each sample: dZ3 = (P - onehot) / B,
// dZ2 = (dZ3 W3^T) * [Z2 > 0], dZ1 = (dZ2 W2^T) * [Z1 > 0]; stored after the
// activations as dZ3 (B x 3), dZ2 (B x 64), dZ1 (B x 64).
__global__ void mlp_backward_act_kernel(const float* __restrict__ params,
                                        const int* __restrict__ labels, int B,
                                        float* __restrict__ act) {
  __shared__ float sp[kParams];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) sp[i] = params[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const float* Z1 = act;
  const float* Z2 = act + 2L * B * kH;
  const float* P = act + 4L * B * kH;
  float* dZ3 = act + 4L * B * kH + (long)B * kOut;
  float* dZ2 = dZ3 + (long)B * kOut;
  float* dZ1 = dZ2 + (long)B * kH;
  float d3[kOut];
  const int y = labels[s];
#pragma unroll
  for (int k = 0; k < kOut; ++k) {
    d3[k] = (P[(long)s * kOut + k] - (k == y ? 1.f : 0.f)) / (float)B;
    dZ3[(long)s * kOut + k] = d3[k];
  }
  float d2[kH];
  for (int i = 0; i < kH; ++i) {
    float g = 0.f;
#pragma unroll
    for (int k = 0; k < kOut; ++k) g = fmaf(d3[k], sp[oW3 + i * kOut + k], g);
    d2[i] = Z2[(long)s * kH + i] > 0.f ? g : 0.f;
    dZ2[(long)s * kH + i] = d2[i];
  }
  for (int i = 0; i < kH; ++i) {
    float g = 0.f;
    for (int j = 0; j < kH; ++j) g = fmaf(d2[j], sp[oW2 + i * kH + j], g);
    dZ1[(long)s * kH + i] = Z1[(long)s * kH + i] > 0.f ? g : 0.f;
  }
}

// One thread per parameter: its gradient summed over the batch in sample
// order.
__global__ void mlp_param_grad_kernel(const float* __restrict__ X, int B,
                                      const float* __restrict__ act, float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float* H1 = act + 1L * B * kH;
  const float* H2 = act + 3L * B * kH;
  const float* dZ3 = act + 4L * B * kH + (long)B * kOut;
  const float* dZ2 = dZ3 + (long)B * kOut;
  const float* dZ1 = dZ2 + (long)B * kH;
  float g = 0.f;
  if (p < ob1) {
    const int i = p / kH, j = p % kH;
    for (int s = 0; s < B; ++s) g = fmaf(X[(long)s * kIn + i], dZ1[(long)s * kH + j], g);
  } else if (p < oW2) {
    const int j = p - ob1;
    for (int s = 0; s < B; ++s) g += dZ1[(long)s * kH + j];
  } else if (p < ob2) {
    const int i = (p - oW2) / kH, j = (p - oW2) % kH;
    for (int s = 0; s < B; ++s) g = fmaf(H1[(long)s * kH + i], dZ2[(long)s * kH + j], g);
  } else if (p < oW3) {
    const int j = p - ob2;
    for (int s = 0; s < B; ++s) g += dZ2[(long)s * kH + j];
  } else if (p < ob3) {
    const int i = (p - oW3) / kOut, k = (p - oW3) % kOut;
    for (int s = 0; s < B; ++s) g = fmaf(H2[(long)s * kH + i], dZ3[(long)s * kOut + k], g);
  } else {
    const int k = p - ob3;
    for (int s = 0; s < B; ++s) g += dZ3[(long)s * kOut + k];
  }
  grad[p] = g;
}

__global__ void mlp_adam_kernel(float* __restrict__ params, const float* __restrict__ grad,
                                float* __restrict__ m, float* __restrict__ v, float lr,
                                float b1, float b2, float eps, float wd, int step) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float g = grad[p] + wd * params[p];
  const float mm = b1 * m[p] + (1.f - b1) * g;
  const float vv = b2 * v[p] + (1.f - b2) * g * g;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(b1, (float)step));
  const float vh = vv / (1.f - powf(b2, (float)step));
  params[p] -= lr * mh / (sqrtf(vh) + eps);
}

size_t act_floats(int B) { return 4L * B * kH + 2L * B * kOut + 2L * B * kH; }

}  // namespace

}  // namespace elgb

// ===========================================================================
// C ABI (include/elgb300.h)
// ===========================================================================
extern "C" {

int ElGBMLPParamCount(void) { return elgb::kParams; }

int ElGBMLPForward(ElGBContext ctx, const float* params, const float* X, int B, float* probs,
                   int* argmax) {
  if (!ctx || !params || !X || B < 0) return elgb::kElArgError;
  if (B == 0) return 0;
  cudaSetDevice(ctx->device);
  elgb::mlp_forward_kernel<<<(B + 127) / 128, 128, 0, ctx->stream>>>(
      params, X, B, probs, argmax, nullptr, nullptr, nullptr);
  ctx->launches += 1;
  return elgb::to_el_error(cudaGetLastError());
}

int ElGBMLPGradient(ElGBContext ctx, const float* params, const float* X, const int* labels,
                    int B, float* grad, float* loss) {
  if (!ctx || !params || !X || !labels || !grad || B <= 0) return elgb::kElArgError;
  cudaSetDevice(ctx->device);
  const size_t need = (elgb::act_floats(B) + (size_t)B) * sizeof(float);
  cudaError_t e = ctx->ensure(need);
  if (e != cudaSuccess) return elgb::kElRuntimeError;
  float* act = static_cast<float*>(ctx->arena);
  float* lps = act + elgb::act_floats(B);
  elgb::mlp_forward_kernel<<<(B + 127) / 128, 128, 0, ctx->stream>>>(params, X, B, nullptr,
                                                                     nullptr, act, labels, lps);
  elgb::mlp_backward_act_kernel<<<(B + 127) / 128, 128, 0, ctx->stream>>>(params, labels, B,
                                                                          act);
  elgb::mlp_param_grad_kernel<<<(elgb::kParams + 127) / 128, 128, 0, ctx->stream>>>(X, B, act,
                                                                                    grad);
  ctx->launches += 3;
  e = cudaGetLastError();
  if (e == cudaSuccess && loss) {
    std::vector<float> h(B);
    e = cudaMemcpyAsync(h.data(), lps, sizeof(float) * B, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    double sum = 0;
    for (float x : h) sum += x;
    *loss = (float)(sum / B);
  }
  return elgb::to_el_error(e);
}

int ElGBMLPAdamStep(ElGBContext ctx, float* params, const float* grad, float* m, float* v,
                    float lr, float beta1, float beta2, float eps, float weight_decay,
                    int step) {
  if (!ctx || !params || !grad || !m || !v || step < 1) return elgb::kElArgError;
  cudaSetDevice(ctx->device);
  elgb::mlp_adam_kernel<<<(elgb::kParams + 127) / 128, 128, 0, ctx->stream>>>(
      params, grad, m, v, lr, beta1, beta2, eps, weight_decay, step);
  ctx->launches += 1;
  return elgb::to_el_error(cudaGetLastError());
}

}  // extern "C"
