// The selector network's inference for one sample inside a CTA (used by the
// batched solver's fused select-and-solve mode).  Layout and summation order
// are those of mlp.cu's mlp_forward_kernel (z_j = b_j + sum_i x_i W[i][j],
// i ascending, fmaf), so the argmax equals ElGBMLPForward's on the same
// features.  Parameters, one flat FP32 vector:
//   W1[16][64] b1[64] W2[64][64] b2[64] W3[64][3] b3[3]   (row-major, in x out)
#pragma once

namespace elgb {
namespace mlpd {

constexpr int kIn = 16, kH = 64, kOut = 3;
constexpr int oW1 = 0, ob1 = oW1 + kIn * kH, oW2 = ob1 + kH, ob2 = oW2 + kH * kH,
              oW3 = ob2 + kH, ob3 = oW3 + kH * kOut, kParams = ob3 + kOut;

// x: kIn features in shared memory; h1, h2: kH floats of shared scratch,
// lg: kOut.  Needs >= kH threads; every thread of the block must call it.
// Returns the argmax class (first maximum) in every thread.
__device__ __forceinline__ int block_argmax(const float* __restrict__ params, const float* x,
                                            float* h1, float* h2, float* lg) {
  const int t = threadIdx.x;
  if (t < kH) {
    float z = params[ob1 + t];
#pragma unroll
    for (int i = 0; i < kIn; ++i) z = fmaf(x[i], params[oW1 + i * kH + t], z);
    h1[t] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  if (t < kH) {
    float z = params[ob2 + t];
    for (int i = 0; i < kH; ++i) z = fmaf(h1[i], params[oW2 + i * kH + t], z);
    h2[t] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  if (t < kOut) {
    float z = params[ob3 + t];
    for (int i = 0; i < kH; ++i) z = fmaf(h2[i], params[oW3 + i * kOut + t], z);
    lg[t] = z;
  }
  __syncthreads();
  int best = 0;
  for (int k = 1; k < kOut; ++k)
    if (lg[k] > lg[best]) best = k;
  __syncthreads();
  return best;
}

}  // namespace mlpd
}  // namespace elgb
