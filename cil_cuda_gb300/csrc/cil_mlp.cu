// Skin-scheduler network: a 12 -> 64 -> 64 -> 2 multilayer perceptron with SiLU activations
// in FP32, trained and evaluated by these kernels (no library GEMMs: the layers are tiny).
//
// Parameter layout (one flat FP32 vector, kMlpParams entries):
//   W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
// Training minimises the mean squared error between the outputs and the targets with Adam.
// Gradients are formed per block in shared memory and summed over blocks in a fixed order,
// so a training step is deterministic.
//
// Inference runs inside the skin-mode rebuild decision (k_skin_begin, one warp per colony,
// mlp_forward_warp): output 0 becomes the skin skin_min + (skin_max - skin_min) * sigmoid(y0)
// and output 1 the cadence round(interval_scale * softplus(y1)).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "cil_gpu.h"
#include "cil_internal.cuh"

namespace cil {
namespace {

constexpr int kIn = kMlpIn, kH = kMlpH, kOut = kMlpOut;
constexpr int kOffW1 = kMlpW1, kOffB1 = kMlpB1, kOffW2 = kMlpW2, kOffB2 = kMlpB2, kOffW3 = kMlpW3, kOffB3 = kMlpB3,
              kParams = kMlpParams;
constexpr int kSamplesPerBlock = 32;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// block of kH threads: forward pass of one sample held in shared memory
__device__ void forward_one(const float *w, const float *x, float *z1, float *h1, float *z2, float *h2,
                            float *y) {
  const int u = threadIdx.x;
  float acc = w[kOffB1 + u];
  for (int k = 0; k < kIn; ++k) acc += w[kOffW1 + u * kIn + k] * x[k];
  z1[u] = acc;
  h1[u] = silu(acc);
  __syncthreads();
  acc = w[kOffB2 + u];
  for (int k = 0; k < kH; ++k) acc += w[kOffW2 + u * kH + k] * h1[k];
  z2[u] = acc;
  h2[u] = silu(acc);
  __syncthreads();
  if (u < kOut) {
    float o = w[kOffB3 + u];
    for (int k = 0; k < kH; ++k) o += w[kOffW3 + u * kH + k] * h2[k];
    y[u] = o;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kH) k_mlp_forward(const float *params, const float *X, int n, float *Y) {
  __shared__ float w[kParams];
  __shared__ float x[kIn], z1[kH], h1[kH], z2[kH], h2[kH], y[kOut];
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = params[i];
  __syncthreads();
  const int s0 = blockIdx.x * kSamplesPerBlock;
  for (int s = s0; s < min(s0 + kSamplesPerBlock, n); ++s) {
    if (threadIdx.x < kIn) x[threadIdx.x] = X[static_cast<size_t>(s) * kIn + threadIdx.x];
    __syncthreads();
    forward_one(w, x, z1, h1, z2, h2, y);
    if (threadIdx.x < kOut) Y[static_cast<size_t>(s) * kOut + threadIdx.x] = y[threadIdx.x];
    __syncthreads();
  }
}

// loss = mean over samples and outputs of ow[o] * (y - t)^2; per-block gradient partials
__global__ void __launch_bounds__(kH) k_mlp_backward(const float *params, const float *X, const float *T,
                                                     const float *ow, int n, float *partial, float *loss_partial) {
  __shared__ float w[kParams];
  __shared__ float g[kParams];
  __shared__ float x[kIn], z1[kH], h1[kH], z2[kH], h2[kH], y[kOut], dy[kOut], dz2[kH], dz1[kH];
  __shared__ float lsum;
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    w[i] = params[i];
    g[i] = 0.0f;
  }
  if (threadIdx.x == 0) lsum = 0.0f;
  __syncthreads();
  const int u = threadIdx.x;
  const float inv = 1.0f / static_cast<float>(n * kOut);
  const int s0 = blockIdx.x * kSamplesPerBlock;
  for (int s = s0; s < min(s0 + kSamplesPerBlock, n); ++s) {
    if (u < kIn) x[u] = X[static_cast<size_t>(s) * kIn + u];
    __syncthreads();
    forward_one(w, x, z1, h1, z2, h2, y);
    if (u < kOut) {
      const float diff = y[u] - T[static_cast<size_t>(s) * kOut + u];
      dy[u] = 2.0f * ow[u] * diff * inv;
      atomicAdd(&lsum, ow[u] * diff * diff * inv);
    }
    __syncthreads();
    // layer 3
    for (int o = 0; o < kOut; ++o) g[kOffW3 + o * kH + u] += dy[o] * h2[u];
    if (u < kOut) g[kOffB3 + u] += dy[u];
    float dh = 0.0f;
    for (int o = 0; o < kOut; ++o) dh += w[kOffW3 + o * kH + u] * dy[o];
    dz2[u] = dh * silu_grad(z2[u]);
    __syncthreads();
    // layer 2: thread u owns row u of W2
    for (int k = 0; k < kH; ++k) g[kOffW2 + u * kH + k] += dz2[u] * h1[k];
    g[kOffB2 + u] += dz2[u];
    dh = 0.0f;
    for (int v = 0; v < kH; ++v) dh += w[kOffW2 + v * kH + u] * dz2[v];
    dz1[u] = dh * silu_grad(z1[u]);
    __syncthreads();
    for (int k = 0; k < kIn; ++k) g[kOffW1 + u * kIn + k] += dz1[u] * x[k];
    g[kOffB1 + u] += dz1[u];
    __syncthreads();
  }
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) partial[static_cast<size_t>(blockIdx.x) * kParams + i] = g[i];
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = lsum;
}

// fixed-order sum of the block partials
__global__ void k_mlp_reduce(const float *partial, int nblocks, float *grad, const float *loss_partial, float *loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) {
    float s = 0.0f;
    for (int b = 0; b < nblocks; ++b) s += partial[static_cast<size_t>(b) * kParams + i];
    grad[i] = s;
  }
  if (i == 0) {
    float l = 0.0f;
    for (int b = 0; b < nblocks; ++b) l += loss_partial[b];
    *loss = l;
  }
}

__global__ void k_adam(float *params, const float *grad, float *m, float *v, int t, float lr, float b1, float b2,
                       float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float gi = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.0f - powf(b1, static_cast<float>(t)));
  const float vh = vi / (1.0f - powf(b2, static_cast<float>(t)));
  params[i] -= lr * mh / (sqrtf(vh) + eps);
}

}  // namespace

int mlp_param_count() { return kParams; }

}  // namespace cil

// ---------------------------------------------------------------- training C ABI
extern "C" {

cil_status cil_mlp_forward(const float *params, const float *X, int32_t n, float *Y) {
  if (!params || !X || !Y || n < 0) return CIL_ERR_CONFIG;
  const int blocks = (n + cil::kSamplesPerBlock - 1) / cil::kSamplesPerBlock;
  if (blocks > 0) cil::k_mlp_forward<<<blocks, cil::kH>>>(params, X, n, Y);
  return cudaGetLastError() == cudaSuccess ? CIL_OK : CIL_ERR_CUDA;
}

cil_status cil_mlp_grad(const float *params, const float *X, const float *T, const float *out_weights, int32_t n,
                        float *workspace, float *grad, float *loss) {
  if (!params || !X || !T || !out_weights || !workspace || !grad || !loss || n <= 0) return CIL_ERR_CONFIG;
  const int blocks = (n + cil::kSamplesPerBlock - 1) / cil::kSamplesPerBlock;
  float *partial = workspace;
  float *lpart = workspace + static_cast<size_t>(blocks) * cil::kParams;
  cil::k_mlp_backward<<<blocks, cil::kH>>>(params, X, T, out_weights, n, partial, lpart);
  cil::k_mlp_reduce<<<(cil::kParams + 255) / 256, 256>>>(partial, blocks, grad, lpart, loss);
  return cudaGetLastError() == cudaSuccess ? CIL_OK : CIL_ERR_CUDA;
}

cil_status cil_mlp_adam(float *params, const float *grad, float *m, float *v, int32_t t, float lr) {
  if (!params || !grad || !m || !v || t < 1) return CIL_ERR_CONFIG;
  cil::k_adam<<<(cil::kParams + 255) / 256, 256>>>(params, grad, m, v, t, lr, 0.9f, 0.999f, 1e-8f);
  return cudaGetLastError() == cudaSuccess ? CIL_OK : CIL_ERR_CUDA;
}

int32_t cil_mlp_num_params(void) { return cil::kParams; }

int64_t cil_mlp_workspace_floats(int32_t n) {
  const int64_t blocks = (n + cil::kSamplesPerBlock - 1) / cil::kSamplesPerBlock;
  return blocks * (cil::kParams + 1);
}

}  // extern "C"
