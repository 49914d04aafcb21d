// Posterior over mixture components per column (MixturePosterior,
// subby/jax/__init__.py:653-678; subby/jax/mixture.py:6-28; oracle
// subby/oracle/oracle.py:1334-1365): softmax over k of logL[k][c] + logw[k],
// max-shifted.  One thread per column, K log-likelihoods read with a stride
// of C (coalesced across the warp's columns).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "common.cuh"
#include "subby_gb300.h"

namespace subby {
namespace {

__global__ void k_mixture(const float *__restrict__ logL, const double *__restrict__ logw, int K, int C,
                          float *__restrict__ out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    float m = -INFINITY;
    for (int k = 0; k < K; ++k) m = fmaxf(m, logL[(size_t)k * C + c] + (float)logw[k]);
    float s = 0.f;
    for (int k = 0; k < K; ++k) s += expf(logL[(size_t)k * C + c] + (float)logw[k] - m);
    const float inv = 1.0f / s;
    for (int k = 0; k < K; ++k) out[(size_t)k * C + c] = expf(logL[(size_t)k * C + c] + (float)logw[k] - m) * inv;
  }
}

}  // namespace
}  // namespace subby

extern "C" int subby_mixture_posterior(const float *logL, const double *log_weights, int K, int C, float *out,
                                       int flags, void *stream_) {
  if (!log_weights || K <= 0 || C < 0) return SUBBY_ERR_ARG;
  if (C == 0) return SUBBY_OK;  // empty device buffers may be null
  if (!logL || !out) return SUBBY_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream_;
  const int block = 256;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = (int)std::min<long long>(((long long)C + block - 1) / block, (long long)nsm * 8);
  if (flags & SUBBY_DEVICE_PTRS) {
    // log_weights is always a host array (K values): staged through device memory
    double *dw = nullptr;
    if (cudaMallocAsync((void **)&dw, sizeof(double) * K, s) != cudaSuccess) return SUBBY_ERR_NOMEM;
    cudaMemcpyAsync(dw, log_weights, sizeof(double) * K, cudaMemcpyHostToDevice, s);
    subby::k_mixture<<<grid, block, 0, s>>>(logL, dw, K, C, out);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(dw, s);
    return e == cudaSuccess ? SUBBY_OK : SUBBY_ERR_CUDA;
  }
  const size_t nb = (size_t)K * C * sizeof(float);
  char *buf = nullptr;
  if (cudaMallocAsync((void **)&buf, 2 * nb + sizeof(double) * K + 256, s) != cudaSuccess) return SUBBY_ERR_NOMEM;
  float *dl = (float *)buf, *dout = (float *)(buf + nb);
  double *dw = (double *)(buf + ((2 * nb + 255) & ~(size_t)255));
  cudaMemcpyAsync(dl, logL, nb, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dw, log_weights, sizeof(double) * K, cudaMemcpyHostToDevice, s);
  subby::k_mixture<<<grid, block, 0, s>>>(dl, dw, K, C, dout);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, nb, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? SUBBY_OK : SUBBY_ERR_CUDA;
}
