// Pipe-throughput probe used by the benchmark to measure the FP64 / FP32 /
// exp peaks of the GPU it runs on (see include/qmc_gb300_probe.h).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qmc_gb300_probe.h"
#include "qmc_device.cuh"

template <typename T>
__global__ void __launch_bounds__(256) fma_probe(int64_t iters, double* out) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (T)(1.0 + 1e-7 * (tid + k));
  const T b = (T)0.9999999, c = (T)1e-7;
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[tid] = (double)s;
}

template <typename T, bool TANG = false>
__global__ void __launch_bounds__(256) exp_probe(int64_t iters, double* out) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = (T)(-1e-3 * (k + 1)) - (T)(1e-9 * tid);
  for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if constexpr (sizeof(T) == 4)
        a[k] = -__expf(a[k]) * (T)1e-3;
      else if (TANG)
        a[k] = -qmc::exp_tang(a[k]) * (T)1e-3;
      else
        a[k] = -exp(a[k]) * (T)1e-3;
    }
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[tid] = (double)s;
}

extern "C" int qmc_probe_fma(int32_t kind, int32_t blocks, int64_t iters, double* out,
                             void* stream) {
  if (blocks <= 0 || iters <= 0 || !out || kind < 0 || kind > 4) return 1;
  cudaStream_t s = (cudaStream_t)stream;
  if (kind == 0) fma_probe<double><<<blocks, 256, 0, s>>>(iters, out);
  if (kind == 1) fma_probe<float><<<blocks, 256, 0, s>>>(iters, out);
  if (kind == 2) exp_probe<float><<<blocks, 256, 0, s>>>(iters, out);
  if (kind == 3) exp_probe<double><<<blocks, 256, 0, s>>>(iters, out);
  if (kind == 4) exp_probe<double, true><<<blocks, 256, 0, s>>>(iters, out);
  return cudaGetLastError() == cudaSuccess ? 0 : 4;
}

__global__ void __launch_bounds__(256) exp64_eval(const double* __restrict__ x, int64_t n,
                                                  double* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = qmc::rexp(x[i]);
}

extern "C" int qmc_probe_exp64(const double* x, int64_t n, double* y, void* stream) {
  if (n < 0 || (n > 0 && (!x || !y))) return 1;
  if (n == 0) return 0;
  exp64_eval<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(x, n, y);
  return cudaGetLastError() == cudaSuccess ? 0 : 4;
}
