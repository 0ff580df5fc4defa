// Compensated walker statistics: mean, unbiased variance and the sampling
// error sqrt(var / n) of the local energies (SolverBase.single_point,
// solver_base.py:316-387, with WaveFunction.sampling_error, wf_base.py:225-229,
// which use torch.mean / torch.var).
//
// Two passes (mean, then squared deviations), each a compensated sum: every
// thread keeps a Neumaier pair (sum, error), pairs are merged with TwoSum in a
// fixed tree order inside the block, blocks write their pairs to scratch and
// the last block to finish (atomic ticket, no waiting) merges them in block
// order. The result depends only on n, never on scheduling.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_gb300.h"
#include "qmc_host.cuh"

namespace qmc {

constexpr int kRedThreads = 256;
constexpr int kRedMaxBlocks = 592;  // 4 x 148+ SMs, enough to stream n at full bandwidth

struct KSum {
  double s, c;
};

__device__ __forceinline__ KSum ksum_add(KSum a, double x) {
  const double t = a.s + x;
  const double e = fabs(a.s) >= fabs(x) ? (a.s - t) + x : (x - t) + a.s;
  return KSum{t, a.c + e};
}
__device__ __forceinline__ KSum ksum_merge(KSum a, KSum b) {
  KSum r = ksum_add(a, b.s);
  r.c += b.c;
  return r;
}

// Block tree merge of two pairs per thread (values v0, v1); thread 0 gets the result.
__device__ inline void block_merge(KSum& v0, KSum& v1, KSum* sh0, KSum* sh1) {
  const int tid = threadIdx.x;
  sh0[tid] = v0;
  sh1[tid] = v1;
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if (tid < h) {
      sh0[tid] = ksum_merge(sh0[tid], sh0[tid + h]);
      sh1[tid] = ksum_merge(sh1[tid], sh1[tid + h]);
    }
    __syncthreads();
  }
  v0 = sh0[0];
  v1 = sh1[0];
}

// pass 0: sum x -> stats[0] = mean. pass 1: sums of d = x - mean and d^2 ->
// stats[1] = (sum d^2 - (sum d)^2 / n) / (n - 1), stats[2] = sqrt(stats[1] / n).
template <int PASS>
__global__ void __launch_bounds__(kRedThreads)
    stats_kernel(const double* __restrict__ x, int64_t n, double* __restrict__ stats,
                 KSum* __restrict__ part, unsigned int* __restrict__ ticket) {
  __shared__ KSum sh0[kRedThreads], sh1[kRedThreads];
  __shared__ bool last;
  const double mean = PASS == 1 ? stats[0] : 0.0;
  KSum a{0.0, 0.0}, b{0.0, 0.0};
  const int64_t stride = (int64_t)gridDim.x * kRedThreads;
  for (int64_t i = (int64_t)blockIdx.x * kRedThreads + threadIdx.x; i < n; i += stride) {
    if (PASS == 0) {
      a = ksum_add(a, x[i]);
    } else {
      const double dv = x[i] - mean;
      a = ksum_add(a, dv * dv);
      b = ksum_add(b, dv);
    }
  }
  block_merge(a, b, sh0, sh1);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last block merges the block pairs in block order
  KSum ta{0.0, 0.0}, tb{0.0, 0.0};
  for (int k = threadIdx.x; k < (int)gridDim.x; k += kRedThreads) {
    const double* p = reinterpret_cast<const double*>(part + 2 * k);
    ta = ksum_merge(ta, KSum{__ldcg(p), __ldcg(p + 1)});
    tb = ksum_merge(tb, KSum{__ldcg(p + 2), __ldcg(p + 3)});
  }
  block_merge(ta, tb, sh0, sh1);
  if (threadIdx.x == 0) {
    const double nd = (double)n;
    if (PASS == 0) {
      stats[0] = (ta.s + ta.c) / nd;
    } else {
      const double sd2 = ta.s + ta.c, sd = tb.s + tb.c;
      const double var = n > 1 ? (sd2 - sd * sd / nd) / (nd - 1.0) : __longlong_as_double(0x7ff8000000000000LL);
      stats[1] = var;
      stats[2] = sqrt(var / nd);
    }
    *ticket = 0u;  // ready for the next pass
  }
}

static int reduce_blocks(int64_t n) {
  int64_t b = (n + 4 * kRedThreads - 1) / (4 * kRedThreads);
  if (b < 1) b = 1;
  if (b > kRedMaxBlocks) b = kRedMaxBlocks;
  return (int)b;
}

}  // namespace qmc

using namespace qmc;

extern "C" {

int64_t qmc_reduce_scratch_bytes(int64_t n) {
  return 16 + (int64_t)reduce_blocks(n) * 2 * (int64_t)sizeof(KSum);
}

int qmc_reduce_stats(const double* x, int64_t n, double* stats, void* scratch,
                     int64_t scratch_bytes, void* stream) {
  if (n < 1 || !x || !stats || !scratch) return QMC_ERR_ARG;
  if (scratch_bytes < qmc_reduce_scratch_bytes(n)) return QMC_ERR_SCRATCH;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* base = (unsigned char*)scratch;
  unsigned int* ticket = (unsigned int*)base;
  KSum* part = (KSum*)(base + 16);
  const int nb = reduce_blocks(n);
  if (cudaMemsetAsync(ticket, 0, sizeof(unsigned int), s) != cudaSuccess) return QMC_ERR_LAUNCH;
  stats_kernel<0><<<nb, kRedThreads, 0, s>>>(x, n, stats, part, ticket);
  stats_kernel<1><<<nb, kRedThreads, 0, s>>>(x, n, stats, part, ticket);
  return launch_status();
}

}  // extern "C"
