/*
 * qmc_gb300_probe.h -- measurement helper of the benchmark; it has no
 * counterpart in the reference.
 *
 * qmc_probe_fma launches `blocks` x 256 threads, each running `iters`
 * iterations of 8 independent fused multiply-add chains (kind 0: FP64,
 * kind 1: FP32) or exp evaluations (kind 2: FP32 __expf, the SFU path;
 * kind 3: FP64 exp, the library's; kind 4: FP64 exp of the fused kernels'
 * radial factors, the table-driven method). out[blocks*256] receives one value
 * per thread so the work cannot be elided. Timing the launch gives the pipe's
 * throughput: kinds 0/1: 2 * 8 * iters * threads flop; kinds 2-4:
 * 8 * iters * threads exp.
 *
 * qmc_probe_exp64 evaluates the FP64 exp of the radial factors, y[i] = exp(x[i]),
 * with the kernels' own function (for the accuracy test against the library's).
 */
#ifndef QMC_GB300_PROBE_H
#define QMC_GB300_PROBE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
int qmc_probe_fma(int32_t kind, int32_t blocks, int64_t iters, double* out, void* stream);
int qmc_probe_exp64(const double* x, int64_t n, double* y, void* stream);
#ifdef __cplusplus
}
#endif
#endif
