/*
 * qmc_gb300_probe.h -- measurement helper of the benchmark; it has no
 * counterpart in the reference.
 *
 * qmc_probe_fma launches `blocks` x 256 threads, each running `iters`
 * iterations of 8 independent fused multiply-add chains (kind 0: FP64,
 * kind 1: FP32) or exp evaluations (kind 2: FP32 __expf, the SFU path;
 * kind 3: FP64 exp). out[blocks*256] receives one value per thread so the work
 * cannot be elided. Timing the launch gives the pipe's throughput:
 * kinds 0/1: 2 * 8 * iters * threads flop; kinds 2/3: 8 * iters * threads exp.
 */
#ifndef QMC_GB300_PROBE_H
#define QMC_GB300_PROBE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
int qmc_probe_fma(int32_t kind, int32_t blocks, int64_t iters, double* out, void* stream);
#ifdef __cplusplus
}
#endif
#endif
