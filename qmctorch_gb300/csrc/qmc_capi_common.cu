// Host-only entry points: status strings, version, scratch sizes.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

using namespace qmc;

extern "C" {

const char* qmc_version(void) { return "qmc_gb300 0.1 (sm_103a)"; }

const char* qmc_status_string(int s) {
  switch (s) {
    case QMC_OK: return "ok";
    case QMC_ERR_ARG: return "invalid argument";
    case QMC_ERR_SHAPE: return "size beyond the compiled limits";
    case QMC_ERR_SCRATCH: return "scratch buffer too small";
    case QMC_ERR_LAUNCH: return "CUDA launch error";
    case QMC_ERR_UNSUPPORTED: return "unsupported option";
    case QMC_ERR_STATIC_LIMIT:
      return "batch needs more scratch than the static array of qmc_wf_psi_static holds";
    case QMC_ERR_TIMEOUT: return "a bounded pipeline wait of a kernel ran out (results are NaN)";
    default: return "unknown status";
  }
}

int64_t qmc_scratch_bytes(const qmc_wf_desc* d, int64_t nw, int32_t kind) {
  if (check_desc(d) != QMC_OK || nw < 0 || kind < 0 || kind > 1) return -1;
  return scratch_slot_bytes(d, kind) * pad_walkers(nw);
}

int64_t qmc_metropolis_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  if (check_desc(d) != QMC_OK || nw < 0) return -1;
  return scratch_slot_bytes(d, 2) * pad_walkers(nw);
}

}  // extern "C"
