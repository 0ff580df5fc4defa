// One (R, JC) instantiation of the Metropolis kernels; the build compiles this
// file once per pair with -DQMC_INST_R=<float|double> -DQMC_INST_JC=<8|16|24>.
#include "qmc_metropolis.cuh"

#if !defined(QMC_INST_R) || !defined(QMC_INST_JC)
#error "compile with -DQMC_INST_R=<float|double> -DQMC_INST_JC=<8|16|24>"
#endif

namespace qmc {
template int launch_metropolis<QMC_INST_R, QMC_INST_JC>(const qmc_wf_desc*,
                                                        const qmc_metropolis_args*,
                                                        unsigned char*, cudaStream_t);
template int plan_metropolis<QMC_INST_R, QMC_INST_JC>(const qmc_wf_desc*, int64_t, int32_t*);
template int launch_metropolis_batch<QMC_INST_R, QMC_INST_JC>(const qmc_wf_desc*,
                                                              const qmc_metropolis_args*,
                                                              void* const*, int, cudaStream_t);
}  // namespace qmc
