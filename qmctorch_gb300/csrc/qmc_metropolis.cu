// Persistent Metropolis sampler: C entry points (kernels in qmc_metropolis.cuh).
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_metropolis.cuh"

// instantiated in qmc_metropolis_inst.cu (one translation unit per pair)
namespace qmc {
#define QMC_MET_EXTERN(R, JC)                                                                  \
  extern template int launch_metropolis<R, JC>(const qmc_wf_desc*, const qmc_metropolis_args*, \
                                               unsigned char*, cudaStream_t);                  \
  extern template int launch_metropolis_batch<R, JC>(const qmc_wf_desc*,                       \
                                                     const qmc_metropolis_args*, void* const*, \
                                                     int, cudaStream_t);                  \
  extern template int plan_metropolis<R, JC>(const qmc_wf_desc*, int64_t, int32_t*);
QMC_MET_EXTERN(float, 8)
QMC_MET_EXTERN(float, 16)
QMC_MET_EXTERN(float, 24)
QMC_MET_EXTERN(double, 8)
QMC_MET_EXTERN(double, 16)
QMC_MET_EXTERN(double, 24)
#undef QMC_MET_EXTERN
}  // namespace qmc


using namespace qmc;

// qmc_sweep.cu: Sherman-Morrison single-electron moves
int qmc_sweep_run(const qmc_wf_desc* d, const qmc_metropolis_args* a, void* stream);
bool qmc_sweep_eligible(const qmc_wf_desc* d, const qmc_metropolis_args* a);

// column-chunk class of the electron-parallel kernels (JC = 8, 16, 24)
static inline int mo_chunk_class(int nmo_used) { return nmo_used <= 8 ? 0 : (nmo_used <= 16 ? 1 : 2); }

extern "C" {

int qmc_metropolis_run(const qmc_wf_desc* d, const qmc_metropolis_args* a, void* scratch,
                       int64_t scratch_bytes, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (!a || a->nwalkers < 0 || a->nstep < 0 || a->ndecor < 1 || a->ntherm < 0) return QMC_ERR_ARG;
  if (a->move_type < 0 || a->move_type > 2 || a->proba < 0 || a->proba > 1) return QMC_ERR_ARG;
  if (a->nwalkers == 0 || a->nstep == 0) return QMC_OK;
  if (!a->pos || !scratch) return QMC_ERR_ARG;
  if (a->samples && a->nsnap < 0) return QMC_ERR_ARG;
  if (a->proposals && !a->uniforms) return QMC_ERR_ARG;
  if (a->proposals && a->move_type == QMC_MOVE_ONE_ELEC && !a->electron_index) return QMC_ERR_ARG;
  if (scratch_bytes < qmc_metropolis_scratch_bytes(d, a->nwalkers)) return QMC_ERR_SCRATCH;
  if (qmc_sweep_eligible(d, a)) return qmc_sweep_run(d, a, stream);
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* scr = (unsigned char*)scratch;
  if (d->precision == QMC_PREC_MIXED) {
    if (d->nmo_used <= 8) return launch_metropolis<float, 8>(d, a, scr, s);
    if (d->nmo_used <= 16) return launch_metropolis<float, 16>(d, a, scr, s);
    return launch_metropolis<float, 24>(d, a, scr, s);
  }
  if (d->nmo_used <= 8) return launch_metropolis<double, 8>(d, a, scr, s);
  if (d->nmo_used <= 16) return launch_metropolis<double, 16>(d, a, scr, s);
  return launch_metropolis<double, 24>(d, a, scr, s);
}

int qmc_metropolis_plan(const qmc_wf_desc* d, int64_t nwalkers, int32_t* plan) {
  int st = check_desc(d);
  if (st) return st;
  if (!plan || nwalkers < 1) return QMC_ERR_ARG;
  if (d->precision == QMC_PREC_MIXED) {
    if (d->nmo_used <= 8) return plan_metropolis<float, 8>(d, nwalkers, plan);
    if (d->nmo_used <= 16) return plan_metropolis<float, 16>(d, nwalkers, plan);
    return plan_metropolis<float, 24>(d, nwalkers, plan);
  }
  if (d->nmo_used <= 8) return plan_metropolis<double, 8>(d, nwalkers, plan);
  if (d->nmo_used <= 16) return plan_metropolis<double, 16>(d, nwalkers, plan);
  return plan_metropolis<double, 24>(d, nwalkers, plan);
}

int qmc_metropolis_run_batch(const qmc_wf_desc* descs, const qmc_metropolis_args* args,
                             void* const* scratch, const int64_t* scratch_bytes, int32_t njobs,
                             void* stream) {
  if (njobs < 1 || njobs > QMC_MAX_BATCH || !descs || !args || !scratch || !scratch_bytes)
    return QMC_ERR_ARG;
  for (int j = 0; j < njobs; ++j) {
    const qmc_wf_desc* d = descs + j;
    const qmc_metropolis_args* a = args + j;
    int st = check_desc(d);
    if (st) return st;
    if (a->nwalkers < 0 || a->nstep < 0 || a->ndecor < 1 || a->ntherm < 0 || a->proba < 0 ||
        a->proba > 1)
      return QMC_ERR_ARG;
    if (a->move_type != QMC_MOVE_ALL_ELEC || a->proposals || a->psi_out)
      return QMC_ERR_UNSUPPORTED;
    if (a->nwalkers > 0 && (!a->pos || !scratch[j])) return QMC_ERR_ARG;
    if (a->samples && a->nsnap < 0) return QMC_ERR_ARG;
    if (scratch_bytes[j] < qmc_metropolis_scratch_bytes(d, a->nwalkers)) return QMC_ERR_SCRATCH;
    if (d->precision != descs[0].precision ||
        mo_chunk_class(d->nmo_used) != mo_chunk_class(descs[0].nmo_used))
      return QMC_ERR_SHAPE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const qmc_wf_desc* d = descs;
  if (d->precision == QMC_PREC_MIXED) {
    if (d->nmo_used <= 8) return launch_metropolis_batch<float, 8>(descs, args, scratch, njobs, s);
    if (d->nmo_used <= 16) return launch_metropolis_batch<float, 16>(descs, args, scratch, njobs, s);
    return launch_metropolis_batch<float, 24>(descs, args, scratch, njobs, s);
  }
  if (d->nmo_used <= 8) return launch_metropolis_batch<double, 8>(descs, args, scratch, njobs, s);
  if (d->nmo_used <= 16) return launch_metropolis_batch<double, 16>(descs, args, scratch, njobs, s);
  return launch_metropolis_batch<double, 24>(descs, args, scratch, njobs, s);
}

}  // extern "C"
