// Host-side helpers shared by the translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_device.cuh"
#include "qmc_ep.cuh"

namespace qmc {

constexpr int kTPB = 32;  // threads (= walkers) per block: one warp, for balance over 152 SMs

__host__ __device__ inline int64_t pad_walkers(int64_t nw) { return (nw + 31) & ~int64_t(31); }

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
static inline int check_desc(const qmc_wf_desc* d) {
  if (!d) return QMC_ERR_ARG;
  if (d->nelec != d->nup + d->ndown || d->nup < 0 || d->ndown < 0) return QMC_ERR_ARG;
  if (d->nup > QMC_MAX_NSPIN || d->ndown > QMC_MAX_NSPIN) return QMC_ERR_SHAPE;
  if (!d->atom_coords || !d->atom_charge || !d->group_atom || !d->group_prim || !d->group_ao ||
      !d->gprim_entry || !d->bas_exp || !d->ao_k || !d->ao_wofs || !d->weight_entry || !d->ao_wd || !d->mo_scf ||
      !d->mo_modifier || !d->ci_weight || !d->cfg_det[0] || !d->cfg_det[1])
    return QMC_ERR_ARG;
  if (!d->contract && !d->ao_wv) return QMC_ERR_ARG;
  if (d->use_jastrow && !d->jastrow_w) return QMC_ERR_ARG;
  if (d->nmo_used > d->nmo || d->nmo_used < 1) return QMC_ERR_ARG;
  if (d->det_mode != QMC_DET_EXCITATION && d->det_mode != QMC_DET_EXPLICIT) return QMC_ERR_ARG;
  if (d->precision != QMC_PREC_FP64 && d->precision != QMC_PREC_MIXED) return QMC_ERR_ARG;
  return QMC_OK;
}

static inline int launch_status() {
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? QMC_OK : QMC_ERR_LAUNCH;
}

template <typename K>
static inline int prepare_smem(K kernel, int64_t bytes) {
  if (bytes > 227 * 1024) return QMC_ERR_SHAPE;
  if (bytes > 48 * 1024) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) !=
        cudaSuccess)
      return QMC_ERR_LAUNCH;
  }
  return QMC_OK;
}

// Per-walker scratch bytes: the fused kernels use the electron-parallel
// layout (kinds 0 psi, 1 local energy, 2 Metropolis); kind 1 also covers the
// staged pooling kernel (one thread per walker, FP64).
static inline int64_t scratch_slot_bytes(const qmc_wf_desc* d, int kind) {
  int64_t b = ep_layout(*d, kind == 2 ? 0 : kind).bytes_per_slot;
  if (kind == 1) {
    qmc_wf_desc dd = *d;
    dd.precision = QMC_PREC_FP64;
    const int64_t t = scratch_layout(dd, 1).bytes_per_slot;
    if (t > b) b = t;
  }
  return b;
}

}  // namespace qmc
