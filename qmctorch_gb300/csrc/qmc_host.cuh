// Host-side helpers shared by the translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <utility>
#include <vector>

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
  if (d->use_jastrow_en && (!d->jastrow_en_w || !d->jastrow_en_atoms)) return QMC_ERR_ARG;
  if (d->radial_type < QMC_RADIAL_GTO || d->radial_type > QMC_RADIAL_STO_PURE) return QMC_ERR_ARG;
  if (d->radial_type == QMC_RADIAL_STO && !d->ao_kr) return QMC_ERR_ARG;
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
  // Metropolis: room for the walkers' current positions as split coordinates
  // (launch plans with pos_global)
  if (kind == 2) b += 3 * (int64_t)d->nelec * (d->precision == QMC_PREC_MIXED ? 8 : 16);
  if (kind == 1) {
    qmc_wf_desc dd = *d;
    dd.precision = QMC_PREC_FP64;
    const int64_t t = scratch_layout(dd, 1).bytes_per_slot;
    if (t > b) b = t;
  }
  return b;
}

// Launch plan of an electron-parallel kernel for nw walkers: walkers per
// block (nwb) and threads per walker (nslot; a thread evaluates electrons
// slot, slot + nslot, ...).
//
// Rule, from sweeps of both on GB300 (H2O cc-pVDZ, 16384 walkers):
// * nwb starts at 32 for FP32 and 16 for FP64 (FP64 threads hold twice the
//   registers, so smaller blocks fill the register file in finer steps) and
//   halves while the blocks would not cover the SMs, or the block does not
//   fit the thread bound or 200 KB of shared memory.
// * nslot = ceil(nelec / k) for the smallest k = 1..8 with which every block
//   of the grid is resident at once (CUDA occupancy calculator). The
//   Metropolis kernel is persistent over its steps, so a partial second wave
//   would run alone at the end; fewer slots also give the determinant phase
//   (two threads per walker) a larger share of the block. If no k gives one
//   wave, the k with the best last-wave fill is taken.
// * The FP64 local-energy kernel (heaviest electron phase: AO Hessian
//   diagonals in FP64) keeps one thread per electron (k = 1).
// Plans are cached per (kernel, device, walker count, shape inputs).
template <typename R, typename K>
static inline EPShape ep_plan(const qmc_wf_desc& d, int kind, int jc, K kernel, int64_t nw,
                              int bound = 0, bool* single_wave = nullptr) {
  // bound: the kernel's threads-per-block limit (0: ep_thread_bound); single_wave
  // (optional) receives whether the plan runs every block at once
  if (bound <= 0) bound = ep_thread_bound<R>(kind);
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  const int ne = d.nelec > 0 ? d.nelec : 1;
  const EPShape s1 = ep_shape<R>(d, kind, 1, jc, ne), s2 = ep_shape<R>(d, kind, 2, jc, ne);
  struct Key {
    const void* kernel;
    int dev, kind, jc, ne, bound;
    int64_t nw, smem1, smem2;
    bool operator==(const Key& o) const {
      return kernel == o.kernel && dev == o.dev && kind == o.kind && jc == o.jc && ne == o.ne &&
             bound == o.bound && nw == o.nw && smem1 == o.smem1 && smem2 == o.smem2;
    }
  };
  struct Plan {
    EPShape s;
    bool one_wave;
  };
  const Key key{(const void*)kernel, dev, kind, jc, ne, bound, nw, s1.smem, s2.smem};
  static std::mutex mu;
  static std::vector<std::pair<Key, Plan>> cache;
  {
    std::lock_guard<std::mutex> g(mu);
    for (const auto& kv : cache)
      if (kv.first == key) {
        if (single_wave) *single_wave = kv.second.one_wave;
        return kv.second.s;
      }
  }
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int nwb0 = kMixed<R> ? 32 : 16;
  while (nwb0 > 8 && (nw + nwb0 - 1) / nwb0 < nsm) nwb0 /= 2;
  const int kmax = (kind == 1 && !kMixed<R>) ? 1 : 8;
  EPShape best = s1;
  best.smem = -1;  // nothing fits yet
  double best_fill = -1.0;
  bool one_wave = false;
  // The Metropolis kernel keeps the current positions in shared memory; when
  // no plan gives one wave that way, a second pass moves them to the
  // (L2-resident) scratch, read once per step by the proposal and written on
  // acceptance, which frees a position row per walker of shared memory.
  for (int pg = 0; pg < (kind == 2 ? 2 : 1) && !one_wave; ++pg)
  for (int nwb = nwb0; nwb >= 1 && !one_wave; nwb /= 2) {
    // the first block size that fits is kept, except by the persistent
    // Metropolis kernel (kind 2), which halves it down to 8 walkers while no
    // thread split gives a single wave (a partial last wave would run alone
    // for all the launch's steps); a smaller size must fill strictly better
    if (best.smem >= 0 && (kind != 2 || nwb < 8)) break;
    for (int k = 1; k <= kmax; ++k) {
      const int nslot = (ne + k - 1) / k;
      if (k > 1 && nslot == (ne + k - 2) / (k - 1)) continue;  // same slot count as k - 1
      const EPShape s = ep_shape<R>(d, kind, nwb, jc, nslot, pg == 1);
      if (s.nthreads > bound || s.smem > 200 * 1024) continue;
      if (prepare_smem(kernel, s.smem) != QMC_OK) continue;
      int occ = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, s.nthreads, s.smem) !=
              cudaSuccess ||
          occ < 1) {
        cudaGetLastError();
        continue;
      }
      const int64_t blocks = (nw + nwb - 1) / nwb, slots = (int64_t)occ * nsm;
      if (blocks <= slots) {  // one wave
        best = s;
        one_wave = true;
        break;
      }
      const double fill = (double)blocks / (double)(((blocks + slots - 1) / slots) * slots);
      if (fill > best_fill) {
        best = s;
        best_fill = fill;
      }
    }
  }
  if (best.smem >= 0) {
    std::lock_guard<std::mutex> g(mu);
    if (cache.size() > 256) cache.clear();
    cache.emplace_back(key, Plan{best, one_wave});
  }
  if (single_wave) *single_wave = one_wave;
  return best;
}

}  // namespace qmc
