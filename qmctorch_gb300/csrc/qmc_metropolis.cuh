// Persistent Metropolis sampler kernels (templates on the compute type R and
// the MO column chunk JC). Each (R, JC) pair is instantiated in its own
// translation unit (qmc_metropolis_inst.cu compiled once per pair), so the
// library builds in parallel; qmc_metropolis.cu holds the C entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_ep.cuh"
#include "qmc_host.cuh"
#include "qmc_rng.cuh"

#include <mutex>

namespace qmc {

// One block advances `nwb` walker chains through all steps. Per move: every
// electron thread writes its proposed coordinates (Philox normals or the
// replay input), the block evaluates psi at the proposal (qmc_ep.cuh), the
// walker's combine thread takes the accept decision, and the electron threads
// copy accepted coordinates. Generator: counter (call, walker, step), key
// (seed); call = move * (nelec + 2) + e for electron e's three normals,
// + nelec for the accept uniform, + nelec + 1 for the one-elec electron index.
template <typename R, int JC>
__device__ __forceinline__ void metropolis_block(const qmc_wf_desc& d, const qmc_metropolis_args& a,
                                                 unsigned char* __restrict__ scr, int64_t ss,
                                                 const EPShape& S, int64_t block,
                                                 unsigned char* smem) {
  const Tables<R> t = load_tables<R>(d, d.nmo_used, S.ncol, smem + S.o_tab);
  const int64_t nw = a.nwalkers;
  const int nwb = S.nwb, ne = d.nelec, nc = 3 * ne, ps = S.pstride;
  const int64_t w0 = block * nwb;
  const int tid = threadIdx.x;
  const int slot = tid / nwb, wl = tid - (tid / nwb) * nwb;
  const int nslot = S.nslot;
  const int64_t w = w0 + wl;
  const bool active = slot < nslot;    // an electron slot (electrons slot, slot + nslot, ...)
  const bool live = active && w < nw;  // ... of a real walker
  XP<R>* PN = reinterpret_cast<XP<R>*>(smem + S.o_pnew);  // proposal
  // current positions: coordinate q of electron e of local walker wl at
  // P[wl * pw + (3 e + q) * pq]; a block row in shared memory, or the
  // [coordinate][walker] array after the determinant work arrays in scratch
  XP<R>* P;
  int64_t pw, pq;
  if (S.pos_global) {
    P = reinterpret_cast<XP<R>*>(scr + ep_layout(d, 0).bytes_per_slot * ss) + w0;
    pw = 1;
    pq = ss;
  } else {
    P = reinterpret_cast<XP<R>*>(smem + S.o_pos);
    pw = ps;
    pq = 1;
  }
  double* PSI = reinterpret_cast<double*>(smem + S.o_psi);
  double* F = reinterpret_cast<double*>(smem + S.o_f);
  int* IEL = reinterpret_cast<int*>(smem + S.o_iel);
  int* ACC = reinterpret_cast<int*>(smem + S.o_acc);
  const EPPtrs ptrs{smem, S};
  const double eps = 1e-16;
  // the first evaluation reads the staged positions from the proposal rows
  ep_stage_positions<R>(a.pos, w0, nw, nwb, nc, ps, PN);
  for (int i = tid; i < nwb * nc; i += blockDim.x) {
    const int wl2 = i / nc, c = i - wl2 * nc;
    P[wl2 * pw + c * pq] = PN[wl2 * ps + c];
  }
  ep_eval<R, JC, false>(d, t, ptrs, PN, scr, ss, w0, nw);
  int nacc = 0;
  double psi_cur = 0.0;  // combine threads: psi at the current positions
  if (tid < nwb) {
    psi_cur = PSI[tid];
    const double f = psi_cur * psi_cur;
    F[tid] = f == 0.0 ? eps : f;
  }
  const double sigma = a.step_size / (2.0 * sqrt(2.0 * log(2.0)));
  const double sd = sqrt(sigma);  // MultivariateNormal(0, sigma I): std = sqrt(sigma)
  Rng rng{(uint32_t)a.seed, (uint32_t)(a.seed >> 32), (uint32_t)w, 0, 0};
  const int nmove = a.move_type == QMC_MOVE_ALL_ELEC_ITER ? ne : 1;
  int64_t isnap = 0, idecor = 0;
  for (int istep = 0; istep < a.nstep; ++istep) {
    rng.step = a.step_offset + istep;
    for (int im = 0; im < nmove; ++im) {
      const uint32_t call0 = (uint32_t)im * (uint32_t)(ne + 2);
      // which electron moves
      if (a.move_type == QMC_MOVE_ONE_ELEC) {
        if (tid < nwb) {
          int iel = 0;
          if (w0 + tid < nw) {
            if (a.proposals) {
              iel = a.electron_index[(int64_t)istep * nw + w0 + tid];
            } else {
              iel = electron_draw(rng, call0 + ne + 1, ne);
            }
          }
          IEL[tid] = iel;
        }
        __syncthreads();
      }
      // proposal
      for (int e = slot; e < ne && active; e += nslot) {
        const bool moves = live && (a.move_type == QMC_MOVE_ALL_ELEC ||
                                    (a.move_type == QMC_MOVE_ALL_ELEC_ITER ? e == im : e == IEL[wl]));
        XP<R>* pn = PN + wl * ps + 3 * e;
        const XP<R> pc[3] = {P[wl * pw + (3 * e) * pq], P[wl * pw + (3 * e + 1) * pq],
                             P[wl * pw + (3 * e + 2) * pq]};
        if (moves) {
          const double* rp =
              !a.proposals ? nullptr
              : a.move_type == QMC_MOVE_ALL_ELEC
                  ? a.proposals + ((int64_t)istep * nw + w) * nc + 3 * e
                  : a.proposals + (((int64_t)istep * nmove + im) * nw + w) * 3;
          propose_electron<R>(rng, call0 + e, a.proba, a.step_size, sd, rp, pc, pn);
        } else {
          for (int q = 0; q < 3; ++q) pn[q] = pc[q];
        }
      }
      __syncthreads();
      ep_eval<R, JC, false>(d, t, ptrs, PN, scr, ss, w0, nw);
      // accept / reject (metropolis.py:141-160, 279-298)
      if (tid < nwb && w0 + tid < nw) {
        double u;
        if (a.proposals) {
          u = a.move_type == QMC_MOVE_ALL_ELEC
                  ? a.uniforms[(int64_t)istep * nw + w0 + tid]
                  : a.uniforms[((int64_t)istep * nmove + im) * nw + w0 + tid];
        } else {
          u = accept_uniform(rng, call0 + ne);
        }
        double fxn = PSI[tid] * PSI[tid];
        if (fxn == 0.0) fxn = eps;
        int acc;
        if constexpr (kMixed<R>) {
          // min(1, fxn / F) - u >= 0 for u in [0, 1) without the FP64 division
          // (a sequence of FP64 instructions in the single-warp phase): the
          // same decision up to the rounding of the ratio
          acc = fxn >= u * F[tid] ? 1 : 0;
        } else {
          double df = fxn / F[tid];
          if (df > 1.0) df = 1.0;
          acc = (df - u >= 0.0) ? 1 : 0;
        }
        ACC[tid] = acc;
        if (acc) {
          F[tid] = fxn;
          psi_cur = PSI[tid];
          ++nacc;
        }
      }
      __syncthreads();
      if (live && ACC[wl])
        for (int e = slot; e < ne; e += nslot)
          for (int q = 0; q < 3; ++q) P[wl * pw + (3 * e + q) * pq] = PN[wl * ps + 3 * e + q];
      __syncthreads();
    }
    if (istep >= a.ntherm) {
      if (idecor % a.ndecor == 0) {
        if (a.samples && isnap < a.nsnap && live)
          for (int e = slot; e < ne; e += nslot) {
            double* out = a.samples + (isnap * nw + w) * nc + 3 * e;
            for (int q = 0; q < 3; ++q) out[q] = xp_value<R>(P[wl * pw + (3 * e + q) * pq]);
          }
        ++isnap;
      }
      ++idecor;
    }
  }
  if (live)
    for (int e = slot; e < ne; e += nslot)
      for (int q = 0; q < 3; ++q) a.pos[w * nc + 3 * e + q] = xp_value<R>(P[wl * pw + (3 * e + q) * pq]);
  if (tid < nwb && w0 + tid < nw) {
    if (a.accepted) a.accepted[w0 + tid] += nacc;
    if (a.psi_out) a.psi_out[w0 + tid] = psi_cur;
  }
}

template <typename R, int JC>
__global__ void __launch_bounds__(EPBound<R>::kThreads)
    metropolis_kernel(const __grid_constant__ qmc_wf_desc d,
                      const __grid_constant__ qmc_metropolis_args a, unsigned char* __restrict__ scr,
                      int64_t ss, const __grid_constant__ EPShape S) {
  extern __shared__ __align__(16) unsigned char smem[];
  metropolis_block<R, JC>(d, a, scr, ss, S, blockIdx.x, smem);
}

// Several independent jobs in one launch: molecules of any size whose MO
// column count falls in this kernel's chunk class (JC), in one precision. The
// job table travels in the kernel parameters with each job's own launch plan
// (walkers per block, electron slots, shared-memory offsets: the plan the job
// would get alone); block b serves job j with block0[j] <= b < block0[j + 1].
// The block size and the dynamic shared memory are the largest over the jobs;
// threads past a job's plan idle through its barriers.
struct MetBatchJob {
  qmc_wf_desc d;
  qmc_metropolis_args a;
  unsigned char* scr;
  int64_t ss;
  EPShape S;
};
struct MetBatch {
  int32_t njobs;
  int64_t block0[QMC_MAX_BATCH + 1];
  MetBatchJob job[QMC_MAX_BATCH];
};
static_assert(sizeof(MetBatch) <= 32000, "kernel parameter block above the 32 KB limit");

template <typename R, int JC>
__global__ void __launch_bounds__(EPBound<R>::kThreads)
    metropolis_batch_kernel(const __grid_constant__ MetBatch b) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t bid = blockIdx.x;
  int j = 0;
  while (j + 1 < b.njobs && b.block0[j + 1] <= bid) ++j;
  const MetBatchJob& J = b.job[j];
  metropolis_block<R, JC>(J.d, J.a, J.scr, J.ss, J.S, bid - b.block0[j], smem);
}

template <typename R, int JC>
int launch_metropolis_batch(const qmc_wf_desc* descs, const qmc_metropolis_args* args,
                            void* const* scratch, int njobs, cudaStream_t s) {
  static MetBatch b;  // host staging of the parameter block (copied at launch)
  static std::mutex mu;
  std::lock_guard<std::mutex> g(mu);
  int64_t smem = 0;
  int nthreads = 32;
  b.njobs = njobs;
  b.block0[0] = 0;
  for (int j = 0; j < njobs; ++j) {
    const int64_t nw = args[j].nwalkers > 0 ? args[j].nwalkers : 1;
    const EPShape S = ep_plan<R>(descs[j], 2, JC, metropolis_batch_kernel<R, JC>, nw);
    if (S.smem < 0 || S.smem > 227 * 1024 || S.nthreads > EPBound<R>::kThreads)
      return QMC_ERR_SHAPE;
    if (S.smem > smem) smem = S.smem;
    if (S.nthreads > nthreads) nthreads = S.nthreads;
    b.job[j].d = descs[j];
    b.job[j].a = args[j];
    b.job[j].scr = (unsigned char*)scratch[j];
    b.job[j].ss = pad_walkers(args[j].nwalkers);
    b.job[j].S = S;
    b.block0[j + 1] = b.block0[j] + (args[j].nwalkers + S.nwb - 1) / S.nwb;
  }
  if (b.block0[njobs] == 0) return QMC_OK;
  int st = prepare_smem(metropolis_batch_kernel<R, JC>, smem);
  if (st) return st;
  metropolis_batch_kernel<R, JC><<<(unsigned)b.block0[njobs], nthreads, smem, s>>>(b);
  return launch_status();
}

// The FP32 kernel bounded at 640 threads per block (96 registers instead of
// 64: no spills at H2O sizes, 4 % more walker-steps/s measured there); taken
// when its plan still runs every block at once, else the 1024-thread instance.
constexpr int kWideThreads = 640;
template <typename R, int JC>
__global__ void __launch_bounds__(kWideThreads)
    metropolis_kernel_wide(const __grid_constant__ qmc_wf_desc d,
                           const __grid_constant__ qmc_metropolis_args a,
                           unsigned char* __restrict__ scr, int64_t ss,
                           const __grid_constant__ EPShape S) {
  extern __shared__ __align__(16) unsigned char smem[];
  metropolis_block<R, JC>(d, a, scr, ss, S, blockIdx.x, smem);
}

// Plan of the wide FP32 instance if it runs in one wave (*use set), else of
// the default instance.
template <typename R, int JC>
EPShape metropolis_plan(const qmc_wf_desc* d, int64_t nw, bool* wide) {
  *wide = false;
  if constexpr (kMixed<R>) {
    bool one = false;
    const EPShape Sw = ep_plan<R>(*d, 2, JC, metropolis_kernel_wide<R, JC>, nw, kWideThreads, &one);
    if (Sw.smem >= 0 && one && Sw.nthreads <= kWideThreads) {
      *wide = true;
      return Sw;
    }
  }
  return ep_plan<R>(*d, 2, JC, metropolis_kernel<R, JC>, nw);
}

// The launch plan launch_metropolis takes for nw walkers: walkers per block,
// threads per walker, threads per block, positions in scratch (0 / 1),
// dynamic shared memory bytes.
template <typename R, int JC>
int plan_metropolis(const qmc_wf_desc* d, int64_t nw, int32_t* out) {
  bool wide = false;
  const EPShape S = metropolis_plan<R, JC>(d, nw, &wide);
  out[0] = S.nwb;
  out[1] = S.nslot;
  out[2] = S.nthreads;
  out[3] = S.pos_global;
  out[4] = (int32_t)S.smem;
  return S.smem < 0 ? QMC_ERR_SHAPE : QMC_OK;
}

template <typename R, int JC>
int launch_metropolis(const qmc_wf_desc* d, const qmc_metropolis_args* a, unsigned char* scr,
                             cudaStream_t s) {
  bool wide = false;
  const EPShape S = metropolis_plan<R, JC>(d, a->nwalkers, &wide);
  if (S.smem < 0 || S.smem > 227 * 1024 || S.nthreads > EPBound<R>::kThreads) return QMC_ERR_SHAPE;
  const dim3 grid((unsigned)((a->nwalkers + S.nwb - 1) / S.nwb));
  if (wide) {
    int st = prepare_smem(metropolis_kernel_wide<R, JC>, S.smem);
    if (st) return st;
    metropolis_kernel_wide<R, JC><<<grid, S.nthreads, S.smem, s>>>(*d, *a, scr,
                                                                   pad_walkers(a->nwalkers), S);
    return launch_status();
  }
  int st = prepare_smem(metropolis_kernel<R, JC>, S.smem);
  if (st) return st;
  metropolis_kernel<R, JC><<<grid, S.nthreads, S.smem, s>>>(*d, *a, scr, pad_walkers(a->nwalkers), S);
  return launch_status();
}

}  // namespace qmc
