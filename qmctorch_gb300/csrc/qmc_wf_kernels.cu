// Fused psi and local-energy kernels (plain FP64 and mixed methods).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "qmc_ep.cuh"
#include "qmc_host.cuh"

namespace qmc {

// ---------------------------------------------------------------------------
// fused psi / local energy (electron-parallel blocks, qmc_ep.cuh)
// ---------------------------------------------------------------------------
template <typename R, int JC>
__global__ void __launch_bounds__(EPBound<R>::kThreads) ep_psi_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                      int64_t nw, double* __restrict__ psi,
                                                      unsigned char* __restrict__ scr, int64_t ss,
                                                      const EPShape S) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables<R> t = load_tables<R>(d, d.nmo_used, S.ncol, smem + S.o_tab);
  const int64_t w0 = (int64_t)blockIdx.x * S.nwb;
  XP<R>* P = reinterpret_cast<XP<R>*>(smem + S.o_pos);
  ep_stage_positions<R>(pos, w0, nw, S.nwb, 3 * d.nelec, S.pstride, P);
  ep_eval<R, JC, false>(d, t, EPPtrs{smem, S}, P, scr, ss, w0, nw);
  const int tid = threadIdx.x;
  if (tid < S.nwb && w0 + tid < nw)
    psi[w0 + tid] = reinterpret_cast<const double*>(smem + S.o_psi)[tid];
}

template <typename R, int JC, bool ELCOOP = false>
__global__ void __launch_bounds__(EPElBound<R>::kThreads) ep_eloc_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                       int64_t nw, double* __restrict__ eloc,
                                                       double* __restrict__ kin,
                                                       double* __restrict__ psi,
                                                       unsigned char* __restrict__ scr, int64_t ss,
                                                       const EPShape S) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables<R> t = load_tables<R>(d, d.nmo_used, S.ncol, smem + S.o_tab);
  const int64_t w0 = (int64_t)blockIdx.x * S.nwb;
  XP<R>* P = reinterpret_cast<XP<R>*>(smem + S.o_pos);
  ep_stage_positions<R>(pos, w0, nw, S.nwb, 3 * d.nelec, S.pstride, P);
  ep_eval<R, JC, true, ELCOOP>(d, t, EPPtrs{smem, S}, P, scr, ss, w0, nw);
  const int tid = threadIdx.x;
  if (tid < S.nwb && w0 + tid < nw) {
    const double k = reinterpret_cast<const double*>(smem + S.o_kin)[tid];
    const double v = reinterpret_cast<const double*>(smem + S.o_v)[tid];
    eloc[w0 + tid] = k + v + d.e_nuc;
    if (kin) kin[w0 + tid] = k;
    if (psi) psi[w0 + tid] = reinterpret_cast<const double*>(smem + S.o_psi)[tid];
  }
}

template <typename R, typename K>
static int launch_prepare(K kernel, const EPShape& S, int kind) {
  if (S.smem < 0 || S.smem > 227 * 1024 || S.nthreads > ep_thread_bound<R>(kind))
    return QMC_ERR_SHAPE;
  return prepare_smem(kernel, S.smem);
}

template <typename R, int JC>
static int launch_psi(const qmc_wf_desc* d, const double* pos, int64_t nw, double* psi,
                      unsigned char* scr, cudaStream_t s) {
  const EPShape S = ep_plan<R>(*d, 0, JC, ep_psi_kernel<R, JC>, nw);
  int st = launch_prepare<R>(ep_psi_kernel<R, JC>, S, 0);
  if (st) return st;
  const dim3 grid((unsigned)((nw + S.nwb - 1) / S.nwb));
  ep_psi_kernel<R, JC><<<grid, S.nthreads, S.smem, s>>>(*d, pos, nw, psi, scr, pad_walkers(nw), S);
  return launch_status();
}

template <typename R>
static int dispatch_psi(const qmc_wf_desc* d, const double* pos, int64_t nw, double* psi,
                        unsigned char* scr, cudaStream_t s) {
  if (d->nmo_used <= 8) return launch_psi<R, 8>(d, pos, nw, psi, scr, s);
  if (d->nmo_used <= 16) return launch_psi<R, 16>(d, pos, nw, psi, scr, s);
  return launch_psi<R, 24>(d, pos, nw, psi, scr, s);
}

template <typename R, int JC, bool ELCOOP>
static int launch_eloc_k(const qmc_wf_desc* d, const double* pos, int64_t nw, double* eloc,
                         double* kin, double* psi, unsigned char* scr, cudaStream_t s) {
  const EPShape S = ep_plan<R>(*d, 1, JC, ep_eloc_kernel<R, JC, ELCOOP>, nw);
  int st = launch_prepare<R>(ep_eloc_kernel<R, JC, ELCOOP>, S, 1);
  if (st) return st;
  const dim3 grid((unsigned)((nw + S.nwb - 1) / S.nwb));
  ep_eloc_kernel<R, JC, ELCOOP><<<grid, S.nthreads, S.smem, s>>>(*d, pos, nw, eloc, kin, psi,
                                                                 scr, pad_walkers(nw), S);
  return launch_status();
}

// Molecules with large excitation-mode channels (beyond the register path)
// run the instance with the cooperative determinant phase.
template <typename R, int JC>
static int launch_eloc(const qmc_wf_desc* d, const double* pos, int64_t nw, double* eloc,
                       double* kin, double* psi, unsigned char* scr, cudaStream_t s) {
  if (coop_el_applies<R>(*d, 4))
    return launch_eloc_k<R, JC, true>(d, pos, nw, eloc, kin, psi, scr, s);
  return launch_eloc_k<R, JC, false>(d, pos, nw, eloc, kin, psi, scr, s);
}

}  // namespace qmc

using namespace qmc;

extern "C" {

int qmc_wf_psi(const qmc_wf_desc* d, const double* pos, int64_t nw, double* psi, void* scratch,
               int64_t scratch_bytes, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || (nw > 0 && (!pos || !psi || !scratch))) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_scratch_bytes(d, nw, 0)) return QMC_ERR_SCRATCH;
  unsigned char* scr = (unsigned char*)scratch;
  cudaStream_t s = (cudaStream_t)stream;
  if (d->precision == QMC_PREC_MIXED) return dispatch_psi<float>(d, pos, nw, psi, scr, s);
  return dispatch_psi<double>(d, pos, nw, psi, scr, s);
}

int qmc_wf_local_energy(const qmc_wf_desc* d, const double* pos, int64_t nw, double* eloc,
                        double* kinetic, double* psi, void* scratch, int64_t scratch_bytes,
                        void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || (nw > 0 && (!pos || !eloc || !scratch))) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_scratch_bytes(d, nw, 1)) return QMC_ERR_SCRATCH;
  unsigned char* scr = (unsigned char*)scratch;
  cudaStream_t s = (cudaStream_t)stream;
  if (d->precision == QMC_PREC_MIXED)
    return launch_eloc<float, 8>(d, pos, nw, eloc, kinetic, psi, scr, s);
  return launch_eloc<double, 8>(d, pos, nw, eloc, kinetic, psi, scr, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Static-scratch variant of qmc_wf_psi for callers that cannot allocate device
// memory (see include/qmc_gb300.h). The workspace is this file-scope array;
// host code may not use its name as a device address, so its address is looked
// up once per device with cudaGetSymbolAddress and passed to the kernel.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_psi_static_scratch[QMC_STATIC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
void* g_static_address[kMaxDevices] = {};

// Device address of g_psi_static_scratch on the current device (looked up on
// the first call per device, with that device current).
int static_scratch_address(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return QMC_ERR_LAUNCH;
  }
  std::lock_guard<std::mutex> lock(g_static_mutex);
  if (g_static_address[dev] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_psi_static_scratch);
    if (e != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return QMC_ERR_LAUNCH;
    }
    g_static_address[dev] = p;
  }
  *out = g_static_address[dev];
  return QMC_OK;
}
}  // namespace

extern "C" int qmc_wf_psi_static(const qmc_wf_desc* d, const double* pos, int64_t nw,
                                 double* psi, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || (nw > 0 && (!pos || !psi))) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  const int64_t need = qmc_scratch_bytes(d, nw, 0);
  if (need < 0) return QMC_ERR_ARG;
  if (need > (int64_t)QMC_STATIC_SCRATCH_BYTES) return QMC_ERR_STATIC_LIMIT;
  void* scr = nullptr;
  if ((st = static_scratch_address(&scr))) return st;
  return qmc_wf_psi(d, pos, nw, psi, scr, need, stream);
}
