// Fused psi and local-energy kernels (FP64 plain method).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "qmc_host.cuh"

namespace qmc {

// ---------------------------------------------------------------------------
// fused psi / local energy
// ---------------------------------------------------------------------------
template <int JC>
__global__ void __launch_bounds__(kTPB) psi_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                   int64_t nw, double* __restrict__ psi,
                                                   double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables t = load_tables(d, d.nmo_used, smem);
  const Layout L = scratch_layout(d, 0);
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  PosView P{pos + w * 3 * d.nelec, 1};
  psi[w] = walker_psi<JC>(d, t, L, P, scr + w, ss);
}

template <int JC>
__global__ void __launch_bounds__(kTPB) eloc_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                    int64_t nw, double* __restrict__ eloc,
                                                    double* __restrict__ kin,
                                                    double* __restrict__ psi,
                                                    double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables t = load_tables(d, d.nmo_used, smem);
  const Layout L = scratch_layout(d, 1);
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  PosView P{pos + w * 3 * d.nelec, 1};
  double k = 0.0, p = 0.0;
  const double e = walker_eloc<JC>(d, t, L, P, scr + w, ss, &k, &p);
  eloc[w] = e;
  if (kin) kin[w] = k;
  if (psi) psi[w] = p;
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
  const int64_t smem = tables_smem_bytes(*d, d->nmo_used);
  const int64_t ss = pad_walkers(nw);
  const dim3 grid((unsigned)((nw + kTPB - 1) / kTPB));
  cudaStream_t s = (cudaStream_t)stream;
  double* scr = (double*)scratch;
  if (d->nmo_used <= 8) {
    if ((st = prepare_smem(psi_kernel<8>, smem))) return st;
    psi_kernel<8><<<grid, kTPB, smem, s>>>(*d, pos, nw, psi, scr, ss);
  } else if (d->nmo_used <= 16) {
    if ((st = prepare_smem(psi_kernel<16>, smem))) return st;
    psi_kernel<16><<<grid, kTPB, smem, s>>>(*d, pos, nw, psi, scr, ss);
  } else {
    if ((st = prepare_smem(psi_kernel<24>, smem))) return st;
    psi_kernel<24><<<grid, kTPB, smem, s>>>(*d, pos, nw, psi, scr, ss);
  }
  return launch_status();
}

int qmc_wf_local_energy(const qmc_wf_desc* d, const double* pos, int64_t nw, double* eloc,
                        double* kinetic, double* psi, void* scratch, int64_t scratch_bytes,
                        void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || (nw > 0 && (!pos || !eloc || !scratch))) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_scratch_bytes(d, nw, 1)) return QMC_ERR_SCRATCH;
  const int64_t smem = tables_smem_bytes(*d, d->nmo_used);
  if ((st = prepare_smem(eloc_kernel<8>, smem))) return st;
  const int64_t ss = pad_walkers(nw);
  const dim3 grid((unsigned)((nw + kTPB - 1) / kTPB));
  eloc_kernel<8><<<grid, kTPB, smem, (cudaStream_t)stream>>>(*d, pos, nw, eloc, kinetic, psi,
                                                              (double*)scratch, ss);
  return launch_status();
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
