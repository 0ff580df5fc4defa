// Persistent Metropolis sampler (one thread per walker chain).
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

namespace qmc {

// ---------------------------------------------------------------------------
// Metropolis
// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of the 4x32 bijection with the published
// multipliers and Weyl key increments.
struct U4 {
  uint32_t x, y, z, w;
};
__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

struct Rng {
  uint32_t k0, k1, walker;
  uint64_t step;
  uint32_t call;
  __device__ __forceinline__ U4 next() {
    return philox(U4{call++, walker, (uint32_t)step, (uint32_t)(step >> 32)}, k0, k1);
  }
  // two standard normals from two 32-bit words (Box-Muller, FP32 transcendentals)
  __device__ __forceinline__ void normal2(uint32_t a, uint32_t b, double& z0, double& z1) {
    const float u1 = ((float)a + 1.0f) * 2.3283064365386963e-10f;  // (0, 1]
    const float u2 = (float)b * 2.3283064365386963e-10f;           // [0, 1)
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z0 = (double)(rad * c);
    z1 = (double)(rad * s);
  }
  // uniform in [0, 1) with 53 random bits
  __device__ __forceinline__ double uniform53(uint32_t hi, uint32_t lo) {
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6)) * 1.1102230246251565e-16;
  }
};

template <int JC>
__global__ void __launch_bounds__(kTPB) metropolis_kernel(const qmc_wf_desc d, const qmc_metropolis_args a,
                                                          double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables t = load_tables(d, d.nmo_used, smem);
  const Layout L = scratch_layout(d, 2);
  const int64_t nw = a.nwalkers;
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int ne = d.nelec, nc = 3 * ne;
  double* sw = scr + w;
  double* xp = sw + L.pos * ss;   // current positions
  double* xn = sw + L.pnew * ss;  // proposal
  for (int c = 0; c < nc; ++c) xp[c * ss] = a.pos[w * nc + c];
  const PosView Pc{xp, ss}, Pn{xn, ss};
  const double eps = 1e-16;
  double psi = walker_psi<JC>(d, t, L, Pc, sw, ss);
  double fx = psi * psi;
  if (fx == 0.0) fx = eps;
  const double sigma = a.step_size / (2.0 * sqrt(2.0 * log(2.0)));
  const double sd = sqrt(sigma);  // MultivariateNormal(0, sigma I): std = sqrt(sigma)
  Rng rng{(uint32_t)a.seed, (uint32_t)(a.seed >> 32), (uint32_t)w, 0, 0};
  const int nmove = a.move_type == QMC_MOVE_ALL_ELEC_ITER ? ne : 1;
  int nacc = 0;
  int64_t isnap = 0, idecor = 0;
  for (int istep = 0; istep < a.nstep; ++istep) {
    rng.step = a.step_offset + istep;
    rng.call = 0;
    for (int im = 0; im < nmove; ++im) {
      double u;
      if (a.move_type == QMC_MOVE_ALL_ELEC) {
        if (a.proposals) {
          const double* pr = a.proposals + ((int64_t)istep * nw + w) * nc;
          for (int c = 0; c < nc; ++c) xn[c * ss] = xp[c * ss] + pr[c];
          u = a.uniforms[(int64_t)istep * nw + w];
        } else {
          for (int c = 0; c < nc; c += 4) {
            const U4 r = rng.next();
            double z[4];
            if (a.proba == QMC_PROBA_NORMAL) {
              rng.normal2(r.x, r.y, z[0], z[1]);
              rng.normal2(r.z, r.w, z[2], z[3]);
#pragma unroll
              for (int q = 0; q < 4; ++q) z[q] *= sd;
            } else {
              const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
              for (int q = 0; q < 4; ++q) z[q] = a.step_size * (2.0 * (rr[q] * 2.3283064365386963e-10) - 1.0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
              if (c + q < nc) xn[(c + q) * ss] = xp[(c + q) * ss] + z[q];
          }
          const U4 r = rng.next();
          u = rng.uniform53(r.x, r.y);
        }
      } else {
        int iel;
        double dz[3];
        if (a.proposals) {
          const int64_t mi = ((int64_t)istep * nmove + im) * nw + w;
          iel = a.move_type == QMC_MOVE_ALL_ELEC_ITER ? im : a.electron_index[(int64_t)istep * nw + w];
          for (int q = 0; q < 3; ++q) dz[q] = a.proposals[mi * 3 + q];
          u = a.uniforms[mi];
        } else {
          const U4 r = rng.next();
          const U4 r2 = rng.next();
          if (a.proba == QMC_PROBA_NORMAL) {
            double z3;
            rng.normal2(r.x, r.y, dz[0], dz[1]);
            rng.normal2(r.z, r.w, dz[2], z3);
            for (int q = 0; q < 3; ++q) dz[q] *= sd;
          } else {
            const uint32_t rr[3] = {r.x, r.y, r.z};
            for (int q = 0; q < 3; ++q) dz[q] = a.step_size * (2.0 * (rr[q] * 2.3283064365386963e-10) - 1.0);
          }
          u = rng.uniform53(r2.x, r2.y);
          iel = a.move_type == QMC_MOVE_ALL_ELEC_ITER
                    ? im
                    : (int)(((uint64_t)r2.z * (uint64_t)ne) >> 32);
        }
        for (int c = 0; c < nc; ++c) xn[c * ss] = xp[c * ss];
        for (int q = 0; q < 3; ++q) xn[(3 * iel + q) * ss] += dz[q];
      }
      const double psin = walker_psi<JC>(d, t, L, Pn, sw, ss);
      double fxn = psin * psin;
      if (fxn == 0.0) fxn = eps;
      double df = fxn / fx;
      if (df > 1.0) df = 1.0;
      if (df - u >= 0.0) {
        for (int c = 0; c < nc; ++c) xp[c * ss] = xn[c * ss];
        fx = fxn;
        psi = psin;
        ++nacc;
      }
    }
    if (istep >= a.ntherm) {
      if (idecor % a.ndecor == 0) {
        if (a.samples && isnap < a.nsnap) {
          double* out = a.samples + (isnap * nw + w) * nc;
          for (int c = 0; c < nc; ++c) out[c] = xp[c * ss];
        }
        ++isnap;
      }
      ++idecor;
    }
  }
  for (int c = 0; c < nc; ++c) a.pos[w * nc + c] = xp[c * ss];
  if (a.accepted) a.accepted[w] += nacc;
  if (a.psi_out) a.psi_out[w] = psi;
}

}  // namespace qmc

using namespace qmc;

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
  const int64_t smem = tables_smem_bytes(*d, d->nmo_used);
  const int64_t ss = pad_walkers(a->nwalkers);
  const dim3 grid((unsigned)((a->nwalkers + kTPB - 1) / kTPB));
  cudaStream_t s = (cudaStream_t)stream;
  double* scr = (double*)scratch;
  if (d->nmo_used <= 8) {
    if ((st = prepare_smem(metropolis_kernel<8>, smem))) return st;
    metropolis_kernel<8><<<grid, kTPB, smem, s>>>(*d, *a, scr, ss);
  } else if (d->nmo_used <= 16) {
    if ((st = prepare_smem(metropolis_kernel<16>, smem))) return st;
    metropolis_kernel<16><<<grid, kTPB, smem, s>>>(*d, *a, scr, ss);
  } else {
    if ((st = prepare_smem(metropolis_kernel<24>, smem))) return st;
    metropolis_kernel<24><<<grid, kTPB, smem, s>>>(*d, *a, scr, ss);
  }
  return launch_status();
}

}  // extern "C"
