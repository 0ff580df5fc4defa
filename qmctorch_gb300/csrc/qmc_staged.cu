// Staged kernels behind the module-level API (AO, MO, Jastrow, Slater pooling).
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

namespace qmc {

// ---------------------------------------------------------------------------
// staged kernels of the module-level API
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) ao_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                 int64_t nw, int mode, double* __restrict__ ao,
                                                 double* __restrict__ dao, double* __restrict__ d2ao) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables<double> t = load_tables<double>(d, 0, 0, smem);
  const int64_t item = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // (walker, electron)
  if (item >= nw * d.nelec) return;
  const double* pe = pos + item * 3;  // pos[w][3*ne] row-major == [(w*ne+e)*3]
  const double ex = pe[0], ey = pe[1], ez = pe[2];
  const int64_t row = item * d.nao;
  if (mode == 0) {
    for_each_ao<double, false>(t, ex, ey, ez, [&](int a, const AOVal<double>& o) { ao[row + a] = o.v; });
  } else {
    for_each_ao<double, true>(t, ex, ey, ez, [&](int a, const AOVal<double>& o) {
      if (mode == 1 || mode == 4) {
        dao[(row + a) * 3] = o.gx;
        dao[(row + a) * 3 + 1] = o.gy;
        dao[(row + a) * 3 + 2] = o.gz;
      }
      if (mode == 2 || mode == 4) d2ao[row + a] = o.lap;
      if (mode == 4) ao[row + a] = o.v;
      if (mode == 3) {
        // sum of the gradient: value-path coefficient convention
        // (_sum_gradient_kernel, atomic_orbitals.py:290-307)
        const double vs = t.vscale ? t.vscale[a] : 1.0;
        ao[row + a] = vs * (o.gx + o.gy + o.gz);
      }
    });
  }
}

__global__ void __launch_bounds__(128) mo_kernel(const qmc_wf_desc d, const double* __restrict__ ao,
                                                 int64_t nrows, double* __restrict__ mo) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables<double> t = load_tables<double>(d, d.nmo, round_up(d.nmo, 8), smem);
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const double* ar = ao + r * d.nao;
  constexpr int JC = 8;
  for (int j0 = 0; j0 < d.nmo; j0 += JC) {
    double acc[JC];
#pragma unroll
    for (int jj = 0; jj < JC; ++jj) acc[jj] = 0.0;
    for (int a = 0; a < d.nao; ++a) {
      const double v = ar[a];
      const double* Wa = t.W + (int64_t)a * t.ncol + j0;
#pragma unroll
      for (int jj = 0; jj < JC; ++jj)
        if (j0 + jj < d.nmo) acc[jj] = fma(v, Wa[jj], acc[jj]);
    }
#pragma unroll
    for (int jj = 0; jj < JC; ++jj)
      if (j0 + jj < d.nmo) mo[r * d.nmo + j0 + jj] = acc[jj];
  }
}

// Jastrow factor and derivatives per walker, each pair visited from both
// electrons so that no per-electron accumulator is needed.
__global__ void __launch_bounds__(128) jastrow_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                      int64_t nw, double* __restrict__ jast,
                                                      double* __restrict__ djast,
                                                      double* __restrict__ d2jast, int sum_grad) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int ne = d.nelec;
  PosView P{pos + w * 3 * ne, 1};
  const double wj = __ldg(d.jastrow_w);
  const double J = exp(jastrow_log<double>(d, P, wj));
  if (jast) jast[w] = J;
  if (!djast && !d2jast) return;
  for (int i = 0; i < ne; ++i) {
    double gx = 0, gy = 0, gz = 0, lp = 0;
    const double xi = P(3 * i), yi = P(3 * i + 1), zi = P(3 * i + 2);
    for (int j = 0; j < ne; ++j) {
      if (j == i) continue;
      const double dx = xi - P(3 * j), dy = yi - P(3 * j + 1), dz = zi - P(3 * j + 2);
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const double ir = 1.0 / r;
      const double iu = 1.0 / (1.0 + wj * r);
      const double k1 = (same_spin(d, i, j) ? 0.25 : 0.5) * iu * iu;
      gx += k1 * dx * ir;
      gy += k1 * dy * ir;
      gz += k1 * dz * ir;
      lp += 2.0 * k1 * ir - 2.0 * wj * k1 * iu;
    }
    if (djast) {
      if (sum_grad) {
        djast[w * ne + i] = J * (gx + gy + gz);
      } else {
        djast[(w * 3 + 0) * ne + i] = J * gx;
        djast[(w * 3 + 1) * ne + i] = J * gy;
        djast[(w * 3 + 2) * ne + i] = J * gz;
      }
    }
    if (d2jast) d2jast[w * ne + i] = J * (lp + gx * gx + gy * gy + gz * gz);
  }
}

// Electron-nucleus Pade factor alone and its derivatives per walker
// (JastrowFactorElectronNuclei.forward, jastrow_factor_electron_nuclei.py:66-161):
// J = exp(sum_{i,A} K(r_iA)), grad_i J = J grad_i U, lap_i J = J (lap_i U + |grad_i U|^2).
__global__ void __launch_bounds__(128) jastrow_en_kernel(const qmc_wf_desc d,
                                                         const double* __restrict__ pos, int64_t nw,
                                                         double* __restrict__ jast,
                                                         double* __restrict__ djast,
                                                         double* __restrict__ d2jast, int sum_grad) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int ne = d.nelec;
  PosView P{pos + w * 3 * ne, 1};
  double u = 0.0;
  for (int i = 0; i < ne; ++i) u += en_terms(d, P(3 * i), P(3 * i + 1), P(3 * i + 2)).u;
  const double J = exp(u);
  if (jast) jast[w] = J;
  if (!djast && !d2jast) return;
  for (int i = 0; i < ne; ++i) {
    const EnTerms en = en_terms(d, P(3 * i), P(3 * i + 1), P(3 * i + 2));
    const double gx = en.g[0], gy = en.g[1], gz = en.g[2];
    if (djast) {
      if (sum_grad) {
        djast[w * ne + i] = J * (gx + gy + gz);
      } else {
        djast[(w * 3 + 0) * ne + i] = J * gx;
        djast[(w * 3 + 1) * ne + i] = J * gy;
        djast[(w * 3 + 2) * ne + i] = J * gz;
      }
    }
    if (d2jast) d2jast[w * ne + i] = J * (en.lap + gx * gx + gy * gy + gz * gz);
  }
}

template <bool OP>
__global__ void __launch_bounds__(kTPB) slater_kernel(const qmc_wf_desc d, const double* __restrict__ mo,
                                                      const double* __restrict__ bop, int ld,
                                                      int64_t nw, double* __restrict__ dets,
                                                      double* __restrict__ op,
                                                      unsigned char* __restrict__ scr, int64_t ss) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const Layout L = scratch_layout(d, 1);  // d.precision is QMC_PREC_FP64 here
  const int ne = d.nelec;
  const CView<double> m{mo + w * ne * ld, ld, 1};
  const CView<double> b = OP ? CView<double>{bop + w * ne * ld, ld, 1} : m;
  const int64_t vm = L.vmax > 0 ? L.vmax : 1;
  SpinWork<double> wk;
  wk.LU = MView<double>{rptr<double>(scr, L.lu, ss, w), (int64_t)L.nmax * ss, ss};
  wk.X = MView<double>{rptr<double>(scr, L.x, ss, w), vm * ss, ss};
  wk.Y = MView<double>{rptr<double>(scr, L.y, ss, w), (int64_t)L.omax * ss, ss};
  wk.rc = wk.LU;  // unused: FP64 needs no refinement
  wk.X64 = wk.X;
  wk.Y64 = wk.Y;
  double* dv = rptr<double>(scr, L.dv, ss, w);
  double* ov = rptr<double>(scr, L.ov, ss, w);
  double dref[2];
  spin_channel<double, OP>(d, 0, m, b, wk, SpinOut<double>{dv, ov, ss, &dref[0]});
  spin_channel<double, OP>(d, 1, CView<double>{m.p + d.nup * m.rs, m.rs, m.cs},
                           CView<double>{b.p + d.nup * b.rs, b.rs, b.cs}, wk,
                           SpinOut<double>{dv + d.ndet[0] * ss, ov + d.ndet[0] * ss, ss, &dref[1]});
  for (int k = 0; k < d.ncfg; ++k) {
    const int iu = __ldg(d.cfg_det[0] + k), idn = __ldg(d.cfg_det[1] + k) + d.ndet[0];
    dets[w * d.ncfg + k] = (dref[0] * dv[iu * ss]) * (dref[1] * dv[idn * ss]);
    if (OP) op[w * d.ncfg + k] = ov[iu * ss] + ov[idn * ss];
  }
}

__global__ void __launch_bounds__(128) potentials_kernel(const qmc_wf_desc d, const double* __restrict__ pos,
                                                         int64_t nw, double* __restrict__ v_en,
                                                         double* __restrict__ v_ee) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const int ne = d.nelec;
  PosView P{pos + w * 3 * ne, 1};
  if (v_en) {
    double v = 0.0;
    for (int e = 0; e < ne; ++e)
      for (int A = 0; A < d.natom; ++A) {
        const double dx = P(3 * e) - __ldg(d.atom_coords + 3 * A),
                     dy = P(3 * e + 1) - __ldg(d.atom_coords + 3 * A + 1),
                     dz = P(3 * e + 2) - __ldg(d.atom_coords + 3 * A + 2);
        v -= __ldg(d.atom_charge + A) / sqrt(dx * dx + dy * dy + dz * dz);
      }
    v_en[w] = v;
  }
  if (v_ee) {
    double v = 0.0;
    for (int i = 0; i < ne - 1; ++i)
      for (int j = i + 1; j < ne; ++j) {
        const double dx = P(3 * i) - P(3 * j), dy = P(3 * i + 1) - P(3 * j + 1),
                     dz = P(3 * i + 2) - P(3 * j + 2);
        v += 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
      }
    v_ee[w] = v;
  }
}

}  // namespace qmc

using namespace qmc;

extern "C" {

int qmc_ao_eval(const qmc_wf_desc* d, const double* pos, int64_t nw, int32_t mode, double* ao,
                double* dao, double* d2ao, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || mode < 0 || mode > 4 || (nw > 0 && !pos)) return QMC_ERR_ARG;
  if ((mode == 0 || mode == 3 || mode == 4) && !ao) return QMC_ERR_ARG;
  if ((mode == 1 || mode == 4) && !dao) return QMC_ERR_ARG;
  if ((mode == 2 || mode == 4) && !d2ao) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  const int64_t smem = tables_smem_bytes<double>(*d, 0);
  if ((st = prepare_smem(ao_kernel, smem))) return st;
  const int64_t items = nw * d->nelec;
  ao_kernel<<<(unsigned)((items + 127) / 128), 128, smem, (cudaStream_t)stream>>>(*d, pos, nw, mode,
                                                                                  ao, dao, d2ao);
  return launch_status();
}

int qmc_mo_eval(const qmc_wf_desc* d, const double* ao, int64_t nrows, double* mo, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nrows < 0 || (nrows > 0 && (!ao || !mo))) return QMC_ERR_ARG;
  if (nrows == 0) return QMC_OK;
  const int64_t smem = tables_smem_bytes<double>(*d, round_up(d->nmo, 8));
  if ((st = prepare_smem(mo_kernel, smem))) return st;
  mo_kernel<<<(unsigned)((nrows + 127) / 128), 128, smem, (cudaStream_t)stream>>>(*d, ao, nrows, mo);
  return launch_status();
}

int qmc_jastrow_ee(const qmc_wf_desc* d, const double* pos, int64_t nw, double* jast, double* djast,
                   double* d2jast, int32_t sum_grad, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (!d->jastrow_w || nw < 0 || (nw > 0 && !pos)) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  jastrow_kernel<<<(unsigned)((nw + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*d, pos, nw, jast,
                                                                                 djast, d2jast,
                                                                                 sum_grad);
  return launch_status();
}

int qmc_jastrow_en(const qmc_wf_desc* d, const double* pos, int64_t nw, double* jast,
                   double* djast, double* d2jast, int32_t sum_grad, void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (!d->use_jastrow_en || nw < 0 || (nw > 0 && !pos)) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  jastrow_en_kernel<<<(unsigned)((nw + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      *d, pos, nw, jast, djast, d2jast, sum_grad);
  return launch_status();
}

int qmc_slater(const qmc_wf_desc* d0, const double* mo, const double* bop, int32_t ld, int64_t nw,
               double* dets, double* op, void* scratch, int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;  // the staged pooling kernel is FP64
  const qmc_wf_desc* d = &dd;
  if (nw < 0 || ld < d->nmo_used || (nw > 0 && (!mo || !dets || !scratch))) return QMC_ERR_ARG;
  if (bop && !op) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_scratch_bytes(d, nw, 1)) return QMC_ERR_SCRATCH;
  const int64_t ss = pad_walkers(nw);
  const dim3 grid((unsigned)((nw + kTPB - 1) / kTPB));
  unsigned char* scr = (unsigned char*)scratch;
  if (bop)
    slater_kernel<true><<<grid, kTPB, 0, (cudaStream_t)stream>>>(dd, mo, bop, ld, nw, dets, op, scr,
                                                                 ss);
  else
    slater_kernel<false><<<grid, kTPB, 0, (cudaStream_t)stream>>>(dd, mo, nullptr, ld, nw, dets,
                                                                  nullptr, scr, ss);
  return launch_status();
}

int qmc_potentials(const qmc_wf_desc* d, const double* pos, int64_t nw, double* v_en, double* v_ee,
                   void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nw < 0 || (nw > 0 && !pos)) return QMC_ERR_ARG;
  if (nw == 0 || (!v_en && !v_ee)) return QMC_OK;
  potentials_kernel<<<(unsigned)((nw + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*d, pos, nw, v_en,
                                                                                    v_ee);
  return launch_status();
}

}  // extern "C"
