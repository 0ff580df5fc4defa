// Hand-written adjoint of psi with respect to the trainable parameters
// (ao.bas_exp, mo.mo_modifier through W = mo_scf * mo_modifier,
// jastrow.jastrow_kernel.weight, fc.weight), FP64, one thread per walker.
// The AO values are recomputed from the positions, not stored by the forward
// pass. Walker contributions, weighted by gout[w], are summed in shared
// memory and added to the outputs with one global atomic per block.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

namespace qmc {

constexpr int kAdjTPB = 64;

// Column set (orbital per position) of unique spin determinant u: explicit
// mode reads it; excitation mode rebuilds it from the flat indices into
// A^-1 A_virt, so it is the determinant the forward pass evaluates
// (single: position i0 / nv takes orbital n + i0 % nv; double: positions
// i0 / nv and i2 / nv take orbitals n + i0 % nv and n + i1 % nv).
__device__ inline void det_columns(const qmc_wf_desc& d, int spin, int u, int* cols) {
  const int n = spin ? d.ndown : d.nup;
  const int* tab = d.det_table[spin];
  if (d.det_mode == QMC_DET_EXPLICIT) {
    for (int j = 0; j < n; ++j) cols[j] = __ldg(tab + (int64_t)u * n + j);
    return;
  }
  for (int j = 0; j < n; ++j) cols[j] = j;
  const int nv = d.max_orb[spin] - n;
  const int ord = __ldg(tab + 5 * u);
  if (ord >= 1) {
    const int i0 = __ldg(tab + 5 * u + 1);
    cols[i0 / nv] = n + i0 % nv;
  }
  if (ord == 2) {
    const int i0 = __ldg(tab + 5 * u + 1), i1 = __ldg(tab + 5 * u + 2), i2 = __ldg(tab + 5 * u + 3);
    cols[i0 / nv] = n + i0 % nv;
    cols[i2 / nv] = n + i1 % nv;
  }
}

struct AdjLayout {  // per-walker scratch, in doubles (item-major)
  int64_t ao, mo, g, lu, inv, dv, total;
};

__host__ __device__ inline AdjLayout adj_layout(const qmc_wf_desc& d) {
  AdjLayout L;
  const int64_t nmax = d.nup > d.ndown ? d.nup : d.ndown;
  int64_t o = 0;
  L.ao = o;
  o += (int64_t)d.nelec * d.nao;
  L.mo = o;
  o += (int64_t)d.nelec * d.nmo_used;
  L.g = o;
  o += (int64_t)d.nelec * d.nmo_used;
  L.lu = o;
  o += nmax * nmax;
  L.inv = o;
  o += nmax * nmax;
  L.dv = o;
  o += d.ndet[0] + d.ndet[1];
  L.total = o;
  return L;
}

__host__ __device__ inline int64_t adj_acc_doubles(const qmc_wf_desc& d, int nent) {
  return (int64_t)d.nao * d.nmo_used + nent + d.ncfg + 1;
}

__global__ void __launch_bounds__(kAdjTPB) psi_adjoint_kernel(
    const qmc_wf_desc d, const double* __restrict__ pos, int64_t nw, const double* __restrict__ gout,
    const int* __restrict__ w_entry, int nent, double* __restrict__ g_exp,
    double* __restrict__ g_W, int ldw, double* __restrict__ g_jw, double* __restrict__ g_ci,
    double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  double* acc = reinterpret_cast<double*>(smem + ((tables_smem_bytes<double>(d, ncol) + 15) & ~15));
  const int nmu = d.nmo_used, ne = d.nelec, nao = d.nao;
  double* accW = acc;                    // [nao][nmu]
  double* accE = accW + nao * nmu;       // [nent]
  double* accC = accE + nent;            // [ncfg]
  double* accJ = accC + d.ncfg;          // [1]
  const int64_t nacc = adj_acc_doubles(d, nent);
  for (int64_t i = threadIdx.x; i < nacc; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) {
    const double gw = gout[w];
    const AdjLayout L = adj_layout(d);
    double* sw = scr + w;
    auto AO = [&](int e, int a) -> double& { return sw[(L.ao + (int64_t)e * nao + a) * ss]; };
    auto MO = [&](int e, int j) -> double& { return sw[(L.mo + (int64_t)e * nmu + j) * ss]; };
    auto G = [&](int e, int j) -> double& { return sw[(L.g + (int64_t)e * nmu + j) * ss]; };
    const PosView P{pos + w * 3 * ne, 1};
    // Jastrow: log J and d log J / d w (pade_jastrow_kernel.py:68-82)
    double logj = 0.0, dlogj = 0.0;
    if (d.use_jastrow) {
      const double wj = __ldg(d.jastrow_w);
      for (int i = 0; i < ne - 1; ++i)
        for (int j = i + 1; j < ne; ++j) {
          const double dx = P(3 * i) - P(3 * j), dy = P(3 * i + 1) - P(3 * j + 1),
                       dz = P(3 * i + 2) - P(3 * j + 2);
          const double r = sqrt(dx * dx + dy * dy + dz * dz);
          const double w0 = same_spin(d, i, j) ? 0.25 : 0.5;
          const double iu = 1.0 / (1.0 + wj * r);
          logj += w0 * r * iu;
          dlogj -= w0 * r * r * iu * iu;
        }
    }
    const double J = d.use_jastrow ? exp(logj) : 1.0;
    // AO and MO values
    for (int e = 0; e < ne; ++e) {
      for_each_ao<double, false>(t, P(3 * e), P(3 * e + 1), P(3 * e + 2),
                                 [&](int a, const AOVal<double>& o) { AO(e, a) = o.v; });
      for (int j = 0; j < nmu; ++j) {
        double s = 0.0;
        for (int a = 0; a < nao; ++a) s = fma(AO(e, a), t.W[(int64_t)a * t.ncol + j], s);
        MO(e, j) = s;
        G(e, j) = 0.0;
      }
    }
    // unique spin determinants
    const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
    MView<double> LU{sw + L.lu * ss, (int64_t)nmax * ss, ss};
    MView<double> INV{sw + L.inv * ss, (int64_t)nmax * ss, ss};
    double* DV = sw + L.dv * ss;
    int piv[QMC_MAX_NSPIN], cols[QMC_MAX_NSPIN];
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
      for (int u = 0; u < d.ndet[s]; ++u) {
        double det = 1.0;
        if (n > 0) {
          det_columns(d, s, u, cols);
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) LU(i, j) = MO(r0 + i, cols[j]);
          det = lu_factor<double>(LU, n, piv);
        }
        DV[((s ? d.ndet[0] : 0) + u) * ss] = det;
      }
    }
    auto dval = [&](int s, int u) { return DV[((s ? d.ndet[0] : 0) + u) * ss]; };
    double psid = 0.0;
    for (int k = 0; k < d.ncfg; ++k) {
      const double dd = dval(0, __ldg(d.cfg_det[0] + k)) * dval(1, __ldg(d.cfg_det[1] + k));
      psid = fma(__ldg(d.ci_weight + k), dd, psid);
      atomicAdd(&accC[k], gw * J * dd);  // d psi / d c_k
    }
    if (d.use_jastrow) atomicAdd(accJ, gw * J * psid * dlogj);  // d psi / d w
    // d psi / d MO = J sum_u coef_u det_u A_u^-T (scattered into the columns of u)
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
      if (n == 0) continue;
      for (int u = 0; u < d.ndet[s]; ++u) {
        double coef = 0.0;
        for (int k = 0; k < d.ncfg; ++k)
          if (__ldg(d.cfg_det[s] + k) == u)
            coef = fma(__ldg(d.ci_weight + k), dval(1 - s, __ldg(d.cfg_det[1 - s] + k)), coef);
        if (coef == 0.0) continue;
        det_columns(d, s, u, cols);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) LU(i, j) = MO(r0 + i, cols[j]);
        const double det = lu_factor<double>(LU, n, piv);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) INV(i, j) = i == j ? 1.0 : 0.0;
        lu_solve<double>(LU, n, piv, INV.c(), INV, n);  // INV = A_u^-1
        const double scale = J * coef * det;
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) G(r0 + i, cols[j]) = fma(scale, INV(j, i), G(r0 + i, cols[j]));
      }
    }
    // d psi / d W[a][j] = sum_e AO[e][a] G[e][j]
    for (int a = 0; a < nao; ++a)
      for (int j = 0; j < nmu; ++j) {
        double s = 0.0;
        for (int e = 0; e < ne; ++e) s = fma(AO(e, a), G(e, j), s);
        if (s != 0.0) atomicAdd(&accW[a * nmu + j], gw * s);
      }
    // d psi / d alpha_p = sum_e H[e][a] dAO[e][a]/d alpha_p, H = G W^T,
    // dAO/d alpha_p = -vs w_p P r^2 exp(-alpha_p r^2) (the norm is a constant)
    for (int e = 0; e < ne; ++e) {
      const double ex = P(3 * e), ey = P(3 * e + 1), ez = P(3 * e + 2);
      for (int g = 0; g < t.ngroup; ++g) {
        const int A = t.group_atom[g];
        const double dx = ex - t.atom_xyz[3 * A], dy = ey - t.atom_xyz[3 * A + 1],
                     dz = ez - t.atom_xyz[3 * A + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const int np = t.group_prim[g + 1] - t.group_prim[g];
        for (int a = t.group_ao[g]; a < t.group_ao[g + 1]; ++a) {
          double h = 0.0;
          for (int j = 0; j < nmu; ++j) h = fma(G(e, j), t.W[(int64_t)a * t.ncol + j], h);
          if (h == 0.0) continue;
          const Poly<double> pl = cart_poly<double, false>(dx, dy, dz, t.ao_k[3 * a],
                                                            t.ao_k[3 * a + 1], t.ao_k[3 * a + 2]);
          const double vs = t.vscale ? t.vscale[a] : 1.0;
          for (int p = 0; p < np; ++p) {
            const int wi = t.ao_wofs[a] + p;
            const double dao = -vs * t.wd[wi] * pl.p * r2 * exp(-t.walpha[wi] * r2);
            atomicAdd(&accE[__ldg(w_entry + wi)], gw * h * dao);
          }
        }
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nao * nmu; i += blockDim.x) {
    const int a = i / nmu, j = i - a * nmu;
    if (accW[i] != 0.0) atomicAdd(&g_W[(int64_t)a * ldw + j], accW[i]);
  }
  for (int i = threadIdx.x; i < nent; i += blockDim.x)
    if (accE[i] != 0.0) atomicAdd(&g_exp[i], accE[i]);
  for (int i = threadIdx.x; i < d.ncfg; i += blockDim.x) atomicAdd(&g_ci[i], accC[i]);
  if (threadIdx.x == 0 && g_jw) atomicAdd(g_jw, accJ[0]);
}

}  // namespace qmc

using namespace qmc;

extern "C" {

int64_t qmc_adjoint_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  if (check_desc(d) != QMC_OK || nw < 0) return -1;
  return adj_layout(*d).total * pad_walkers(nw) * (int64_t)sizeof(double);
}

int qmc_wf_psi_adjoint(const qmc_wf_desc* d0, const double* pos, int64_t nw, const double* gout,
                       const int32_t* weight_entry, int32_t nentries, double* grad_exp,
                       double* grad_W, int32_t ldw, double* grad_jastrow_w, double* grad_ci,
                       void* scratch, int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;  // the adjoint is FP64
  const qmc_wf_desc* d = &dd;
  if (nw < 0 || nentries < 0 || ldw < d->nmo_used) return QMC_ERR_ARG;
  if (nw > 0 && (!pos || !gout || !weight_entry || !grad_exp || !grad_W || !grad_ci || !scratch))
    return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_adjoint_scratch_bytes(d, nw)) return QMC_ERR_SCRATCH;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = ((tables_smem_bytes<double>(*d, ncol) + 15) & ~int64_t(15)) +
                       adj_acc_doubles(*d, nentries) * 8;
  if ((st = prepare_smem(psi_adjoint_kernel, smem))) return st;
  const dim3 grid((unsigned)((nw + kAdjTPB - 1) / kAdjTPB));
  psi_adjoint_kernel<<<grid, kAdjTPB, smem, (cudaStream_t)stream>>>(
      dd, pos, nw, gout, weight_entry, nentries, grad_exp, grad_W, ldw,
      d->use_jastrow ? grad_jastrow_w : nullptr, grad_ci, (double*)scratch, pad_walkers(nw));
  return launch_status();
}

}  // extern "C"
