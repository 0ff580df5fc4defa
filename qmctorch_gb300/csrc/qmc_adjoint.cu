// Hand-written adjoint of psi with respect to the trainable parameters
// (ao.bas_exp, mo.mo_modifier through W = mo_scf * mo_modifier,
// jastrow.jastrow_kernel.weight, fc.weight), FP64, one thread per walker.
// The AO values are recomputed from the positions, not stored by the forward
// pass. Each walker writes its contributions, weighted by gout[w], to its own
// slots of the scratch; adj_reduce_kernel then sums every parameter over the
// walkers in a fixed order, so the gradients are bitwise reproducible and
// independent of the launch configuration (no atomics).
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

namespace qmc {

constexpr int kAdjTPB = 64;

struct AdjLayout {  // per-walker scratch, in doubles (item-major)
  int64_t ao, mo, g, lu, inv, dv, gacc, total;
};

// Per-walker gradient slots: W [nao][nmu], exponents [nweight] (one per basis
// entry), CI weights [ncfg], Pade weight [1].
// gradient slots per walker: W, exponents, CI weights, the e-e and the e-n
// Pade weights
__host__ __device__ inline int64_t adj_acc_doubles(const qmc_wf_desc& d) {
  return (int64_t)d.nao * d.nmo_used + d.nweight + d.ncfg + 2;
}

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
  L.gacc = o;
  o += adj_acc_doubles(d);
  L.total = o;
  return L;
}

__global__ void __launch_bounds__(kAdjTPB) psi_adjoint_kernel(
    const qmc_wf_desc d, const double* __restrict__ pos, int64_t nw, const double* __restrict__ gout,
    const int* __restrict__ w_entry, double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  const int nmu = d.nmo_used, ne = d.nelec, nao = d.nao;
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) {
    const double gw = gout[w];
    const AdjLayout L = adj_layout(d);
    double* sw = scr + w;
    // this walker's gradient slots
    double* const accW = sw + L.gacc * ss;  // [nao * nmu] (stride ss)
    double* const accE = accW + (int64_t)nao * nmu * ss;
    double* const accC = accE + (int64_t)d.nweight * ss;
    double* const accJ = accC + (int64_t)d.ncfg * ss;
    for (int64_t i = 0; i < adj_acc_doubles(d); ++i) accW[i * ss] = 0.0;
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
    double dlogj_en = 0.0;  // d log J / d w_en (elec_nuclei pade_jastrow_kernel.py:48-61)
    if (d.use_jastrow_en)
      for (int i = 0; i < ne; ++i) {
        const EnTerms en = en_terms(d, P(3 * i), P(3 * i + 1), P(3 * i + 2));
        logj += en.u;
        dlogj_en += en.du;
      }
    const double J = (d.use_jastrow || d.use_jastrow_en) ? exp(logj) : 1.0;
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
      accC[k * ss] += gw * J * dd;  // d psi / d c_k
    }
    if (d.use_jastrow) accJ[0] += gw * J * psid * dlogj;  // d psi / d w
    if (d.use_jastrow_en) accJ[ss] += gw * J * psid * dlogj_en;  // d psi / d w_en
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
        accW[((int64_t)a * nmu + j) * ss] = gw * s;
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
            double dao;
            if (t.radial != QMC_RADIAL_GTO)  // Slater type: d/d alpha r^n e^(-alpha r)
              dao = vs * t.wd[wi] *
                    sto_dalpha(pl.p, 0.0, 0.0, 0.0, 0.0, 0, dx, dy, dz, r2, t.ao_kr(a),
                               t.walpha[wi]).v;
            else
              dao = -vs * t.wd[wi] * pl.p * r2 * exp(-t.walpha[wi] * r2);
            accE[(int64_t)__ldg(w_entry + wi) * ss] += gw * h * dao;
          }
        }
      }
    }
  }
}


// ---------------------------------------------------------------------------
// Adjoint of the local energy
// ---------------------------------------------------------------------------
// E_L = KE + V, KE = sum_k c_k D_k T_k / sum_k c_k D_k with D_k = D_up D_down
// of configuration k, T_k = Tr(A_up^-1 B_up) + Tr(A_down^-1 B_down) and
// B = -1/2 (lap MO + 2 grad(U) . grad MO + (lap U + |grad U|^2) MO),
// U = log J (slater_jastrow.py:312-344, 449-482). V does not depend on the
// parameters. Per unique spin determinant with explicit columns (X = A_u^-1):
//   dKE/dA_u = dD_u D_u X^T - dT_u (X B_u X)^T,   dKE/dB_u = dT_u X^T,
// then through B to the MO values, gradients and laplacians, to W and (with
// the primitive-level exponent derivatives of value, gradient and laplacian,
// norms fixed) to the exponents, and through grad U, lap U to the Pade weight.
struct ElAdjLayout {  // per-walker scratch, in doubles (item-major)
  int64_t aov, aox, aoy, aoz, aol, ma, mx, my, mz, ml, b, ga, gb, lu, x, y, z, dv, tv, gj, lj,
      dgw, dlw, gacc, total;
};

__host__ __device__ inline ElAdjLayout el_adj_layout(const qmc_wf_desc& d) {
  ElAdjLayout L;
  const int64_t ne = d.nelec, nao = d.nao, nmu = d.nmo_used;
  const int64_t nmax = d.nup > d.ndown ? d.nup : d.ndown, nd = d.ndet[0] + d.ndet[1];
  int64_t o = 0;
  auto take = [&](int64_t n) {
    const int64_t r = o;
    o += n;
    return r;
  };
  L.aov = take(ne * nao);
  L.aox = take(ne * nao);
  L.aoy = take(ne * nao);
  L.aoz = take(ne * nao);
  L.aol = take(ne * nao);
  L.ma = take(ne * nmu);
  L.mx = take(ne * nmu);
  L.my = take(ne * nmu);
  L.mz = take(ne * nmu);
  L.ml = take(ne * nmu);
  L.b = take(ne * nmu);
  L.ga = take(ne * nmu);
  L.gb = take(ne * nmu);
  L.lu = take(nmax * nmax);
  L.x = take(nmax * nmax);
  L.y = take(nmax * nmax);
  L.z = take(nmax * nmax);
  L.dv = take(nd);
  L.tv = take(nd);
  L.gj = take(3 * ne);
  L.lj = take(ne);
  L.dgw = take(3 * ne);
  L.dlw = take(ne);
  L.gacc = take(adj_acc_doubles(d));
  L.total = o;
  return L;
}

__global__ void __launch_bounds__(kAdjTPB) eloc_adjoint_kernel(
    const qmc_wf_desc d, const double* __restrict__ pos, int64_t nw, const double* __restrict__ gout,
    const int* __restrict__ w_entry, double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  const int nmu = d.nmo_used, ne = d.nelec, nao = d.nao;
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w < nw) {
    const double gw = gout[w];
    const ElAdjLayout L = el_adj_layout(d);
    double* sw = scr + w;
    // this walker's gradient slots
    double* const accW = sw + L.gacc * ss;  // [nao * nmu] (stride ss)
    double* const accE = accW + (int64_t)nao * nmu * ss;
    double* const accC = accE + (int64_t)d.nweight * ss;
    double* const accJ = accC + (int64_t)d.ncfg * ss;
    for (int64_t i = 0; i < adj_acc_doubles(d); ++i) accW[i * ss] = 0.0;
    auto R2 = [&](int64_t base, int e, int k, int n) -> double& {
      return sw[(base + (int64_t)e * n + k) * ss];
    };
    auto AV = [&](int e, int a) -> double& { return R2(L.aov, e, a, nao); };
    auto AX = [&](int e, int a) -> double& { return R2(L.aox, e, a, nao); };
    auto AY = [&](int e, int a) -> double& { return R2(L.aoy, e, a, nao); };
    auto AZ = [&](int e, int a) -> double& { return R2(L.aoz, e, a, nao); };
    auto AL = [&](int e, int a) -> double& { return R2(L.aol, e, a, nao); };
    auto MA = [&](int e, int j) -> double& { return R2(L.ma, e, j, nmu); };
    auto MX = [&](int e, int j) -> double& { return R2(L.mx, e, j, nmu); };
    auto MY = [&](int e, int j) -> double& { return R2(L.my, e, j, nmu); };
    auto MZ = [&](int e, int j) -> double& { return R2(L.mz, e, j, nmu); };
    auto ML = [&](int e, int j) -> double& { return R2(L.ml, e, j, nmu); };
    auto BK = [&](int e, int j) -> double& { return R2(L.b, e, j, nmu); };
    auto GA = [&](int e, int j) -> double& { return R2(L.ga, e, j, nmu); };
    auto GB = [&](int e, int j) -> double& { return R2(L.gb, e, j, nmu); };
    auto GJ = [&](int e, int x) -> double& { return R2(L.gj, e, x, 3); };
    auto LJ = [&](int e) -> double& { return sw[(L.lj + e) * ss]; };
    auto DGW = [&](int e, int x) -> double& { return R2(L.dgw, e, x, 3); };
    auto DLW = [&](int e) -> double& { return sw[(L.dlw + e) * ss]; };
    const PosView P{pos + w * 3 * ne, 1};
    // Jastrow: grad U, lap U + |grad U|^2 per electron and their w-derivatives
    // (K = w0 r / (1 + w r), K' = w0 / (1 + w r)^2, K'' = -2 w w0 / (1 + w r)^3)
    const double wj = d.use_jastrow ? __ldg(d.jastrow_w) : 0.0;
    for (int i = 0; i < ne; ++i) {
      double g[3] = {0.0, 0.0, 0.0}, dg[3] = {0.0, 0.0, 0.0}, lap = 0.0, dlap = 0.0;
      if (d.use_jastrow)
        for (int j = 0; j < ne; ++j) {
          if (j == i) continue;
          const double dx[3] = {P(3 * i) - P(3 * j), P(3 * i + 1) - P(3 * j + 1),
                                P(3 * i + 2) - P(3 * j + 2)};
          const double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
          const double w0 = same_spin(d, i, j) ? 0.25 : 0.5;
          const double u = 1.0 / (1.0 + wj * r), u2 = u * u, u3 = u2 * u;
          const double k1 = w0 * u2, k2 = -2.0 * wj * w0 * u3;
          const double dk1 = -2.0 * w0 * r * u3, dk2 = -2.0 * w0 * u3 + 6.0 * w0 * wj * r * u3 * u;
          for (int x = 0; x < 3; ++x) {
            g[x] += k1 * dx[x] / r;
            dg[x] += dk1 * dx[x] / r;
          }
          lap += 2.0 * k1 / r + k2;
          dlap += 2.0 * dk1 / r + dk2;
        }
      if (d.use_jastrow_en) {
        const EnTerms en = en_terms(d, P(3 * i), P(3 * i + 1), P(3 * i + 2));
        for (int x = 0; x < 3; ++x) g[x] += en.g[x];
        lap += en.lap;
      }
      for (int x = 0; x < 3; ++x) {
        GJ(i, x) = g[x];
        DGW(i, x) = dg[x];
      }
      LJ(i) = lap + g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
      DLW(i) = dlap;
    }
    // AO values, gradients, laplacians; MO rows; kinetic operator B
    for (int e = 0; e < ne; ++e) {
      for_each_ao<double, true>(t, P(3 * e), P(3 * e + 1), P(3 * e + 2),
                                [&](int a, const AOVal<double>& o) {
                                  AV(e, a) = o.v;
                                  AX(e, a) = o.gx;
                                  AY(e, a) = o.gy;
                                  AZ(e, a) = o.gz;
                                  AL(e, a) = o.lap;
                                });
      for (int j = 0; j < nmu; ++j) {
        double sa = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, sl = 0.0;
        for (int a = 0; a < nao; ++a) {
          const double wv = t.W[(int64_t)a * t.ncol + j];
          sa = fma(AV(e, a), wv, sa);
          sx = fma(AX(e, a), wv, sx);
          sy = fma(AY(e, a), wv, sy);
          sz = fma(AZ(e, a), wv, sz);
          sl = fma(AL(e, a), wv, sl);
        }
        MA(e, j) = sa;
        MX(e, j) = sx;
        MY(e, j) = sy;
        MZ(e, j) = sz;
        ML(e, j) = sl;
        BK(e, j) = -0.5 * (sl + 2.0 * (GJ(e, 0) * sx + GJ(e, 1) * sy + GJ(e, 2) * sz) + LJ(e) * sa);
        GA(e, j) = 0.0;
        GB(e, j) = 0.0;
      }
    }
    // unique spin determinants: D_u and T_u = Tr(A_u^-1 B_u)
    const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
    MView<double> LU{sw + L.lu * ss, (int64_t)nmax * ss, ss};
    MView<double> X{sw + L.x * ss, (int64_t)nmax * ss, ss};
    MView<double> Y{sw + L.y * ss, (int64_t)nmax * ss, ss};
    MView<double> Z{sw + L.z * ss, (int64_t)nmax * ss, ss};
    double* DV = sw + L.dv * ss;
    double* TV = sw + L.tv * ss;
    int piv[QMC_MAX_NSPIN], cols[QMC_MAX_NSPIN];
    auto inverse = [&](int s, int u, int n, int r0) {  // LU, X = A_u^-1; returns det
      det_columns(d, s, u, cols);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) LU(i, j) = MA(r0 + i, cols[j]);
      const double det = lu_factor<double>(LU, n, piv);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) X(i, j) = i == j ? 1.0 : 0.0;
      lu_solve<double>(LU, n, piv, X.c(), X, n);
      return det;
    };
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
      for (int u = 0; u < d.ndet[s]; ++u) {
        double det = 1.0, tr = 0.0;
        if (n > 0) {
          det = inverse(s, u, n, r0);
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) tr = fma(X(j, i), BK(r0 + i, cols[j]), tr);
        }
        const int k = (s ? d.ndet[0] : 0) + u;
        DV[k * ss] = det;
        TV[k * ss] = tr;
      }
    }
    auto dv = [&](int s, int u) { return DV[((s ? d.ndet[0] : 0) + u) * ss]; };
    auto tv = [&](int s, int u) { return TV[((s ? d.ndet[0] : 0) + u) * ss]; };
    double S = 0.0, num = 0.0;
    for (int k = 0; k < d.ncfg; ++k) {
      const int uu = __ldg(d.cfg_det[0] + k), ud = __ldg(d.cfg_det[1] + k);
      const double dk = dv(0, uu) * dv(1, ud), c = __ldg(d.ci_weight + k);
      S = fma(c, dk, S);
      num = fma(c * dk, tv(0, uu) + tv(1, ud), num);
    }
    const double ke = num / S;
    for (int k = 0; k < d.ncfg; ++k) {
      const int uu = __ldg(d.cfg_det[0] + k), ud = __ldg(d.cfg_det[1] + k);
      const double dk = dv(0, uu) * dv(1, ud);
      accC[k * ss] += gw * dk * (tv(0, uu) + tv(1, ud) - ke) / S;
    }
    // into the matrices: G_A = dKE/dA, G_B = dKE/dB (weighted by gout)
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
      if (n == 0) continue;
      for (int u = 0; u < d.ndet[s]; ++u) {
        double dT = 0.0, dD = 0.0;
        for (int k = 0; k < d.ncfg; ++k) {
          if (__ldg(d.cfg_det[s] + k) != u) continue;
          const int uo = __ldg(d.cfg_det[1 - s] + k);
          const int uu = s ? uo : u, ud = s ? u : uo;
          const double c = __ldg(d.ci_weight + k), dk = dv(0, uu) * dv(1, ud);
          dT = fma(gw * c, dk / S, dT);
          dD = fma(gw * c * (tv(0, uu) + tv(1, ud) - ke) / S, dv(1 - s, uo), dD);
        }
        if (dT == 0.0 && dD == 0.0) continue;
        const double det = inverse(s, u, n, r0);
        // Z = B_u X, Y = X Z = X B_u X
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double z = 0.0;
            for (int k = 0; k < n; ++k) z = fma(BK(r0 + i, cols[k]), X(k, j), z);
            Z(i, j) = z;
          }
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            double y = 0.0;
            for (int k = 0; k < n; ++k) y = fma(X(i, k), Z(k, j), y);
            Y(i, j) = y;
          }
        const double sd = dD * det;
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) {
            GA(r0 + i, cols[j]) += sd * X(j, i) - dT * Y(j, i);
            GB(r0 + i, cols[j]) += dT * X(j, i);
          }
      }
    }
    // through B: dA_total = G_A - lapJ/2 G_B, d lapMO = -G_B/2, d gradMO = -gradU G_B;
    // Jastrow weight through grad U and lap U + |grad U|^2
    double dwj = 0.0, dwn = 0.0;
    for (int e = 0; e < ne; ++e) {
      double dg[3] = {0.0, 0.0, 0.0}, dl = 0.0;
      for (int j = 0; j < nmu; ++j) {
        const double gb = GB(e, j);
        dg[0] -= gb * MX(e, j);
        dg[1] -= gb * MY(e, j);
        dg[2] -= gb * MZ(e, j);
        dl -= 0.5 * gb * MA(e, j);
        GA(e, j) -= 0.5 * LJ(e) * gb;
      }
      if (d.use_jastrow) {
        double gdg = 0.0;
        for (int x = 0; x < 3; ++x) {
          dwj = fma(dg[x], DGW(e, x), dwj);
          gdg = fma(GJ(e, x), DGW(e, x), gdg);
        }
        dwj = fma(dl, DLW(e) + 2.0 * gdg, dwj);
      }
      if (d.use_jastrow_en) {  // through grad U_en and lap U_en + |grad U|^2
        const EnTerms en = en_terms(d, P(3 * e), P(3 * e + 1), P(3 * e + 2));
        double gdg = 0.0;
        for (int x = 0; x < 3; ++x) {
          dwn = fma(dg[x], en.dg[x], dwn);
          gdg = fma(GJ(e, x), en.dg[x], gdg);
        }
        dwn = fma(dl, en.dlap + 2.0 * gdg, dwn);
      }
    }
    if (d.use_jastrow) accJ[0] += dwj;
    if (d.use_jastrow_en) accJ[ss] += dwn;
    // W[a][j]: sum_e AO(e,a) dA(e,j) - (lap AO(e,a) / 2 + gradU(e) . grad AO(e,a)) G_B(e,j)
    for (int a = 0; a < nao; ++a)
      for (int j = 0; j < nmu; ++j) {
        double sum = 0.0;
        for (int e = 0; e < ne; ++e) {
          const double hb = 0.5 * AL(e, a) + GJ(e, 0) * AX(e, a) + GJ(e, 1) * AY(e, a) +
                            GJ(e, 2) * AZ(e, a);
          sum = fma(AV(e, a), GA(e, j), sum);
          sum = fma(-hb, GB(e, j), sum);
        }
        accW[((int64_t)a * nmu + j) * ss] = sum;
      }
    // exponents: hA = sum_j dA W, hB = sum_j G_B W per AO; per primitive p
    //   d val / d alpha  = -vs w_p P r^2 e_p
    //   d grad / d alpha = w_p e_p (-r^2 dP - 2 r P (1 - alpha r^2))
    //   d lap / d alpha  = vs w_p e_p (-r^2 lapP + P (8 r^2 alpha - 4 r^4 alpha^2
    //                      - (6 + 4 l)(1 - alpha r^2)))
    for (int e = 0; e < ne; ++e) {
      const double ex = P(3 * e), ey = P(3 * e + 1), ez = P(3 * e + 2);
      const double gx = GJ(e, 0), gy = GJ(e, 1), gz = GJ(e, 2);
      for (int g = 0; g < t.ngroup; ++g) {
        const int A = t.group_atom[g];
        const double dx = ex - t.atom_xyz[3 * A], dy = ey - t.atom_xyz[3 * A + 1],
                     dz = ez - t.atom_xyz[3 * A + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const int np = t.group_prim[g + 1] - t.group_prim[g];
        for (int a = t.group_ao[g]; a < t.group_ao[g + 1]; ++a) {
          double ha = 0.0, hb = 0.0;
          for (int j = 0; j < nmu; ++j) {
            const double wv = t.W[(int64_t)a * t.ncol + j];
            ha = fma(GA(e, j), wv, ha);
            hb = fma(GB(e, j), wv, hb);
          }
          if (ha == 0.0 && hb == 0.0) continue;
          const int kx = t.ao_k[3 * a], ky = t.ao_k[3 * a + 1], kz = t.ao_k[3 * a + 2];
          const Poly<double> pl = cart_poly<double, true>(dx, dy, dz, kx, ky, kz);
          const int l = kx + ky + kz;
          const double vs = t.vscale ? t.vscale[a] : 1.0;
          for (int p = 0; p < np; ++p) {
            const int wi = t.ao_wofs[a] + p;
            const double al = t.walpha[wi], wp = t.wd[wi];
            double dval, dgx, dgy, dgz, dlap;
            if (t.radial != QMC_RADIAL_GTO) {  // Slater type
              const StoDAlpha sd = sto_dalpha(pl.p, pl.dx, pl.dy, pl.dz, pl.lap, l, dx, dy, dz,
                                              r2, t.ao_kr(a), al);
              dval = vs * wp * sd.v;
              dgx = wp * sd.gx;
              dgy = wp * sd.gy;
              dgz = wp * sd.gz;
              dlap = vs * wp * sd.lap;
            } else {
              const double ep = exp(-al * r2);
              const double q = 1.0 - al * r2;
              dval = -vs * wp * pl.p * r2 * ep;
              dgx = wp * ep * (-r2 * pl.dx - 2.0 * dx * pl.p * q);
              dgy = wp * ep * (-r2 * pl.dy - 2.0 * dy * pl.p * q);
              dgz = wp * ep * (-r2 * pl.dz - 2.0 * dz * pl.p * q);
              dlap = vs * wp * ep *
                     (-r2 * pl.lap + pl.p * (8.0 * r2 * al - 4.0 * r2 * r2 * al * al -
                                             (double)(6 + 4 * l) * q));
            }
            const double c = ha * dval - hb * (0.5 * dlap + gx * dgx + gy * dgy + gz * dgz);
            accE[(int64_t)__ldg(w_entry + wi) * ss] += c;
          }
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Electron-position gradients of psi (Jacobi formula)
// ---------------------------------------------------------------------------
// grad_i psi = J grad_i Sigma + J grad_i U Sigma with Sigma = sum_k c_k D_k and
// grad_i Sigma = sum_k c_k D_k Tr(A_u^-1 grad_i A_u) over the determinant u of
// electron i's spin; only row i of grad_i A_u is non-zero, so the trace is
// sum_j (A_u^-1)[j][i] grad MO_cols[j](r_i) (slater_jastrow.py:346-447).
struct GradLayout {
  int64_t aov, aox, aoy, aoz, ma, mx, my, mz, lu, x, dv, gd, total;
};

__host__ __device__ inline GradLayout grad_layout(const qmc_wf_desc& d) {
  GradLayout L;
  const int64_t ne = d.nelec, nao = d.nao, nmu = d.nmo_used;
  const int64_t nmax = d.nup > d.ndown ? d.nup : d.ndown, nd = d.ndet[0] + d.ndet[1];
  int64_t o = 0;
  auto take = [&](int64_t n) {
    const int64_t r = o;
    o += n;
    return r;
  };
  L.aov = take(ne * nao);
  L.aox = take(ne * nao);
  L.aoy = take(ne * nao);
  L.aoz = take(ne * nao);
  L.ma = take(ne * nmu);
  L.mx = take(ne * nmu);
  L.my = take(ne * nmu);
  L.mz = take(ne * nmu);
  L.lu = take(nmax * nmax);
  L.x = take(nmax * nmax);
  L.dv = take(nd);
  L.gd = take(nd * nmax * 3);  // per determinant: d log D_u / d r_i for its spin's electrons
  L.total = o;
  return L;
}

__global__ void __launch_bounds__(kAdjTPB) grad_kernel(const qmc_wf_desc d,
                                                       const double* __restrict__ pos, int64_t nw,
                                                       int pdf, double* __restrict__ out,
                                                       double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  const int nmu = d.nmo_used, ne = d.nelec, nao = d.nao;
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const GradLayout L = grad_layout(d);
  double* sw = scr + w;
  auto R2 = [&](int64_t base, int e, int k, int n) -> double& {
    return sw[(base + (int64_t)e * n + k) * ss];
  };
  const PosView P{pos + w * 3 * ne, 1};
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  // Jastrow: U and grad_i U
  double logj = 0.0;
  double* o = out + w * 3 * ne;
  for (int i = 0; i < 3 * ne; ++i) o[i] = 0.0;
  const double wj = d.use_jastrow ? __ldg(d.jastrow_w) : 0.0;
  // AO values and gradients, MO rows
  for (int e = 0; e < ne; ++e) {
    for_each_ao<double, true>(t, P(3 * e), P(3 * e + 1), P(3 * e + 2),
                              [&](int a, const AOVal<double>& v) {
                                R2(L.aov, e, a, nao) = v.v;
                                R2(L.aox, e, a, nao) = v.gx;
                                R2(L.aoy, e, a, nao) = v.gy;
                                R2(L.aoz, e, a, nao) = v.gz;
                              });
    for (int j = 0; j < nmu; ++j) {
      double sa = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
      for (int a = 0; a < nao; ++a) {
        const double wv = t.W[(int64_t)a * t.ncol + j];
        sa = fma(R2(L.aov, e, a, nao), wv, sa);
        sx = fma(R2(L.aox, e, a, nao), wv, sx);
        sy = fma(R2(L.aoy, e, a, nao), wv, sy);
        sz = fma(R2(L.aoz, e, a, nao), wv, sz);
      }
      R2(L.ma, e, j, nmu) = sa;
      R2(L.mx, e, j, nmu) = sx;
      R2(L.my, e, j, nmu) = sy;
      R2(L.mz, e, j, nmu) = sz;
    }
  }
  // determinants and d log D_u / d r_i
  MView<double> LU{sw + L.lu * ss, (int64_t)nmax * ss, ss};
  MView<double> X{sw + L.x * ss, (int64_t)nmax * ss, ss};
  double* DV = sw + L.dv * ss;
  int piv[QMC_MAX_NSPIN], cols[QMC_MAX_NSPIN];
  for (int s = 0; s < 2; ++s) {
    const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
    for (int u = 0; u < d.ndet[s]; ++u) {
      const int k = (s ? d.ndet[0] : 0) + u;
      double det = 1.0;
      if (n > 0) {
        det_columns(d, s, u, cols);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) LU(i, j) = R2(L.ma, r0 + i, cols[j], nmu);
        det = lu_factor<double>(LU, n, piv);
        for (int i = 0; i < n; ++i)
          for (int j = 0; j < n; ++j) X(i, j) = i == j ? 1.0 : 0.0;
        lu_solve<double>(LU, n, piv, X.c(), X, n);
        for (int i = 0; i < n; ++i) {
          double gx = 0.0, gy = 0.0, gz = 0.0;
          for (int j = 0; j < n; ++j) {
            const double xv = X(j, i);
            gx = fma(xv, R2(L.mx, r0 + i, cols[j], nmu), gx);
            gy = fma(xv, R2(L.my, r0 + i, cols[j], nmu), gy);
            gz = fma(xv, R2(L.mz, r0 + i, cols[j], nmu), gz);
          }
          sw[(L.gd + ((int64_t)k * nmax + i) * 3 + 0) * ss] = gx;
          sw[(L.gd + ((int64_t)k * nmax + i) * 3 + 1) * ss] = gy;
          sw[(L.gd + ((int64_t)k * nmax + i) * 3 + 2) * ss] = gz;
        }
      }
      DV[k * ss] = det;
    }
  }
  auto dvk = [&](int s, int u) { return DV[((s ? d.ndet[0] : 0) + u) * ss]; };
  double sigma = 0.0;
  for (int k = 0; k < d.ncfg; ++k) {
    const int uu = __ldg(d.cfg_det[0] + k), ud = __ldg(d.cfg_det[1] + k);
    const double cd = __ldg(d.ci_weight + k) * dvk(0, uu) * dvk(1, ud);
    sigma += cd;
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0;
      const int kk = s ? d.ndet[0] + ud : uu;
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < 3; ++q)
          o[3 * (r0 + i) + q] = fma(cd, sw[(L.gd + ((int64_t)kk * nmax + i) * 3 + q) * ss],
                                    o[3 * (r0 + i) + q]);
    }
  }
  // Jastrow: grad_i U (Pade kernels, K' = w0 / (1 + w r)^2 for e-e pairs and
  // 1 / (1 + w_en r)^2 for electron-nucleus pairs) and psi = J Sigma
  double J = 1.0;
  if (d.use_jastrow || d.use_jastrow_en) {
    for (int i = 0; i < ne; ++i) {
      double g[3] = {0.0, 0.0, 0.0};
      if (d.use_jastrow_en) {
        const EnTerms en = en_terms(d, P(3 * i), P(3 * i + 1), P(3 * i + 2));
        logj += en.u;
        for (int q = 0; q < 3; ++q) g[q] += en.g[q];
      }
      for (int j = 0; j < ne && d.use_jastrow; ++j) {
        if (j == i) continue;
        const double dx[3] = {P(3 * i) - P(3 * j), P(3 * i + 1) - P(3 * j + 1),
                              P(3 * i + 2) - P(3 * j + 2)};
        const double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        const double w0 = same_spin(d, i, j) ? 0.25 : 0.5;
        const double u = 1.0 / (1.0 + wj * r);
        if (j > i) logj += w0 * r * u;
        for (int q = 0; q < 3; ++q) g[q] += w0 * u * u * dx[q] / r;
      }
      for (int q = 0; q < 3; ++q) o[3 * i + q] = fma(g[q], sigma, o[3 * i + q]);
    }
    J = exp(logj);
  }
  const double scale = pdf ? 2.0 * J * J * sigma : J;  // grad psi or grad psi^2 = 2 psi grad psi
  for (int i = 0; i < 3 * ne; ++i) o[i] *= scale;
}

// Sum of parameter i's walker slots in a fixed order (per-thread strided
// partial sums, then a fixed tree), added to its output: W (row stride ldw),
// exponents, CI weights, Pade weight. One block per parameter.
constexpr int kRedTPB = 256;
__global__ void __launch_bounds__(kRedTPB) adj_reduce_kernel(
    const double* __restrict__ gacc, int64_t nw, int64_t ss, int nao, int nmu, int nweight,
    int nent, int ncfg, double* __restrict__ g_W, int ldw, double* __restrict__ g_exp,
    double* __restrict__ g_ci, double* __restrict__ g_jw, double* __restrict__ g_jwn) {
  __shared__ double sh[kRedTPB];
  const int64_t i = blockIdx.x;
  const double* row = gacc + i * ss;
  double s = 0.0;
  for (int64_t w = threadIdx.x; w < nw; w += kRedTPB) s += row[w];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = kRedTPB / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double v = sh[0];
  const int64_t nw_ = (int64_t)nao * nmu;
  if (i < nw_) {
    g_W[(i / nmu) * ldw + i % nmu] += v;
  } else if (i < nw_ + nweight) {
    const int e = (int)(i - nw_);
    if (e < nent) g_exp[e] += v;
  } else if (i < nw_ + nweight + ncfg) {
    g_ci[i - nw_ - nweight] += v;
  } else if (i == nw_ + nweight + ncfg) {
    if (g_jw) g_jw[0] += v;
  } else if (g_jwn) {
    g_jwn[0] += v;
  }
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
  if (nentries > d->nweight) return QMC_ERR_ARG;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = tables_smem_bytes<double>(*d, ncol);
  if ((st = prepare_smem(psi_adjoint_kernel, smem))) return st;
  const dim3 grid((unsigned)((nw + kAdjTPB - 1) / kAdjTPB));
  const int64_t ss = pad_walkers(nw);
  cudaStream_t cs = (cudaStream_t)stream;
  psi_adjoint_kernel<<<grid, kAdjTPB, smem, cs>>>(dd, pos, nw, gout, weight_entry, (double*)scratch, ss);
  const double* gacc = (const double*)scratch + adj_layout(dd).gacc * ss;
  adj_reduce_kernel<<<(unsigned)adj_acc_doubles(dd), kRedTPB, 0, cs>>>(
      gacc, nw, ss, dd.nao, dd.nmo_used, dd.nweight, nentries, dd.ncfg, grad_W, ldw, grad_exp,
      grad_ci, d->use_jastrow ? grad_jastrow_w : nullptr,
      d->use_jastrow_en ? grad_jastrow_w + 1 : nullptr);
  return launch_status();
}

int64_t qmc_eloc_adjoint_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  if (check_desc(d) != QMC_OK || nw < 0) return -1;
  return el_adj_layout(*d).total * pad_walkers(nw) * (int64_t)sizeof(double);
}

int qmc_wf_local_energy_adjoint(const qmc_wf_desc* d0, const double* pos, int64_t nw,
                                const double* gout, const int32_t* weight_entry, int32_t nentries,
                                double* grad_exp, double* grad_W, int32_t ldw,
                                double* grad_jastrow_w, double* grad_ci, void* scratch,
                                int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;  // the adjoint is FP64
  const qmc_wf_desc* d = &dd;
  if (nw < 0 || nentries < 0 || ldw < d->nmo_used) return QMC_ERR_ARG;
  if (nw > 0 && (!pos || !gout || !weight_entry || !grad_exp || !grad_W || !grad_ci || !scratch))
    return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (scratch_bytes < qmc_eloc_adjoint_scratch_bytes(d, nw)) return QMC_ERR_SCRATCH;
  if (nentries > d->nweight) return QMC_ERR_ARG;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = tables_smem_bytes<double>(*d, ncol);
  if ((st = prepare_smem(eloc_adjoint_kernel, smem))) return st;
  const dim3 grid((unsigned)((nw + kAdjTPB - 1) / kAdjTPB));
  const int64_t ss = pad_walkers(nw);
  cudaStream_t cs = (cudaStream_t)stream;
  eloc_adjoint_kernel<<<grid, kAdjTPB, smem, cs>>>(dd, pos, nw, gout, weight_entry, (double*)scratch, ss);
  const double* gacc = (const double*)scratch + el_adj_layout(dd).gacc * ss;
  adj_reduce_kernel<<<(unsigned)adj_acc_doubles(dd), kRedTPB, 0, cs>>>(
      gacc, nw, ss, dd.nao, dd.nmo_used, dd.nweight, nentries, dd.ncfg, grad_W, ldw, grad_exp,
      grad_ci, d->use_jastrow ? grad_jastrow_w : nullptr,
      d->use_jastrow_en ? grad_jastrow_w + 1 : nullptr);
  return launch_status();
}

int64_t qmc_grad_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  if (check_desc(d) != QMC_OK || nw < 0) return -1;
  return grad_layout(*d).total * pad_walkers(nw) * (int64_t)sizeof(double);
}

int qmc_wf_gradients(const qmc_wf_desc* d0, const double* pos, int64_t nw, int32_t pdf,
                     double* grad, void* scratch, int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;
  const qmc_wf_desc* d = &dd;
  if (nw < 0) return QMC_ERR_ARG;
  if (nw == 0) return QMC_OK;
  if (!pos || !grad || !scratch) return QMC_ERR_ARG;
  if (scratch_bytes < qmc_grad_scratch_bytes(d, nw)) return QMC_ERR_SCRATCH;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = tables_smem_bytes<double>(*d, ncol);
  if ((st = prepare_smem(grad_kernel, smem))) return st;
  const dim3 grid((unsigned)((nw + kAdjTPB - 1) / kAdjTPB));
  grad_kernel<<<grid, kAdjTPB, smem, (cudaStream_t)stream>>>(dd, pos, nw, pdf ? 1 : 0, grad,
                                                             (double*)scratch, pad_walkers(nw));
  return launch_status();
}

}  // extern "C"
