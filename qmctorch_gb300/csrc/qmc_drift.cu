// Drift-diffusion (generalized) Metropolis and Hamiltonian Monte Carlo on the
// device, FP64, one thread per walker for all steps of a call
// (generalized_metropolis.py:46-219, hamiltonian.py:75-201); the HMC kernel is
// at the end of the file.
//
// The reference's chain, kept as it is so that replayed draws give its chains:
// every proposal starts from the walkers' positions at the start of the call
// (move() clones walkers.pos, which is written back only after the last step)
// with one electron e moved by step * drift_i(e) + eta, eta ~ N(0, sqrt(step) I);
// the transition kernel is exp(-|x_f - x_i - step drift_i| / (2 step)) with the
// norm (not its square) of the whole walker vector; zero densities become
// 1e-16 after the drift is taken, so a proposal whose density is zero (or
// underflows) has a NaN drift there and is rejected; accept when
// min(1, T_if rho_f / (T_fi rho_i)) - u >= 0.
//
// Because each proposal differs from the start positions in one electron only,
// the start positions' MO rows (values and gradients), spin determinants,
// determinant gradients and Jastrow gradient are computed once per call; a
// step evaluates the moved electron's MO row, refactors the determinants of
// its spin with that row replaced, and updates the Jastrow terms of its pairs.
// psi and its electron gradient at the proposal are therefore the full
// Jacobi-formula values (slater_jastrow.py:346-447), not an approximation.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"
#include "qmc_rng.cuh"

namespace qmc {

constexpr int kDriftTPB = 64;

struct DriftLayout {  // per-walker doubles, item-major
  int64_t xi, ma, mx, my, mz, ao, nr, lu, x, dv0, gd0, dvf, gdf, jg0, dri, drf, total;
};

__host__ __device__ inline DriftLayout drift_layout(const qmc_wf_desc& d) {
  DriftLayout L;
  const int64_t ne = d.nelec, nmu = d.nmo_used, nao = d.nao;
  const int64_t nmax = d.nup > d.ndown ? d.nup : d.ndown, nd = d.ndet[0] + d.ndet[1];
  int64_t o = 0;
  auto take = [&](int64_t n) {
    const int64_t r = o;
    o += n;
    return r;
  };
  L.xi = take(3 * ne);        // current (accepted) positions
  L.ma = take(ne * nmu);      // start positions: MO values
  L.mx = take(ne * nmu);      // and their gradients
  L.my = take(ne * nmu);
  L.mz = take(ne * nmu);
  L.ao = take(4 * nao);       // AO values and gradients of one electron
  L.nr = take(4 * nmu);       // the moved electron's MO row (value, gradient)
  L.lu = take(nmax * nmax);
  L.x = take(nmax * nmax);    // inverse of one spin determinant
  L.dv0 = take(nd);           // spin determinants at the start positions
  L.gd0 = take(nd * nmax * 3);  // their d log D / d r_i
  L.dvf = take(nd);           // the moved spin's determinants at the proposal
  L.gdf = take(nd * nmax * 3);
  L.jg0 = take(3 * ne);       // grad log J at the start positions
  L.dri = take(3 * ne);       // drift at x_i
  L.drf = take(3 * ne);       // drift at the proposal
  L.total = o;
  return L;
}

// MO values and gradients of one electron at (x, y, z): AO values and
// gradients through the scratch, then the contraction with W; row element j
// of quantity q (0 value, 1..3 gradient) goes to sw[(dst[q] + j) * ss].
__device__ inline void drift_rows(const Tables<double>& t, int nmu, double* sw, int64_t ss,
                                  int64_t ao, double x, double y, double z, const int64_t (&dst)[4]) {
  const int nao = t.nao;
  for_each_ao<double, true>(t, x, y, z, [&](int a, const AOVal<double>& v) {
    sw[(ao + a) * ss] = v.v;
    sw[(ao + nao + a) * ss] = v.gx;
    sw[(ao + 2 * nao + a) * ss] = v.gy;
    sw[(ao + 3 * nao + a) * ss] = v.gz;
  });
  for (int j = 0; j < nmu; ++j) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int a = 0; a < nao; ++a) {
      const double w = t.W[(int64_t)a * t.ncol + j];
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q] = fma(sw[(ao + q * nao + a) * ss], w, s[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) sw[(dst[q] + j) * ss] = s[q];
  }
}

// Spin determinant u of spin s from the start rows, with electron er's row
// taken from the moved row (er < 0: none); writes d log D / d r_i of the
// spin's electrons to sw[(gd + i * 3 + q) * ss] and returns D.
__device__ inline double drift_det(const qmc_wf_desc& d, const DriftLayout& L, double* sw,
                                   int64_t ss, int s, int u, int er, int64_t gd) {
  const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0, nmu = d.nmo_used;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  if (n == 0) return 1.0;
  int cols[QMC_MAX_NSPIN], piv[QMC_MAX_NSPIN];
  det_columns(d, s, u, cols);
  auto row = [&](int q, int i, int c) -> double {
    if (r0 + i == er) return sw[(L.nr + (int64_t)q * nmu + c) * ss];
    const int64_t base = q == 0 ? L.ma : (q == 1 ? L.mx : (q == 2 ? L.my : L.mz));
    return sw[(base + (int64_t)(r0 + i) * nmu + c) * ss];
  };
  MView<double> LU{sw + L.lu * ss, (int64_t)nmax * ss, ss};
  MView<double> X{sw + L.x * ss, (int64_t)nmax * ss, ss};
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) LU(i, j) = row(0, i, cols[j]);
  const double det = lu_factor<double>(LU, n, piv);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) X(i, j) = i == j ? 1.0 : 0.0;
  lu_solve<double>(LU, n, piv, X.c(), X, n);
  for (int i = 0; i < n; ++i) {
    double g[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < n; ++j) {
      const double xv = X(j, i);
#pragma unroll
      for (int q = 0; q < 3; ++q) g[q] = fma(xv, row(q + 1, i, cols[j]), g[q]);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) sw[(gd + (int64_t)i * 3 + q) * ss] = g[q];
  }
  return det;
}

// Electron-electron Pade pair of electrons i and j at the given coordinates:
// adds w0 r / (1 + w r) to *u and w0 / (1 + w r)^2 (x_i - x_j) / r to g.
__device__ __forceinline__ void pade_pair(double w0, double w, const double (&xi)[3],
                                          const double (&xj)[3], double* u, double (&g)[3]) {
  const double dx[3] = {xi[0] - xj[0], xi[1] - xj[1], xi[2] - xj[2]};
  const double r = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
  const double iu = 1.0 / (1.0 + w * r);
  *u += w0 * r * iu;
#pragma unroll
  for (int q = 0; q < 3; ++q) g[q] += w0 * iu * iu * dx[q] / r;
}

// Sum over the CI configurations: returns Sigma = sum_k c_k D_k^up D_k^dn and
// writes grad Sigma (the Jacobi traces weighted by each configuration) to
// sw[(out + c) * ss]; the moved spin sm's determinants come from dvf / gdf
// (sm < 0: none moved), the others from dv0 / gd0.
__device__ inline double drift_slater(const qmc_wf_desc& d, const DriftLayout& L, double* sw,
                                      int64_t ss, int sm, int64_t out) {
  const int nc = 3 * d.nelec, nmax = d.nup > d.ndown ? d.nup : d.ndown;
  auto S = [&](int64_t item) -> double& { return sw[item * ss]; };
  for (int c = 0; c < nc; ++c) S(out + c) = 0.0;
  double sigma = 0.0;
  for (int k = 0; k < d.ncfg; ++k) {
    const int uu = __ldg(d.cfg_det[0] + k), ud = __ldg(d.cfg_det[1] + k);
    const int k0 = uu, k1 = d.ndet[0] + ud;
    const double dv0 = S((sm == 0 ? L.dvf : L.dv0) + k0);
    const double dv1 = S((sm == 1 ? L.dvf : L.dv0) + k1);
    const double cd = __ldg(d.ci_weight + k) * dv0 * dv1;
    sigma += cd;
    for (int s = 0; s < 2; ++s) {
      const int n = s ? d.ndown : d.nup, r0 = s ? d.nup : 0, kk = s ? k1 : k0;
      const int64_t gd = (s == sm ? L.gdf : L.gd0) + (int64_t)kk * nmax * 3;
      for (int i = 0; i < n; ++i)
        for (int q = 0; q < 3; ++q)
          S(out + 3 * (r0 + i) + q) = fma(cd, S(gd + i * 3 + q), S(out + 3 * (r0 + i) + q));
    }
  }
  return sigma;
}

// Full evaluation at positions P (coordinate c at P[c * ps]): the MO rows and
// their gradients into ma..mz, the spin determinants and their electron
// gradients into dv0 / gd0, the Jastrow gradient into jg0, and
// grad log psi = grad Sigma / Sigma + grad log J into sw[(out + c) * ss].
// Returns Sigma; *logj = log J.
__device__ inline double drift_full_eval(const qmc_wf_desc& d, const Tables<double>& t,
                                         const DriftLayout& L, double* sw, int64_t ss,
                                         const double* P, int64_t ps, int64_t out,
                                         double* logj) {
  const int ne = d.nelec, nmu = d.nmo_used, nc = 3 * ne;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  auto S = [&](int64_t item) -> double& { return sw[item * ss]; };
  auto xyz = [&](int e, double (&p)[3]) {
    for (int q = 0; q < 3; ++q) p[q] = P[(3 * e + q) * ps];
  };
  for (int e = 0; e < ne; ++e) {
    const int64_t dst[4] = {L.ma + (int64_t)e * nmu, L.mx + (int64_t)e * nmu,
                            L.my + (int64_t)e * nmu, L.mz + (int64_t)e * nmu};
    drift_rows(t, nmu, sw, ss, L.ao, P[3 * e * ps], P[(3 * e + 1) * ps], P[(3 * e + 2) * ps],
               dst);
  }
  for (int s = 0; s < 2; ++s)
    for (int u = 0; u < d.ndet[s]; ++u) {
      const int k = (s ? d.ndet[0] : 0) + u;
      S(L.dv0 + k) = drift_det(d, L, sw, ss, s, u, -1, L.gd0 + (int64_t)k * nmax * 3);
    }
  const double wj = d.use_jastrow ? __ldg(d.jastrow_w) : 0.0;
  double lj = 0.0;
  for (int i = 0; i < ne; ++i) {
    double g[3] = {0.0, 0.0, 0.0}, pi[3];
    xyz(i, pi);
    double ui = 0.0;
    if (d.use_jastrow_en) {
      const EnTerms en = en_terms(d, pi[0], pi[1], pi[2]);
      lj += en.u;
      for (int q = 0; q < 3; ++q) g[q] += en.g[q];
    }
    if (d.use_jastrow) {
      for (int j = 0; j < ne; ++j) {
        if (j == i) continue;
        double pj[3], uj = 0.0;
        xyz(j, pj);
        pade_pair(same_spin(d, i, j) ? 0.25 : 0.5, wj, pi, pj, &uj, g);
        if (j > i) ui += uj;
      }
    }
    lj += ui;
    for (int q = 0; q < 3; ++q) S(L.jg0 + 3 * i + q) = g[q];
  }
  const double sigma = drift_slater(d, L, sw, ss, -1, out);
  for (int c = 0; c < nc; ++c) S(out + c) = S(out + c) / sigma + S(L.jg0 + c);
  *logj = lj;
  return sigma;
}

__global__ void __launch_bounds__(kDriftTPB) drift_kernel(const qmc_wf_desc d,
                                                          const qmc_drift_args a,
                                                          double* __restrict__ scr, int64_t ss,
                                                          double sd) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= a.nwalkers) return;
  const int ne = d.nelec, nmu = d.nmo_used, nc = 3 * ne;
  const DriftLayout L = drift_layout(d);
  double* sw = scr + w;
  auto S = [&](int64_t item) -> double& { return sw[item * ss]; };
  double* xs = a.pos + w * nc;  // start positions (read-only until the end)
  const double wj = d.use_jastrow ? __ldg(d.jastrow_w) : 0.0;
  const double step = a.step_size;
  auto xyz = [&](int e, double (&p)[3]) {
    for (int q = 0; q < 3; ++q) p[q] = xs[3 * e + q];
  };

  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  // ---- start positions: MO rows, spin determinants, Jastrow, drift ----
  double logj0, rhoi;
  {
    const double sigma = drift_full_eval(d, t, L, sw, ss, xs, 1, L.dri, &logj0);
    const double psi = exp(logj0) * sigma;
    rhoi = psi * psi;
    if (rhoi == 0.0) {
      // the reference's drift grad(rho) / (2 rho) is undefined where rho is
      // zero (underflow included): every later transition kernel is NaN and
      // every move of this walker is rejected
      rhoi = 1e-16;
      for (int c = 0; c < nc; ++c) S(L.dri + c) = nan("");
    }
    for (int c = 0; c < nc; ++c) S(L.xi + c) = xs[c];
  }

  Rng rng{(uint32_t)a.seed, (uint32_t)(a.seed >> 32), (uint32_t)w, 0, 0};
  const bool replay = a.electron_index != nullptr;
  int nacc = 0, idecor = 0;
  int64_t isnap = 0;
  for (int istep = 0; istep < a.nstep; ++istep) {
    // ---- draws: the moved electron, its noise, the acceptance uniform ----
    int e;
    double eta[3], uacc;
    if (replay) {
      const int64_t o = (int64_t)istep * a.nwalkers + w;
      e = a.electron_index[o];
      for (int q = 0; q < 3; ++q) eta[q] = a.normals[o * 3 + q];
      uacc = a.uniforms[o];
    } else {
      rng.step = a.step_offset + istep;
      rng.call = 0;
      const U4 r0 = rng.next();
      e = (int)(((uint64_t)r0.x * (uint64_t)ne) >> 32);
      uacc = rng.uniform53(r0.y, r0.z);
      const U4 r1 = rng.next();
      double z3;
      rng.normal2(r1.x, r1.y, eta[0], eta[1]);
      rng.normal2(r1.z, r1.w, eta[2], z3);
      for (int q = 0; q < 3; ++q) eta[q] *= sd;
    }
    if (e < 0 || e >= ne) e = 0;  // replayed indices are checked by the host
    // proposal: start positions with electron e at xs_e + (step drift_i(e) + eta)
    double pe[3], pe0[3];
    xyz(e, pe0);
    for (int q = 0; q < 3; ++q)
      pe[q] = __dadd_rn(pe0[q], __dadd_rn(__dmul_rn(step, S(L.dri + 3 * e + q)), eta[q]));

    // ---- psi and drift at the proposal ----
    const int64_t nrd[4] = {L.nr, L.nr + nmu, L.nr + 2 * nmu, L.nr + 3 * nmu};
    drift_rows(t, nmu, sw, ss, L.ao, pe[0], pe[1], pe[2], nrd);
    const int sm = e < d.nup ? 0 : 1;
    for (int u = 0; u < d.ndet[sm]; ++u) {
      const int k = (sm ? d.ndet[0] : 0) + u;
      S(L.dvf + k) = drift_det(d, L, sw, ss, sm, u, e, L.gdf + (int64_t)k * nmax * 3);
    }
    const double sigma = drift_slater(d, L, sw, ss, sm, L.drf);
    // Jastrow: the pairs of e and its electron-nucleus terms change
    double logj = logj0, ge[3] = {0.0, 0.0, 0.0};
    if (d.use_jastrow_en) {
      const EnTerms en1 = en_terms(d, pe[0], pe[1], pe[2]);
      const EnTerms en0 = en_terms(d, pe0[0], pe0[1], pe0[2]);
      logj += en1.u - en0.u;
      for (int q = 0; q < 3; ++q) ge[q] += en1.g[q];
    }
    for (int j = 0; j < ne; ++j) {
      double gj[3];
      for (int q = 0; q < 3; ++q) gj[q] = S(L.jg0 + 3 * j + q);
      if (j != e && d.use_jastrow) {
        double pj[3], u1 = 0.0, u0 = 0.0, g1[3] = {0.0, 0.0, 0.0}, g0[3] = {0.0, 0.0, 0.0};
        xyz(j, pj);
        const double w0 = same_spin(d, e, j) ? 0.25 : 0.5;
        pade_pair(w0, wj, pj, pe, &u1, g1);   // pair (j, e) at the proposal
        pade_pair(w0, wj, pj, pe0, &u0, g0);  // and at the start
        logj += u1 - u0;
        for (int q = 0; q < 3; ++q) {
          gj[q] += g1[q] - g0[q];
          ge[q] -= g1[q];  // grad_e of the pair is minus grad_j
        }
      }
      if (j != e)
        for (int q = 0; q < 3; ++q) S(L.drf + 3 * j + q) = S(L.drf + 3 * j + q) / sigma + gj[q];
    }
    for (int q = 0; q < 3; ++q) S(L.drf + 3 * e + q) = S(L.drf + 3 * e + q) / sigma + ge[q];
    const double psif = exp(logj) * sigma;
    double rhof = psif * psif;
    const bool defined = rhof != 0.0;  // else the reference's drift is NaN: rejected
    if (rhof == 0.0) rhof = 1e-16;

    // ---- transition kernels and the decision ----
    double a1 = 0.0, a2 = 0.0;
    for (int c = 0; c < nc; ++c) {
      const int ec = c / 3;
      const double xf = ec == e ? pe[c - 3 * e] : xs[c];
      const double xi = S(L.xi + c);
      const double t1 = __dsub_rn(__dsub_rn(xi, xf), __dmul_rn(S(L.drf + c), step));
      const double t2 = __dsub_rn(__dsub_rn(xf, xi), __dmul_rn(S(L.dri + c), step));
      a1 = fma(t1, t1, a1);
      a2 = fma(t2, t2, a2);
    }
    const double tif = exp(-0.5 * sqrt(a1) / step), tfi = exp(-0.5 * sqrt(a2) / step);
    double p = (tif * rhof) / (tfi * rhoi);
    if (p > 1.0) p = 1.0;
    if (defined && p - uacc >= 0.0) {
      ++nacc;
      for (int c = 0; c < nc; ++c) {
        const int ec = c / 3;
        S(L.xi + c) = ec == e ? pe[c - 3 * e] : xs[c];
        S(L.dri + c) = S(L.drf + c);
      }
      rhoi = rhof;
    }
    if (istep >= a.ntherm) {
      if (idecor % a.ndecor == 0 && a.samples && isnap < a.nsnap) {
        double* o = a.samples + (isnap * a.nwalkers + w) * nc;
        for (int c = 0; c < nc; ++c) o[c] = S(L.xi + c);
        ++isnap;
      }
      ++idecor;
    }
  }
  for (int c = 0; c < nc; ++c) xs[c] = S(L.xi + c);
  if (a.accepted) a.accepted[w] += nacc;
}

// ---------------------------------------------------------------------------
// Hamiltonian Monte Carlo (hamiltonian.py:75-201)
// ---------------------------------------------------------------------------
// Per step and walker: momenta p ~ N(0, I) over all 3 Ne coordinates,
// H_start = U(q) + |p|^2 / 2 with U = -log psi^2, a leapfrog trajectory of L
// steps of size eps (half momentum step, L - 1 full position + momentum steps,
// a last position step and half momentum step) with the force
// -grad U = 2 grad psi / psi from the full Jacobi evaluation at each point,
// p negated, and the end point rejected when exp(H_start - H_end) < u. The
// trajectory's positions, momenta and forces live in the walker's work
// arrays (xi, dri, drf); pos holds the chain's current positions.
__global__ void __launch_bounds__(kDriftTPB) hmc_kernel(const qmc_wf_desc d,
                                                        const qmc_hmc_args a,
                                                        double* __restrict__ scr, int64_t ss) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ncol = round_up(d.nmo_used, 8);
  const Tables<double> t = load_tables<double>(d, d.nmo_used, ncol, smem);
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= a.nwalkers) return;
  const int nc = 3 * d.nelec;
  const DriftLayout L = drift_layout(d);
  double* sw = scr + w;
  auto S = [&](int64_t item) -> double& { return sw[item * ss]; };
  double* x0 = a.pos + w * nc;  // the chain's current positions
  const double eps = a.step_size, heps = 0.5 * a.step_size;
  const bool replay = a.momenta != nullptr;
  Rng rng{(uint32_t)a.seed, (uint32_t)(a.seed >> 32), (uint32_t)w, 0, 0};
  int nacc = 0, idecor = 0;
  int64_t isnap = 0;
  double* q = sw + L.xi * ss;  // trajectory positions, stride ss
  for (int istep = 0; istep < a.nstep; ++istep) {
    // momenta (replayed, or Box-Muller pairs of the step's Philox stream)
    rng.step = a.step_offset + istep;
    rng.call = 0;
    double psq = 0.0;
    for (int c = 0; c < nc; c += 4) {
      double z[4];
      if (replay) {
        for (int k = 0; k < 4 && c + k < nc; ++k)
          z[k] = a.momenta[((int64_t)istep * a.nwalkers + w) * nc + c + k];
      } else {
        const U4 r = rng.next();
        rng.normal2(r.x, r.y, z[0], z[1]);
        rng.normal2(r.z, r.w, z[2], z[3]);
      }
      for (int k = 0; k < 4 && c + k < nc; ++k) {
        S(L.dri + c + k) = z[k];
        psq = fma(z[k], z[k], psq);
      }
    }
    for (int c = 0; c < nc; ++c) S(L.xi + c) = x0[c];
    double logj;
    double sigma = drift_full_eval(d, t, L, sw, ss, x0, 1, L.drf, &logj);
    const double h0 = -2.0 * (logj + log(fabs(sigma))) + 0.5 * psq;
    // half step in momentum: p -= (eps / 2) grad U, grad U = -2 grad log psi
    for (int c = 0; c < nc; ++c)
      S(L.dri + c) = __dsub_rn(S(L.dri + c), __dmul_rn(heps, -2.0 * S(L.drf + c)));
    for (int l = 0; l < a.traj_length; ++l) {
      for (int c = 0; c < nc; ++c) q[c * ss] = __dadd_rn(q[c * ss], __dmul_rn(eps, S(L.dri + c)));
      sigma = drift_full_eval(d, t, L, sw, ss, q, ss, L.drf, &logj);
      const double f = l + 1 < a.traj_length ? eps : heps;  // the last momentum step is a half step
      for (int c = 0; c < nc; ++c)
        S(L.dri + c) = __dsub_rn(S(L.dri + c), __dmul_rn(f, -2.0 * S(L.drf + c)));
    }
    // p is negated before the kinetic energy, which its sign does not change
    psq = 0.0;
    for (int c = 0; c < nc; ++c) psq = fma(S(L.dri + c), S(L.dri + c), psq);
    const double h1 = -2.0 * (logj + log(fabs(sigma))) + 0.5 * psq;
    double u;
    if (replay) {
      u = a.uniforms[(int64_t)istep * a.nwalkers + w];
    } else {
      rng.call = (uint32_t)((nc + 3) / 4);
      const U4 r = rng.next();
      u = rng.uniform53(r.x, r.y);
    }
    if (!(exp(h0 - h1) < u)) {
      ++nacc;
      for (int c = 0; c < nc; ++c) x0[c] = q[c * ss];
    }
    if (istep >= a.ntherm) {
      if (idecor % a.ndecor == 0 && a.samples && isnap < a.nsnap) {
        double* o = a.samples + (isnap * a.nwalkers + w) * nc;
        for (int c = 0; c < nc; ++c) o[c] = x0[c];
        ++isnap;
      }
      ++idecor;
    }
  }
  if (a.accepted) a.accepted[w] += nacc;
}

}  // namespace qmc

using namespace qmc;

extern "C" {

int64_t qmc_drift_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  if (check_desc(d) != QMC_OK || nw < 0) return -1;
  return drift_layout(*d).total * pad_walkers(nw) * (int64_t)sizeof(double);
}

int qmc_drift_run(const qmc_wf_desc* d0, const qmc_drift_args* a, void* scratch,
                  int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  if (!a) return QMC_ERR_ARG;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;  // the drift sampler is FP64
  const qmc_wf_desc* d = &dd;
  if (a->nwalkers < 0 || a->nstep < 0 || a->ntherm < 0 || a->ndecor < 1 || a->nsnap < 0 ||
      !(a->step_size > 0.0))
    return QMC_ERR_ARG;
  const int nrep = (a->electron_index != nullptr) + (a->normals != nullptr) +
                   (a->uniforms != nullptr);
  if (nrep != 0 && nrep != 3) return QMC_ERR_ARG;  // replay needs all three inputs
  if (a->nwalkers == 0 || a->nstep == 0) return QMC_OK;
  if (!a->pos || !scratch) return QMC_ERR_ARG;
  if (a->nsnap > 0 && !a->samples) return QMC_ERR_ARG;
  if (scratch_bytes < qmc_drift_scratch_bytes(d, a->nwalkers)) return QMC_ERR_SCRATCH;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = tables_smem_bytes<double>(*d, ncol);
  if ((st = prepare_smem(drift_kernel, smem))) return st;
  const dim3 grid((unsigned)((a->nwalkers + kDriftTPB - 1) / kDriftTPB));
  const double sd = sqrt(sqrt(a->step_size));  // covariance sqrt(step) I
  drift_kernel<<<grid, kDriftTPB, smem, (cudaStream_t)stream>>>(
      dd, *a, (double*)scratch, pad_walkers(a->nwalkers), sd);
  return launch_status();
}

int64_t qmc_hmc_scratch_bytes(const qmc_wf_desc* d, int64_t nw) {
  return qmc_drift_scratch_bytes(d, nw);
}

int qmc_hmc_run(const qmc_wf_desc* d0, const qmc_hmc_args* a, void* scratch,
                int64_t scratch_bytes, void* stream) {
  int st = check_desc(d0);
  if (st) return st;
  if (!a) return QMC_ERR_ARG;
  qmc_wf_desc dd = *d0;
  dd.precision = QMC_PREC_FP64;  // the HMC sampler is FP64
  const qmc_wf_desc* d = &dd;
  if (a->nwalkers < 0 || a->nstep < 0 || a->ntherm < 0 || a->ndecor < 1 || a->nsnap < 0 ||
      a->traj_length < 1 || !(a->step_size > 0.0))
    return QMC_ERR_ARG;
  if ((a->momenta != nullptr) != (a->uniforms != nullptr)) return QMC_ERR_ARG;
  if (a->nwalkers == 0 || a->nstep == 0) return QMC_OK;
  if (!a->pos || !scratch) return QMC_ERR_ARG;
  if (a->nsnap > 0 && !a->samples) return QMC_ERR_ARG;
  if (scratch_bytes < qmc_hmc_scratch_bytes(d, a->nwalkers)) return QMC_ERR_SCRATCH;
  const int ncol = round_up(d->nmo_used, 8);
  const int64_t smem = tables_smem_bytes<double>(*d, ncol);
  if ((st = prepare_smem(hmc_kernel, smem))) return st;
  const dim3 grid((unsigned)((a->nwalkers + kDriftTPB - 1) / kDriftTPB));
  hmc_kernel<<<grid, kDriftTPB, smem, (cudaStream_t)stream>>>(dd, *a, (double*)scratch,
                                                               pad_walkers(a->nwalkers));
  return launch_status();
}

}  // extern "C"
