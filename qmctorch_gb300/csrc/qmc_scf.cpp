// Gaussian integrals of the restricted Hartree-Fock calculator (host code).
//
// The reference obtains its molecular orbitals from pyscf (RHF on the basis,
// qmctorch/scf/calculator/pyscf.py:88-103). pyscf is not available where this
// package runs, so the SCF is done here on the basis functions exactly as the
// AO layer evaluates them: chi_mu = sum_{p in mu} w_p x^kx y^ky z^kz
// exp(-a_p |r - A_p|^2) with w_p = contraction coefficient x primitive norm.
//
// Method: McMurchie-Davidson. For a primitive pair (a on A, b on B) with
// p = a + b, P = (a A + b B) / p, the product expands in Hermite Gaussians
// with the 1D coefficients E_t^{ij} (per cartesian direction):
//   E_0^{00} = 1,
//   E_t^{i+1,j} = E_{t-1}^{ij} / (2p) + X_PA E_t^{ij} + (t + 1) E_{t+1}^{ij},
//   E_t^{i,j+1} = E_{t-1}^{ij} / (2p) + X_PB E_t^{ij} + (t + 1) E_{t+1}^{ij},
// times K_AB = exp(-a b / p |A - B|^2). Overlap (pi/p)^(3/2) E_0^x E_0^y E_0^z;
// kinetic energy from 1D overlaps s(i, j): t(i, j) = b (2j + 1) s(i, j)
// - 2 b^2 s(i, j + 2) - j (j - 1) / 2 s(i, j - 2); nuclear attraction
// -Z_C 2 pi / p sum_tuv E_t E_u E_v R_tuv(p, P - C); electron repulsion
// 2 pi^(5/2) / (p q sqrt(p + q)) sum_tuv E^ab_tuv sum_t'u'v' (-1)^(t'+u'+v')
// E^cd_t'u'v' R_{t+t',u+u',v+v'}(p q / (p + q), P - Q), with the Hermite
// integrals R^n_{000}(alpha, X) = (-2 alpha)^n F_n(alpha |X|^2) and
// R^n_{t+1,u,v} = t R^{n+1}_{t-1,u,v} + X_x R^{n+1}_{t,u,v} (likewise u, v).
// The Boys function F_n(T) = int_0^1 s^2n exp(-T s^2) ds is summed from its
// power series F_n(T) = exp(-T) sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
// for T < 40 and from its large-T limit (2n-1)!! / 2^(n+1) sqrt(pi / T^(2n+1))
// above (exp(-40) is below double precision), then recurred downwards,
// F_{n-1} = (2 T F_n + exp(-T)) / (2n - 1).
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>
#include <vector>

#include "../../include/qmc_gb300.h"

namespace {

constexpr int kMaxL = 2;                 // d functions
constexpr int kMaxE = 2 * kMaxL + 2;     // j + 2 for the kinetic energy
constexpr int kMaxHerm = 4 * kMaxL;      // t + u + v of an ERI
constexpr double kPi = 3.14159265358979323846;

void boys(int nmax, double T, double* F) {
  const double eT = std::exp(-T);
  if (T < 40.0) {
    double term = 1.0 / (2 * nmax + 1), sum = term;
    for (int k = 1; k < 400; ++k) {
      term *= 2.0 * T / (2 * nmax + 2 * k + 1);
      sum += term;
      if (term < 1e-17 * sum) break;
    }
    F[nmax] = eT * sum;
  } else {
    double df = 1.0;  // (2n - 1)!!
    for (int i = 1; i <= nmax; ++i) df *= (2 * i - 1);
    F[nmax] = df / std::pow(2.0, nmax + 1) * std::sqrt(kPi / std::pow(T, 2 * nmax + 1));
  }
  for (int n = nmax; n > 0; --n) F[n - 1] = (2.0 * T * F[n] + eT) / (2 * n - 1);
}

// 1D Hermite expansion coefficients E[i][j][t] for i <= imax, j <= jmax.
struct E1 {
  double e[kMaxL + 1][kMaxE + 1][kMaxL + kMaxE + 2];
};

void hermite_e(int imax, int jmax, double p, double xpa, double xpb, E1& E) {
  const double h = 0.5 / p;
  for (int i = 0; i <= kMaxL; ++i)
    for (int j = 0; j <= kMaxE; ++j)
      for (int t = 0; t < kMaxL + kMaxE + 2; ++t) E.e[i][j][t] = 0.0;
  E.e[0][0][0] = 1.0;
  for (int i = 0; i <= imax; ++i) {
    if (i > 0)
      for (int t = 0; t <= i; ++t) {
        const int j = 0;
        double v = xpa * E.e[i - 1][j][t] + (t + 1) * E.e[i - 1][j][t + 1];
        if (t > 0) v += h * E.e[i - 1][j][t - 1];
        E.e[i][j][t] = v;
      }
    for (int j = 1; j <= jmax; ++j)
      for (int t = 0; t <= i + j; ++t) {
        double v = xpb * E.e[i][j - 1][t] + (t + 1) * E.e[i][j - 1][t + 1];
        if (t > 0) v += h * E.e[i][j - 1][t - 1];
        E.e[i][j][t] = v;
      }
  }
}

// R_tuv(alpha, X) for t + u + v <= L into R[(t * (L+1) + u) * (L+1) + v].
void hermite_r(int L, double alpha, const double X[3], std::vector<double>& R,
               std::vector<double>& work) {
  const int n1 = L + 1;
  double F[kMaxHerm + 1];
  boys(L, alpha * (X[0] * X[0] + X[1] * X[1] + X[2] * X[2]), F);
  // work[n][t][u][v], n <= L; every entry read was written at the order above
  if (work.size() < (size_t)n1 * n1 * n1 * n1) work.resize((size_t)n1 * n1 * n1 * n1);
  auto W = [&](int n, int t, int u, int v) -> double& {
    return work[(((size_t)n * n1 + t) * n1 + u) * n1 + v];
  };
  double m2a = 1.0;
  for (int n = 0; n <= L; ++n) {
    W(n, 0, 0, 0) = m2a * F[n];
    m2a *= -2.0 * alpha;
  }
  for (int n = L - 1; n >= 0; --n) {
    const int top = L - n;  // t + u + v reachable at this order
    for (int t = 0; t <= top; ++t)
      for (int u = 0; u <= top - t; ++u)
        for (int v = 0; v <= top - t - u; ++v) {
          if (t + u + v == 0) continue;
          double val;
          if (t > 0) {
            val = X[0] * W(n + 1, t - 1, u, v);
            if (t > 1) val += (t - 1) * W(n + 1, t - 2, u, v);
          } else if (u > 0) {
            val = X[1] * W(n + 1, t, u - 1, v);
            if (u > 1) val += (u - 1) * W(n + 1, t, u - 2, v);
          } else {
            val = X[2] * W(n + 1, t, u, v - 1);
            if (v > 1) val += (v - 1) * W(n + 1, t, u, v - 2);
          }
          W(n, t, u, v) = val;
        }
  }
  if (R.size() < (size_t)n1 * n1 * n1) R.resize((size_t)n1 * n1 * n1);
  for (int t = 0; t <= L; ++t)
    for (int u = 0; u <= L - t; ++u)
      for (int v = 0; v <= L - t - u; ++v) R[((size_t)t * n1 + u) * n1 + v] = W(0, t, u, v);
}

struct Prim {
  double a, w, A[3];
  int k[3], ao;
};

// A primitive pair of a pair of AOs: Hermite coefficients of the product.
struct PairData {
  double p, P[3], pref;  // pref = w_a w_b K_AB
  int L[3];              // Hermite orders per direction (ka + kb)
  std::vector<double> E;  // E[(t * (L1+1) + u) * (L2+1) + v]
};

}  // namespace

using qmc_gto = qmc_gto_basis;

static std::vector<Prim> prims_of(const qmc_gto* b) {
  std::vector<Prim> P(b->nprim);
  for (int i = 0; i < b->nprim; ++i) {
    P[i].a = b->prim_exp[i];
    P[i].w = b->prim_coef[i];
    for (int d = 0; d < 3; ++d) {
      P[i].A[d] = b->prim_center[3 * i + d];
      P[i].k[d] = b->prim_k[3 * i + d];
    }
    P[i].ao = b->prim_ao[i];
  }
  return P;
}

static int check_basis(const qmc_gto* b) {
  if (!b || b->nao < 1 || b->nprim < 1 || !b->prim_ao || !b->prim_center || !b->prim_exp ||
      !b->prim_coef || !b->prim_k)
    return QMC_ERR_ARG;
  for (int i = 0; i < b->nprim; ++i) {
    if (b->prim_ao[i] < 0 || b->prim_ao[i] >= b->nao || !(b->prim_exp[i] > 0.0))
      return QMC_ERR_ARG;
    for (int d = 0; d < 3; ++d)
      if (b->prim_k[3 * i + d] < 0 || b->prim_k[3 * i + d] > kMaxL) return QMC_ERR_SHAPE;
    if (b->prim_k[3 * i] + b->prim_k[3 * i + 1] + b->prim_k[3 * i + 2] > kMaxL)
      return QMC_ERR_SHAPE;
  }
  return QMC_OK;
}

static int nthreads_for(int64_t work) {
  const unsigned hc = std::thread::hardware_concurrency();
  int n = hc ? (int)hc : 4;
  if (work < 64) n = 1;
  return std::max(1, std::min(n, 64));
}

extern "C" {

int qmc_scf_one_electron(const qmc_gto_basis* b, int32_t natom, const double* atom_xyz,
                         const double* atom_z, double* S, double* T, double* V) {
  int st = check_basis(b);
  if (st) return st;
  if (natom < 0 || (natom > 0 && (!atom_xyz || !atom_z)) || !S || !T || !V) return QMC_ERR_ARG;
  const std::vector<Prim> P = prims_of(b);
  const int n = b->nao, np = b->nprim;
  std::fill(S, S + (size_t)n * n, 0.0);
  std::fill(T, T + (size_t)n * n, 0.0);
  std::fill(V, V + (size_t)n * n, 0.0);
  std::vector<double> R, work;
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) {
      const Prim& pa = P[i];
      const Prim& pb = P[j];
      const double p = pa.a + pb.a, mu = pa.a * pb.a / p;
      double Pc[3], ab2 = 0.0;
      E1 E[3];
      double s1[3], t1[3];
      for (int d = 0; d < 3; ++d) {
        Pc[d] = (pa.a * pa.A[d] + pb.a * pb.A[d]) / p;
        const double dab = pa.A[d] - pb.A[d];
        ab2 += dab * dab;
        hermite_e(pa.k[d], pb.k[d] + 2, p, Pc[d] - pa.A[d], Pc[d] - pb.A[d], E[d]);
        const int ka = pa.k[d], kb = pb.k[d];
        const double sq = std::sqrt(kPi / p);
        s1[d] = E[d].e[ka][kb][0] * sq;
        double tk = pb.a * (2 * kb + 1) * s1[d] - 2.0 * pb.a * pb.a * E[d].e[ka][kb + 2][0] * sq;
        if (kb >= 2) tk -= 0.5 * kb * (kb - 1) * E[d].e[ka][kb - 2][0] * sq;
        t1[d] = tk;
      }
      const double K = std::exp(-mu * ab2) * pa.w * pb.w;
      const size_t o = (size_t)pa.ao * n + pb.ao;
      S[o] += K * s1[0] * s1[1] * s1[2];
      T[o] += K * (t1[0] * s1[1] * s1[2] + s1[0] * t1[1] * s1[2] + s1[0] * s1[1] * t1[2]);
      const int Lx = pa.k[0] + pb.k[0], Ly = pa.k[1] + pb.k[1], Lz = pa.k[2] + pb.k[2];
      const int L = Lx + Ly + Lz, n1 = L + 1;
      double vsum = 0.0;
      for (int c = 0; c < natom; ++c) {
        const double X[3] = {Pc[0] - atom_xyz[3 * c], Pc[1] - atom_xyz[3 * c + 1],
                             Pc[2] - atom_xyz[3 * c + 2]};
        hermite_r(L, p, X, R, work);
        double acc = 0.0;
        for (int t = 0; t <= Lx; ++t)
          for (int u = 0; u <= Ly; ++u)
            for (int v = 0; v <= Lz; ++v)
              acc += E[0].e[pa.k[0]][pb.k[0]][t] * E[1].e[pa.k[1]][pb.k[1]][u] *
                     E[2].e[pa.k[2]][pb.k[2]][v] * R[((size_t)t * n1 + u) * n1 + v];
        vsum -= atom_z[c] * acc;
      }
      V[o] += K * 2.0 * kPi / p * vsum;
    }
  return QMC_OK;
}

int qmc_scf_eri(const qmc_gto_basis* b, double* eri) {
  int st = check_basis(b);
  if (st) return st;
  if (!eri) return QMC_ERR_ARG;
  const std::vector<Prim> P = prims_of(b);
  const int n = b->nao;
  // primitives of each AO
  std::vector<std::vector<int>> of(n);
  for (int i = 0; i < b->nprim; ++i) of[P[i].ao].push_back(i);
  // AO pairs mu >= nu with their primitive-pair Hermite data
  std::vector<std::pair<int, int>> pairs;
  for (int m = 0; m < n; ++m)
    for (int v = 0; v <= m; ++v) pairs.emplace_back(m, v);
  const int64_t npair = (int64_t)pairs.size();
  std::vector<std::vector<PairData>> pd(npair);
  for (int64_t ip = 0; ip < npair; ++ip) {
    for (int ia : of[pairs[ip].first])
      for (int ib : of[pairs[ip].second]) {
        const Prim& pa = P[ia];
        const Prim& pb = P[ib];
        PairData q;
        q.p = pa.a + pb.a;
        double ab2 = 0.0;
        E1 E[3];
        for (int d = 0; d < 3; ++d) {
          q.P[d] = (pa.a * pa.A[d] + pb.a * pb.A[d]) / q.p;
          const double dab = pa.A[d] - pb.A[d];
          ab2 += dab * dab;
          hermite_e(pa.k[d], pb.k[d], q.p, q.P[d] - pa.A[d], q.P[d] - pb.A[d], E[d]);
          q.L[d] = pa.k[d] + pb.k[d];
        }
        q.pref = pa.w * pb.w * std::exp(-pa.a * pb.a / q.p * ab2);
        if (std::fabs(q.pref) < 1e-300) continue;
        const int l1 = q.L[1] + 1, l2 = q.L[2] + 1;
        q.E.assign((size_t)(q.L[0] + 1) * l1 * l2, 0.0);
        for (int t = 0; t <= q.L[0]; ++t)
          for (int u = 0; u <= q.L[1]; ++u)
            for (int v = 0; v <= q.L[2]; ++v)
              q.E[((size_t)t * l1 + u) * l2 + v] = E[0].e[pa.k[0]][pb.k[0]][t] *
                                                   E[1].e[pa.k[1]][pb.k[1]][u] *
                                                   E[2].e[pa.k[2]][pb.k[2]][v];
        pd[ip].push_back(std::move(q));
      }
  }
  // (ab|cd) of two AO pairs
  auto quartet = [&](int64_t i1, int64_t i2, std::vector<double>& R,
                     std::vector<double>& work) -> double {
    double sum = 0.0;
    for (const PairData& x : pd[i1])
      for (const PairData& y : pd[i2]) {
        const double p = x.p, q = y.p, alpha = p * q / (p + q);
        const double X[3] = {x.P[0] - y.P[0], x.P[1] - y.P[1], x.P[2] - y.P[2]};
        const int Lx = x.L[0] + y.L[0], Ly = x.L[1] + y.L[1], Lz = x.L[2] + y.L[2];
        const int L = Lx + Ly + Lz, n1 = L + 1;
        hermite_r(L, alpha, X, R, work);
        const int a1 = x.L[1] + 1, a2 = x.L[2] + 1, b1 = y.L[1] + 1, b2 = y.L[2] + 1;
        double acc = 0.0;
        for (int t = 0; t <= x.L[0]; ++t)
          for (int u = 0; u <= x.L[1]; ++u)
            for (int v = 0; v <= x.L[2]; ++v) {
              const double ex = x.E[((size_t)t * a1 + u) * a2 + v];
              if (ex == 0.0) continue;
              double inner = 0.0;
              for (int t2 = 0; t2 <= y.L[0]; ++t2)
                for (int u2 = 0; u2 <= y.L[1]; ++u2)
                  for (int v2 = 0; v2 <= y.L[2]; ++v2) {
                    const double sgn = ((t2 + u2 + v2) & 1) ? -1.0 : 1.0;
                    inner += sgn * y.E[((size_t)t2 * b1 + u2) * b2 + v2] *
                             R[((size_t)(t + t2) * n1 + (u + u2)) * n1 + (v + v2)];
                  }
              acc += ex * inner;
            }
        sum += x.pref * y.pref * 2.0 * std::pow(kPi, 2.5) / (p * q * std::sqrt(p + q)) * acc;
      }
    return sum;
  };
  // Schwarz bounds sqrt((ab|ab)) per AO pair
  std::vector<double> Q(npair);
  {
    std::atomic<int64_t> next{0};
    const int nt = nthreads_for(npair);
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k)
      th.emplace_back([&]() {
        std::vector<double> R, work;
        for (int64_t i; (i = next.fetch_add(1)) < npair;)
          Q[i] = std::sqrt(std::fabs(quartet(i, i, R, work)));
      });
    for (auto& t : th) t.join();
  }
  std::fill(eri, eri + (size_t)n * n * n * n, 0.0);
  const size_t n2 = (size_t)n * n, n3 = n2 * n;
  std::atomic<int64_t> next{0};
  const int nt = nthreads_for(npair);
  std::vector<std::thread> th;
  for (int k = 0; k < nt; ++k)
    th.emplace_back([&]() {
      std::vector<double> R, work;
      for (int64_t i1; (i1 = next.fetch_add(1)) < npair;) {
        const int a = pairs[i1].first, bb = pairs[i1].second;
        for (int64_t i2 = 0; i2 <= i1; ++i2) {
          if (Q[i1] * Q[i2] < 1e-14) continue;
          const int c = pairs[i2].first, d = pairs[i2].second;
          const double v = quartet(i1, i2, R, work);
          const size_t idx[8] = {a * n3 + bb * n2 + c * n + d, bb * n3 + a * n2 + c * n + d,
                                 a * n3 + bb * n2 + d * n + c, bb * n3 + a * n2 + d * n + c,
                                 c * n3 + d * n2 + a * n + bb, d * n3 + c * n2 + a * n + bb,
                                 c * n3 + d * n2 + bb * n + a, d * n3 + c * n2 + bb * n + a};
          for (size_t x : idx) eri[x] = v;
        }
      }
    });
  for (auto& t : th) t.join();
  return QMC_OK;
}

}  // extern "C"
