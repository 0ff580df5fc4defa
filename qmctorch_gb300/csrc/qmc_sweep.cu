// Single-electron Metropolis moves of a single-determinant Slater-Jastrow
// wave function with Sherman-Morrison updates (one warp per walker chain).
//
// The reference evaluates the full wave function for every single-electron
// proposal (Metropolis.move / __call__, metropolis.py:85-177, 227-254). For a
// single Slater determinant per spin the density ratio of moving electron l of
// spin s from r to r' is
//   psi(R')^2 / psi(R)^2 = (phi(r')^T A_s^-1 e_l)^2 * exp(2 dU),
//   dU = sum_{j != e} K(|r' - r_j|) - K(|r - r_j|),
// with A_s[l][k] = phi_k(r_l) and K the Pade kernel, so a move costs one AO
// row, one MO row and O(n^2) work instead of a full evaluation. After an
// accepted move A_s^-1 is updated by the rank-1 Sherman-Morrison formula
//   A'^-1 = A^-1 - (A^-1 e_l) (y - e_l)^T / y_l,   y = phi(r')^T A^-1,
// and every nelec moves it is rebuilt from scratch (warp Gauss-Jordan with
// partial pivoting) so that rounding does not accumulate. The proposals,
// uniforms and electron indices are the generic Metropolis kernel's (same
// counters), so both kernels take the same decisions up to the rounding of
// the ratio.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_ep.cuh"
#include "qmc_host.cuh"
#include "qmc_rng.cuh"

namespace qmc {

struct SweepShape {
  int nww;       // walkers (one warp each) per block
  int nthreads;  // 32 * nww
  int ncol;      // W columns kept in shared memory (orbitals < nmax, zero padded)
  int n[2];      // electrons per spin
  int ld[2];     // row stride of A_s^-1 (odd: conflict-free column access)
  int nmax, ldm; // Gauss-Jordan work matrix
  int64_t o_tab, o_gpatom, o_meta, o_aoord, o_wt, o_warp, warp_bytes, smem;
  int64_t o_p, o_v[2], o_m, o_ao, o_phi, o_y, o_col, o_e, o_d;
};

inline int64_t align16(int64_t n) { return (n + 15) & ~int64_t(15); }

// Row stride (entries) of the transposed MO coefficients WT: 16 bytes past a
// multiple of 128, so that 16-byte loads of consecutive rows hit distinct banks.
template <typename R>
__host__ __device__ inline int wt_ld(int nao) {
  const int bytes = ((pad4(nao) * (int)sizeof(R) + 127) / 128) * 128 + 16;
  return bytes / (int)sizeof(R);
}

template <typename R>
inline SweepShape sweep_shape(const qmc_wf_desc& d, int nww, int jc) {
  SweepShape s;
  s.nww = nww;
  s.nthreads = 32 * nww;
  s.n[0] = d.nup;
  s.n[1] = d.ndown;
  s.nmax = d.nup > d.ndown ? d.nup : d.ndown;
  s.ld[0] = d.nup | 1;
  s.ld[1] = d.ndown | 1;
  s.ldm = s.nmax | 1;
  s.ncol = round_up(s.nmax > 0 ? s.nmax : 1, jc);  // whole JC-column chunks
  const int64_t rs = sizeof(R);
  s.o_tab = 0;
  s.o_gpatom = align16(tables_smem_bytes<R>(d, s.ncol));
  s.o_meta = s.o_gpatom + align16((int64_t)d.ngprim * 4);
  s.o_aoord = s.o_meta + align16((int64_t)d.nao * 16);
  s.o_wt = s.o_aoord + align16((int64_t)round_up(d.nao, 32) * 4);
  s.o_warp = s.o_wt + align16((int64_t)s.nmax * wt_ld<R>(d.nao) * rs);
  int64_t q = 0;
  s.o_p = q;
  q += align16(3 * (int64_t)d.nelec * (int64_t)sizeof(XP<R>));
  for (int k = 0; k < 2; ++k) {
    s.o_v[k] = q;
    q += align16((int64_t)s.n[k] * s.ld[k] * rs);
  }
  s.o_m = q;
  q += align16((int64_t)s.nmax * s.ldm * rs);
  s.o_ao = q;
  q += align16((int64_t)pad4(d.nao) * rs);
  s.o_phi = q;
  q += align16((int64_t)s.nmax * rs);
  s.o_y = q;
  q += align16((int64_t)s.nmax * rs);
  s.o_col = q;
  q += align16((int64_t)s.nmax * rs);
  s.o_e = q;
  q += align16((int64_t)d.ngprim * rs);
  s.o_d = q;
  q += align16((int64_t)d.natom * 4 * rs);
  s.warp_bytes = q;
  s.smem = s.o_warp + (int64_t)nww * q;
  return s;
}

constexpr unsigned kFull = 0xffffffffu;

// Per-block tables of the single-electron AO and MO rows:
// * gp_atom4[i] = 4 x atom of group primitive i (offset into D);
// * meta[a] = {4 x atom, p0 | np << 16, weight offset, kx | ky << 8 | kz << 16
//   | split << 24} of AO a, read with one 16-byte load;
// * ao_ord: the order in which the lanes take the AOs (ranked by primitive
//   count, dealt in a snake order so that the lanes holding the longest sums
//   in one round get the shortest in the next), -1 = none;
// * WT[j][a] = W[a][j] for j < nmax, rows of ldt entries (16 bytes past a
//   multiple of 128: conflict-free 16-byte loads), zero past nao.
struct AORowTabs {
  const int* gp_atom4;  // [ngprim]
  const int4* meta;     // [nao]
  const int* ao_ord;    // [round_up(nao, 32)]
};

template <typename R>
__device__ inline AORowTabs build_ao_row_tabs(const Tables<R>& t, int nmax, int* gp_atom4,
                                              int4* meta, int* ao_ord, R* WT) {
  const int tid = threadIdx.x, nt = blockDim.x, nslot = round_up(t.nao, 32);
  for (int g = tid; g < t.ngroup; g += nt) {
    const int p0 = t.group_prim[g], np = t.group_prim[g + 1] - p0, A4 = 4 * t.group_atom[g];
    for (int p = p0; p < p0 + np; ++p) gp_atom4[p] = A4;
    for (int a = t.group_ao[g]; a < t.group_ao[g + 1]; ++a)
      meta[a] = make_int4(A4, p0 | (np << 16), t.ao_wofs[a],
                          t.ao_k[3 * a] | (t.ao_k[3 * a + 1] << 8) | (t.ao_k[3 * a + 2] << 16) |
                              (t.group_split[g] << 24));
  }
  for (int i = tid; i < nslot; i += nt) ao_ord[i] = -1;
  const int ldt = wt_ld<R>(t.nao);
  for (int i = tid; i < nmax * ldt; i += nt) {
    const int j = i / ldt, a = i - j * ldt;
    WT[i] = a < t.nao ? t.W[a * t.ncol + j] : (R)0;
  }
  __syncthreads();
  auto np = [&](int a) { return meta[a].y >> 16; };
  for (int a = tid; a < t.nao; a += nt) {
    const int c = np(a);
    int r = 0;
    for (int b = 0; b < t.nao; ++b) {
      const int cb = np(b);
      r += (cb > c) || (cb == c && b < a);
    }
    const int round = r >> 5, pos = r & 31;
    ao_ord[32 * round + ((round & 1) ? 31 - pos : pos)] = a;
  }
  __syncthreads();
  return AORowTabs{gp_atom4, meta, ao_ord};
}

// 16-byte aligned groups of four values (AO rows and WT rows are padded).
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x;
  v[1] = q.y;
  v[2] = q.z;
  v[3] = q.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 q0 = *reinterpret_cast<const double2*>(p);
  const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
  v[0] = q0.x;
  v[1] = q0.y;
  v[2] = q1.x;
  v[3] = q1.y;
}

// AO values of one electron at (ex, ey, ez) into AO[0..nao) in three
// warp-uniform phases: electron-atom differences (D[4A..4A+3] = dx, dy, dz,
// r^2), one exp per group primitive (E), then per AO its polynomial times
// sum_p w_p E_p. The plain method skips exps with alpha r^2 > kRadialCut.
template <typename R>
__device__ inline void warp_ao_row(const Tables<R>& t, const AORowTabs& x, XP<R> ex, XP<R> ey,
                                   XP<R> ez, R* E, R* D, R* AO, int lane) {
  for (int A = lane; A < t.natom; A += 32) {
    const R dx = dif(ex, t.atom_p[3 * A]), dy = dif(ey, t.atom_p[3 * A + 1]),
            dz = dif(ez, t.atom_p[3 * A + 2]);
    D[4 * A] = dx;
    D[4 * A + 1] = dy;
    D[4 * A + 2] = dz;
    D[4 * A + 3] = dx * dx + dy * dy + dz * dz;
  }
  __syncwarp();
  const int ngp = t.group_prim[t.ngroup];
  for (int i = lane; i < ngp; i += 32) {
    const R ar = t.alpha[i] * D[x.gp_atom4[i] + 3];
    E[i] = (!kMixed<R> && ar > (R)kRadialCut) ? (R)0 : rexp(-ar);
  }
  __syncwarp();
  const int nslot = round_up(t.nao, 32);
  for (int k = lane; k < nslot; k += 32) {
    const int a = x.ao_ord[k];
    if (a < 0) continue;
    const int4 m = x.meta[a];
    R dd[4];
    ld4(D + m.x, dd);
    const int p0 = m.y & 0xffff, np = m.y >> 16;
    const R* wp = t.wd + m.z;
    R G = (R)0;
    if (!(m.w >> 24)) {
      const R* ep = E + p0;
      for (int p = 0; p < np; ++p) G = fma(wp[p], ep[p], G);
    } else {  // components with their own exponents
      const R* ap = t.walpha + m.z;
      for (int p = 0; p < np; ++p) G = fma(wp[p], rexp(-ap[p] * dd[3]), G);
    }
    const R P = pk0(dd[0], m.w & 0xff) * pk0(dd[1], (m.w >> 8) & 0xff) *
                pk0(dd[2], (m.w >> 16) & 0xff);
    AO[a] = (t.vscale ? t.vscale[a] : (R)1) * (P * G);
  }
  __syncwarp();
}

// out[j] = sum_a AO[a] WT[j][a] for j < n (lane j; 16-byte loads, four
// partial sums; AO and WT rows zero-padded to a multiple of four).
template <typename R>
__device__ inline void warp_mo_row_t(const R* WT, int ldt, int na4, const R* AO, int n, R* out,
                                     int lane) {
  for (int j = lane; j < n; j += 32) {
    const R* wr = WT + j * ldt;
    R s0 = (R)0, s1 = (R)0, s2 = (R)0, s3 = (R)0;
    for (int a = 0; a < na4; a += 4) {
      R v[4], w[4];
      ld4(AO + a, v);
      ld4(wr + a, w);
      s0 = fma(v[0], w[0], s0);
      s1 = fma(v[1], w[1], s1);
      s2 = fma(v[2], w[2], s2);
      s3 = fma(v[3], w[3], s3);
    }
    out[j] = (s0 + s1) + (s2 + s3);
  }
  __syncwarp();
}

// Rows of the Slater matrix of spin s: lane l evaluates electron s*nup + l
// (all its AOs, in registers) and writes M[l][0..n) in chunks of JC columns.
template <typename R, int JC>
__device__ inline void lane_slater_rows(const Tables<R>& t, const XP<R>* P, int e0, int n, R* M,
                                        int ldm, int lane) {
  for (int l = lane; l < n; l += 32) {
    const int e = e0 + l;
    const XP<R> ex = P[3 * e], ey = P[3 * e + 1], ez = P[3 * e + 2];
    for (int j0 = 0; j0 < n; j0 += JC) {
      R acc[JC];
#pragma unroll
      for (int jj = 0; jj < JC; ++jj) acc[jj] = (R)0;
      auto add = [&](int a, const AOVal<R>& o) {
        R wv[JC];
        load_w<JC>(t.W + (int64_t)a * t.ncol + j0, wv);
#pragma unroll
        for (int jj = 0; jj < JC; ++jj) acc[jj] = fma(o.v, wv[jj], acc[jj]);
      };
      for_each_ao_ep<R, false>(t, ex, ey, ez, add);
#pragma unroll
      for (int jj = 0; jj < JC; ++jj)
        if (j0 + jj < n) M[l * ldm + j0 + jj] = acc[jj];
    }
  }
  __syncwarp();
}

// V = M^-1 (n x n, row strides ldm / ldv) by Gauss-Jordan elimination with
// partial pivoting; M is destroyed. Lane i owns rows i, i + 32, ...
template <typename R>
__device__ inline void warp_inverse(R* M, int ldm, R* V, int ldv, int n, int lane) {
  for (int i = lane; i < n; i += 32)
    for (int j = 0; j < n; ++j) V[i * ldv + j] = (i == j) ? (R)1 : (R)0;
  __syncwarp();
  for (int p = 0; p < n; ++p) {
    R best = (R)-1;
    int bi = p;
    for (int i = p + lane; i < n; i += 32) {
      const R v = fabs(M[i * ldm + p]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const R ob = __shfl_xor_sync(kFull, best, off);
      const int oi = __shfl_xor_sync(kFull, bi, off);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (bi != p) {
      for (int j = lane; j < n; j += 32) {
        const R m0 = M[p * ldm + j], v0 = V[p * ldv + j];
        M[p * ldm + j] = M[bi * ldm + j];
        V[p * ldv + j] = V[bi * ldv + j];
        M[bi * ldm + j] = m0;
        V[bi * ldv + j] = v0;
      }
      __syncwarp();
    }
    const R inv = (R)1 / M[p * ldm + p];
    __syncwarp();
    for (int j = lane; j < n; j += 32) {
      M[p * ldm + j] *= inv;
      V[p * ldv + j] *= inv;
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
      if (i == p) continue;
      const R f = M[i * ldm + p];
      if (f == (R)0) continue;
      for (int j = p; j < n; ++j) M[i * ldm + j] = fma(-f, M[p * ldm + j], M[i * ldm + j]);
      for (int j = 0; j < n; ++j) V[i * ldv + j] = fma(-f, V[p * ldv + j], V[i * ldv + j]);
    }
    __syncwarp();
  }
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(kFull, v, off);
  return v;
}

// One block = nww walker chains, one warp each; the warps share only the
// basis / MO tables and never wait for one another after loading them.
template <typename R, int JC>
__global__ void __launch_bounds__(256, kMixed<R> ? 3 : 2)
    sweep_kernel(const qmc_wf_desc d, const qmc_metropolis_args a, const SweepShape S) {
  extern __shared__ __align__(16) unsigned char smem[];
  const Tables<R> t = load_tables<R>(d, S.nmax, S.ncol, smem + S.o_tab);
  R* const WT = reinterpret_cast<R*>(smem + S.o_wt);
  const AORowTabs xt = build_ao_row_tabs<R>(t, S.nmax, reinterpret_cast<int*>(smem + S.o_gpatom),
                                            reinterpret_cast<int4*>(smem + S.o_meta),
                                            reinterpret_cast<int*>(smem + S.o_aoord), WT);
  const int ldt = wt_ld<R>(d.nao), na4 = pad4(d.nao);
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t nw = a.nwalkers;
  const int64_t w = (int64_t)blockIdx.x * S.nww + wib;
  if (w >= nw) return;  // whole warps only: no block barrier follows
  unsigned char* base = smem + S.o_warp + (int64_t)wib * S.warp_bytes;
  XP<R>* P = reinterpret_cast<XP<R>*>(base + S.o_p);
  R* const V0 = reinterpret_cast<R*>(base + S.o_v[0]);
  R* const V1 = reinterpret_cast<R*>(base + S.o_v[1]);
  R* M = reinterpret_cast<R*>(base + S.o_m);
  R* AO = reinterpret_cast<R*>(base + S.o_ao);
  R* PHI = reinterpret_cast<R*>(base + S.o_phi);
  R* Y = reinterpret_cast<R*>(base + S.o_y);
  R* COL = reinterpret_cast<R*>(base + S.o_col);
  R* E = reinterpret_cast<R*>(base + S.o_e);
  R* D = reinterpret_cast<R*>(base + S.o_d);
  const int ne = d.nelec, nc = 3 * ne, nup = d.nup;
  for (int i = lane; i < nc; i += 32) P[i] = split_xp<R>(a.pos[w * nc + i]);
  for (int i = d.nao + lane; i < pad4(d.nao); i += 32) AO[i] = (R)0;
  __syncwarp();

  auto rebuild = [&]() {
    for (int s = 0; s < 2; ++s) {
      const int n = s ? S.n[1] : S.n[0];
      if (n == 0) continue;
      lane_slater_rows<R, JC>(t, P, s * nup, n, M, S.ldm, lane);
      warp_inverse<R>(M, S.ldm, s ? V1 : V0, s ? S.ld[1] : S.ld[0], n, lane);
    }
  };
  rebuild();

  const R wj = d.use_jastrow ? (R)__ldg(d.jastrow_w) : (R)0;
  const bool ci_zero = __ldg(d.ci_weight) == 0.0;  // psi = 0: the reference accepts every move
  const double sigma = a.step_size / (2.0 * sqrt(2.0 * log(2.0)));
  const double sd = sqrt(sigma);
  Rng rng{(uint32_t)a.seed, (uint32_t)(a.seed >> 32), (uint32_t)w, 0, 0};
  const int nmove = a.move_type == QMC_MOVE_ALL_ELEC_ITER ? ne : 1;
  int nacc = 0, since_rebuild = 0;
  int64_t isnap = 0, idecor = 0;
  // Generated random numbers are drawn 32 moves at a time, lane k holding
  // those of move base + k (moves of one step for all-elec-iter, steps for
  // one-elec), and broadcast when the move comes.
  R bz[3] = {(R)0, (R)0, (R)0};
  double bu = 0.0;
  int be = 0;
  const bool iter = a.move_type == QMC_MOVE_ALL_ELEC_ITER;
  for (int istep = 0; istep < a.nstep; ++istep) {
    rng.step = a.step_offset + istep;
    for (int im = 0; im < nmove; ++im) {
      if (since_rebuild >= ne) {
        rebuild();
        since_rebuild = 0;
      }
      ++since_rebuild;
      const int slot = (iter ? im : istep) & 31;
      if (!a.proposals && slot == 0) {
        Rng r = rng;
        int jm = im;
        if (iter) {
          jm = im + lane;
        } else {
          r.step = a.step_offset + istep + lane;
        }
        const uint32_t c0 = (uint32_t)jm * (uint32_t)(ne + 2);
        be = iter ? jm : electron_draw(r, c0 + ne + 1, ne);
        draw_displacement<R>(r, c0 + be, a.proba, a.step_size, sd, bz);
        bu = accept_uniform(r, c0 + ne);
      }
      XP<R> pn[3];
      double u;
      int e;
      if (a.proposals) {
        e = iter ? im : a.electron_index[(int64_t)istep * nw + w];
        const int64_t mv = ((int64_t)istep * nmove + im) * nw + w;
        replay_displacement<R>(a.proposals + mv * 3, P + 3 * e, pn);
        u = a.uniforms[mv];
      } else {
        e = __shfl_sync(kFull, be, slot);
        u = __shfl_sync(kFull, bu, slot);
        for (int q = 0; q < 3; ++q) pn[q] = xp_add<R>(P[3 * e + q], __shfl_sync(kFull, bz[q], slot));
      }
      const int s = e < nup ? 0 : 1, l = e - s * nup;
      const int n = s ? S.n[1] : S.n[0], ld = s ? S.ld[1] : S.ld[0];
      R* const Vs = s ? V1 : V0;
      // determinant ratio y_l, y = phi(r')^T A^-1
      warp_ao_row<R>(t, xt, pn[0], pn[1], pn[2], E, D, AO, lane);
      warp_mo_row_t<R>(WT, ldt, na4, AO, n, PHI, lane);
      for (int j = lane; j < n; j += 32) {
        R y = (R)0;
        for (int k = 0; k < n; ++k) y = fma(PHI[k], Vs[k * ld + j], y);
        Y[j] = y;
      }
      // Jastrow: change of the Pade sum of electron e's pairs
      R du = (R)0;
      if (d.use_jastrow) {
        const XP<R> ox = P[3 * e], oy = P[3 * e + 1], oz = P[3 * e + 2];
        for (int j = lane; j < ne; j += 32) {
          if (j == e) continue;
          const R w0 = same_spin(d, e, j) ? (R)0.25 : (R)0.5;
          const XP<R> jx = P[3 * j], jy = P[3 * j + 1], jz = P[3 * j + 2];
          R dx = dif(pn[0], jx), dy = dif(pn[1], jy), dz = dif(pn[2], jz);
          const R rn = rsqrt_(dx * dx + dy * dy + dz * dz);
          dx = dif(ox, jx);
          dy = dif(oy, jy);
          dz = dif(oz, jz);
          const R ro = rsqrt_(dx * dx + dy * dy + dz * dz);
          du += w0 * rn / ((R)1 + wj * rn) - w0 * ro / ((R)1 + wj * ro);
        }
        du = warp_sum<R>(du);
      }
      // electron-nucleus Pade factor: change of electron e's row over the nuclei
      if (d.use_jastrow_en) {
        const XP<R> ox = P[3 * e], oy = P[3 * e + 1], oz = P[3 * e + 2];
        const R wn = (R)__ldg(d.jastrow_en_w);
        R dn = (R)0;
        for (int A = lane; A < t.natom; A += 32) {
          const XP<R> ax = t.en_p[3 * A], ay = t.en_p[3 * A + 1], az = t.en_p[3 * A + 2];
          R dx = dif(pn[0], ax), dy = dif(pn[1], ay), dz = dif(pn[2], az);
          const R rn = rsqrt_(dx * dx + dy * dy + dz * dz);
          dx = dif(ox, ax);
          dy = dif(oy, ay);
          dz = dif(oz, az);
          const R ro = rsqrt_(dx * dx + dy * dy + dz * dz);
          dn += rn / ((R)1 + wn * rn) - ro / ((R)1 + wn * ro);
        }
        du += warp_sum<R>(dn);
      }
      __syncwarp();
      const R ratio = Y[l];
      // accept (metropolis.py:141-160, 279-298): min(1, psi'^2 / psi^2) - u >= 0
      const double q = (double)ratio * (double)rexp(du);
      double df = ci_zero ? 1.0 : q * q;
      if (df > 1.0) df = 1.0;
      if (df - u >= 0.0) {
        ++nacc;
        for (int k = lane; k < n; k += 32) COL[k] = Vs[k * ld + l];
        __syncwarp();
        const R ir = (R)1 / ratio;
        for (int j = lane; j < n; j += 32) {
          const R yj = (Y[j] - (j == l ? (R)1 : (R)0)) * ir;
          for (int k = 0; k < n; ++k) Vs[k * ld + j] = fma(-COL[k], yj, Vs[k * ld + j]);
        }
        if (lane == 0) {
          P[3 * e] = pn[0];
          P[3 * e + 1] = pn[1];
          P[3 * e + 2] = pn[2];
        }
      }
      __syncwarp();
    }
    if (istep >= a.ntherm) {
      if (idecor % a.ndecor == 0) {
        if (a.samples && isnap < a.nsnap) {
          double* out = a.samples + (isnap * nw + w) * nc;
          for (int i = lane; i < nc; i += 32) out[i] = xp_value<R>(P[i]);
        }
        ++isnap;
      }
      ++idecor;
    }
  }
  for (int i = lane; i < nc; i += 32) a.pos[w * nc + i] = xp_value<R>(P[i]);
  if (lane == 0 && a.accepted) a.accepted[w] += nacc;
}

// Walkers per block: the count that keeps the most warps resident per SM
// (CUDA occupancy calculator), preferring larger blocks on ties.
template <typename R, int JC>
static int launch_sweep(const qmc_wf_desc* d, const qmc_metropolis_args* a, cudaStream_t st) {
  SweepShape best = sweep_shape<R>(*d, 1, JC);
  int best_warps = 0;
  for (int nww = 8; nww >= 1; nww /= 2) {
    const SweepShape s = sweep_shape<R>(*d, nww, JC);
    if (s.smem > 200 * 1024) continue;
    if (prepare_smem(sweep_kernel<R, JC>, s.smem) != QMC_OK) continue;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sweep_kernel<R, JC>, s.nthreads, s.smem) !=
        cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (occ * nww > best_warps) {
      best_warps = occ * nww;
      best = s;
    }
  }
  if (best_warps == 0) return QMC_ERR_SHAPE;
  int stt = prepare_smem(sweep_kernel<R, JC>, best.smem);
  if (stt) return stt;
  const dim3 grid((unsigned)((a->nwalkers + best.nww - 1) / best.nww));
  sweep_kernel<R, JC><<<grid, best.nthreads, best.smem, st>>>(*d, *a, best);
  return launch_status();
}

}  // namespace qmc

// Used by qmc_metropolis_run for one-elec and all-elec-iter moves of a single
// ground-state determinant (excitation recipe, one configuration, one
// determinant per spin).
int qmc_sweep_run(const qmc_wf_desc* d, const qmc_metropolis_args* a, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  const int nmax = d->nup > d->ndown ? d->nup : d->ndown;
  if (d->precision == QMC_PREC_MIXED) {
    if (nmax <= 8) return qmc::launch_sweep<float, 8>(d, a, s);
    if (nmax <= 16) return qmc::launch_sweep<float, 16>(d, a, s);
    return qmc::launch_sweep<float, 24>(d, a, s);
  }
  if (nmax <= 8) return qmc::launch_sweep<double, 8>(d, a, s);
  if (nmax <= 16) return qmc::launch_sweep<double, 16>(d, a, s);
  return qmc::launch_sweep<double, 24>(d, a, s);
}

bool qmc_sweep_eligible(const qmc_wf_desc* d, const qmc_metropolis_args* a) {
  return a->move_type != QMC_MOVE_ALL_ELEC && d->det_mode == QMC_DET_EXCITATION && d->ncfg == 1 &&
         d->radial_type == QMC_RADIAL_GTO &&
         d->ndet[0] == 1 && d->ndet[1] == 1 && !a->psi_out && d->nup <= QMC_MAX_NSPIN &&
         d->ndown <= QMC_MAX_NSPIN;
}
