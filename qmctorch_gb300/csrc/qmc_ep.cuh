// Electron-parallel evaluation of psi / E_L for a block of walkers.
//
// A block owns `nwb` walkers and runs nwb * nelec threads: thread t handles
// electron e = t / nwb of walker wl = t % nwb (with nwb = 32 one warp is one
// electron of 32 walkers, so control flow is warp-uniform). Phases, separated
// by block barriers that every thread reaches:
//   1. electron phase (all threads): the electron's Jastrow row, its Coulomb
//      terms and its MO row (plus the kinetic-operator row for E_L), written
//      to shared memory;
//   2. determinant phase (threads < 2 nwb): one thread per (walker, spin) runs
//      the LU / excitation / trace work of spin_channel on the shared-memory MO
//      rows, so both spins proceed in parallel;
//   3. combine phase (threads < nwb): CI sum, Jastrow factor, energies.
// Compared with one thread per walker this gives nelec times more threads
// (about 34 warps per SM for 16384 H2O walkers) to hide FP32 and L1 latency.
//
// Positions live in shared memory as split coordinates XP<R> (see
// qmc_device.cuh): FP64 values for the plain method, FP32 pairs h + l for the
// mixed method, so that every difference in the inner loops is FP32 work.
#pragma once

#include "qmc_device.cuh"

namespace qmc {

// Per-walker scratch: the determinant-phase work arrays of both spins. The
// relative determinant values are FP64 for the local energy and of the
// compute type for psi.
struct EPLayout {
  Region lu[2], x[2], y[2], x64[2], y64[2], rc[2], dv, ov;
  int64_t bytes_per_slot;
  int nmax, vmax, omax;
};

// The mixed local energy solves a spin channel in registers (el_channel_regs)
// for excitation expansions with at most 5 electrons and 2 virtual orbitals
// per spin (H2O cc-pVDZ with single_double(4,4): 5 and 2).
constexpr int kElRegMaxN = 5, kElRegNV = 2;
__host__ __device__ inline bool el_regs(const qmc_wf_desc& d) {
  if (d.precision != QMC_PREC_MIXED || d.det_mode != QMC_DET_EXCITATION) return false;
  for (int s = 0; s < 2; ++s) {
    const int n = s ? d.ndown : d.nup;
    if (n < 1 || n > kElRegMaxN || d.max_orb[s] - n > kElRegNV || d.max_orb[s] < n) return false;
  }
  return true;
}

__host__ __device__ inline EPLayout ep_layout(const qmc_wf_desc& d, int kind) {
  EPLayout L;
  const bool mixed = d.precision == QMC_PREC_MIXED;
  const int rsz = mixed ? 4 : 8;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  int vmax = 0, omax = nmax;
  if (d.det_mode == QMC_DET_EXCITATION) {
    const int v0 = d.max_orb[0] - d.nup, v1 = d.max_orb[1] - d.ndown;
    vmax = v0 > v1 ? v0 : v1;
    omax = d.max_orb[0] > d.max_orb[1] ? d.max_orb[0] : d.max_orb[1];
  }
  L.nmax = nmax;
  L.vmax = vmax;
  L.omax = omax;
  int64_t o = 0;
  auto add = [&](Region& r, int64_t count, int esize) {
    r.off = o;
    r.esize = esize;
    o += count * esize;
    o = align8(o);
  };
  const bool el = kind == 1;
  // psi / Metropolis in excitation mode factor the Slater matrix in place in
  // the block's shared-memory MO rows (ep_det): no LU or A^-1 A_virt arrays;
  // the mixed local energy of small excitation expansions solves in
  // registers (el_channel_regs): only the determinant and trace values
  const bool inplace = (!el && d.det_mode == QMC_DET_EXCITATION) || (el && el_regs(d));
  const bool work = !inplace || !el;  // the E_L work arrays, unless in registers
  for (int s = 0; s < 2; ++s) {
    add(L.lu[s], inplace ? 0 : (int64_t)nmax * nmax, rsz);
    add(L.x[s], inplace ? 0 : (int64_t)nmax * vmax, rsz);
    add(L.y[s], (el && work) ? (int64_t)nmax * omax : 0, rsz);
    add(L.x64[s], (el && mixed && work) ? (int64_t)nmax * vmax : 0, 8);
    add(L.y64[s], (el && mixed && work) ? (int64_t)nmax * omax : 0, 8);
    add(L.rc[s], (el && mixed && work) ? nmax : 0, rsz);
  }
  add(L.dv, d.ndet[0] + d.ndet[1], el ? 8 : rsz);
  add(L.ov, el ? d.ndet[0] + d.ndet[1] : 0, 8);
  L.bytes_per_slot = o;
  return L;
}

// ---------------------------------------------------------------------------
// shared-memory and scratch layouts
// ---------------------------------------------------------------------------
constexpr int64_t kDetSmemBytes = 16384;

struct EPShape {
  int nwb;       // walkers per block
  int nslot;     // threads per walker in the electron phase (electron e on slot e % nslot)
  int nthreads;  // threads per block
  int ncol;      // W columns stored per AO (nmo_used rounded up to the MO chunk)
  int pstride;   // split coordinates per walker row of the position arrays: 3 nelec made
                 // odd, so that the 32 walkers of a warp read distinct banks
  int pos_global;  // Metropolis: the current positions live in the HBM scratch (after the
                   // determinant work arrays, [coordinate][walker]) instead of shared memory
  int64_t smem;  // dynamic shared memory bytes
  int64_t o_tab, o_pos, o_pnew, o_mo, o_bk, o_jrow, o_vrow, o_dref, o_psi, o_f, o_kin, o_v,
      o_iel, o_acc;
  int64_t o_det;  // determinant-phase work arrays of the block's walkers, or -1: HBM scratch
};

template <typename R>
__host__ __device__ inline EPShape ep_shape(const qmc_wf_desc& d, int kind, int nwb, int jc,
                                           int nslot, bool pos_global = false) {
  EPShape s;
  s.nwb = nwb;
  s.nslot = nslot;
  s.pos_global = (kind == 2 && pos_global) ? 1 : 0;
  int nt = nwb * nslot;
  if (nt < 2 * nwb) nt = 2 * nwb;
  s.nthreads = ((nt + 31) / 32) * 32;
  s.ncol = round_up(d.nmo_used, jc);
  const int64_t nc = 3 * (int64_t)d.nelec, nmu = d.nmo_used;
  const int64_t xps = 2 * (int64_t)sizeof(R);  // bytes of one split coordinate
  int64_t o = 0;
  s.o_tab = o;
  o += tables_smem_bytes<R>(d, s.ncol);
  o = (o + 15) & ~int64_t(15);
  s.pstride = (int)(nc | 1);
  s.o_pos = o;
  if (!s.pos_global) o += align8(nwb * s.pstride * xps);
  s.o_pnew = o;
  if (kind == 2) o += align8(nwb * s.pstride * xps);
  s.o_mo = o;
  o += align8(d.nelec * nmu * nwb * (int64_t)sizeof(R));
  s.o_bk = o;
  if (kind == 1) o += align8(d.nelec * nmu * nwb * (int64_t)sizeof(R));
  s.o_jrow = o;
  o += align8((int64_t)d.nelec * nwb * 8);
  s.o_vrow = o;
  if (kind == 1) o += align8((int64_t)d.nelec * nwb * 8);
  s.o_dref = o;
  o += 2 * nwb * 8;
  s.o_psi = o;
  o += nwb * 8;
  s.o_f = o;
  o += nwb * 8;
  s.o_kin = o;
  o += nwb * 8;
  s.o_v = o;
  o += nwb * 8;
  s.o_iel = o;
  o += align8(nwb * 4);
  s.o_acc = o;
  o += align8(nwb * 4);
  // the determinant phase works in shared memory when the block's arrays are
  // small (the psi / Metropolis kernels of small molecules), else in HBM scratch
  const int64_t det_bytes = (int64_t)nwb * ep_layout(d, kind == 1 ? 1 : 0).bytes_per_slot;
  if (det_bytes <= kDetSmemBytes) {
    o = (o + 15) & ~int64_t(15);
    s.o_det = o;
    o += det_bytes;
  } else {
    s.o_det = -1;
  }
  s.smem = o;
  return s;
}

// Thread bound of the electron-parallel kernels: 1024 threads (64 registers)
// for FP32, 512 (128 registers) for FP64, whose accumulators are twice as wide.
template <typename R>
struct EPBound {
  static constexpr int kThreads = kMixed<R> ? 1024 : 512;
};
// The FP32 local-energy kernel (electron phase with gradient and laplacian
// accumulators, determinant phase in registers) is bounded at 640 threads:
// 96 registers, and still 4 blocks of 32 x 5 threads per SM.
template <typename R>
struct EPElBound {
  static constexpr int kThreads = kMixed<R> ? 640 : 512;
};
template <typename R>
__host__ __device__ constexpr int ep_thread_bound(int kind) {
  return kind == 1 ? EPElBound<R>::kThreads : EPBound<R>::kThreads;
}


// ---------------------------------------------------------------------------
// AO groups
// ---------------------------------------------------------------------------
// Radial sums G_n = sum_p w_cp alpha_p^n exp(-alpha_p r^2) of NC components.
// CUT: skip primitives with alpha r^2 > kRadialCut (exp < 1e-20): the FP64
// electron-parallel kernels and the FP64 single-electron ratio; the mixed
// method evaluates every term (its FP32 exp is cheap and flushes far below).
constexpr float kRadialCut = 46.0f;

template <typename R, bool DERIV, int NC, bool CUT = false>
__device__ __forceinline__ void group_radial(const Tables<R>& t, int g, R r2, R (&G0)[NC],
                                             R (&G1)[NC], R (&G2)[NC]) {
  const int p0 = t.group_prim[g], np = t.group_prim[g + 1] - p0;
  const int wb = t.ao_wofs[t.group_ao[g]];  // weights of component c at wb + c * np
#pragma unroll
  for (int c = 0; c < NC; ++c) G0[c] = G1[c] = G2[c] = (R)0;
  if (!t.group_split[g]) {
    for (int p = 0; p < np; ++p) {
      const R al = t.alpha[p0 + p];
      if (CUT && al * r2 > (R)kRadialCut) continue;
      const R e0 = rexp(-al * r2);
      const R e1 = al * e0, e2 = al * e1;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const R w = t.wd[wb + c * np + p];
        G0[c] = fma(w, e0, G0[c]);
        if (DERIV) {
          G1[c] = fma(w, e1, G1[c]);
          G2[c] = fma(w, e2, G2[c]);
        }
      }
    }
  } else {
    // components with their own exponents
    for (int p = 0; p < np; ++p) {
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        const int wi = wb + c * np + p;
        const R al = t.walpha[wi];
        if (CUT && al * r2 > (R)kRadialCut) continue;
        const R e0 = rexp(-al * r2);
        const R w = t.wd[wi];
        G0[c] = fma(w, e0, G0[c]);
        if (DERIV) {
          G1[c] = fma(w, al * e0, G1[c]);
          G2[c] = fma(w, al * al * e0, G2[c]);
        }
      }
    }
  }
}

// AO from its polynomial P (gradient dP, laplacian lapP, degree l) and the
// radial sums: val = P G0, grad = dP G0 - 2 r P G1,
// lap = lapP G0 + P (4 r^2 G2 - (6 + 4 l) G1) (Euler: r . grad P = l P).
template <typename R, bool DERIV>
__device__ __forceinline__ AOVal<R> ao_from(R P, R px, R py, R pz, R lapP, int l, R dx, R dy, R dz,
                                            R r2, R g0, R g1, R g2, R vs) {
  AOVal<R> o;
  o.v = vs * (P * g0);
  if (DERIV) {
    const R pg1 = (R)(-2) * P * g1;
    o.gx = fma(px, g0, dx * pg1);
    o.gy = fma(py, g0, dy * pg1);
    o.gz = fma(pz, g0, dz * pg1);
    o.lap = vs * fma(lapP, g0, P * ((R)4 * r2 * g2 - (R)(6 + 4 * l) * g1));
  }
  return o;
}

// x^k, d/dx x^k, d2/dx2 x^k by selects (loops only for k > 2).
template <typename R>
__device__ __forceinline__ R pk0(R x, int k) {
  return k == 0 ? (R)1 : (k == 1 ? x : (k == 2 ? x * x : ipow(x, k)));
}
template <typename R>
__device__ __forceinline__ R pk1(R x, int k) {
  return k == 0 ? (R)0 : (k == 1 ? (R)1 : (k == 2 ? (R)2 * x : (R)k * ipow(x, k - 1)));
}
template <typename R>
__device__ __forceinline__ R pk2(R x, int k) {
  return k < 2 ? (R)0 : (k == 2 ? (R)2 : (R)(k * (k - 1)) * ipow(x, k - 2));
}

template <typename R, bool DERIV, int NC, typename F, bool CUT = false>
__device__ __forceinline__ void group_generic(const Tables<R>& t, int g, R dx, R dy, R dz, R r2,
                                              F& f) {
  R G0[NC], G1[NC], G2[NC];
  group_radial<R, DERIV, NC, CUT>(t, g, r2, G0, G1, G2);
  const int a0 = t.group_ao[g];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const int a = a0 + c;
    const int kx = t.ao_k[3 * a], ky = t.ao_k[3 * a + 1], kz = t.ao_k[3 * a + 2];
    const R px = pk0(dx, kx), py = pk0(dy, ky), pz = pk0(dz, kz);
    R qx = 0, qy = 0, qz = 0, lapP = 0;
    if (DERIV) {
      qx = pk1(dx, kx) * py * pz;
      qy = px * pk1(dy, ky) * pz;
      qz = px * py * pk1(dz, kz);
      lapP = pk2(dx, kx) * py * pz + px * pk2(dy, ky) * pz + px * py * pk2(dz, kz);
    }
    const R vs = t.vscale ? t.vscale[a] : (R)1;
    f(a, ao_from<R, DERIV>(px * py * pz, qx, qy, qz, lapP, kx + ky + kz, dx, dy, dz, r2, G0[c],
                           G1[c], G2[c], vs));
  }
}

template <typename R, bool DERIV, int NC, typename F, bool CUT = false>
__device__ __forceinline__ void group_s(const Tables<R>& t, int g, R dx, R dy, R dz, R r2, F& f) {
  R G0[NC], G1[NC], G2[NC];
  group_radial<R, DERIV, NC, CUT>(t, g, r2, G0, G1, G2);
  const int a0 = t.group_ao[g];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const R vs = t.vscale ? t.vscale[a0 + c] : (R)1;
    f(a0 + c, ao_from<R, DERIV>((R)1, (R)0, (R)0, (R)0, (R)0, 0, dx, dy, dz, r2, G0[c], G1[c],
                                G2[c], vs));
  }
}

template <typename R, bool DERIV, typename F, bool CUT = false>
__device__ __forceinline__ void group_p(const Tables<R>& t, int g, R dx, R dy, R dz, R r2, F& f) {
  R G0[3], G1[3], G2[3];
  group_radial<R, DERIV, 3, CUT>(t, g, r2, G0, G1, G2);
  const int a0 = t.group_ao[g];
  const R o = (R)0, i = (R)1;
  auto vs = [&](int c) { return t.vscale ? t.vscale[a0 + c] : (R)1; };
  f(a0, ao_from<R, DERIV>(dx, i, o, o, o, 1, dx, dy, dz, r2, G0[0], G1[0], G2[0], vs(0)));
  f(a0 + 1, ao_from<R, DERIV>(dy, o, i, o, o, 1, dx, dy, dz, r2, G0[1], G1[1], G2[1], vs(1)));
  f(a0 + 2, ao_from<R, DERIV>(dz, o, o, i, o, 1, dx, dy, dz, r2, G0[2], G1[2], G2[2], vs(2)));
}

// cartesian d shell, components xx, xy, xz, yy, yz, zz (pyscf.py:120-122)
template <typename R, bool DERIV, typename F, bool CUT = false>
__device__ __forceinline__ void group_d(const Tables<R>& t, int g, R dx, R dy, R dz, R r2, F& f) {
  R G0[6], G1[6], G2[6];
  group_radial<R, DERIV, 6, CUT>(t, g, r2, G0, G1, G2);
  const int a0 = t.group_ao[g];
  const R o = (R)0, two = (R)2;
  auto vs = [&](int c) { return t.vscale ? t.vscale[a0 + c] : (R)1; };
  f(a0, ao_from<R, DERIV>(dx * dx, two * dx, o, o, two, 2, dx, dy, dz, r2, G0[0], G1[0], G2[0],
                          vs(0)));
  f(a0 + 1, ao_from<R, DERIV>(dx * dy, dy, dx, o, o, 2, dx, dy, dz, r2, G0[1], G1[1], G2[1],
                              vs(1)));
  f(a0 + 2, ao_from<R, DERIV>(dx * dz, dz, o, dx, o, 2, dx, dy, dz, r2, G0[2], G1[2], G2[2],
                              vs(2)));
  f(a0 + 3, ao_from<R, DERIV>(dy * dy, o, two * dy, o, two, 2, dx, dy, dz, r2, G0[3], G1[3], G2[3],
                              vs(3)));
  f(a0 + 4, ao_from<R, DERIV>(dy * dz, o, dz, dy, o, 2, dx, dy, dz, r2, G0[4], G1[4], G2[4],
                              vs(4)));
  f(a0 + 5, ao_from<R, DERIV>(dz * dz, o, o, two * dz, two, 2, dx, dy, dz, r2, G0[5], G1[5], G2[5],
                              vs(5)));
}

// The AOs of group g at electron-atom difference (dx, dy, dz), r2 = |d|^2.
template <typename R, bool DERIV, typename F, bool CUT = false>
__device__ __forceinline__ void ao_group(const Tables<R>& t, int g, R dx, R dy, R dz, R r2, F& f) {
  const int nc = t.group_ao[g + 1] - t.group_ao[g];
  switch (t.group_kind[g]) {
    case GK_S:
      if (nc == 1) group_s<R, DERIV, 1, F, CUT>(t, g, dx, dy, dz, r2, f);
      else if (nc == 2) group_s<R, DERIV, 2, F, CUT>(t, g, dx, dy, dz, r2, f);
      else group_generic<R, DERIV, QMC_MAX_COMP, F, CUT>(t, g, dx, dy, dz, r2, f);
      break;
    case GK_P: group_p<R, DERIV, F, CUT>(t, g, dx, dy, dz, r2, f); break;
    case GK_D: group_d<R, DERIV, F, CUT>(t, g, dx, dy, dz, r2, f); break;
    default:
      switch (nc) {
        case 1: group_generic<R, DERIV, 1, F, CUT>(t, g, dx, dy, dz, r2, f); break;
        case 2: group_generic<R, DERIV, 2, F, CUT>(t, g, dx, dy, dz, r2, f); break;
        case 3: group_generic<R, DERIV, 3, F, CUT>(t, g, dx, dy, dz, r2, f); break;
        case 4: group_generic<R, DERIV, 4, F, CUT>(t, g, dx, dy, dz, r2, f); break;
        case 5: group_generic<R, DERIV, 5, F, CUT>(t, g, dx, dy, dz, r2, f); break;
        default: group_generic<R, DERIV, 6, F, CUT>(t, g, dx, dy, dz, r2, f); break;
      }
  }
}

// The Slater-type AOs of group g (each AO sums its own primitives).
template <typename R, bool DERIV, typename F>
__device__ __forceinline__ void group_sto(const Tables<R>& t, int g, R dx, R dy, R dz, R r2,
                                          F& f) {
  const int np = t.group_prim[g + 1] - t.group_prim[g];
  for (int a = t.group_ao[g]; a < t.group_ao[g + 1]; ++a) {
    const int kx = t.ao_k[3 * a], ky = t.ao_k[3 * a + 1], kz = t.ao_k[3 * a + 2];
    const R px = pk0(dx, kx), py = pk0(dy, ky), pz = pk0(dz, kz);
    R qx = 0, qy = 0, qz = 0, lapP = 0;
    if (DERIV) {
      qx = pk1(dx, kx) * py * pz;
      qy = px * pk1(dy, ky) * pz;
      qz = px * py * pk1(dz, kz);
      lapP = pk2(dx, kx) * py * pz + px * pk2(dy, ky) * pz + px * py * pk2(dz, kz);
    }
    const R vs = t.vscale ? t.vscale[a] : (R)1;
    AOVal<R> o{};
    for (int p = 0; p < np; ++p) {
      const int wi = t.ao_wofs[a] + p;
      const R wg = t.wd[wi];
      const AOVal<R> q = sto_from<R, DERIV>(px * py * pz, qx, qy, qz, lapP, kx + ky + kz, dx, dy,
                                            dz, r2, t.ao_kr(a), t.walpha[wi], vs * wg, wg);
      o.v += q.v;
      if (DERIV) {
        o.gx += q.gx;
        o.gy += q.gy;
        o.gz += q.gz;
        o.lap += q.lap;
      }
    }
    f(a, o);
  }
}

// All AOs of one electron (split coordinates ex, ey, ez); the electron-atom
// difference is formed once per atom (groups are stored atom by atom).
template <typename R, bool DERIV, typename F>
__device__ __forceinline__ void for_each_ao_ep(const Tables<R>& t, XP<R> ex, XP<R> ey, XP<R> ez,
                                               F& f) {
  int last = -1;
  R dx = 0, dy = 0, dz = 0, r2 = 0;
  const bool sto = t.radial != QMC_RADIAL_GTO;
  for (int g = 0; g < t.ngroup; ++g) {
    const int A = t.group_atom[g];
    if (A != last) {
      dx = dif(ex, t.atom_p[3 * A]);
      dy = dif(ey, t.atom_p[3 * A + 1]);
      dz = dif(ez, t.atom_p[3 * A + 2]);
      r2 = dx * dx + dy * dy + dz * dz;
      last = A;
    }
    // FP64: primitives with alpha r^2 > 46 (exp < 1e-20) are skipped, as a
    // zero contribution (the FP64 exp is the plain method's costliest
    // operation; long chains skip most of the far atoms' primitives)
    if (sto)
      group_sto<R, DERIV>(t, g, dx, dy, dz, r2, f);
    else
      ao_group<R, DERIV, F, !kMixed<R>>(t, g, dx, dy, dz, r2, f);
  }
}

// JC consecutive W values with vector loads (rows are 16-byte aligned and
// padded to a multiple of JC).
template <int JC>
__device__ __forceinline__ void load_w(const float* p, float (&w)[JC]) {
#pragma unroll
  for (int q = 0; q < JC / 4; ++q) {
    const float4 v = reinterpret_cast<const float4*>(p)[q];
    w[4 * q] = v.x;
    w[4 * q + 1] = v.y;
    w[4 * q + 2] = v.z;
    w[4 * q + 3] = v.w;
  }
}
template <int JC>
__device__ __forceinline__ void load_w(const double* p, double (&w)[JC]) {
#pragma unroll
  for (int q = 0; q < JC / 2; ++q) {
    const double2 v = reinterpret_cast<const double2*>(p)[q];
    w[2 * q] = v.x;
    w[2 * q + 1] = v.y;
  }
}

// ---------------------------------------------------------------------------
// phase 1: one electron of one walker
// ---------------------------------------------------------------------------
// pw: the walker's split coordinates (shared memory). mo / bk: element (e, j)
// of this walker at [(e * nmu + j) * nwb]. jrow: log J partial of this
// electron; vrow (E_L): its V_en plus half its V_ee row.
template <typename R, int JC, bool KIN>
__device__ inline void ep_electron(const qmc_wf_desc& d, const Tables<R>& t, const XP<R>* pw,
                                   int e, R* mo, R* bk, int nwb, double* jrow, double* vrow) {
  const int ne = d.nelec, nmu = d.nmo_used;
  const XP<R> ex = pw[3 * e], ey = pw[3 * e + 1], ez = pw[3 * e + 2];
  R gx = (R)0, gy = (R)0, gz = (R)0, jl = (R)0;
  {
    const R w = d.use_jastrow ? (R)__ldg(d.jastrow_w) : (R)0;
    R ks = (R)0, vs = (R)0, lp = (R)0;
    if (d.use_jastrow || KIN) {
      for (int j = KIN ? 0 : e + 1; j < ne; ++j) {
        if (j == e) continue;
        const R dx = dif(ex, pw[3 * j]), dy = dif(ey, pw[3 * j + 1]), dz = dif(ez, pw[3 * j + 2]);
        const R r = psqrt(dx * dx + dy * dy + dz * dz);
        if (KIN) vs += prcp(r);
        if (d.use_jastrow) {
          const R w0 = same_spin(d, e, j) ? (R)0.25 : (R)0.5;
          const R iu = prcp((R)1 + w * r);
          ks += w0 * r * iu;
          if (KIN) {
            const R ir = prcp(r);
            const R k1 = w0 * iu * iu;                       // dK/dr
            gx += k1 * dx * ir;
            gy += k1 * dy * ir;
            gz += k1 * dz * ir;
            lp += (R)2 * k1 * ir - (R)2 * w * k1 * iu;        // 2K'/r + K''
          }
        }
      }
    }
    // electron-nucleus Pade factor: K = r / (1 + w r) for every nucleus
    R kn = (R)0;
    if (d.use_jastrow_en) {
      const R wn = (R)__ldg(d.jastrow_en_w);
      for (int A = 0; A < t.natom; ++A) {
        const R dx = dif(ex, t.en_p[3 * A]), dy = dif(ey, t.en_p[3 * A + 1]),
                dz = dif(ez, t.en_p[3 * A + 2]);
        const R r = psqrt(dx * dx + dy * dy + dz * dz);
        const R iu = prcp((R)1 + wn * r);
        kn += r * iu;
        if (KIN) {
          const R ir = prcp(r);
          const R k1 = iu * iu;  // dK/dr
          gx += k1 * dx * ir;
          gy += k1 * dy * ir;
          gz += k1 * dz * ir;
          lp += (R)2 * k1 * ir - (R)2 * wn * k1 * iu;  // 2K'/r + K''
        }
      }
    }
    if (KIN) {
      jl = lp + gx * gx + gy * gy + gz * gz;  // lap(J)/J of this electron
      *jrow = 0.5 * (double)ks + (double)kn;  // e-e pairs visited from both ends
      R ven = (R)0;
      for (int A = 0; A < t.natom; ++A) {
        const R dx = dif(ex, t.atom_p[3 * A]), dy = dif(ey, t.atom_p[3 * A + 1]),
                dz = dif(ez, t.atom_p[3 * A + 2]);
        ven -= pdiv((R)t.atom_z[A], psqrt(dx * dx + dy * dy + dz * dz));
      }
      *vrow = 0.5 * (double)vs + (double)ven;
    } else {
      *jrow = (double)ks + (double)kn;
    }
  }
  const int64_t cs = nwb;
  R* mrow = mo + (int64_t)e * nmu * cs;
  R* brow = KIN ? bk + (int64_t)e * nmu * cs : nullptr;
  for (int j0 = 0; j0 < nmu; j0 += JC) {
    R a0[JC], ad[JC], al[JC];
#pragma unroll
    for (int jj = 0; jj < JC; ++jj) a0[jj] = ad[jj] = al[jj] = (R)0;
    auto acc = [&](int a, const AOVal<R>& o) {
      // FP64: an AO whose primitives were all cut (far atom) is zero with its
      // derivatives, and its FMAs would add zeros: skipped (the lanes of a warp
      // evaluate the same electron index of different walkers, so the branch
      // is mostly uniform)
      if constexpr (!kMixed<R>) {
        if (o.v == (R)0 && (!KIN || (o.gx == (R)0 && o.gy == (R)0 && o.gz == (R)0 &&
                                     o.lap == (R)0)))
          return;
      }
      R wv[JC];
      load_w<JC>(t.W + (int64_t)a * t.ncol + j0, wv);
      R gdot = (R)0;
      if (KIN) gdot = (R)2 * (gx * o.gx + gy * o.gy + gz * o.gz);
#pragma unroll
      for (int jj = 0; jj < JC; ++jj) {
        a0[jj] = fma(o.v, wv[jj], a0[jj]);
        if (KIN) {
          ad[jj] = fma(gdot, wv[jj], ad[jj]);
          al[jj] = fma(o.lap, wv[jj], al[jj]);
        }
      }
    };
    for_each_ao_ep<R, KIN>(t, ex, ey, ez, acc);
#pragma unroll
    for (int jj = 0; jj < JC; ++jj) {
      if (j0 + jj < nmu) {
        mrow[(j0 + jj) * cs] = a0[jj];
        if (KIN) brow[(j0 + jj) * cs] = (R)(-0.5) * (al[jj] + ad[jj] + jl * a0[jj]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// phases 2 and 3
// ---------------------------------------------------------------------------
// psi / Metropolis determinant phase of one (walker, spin) channel in
// excitation mode for n = N <= 8 occupied and nv <= kRegNV virtual columns:
// the spin's MO rows are loaded into registers once, factored (LU with partial
// pivoting) and A^-1 A_virt solved there -- the operations of lu_factor and
// lu_solve in the same order, so bitwise the same values -- and only
// A^-1 A_virt is written back (in place over the virtual columns) for the
// excitation determinants. Returns det(A) in FP64 (product of the pivots).
constexpr int kRegNV = 2;
// largest n of the register path: 5 under the 64-register bound of the FP32
// kernels (more spills); the FP64 kernel keeps the shared-memory LU (its
// register file is full with the FP64 electron phase: the register path
// measured 17 % slower there)
template <typename R>
constexpr int kRegMaxN = kMixed<R> ? 5 : 0;

template <typename R, int N>
__device__ inline double lu_solve_regs(R* rows, int64_t rs, int64_t cs, int nv) {
  constexpr int NC = N + kRegNV;
  R a[N][NC];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < NC; ++j) a[i][j] = (j < N + nv) ? rows[i * rs + j * cs] : (R)0;
  double det = 1.0;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    int p = k;
    R amax = fabs(a[k][k]);
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const R v = fabs(a[i][k]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    // row interchange: the occupied columns as lu_factor does at this step,
    // the virtual columns as lu_solve's pivot pass does afterwards (the same
    // transpositions in the same order)
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const bool sw = (i == p);
#pragma unroll
      for (int j = 0; j < NC; ++j) {
        const R x = a[k][j], y = a[i][j];
        a[k][j] = sw ? y : x;
        a[i][j] = sw ? x : y;
      }
    }
    if (p != k) det = -det;
    const R akk = a[k][k];
    det *= to_f64(akk);
    const R inv = akk != (R)0 ? (R)1 / akk : (R)0;
    a[k][k] = inv;
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const R l = a[i][k] * inv;
      a[i][k] = l;
#pragma unroll
      for (int j = k + 1; j < N; ++j) a[i][j] = fma(-l, a[k][j], a[i][j]);
    }
  }
#pragma unroll
  for (int c = 0; c < kRegNV; ++c) {
    if (c >= nv) break;
    const int j = N + c;
#pragma unroll
    for (int i = 1; i < N; ++i) {
      R s = a[i][j];
#pragma unroll
      for (int k = 0; k < i; ++k) s = fma(-a[i][k], a[k][j], s);
      a[i][j] = s;
    }
#pragma unroll
    for (int i = N - 1; i >= 0; --i) {
      R s = a[i][j];
#pragma unroll
      for (int k = i + 1; k < N; ++k) s = fma(-a[i][k], a[k][j], s);
      a[i][j] = s * a[i][i];
    }
#pragma unroll
    for (int i = 0; i < N; ++i) rows[i * rs + j * cs] = a[i][j];
  }
  return det;
}

// Dispatch of lu_solve_regs on n; false when n or nv is beyond the register path.
template <typename R>
__device__ inline bool lu_solve_regs_n(R* rows, int64_t rs, int64_t cs, int n, int nv,
                                       double* det) {
  if (nv > kRegNV || n > kRegMaxN<R>) return false;
  if constexpr (kRegMaxN<R> < 1) return false;
  switch (n) {
    case 1: *det = lu_solve_regs<R, 1>(rows, rs, cs, nv); return true;
    case 2: *det = lu_solve_regs<R, 2>(rows, rs, cs, nv); return true;
    case 3: *det = lu_solve_regs<R, 3>(rows, rs, cs, nv); return true;
    case 4: *det = lu_solve_regs<R, 4>(rows, rs, cs, nv); return true;
    case 5: *det = lu_solve_regs<R, 5>(rows, rs, cs, nv); return true;
    default: break;
  }
  return false;
}

// Excitation determinant values relative to det(A) (det_unique_single_double,
// slater_pooling.py:147-260) from X = A^-1 A_virt: 1 (ground state), X_ij
// (single), det of the 2 x 2 block of X (double).
template <typename R, typename T>
__device__ inline void excitation_values(const qmc_wf_desc& d, const int* tab, int spin,
                                         CView<R> X, int nv, T* dv, int64_t s) {
  const int nd = d.ndet[spin];
  for (int u = 0; u < nd; ++u) {
    const int ord = tab[5 * u];
    R v = (R)1;
    if (ord == 1) {
      const int i0 = tab[5 * u + 1];
      v = X(i0 / nv, i0 % nv);
    } else if (ord >= 2) {
      const int i0 = tab[5 * u + 1], i1 = tab[5 * u + 2];
      const int i2 = tab[5 * u + 3], i3 = tab[5 * u + 4];
      const R t00 = X(i0 / nv, i0 % nv), t01 = X(i1 / nv, i1 % nv);
      const R t10 = X(i2 / nv, i2 % nv), t11 = X(i3 / nv, i3 % nv);
      v = t00 * t11 - t01 * t10;
    }
    dv[u * s] = (T)v;
  }
}

// Row interchanges of a solve: the pivots of the factorisation applied to x
// in order (lu_solve's pivot pass), with selects on the register array.
template <typename R, int N>
__device__ __forceinline__ void apply_pivots(const int (&piv)[N], R (&x)[N]) {
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const bool sw = piv[k] == i;
      const R a = x[k], b = x[i];
      x[k] = sw ? b : a;
      x[i] = sw ? a : b;
    }
}

// Forward and back substitution with the factors a[0..N)[0..N) (unit lower,
// upper with inverted diagonal), lu_solve's order.
template <typename R, int N, int NC>
__device__ __forceinline__ void lu_subst(const R (&a)[N][NC], R (&x)[N]) {
#pragma unroll
  for (int i = 1; i < N; ++i) {
    R s = x[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s = fma(-a[i][k], x[k], s);
    x[i] = s;
  }
#pragma unroll
  for (int i = N - 1; i >= 0; --i) {
    R s = x[i];
#pragma unroll
    for (int k = i + 1; k < N; ++k) s = fma(-a[i][k], x[k], s);
    x[i] = s * a[i][i];
  }
}

// Local-energy determinant phase of one (walker, spin) channel, mixed method,
// excitation mode (spin_channel with OP and the refinement, slater_pooling.py:
// 147-260, 437-723), with the LU, the solves and their FP64 refinement in
// registers: the operations of spin_channel in the same order (bitwise the
// same values) without its HBM work arrays. mo / bk: the spin's MO and
// kinetic rows in shared memory. Writes the determinant values (relative to
// det A, FP64) and traces per unique determinant, and det A to *dref.
template <typename R, int N>
__device__ inline void el_channel_regs(const qmc_wf_desc& d, int spin, CView<R> mo, CView<R> bk,
                                       int nv, const int* tab, double* dv, double* ov, int64_t s,
                                       double* dref) {
  static_assert(kMixed<R>, "the register local-energy path is the mixed method's");
  // LU of the occupied block (lu_factor's operations and pivots)
  R a[N][N];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) a[i][j] = mo(i, j);
  int piv[N];
  double det = 1.0;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    int p = k;
    R amax = fabs(a[k][k]);
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const R v = fabs(a[i][k]);
      if (v > amax) {
        amax = v;
        p = i;
      }
    }
    piv[k] = p;
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const bool sw = (i == p);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const R x = a[k][j], y = a[i][j];
        a[k][j] = sw ? y : x;
        a[i][j] = sw ? x : y;
      }
    }
    if (p != k) det = -det;
    const R akk = a[k][k];
    det *= to_f64(akk);
    const R inv = akk != (R)0 ? (R)1 / akk : (R)0;
    a[k][k] = inv;
#pragma unroll
    for (int i = k + 1; i < N; ++i) {
      const R l = a[i][k] * inv;
      a[i][k] = l;
#pragma unroll
      for (int j = k + 1; j < N; ++j) a[i][j] = fma(-l, a[k][j], a[i][j]);
    }
  }
  *dref = det;
  // x = A^-1 b of column c of the MO (kin = false) or kinetic (kin = true)
  // rows, with one FP64 refinement step (lu_solve, then lu_refine)
  auto solve = [&](bool kin, int c, double (&x64)[N]) {
    R x[N];
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = kin ? bk(i, c) : mo(i, c);
    apply_pivots<R, N>(piv, x);
    lu_subst<R, N, N>(a, x);
    R rc[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      // residual b - A x in double-float arithmetic (an FP32 pair, about 48
      // bits, enough for one refinement step from FP32): products split exactly
      // by fma, sums compensated (two-sum) -- no FP64 instruction: the FP32 <->
      // FP64 conversions of an FP64 residual issue on the FP64 pipe and hold
      // registers
      R sh = kin ? bk(i, c) : mo(i, c), sl = (R)0;
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const R ph = -mo(i, k) * x[k];
        const R pl = fma(-mo(i, k), x[k], -ph);
        const R t = sh + ph;
        const R bb = t - sh;
        const R err = (sh - (t - bb)) + (ph - bb);
        sh = t;
        sl += err + pl;
      }
      rc[i] = sh + sl;
    }
    apply_pivots<R, N>(piv, rc);
    lu_subst<R, N, N>(a, rc);
#pragma unroll
    for (int i = 0; i < N; ++i) x64[i] = (double)x[i] + (double)rc[i];
  };
  // X = A^-1 A_virt, refined
  double x64[N][kElRegNV];
#pragma unroll
  for (int c = 0; c < kElRegNV; ++c) {
    if (c >= nv) break;
    double y[N];
    solve(false, N + c, y);
#pragma unroll
    for (int i = 0; i < N; ++i) x64[i][c] = y[i];
  }
  // Y = A^-1 [B_occ | B_virt], refined: trace of the occupied block and
  // M = Y_virt - Y_occ X (virtual columns first, then the occupied columns
  // subtracted in order, as M is formed element by element)
  double m64[N][kElRegNV];
  double base = 0.0;
#pragma unroll
  for (int cc = 0; cc < N + kElRegNV; ++cc) {
    const int c = cc < kElRegNV ? N + cc : cc - kElRegNV;  // virtual, then occupied
    if (cc < kElRegNV && cc >= nv) continue;
    double y[N];
    solve(true, c, y);
    if (cc < kElRegNV) {
#pragma unroll
      for (int i = 0; i < N; ++i) m64[i][cc] = y[i];
    } else {
      base += y[c];
#pragma unroll
      for (int ic = 0; ic < kElRegNV; ++ic) {
        if (ic >= nv) break;
#pragma unroll
        for (int i = 0; i < N; ++i) m64[i][ic] = fma(-y[i], x64[c][ic], m64[i][ic]);
      }
    }
  }
  // excitation determinants and traces (spin_channel's loop with OP); entries
  // of order >= 1 exist only when there are virtual columns
  const int nd = d.ndet[spin];
  nv = nv > 0 ? nv : 1;
  for (int u = 0; u < nd; ++u) {
    const int ord = tab[5 * u];
    double dvu = 1.0, ovu = base;
    if (ord == 1) {
      const int i0 = tab[5 * u + 1];
      const double m = x64[i0 / nv][i0 % nv];
      dvu = m;
      ovu = fma(1.0 / m, m64[i0 / nv][i0 % nv], base);
    } else if (ord >= 2) {
      const int i0 = tab[5 * u + 1], i1 = tab[5 * u + 2];
      const int i2 = tab[5 * u + 3], i3 = tab[5 * u + 4];
      const double t00 = x64[i0 / nv][i0 % nv], t01 = x64[i1 / nv][i1 % nv];
      const double t10 = x64[i2 / nv][i2 % nv], t11 = x64[i3 / nv][i3 % nv];
      const double dt = t00 * t11 - t01 * t10;
      dvu = dt;
      const double m00 = m64[i0 / nv][i0 % nv], m01 = m64[i1 / nv][i1 % nv];
      const double m10 = m64[i2 / nv][i2 % nv], m11 = m64[i3 / nv][i3 % nv];
      const double idt = 1.0 / dt;
      ovu = base + idt * (t11 * m00 - t01 * m10 - t10 * m01 + t00 * m11);
    }
    dv[u * s] = dvu;
    ov[u * s] = ovu;
  }
}

template <typename R>
__device__ inline bool el_channel_regs_n(const qmc_wf_desc& d, int spin, CView<R> mo,
                                         CView<R> bk, int n, int nv, const int* tab, double* dv,
                                         double* ov, int64_t s, double* dref) {
  if constexpr (!kMixed<R>) {
    return false;
  } else {
    switch (n) {
      case 1: el_channel_regs<R, 1>(d, spin, mo, bk, nv, tab, dv, ov, s, dref); return true;
      case 2: el_channel_regs<R, 2>(d, spin, mo, bk, nv, tab, dv, ov, s, dref); return true;
      case 3: el_channel_regs<R, 3>(d, spin, mo, bk, nv, tab, dv, ov, s, dref); return true;
      case 4: el_channel_regs<R, 4>(d, spin, mo, bk, nv, tab, dv, ov, s, dref); return true;
      case 5: el_channel_regs<R, 5>(d, spin, mo, bk, nv, tab, dv, ov, s, dref); return true;
      default: return false;
    }
  }
}

template <typename R, bool OP>
__device__ inline void ep_det(const qmc_wf_desc& d, const EPLayout& L, unsigned char* scr,
                              int64_t ss, int64_t w, int spin, R* mo_s, const R* bk_s, int wl,
                              int nwb, double* dref, const int* dtab) {
  using T = typename std::conditional<OP, double, R>::type;
  const int row0 = spin ? d.nup : 0;
  const int64_t cs = nwb, rs = (int64_t)d.nmo_used * nwb;
  const CView<R> mo{mo_s + row0 * rs + wl, rs, cs};
  const CView<R> bk{(OP ? bk_s : mo_s) + row0 * rs + wl, rs, cs};
  const int64_t vm = L.vmax > 0 ? L.vmax : 1;
  SpinWork<R> wk;
  wk.LU = MView<R>{rptr<R>(scr, L.lu[spin], ss, w), (int64_t)L.nmax * ss, ss};
  wk.X = MView<R>{rptr<R>(scr, L.x[spin], ss, w), vm * ss, ss};
  wk.Y = MView<R>{rptr<R>(scr, L.y[spin], ss, w), (int64_t)L.omax * ss, ss};
  wk.rc = MView<R>{rptr<R>(scr, L.rc[spin], ss, w), ss, ss};
  wk.X64 = MView<double>{rptr<double>(scr, L.x64[spin], ss, w), vm * ss, ss};
  wk.Y64 = MView<double>{rptr<double>(scr, L.y64[spin], ss, w), (int64_t)L.omax * ss, ss};
  T* dv = rptr<T>(scr, L.dv, ss, w) + (spin ? d.ndet[0] * ss : 0);
  if constexpr (OP) {
    if (el_regs(d)) {
      const int n = spin ? d.ndown : d.nup;
      double* ovp = rptr<double>(scr, L.ov, ss, w) + (spin ? d.ndet[0] * ss : 0);
      const int nv = d.max_orb[spin] - n;
      if (el_channel_regs_n<R>(d, spin, mo, bk, n, nv, dtab, (double*)dv, ovp, ss,
                               &dref[spin * nwb + wl]))
        return;
    }
  }
  if (!OP && d.det_mode == QMC_DET_EXCITATION) {
    // in place (the MO rows are recomputed before every evaluation): the LU of
    // the occupied columns and A^-1 A_virt over the virtual columns of the
    // spin's MO rows, the same operations in the same order as on copies
    R* rows = mo_s + row0 * rs + wl;
    const int n = spin ? d.ndown : d.nup;
    const int nv = d.max_orb[spin] - n;
    double det;
    if (n > 0 && lu_solve_regs_n<R>(rows, rs, cs, n, nv, &det)) {
      dref[spin * nwb + wl] = det;
      excitation_values<R, T>(d, dtab, spin, CView<R>{rows + n * cs, rs, cs}, nv > 0 ? nv : 1,
                              dv, ss);
      return;
    }
    wk.LU = MView<R>{rows, rs, cs};
    wk.X = MView<R>{rows + n * cs, rs, cs};
  }
  double* ov = OP ? rptr<double>(scr, L.ov, ss, w) + (spin ? d.ndet[0] * ss : 0) : nullptr;
  spin_channel<R, OP, T>(d, spin, mo, bk, wk, SpinOut<T>{dv, ov, ss, &dref[spin * nwb + wl]});
}

// Block-cooperative LU of the psi / Metropolis determinant phase for spin
// channels beyond the register path (excitation mode, in place in the
// shared-memory MO rows). The nslot threads of a walker split its two
// channels: slots of even parity serve spin up, odd spin down; the T threads
// of a channel (rank r = slot / 2) swap the pivot rows by columns j = r mod T
// and eliminate rows i = k + 1 + r mod T. Every element sees lu_factor's
// operations in lu_factor's order (the same pivot choice, l = a_ik / a_kk as
// a_ik * (1 / a_kk), one fma per update), so the factors, pivots and det are
// bitwise those of the one-thread factorisation. Rank 0 of a channel is the
// thread the one-thread path runs on (slot = spin, tid < 2 nwb): it keeps the
// pivots and det, and then solves the virtual columns and forms the
// excitation values as ep_det does. Three block barriers per elimination step.
constexpr int kCoopMinN = 6;

template <typename R>
__host__ __device__ inline bool coop_lu_applies(const qmc_wf_desc& d, int nslot) {
  if (d.det_mode != QMC_DET_EXCITATION || nslot < 4) return false;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  if (nmax < kCoopMinN) return false;
  for (int s = 0; s < 2; ++s) {  // the register path serves both channels
    const int n = s ? d.ndown : d.nup;
    const int nv = d.max_orb[s] - n;
    if (n > kRegMaxN<R> || nv > kRegNV) return true;
  }
  return false;
}

// The elimination steps of the block-cooperative LU of this thread's channel
// matrix A(i, j) = A[i rs + j cs] (n x n; on: the thread serves a channel of
// rank r among nt threads). Every thread of the block calls it: three block
// barriers per step up to nmax, and one at the end, after which the factors
// (unit lower, upper with inverted diagonal, as lu_factor leaves them), the
// pivots piv[0..n) and det (the return value) are valid on every thread of the
// channel.
template <typename R>
__device__ inline double coop_lu_steps(R* A, int64_t rs, int64_t cs, int n, int nmax, bool on,
                                       int r, int nt, int* piv) {
  double det = 1.0;
  for (int k = 0; k < nmax; ++k) {
    const bool act = on && k < n;
    int p = k;
    if (act) {
      R amax = fabs(A[k * rs + k * cs]);
      for (int i = k + 1; i < n; ++i) {
        const R v = fabs(A[i * rs + k * cs]);
        if (v > amax) {
          amax = v;
          p = i;
        }
      }
    }
    __syncthreads();  // column k read by every thread of the channel
    if (act && p != k)
      for (int j = r; j < n; j += nt) {
        const R tmp = A[k * rs + j * cs];
        A[k * rs + j * cs] = A[p * rs + j * cs];
        A[p * rs + j * cs] = tmp;
      }
    __syncthreads();  // pivot row in place
    R inv = (R)0;
    if (act) {
      const R akk = A[k * rs + k * cs];
      piv[k] = p;
      if (p != k) det = -det;
      det *= to_f64(akk);
      inv = akk != (R)0 ? (R)1 / akk : (R)0;
      for (int i = k + 1 + r; i < n; i += nt) {
        const R l = A[i * rs + k * cs] * inv;
        A[i * rs + k * cs] = l;
        for (int j = k + 1; j < n; ++j) A[i * rs + j * cs] = fma(-l, A[k * rs + j * cs], A[i * rs + j * cs]);
      }
    }
    __syncthreads();  // step k's updates and a_kk reads done
    // a_kk is read by no later step of the factorisation: stored after the barrier
    if (act && r == 0) A[k * rs + k * cs] = inv;
  }
  __syncthreads();  // the inverted diagonal in place for the solves
  return det;
}

// Thread roles of the cooperative determinant phase: the walker's even slots
// serve spin up, the odd ones spin down; rank r = slot / 2.
struct CoopRole {
  int slot, wl, spin, r, nt;
  bool on;
  __device__ CoopRole(int nwb, int nslot) {
    const int tid = threadIdx.x;
    slot = tid / nwb;
    wl = tid - slot * nwb;
    spin = slot & 1;
    r = slot >> 1;
    nt = (nslot - spin + 1) >> 1;
    on = slot < nslot;
  }
};

// The local-energy kernel's cooperative path: the channels beyond the
// register path of the mixed local energy (el_regs), from six electrons.
template <typename R>
__host__ __device__ inline bool coop_el_applies(const qmc_wf_desc& d, int nslot) {
  if (d.det_mode != QMC_DET_EXCITATION || nslot < 4 || el_regs(d)) return false;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  return nmax >= kCoopMinN;
}

template <typename R, typename T>
__device__ inline void ep_det_coop(const qmc_wf_desc& d, const EPLayout& L, unsigned char* dbase,
                                   int64_t dss, int64_t w0, int64_t nw, bool dsm, R* MO, int nwb,
                                   int nslot, double* DREF) {
  const CoopRole c(nwb, nslot);
  const int spin = c.spin, wl = c.wl;
  const int n = spin ? d.ndown : d.nup;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  const int64_t cs = nwb, rs = (int64_t)d.nmo_used * nwb;
  R* A = MO + (spin ? d.nup : 0) * rs + wl;
  int piv[QMC_MAX_NSPIN];
  const double det = coop_lu_steps<R>(A, rs, cs, n, nmax, c.on, c.r, c.nt, piv);
  if (threadIdx.x < 2 * nwb && w0 + wl < nw) {
    using V = T;
    const int64_t w = dsm ? wl : w0 + wl;
    V* dv = rptr<V>(dbase, L.dv, dss, w) + (spin ? d.ndet[0] * dss : 0);
    const int nv = d.max_orb[spin] - n;
    if (n == 0) {
      for (int u = 0; u < d.ndet[spin]; ++u) dv[u * dss] = (V)1;
      DREF[spin * nwb + wl] = 1.0;
      return;
    }
    DREF[spin * nwb + wl] = det;
    const MView<R> LU{A, rs, cs};
    const MView<R> X{A + n * cs, rs, cs};
    if (nv > 0) lu_solve<R>(LU, n, piv, X.c(), X, nv);
    excitation_values<R, V>(d, d.det_table[spin], spin, X.c(), nv > 0 ? nv : 1, dv, dss);
  }
}

// Local-energy determinant phase of large excitation-mode channels with the
// walker's threads: the channel's T threads copy the occupied block to the LU
// work array by rows, factor it cooperatively (coop_lu_steps), and solve the
// right-hand sides by columns (A^-1 A_virt and A^-1 [B_occ | B_virt], each
// column with its FP64 residual refinement in the mixed method: the column
// solves are independent, so the values are spin_channel's bitwise); the
// channel's first thread then forms the determinant ratios and traces
// (excitation_tail). Two more block barriers.
template <typename R>
__device__ inline void ep_det_el_coop(const qmc_wf_desc& d, const EPLayout& L,
                                      unsigned char* dbase, int64_t dss, int64_t w0, int64_t nw,
                                      bool dsm, R* MO, R* BK, int nwb, int nslot, double* DREF) {
  constexpr bool REFINE = kMixed<R>;
  const CoopRole c(nwb, nslot);
  const int spin = c.spin, wl = c.wl, r = c.r, nt = c.nt;
  const int n = spin ? d.ndown : d.nup;
  const int nv = d.max_orb[spin] - n;
  const int nmax = d.nup > d.ndown ? d.nup : d.ndown;
  const int64_t cs = nwb, rs = (int64_t)d.nmo_used * nwb;
  const int row0 = spin ? d.nup : 0;
  const CView<R> mo{MO + row0 * rs + wl, rs, cs};
  const CView<R> bk{BK + row0 * rs + wl, rs, cs};
  const CView<R> avirt{mo.p + n * cs, rs, cs};
  const int64_t w = dsm ? wl : w0 + wl;
  const int64_t vm = L.vmax > 0 ? L.vmax : 1;
  SpinWork<R> wk;
  wk.LU = MView<R>{rptr<R>(dbase, L.lu[spin], dss, w), (int64_t)L.nmax * dss, dss};
  wk.X = MView<R>{rptr<R>(dbase, L.x[spin], dss, w), vm * dss, dss};
  wk.Y = MView<R>{rptr<R>(dbase, L.y[spin], dss, w), (int64_t)L.omax * dss, dss};
  wk.rc = MView<R>{rptr<R>(dbase, L.rc[spin], dss, w), dss, dss};
  wk.X64 = MView<double>{rptr<double>(dbase, L.x64[spin], dss, w), vm * dss, dss};
  wk.Y64 = MView<double>{rptr<double>(dbase, L.y64[spin], dss, w), (int64_t)L.omax * dss, dss};
  if (c.on)
    for (int i = r; i < n; i += nt)
      for (int j = 0; j < n; ++j) wk.LU(i, j) = mo(i, j);
  __syncthreads();  // the occupied block copied
  int piv[QMC_MAX_NSPIN];
  const double det = coop_lu_steps<R>(wk.LU.p, wk.LU.rs, wk.LU.cs, n, nmax, c.on, r, nt, piv);
  if (c.on && n > 0) {
    // this thread's columns; a private residual column for the refinements
    R rcl[QMC_MAX_NSPIN];
    const MView<R> rc{rcl, 1, 1};
    auto col = [](MView<R> m, int j) { return MView<R>{m.p + j * m.cs, m.rs, m.cs}; };
    auto ccol = [](CView<R> m, int j) { return CView<R>{m.p + j * m.cs, m.rs, m.cs}; };
    for (int j = r; j < nv; j += nt) lu_solve<R>(wk.LU, n, piv, ccol(avirt, j), col(wk.X, j), 1);
    for (int j = r; j < n + nv; j += nt) lu_solve<R>(wk.LU, n, piv, ccol(bk, j), col(wk.Y, j), 1);
    if (REFINE) {
      for (int j = r; j < nv; j += nt)
        lu_refine<R>(wk.LU, n, piv, mo, ccol(avirt, j), col(wk.X, j),
                     MView<double>{wk.X64.p + j * wk.X64.cs, wk.X64.rs, wk.X64.cs}, rc, 1);
      for (int j = r; j < n + nv; j += nt)
        lu_refine<R>(wk.LU, n, piv, mo, ccol(bk, j), col(wk.Y, j),
                     MView<double>{wk.Y64.p + j * wk.Y64.cs, wk.Y64.rs, wk.Y64.cs}, rc, 1);
    }
  }
  __syncthreads();  // every column solved
  if (threadIdx.x < 2 * nwb && w0 + wl < nw) {
    double* dv = rptr<double>(dbase, L.dv, dss, w) + (spin ? d.ndet[0] * dss : 0);
    double* ov = rptr<double>(dbase, L.ov, dss, w) + (spin ? d.ndet[0] * dss : 0);
    if (n == 0) {
      for (int u = 0; u < d.ndet[spin]; ++u) {
        dv[u * dss] = 1.0;
        ov[u * dss] = 0.0;
      }
      DREF[spin * nwb + wl] = 1.0;
      return;
    }
    DREF[spin * nwb + wl] = det;
    excitation_tail<R, true, double>(d, spin, n, nv, wk, SpinOut<double>{dv, ov, dss, &DREF[spin * nwb + wl]});
  }
}

struct EPPtrs {
  unsigned char* smem;
  EPShape S;
};

// Evaluate psi (and, with KIN, the kinetic energy and potentials) for the
// block's walkers at split positions `pbuf` (shared memory, [nwb][3 nelec]).
// Results in shared memory: psi[wl], and with KIN kin[wl], v[wl] (V_en + V_ee),
// written by thread wl (< nwb) and visible to that thread on return: no
// barrier follows the combine phase, so a caller reads only its own walker's
// results, and its next write to the block's rows (positions, proposal) comes
// after a barrier. Every thread of the block must call this (it contains block
// barriers).
// ELCOOP: the local-energy kernel instance with the cooperative determinant
// phase of large channels (a separate instance: its work arrays and pivots
// would cost the small-molecule local-energy kernel registers).
template <typename R, int JC, bool KIN, bool ELCOOP = false>
__device__ inline void ep_eval(const qmc_wf_desc& d, const Tables<R>& t, const EPPtrs& p,
                               const XP<R>* pbuf, unsigned char* scr, int64_t ss, int64_t w0,
                               int64_t nw) {
  const EPShape& S = p.S;
  const int nwb = S.nwb, ne = d.nelec, nc = 3 * ne;
  const int tid = threadIdx.x;
  R* MO = reinterpret_cast<R*>(p.smem + S.o_mo);
  R* BK = reinterpret_cast<R*>(p.smem + S.o_bk);
  double* JR = reinterpret_cast<double*>(p.smem + S.o_jrow);
  double* VR = reinterpret_cast<double*>(p.smem + S.o_vrow);
  double* DREF = reinterpret_cast<double*>(p.smem + S.o_dref);
  double* PSI = reinterpret_cast<double*>(p.smem + S.o_psi);
  double* KINV = reinterpret_cast<double*>(p.smem + S.o_kin);
  double* V = reinterpret_cast<double*>(p.smem + S.o_v);
  {
    // electrons dealt to the walker's slots in snake order (slot s takes s,
    // 2 nslot - 1 - s, 2 nslot + s, ...): psi's Jastrow row of electron e has
    // ne - 1 - e pairs, and the snake evens the slots' pair counts; each
    // electron's arithmetic does not depend on the thread that runs it
    const int slot = tid / nwb, wl = tid - (tid / nwb) * nwb;
    const int ns = S.nslot;
    for (int b = 0; b < ne && slot < ns; b += ns) {
      const int e = ((b / ns) & 1) ? b + ns - 1 - slot : b + slot;
      if (e < ne)
        ep_electron<R, JC, KIN>(d, t, pbuf + wl * S.pstride, e, MO + wl, BK + wl, nwb,
                                &JR[e * nwb + wl], &VR[e * nwb + wl]);
    }
  }
  __syncthreads();
  const EPLayout L = ep_layout(d, KIN ? 1 : 0);
  const bool dsm = S.o_det >= 0;  // work arrays in shared memory: slot = local walker
  unsigned char* const dbase = dsm ? p.smem + S.o_det : scr;
  const int64_t dss = dsm ? nwb : ss;
  if (!KIN && coop_lu_applies<R>(d, S.nslot)) {
    ep_det_coop<R, R>(d, L, dbase, dss, w0, nw, dsm, MO, nwb, S.nslot, DREF);
  } else if (KIN && ELCOOP && coop_el_applies<R>(d, S.nslot)) {
    if constexpr (KIN && ELCOOP) ep_det_el_coop<R>(d, L, dbase, dss, w0, nw, dsm, MO, BK, nwb, S.nslot, DREF);
  } else if (tid < 2 * nwb) {
    const int spin = tid / nwb, wl = tid - spin * nwb;
    if (w0 + wl < nw)
      ep_det<R, KIN>(d, L, dbase, dss, dsm ? wl : w0 + wl, spin, MO, BK, wl, nwb, DREF,
                     d.det_table[spin]);
  }
  __syncthreads();
  if (tid < nwb && w0 + tid < nw) {
    using T = typename std::conditional<KIN, double, R>::type;
    const int wl = tid;
    const int64_t w = w0 + wl;
    double kin = 0.0;
    const int64_t slot = dsm ? wl : w;
    const T* dv = rptr<T>(dbase, L.dv, dss, slot);
    const double* ov = KIN ? rptr<double>(dbase, L.ov, dss, slot) : nullptr;
    const double psid = ci_combine<T, KIN, T>(d, dv, ov, dss, DREF[wl], DREF[nwb + wl], &kin,
                                               (!KIN && kMixed<R>) ? (const T*)t.ciw : nullptr);
    double logj = 0.0, v = 0.0;
    for (int e = 0; e < ne; ++e) {
      logj += JR[e * nwb + wl];
      if (KIN) v += VR[e * nwb + wl];
    }
    double jf = 1.0;
    if (d.use_jastrow || d.use_jastrow_en) {
      if constexpr (kMixed<R> && !KIN) jf = exp_mixed(logj);
      else jf = exp(logj);
    }
    PSI[wl] = psid * jf;
    if (KIN) {
      KINV[wl] = kin;
      V[wl] = v;
    }
  }
}

// Stage the positions of walkers [w0, w0 + nwb) into shared memory as split
// coordinates, rows of `ps` entries; slots past the last walker repeat walker
// nw - 1 (a valid configuration, never stored).
template <typename R>
__device__ inline void ep_stage_positions(const double* pos, int64_t w0, int64_t nw, int nwb,
                                          int nc, int ps, XP<R>* P) {
  for (int i = threadIdx.x; i < nwb * nc; i += blockDim.x) {
    const int wl = i / nc, c = i - wl * nc;
    int64_t w = w0 + wl;
    if (w >= nw) w = nw - 1;
    P[wl * ps + c] = split_xp<R>(pos[w * nc + c]);
  }
  __syncthreads();
}

// x + dz for a split coordinate: FP64 addition (plain method) or an FP32
// two-sum with renormalisation (mixed method; dl carries the part of a FP64
// increment below FP32 precision, 0 for generated FP32 increments).
template <typename R>
__device__ __forceinline__ XP<R> xp_add(XP<R> x, R dz, R dl = (R)0) {
  if constexpr (std::is_same<R, float>::value) {
    const float s = x.h + dz;
    const float bb = s - x.h;
    const float err = (x.h - (s - bb)) + (dz - bb);
    const float lo = x.l + err + dl;
    const float h = s + lo;
    return XP<R>{h, lo - (h - s)};
  } else {
    return XP<R>{x.h + dz, 0.0};
  }
}

template <typename R>
__device__ __forceinline__ double xp_value(XP<R> x) {
  return to_f64(x.h) + to_f64(x.l);
}

}  // namespace qmc
