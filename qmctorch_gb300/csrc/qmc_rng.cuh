// Counter-based generator of the Metropolis kernels.
#pragma once
#include <stdint.h>

#include "qmc_ep.cuh"

namespace qmc {

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
  __device__ __forceinline__ void normal2f(uint32_t a, uint32_t b, float& z0, float& z1) {
    const float u1 = ((float)a + 1.0f) * 2.3283064365386963e-10f;
    const float u2 = (float)b * 2.3283064365386963e-10f;
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
  }
  // uniform in [0, 1) with 53 random bits
  __device__ __forceinline__ double uniform53(uint32_t hi, uint32_t lo) {
    return ((double)(hi >> 5) * 67108864.0 + (double)(lo >> 6)) * 1.1102230246251565e-16;
  }
};

// Generated displacement of one electron, counter `call` (normal: two
// Box-Muller pairs scaled by sd; uniform: step * (2u - 1)).
template <typename R>
__device__ __forceinline__ void draw_displacement(Rng& rng, uint32_t call, int proba, double step,
                                                  double sd, R (&z)[3]) {
  rng.call = call;
  const U4 r = rng.next();
  if (proba == QMC_PROBA_NORMAL) {
    float f0, f1, f2, f3;
    rng.normal2f(r.x, r.y, f0, f1);
    rng.normal2f(r.z, r.w, f2, f3);
    z[0] = (R)f0 * (R)sd;
    z[1] = (R)f1 * (R)sd;
    z[2] = (R)f2 * (R)sd;
  } else {
    const uint32_t rr[3] = {r.x, r.y, r.z};
    for (int q = 0; q < 3; ++q)
      z[q] = (R)step * ((R)2 * ((R)rr[q] * (R)2.3283064365386963e-10) - (R)1);
  }
}

// Replayed displacement (three FP64 values): pn = pc + rp, keeping in the
// low part of a split coordinate what FP32 cannot hold.
template <typename R>
__device__ __forceinline__ void replay_displacement(const double* rp, const XP<R>* pc, XP<R>* pn) {
  for (int q = 0; q < 3; ++q) {
    const R zh = (R)rp[q];
    pn[q] = xp_add<R>(pc[q], zh, (R)(rp[q] - (double)zh));
  }
}

// Proposed coordinates of one electron: pc + displacement, the displacement
// either replayed (rp: three FP64 values) or drawn with counter `call`.
template <typename R>
__device__ __forceinline__ void propose_electron(Rng& rng, uint32_t call, int proba, double step,
                                                 double sd, const double* rp, const XP<R>* pc,
                                                 XP<R>* pn) {
  if (rp) {
    replay_displacement<R>(rp, pc, pn);
    return;
  }
  R z[3];
  draw_displacement<R>(rng, call, proba, step, sd, z);
  for (int q = 0; q < 3; ++q) pn[q] = xp_add<R>(pc[q], z[q]);
}

// Accept uniform of a move (replayed, or counter `call`) and the electron
// index of a one-elec move (counter `call`).
__device__ __forceinline__ double accept_uniform(Rng& rng, uint32_t call) {
  rng.call = call;
  const U4 r = rng.next();
  return rng.uniform53(r.x, r.y);
}
__device__ __forceinline__ int electron_draw(Rng& rng, uint32_t call, int ne) {
  rng.call = call;
  const U4 r = rng.next();
  return (int)(((uint64_t)r.x * (uint64_t)ne) >> 32);
}

}  // namespace qmc
