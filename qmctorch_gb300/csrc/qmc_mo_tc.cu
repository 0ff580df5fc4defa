// AO -> MO contraction on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators): MO = AO @ W, W = mo_scf * mo_modifier, for the mixed-precision
// module path (MolecularOrbitals.forward, molecular_orbitals.py:79-95).
//
// Split-BF16 x3 with FP32 accumulation. Every FP64 operand x is split into
// x_hi = bf16(x) and x_lo = bf16(x - x_hi) (x_hi + x_lo holds ~16 significant
// bits). The three products a_hi b_hi + a_hi b_lo + a_lo b_hi are one BF16 GEMM
// of depth 3 K over the concatenated operands
//     A' = [a_hi | a_hi | a_lo],   B' = [b_hi | b_lo | b_hi],
// so a single chain of tcgen05.mma instructions accumulates all of them in
// TMEM. Error per output: about 2^-16 of sum_k |a_k| |b_k| (the dropped
// a_lo b_lo term and the split residuals), plus FP32 accumulation rounding.
//
// Tiles: one CTA per 128 AO rows at a time (M = 128 = TMEM lanes), persistent
// over row tiles. B' (N x 3K, N = nmo rounded up to 16) is built once per CTA
// in shared memory; the A' tile is staged by all threads (FP64 loads, split,
// 16-byte shared stores) in the canonical K-major no-swizzle layout of the
// tensor core: 8 x 16-byte core matrices, adjacent along K 128 bytes apart
// (leading byte offset), adjacent 8-row groups 3K * 16 bytes apart (stride
// byte offset). One elected thread issues the 3K / 16 MMAs (128 x N x 16
// each) and commits them to an mbarrier; the eight warps then read the FP32
// accumulators back with tcgen05.ld (warp w: lanes 32 (w % 4) .. + 31, column
// chunks of 16 alternating between the two warpgroups) and store FP64.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "qmc_host.cuh"

namespace qmc {
namespace tc {

constexpr int kM = 128;          // rows per tile (TMEM lanes, MMA M)
constexpr int kThreads = 256;    // 8 warps: two warpgroups share the epilogue columns
constexpr int kMaxN = 256;       // MMA N limit for M = 128
constexpr uint64_t kWaitNs = 1000000000ull;  // mbarrier wait limit: 1 s

struct Shape {
  int kp;        // K of one piece (nao rounded up to 16)
  int kk;        // GEMM depth 3 kp
  int n;         // MMA N (nmo rounded up to 16)
  int tmem_cols; // power of two >= max(32, n)
  int64_t a_off, b_off, bar_off, smem;
};

__host__ __device__ inline Shape shape(int nao, int nmo) {
  Shape s;
  s.kp = (nao + 15) & ~15;
  s.kk = 3 * s.kp;
  s.n = (nmo + 15) & ~15;
  s.tmem_cols = 32;
  while (s.tmem_cols < s.n) s.tmem_cols *= 2;
  s.a_off = 0;
  s.b_off = s.a_off + (int64_t)kM * s.kk * 2;
  s.bar_off = s.b_off + (int64_t)s.n * s.kk * 2;
  s.smem = s.bar_off + 16 + 1024;  // mbarrier (8 B), TMEM address (4 B); 1 KB for base alignment
  return s;
}

// Byte offset of the 16-byte chunk holding elements (r, 8 c .. 8 c + 7) of a
// K-major operand with depth kk in the no-swizzle canonical layout.
__host__ __device__ inline uint32_t chunk_offset(int r, int c, int kk) {
  return (uint32_t)((r >> 3) * (kk * 16) + c * 128 + (r & 7) * 16);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (K direction), stride byte offset (8-row groups), version 1 at bit
// 46, no swizzle.
__device__ inline uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ inline uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ inline uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for the completion of phase `parity` of the mbarrier at
// shared address `bar`; false after kWaitNs.
__device__ inline bool mbar_wait(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

__device__ inline uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// Split 8 FP64 values into their BF16 hi and lo parts, packed as 16 bytes each.
__device__ inline void split8(const double (&v)[8], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const __nv_bfloat16 h0 = __double2bfloat16(v[2 * j]), h1 = __double2bfloat16(v[2 * j + 1]);
    const __nv_bfloat16 l0 = __double2bfloat16(v[2 * j] - (double)__bfloat162float(h0));
    const __nv_bfloat16 l1 = __double2bfloat16(v[2 * j + 1] - (double)__bfloat162float(h1));
    h[j] = pack_bf16x2(h0, h1);
    l[j] = pack_bf16x2(l0, l1);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ inline void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ inline void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
__device__ inline void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
// Make this thread's generic-proxy shared-memory writes visible to the
// tensor core (async proxy).
__device__ inline void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

__global__ void __launch_bounds__(kThreads) mo_tc_kernel(const double* __restrict__ ao,
                                                         int64_t nrows, int nao, int nmo,
                                                         const double* __restrict__ mo_scf,
                                                         const double* __restrict__ mo_mod,
                                                         double* __restrict__ mo) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const Shape S = shape(nao, nmo);
  // 1 KB-aligned base (the dynamic shared-memory window is only 16-byte aligned)
  const uint32_t raw_addr = (uint32_t)__cvta_generic_to_shared(smem_raw);
  const uint32_t pad = (1024u - (raw_addr & 1023u)) & 1023u;
  unsigned char* smem = smem_raw + pad;
  const uint32_t base = raw_addr + pad;
  const uint32_t a_addr = base + (uint32_t)S.a_off, b_addr = base + (uint32_t)S.b_off;
  const uint32_t bar = base + (uint32_t)S.bar_off;
  volatile uint32_t* tmem_slot = reinterpret_cast<volatile uint32_t*>(smem + S.bar_off + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cpk = S.kp >> 3;  // 16-byte chunks per piece and row

  // -- set-up: TMEM columns (warp 0), the mbarrier, B' in shared memory ------
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     base + (uint32_t)S.bar_off + 8),
                 "r"((uint32_t)S.tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // B'[n][k]: W[k][n] split; pieces [hi | lo | hi]; zero past nao / nmo
  for (int i = tid; i < S.n * cpk; i += kThreads) {
    const int nr = i & 7, c = (i >> 3) % cpk, ng = (i >> 3) / cpk;
    const int n = ng * 8 + nr;
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int k = c * 8 + j;
      v[j] = (n < nmo && k < nao) ? __ldg(mo_scf + (int64_t)k * nmo + n) *
                                        __ldg(mo_mod + (int64_t)k * nmo + n)
                                  : 0.0;
    }
    uint4 hi, lo;
    split8(v, hi, lo);
    *reinterpret_cast<uint4*>(smem + S.b_off + chunk_offset(n, c, S.kk)) = hi;
    *reinterpret_cast<uint4*>(smem + S.b_off + chunk_offset(n, cpk + c, S.kk)) = lo;
    *reinterpret_cast<uint4*>(smem + S.b_off + chunk_offset(n, 2 * cpk + c, S.kk)) = hi;
  }
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  const uint32_t idesc = instr_desc(kM, S.n);
  const uint32_t lbo = 128, sbo = (uint32_t)S.kk * 16;
  const int nsteps = S.kk / 16;
  const int64_t ntiles = (nrows + kM - 1) / kM;
  const int q = warp & 3, half = warp >> 2;
  const int nchunk = S.n / 16;
  uint32_t phase = 0;

  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t row0 = tile * kM;
    // -- stage A' = [hi | hi | lo] of rows row0 .. row0 + 127 ---------------
    for (int i = tid; i < kM * cpk; i += kThreads) {
      const int rr = i & 7, c = (i >> 3) % cpk, rg = (i >> 3) / cpk;
      const int r = rg * 8 + rr;
      const int64_t row = row0 + r;
      double v[8];
      const double* src = ao + row * nao + c * 8;
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = (row < nrows && c * 8 + j < nao) ? __ldg(src + j) : 0.0;
      uint4 hi, lo;
      split8(v, hi, lo);
      *reinterpret_cast<uint4*>(smem + S.a_off + chunk_offset(r, c, S.kk)) = hi;
      *reinterpret_cast<uint4*>(smem + S.a_off + chunk_offset(r, cpk + c, S.kk)) = hi;
      *reinterpret_cast<uint4*>(smem + S.a_off + chunk_offset(r, 2 * cpk + c, S.kk)) = lo;
    }
    fence_proxy_async();
    fence_before_sync();  // the previous tile's tcgen05.ld before the next MMA
    __syncthreads();
    fence_after_sync();
    // -- one thread issues the MMA chain and commits it to the mbarrier ----
    if (tid == 0) {
      for (int s = 0; s < nsteps; ++s) {
        const uint64_t ad = smem_desc(a_addr + (uint32_t)s * 256u, lbo, sbo);
        const uint64_t bd = smem_desc(b_addr + (uint32_t)s * 256u, lbo, sbo);
        const uint32_t acc = s > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
              bar)
          : "memory");
    }
    const bool ok = mbar_wait(bar, phase);
    phase ^= 1u;
    if (__syncthreads_or(!ok)) {
      // the MMAs did not complete within the limit: mark this tile's rows
      // NaN, give the tensor core a second bounded wait, release TMEM, stop
      for (int i = tid; i < kM * nmo; i += kThreads) {
        const int64_t row = row0 + i / nmo;
        if (row < nrows) mo[row * nmo + i % nmo] = __longlong_as_double(0x7ff8000000000000ll);
      }
      if (!ok) mbar_wait(bar, phase ^ 1u);
      break;
    }
    fence_after_sync();
    // -- epilogue: TMEM -> registers -> FP64 rows --------------------------
    const int64_t row = row0 + q * 32 + lane;
    for (int ch = half; ch < nchunk; ch += 2) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(ch * 16), v);
      if (row < nrows) {
        double* dst = mo + row * nmo + ch * 16;
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (ch * 16 + j < nmo) dst[j] = (double)v[j];
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"((uint32_t)S.tmem_cols)
                 : "memory");
}

}  // namespace tc
}  // namespace qmc

using namespace qmc;

extern "C" {

int qmc_mo_eval_tc(const qmc_wf_desc* d, const double* ao, int64_t nrows, double* mo,
                   void* stream) {
  int st = check_desc(d);
  if (st) return st;
  if (nrows < 0 || (nrows > 0 && (!ao || !mo))) return QMC_ERR_ARG;
  if (d->nao < 1 || d->nmo < 1) return QMC_ERR_ARG;
  const tc::Shape S = tc::shape(d->nao, d->nmo);
  if (S.n > tc::kMaxN || S.smem > 227 * 1024) return QMC_ERR_SHAPE;
  if (nrows == 0) return QMC_OK;
  if ((st = prepare_smem(tc::mo_tc_kernel, S.smem))) return st;
  int dev = 0, nsm = 1, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tc::mo_tc_kernel, tc::kThreads,
                                                    (size_t)S.smem) != cudaSuccess ||
      occ < 1) {
    cudaGetLastError();
    return QMC_ERR_LAUNCH;
  }
  // resident CTAs of one SM must fit its 512 TMEM columns together, so that
  // no tcgen05.alloc waits on another CTA
  if (occ > 512 / S.tmem_cols) occ = 512 / S.tmem_cols;
  const int64_t ntiles = (nrows + tc::kM - 1) / tc::kM;
  int64_t grid = (int64_t)nsm * occ;
  if (grid > ntiles) grid = ntiles;
  tc::mo_tc_kernel<<<(unsigned)grid, tc::kThreads, S.smem, (cudaStream_t)stream>>>(
      ao, nrows, d->nao, d->nmo, d->mo_scf, d->mo_modifier, mo);
  return launch_status();
}

}  // extern "C"
