// AO -> MO contraction on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators): MO = AO @ W, W = mo_scf * mo_modifier, for the mixed-precision
// module path (MolecularOrbitals.forward, molecular_orbitals.py:79-95).
//
// Split-BF16 x3 with FP32 accumulation. Every FP64 operand x is split into
// x_hi = bf16(x) and x_lo = bf16(x - x_hi) (x_hi + x_lo holds ~16 significant
// bits). The three products a_hi b_hi + a_hi b_lo + a_lo b_hi form one chain
// of tcgen05.mma instructions of depth 3 K accumulated in TMEM: shared memory
// holds each operand once as [hi | lo] and the MMA descriptors of the three
// K segments point at (a_hi, b_hi), (a_hi, b_lo), (a_lo, b_hi). Error per
// output: about 2^-16 of sum_k |a_k| |b_k| (the dropped a_lo b_lo term and the
// split residuals), plus FP32 accumulation rounding.
//
// Operand layout: canonical K-major, no swizzle: 8-row x 16-byte core
// matrices, adjacent along K 128 bytes apart (leading byte offset), adjacent
// 8-row groups 2 K' * 16 bytes apart (stride byte offset; K' = nao rounded up
// to 16).
//
// Warp-specialised persistent CTA (17 warps), one 128-row tile of AO rows at
// a time (M = 128 = TMEM lanes):
//   warps 0-7   producers: FP64 AO rows -> split -> 16-byte shared stores into
//               one of two A buffers;
//   warp 8      allocates TMEM; lane 0 issues the MMA chain of a tile into one
//               of two TMEM accumulators and commits it to two mbarriers
//               (A buffer free, accumulator full);
//   warps 9-16  epilogue: tcgen05.ld of the accumulator (warp w reads TMEM
//               lanes 32 (w % 4) .. + 31; the two groups of four alternate
//               16-column chunks) and FP64 stores of the MO rows.
// So the loads of tile i + 1, the MMAs of tile i and the stores of tile i - 1
// overlap. Every pipeline wait is bounded (1 s by default, host-settable
// with qmc_set_wait_limit_ns); on a timeout the CTA raises a shared abort
// flag, all roles leave their loops, the CTA's tiles are written as NaN, the
// device status word g_tc_timeout is set (read and cleared by
// qmc_mo_eval_tc_status), and TMEM is released after a wait of the default
// limit for the last committed MMA chain.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "qmc_host.cuh"

namespace qmc {
namespace tc {

constexpr int kM = 128;                 // rows per tile (TMEM lanes, MMA M)
constexpr int kProducerWarps = 8;
constexpr int kMmaWarp = kProducerWarps;  // warp 8
constexpr int kEpilogueWarps = 8;
constexpr int kWarps = kProducerWarps + 1 + kEpilogueWarps;
constexpr int kThreads = kWarps * 32;   // 544
constexpr int kProducerThreads = kProducerWarps * 32;
constexpr int kEpilogueThreads = kEpilogueWarps * 32;
constexpr int kMaxN = 256;              // MMA N limit for M = 128
constexpr int kLoadItems = 3;           // producer items (8 FP64 each) in flight per thread
constexpr uint64_t kWaitNs = 1000000000ull;  // default pipeline wait limit: 1 s

// Set by a CTA whose pipeline wait ran out (one word per device).
__device__ int g_tc_timeout = 0;

struct Shape {
  int kp;        // K of one piece (nao rounded up to 16)
  int kc;        // stored depth 2 kp ([hi | lo])
  int n;         // MMA N (nmo rounded up to 16)
  int acc_cols;  // TMEM columns of one accumulator: power of two >= max(32, n)
  int64_t a_off[2], b_off, st_off, bar_off, smem;
};

// Epilogue staging: per epilogue warp a 32-row x 16-column FP32 block, rows
// kStageStride floats apart (20: the 16-byte row stores of a quarter warp fall
// on distinct banks).
constexpr int kStageStride = 20;
constexpr int kStageBytes = 32 * kStageStride * 4;

// barriers at bar_off: full[2], empty[2], dfull[2], dempty[2] (8 B each), then
// the TMEM address (4 B) and the abort flag (4 B)
constexpr int kBarFull = 0, kBarEmpty = 2, kBarDFull = 4, kBarDEmpty = 6, kNumBars = 8;

__host__ __device__ inline Shape shape(int nao, int nmo) {
  Shape s;
  s.kp = (nao + 15) & ~15;
  s.kc = 2 * s.kp;
  s.n = (nmo + 15) & ~15;
  s.acc_cols = 32;
  while (s.acc_cols < s.n) s.acc_cols *= 2;
  const int64_t a_bytes = (int64_t)kM * s.kc * 2;
  s.a_off[0] = 0;
  s.a_off[1] = a_bytes;
  s.b_off = 2 * a_bytes;
  s.st_off = s.b_off + (int64_t)s.n * s.kc * 2;
  s.bar_off = s.st_off + (int64_t)kEpilogueWarps * kStageBytes;
  s.smem = s.bar_off + kNumBars * 8 + 8 + 1024;  // 1 KB for base alignment
  return s;
}

// Byte offset of the 16-byte chunk holding elements (r, 8 c .. 8 c + 7) of a
// K-major operand of stored depth kc in the no-swizzle canonical layout.
__host__ __device__ inline uint32_t chunk_offset(int r, int c, int kc) {
  return (uint32_t)((r >> 3) * (kc * 16) + c * 128 + (r & 7) * 16);
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
// shared address `bar`. Returns false after limit_ns or when another thread
// raised the abort flag (and then raises it itself). A limit of 0 gives up at
// once, without polling (the pipeline aborts deterministically).
__device__ inline bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                 uint64_t limit_ns) {
  if (limit_ns == 0) {
    *abort_flag = 1;
    return false;
  }
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
    if (*abort_flag) return false;
    if (global_ns() - t0 > limit_ns) {
      *abort_flag = 1;
      return false;
    }
  }
}

__device__ inline void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

__device__ inline void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
      : "memory");
}

__device__ inline uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// f32_trunc and f64_from_f32 (integer conversions that keep the FP64 pipe
// free) are shared with the fused kernels: qmc_device.cuh.

// Split 8 FP64 values into their BF16 hi and lo parts, packed as 16 bytes each.
// The split runs in FP32 (x truncated to FP32 first: its 24 bits hold the 16
// that hi + lo keep, and x_f - hi is exact in FP32), with no FP64 arithmetic.
__device__ inline void split8(const double (&v)[8], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float f0 = f32_trunc(v[2 * j]), f1 = f32_trunc(v[2 * j + 1]);
    const __nv_bfloat16 h0 = __float2bfloat16(f0), h1 = __float2bfloat16(f1);
    const __nv_bfloat16 l0 = __float2bfloat16(f0 - __bfloat162float(h0));
    const __nv_bfloat16 l1 = __float2bfloat16(f1 - __bfloat162float(h1));
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

// FP64 values (row, 8 c .. 8 c + 7) of a row-major [nrows][nao] array, zero
// outside it; 16-byte loads when the chunk is 16-byte aligned.
__device__ inline void load8(const double* __restrict__ ao, int64_t row, int64_t nrows, int nao,
                             int c, double (&v)[8]) {
  const int k0 = c * 8;
  if (row < nrows && k0 + 8 <= nao) {
    const double* src = ao + row * nao + k0;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double2 t = __ldg(reinterpret_cast<const double2*>(src) + j);
        v[2 * j] = t.x;
        v[2 * j + 1] = t.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = __ldg(src + j);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j)
      v[j] = (row < nrows && k0 + j < nao) ? __ldg(ao + row * nao + k0 + j) : 0.0;
  }
}

// Bounded wait used once, at exit after an abort, for the tensor core to
// finish the last committed MMA chain before TMEM is released.
__device__ inline void mbar_wait_final(uint32_t bar, uint32_t parity) {
  volatile int never = 0;
  mbar_wait(bar, parity, &never, kWaitNs);
}

__global__ void __launch_bounds__(kThreads, 1) mo_tc_kernel(const double* __restrict__ ao,
                                                            int64_t nrows, int nao, int nmo,
                                                            const double* __restrict__ mo_scf,
                                                            const double* __restrict__ mo_mod,
                                                            double* __restrict__ mo, int vec,
                                                            uint64_t wait_ns) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const Shape S = shape(nao, nmo);
  // 1 KB-aligned base (the dynamic shared-memory window is only 16-byte aligned)
  const uint32_t raw_addr = (uint32_t)__cvta_generic_to_shared(smem_raw);
  const uint32_t pad = (1024u - (raw_addr & 1023u)) & 1023u;
  unsigned char* smem = smem_raw + pad;
  const uint32_t base = raw_addr + pad;
  const uint32_t b_addr = base + (uint32_t)S.b_off;
  const uint32_t bars = base + (uint32_t)S.bar_off;  // mbarrier k at bars + 8 k
  const uint32_t tmem_slot_addr = bars + kNumBars * 8;
  volatile uint32_t* tmem_slot =
      reinterpret_cast<volatile uint32_t*>(smem + S.bar_off + kNumBars * 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + S.bar_off + kNumBars * 8 + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cpk = S.kp >> 3;  // 16-byte chunks per piece and row
  const int64_t ntiles = (nrows + kM - 1) / kM;

  // -- set-up: two TMEM accumulators (warp 8), mbarriers, B = [W_hi | W_lo] -
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     tmem_slot_addr),
                 "r"((uint32_t)(2 * S.acc_cols))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    const uint32_t counts[kNumBars] = {kProducerThreads, kProducerThreads, 1, 1, 1, 1,
                                       kEpilogueThreads, kEpilogueThreads};
    for (int k = 0; k < kNumBars; ++k)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bars + 8 * k),
                   "r"(counts[k])
                   : "memory");
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
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
    *reinterpret_cast<uint4*>(smem + S.b_off + chunk_offset(n, c, S.kc)) = hi;
    *reinterpret_cast<uint4*>(smem + S.b_off + chunk_offset(n, cpk + c, S.kc)) = lo;
  }
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  int last = -1;  // MMA thread: index of the last tile whose chain was committed
  if (warp < kProducerWarps) {
    // -- producers: AO rows of tile i -> [hi | lo] into A buffer i % 2 ------
    const int nitems = kM * cpk;
    // q / cpk for q < 2^22 as the high word of q * ceil(2^32 / cpk) (cpk <= 32:
    // the rounding excess of the multiplier stays below one quotient step)
    const uint32_t mcpk = (uint32_t)((0x100000000ull + (uint64_t)cpk - 1) / (uint64_t)cpk);
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int b = i & 1, use = i >> 1;
      if (use > 0 &&
          !mbar_wait(bars + 8 * (kBarEmpty + b), (uint32_t)((use - 1) & 1), abort_flag, wait_ns))
        break;
      const int64_t row0 = tile * kM;
      unsigned char* A = smem + S.a_off[b];
      // kLoadItems items per thread and iteration: their 16-byte loads are all
      // issued before the first split, so that enough bytes are in flight
      for (int it = tid; it < nitems; it += kLoadItems * kProducerThreads) {
        double v[kLoadItems][8];
        // item iu: rows 8 (q / cpk) + iu % 8, chunk q % cpk of q = iu / 8
        auto row_of = [&](int iu) {
          return (int)__umulhi((uint32_t)iu >> 3, mcpk) * 8 + (iu & 7);
        };
        auto chunk_of = [&](int iu) {
          const uint32_t q = (uint32_t)iu >> 3;
          return (int)(q - __umulhi(q, mcpk) * (uint32_t)cpk);
        };
#pragma unroll
        for (int u = 0; u < kLoadItems; ++u) {
          const int iu = it + u * kProducerThreads;
          if (iu < nitems) load8(ao, row0 + row_of(iu), nrows, nao, chunk_of(iu), v[u]);
        }
#pragma unroll
        for (int u = 0; u < kLoadItems; ++u) {
          const int iu = it + u * kProducerThreads;
          if (iu < nitems) {
            const int r = row_of(iu), c = chunk_of(iu);
            uint4 hi, lo;
            split8(v[u], hi, lo);
            *reinterpret_cast<uint4*>(A + chunk_offset(r, c, S.kc)) = hi;
            *reinterpret_cast<uint4*>(A + chunk_offset(r, cpk + c, S.kc)) = lo;
          }
        }
      }
      fence_proxy_async();
      mbar_arrive(bars + 8 * (kBarFull + b));
    }
  } else if (warp == kMmaWarp) {
    // -- one thread issues the MMA chain of tile i into accumulator i % 2 ---
    if (lane == 0) {
      const uint32_t idesc = instr_desc(kM, S.n);
      const uint32_t lbo = 128, sbo = (uint32_t)S.kc * 16;
      const int spp = S.kp / 16;  // MMA steps per K segment
      int i = 0;
      for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
        const int b = i & 1, use = i >> 1;
        if (!mbar_wait(bars + 8 * (kBarFull + b), (uint32_t)(use & 1), abort_flag, wait_ns)) break;
        if (use > 0 && !mbar_wait(bars + 8 * (kBarDEmpty + b), (uint32_t)((use - 1) & 1),
                                  abort_flag, wait_ns))
          break;
        fence_after_sync();
        const uint32_t dt = tmem + (uint32_t)(b * S.acc_cols);
        const uint32_t a_base = base + (uint32_t)S.a_off[b];
        for (int s = 0; s < 3 * spp; ++s) {
          const int seg = s / spp, sub = s - seg * spp;
          // segments: (a_hi, b_hi), (a_hi, b_lo), (a_lo, b_hi)
          const int ap = seg == 2 ? 1 : 0, bp = seg == 1 ? 1 : 0;
          const uint64_t ad = smem_desc(a_base + (uint32_t)((ap * cpk + 2 * sub) * 128), lbo, sbo);
          const uint64_t bd = smem_desc(b_addr + (uint32_t)((bp * cpk + 2 * sub) * 128), lbo, sbo);
          const uint32_t acc = s > 0 ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
              : "memory");
        }
        mma_commit(bars + 8 * (kBarEmpty + b));
        mma_commit(bars + 8 * (kBarDFull + b));
        last = i;
      }
    }
    __syncwarp();
  } else {
    // -- epilogue: accumulator i % 2 -> registers -> FP64 rows --------------
    const int q = warp & 3, half = (warp - kMmaWarp - 1) >> 2;
    const int nchunk = S.n / 16;
    int i = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++i) {
      const int d = i & 1, use = i >> 1;
      bool ok = mbar_wait(bars + 8 * (kBarDFull + d), (uint32_t)(use & 1), abort_flag, wait_ns);
      ok = __all_sync(0xffffffffu, ok);  // tcgen05.ld below needs the whole warp
      if (!ok) break;
      fence_after_sync();
      const uint32_t dt = tmem + (uint32_t)(d * S.acc_cols) + ((uint32_t)(q * 32) << 16);
      const int64_t row0 = tile * kM + q * 32;  // this warp's 32 rows
      // transpose through shared memory: lane l holds row l's 16 columns after
      // tcgen05.ld; after the exchange, lane l writes columns 2 (l % 8), + 1 of
      // row 4 j + l / 8, so each store instruction covers four rows' 128
      // contiguous bytes instead of 16 bytes of 32 rows
      float* stg = reinterpret_cast<float*>(smem + S.st_off) +
                   (warp - kMmaWarp - 1) * (kStageBytes / 4);
      const int rsub = lane >> 3, csub = 2 * (lane & 7);
      for (int ch = half; ch < nchunk; ch += 2) {
        float v[16];
        tmem_ld16(dt + (uint32_t)(ch * 16), v);
#pragma unroll
        for (int j = 0; j < 4; ++j)
          *reinterpret_cast<float4*>(stg + lane * kStageStride + 4 * j) =
              make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        __syncwarp();
        const int col = ch * 16 + csub;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int r = 4 * j + rsub;
          const int64_t row = row0 + r;
          const float2 f = *reinterpret_cast<const float2*>(stg + r * kStageStride + csub);
          if (row < nrows && col < nmo) {
            double* dst = mo + row * nmo + col;
            if (vec) {  // nmo even: col + 1 < nmo and 16-byte alignment
              *reinterpret_cast<double2*>(dst) = make_double2(f64_from_f32(f.x), f64_from_f32(f.y));
            } else {
              dst[0] = f64_from_f32(f.x);
              if (col + 1 < nmo) dst[1] = f64_from_f32(f.y);
            }
          }
        }
        __syncwarp();
      }
      fence_before_sync();
      mbar_arrive(bars + 8 * (kBarDEmpty + d));
    }
  }

  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (*abort_flag) {
    // a wait ran out: this CTA's rows are written as NaN, the status word is
    // set, and the tensor core gets a bounded wait for its last committed
    // chain before TMEM is freed
    if (tid == 0) atomicExch(&g_tc_timeout, 1);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
      for (int idx = tid; idx < kM * nmo; idx += kThreads) {
        const int64_t row = tile * kM + idx / nmo;
        if (row < nrows) mo[row * nmo + idx % nmo] = __longlong_as_double(0x7ff8000000000000ll);
      }
    if (last >= 0) mbar_wait_final(bars + 8 * (kBarDFull + (last & 1)), (uint32_t)((last >> 1) & 1));
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
  }
  if (warp == kMmaWarp)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"((uint32_t)(2 * S.acc_cols))
                 : "memory");
}

}  // namespace tc
}  // namespace qmc

using namespace qmc;

namespace {
std::atomic<uint64_t> g_wait_limit_ns{qmc::tc::kWaitNs};
}

extern "C" {

uint64_t qmc_set_wait_limit_ns(uint64_t ns) { return g_wait_limit_ns.exchange(ns); }

int qmc_mo_eval_tc_status(void* stream) {
  if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) {
    cudaGetLastError();
    return QMC_ERR_LAUNCH;
  }
  int flag = 0;
  if (cudaMemcpyFromSymbol(&flag, tc::g_tc_timeout, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return QMC_ERR_LAUNCH;
  }
  if (!flag) return QMC_OK;
  const int zero = 0;
  if (cudaMemcpyToSymbol(tc::g_tc_timeout, &zero, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return QMC_ERR_LAUNCH;
  }
  return QMC_ERR_TIMEOUT;
}

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
  if (occ > 512 / (2 * S.acc_cols)) occ = 512 / (2 * S.acc_cols);
  const int64_t ntiles = (nrows + tc::kM - 1) / tc::kM;
  int64_t grid = (int64_t)nsm * occ;
  if (grid > ntiles) grid = ntiles;
  const int vec = (d->nmo % 2 == 0) && ((reinterpret_cast<uintptr_t>(mo) & 15) == 0);
  tc::mo_tc_kernel<<<(unsigned)grid, tc::kThreads, S.smem, (cudaStream_t)stream>>>(
      ao, nrows, d->nao, d->nmo, d->mo_scf, d->mo_modifier, mo, vec, g_wait_limit_ns.load());
  return launch_status();
}

}  // extern "C"
