// Pipelined tensor-core tile pass: 12-bit tiles, fused 4-qubit blocks as
// tcgen05 MMAs, two tiles in flight per CTA.
//
// A 16 x 16 complex block M on 4 tile bits is the real 32 x 32 matrix acting
// on the (re, im) pairs of the 16 amplitudes that differ only in those bits.
// The other 8 tile bits index 256 rows: the tile (2^12 amplitudes, 32 KB)
// is the A operand of two M = 128, N = 32, K = 32 MMAs (row bit 7 picks the
// half), stored K-major with the 128-byte swizzle; B is M's real form; the
// two 128 x 32 fp32 results accumulate in tensor memory.  fp32 accuracy
// comes from the three-term TF32 split
//   A B ~= A_hi B_hi + A_hi B_lo + A_lo B_hi,   x_hi = tf32(x), x_lo = tf32(x - x_hi),
// both parts rounded to nearest by the kernel (the tensor core would drop
// the low 13 mantissa bits, a bias toward zero that shrinks the norm over
// hundreds of ops).
// This replaces, for a whole fused block at once, the numpy passes of
// linalg.targeted_left_multiply (cirq-core/cirq/linalg/transformations.py:105-172)
// and the gates' _apply_unitary_ (cirq-core/cirq/ops/common_gates.py).
//
// One CTA per SM (448 threads) runs two independent slot pipelines; each
// slot (A_hi + A_lo, 64 KB) holds one tile and has its own warps:
//   4 epilogue warps  tcgen05.ld of their 32-lane quarter of the slot's
//                     accumulators, the pass's diagonal ops on CUDA cores,
//                     the hi/lo split, and the write of the next op's A
//                     operand in shared memory (or of the natural-order tile
//                     after the last op); they also split each loaded tile;
//   1 MMA warp        one thread issues the slot's MMAs and commits them to
//                     an mbarrier;
//   2 producer warps  cp.async loads of the slot's tiles into the first op's
//                     A layout, 16-byte streaming stores of finished tiles.
// The slots take alternate tiles, so the tensor pipe runs one slot's MMAs
// while the other slot's warps read back, split, load or store.
// Slot s has four mbarriers: full (loaded), ready (A written, accumulator
// free: next op may issue), done (MMAs complete), final (natural-order tile
// written).  Every wait is bounded: a wait that runs out raises the CTA's
// abort flag, every role leaves its loop, the MMA thread drains its
// outstanding MMAs (bounded), tensor memory is freed and the context's
// abort flag reports it to the host.

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "gbq_internal.cuh"
#include "gbq_tile.cuh"

namespace gbq {

namespace {

constexpr int kTL = GBQ_TC_TILE_BITS;  // 12
constexpr int kTS = 1 << kTL;          // amplitudes per tile
constexpr int kTBytes = kTS * 8;       // 32 KB
constexpr int kTHalfBytes = kTBytes / 2;
constexpr int kTMatBytes = 8192;       // one matrix: hi and lo real forms, 4 KB each
constexpr int kTMaxMats = GBQ_TC_MAX_MATS;
constexpr int kTEpi = 4, kTProd = 2;   // per slot: epilogue warps, producer warps
constexpr int kTMmaWarp0 = 2 * kTEpi;  // one MMA-issuing warp per slot
constexpr int kTProdWarp0 = kTMmaWarp0 + 2;
constexpr int kTThreads = 32 * (kTProdWarp0 + 2 * kTProd);
constexpr int kTProdThreads = 32 * kTProd;  // per slot
constexpr int kTSmem = 4 * kTBytes + kTMaxMats * kTMatBytes + 1024;
constexpr uint32_t kTTmemCols = 128;   // 2 slots x 2 halves x 32 columns
constexpr long kTSpin = 1L << 24;      // try_wait polls before a wait is given up
constexpr int kTNH = kTS >> 5;         // tile-index values of bits 5..11
// Instruction descriptor: D f32, A and B tf32, both K-major, N = 32, M = 128.
constexpr uint32_t kTIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

// Natural-order layout of a finished tile (pair index of tile index i):
// i ^ swizzle, the swizzle XORs bits 1..3 from tile bits 4..11 so that the
// pairs 2j, 2j + 1 stay adjacent for 16-byte loads.
__host__ __device__ constexpr uint32_t tc_nat_col(int b) {
  constexpr uint32_t sw[8] = {2, 4, 8, 6, 10, 12, 14, 2};
  return (1u << b) ^ (b >= 4 ? sw[b - 4] : 0u);
}

__device__ __forceinline__ uint32_t tsu32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: 128-byte swizzle, K-major, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ float tc_tf32(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(kTIdesc), "r"(acc));
}

__device__ __forceinline__ void tc_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool tc_try(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded blocking wait (one thread); false when it ran out or *abort rose.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile int* abort) {
  for (long it = 0; it < kTSpin; ++it) {
    if (tc_try(bar, parity)) return true;
    if ((it & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  return false;
}

// The same for a whole warp, with a warp-uniform result.
__device__ __forceinline__ bool tc_wait_warp(uint32_t bar, uint32_t parity, volatile int* abort) {
  for (long it = 0; it < kTSpin; ++it) {
    if (__all_sync(0xffffffffu, tc_try(bar, parity))) return true;
    if ((it & 255) == 255 && __any_sync(0xffffffffu, *abort != 0)) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
        "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
        "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
        "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tc_fence_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// Epilogue of op o (or of the split stage, o = -1) for slot s: reads the
// accumulators, applies the op's diagonal ops, writes the next layout.
__device__ __forceinline__ void tc_epilogue_op(const TcArgs& a, int o, uint32_t tmem_slot_col, int w, int l,
                                               uint64_t gbase, float2* hi, float2* lo) {
  const TcOpDev& op = a.ops[o];
  uint32_t v0[32], v1[32];
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t taddr = tmem_slot_col + ((uint32_t)(32 * w) << 16);
  tc_ld32(taddr, v0);
  tc_ld32(taddr + 32, v1);
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
  float2 amp[32];
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    amp[c] = make_float2(__uint_as_float(v0[2 * c]), __uint_as_float(v0[2 * c + 1]));
    amp[16 + c] = make_float2(__uint_as_float(v1[2 * c]), __uint_as_float(v1[2 * c + 1]));
  }
  const int mrow = 32 * w + l;  // row bits 0..6; row bit 7 = the half
  for (int dd = 0; dd < op.ndiag; ++dd) {
    const TcDiagDev& dg = a.diags[op.diag0 + dd];
    uint32_t ib = 0;
    for (int j = 0; j < dg.k; ++j)
      if (dg.dext[j] >= 0) ib |= (uint32_t)((gbase >> dg.dext[j]) & 1ull) << j;
#pragma unroll
    for (int q = 0; q < 7; ++q)
      if ((mrow >> q) & 1) ib ^= dg.trow[q];
    const float2* tab = a.ti.mats + dg.mat;
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      uint32_t idx = ib;
      if (e & 1) idx ^= dg.ttgt[0];
      if (e & 2) idx ^= dg.ttgt[1];
      if (e & 4) idx ^= dg.ttgt[2];
      if (e & 8) idx ^= dg.ttgt[3];
      if (e & 16) idx ^= dg.trow[7];
      amp[e] = cmul(__ldg(tab + idx), amp[e]);
    }
  }
  uint32_t pb = 0;
#pragma unroll
  for (int q = 0; q < 7; ++q)
    if ((mrow >> q) & 1) pb ^= op.rnext[q];
  const bool last = o + 1 == a.nops;
#pragma unroll
  for (int e = 0; e < 32; ++e) {
    uint32_t pos = pb;
    if (e & 1) pos ^= op.tnext[0];
    if (e & 2) pos ^= op.tnext[1];
    if (e & 4) pos ^= op.tnext[2];
    if (e & 8) pos ^= op.tnext[3];
    if (e & 16) pos ^= op.rnext[7];
    if (last) {
      hi[pos] = amp[e];
    } else {
      const float2 hv = make_float2(tc_tf32(amp[e].x), tc_tf32(amp[e].y));
      hi[pos] = hv;
      lo[pos] = make_float2(tc_tf32(amp[e].x - hv.x), tc_tf32(amp[e].y - hv.y));
    }
  }
}

__global__ void __launch_bounds__(kTThreads, 1) k_tc_pass(const __grid_constant__ TcArgs a) {
  extern __shared__ unsigned char smraw[];
  __shared__ uint64_t ttab[3 * kTileTab];
  __shared__ uint64_t hoff[kTNH];   // global offset of tile index (j << 5)
  __shared__ uint16_t lhigh[kTNH];  // first-op layout pair index of tile index (j << 5)
  __shared__ uint16_t nhigh[kTNH];  // natural layout pair index of tile index (j << 5)
  __shared__ __align__(8) uint64_t bar_full[2], bar_ready[2], bar_done[2], bar_final[2], bar_drain[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  unsigned char* bmem = base + 4 * kTBytes;
  const int t = threadIdx.x;
  const int warp = __shfl_sync(0xffffffffu, t >> 5, 0), lane = t & 31;
  const TileInfo& ti = a.ti;

  for (int e = t; e < 3 * kTileTab; e += kTThreads) {
    const int part = e / kTileTab;
    ttab[e] = tile_base(ti, (int64_t)(e % kTileTab) << (8 * part));
  }
  for (int j = t; j < kTNH; j += kTThreads) {
    hoff[j] = lin_off<kTL>(ti, (uint32_t)j << 5);
    uint32_t lp = 0, np = 0;
#pragma unroll
    for (int b = 5; b < kTL; ++b)
      if ((j >> (b - 5)) & 1) {
        lp ^= a.lcol[b];
        np ^= tc_nat_col(b);
      }
    lhigh[j] = (uint16_t)lp;
    nhigh[j] = (uint16_t)np;
  }
  // B operands: real forms of every matrix of the pass, hi and lo parts
  for (int o = 0; o < a.nops; ++o) {
    const TcOpDev& op = a.ops[o];
    for (int s = 0; s < (1 << op.nsel); ++s) {
      const float2* src = ti.mats + op.mat + (int64_t)s * 256;
      unsigned char* bh = bmem + (op.bslot + s) * kTMatBytes;
      for (int e = t; e < 1024; e += kTThreads) {
        const int rp = e >> 5, kp = e & 31;
        const float2 m = src[(rp >> 1) * 16 + (kp >> 1)];
        const float v = (kp & 1) == 0 ? ((rp & 1) == 0 ? m.x : m.y) : ((rp & 1) == 0 ? -m.y : m.x);
        const float h = tc_tf32(v);
        const uint32_t off = (uint32_t)rp * 128u + ((((uint32_t)kp >> 2) ^ ((uint32_t)rp & 7u)) << 4) +
                             ((uint32_t)kp & 3u) * 4u;
        *reinterpret_cast<float*>(bh + off) = h;
        *reinterpret_cast<float*>(bh + 4096 + off) = tc_tf32(v - h);
      }
    }
  }
  if (t == 0) {
    abort_sh = 0;
    for (int s = 0; s < 2; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(tsu32(&bar_full[s])), "r"(kTProdThreads));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(tsu32(&bar_ready[s])), "r"(32 * kTEpi));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(tsu32(&bar_done[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(tsu32(&bar_final[s])), "r"(32 * kTEpi));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(tsu32(&bar_drain[s])));
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == kTMmaWarp0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tsu32(&tmem_base_sh)),
                 "r"(kTTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  tc_fence_async();
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_sh;
  volatile int* abort = &abort_sh;
  const int64_t step = gridDim.x;
  const int64_t count = blockIdx.x < ti.ntiles ? (ti.ntiles - 1 - blockIdx.x) / step + 1 : 0;

  // Two independent slot pipelines: slot s owns epilogue warps 4s..4s+3,
  // MMA warp kTMmaWarp0 + s and producer warps kTProdWarp0 + kTProd * s ...,
  // and processes this CTA's tiles k = s, s + 2, s + 4, ...
  int s = 0, role = 0;
  if (warp < 2 * kTEpi) {
    s = warp / kTEpi;
    role = 0;
  } else if (warp < kTMmaWarp0 + 2) {
    s = warp - kTMmaWarp0;
    role = 1;
  } else {
    s = (warp - kTProdWarp0) / kTProd;
    role = 2;
  }
  float2* Ahi = reinterpret_cast<float2*>(base + s * 2 * kTBytes);
  float2* Alo = reinterpret_cast<float2*>(base + s * 2 * kTBytes + kTBytes);
  const uint32_t full = tsu32(&bar_full[s]), ready = tsu32(&bar_ready[s]), done = tsu32(&bar_done[s]),
                 fin = tsu32(&bar_final[s]);

  if (role == 0) {
    // ---- epilogue warps of slot s
    const int w = warp & 3;
    const int et = t - 32 * kTEpi * s;  // 0..127 within the slot's group
    uint32_t ndone = 0;
    for (int64_t k = s, it = 0; k < count; k += 2, ++it) {
      if (!tc_wait_warp(full, (uint32_t)(it & 1), abort)) break;
      const uint64_t gbase = tile_base_fast(ttab, blockIdx.x + k * step);
      // three-term split of the loaded tile in place (16-byte chunks)
      float4* h4 = reinterpret_cast<float4*>(Ahi);
      float4* l4 = reinterpret_cast<float4*>(Alo);
#pragma unroll 4
      for (int f = et; f < kTS / 2; f += 32 * kTEpi) {
        const float4 v = h4[f];
        const float4 hv = make_float4(tc_tf32(v.x), tc_tf32(v.y), tc_tf32(v.z), tc_tf32(v.w));
        h4[f] = hv;
        l4[f] = make_float4(tc_tf32(v.x - hv.x), tc_tf32(v.y - hv.y), tc_tf32(v.z - hv.z), tc_tf32(v.w - hv.w));
      }
      tc_fence_async();
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      tc_arrive(ready);
      bool ok = true;
      for (int o = 0; o < a.nops; ++o) {
        if (!tc_wait_warp(done, ndone & 1u, abort)) {
          ok = false;
          break;
        }
        ++ndone;
        tc_epilogue_op(a, o, tmem + (uint32_t)(64 * s), w, lane, gbase, Ahi, Alo);
        if (o + 1 < a.nops) tc_fence_async();
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        tc_arrive(o + 1 < a.nops ? ready : fin);
      }
      if (!ok) break;
    }
  } else if (role == 1) {
    // ---- MMA issuer of slot s: one thread
    if (lane == 0) {
      uint32_t nready = 0;
      bool issued = false;
      for (int64_t k = s; k < count && !*abort; k += 2) {
        const uint64_t gbase = tile_base_fast(ttab, blockIdx.x + k * step);
        bool ok = true;
        for (int o = 0; o < a.nops; ++o) {
          if (!tc_wait(ready, nready & 1u, abort)) {
            ok = false;
            break;
          }
          ++nready;
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const TcOpDev& op = a.ops[o];
          uint32_t sel = 0;
          for (int q = 0; q < op.nsel; ++q) sel |= (uint32_t)((gbase >> op.selg[q]) & 1ull) << q;
          const uint32_t bh = tsu32(bmem) + (uint32_t)(op.bslot + (int)sel) * kTMatBytes;
          const uint32_t ah = tsu32(Ahi), al = tsu32(Alo);
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
            for (int p = 0; p < 3; ++p) {
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                // the two halves' accumulation chains interleave
                const uint32_t A = (p == 2 ? al : ah) + (uint32_t)(h * kTHalfBytes);
                const uint32_t B = p == 1 ? bh + 4096 : bh;
                tc_mma(tmem + (uint32_t)(64 * s + 32 * h), tc_desc(A + 32 * ks), tc_desc(B + 32 * ks),
                       (p | ks) != 0);
              }
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(done)
                       : "memory");
          issued = true;
        }
        if (!ok) break;
      }
      if (issued) {
        // every MMA issued so far completes before tensor memory is freed
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                         tsu32(&bar_drain[s]))
                     : "memory");
        volatile int never = 0;
        tc_wait(tsu32(&bar_drain[s]), 0, &never);
      }
    }
  } else {
    // ---- producers of slot s: loads into the first op's layout, natural-order stores
    const int pt = t - 32 * (kTProdWarp0 + kTProd * s);  // 0..kTProdThreads-1
    const int pw = pt >> 5;
    const uint64_t lo_l = lin_off<kTL>(ti, (uint32_t)lane);
    uint32_t lp_l = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b)
      if ((lane >> b) & 1) lp_l ^= a.lcol[b];
    auto load = [&](int64_t kk) {
      const uint64_t gb = tile_base_fast(ttab, blockIdx.x + kk * step);
      const float2* g = a.psi + gb + lo_l;
#pragma unroll 4
      for (int jj = pw; jj < kTNH; jj += kTProd) {
        const uint32_t sa = tsu32(Ahi + (lp_l ^ lhigh[jj]));
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(g + hoff[jj]) : "memory");
      }
      asm volatile("cp.async.mbarrier.arrive.noinc.shared.b64 [%0];\n" ::"r"(full) : "memory");
    };
    if (s < count) load(s);
    for (int64_t kk = s, it = 0; kk < count; kk += 2, ++it) {
      const bool ok = tc_wait(fin, (uint32_t)(it & 1), abort);
      // every producer of the slot leaves at the same iteration (they meet at a named barrier below)
      uint32_t any_fail;
      asm volatile(
          "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, %2, %3, p;\n"
          "selp.u32 %0, 1, 0, q;\n}\n"
          : "=r"(any_fail)
          : "r"((uint32_t)!ok), "r"(4 + s), "n"(kTProdThreads)
          : "memory");
      if (any_fail) break;
      const uint64_t gb = tile_base_fast(ttab, blockIdx.x + kk * step);
#pragma unroll 4
      for (int j = pt; j < kTS / 2; j += kTProdThreads) {
        const uint32_t i2 = (uint32_t)(2 * j);
        uint32_t np = nhigh[i2 >> 5];
        uint64_t go = hoff[i2 >> 5];
#pragma unroll
        for (int b = 1; b < 5; ++b)
          if ((i2 >> b) & 1) {
            np ^= tc_nat_col(b);
            go += ti.gw[b];
          }
        const float4 v = *reinterpret_cast<const float4*>(Ahi + np);
        __stcs(reinterpret_cast<float4*>(a.psi + gb + go), v);
      }
      // every producer has read the slot before any refills it
      asm volatile("bar.sync %0, %1;\n" ::"r"(2 + s), "n"(kTProdThreads) : "memory");
      if (kk + 2 < count) load(kk + 2);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (t == 0 && *abort && a.abort) atomicExch(a.abort, 1);
  if (warp == kTMmaWarp0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTTmemCols));
  }
}

int tc_fail(const std::string& msg) {
  set_error(msg);
  return GBQ_ERR_ARG;
}

// rank over GF(2) of the low 4 bits of v[0..n-1]
int tc_rank4(const uint32_t* v, int n) {
  uint32_t basis[4] = {0, 0, 0, 0};
  int r = 0;
  for (int i = 0; i < n; ++i) {
    uint32_t x = v[i] & 15u;
    for (int b = 3; b >= 0; --b)
      if ((x >> b) & 1u) {
        if (!basis[b]) {
          basis[b] = x;
          ++r;
          break;
        }
        x ^= basis[b];
      }
  }
  return r;
}

}  // namespace

// Pair index column (8-byte units) of tile bit b in the A layout of an MMA op
// with targets tg[0..3] and row order rows[0..7]: target p -> 1 << p; row q < 3
// -> (16 << q) ^ (2 << q) (the 128-byte swizzle of the 16-byte chunk); row
// q = 3..6 -> 16 << q; row 7 (the half) -> 2048.
static uint32_t tc_op_col(const int* tg, const int* rows, int b) {
  for (int p = 0; p < 4; ++p)
    if (tg[p] == b) return 1u << p;
  for (int q = 0; q < 8; ++q)
    if (rows[q] == b) {
      if (q < 3) return (16u << q) ^ (2u << q);
      if (q < 7) return 16u << q;
      return 2048u;
    }
  return 0;
}

int build_tc_args(const gbq_pass& p, const gbq_op* ops, int nbits, const TileInfo& ti, uint64_t inmask,
                  TcArgs& A) {
  memset(&A, 0, sizeof(A));
  A.ti = ti;
  if (p.L != kTL) return tc_fail("pass: pipelined tensor-core passes use 12-bit tiles");
  if (p.m < 5) return tc_fail("pass: pipelined tensor-core passes need m >= 5");
  const gbq_op* po = ops + p.op_begin;
  if (p.op_count < 1 || po[0].kind != GBQ_OP_MMA)
    return tc_fail("pass: the first op of a tensor-core pass must be an MMA op");
  int tg[GBQ_MAX_MMA_OPS][4];
  int nm = 0, nd = 0, slots = 0;
  for (int o = 0; o < p.op_count; ++o) {
    const gbq_op& op = po[o];
    if (op.kind == GBQ_OP_MMA) {
      if (nm >= GBQ_MAX_MMA_OPS) return tc_fail("pass: too many MMA ops (max 8)");
      if (op.k != 4) return tc_fail("op: an MMA op acts on exactly 4 tile bits");
      if (op.nsel < 0 || op.nsel > 3) return tc_fail("op: MMA selectors must number 0..3");
      if (op.mat < 0) return tc_fail("op: negative matrix offset");
      uint32_t seen = 0;
      for (int j = 0; j < 4; ++j) {
        const int b = op.bits[j];
        if (b < 0 || b >= kTL || ((seen >> b) & 1u)) return tc_fail("op: MMA target bits must be distinct tile bits");
        seen |= 1u << b;
        tg[nm][j] = b;
      }
      TcOpDev& d = A.ops[nm];
      d.mat = op.mat;
      d.nsel = op.nsel;
      for (int s = 0; s < op.nsel; ++s) {
        const int c = op.sel[s];
        const int g = -c - 1;
        if (c >= 0 || g >= nbits || ((inmask >> g) & 1ull))
          return tc_fail("op: MMA selectors must be global bits outside the tile");
        d.selg[s] = (int8_t)g;
      }
      d.bslot = (int16_t)slots;
      slots += 1 << op.nsel;
      if (slots > kTMaxMats)
        return tc_fail("pass: MMA matrices exceed " + std::to_string(kTMaxMats) + " per pass");
      d.diag0 = (int8_t)nd;
      ++nm;
    } else if (op.kind == GBQ_OP_DIAG) {
      if (op.k < 1 || op.k > GBQ_MAX_DIAG_K) return tc_fail("op: diagonal width must be 1..8");
      if (op.mat < 0) return tc_fail("op: negative matrix offset");
      if (nd >= GBQ_MAX_OPS_PER_PASS) return tc_fail("pass: too many diagonal ops");
      TcDiagDev& d = A.diags[nd];
      d.mat = op.mat;
      d.k = op.k;
      for (int j = 0; j < 8; ++j) d.dext[j] = -1;
      for (int j = 0; j < op.k; ++j) {
        const int c = op.bits[j];
        if (c >= kTL) return tc_fail("op: diagonal bit code out of range");
        if (c < 0) {
          const int g = -c - 1;
          if (g >= nbits || ((inmask >> g) & 1ull)) return tc_fail("op: diagonal global bit invalid");
          d.dext[j] = (int8_t)g;
        }
      }
      A.ops[nm - 1].ndiag++;
      ++nd;
    } else {
      return tc_fail("pass: a tensor-core pass holds only MMA and DIAG ops");
    }
  }
  A.nops = nm;
  A.ndiag = nd;
  A.nmats = slots;
  // Row orders, last op first.  The read-back of op o writes, per warp, the
  // 32 rows whose row bits 0..4 are the lane bits; those bits should have
  // independent bank columns (low 4 bits of the pair index) in the layout
  // written to, so that a half-warp hits 16 distinct bank pairs.
  int rows[GBQ_MAX_MMA_OPS][8];
  for (int o = nm - 1; o >= 0; --o) {
    int nt[8], c = 0;
    for (int b = 0; b < kTL; ++b)
      if (b != tg[o][0] && b != tg[o][1] && b != tg[o][2] && b != tg[o][3]) nt[c++] = b;
    auto next_col = [&](int b) -> uint32_t {
      return o + 1 < nm ? tc_op_col(tg[o + 1], rows[o + 1], b) : tc_nat_col(b);
    };
    int best = -1, bi[4] = {0, 1, 2, 3};
    for (int i0 = 0; i0 < 8; ++i0)
      for (int i1 = i0 + 1; i1 < 8; ++i1)
        for (int i2 = i1 + 1; i2 < 8; ++i2)
          for (int i3 = i2 + 1; i3 < 8; ++i3) {
            const uint32_t v[4] = {next_col(nt[i0]), next_col(nt[i1]), next_col(nt[i2]), next_col(nt[i3])};
            const int r = tc_rank4(v, 4);
            if (r > best) {
              best = r;
              bi[0] = i0, bi[1] = i1, bi[2] = i2, bi[3] = i3;
            }
          }
    bool used[8] = {false, false, false, false, false, false, false, false};
    for (int q = 0; q < 4; ++q) {
      rows[o][q] = nt[bi[q]];
      used[bi[q]] = true;
    }
    int q = 4;
    for (int i = 0; i < 8; ++i)
      if (!used[i]) rows[o][q++] = nt[i];
  }
  for (int o = 0; o < nm; ++o) {
    TcOpDev& d = A.ops[o];
    for (int j = 0; j < 4; ++j)
      d.tnext[j] = (uint16_t)(o + 1 < nm ? tc_op_col(tg[o + 1], rows[o + 1], tg[o][j]) : tc_nat_col(tg[o][j]));
    for (int q = 0; q < 8; ++q)
      d.rnext[q] = (uint16_t)(o + 1 < nm ? tc_op_col(tg[o + 1], rows[o + 1], rows[o][q]) : tc_nat_col(rows[o][q]));
  }
  for (int b = 0; b < kTL; ++b) A.lcol[b] = (uint16_t)tc_op_col(tg[0], rows[0], b);
  // diagonal table-index columns in the row/target coordinates of their MMA op
  {
    int o = -1, seen_d = 0;
    for (int i = 0; i < p.op_count; ++i) {
      const gbq_op& op = po[i];
      if (op.kind == GBQ_OP_MMA) {
        ++o;
        continue;
      }
      TcDiagDev& d = A.diags[seen_d++];
      for (int j = 0; j < op.k; ++j) {
        const int c = op.bits[j];
        if (c < 0) continue;
        bool placed = false;
        for (int pp = 0; pp < 4; ++pp)
          if (tg[o][pp] == c) {
            d.ttgt[pp] |= (uint16_t)(1u << j);
            placed = true;
          }
        for (int q = 0; q < 8; ++q)
          if (rows[o][q] == c) {
            d.trow[q] |= (uint16_t)(1u << j);
            placed = true;
          }
        if (!placed) return tc_fail("op: internal diagonal placement error");
      }
    }
  }
  return GBQ_OK;
}

int launch_tc_pass(Ctx* c, const TcArgs& a) {
  static int ready = 0;
  cudaError_t e;
  if (!ready) {
    e = cudaFuncSetAttribute(k_tc_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, kTSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tc_pass)");
    e = cudaFuncSetAttribute(k_tc_pass, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tc_pass carveout)");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tc_pass, kTThreads, kTSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor(k_tc_pass)");
    if (nb < 1) return tc_fail("k_tc_pass does not fit an SM");
    if (getenv("GBQ_DEBUG")) {
      cudaFuncAttributes fa;
      cudaFuncGetAttributes(&fa, k_tc_pass);
      fprintf(stderr, "k_tc_pass: %d blocks/SM, %d B dynamic smem, %d regs, %zu B static\n", nb, kTSmem,
              fa.numRegs, fa.sharedSizeBytes);
    }
    ready = 1;
  }
  int64_t grid = (int64_t)c->sm_count;  // one CTA per SM (tensor memory and shared memory)
  if (grid > a.ti.ntiles) grid = a.ti.ntiles;
  k_tc_pass<<<(unsigned)grid, kTThreads, kTSmem, c->stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_tc_pass launch");
  c->launches += 1;
  return GBQ_OK;
}

}  // namespace gbq
