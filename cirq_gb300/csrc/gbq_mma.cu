// Tensor-core tile pass: fused 4-qubit blocks applied with tcgen05 MMAs.
//
// A 16 x 16 complex matrix M acting on 4 tile bits is a real 32 x 32 matrix
// acting on the (re, im) pairs of the 16 amplitudes that differ only in those
// bits.  The tile (2^11 amplitudes, 16 KB) sits in shared memory as the A
// operand of one M = 128, N = 32 MMA: row n holds the 16 amplitudes whose
// other 7 tile bits spell n, stored (re, im, re, im, ...) -- K-major with the
// 128-byte swizzle.  B is the real form of M (N = 32 output components x K =
// 32 input components, also K-major).  D (128 x 32 fp32) accumulates in
// tensor memory (32 columns), is read back with tcgen05.ld and written to
// shared memory in the layout of the next op (or in natural order after the
// last op).  fp32 accuracy comes from the three-term TF32 split
//   A B ~= A_hi B_hi + A_hi B_lo + A_lo B_hi,   x_hi = tf32(x), x_lo = x - x_hi,
// with every x_hi rounded to TF32 by the kernel itself (relative error of
// one product ~2^-21).
//
// Diagonal ops of the pass are applied on the CUDA cores to the result of
// the MMA op before them, while it is in registers.  The host picks each
// op's row order (which non-target tile bits become the lane bits of the
// read-back) so that the shared-memory writes of a half-warp fall in 16
// distinct bank pairs wherever the bit assignment allows it.
//
// One elected thread issues the MMAs and commits them to an mbarrier; every
// wait on it is bounded.  A wait that runs out sets the context's abort flag,
// the CTA drains its copies, frees its tensor memory and returns.

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "gbq_internal.cuh"
#include "gbq_tile.cuh"

namespace gbq {

namespace {

constexpr int kML = GBQ_MMA_TILE_BITS;  // 11
constexpr int kMTS = 1 << kML;          // amplitudes per tile
constexpr int kMTileBytes = kMTS * 8;   // 16 KB
constexpr int kMMatBytes = 8192;        // one matrix: hi and lo real forms, 4 KB each
constexpr int kMSmem = 3 * kMTileBytes + GBQ_MAX_MMA_MATS * kMMatBytes + 1024;
constexpr long kSpinLimit = 1L << 26;   // mbarrier polls before a wait is given up
// Instruction descriptor: D f32, A and B tf32, both K-major, N = 32, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);
// Natural-order layout used before the final store: amplitude i at
// i ^ swizzle, the swizzle XORs bits 1..3 from tile bits 4..10 (pairs 2m,
// 2m + 1 stay adjacent for 16-byte stores).
// Swizzle columns of tile bits 4..10, 4 bits each: 2, 4, 8, 6, 10, 12, 14.
constexpr uint32_t kNatSwz = 0xECA6842u;

__host__ __device__ constexpr uint32_t nat_col(int b) {
  return (1u << b) ^ (b >= 4 ? (kNatSwz >> (4 * (b - 4))) & 15u : 0u);
}

__device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: 128-byte swizzle, K-major, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
      "[%16];\n"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void fence_to_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}

__global__ void __launch_bounds__(kThreads, 2) k_mma_pass(const __grid_constant__ MmaArgs a) {
  extern __shared__ unsigned char smraw[];
  __shared__ uint64_t ttab[3 * kTileTab];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t)1023);
  unsigned char* stage[2] = {base, base + kMTileBytes};
  unsigned char* lo_buf = base + 2 * kMTileBytes;
  unsigned char* bmem = base + 3 * kMTileBytes;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const TileInfo& ti = a.ti;

  tile_tables_build(ti, ttab);
  // B operands: real forms of every matrix of the pass, hi and lo parts.
  for (int o = 0; o < a.nops; ++o) {
    const MmaOpDev& op = a.ops[o];
    for (int s = 0; s < (1 << op.nsel); ++s) {
      const float2* src = ti.mats + op.mat + (int64_t)s * 256;
      unsigned char* bh = bmem + (op.bslot + s) * kMMatBytes;
      for (int e = t; e < 1024; e += kThreads) {
        const int rp = e >> 5, kp = e & 31;
        const float2 m = src[(rp >> 1) * 16 + (kp >> 1)];
        const float v = (kp & 1) == 0 ? ((rp & 1) == 0 ? m.x : m.y) : ((rp & 1) == 0 ? -m.y : m.x);
        const float h = tf32_round(v);
        const uint32_t off = (uint32_t)rp * 128u + ((((uint32_t)kp >> 2) ^ ((uint32_t)rp & 7u)) << 4) +
                             ((uint32_t)kp & 3u) * 4u;
        *reinterpret_cast<float*>(bh + off) = h;
        *reinterpret_cast<float*>(bh + 4096 + off) = v - h;
      }
    }
  }
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(su32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;\n" ::"r"(su32(&tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  fence_to_async();
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  const uint32_t bar = su32(&mbar);

  // Per-thread load geometry: amplitude i = t + 256 s (s = 0..7).
  uint64_t goff_t = 0;
  uint32_t lpos_t = 0;
#pragma unroll
  for (int b = 0; b < 8; ++b)
    if ((t >> b) & 1) {
      goff_t += ti.gw[b];
      lpos_t ^= a.lcol[b];
    }
  // Store geometry: amplitude pair i = 2 (t + 256 q) (q = 0..3).
  uint64_t soff_t = 0;
#pragma unroll
  for (int b = 1; b < 9; ++b)
    if (((2 * t) >> b) & 1) soff_t += ti.gw[b];
  const uint32_t spos_t = nat_col(1) * ((t >> 0) & 1) ^ nat_col(2) * ((t >> 1) & 1) ^
                          nat_col(3) * ((t >> 2) & 1) ^ nat_col(4) * ((t >> 3) & 1) ^
                          nat_col(5) * ((t >> 4) & 1) ^ nat_col(6) * ((t >> 5) & 1) ^
                          nat_col(7) * ((t >> 6) & 1) ^ nat_col(8) * ((t >> 7) & 1);
  const int q4 = warp & 3, h = warp >> 2;
  const int nrow = 32 * q4 + lane;  // TMEM lane = row of A
  const uint32_t taddr = tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(16 * h);

  const int64_t step = gridDim.x;
  bool aborted = false;
  uint32_t phase = 0;
  auto issue_load = [&](int64_t tile, unsigned char* dst) {
    const uint64_t gb = tile_base_fast(ttab, tile);
    const float2* g = a.psi + gb + goff_t;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      uint64_t go = 0;
      uint32_t lp = lpos_t;
#pragma unroll
      for (int b = 0; b < 3; ++b)
        if ((s >> b) & 1) {
          go += ti.gw[8 + b];
          lp ^= a.lcol[8 + b];
        }
      cp_async8(reinterpret_cast<float2*>(dst) + lp, g + go);
    }
  };
  if ((int64_t)blockIdx.x < ti.ntiles) issue_load(blockIdx.x, stage[0]);
  cp_async_commit();
  int cur = 0;
  for (int64_t tile = blockIdx.x; tile < ti.ntiles; tile += step) {
    if (tile + step < ti.ntiles) issue_load(tile + step, stage[cur ^ 1]);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    unsigned char* sbuf = stage[cur];
    const uint64_t gbase = tile_base_fast(ttab, tile);
    // three-term split of the loaded tile
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float4* hp = reinterpret_cast<float4*>(sbuf) + t + kThreads * c;
      float4* lp = reinterpret_cast<float4*>(lo_buf) + t + kThreads * c;
      const float4 v = *hp;
      const float4 hv = make_float4(tf32_round(v.x), tf32_round(v.y), tf32_round(v.z), tf32_round(v.w));
      *hp = hv;
      *lp = make_float4(v.x - hv.x, v.y - hv.y, v.z - hv.z, v.w - hv.w);
    }
    fence_to_async();
    __syncthreads();
    for (int o = 0; o < a.nops; ++o) {
      const MmaOpDev& op = a.ops[o];
      if (t == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        uint32_t sel = 0;
        for (int s = 0; s < op.nsel; ++s) sel |= (uint32_t)((gbase >> op.selg[s]) & 1ull) << s;
        const uint32_t bh = su32(bmem) + (uint32_t)(op.bslot + (int)sel) * kMMatBytes;
        const uint32_t ah = su32(sbuf), al = su32(lo_buf);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const uint32_t A = p == 2 ? al : ah;
          const uint32_t B = p == 1 ? bh + 4096 : bh;
#pragma unroll
          for (int ks = 0; ks < 4; ++ks)
            mma_tf32(tmem, sw128_desc(A + 32 * ks), sw128_desc(B + 32 * ks), (p | ks) != 0);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                     : "memory");
      }
      const bool ok = mbar_wait(bar, phase);
      phase ^= 1u;
      if (__syncthreads_or(!ok)) {
        aborted = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      uint32_t v[16];
      tmem_ld16(taddr, v);
      float2 amp[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) amp[r] = make_float2(__uint_as_float(v[2 * r]), __uint_as_float(v[2 * r + 1]));
      // diagonal ops that follow this MMA op
      for (int dd = 0; dd < op.ndiag; ++dd) {
        const MmaDiagDev& dg = a.diags[op.diag0 + dd];
        uint32_t ib = 0;
        for (int j = 0; j < dg.k; ++j)
          if (dg.dext[j] >= 0) ib |= (uint32_t)((gbase >> dg.dext[j]) & 1ull) << j;
#pragma unroll
        for (int qb = 0; qb < 7; ++qb)
          if ((nrow >> qb) & 1) ib ^= dg.trow[qb];
        if (h) ib ^= dg.ttgt[3];
        const float2* tab = ti.mats + dg.mat;
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          uint32_t idx = ib;
          if (r & 1) idx ^= dg.ttgt[0];
          if (r & 2) idx ^= dg.ttgt[1];
          if (r & 4) idx ^= dg.ttgt[2];
          amp[r] = cmul(__ldg(tab + idx), amp[r]);
        }
      }
      uint32_t pb = h ? op.tnext[3] : 0u;
#pragma unroll
      for (int qb = 0; qb < 7; ++qb)
        if ((nrow >> qb) & 1) pb ^= op.rnext[qb];
      const bool last = o + 1 == a.nops;
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        uint32_t pos = pb;
        if (r & 1) pos ^= op.tnext[0];
        if (r & 2) pos ^= op.tnext[1];
        if (r & 4) pos ^= op.tnext[2];
        float2* hp = reinterpret_cast<float2*>(sbuf) + pos;
        if (last) {
          *hp = amp[r];
        } else {
          const float2 hv = make_float2(tf32_round(amp[r].x), tf32_round(amp[r].y));
          *hp = hv;
          reinterpret_cast<float2*>(lo_buf)[pos] = make_float2(amp[r].x - hv.x, amp[r].y - hv.y);
        }
      }
      fence_to_async();
      __syncthreads();
    }
    if (aborted) break;
    // natural-order tile -> global, 16-byte stores
    float2* g = a.psi + gbase + soff_t;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      uint64_t go = 0;
      uint32_t sp = spos_t;
      if (c & 1) {
        go += ti.gw[9];
        sp ^= nat_col(9);
      }
      if (c & 2) {
        go += ti.gw[10];
        sp ^= nat_col(10);
      }
      const float4 v = *reinterpret_cast<const float4*>(reinterpret_cast<float2*>(sbuf) + sp);
      __stcs(reinterpret_cast<float4*>(g + go), v);
    }
    __syncthreads();
    cur ^= 1;
  }
  cp_async_wait<0>();
  if (aborted && t == 0) atomicExch(a.abort, 1);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;\n" ::"r"(tmem));
}

int mma_fail(const std::string& msg) {
  set_error(msg);
  return GBQ_ERR_ARG;
}

int rank4(const uint32_t* v, int n) {
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

// Amplitude-position column of tile bit b in the layout of an MMA op with
// targets tg[0..3] and row order rows[0..6].
static uint32_t op_col(const int* tg, const int* rows, int b) {
  for (int p = 0; p < 4; ++p)
    if (tg[p] == b) return 1u << p;
  for (int q = 0; q < 7; ++q)
    if (rows[q] == b) return (1u << (4 + q)) ^ (q < 3 ? (2u << q) : 0u);
  return 0;
}

int build_mma_args(const gbq_pass& p, const gbq_op* ops, int nbits, const TileInfo& ti, uint64_t inmask,
                   MmaArgs& A) {
  memset(&A, 0, sizeof(A));
  A.ti = ti;
  if (p.L != kML) return mma_fail("pass: tensor-core passes use 11-bit tiles");
  if (p.m < 1) return mma_fail("pass: tensor-core passes need m >= 1");
  const gbq_op* po = ops + p.op_begin;
  if (p.op_count < 1 || po[0].kind != GBQ_OP_MMA)
    return mma_fail("pass: the first op of a tensor-core pass must be an MMA op");
  int tg[GBQ_MAX_MMA_OPS][4];
  int nm = 0, nd = 0, slots = 0;
  for (int o = 0; o < p.op_count; ++o) {
    const gbq_op& op = po[o];
    if (op.kind == GBQ_OP_MMA) {
      if (nm >= GBQ_MAX_MMA_OPS) return mma_fail("pass: too many MMA ops (max 8)");
      if (op.k != 4) return mma_fail("op: an MMA op acts on exactly 4 tile bits");
      if (op.nsel < 0 || op.nsel > 3) return mma_fail("op: MMA selectors must number 0..3");
      if (op.mat < 0) return mma_fail("op: negative matrix offset");
      uint32_t seen = 0;
      for (int j = 0; j < 4; ++j) {
        const int b = op.bits[j];
        if (b < 0 || b >= kML || ((seen >> b) & 1u)) return mma_fail("op: MMA target bits must be distinct tile bits");
        seen |= 1u << b;
        tg[nm][j] = b;
      }
      MmaOpDev& d = A.ops[nm];
      d.mat = op.mat;
      d.nsel = op.nsel;
      for (int s = 0; s < op.nsel; ++s) {
        const int c = op.sel[s];
        const int g = -c - 1;
        if (c >= 0 || g >= nbits || ((inmask >> g) & 1ull))
          return mma_fail("op: MMA selectors must be global bits outside the tile");
        d.selg[s] = (int8_t)g;
      }
      d.bslot = (int16_t)slots;
      slots += 1 << op.nsel;
      if (slots > GBQ_MAX_MMA_MATS)
        return mma_fail("pass: MMA matrices exceed " + std::to_string(GBQ_MAX_MMA_MATS) + " per pass");
      d.diag0 = (int8_t)nd;
      ++nm;
    } else if (op.kind == GBQ_OP_DIAG) {
      if (op.k < 1 || op.k > GBQ_MAX_DIAG_K) return mma_fail("op: diagonal width must be 1..8");
      if (op.mat < 0) return mma_fail("op: negative matrix offset");
      if (nd >= GBQ_MAX_OPS_PER_PASS) return mma_fail("pass: too many diagonal ops");
      MmaDiagDev& d = A.diags[nd];
      d.mat = op.mat;
      d.k = op.k;
      for (int j = 0; j < 8; ++j) d.dext[j] = -1;
      for (int j = 0; j < op.k; ++j) {
        const int c = op.bits[j];
        if (c >= kML) return mma_fail("op: diagonal bit code out of range");
        if (c < 0) {
          const int g = -c - 1;
          if (g >= nbits || ((inmask >> g) & 1ull)) return mma_fail("op: diagonal global bit invalid");
          d.dext[j] = (int8_t)g;
        }
      }
      A.ops[nm - 1].ndiag++;
      ++nd;
    } else {
      return mma_fail("pass: a tensor-core pass holds only MMA and DIAG ops");
    }
  }
  A.nops = nm;
  A.ndiag = nd;
  A.nmats = slots;
  // Row orders, last op first: the lane bits (rows 0..3) of op o should have
  // independent bank columns in the layout the read-back writes to.
  int rows[GBQ_MAX_MMA_OPS][7];
  for (int o = nm - 1; o >= 0; --o) {
    int nt[7], c = 0;
    for (int b = 0; b < kML; ++b)
      if (b != tg[o][0] && b != tg[o][1] && b != tg[o][2] && b != tg[o][3]) nt[c++] = b;
    auto next_col = [&](int b) -> uint32_t {
      return o + 1 < nm ? op_col(tg[o + 1], rows[o + 1], b) : nat_col(b);
    };
    int best = -1, bi[4] = {0, 1, 2, 3};
    for (int i0 = 0; i0 < 7; ++i0)
      for (int i1 = i0 + 1; i1 < 7; ++i1)
        for (int i2 = i1 + 1; i2 < 7; ++i2)
          for (int i3 = i2 + 1; i3 < 7; ++i3) {
            const uint32_t v[4] = {next_col(nt[i0]), next_col(nt[i1]), next_col(nt[i2]), next_col(nt[i3])};
            const int r = rank4(v, 4);
            if (r > best) {
              best = r;
              bi[0] = i0, bi[1] = i1, bi[2] = i2, bi[3] = i3;
            }
          }
    bool used[7] = {false, false, false, false, false, false, false};
    for (int q = 0; q < 4; ++q) {
      rows[o][q] = nt[bi[q]];
      used[bi[q]] = true;
    }
    int q = 4;
    for (int i = 0; i < 7; ++i)
      if (!used[i]) rows[o][q++] = nt[i];
  }
  for (int o = 0; o < nm; ++o) {
    MmaOpDev& d = A.ops[o];
    for (int j = 0; j < 4; ++j)
      d.tnext[j] = (uint16_t)(o + 1 < nm ? op_col(tg[o + 1], rows[o + 1], tg[o][j]) : nat_col(tg[o][j]));
    for (int q = 0; q < 7; ++q)
      d.rnext[q] = (uint16_t)(o + 1 < nm ? op_col(tg[o + 1], rows[o + 1], rows[o][q]) : nat_col(rows[o][q]));
  }
  for (int b = 0; b < kML; ++b) A.lcol[b] = (uint16_t)op_col(tg[0], rows[0], b);
  // diagonal table-index columns in the row/target coordinates of their MMA op
  {
    int o = -1, seen_d = 0;
    for (int i = 0; i < p.op_count; ++i) {
      const gbq_op& op = po[i];
      if (op.kind == GBQ_OP_MMA) {
        ++o;
        continue;
      }
      MmaDiagDev& d = A.diags[seen_d++];
      for (int j = 0; j < op.k; ++j) {
        const int c = op.bits[j];
        if (c < 0) continue;
        bool placed = false;
        for (int pp = 0; pp < 4; ++pp)
          if (tg[o][pp] == c) {
            d.ttgt[pp] |= (uint16_t)(1u << j);
            placed = true;
          }
        for (int q = 0; q < 7; ++q)
          if (rows[o][q] == c) {
            d.trow[q] |= (uint16_t)(1u << j);
            placed = true;
          }
        if (!placed) return mma_fail("op: internal diagonal placement error");
      }
    }
  }
  return GBQ_OK;
}

int launch_mma_pass(Ctx* c, const MmaArgs& a) {
  static int blocks_per_sm = -1;
  cudaError_t e;
  if (blocks_per_sm < 0) {
    e = cudaFuncSetAttribute(k_mma_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, kMSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_mma_pass)");
    e = cudaFuncSetAttribute(k_mma_pass, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_mma_pass carveout)");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_mma_pass, kThreads, kMSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    blocks_per_sm = nb > 0 ? nb : 1;
    if (getenv("GBQ_DEBUG")) {
      cudaFuncAttributes fa;
      cudaFuncGetAttributes(&fa, k_mma_pass);
      int smem_sm = 0, smem_blk = 0;
      cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c->device);
      cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
      fprintf(stderr, "k_mma_pass: %d blocks/SM, %d B dynamic smem, %d regs, %zu B static, SM smem %d, block optin %d\n",
              blocks_per_sm, kMSmem, fa.numRegs, fa.sharedSizeBytes, smem_sm, smem_blk);
    }
  }
  int64_t grid = (int64_t)c->sm_count * blocks_per_sm;
  if (grid > a.ti.ntiles) grid = a.ti.ntiles;
  k_mma_pass<<<(unsigned)grid, kThreads, kMSmem, c->stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_mma_pass launch");
  c->launches += 1;
  return GBQ_OK;
}

}  // namespace gbq
