// Tile-pass device code (included by the per-tile-width translation units).
//
// One launch = one pass over the state.  A persistent grid of CTAs walks the
// tiles; each tile is 2^LT amplitudes: tile bits 0..m-1 are the global index
// bits 0..m-1 (contiguous runs, read with 128-bit loads) and tile bits
// m..LT-1 are global bits chosen by the host planner.  The tile is staged in
// shared memory, every op of the pass is applied there, and it is written
// back in place: HBM traffic per pass is one read and one write of the state
// whatever the number of ops.
//
// Replaces the numpy passes of the reference, one per operation:
// linalg.targeted_left_multiply (cirq-core/cirq/linalg/transformations.py:105-172),
// linalg.apply_matrix_to_slices (transformations.py:310-380), the gates'
// own _apply_unitary_ (cirq-core/cirq/ops/common_gates.py:123-134, 658-669,
// 1072-1082) and the Kraus/unitary channel paths
// (cirq-core/cirq/protocols/apply_channel_protocol.py:274-356).
//
// Addressing: amplitude i of the tile lives at shared index phys(i) =
// i ^ swz(i) (see gbq_internal.cuh).  phys is linear over GF(2), so the
// shared index of any group member is an XOR of per-bit "columns" that the
// host precomputes for every op (OpDev::pcol for target bits, OpDev::gcol
// for group-index bits).  A thread therefore finds all its addresses with a
// handful of XORs, and group-index bits 0..3 (the lanes of a half-warp) are
// chosen so that a half-warp touches 16 distinct 8-byte bank pairs.

#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "gbq_internal.cuh"

namespace gbq {

__device__ __forceinline__ uint32_t phys_dev(uint32_t i) {
  uint32_t s = (__popc(i & kSwzRow0) & 1) | ((__popc(i & kSwzRow1) & 1) << 1) |
               ((__popc(i & kSwzRow2) & 1) << 2) | ((__popc(i & kSwzRow3) & 1) << 3);
  return i ^ s;
}

// Register dense ops of width <= 2 use packed f32x2 FMAs (sm_100 family):
// acc += m * a as two fma.rn.f32x2, m * (a.x, a.x) and (i m) * (a.y, a.y).
#ifndef GBQ_FFMA2
#define GBQ_FFMA2 1
#endif

__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Probe accumulation: the warp's float sum of v is added (in double) to the
// warp's own accumulator acc[pidx * kProbeWarps + warp] in shared memory (no
// atomics, no barrier); the pass kernel sums the warps' accumulators and
// writes them once per CTA when its tiles are done.
constexpr int kProbeWarps = kThreads / 32;
__device__ __forceinline__ void probe_add(float v, int pidx, double* acc) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) acc[pidx * kProbeWarps + (threadIdx.x >> 5)] += (double)v;
}

// A probe's CTA total: the sum of its warps' accumulators.
__device__ __forceinline__ double probe_total(const double* acc, int pidx) {
  double v = 0.0;
#pragma unroll
  for (int w = 0; w < kProbeWarps; ++w) v += acc[pidx * kProbeWarps + w];
  return v;
}

// Block sum of v stored to *out by thread 0 (all threads must call).
__device__ __forceinline__ void cta_sum_store(double v, double* out, double* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < kThreads / 32 ? red[lane] : 0.0;
    v = warp_sum(v);
    if (lane == 0) *out = v;
  }
  __syncthreads();
}

// global offset of tile index i (XOR of the global weights of its bits)
template <int LT>
__device__ __forceinline__ uint64_t lin_off(const TileInfo& ti, uint32_t i) {
  uint64_t r = 0;
#pragma unroll
  for (int b = 0; b < LT; ++b)
    if ((i >> b) & 1u) r ^= ti.gw[b];
  return r;
}

__device__ __forceinline__ uint64_t tile_base(const TileInfo& ti, int64_t tile) {
  uint64_t g = 0;
  const int nnt = ti.nbits - ti.L;
  for (int j = 0; j < nnt; ++j) g |= (uint64_t)((tile >> j) & 1) << ti.nt[j];
  return g;
}

// Matrix pool of the point a tile belongs to (batched points) or the pass's pool.
__device__ __forceinline__ const float2* tile_mats(const TileInfo& ti, uint64_t gbase) {
  return ti.pstride ? ti.mats + (int64_t)(gbase >> ti.pshift) * ti.pstride : ti.mats;
}

// Base index of a tile from three 256-entry tables (tile-number bits 0-7,
// 8-15, 16-23 deposited at the out-of-tile global bits), built once per
// launch; tile numbers need at most 24 bits (states of <= 37 bits).
constexpr int kTileTab = 256;
__device__ __forceinline__ void tile_tables_build(const TileInfo& ti, uint64_t* tab) {
  for (int e = threadIdx.x; e < 3 * kTileTab; e += kThreads) {
    const int part = e / kTileTab;
    tab[e] = tile_base(ti, (int64_t)(e % kTileTab) << (8 * part));
  }
}
__device__ __forceinline__ uint64_t tile_base_fast(const uint64_t* tab, int64_t tile) {
  return tab[tile & 255] | tab[kTileTab + ((tile >> 8) & 255)] | tab[2 * kTileTab + ((tile >> 16) & 255)];
}

// ---- dense k-bit op (and dense probe) ---------------------------------------------
template <int K, int LT, bool DUAL, bool PROBE>
__device__ __forceinline__ void op_dense(const TileInfo& ti, const OpDev& op, float2* smA,
                                         float2* smB, uint64_t gbase, int64_t tile,
                                         double* red) {
  constexpr int D = 1 << K;
  constexpr int NG = 1 << (LT - K);
  constexpr int W = NG >= kThreads ? NG / kThreads : 1;
  constexpr int R0 = NG >= kThreads ? 1 : kThreads / NG;
  constexpr int R = R0 > D ? D : R0;
  constexpr int RPI = D / R;
  constexpr int NTB = (LT - K) < 8 ? (LT - K) : 8;
  constexpr int NWB = (LT - K) > 8 ? (LT - K) - 8 : 0;
  const int t = threadIdx.x;
  const bool active = (R == 1) || (t < NG * R);

  uint32_t pbt = 0;
#pragma unroll
  for (int b = 0; b < NTB; ++b)
    if ((t >> b) & 1) pbt ^= op.gcol[b];
  uint32_t poff[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> b) & 1) o ^= op.pcol[b];
    poff[j] = o;
  }
  const int r0 = (R == 1) ? 0 : (t >> (LT - K)) * RPI;

  // selector value = part fixed by the thread index / tile base, plus bits
  // carried by the group's w index (group-index bits >= 8)
  uint32_t sel_t = 0;
  int wsh[3] = {-1, -1, -1};
  const uint32_t gt = (R == 1) ? (uint32_t)t : (uint32_t)(t & (NG - 1));
  for (int s = 0; s < op.nsel; ++s) {
    const int c = op.selg[s];
    if (c < 0) sel_t |= (uint32_t)((gbase >> (-c - 1)) & 1u) << s;
    else if (c < 8 || R > 1) sel_t |= ((gt >> c) & 1u) << s;
    else wsh[s] = c - 8;
  }
  const float2* mbase = tile_mats(ti, gbase) + op.mat;

  float2 va[W][D];
  float2 vb[DUAL ? W : 1][DUAL ? D : 1];
  uint32_t pb[W];
  const float2* mp[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    uint32_t p = pbt;
#pragma unroll
    for (int b = 0; b < NWB; ++b)
      if ((w >> b) & 1) p ^= op.gcol[8 + b];
    pb[w] = p;
    uint32_t sel = sel_t;
    if (W > 1) {
#pragma unroll
      for (int s = 0; s < 3; ++s)
        if (wsh[s] >= 0) sel |= (((uint32_t)w >> wsh[s]) & 1u) << s;
    }
    mp[w] = mbase + (int64_t)sel * (D * D);
    if (active) {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        va[w][j] = smA[p ^ poff[j]];
        if constexpr (DUAL) vb[w][j] = smB[p ^ poff[j]];
      }
    }
  }

  if constexpr (PROBE) {
    // Re <lam| D |psi> over this thread's rows (smA = psi, smB = lam)
    float part = 0.f;
    if (active) {
#pragma unroll
      for (int w = 0; w < W; ++w) {
#pragma unroll
        for (int r = 0; r < D; ++r) {
          if (R > 1 && (r < r0 || r >= r0 + RPI)) continue;
          const float2* row = mp[w] + r * D;
          float2 acc = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; c += 2) {
            const float4 mm = __ldg(reinterpret_cast<const float4*>(row + c));
            cfma(acc, make_float2(mm.x, mm.y), va[w][c]);
            cfma(acc, make_float2(mm.z, mm.w), va[w][c + 1]);
          }
          part = fmaf(vb[w][r].x, acc.x, part);
          part = fmaf(vb[w][r].y, acc.y, part);
        }
      }
    }
    probe_add(part, op.pidx, red);
  } else {
    if constexpr (R > 1) __syncthreads();  // other threads still read this group
    if (!active) return;
    if constexpr (K <= 2) {
      // small matrices: keep them in registers; reload only when the
      // selector gives groups of this thread different matrices
      float2 m[D * D];
#pragma unroll
      for (int e = 0; e < D * D; e += 2) {
        const float4 mm = __ldg(reinterpret_cast<const float4*>(mp[0] + e));
        m[e] = make_float2(mm.x, mm.y);
        m[e + 1] = make_float2(mm.z, mm.w);
      }
#pragma unroll
      for (int w = 0; w < W; ++w) {
        if (w > 0 && op.nsel) {
#pragma unroll
          for (int e = 0; e < D * D; e += 2) {
            const float4 mm = __ldg(reinterpret_cast<const float4*>(mp[w] + e));
            m[e] = make_float2(mm.x, mm.y);
            m[e + 1] = make_float2(mm.z, mm.w);
          }
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
          if (R > 1 && (r < r0 || r >= r0 + RPI)) continue;
          float2 acc = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; ++c) cfma(acc, m[r * D + c], va[w][c]);
          smA[pb[w] ^ poff[r]] = acc;
          if constexpr (DUAL) {
            float2 accb = make_float2(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < D; ++c) cfma(accb, m[r * D + c], vb[w][c]);
            smB[pb[w] ^ poff[r]] = accb;
          }
        }
      }
    } else {
#pragma unroll
      for (int w = 0; w < W; ++w) {
#pragma unroll
        for (int r = 0; r < D; ++r) {
          if (R > 1 && (r < r0 || r >= r0 + RPI)) continue;
          const float2* row = mp[w] + r * D;
          float2 acc = make_float2(0.f, 0.f);
          float2 accb = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; c += 2) {
            const float4 mm = __ldg(reinterpret_cast<const float4*>(row + c));
            cfma(acc, make_float2(mm.x, mm.y), va[w][c]);
            cfma(acc, make_float2(mm.z, mm.w), va[w][c + 1]);
            if constexpr (DUAL) {
              cfma(accb, make_float2(mm.x, mm.y), vb[w][c]);
              cfma(accb, make_float2(mm.z, mm.w), vb[w][c + 1]);
            }
          }
          smA[pb[w] ^ poff[r]] = acc;
          if constexpr (DUAL) smB[pb[w] ^ poff[r]] = accb;
        }
      }
    }
  }
}

// ---- diagonal op (and diagonal probe) ------------------------------------------------
template <int LT, bool DUAL, bool PROBE>
__device__ __forceinline__ void op_diag(const TileInfo& ti, const OpDev& op, float2* smA,
                                        float2* smB, uint64_t gbase, int64_t tile, double* red) {
  constexpr int A = (1 << LT) / kThreads;  // amplitude i = t + j * kThreads
  const int t = threadIdx.x;
  uint32_t it = 0;
#pragma unroll
  for (int b = 0; b < 8; ++b)
    if ((t >> b) & 1) it ^= op.dcol[b];
  uint32_t ext = 0;
  for (int j = 0; j < op.k; ++j)
    if (op.dext[j] >= 0) ext |= (uint32_t)((gbase >> op.dext[j]) & 1u) << j;
  it ^= ext;
  const uint32_t pt = phys_dev((uint32_t)t);
  const float2* tab = tile_mats(ti, gbase) + op.mat;
  float part = 0.f;
#pragma unroll
  for (int j = 0; j < A; ++j) {
    uint32_t ij = it;
#pragma unroll
    for (int b = 0; b < LT - 8; ++b)
      if ((j >> b) & 1) ij ^= op.dcol[8 + b];
    const uint32_t p = pt ^ phys_const((uint32_t)j * kThreads);
    const float2 d = __ldg(tab + ij);
    if constexpr (PROBE) {
      const float2 y = cmul(d, smA[p]);
      const float2 l = smB[p];
      part = fmaf(l.x, y.x, fmaf(l.y, y.y, part));
    } else {
      smA[p] = cmul(d, smA[p]);
      if constexpr (DUAL) smB[p] = cmul(d, smB[p]);
    }
  }
  if constexpr (PROBE)
    probe_add(part, op.pidx, red);
}

// KMAX: widest shared-memory dense op the kernel variant contains (0 or 5);
// the KMAX = 0 variant (register phases only) keeps register pressure down.
template <int LT, int KMAX, bool DUAL>
__device__ __forceinline__ void dispatch(const TileInfo& ti, const OpDev& op, float2* smA,
                                         float2* smB, uint64_t gbase, int64_t tile, double* red) {
  switch (op.kind * 8 + op.k) {
    case GBQ_OP_DENSE * 8 + 1:
      if constexpr (KMAX >= 1) op_dense<1, LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      break;
    case GBQ_OP_DENSE * 8 + 2:
      if constexpr (KMAX >= 2) op_dense<2, LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      break;
    case GBQ_OP_DENSE * 8 + 3:
      if constexpr (KMAX >= 3) op_dense<3, LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      break;
    case GBQ_OP_DENSE * 8 + 4:
      if constexpr (KMAX >= 4) op_dense<4, LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      break;
    case GBQ_OP_DENSE * 8 + 5:
      if constexpr (KMAX >= 5) op_dense<5, LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      break;
    default:
      if (op.kind == GBQ_OP_DIAG) {
        op_diag<LT, DUAL, false>(ti, op, smA, smB, gbase, tile, red);
      } else if constexpr (DUAL) {
        if (op.kind == GBQ_OP_PROBE_DIAG) {
          op_diag<LT, true, true>(ti, op, smA, smB, gbase, tile, red);
        } else if (op.kind == GBQ_OP_PROBE) {
          if constexpr (KMAX >= 3) {
            if (op.k == 1) op_dense<1, LT, true, true>(ti, op, smA, smB, gbase, tile, red);
            else if (op.k == 2) op_dense<2, LT, true, true>(ti, op, smA, smB, gbase, tile, red);
            else if (op.k == 3) op_dense<3, LT, true, true>(ti, op, smA, smB, gbase, tile, red);
          }
        }
      }
      break;
  }
}

// ---- tile load (asynchronous) / store -------------------------------------------------
// Loads: amplitude i = t + j * kThreads of the tile (a warp copies 32
// consecutive amplitudes = 256 contiguous bytes) with 8-byte cp.async, so the
// next tile streams into the second shared buffer while the current one is
// being processed.
__device__ __forceinline__ void cp_async8(float2* sdst, const float2* gsrc) {
  const uint32_t sa = (uint32_t)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// global offset of the tile-index bits >= `lo` of the compile-time value x
template <int LT>
__device__ __forceinline__ uint64_t hi_part(const TileInfo& ti, uint32_t x) {
  uint64_t r = 0;
#pragma unroll
  for (int b = 8; b < LT; ++b)
    if ((x >> b) & 1u) r |= ti.gw[b];
  return r;
}

template <int LT>
__device__ __forceinline__ void load_tile_async(const TileInfo& ti, const float2* __restrict__ src,
                                                float2* sm, uint64_t gbase, uint64_t lo_t,
                                                uint32_t lp_t) {
  constexpr int NA = 1 << (LT - 8);  // amplitudes per thread
  const float2* g = src + (gbase | lo_t);
#pragma unroll
  for (int j = 0; j < NA; ++j) {
    cp_async8(sm + (lp_t ^ phys_const((uint32_t)j * kThreads)), g + hi_part<LT>(ti, (uint32_t)j * kThreads));
  }
}

template <int LT>
__device__ __forceinline__ void store_tile(const TileInfo& ti, float2* __restrict__ dst,
                                           const float2* sm, uint64_t gbase, uint64_t off_t,
                                           uint32_t ph_t) {
  constexpr int NJ = 1 << (LT - 9);
  float2* g = dst + (gbase | off_t);
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const uint32_t p = ph_t ^ phys_const((uint32_t)j * (2 * kThreads));
    const float2 x = sm[p], y = sm[p ^ 1u];
    __stcs(reinterpret_cast<float4*>(g + hi_part<LT>(ti, (uint32_t)j * (2 * kThreads))),
           make_float4(x.x, x.y, y.x, y.y));
  }
}

// Per-launch setup shared by the pass and batch kernels.  Stores: float4
// pairs p = t + j * kThreads <-> tile index 2p.  Loads: amplitude
// i = t + j * kThreads.  Only the thread part is per-thread; the j parts are
// shared tables.
struct TileSetup {
  uint64_t off_t;  // store: global offset of tile index 2t
  uint32_t ph_t;   // store: shared index of tile index 2t
  uint64_t lo_t;   // load: global offset of tile index t
  uint32_t lp_t;   // load: shared index of tile index t
};

template <int LT>
__device__ __forceinline__ TileSetup tile_setup(const TileInfo& ti) {
  TileSetup s;
  s.off_t = lin_off<LT>(ti, (uint32_t)threadIdx.x << 1);
  s.ph_t = phys_dev((uint32_t)threadIdx.x << 1);
  s.lo_t = lin_off<LT>(ti, (uint32_t)threadIdx.x);
  s.lp_t = phys_dev((uint32_t)threadIdx.x);
  return s;
}

// ---- register phases -------------------------------------------------------------
// Inside a phase every thread owns A = 2^R amplitudes (R = LT - 8) that
// differ only in the R register bits of the current layout; register ops act
// on them in registers, with no shared-memory traffic and no barrier.

__host__ __device__ constexpr int popc_const(int x) { return x ? (x & 1) + popc_const(x >> 1) : 0; }
// Deposits the low bits of x into the set positions of mask.
__host__ __device__ constexpr int dep_const(int x, int mask) {
  int r = 0, i = 0;
  for (int b = 0; b < 8; ++b)
    if ((mask >> b) & 1) {
      if ((x >> i) & 1) r |= 1 << b;
      ++i;
    }
  return r;
}

template <int LT, bool DUAL>
struct RegState {
  static constexpr int R = LT - 8;
  static constexpr int A = 1 << R;
  float2 v[A];
  float2 w[DUAL ? A : 1];
  uint32_t phys_t;  // shared index of slot 0
  uint32_t pc[R];   // shared-index column of register position p
  uint32_t tidx;    // tile index of slot 0 (thread bits only)
};

template <int LT, bool DUAL>
__device__ __forceinline__ uint32_t slot_phys(const RegState<LT, DUAL>& st, int s) {
  uint32_t p = st.phys_t;
#pragma unroll
  for (int b = 0; b < RegState<LT, DUAL>::R; ++b)
    if ((s >> b) & 1) p ^= st.pc[b];
  return p;
}

// Shared index and tile index of a thread's slot 0 in a layout.
__device__ __forceinline__ uint32_t layout_entry(const OpDev& op, int t) {
  uint32_t ph = 0, ti = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if ((t >> j) & 1) {
      ph ^= op.gcol[j];
      ti ^= op.tcol[j];
    }
  return ph | (ti << 16);
}

// lt: this thread's precomputed layout_entry, or ~0u to compute it here.
template <int LT, bool DUAL>
__device__ __forceinline__ void phase_enter(RegState<LT, DUAL>& st, const OpDev& op,
                                            const float2* smA, const float2* smB,
                                            uint32_t lt = ~0u) {
  constexpr int R = RegState<LT, DUAL>::R;
  if (lt == ~0u) lt = layout_entry(op, threadIdx.x);
  st.phys_t = lt & 0xffffu;
  st.tidx = lt >> 16;
#pragma unroll
  for (int p = 0; p < R; ++p) st.pc[p] = op.pcol[p];
#pragma unroll
  for (int s = 0; s < RegState<LT, DUAL>::A; ++s) {
    const uint32_t a = slot_phys(st, s);
    st.v[s] = smA[a];
    if constexpr (DUAL) st.w[s] = smB[a];
  }
}

template <int LT, bool DUAL>
__device__ __forceinline__ void phase_exit(const RegState<LT, DUAL>& st, float2* smA, float2* smB) {
#pragma unroll
  for (int s = 0; s < RegState<LT, DUAL>::A; ++s) {
    const uint32_t a = slot_phys(st, s);
    smA[a] = st.v[s];
    if constexpr (DUAL) smB[a] = st.w[s];
  }
}

template <int LT, bool DUAL>
__device__ __forceinline__ const float2* reg_matrix(const TileInfo& ti, const OpDev& op,
                                                    const RegState<LT, DUAL>& st, uint64_t gbase,
                                                    int dd) {
  uint32_t sel = 0;
  const int ns = op.nsel;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (s < ns) {
      const int c = op.selg[s];
      const uint32_t bit = c >= 0 ? (st.tidx >> c) & 1u : (uint32_t)((gbase >> (-c - 1)) & 1u);
      sel |= bit << s;
    }
  }
  return tile_mats(ti, gbase) + op.mat + (int64_t)sel * dd;
}

// Dense op (or dense probe) on the register positions in MASK.
template <int MASK, int LT, bool DUAL, bool PROBE>
__device__ __forceinline__ void reg_dense(const TileInfo& ti, const OpDev& op,
                                          RegState<LT, DUAL>& st, uint64_t gbase, int64_t tile,
                                          double* red) {
  constexpr int R = RegState<LT, DUAL>::R;
  constexpr int A = RegState<LT, DUAL>::A;
  constexpr int K = popc_const(MASK);
  constexpr int D = 1 << K;
  constexpr int NG = A / D;
  constexpr int REST = (A - 1) & ~MASK;
  const float2* mp = reg_matrix(ti, op, st, gbase, D * D);
  float part = 0.f;
#if GBQ_FFMA2
  if constexpr (K <= 2 && !PROBE) {
    // Packed form: acc += m * a as two f32x2 FMAs, m * (a.x, a.x) and
    // (i m) * (a.y, a.y).
    float2 m[D * D], im[D * D];
#pragma unroll
    for (int e = 0; e < D * D; e += 2) {
      const float4 mm = __ldg(reinterpret_cast<const float4*>(mp + e));
      m[e] = make_float2(mm.x, mm.y);
      m[e + 1] = make_float2(mm.z, mm.w);
      im[e] = make_float2(-mm.y, mm.x);
      im[e + 1] = make_float2(-mm.w, mm.z);
    }
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int s0 = dep_const(g, REST);
      float2 ax[D], ay[D], bx[DUAL ? D : 1], by[DUAL ? D : 1];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const float2 a = st.v[s0 | dep_const(j, MASK)];
        ax[j] = make_float2(a.x, a.x);
        ay[j] = make_float2(a.y, a.y);
        if constexpr (DUAL) {
          const float2 b = st.w[s0 | dep_const(j, MASK)];
          bx[j] = make_float2(b.x, b.x);
          by[j] = make_float2(b.y, b.y);
        }
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) {
          acc = __ffma2_rn(m[r * D + c], ax[c], acc);
          acc = __ffma2_rn(im[r * D + c], ay[c], acc);
        }
        st.v[s0 | dep_const(r, MASK)] = acc;
        if constexpr (DUAL) {
          float2 accb = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; ++c) {
            accb = __ffma2_rn(m[r * D + c], bx[c], accb);
            accb = __ffma2_rn(im[r * D + c], by[c], accb);
          }
          st.w[s0 | dep_const(r, MASK)] = accb;
        }
      }
    }
  } else
#endif
  if constexpr (K <= 2) {
    float2 m[D * D];
#pragma unroll
    for (int e = 0; e < D * D; e += 2) {
      const float4 mm = __ldg(reinterpret_cast<const float4*>(mp + e));
      m[e] = make_float2(mm.x, mm.y);
      m[e + 1] = make_float2(mm.z, mm.w);
    }
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int s0 = dep_const(g, REST);
      float2 in[D];
      float2 inb[DUAL ? D : 1];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        in[j] = st.v[s0 | dep_const(j, MASK)];
        if constexpr (DUAL) inb[j] = st.w[s0 | dep_const(j, MASK)];
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) cfma(acc, m[r * D + c], in[c]);
        if constexpr (PROBE) {
          const float2 l = st.w[s0 | dep_const(r, MASK)];
          part = fmaf(l.x, acc.x, fmaf(l.y, acc.y, part));
        } else {
          st.v[s0 | dep_const(r, MASK)] = acc;
          if constexpr (DUAL) {
            float2 accb = make_float2(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < D; ++c) cfma(accb, m[r * D + c], inb[c]);
            st.w[s0 | dep_const(r, MASK)] = accb;
          }
        }
      }
    }
  } else {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int s0 = dep_const(g, REST);
      float2 in[D];
      float2 inb[DUAL ? D : 1];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        in[j] = st.v[s0 | dep_const(j, MASK)];
        if constexpr (DUAL) inb[j] = st.w[s0 | dep_const(j, MASK)];
      }
#pragma unroll
      for (int r = 0; r < D; ++r) {
        const float2* row = mp + r * D;
        float2 acc = make_float2(0.f, 0.f);
        float2 accb = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; c += 2) {
          const float4 mm = __ldg(reinterpret_cast<const float4*>(row + c));
          cfma(acc, make_float2(mm.x, mm.y), in[c]);
          cfma(acc, make_float2(mm.z, mm.w), in[c + 1]);
          if constexpr (DUAL && !PROBE) {
            cfma(accb, make_float2(mm.x, mm.y), inb[c]);
            cfma(accb, make_float2(mm.z, mm.w), inb[c + 1]);
          }
        }
        if constexpr (PROBE) {
          const float2 l = st.w[s0 | dep_const(r, MASK)];
          part = fmaf(l.x, acc.x, fmaf(l.y, acc.y, part));
        } else {
          st.v[s0 | dep_const(r, MASK)] = acc;
          if constexpr (DUAL) st.w[s0 | dep_const(r, MASK)] = accb;
        }
      }
    }
  }
  if constexpr (PROBE)
    probe_add(part, op.pidx, red);
  (void)R;
}

// Diagonal op (or diagonal probe) in registers; bits may be register,
// thread or out-of-tile bits.
template <int LT, bool DUAL, bool PROBE>
__device__ __forceinline__ void reg_diag(const TileInfo& ti, const OpDev& op,
                                         RegState<LT, DUAL>& st, uint64_t gbase, int64_t tile,
                                         double* red) {
  constexpr int R = RegState<LT, DUAL>::R;
  constexpr int A = RegState<LT, DUAL>::A;
  uint32_t base = 0;
  const int nk = op.k;
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (j < nk && op.dext[j] >= 0) base |= (uint32_t)((gbase >> op.dext[j]) & 1u) << j;
#pragma unroll
  for (int b = 0; b < LT; ++b)
    if ((st.tidx >> b) & 1u) base ^= op.dcol[b];
  uint32_t rc[R];
#pragma unroll
  for (int p = 0; p < R; ++p) rc[p] = op.dcol[op.rbits[p]];
  const float2* tab = tile_mats(ti, gbase) + op.mat;
  float part = 0.f;
#pragma unroll
  for (int s = 0; s < A; ++s) {
    uint32_t idx = base;
#pragma unroll
    for (int p = 0; p < R; ++p)
      if ((s >> p) & 1) idx ^= rc[p];
    const float2 d = __ldg(tab + idx);
    if constexpr (PROBE) {
      const float2 y = cmul(d, st.v[s]);
      const float2 l = st.w[s];
      part = fmaf(l.x, y.x, fmaf(l.y, y.y, part));
    } else {
      st.v[s] = cmul(d, st.v[s]);
      if constexpr (DUAL) st.w[s] = cmul(d, st.w[s]);
    }
  }
  if constexpr (PROBE)
    probe_add(part, op.pidx, red);
}

template <int LT, bool DUAL, bool PROBE, int RK, int M>
__device__ __forceinline__ void reg_dense_case(const TileInfo& ti, const OpDev& op, RegState<LT, DUAL>& st,
                                               uint64_t gbase, int64_t tile, double* red) {
  if constexpr (M < (1 << RegState<LT, DUAL>::R) && (!PROBE || popc_const(M) <= 3) && popc_const(M) <= RK)
    reg_dense<M, LT, DUAL, PROBE>(ti, op, st, gbase, tile, red);
}

// One switch over the register-position mask (a jump, not a chain of tests).
template <int LT, int KMAX, bool DUAL, bool PROBE, int RK>
__device__ __forceinline__ void reg_dense_dispatch(const TileInfo& ti, const OpDev& op,
                                                   RegState<LT, DUAL>& st, uint64_t gbase,
                                                   int64_t tile, double* red) {
#define GBQ_RCASE(M) \
  case M:            \
    reg_dense_case<LT, DUAL, PROBE, RK, M>(ti, op, st, gbase, tile, red); \
    break;
  switch (op.rmask) {
    GBQ_RCASE(1) GBQ_RCASE(2) GBQ_RCASE(3) GBQ_RCASE(4) GBQ_RCASE(5) GBQ_RCASE(6) GBQ_RCASE(7)
    GBQ_RCASE(8) GBQ_RCASE(9) GBQ_RCASE(10) GBQ_RCASE(11) GBQ_RCASE(12) GBQ_RCASE(13) GBQ_RCASE(14)
    GBQ_RCASE(15)
    default:
      break;
  }
#undef GBQ_RCASE
}

// Barrier among the threads that run the ops: the whole CTA, or (NB) the
// 256 consumer threads of a warp-specialised CTA (named barrier 1).
template <bool NB>
__device__ __forceinline__ void ops_barrier() {
  if constexpr (NB)
    asm volatile("bar.sync 1, 256;\n" ::: "memory");
  else
    __syncthreads();
}

// ltab (optional): ltab[q * kThreads + t] = layout_entry of the q-th layout
// op of the pass for thread t, for q < nltab.
template <int LT, int KMAX, bool DUAL, int RK = 4, bool NB = false>
__device__ __forceinline__ void run_ops(const TileInfo& ti, const OpDev* sops, float2* smA,
                                        float2* smB, uint64_t gbase, int64_t tile, double* red,
                                        const uint32_t* ltab = nullptr, int nltab = 0) {
  if constexpr (LT <= 12) {
    RegState<LT, DUAL> st;
    bool in_phase = false;
    int nl = 0;
    for (int o = 0; o < ti.nops; ++o) {
      const OpDev& op = sops[o];
      const int kind = op.kind;
      if (kind == GBQ_OP_LAYOUT) {
        if (in_phase) {
          phase_exit(st, smA, smB);
          ops_barrier<NB>();
        }
        phase_enter(st, op, smA, smB, nl < nltab ? ltab[nl * kThreads + threadIdx.x] : ~0u);
        ++nl;
        in_phase = true;
      } else if (kind == GBQ_OP_RDENSE) {
        reg_dense_dispatch<LT, KMAX, DUAL, false, RK>(ti, op, st, gbase, tile, red);
      } else if (kind == GBQ_OP_RDIAG) {
        reg_diag<LT, DUAL, false>(ti, op, st, gbase, tile, red);
      } else if (kind == GBQ_OP_RPROBE) {
        if constexpr (DUAL) reg_dense_dispatch<LT, KMAX, true, true, RK>(ti, op, st, gbase, tile, red);
      } else if (kind == GBQ_OP_RPROBE_DIAG) {
        if constexpr (DUAL) reg_diag<LT, true, true>(ti, op, st, gbase, tile, red);
      } else {
        if (in_phase) {
          phase_exit(st, smA, smB);
          ops_barrier<NB>();
          in_phase = false;
        }
        dispatch<LT, KMAX, DUAL>(ti, op, smA, smB, gbase, tile, red);
        ops_barrier<NB>();
      }
    }
    if (in_phase) {
      phase_exit(st, smA, smB);
      ops_barrier<NB>();
    }
  } else {
    for (int o = 0; o < ti.nops; ++o) {
      dispatch<LT, KMAX, DUAL>(ti, sops[o], smA, smB, gbase, tile, red);
      ops_barrier<NB>();
    }
  }
}

// STAGES shared buffers per state: tile i is processed in one while the next
// STAGES - 1 tiles stream into the others (cp.async groups), so the memory
// system stays busy while the CTA computes.
// RK: widest register dense op compiled in (2 or 4); the RK = 2 lean variant
// targets 3 CTAs per SM.
template <int LT, int KMAX, bool DUAL, int STAGES, int RK>
__global__ void __launch_bounds__(kThreads, (KMAX == 0 && RK <= 2 && !DUAL) ? 3 : 2)
    k_tile_pass(const __grid_constant__ PassArgs a) {
  constexpr int kStages = STAGES;
  // The lean variant reads its ops straight from the kernel parameters
  // (uniform indices hit the constant cache) so that three CTAs of 2^12
  // amplitude tiles fit in shared memory.
  constexpr bool kParamOps = (KMAX == 0 && RK <= 2 && !DUAL);
  extern __shared__ float4 smraw[];
  __shared__ OpDev sops_sh[kParamOps ? 1 : GBQ_MAX_OPS_PER_PASS];
  __shared__ uint64_t ttab[3 * kTileTab];
  __shared__ double red[DUAL ? GBQ_MAX_OPS_PER_PASS * kProbeWarps : 1];  // per-warp probe accumulators
  constexpr int TS = 1 << LT;
  constexpr int NS = DUAL ? 2 : 1;
  float2* buf = reinterpret_cast<float2*>(smraw);  // [kStages][NS][TS]
  const OpDev* sops = kParamOps ? a.ops : sops_sh;
  if constexpr (!kParamOps) {
    const int nwords = a.ti.nops * (int)(sizeof(OpDev) / 4);
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.ops);
    uint32_t* dst = reinterpret_cast<uint32_t*>(sops_sh);
    for (int i = threadIdx.x; i < nwords; i += kThreads) dst[i] = src[i];
  }
  tile_tables_build(a.ti, ttab);
  const TileSetup ts = tile_setup<LT>(a.ti);
  if constexpr (DUAL) {
    for (int i = threadIdx.x; i < GBQ_MAX_OPS_PER_PASS * kProbeWarps; i += kThreads) red[i] = 0.0;
  }
  __syncthreads();
  const int64_t step = gridDim.x;
  // prologue: the first kStages - 1 tiles
#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    const int64_t tl = blockIdx.x + s * step;
    if (tl < a.ti.ntiles) {
      const uint64_t gb = tile_base_fast(ttab, tl);
      float2* b = buf + s * NS * TS;
      load_tile_async<LT>(a.ti, a.psi, b, gb, ts.lo_t, ts.lp_t);
      if constexpr (DUAL) load_tile_async<LT>(a.ti, a.lam, b + TS, gb, ts.lo_t, ts.lp_t);
    }
    cp_async_commit();
  }
  int cur = 0;
  for (int64_t tile = blockIdx.x; tile < a.ti.ntiles; tile += step) {
    const int64_t ahead = tile + (kStages - 1) * step;
    const int slot_ahead = (cur + kStages - 1) % kStages;
    if (ahead < a.ti.ntiles) {
      const uint64_t gn = tile_base_fast(ttab, ahead);
      float2* nb = buf + slot_ahead * NS * TS;
      load_tile_async<LT>(a.ti, a.psi, nb, gn, ts.lo_t, ts.lp_t);
      if constexpr (DUAL) load_tile_async<LT>(a.ti, a.lam, nb + TS, gn, ts.lo_t, ts.lp_t);
    }
    cp_async_commit();
    cp_async_wait<kStages - 1>();
    __syncthreads();
    float2* smA = buf + cur * NS * TS;
    float2* smB = smA + TS;
    const uint64_t gbase = tile_base_fast(ttab, tile);
    run_ops<LT, KMAX, DUAL, RK>(a.ti, sops, smA, smB, gbase, tile, red);
    store_tile<LT>(a.ti, a.psi, smA, gbase, ts.off_t, ts.ph_t);
    if constexpr (DUAL) store_tile<LT>(a.ti, a.lam, smB, gbase, ts.off_t, ts.ph_t);
    __syncthreads();
    cur = (cur + 1) % kStages;
  }
  cp_async_wait<0>();
  if constexpr (DUAL) {
    // probe totals of this CTA: into the partial of its first tile, zeros
    // into those of its other tiles (the slot sums over all tiles)
    __syncthreads();
    for (int o = 0; o < a.ti.nops; ++o) {
      const OpDev& op = sops[o];
      const int kind = op.kind;
      if (kind != GBQ_OP_PROBE && kind != GBQ_OP_PROBE_DIAG && kind != GBQ_OP_RPROBE &&
          kind != GBQ_OP_RPROBE_DIAG)
        continue;
      double* dst = a.ti.partial + (int64_t)op.slot * a.ti.ntiles;
      for (int64_t tile = blockIdx.x + (int64_t)threadIdx.x * step; tile < a.ti.ntiles;
           tile += (int64_t)kThreads * step)
        dst[tile] = tile == (int64_t)blockIdx.x ? probe_total(red, op.pidx) : 0.0;
    }
  }
}

template <int LT, int KMAX, bool DUAL, int STAGES, int RK>
int launch_tile_pass_stages(Ctx* c, const PassArgs& a) {
  const int smem = STAGES * (DUAL ? 2 : 1) * (1 << LT) * (int)sizeof(float2);
  static int blocks_per_sm = -1;
  cudaError_t e;
  if (blocks_per_sm < 0) {
    e = cudaFuncSetAttribute(k_tile_pass<LT, KMAX, DUAL, STAGES, RK>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tile_pass)");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tile_pass<LT, KMAX, DUAL, STAGES, RK>,
                                                      kThreads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    blocks_per_sm = nb > 0 ? nb : 1;
    if (const char* cap = getenv("GBQ_CTAS_PER_SM")) {
      const int want = atoi(cap);
      if (want > 0 && want < blocks_per_sm) blocks_per_sm = want;
    }
    if (getenv("GBQ_DEBUG"))
      fprintf(stderr, "k_tile_pass<L=%d,K=%d,dual=%d,stages=%d,rk=%d>: %d blocks/SM, %d B smem\n", LT,
              KMAX, (int)DUAL, STAGES, RK, blocks_per_sm, smem);
  }
  int64_t grid = (int64_t)c->sm_count * blocks_per_sm;
  if (grid > a.ti.ntiles) grid = a.ti.ntiles;
  k_tile_pass<LT, KMAX, DUAL, STAGES, RK><<<(unsigned)grid, kThreads, smem, c->stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_tile_pass launch");
  c->launches += 1;
  return GBQ_OK;
}

// ---- warp-specialised pass -----------------------------------------------------
// Eight consumer warps run the ops; a ninth (producer) warp streams tiles
// through WS_STAGES shared buffers: it copies tile i into buffer i % S with
// cp.async (completion signalled on full[b] by cp.async.mbarrier.arrive), and
// once the consumers have released buffer b (empty[b]) it writes tile i - S
// back with 16-byte stores before refilling b.  Loads, write-backs and the
// FMA-bound register phases of other tiles run at the same time, on different
// pipes.  Every mbarrier wait is bounded; a consumer-wide vote after each wait
// keeps the named barriers of the consumers consistent if one gives up.
constexpr int kWsStages = 3;
constexpr int kWsProducers = 2;  // producer warps per CTA
constexpr int kWsThreads = kThreads + 32 * kWsProducers;
constexpr long kWsSpin = 1L << 26;
// Layout ops whose per-thread (shared index, tile index) of slot 0 are
// computed once per CTA (8 KB; two CTAs of 2^12 tiles still fit an SM).
#ifndef GBQ_WS_LTABS
#define GBQ_WS_LTABS 8
#endif
constexpr int kWsLayoutTabs = GBQ_WS_LTABS;

__device__ __forceinline__ uint32_t ws_su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Bounded wait for the phase with the given parity; gives up (returns
// false) after kWsSpin polls or when another thread has raised *abort.
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const uint32_t a = ws_su32(bar);
  for (long it = 0; it < kWsSpin; ++it) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((it & 255) == 255 && *abort) return false;
  }
  *abort = 1;
  return false;
}

// Named-barrier OR over the 256 consumer threads.
__device__ __forceinline__ bool consumers_any(bool v) {
  uint32_t r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, 1, 256, p;\n"
      "selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v)
      : "memory");
  return r != 0;
}

template <int LT>
__global__ void __launch_bounds__(kWsThreads, 2) k_tile_ws(const __grid_constant__ PassArgs a) {
  constexpr int TS = 1 << LT;
  constexpr int S = kWsStages;
  constexpr int NH = TS >> 5;  // tile-index values of bits 5..LT-1
  extern __shared__ float4 smraw[];
  __shared__ uint64_t ttab[3 * kTileTab];
  __shared__ uint64_t hoff[NH];   // global offset of tile index (j << 5)
  __shared__ uint16_t hphys[NH];  // shared index of tile index (j << 5)
  __shared__ __align__(8) uint64_t full[S], empty[S];
  __shared__ int abort_flag;
  __shared__ double red[kThreads / 32];
  __shared__ uint32_t ltab[(kWsLayoutTabs > 0 ? kWsLayoutTabs : 1) * kThreads];  // consumers' layout entries
  float2* buf = reinterpret_cast<float2*>(smraw);  // [S][TS]
  const TileInfo& ti = a.ti;
  const int t = threadIdx.x;
  int nltab = 0;
  for (int o = 0; o < ti.nops && nltab < kWsLayoutTabs; ++o)
    if (a.ops[o].kind == GBQ_OP_LAYOUT) {
      if (t < kThreads) ltab[nltab * kThreads + t] = layout_entry(a.ops[o], t);
      ++nltab;
    }
  for (int e = t; e < 3 * kTileTab; e += kWsThreads) {
    const int part = e / kTileTab;
    ttab[e] = tile_base(ti, (int64_t)(e % kTileTab) << (8 * part));
  }
  for (int j = t; j < NH; j += kWsThreads) {
    hoff[j] = lin_off<LT>(ti, (uint32_t)j << 5);
    hphys[j] = (uint16_t)phys_dev((uint32_t)j << 5);
  }
  if (t == 0) {
    abort_flag = 0;
    for (int b = 0; b < S; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(ws_su32(&full[b])), "r"(32 * kWsProducers));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 256;\n" ::"r"(ws_su32(&empty[b])));
    }
  }
  __syncthreads();
  const int64_t step = gridDim.x;
  const int64_t count = blockIdx.x < ti.ntiles ? (ti.ntiles - 1 - blockIdx.x) / step + 1 : 0;
  volatile int* abort = &abort_flag;
  // warp-uniform role (the shuffle lets the compiler keep the consumer's op
  // loop on the uniform datapath)
  const int warp_u = __shfl_sync(0xffffffffu, t >> 5, 0);
  if (warp_u >= kThreads / 32) {
    // ---- producer warp
    const int pt = t - kThreads;  // producer thread
    const int lane = pt & 31, pw = pt >> 5;
    const uint64_t lo_l = lin_off<LT>(ti, (uint32_t)lane);             // load: tile index lane + 32 j
    const uint32_t lp_l = phys_dev((uint32_t)lane);
    const uint64_t so_l = lin_off<LT>(ti, (uint32_t)(2 * lane) & 31u);  // store: tile index 2 lane + 64 j
    const uint32_t sp_l = phys_dev((uint32_t)(2 * lane) & 31u);
    const int shalf = (2 * lane) >> 5;                                // bit 5 of 2 lane
    for (int64_t i = 0; i < count + S; ++i) {
      const int b = (int)(i % S);
      float2* sb = buf + (size_t)b * TS;
      if (i >= S) {
        if (!ws_wait(&empty[b], (uint32_t)(((i - S) / S) & 1), abort)) break;
        const uint64_t gb = tile_base_fast(ttab, blockIdx.x + (i - S) * step);
        float2* g = a.psi + gb + so_l;
#pragma unroll 4
        for (int j = pw; j < NH / 2; j += kWsProducers) {
          const int h = 2 * j + shalf;
          const uint32_t p = sp_l ^ hphys[h];
          const float2 x = sb[p], y = sb[p ^ 1u];
          __stcs(reinterpret_cast<float4*>(g + hoff[h]), make_float4(x.x, x.y, y.x, y.y));
        }
      }
      if (i < count) {
        const uint64_t gb = tile_base_fast(ttab, blockIdx.x + i * step);
        const float2* g = a.psi + gb + lo_l;
        // each producer warp refills exactly the 64-amplitude groups
        // (tile index >> 6 = jj) whose write-back it has just read, so no
        // warp overwrites data another warp still has to store
#pragma unroll 4
        for (int jj = pw; jj < NH / 2; jj += kWsProducers) {
          cp_async8(sb + (lp_l ^ hphys[2 * jj]), g + hoff[2 * jj]);
          cp_async8(sb + (lp_l ^ hphys[2 * jj + 1]), g + hoff[2 * jj + 1]);
        }
        asm volatile("cp.async.mbarrier.arrive.noinc.shared.b64 [%0];\n" ::"r"(ws_su32(&full[b])) : "memory");
      }
    }
    cp_async_wait<0>();
  } else {
    // ---- consumer warps
    for (int64_t i = 0; i < count; ++i) {
      const int b = (int)(i % S);
      const bool ok = ws_wait(&full[b], (uint32_t)((i / S) & 1), abort);
      if (consumers_any(!ok)) break;
      float2* sb = buf + (size_t)b * TS;
      const int64_t tile = blockIdx.x + i * step;
      const uint64_t gbase = tile_base_fast(ttab, tile);
      run_ops<LT, 0, false, 2, true>(ti, a.ops, sb, nullptr, gbase, tile, red, ltab, nltab);
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(ws_su32(&empty[b])) : "memory");
    }
  }
  if (t == 0 || t == kThreads) {  // one consumer and one producer thread report an abort
    if (*abort && a.abort) atomicExch(a.abort, 1);
  }
}

template <int LT>
int launch_tile_ws(Ctx* c, const PassArgs& a) {
  constexpr int smem = kWsStages * (1 << LT) * (int)sizeof(float2);
  static int blocks_per_sm = -1;
  cudaError_t e;
  if (blocks_per_sm < 0) {
    e = cudaFuncSetAttribute(k_tile_ws<LT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tile_ws)");
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tile_ws<LT>, kWsThreads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    blocks_per_sm = nb > 0 ? nb : 1;
    if (getenv("GBQ_DEBUG"))
      fprintf(stderr, "k_tile_ws<L=%d>: %d blocks/SM, %d B smem\n", LT, blocks_per_sm, smem);
  }
  int64_t grid = (int64_t)c->sm_count * blocks_per_sm;
  if (grid > a.ti.ntiles) grid = a.ti.ntiles;
  k_tile_ws<LT><<<(unsigned)grid, kWsThreads, smem, c->stream>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_tile_ws launch");
  c->launches += 1;
  return GBQ_OK;
}

// Warp-specialised passes: single state, register/diag ops of width <= 2
// only, tile bits 0..4 = global bits 0..4.  GBQ_WS=0 turns them off.
inline bool ws_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("GBQ_WS");
    on = (e && atoi(e) == 0) ? 0 : 1;
  }
  return on == 1;
}

// Widest register dense op of a pass.
inline int pass_rkmax(const PassArgs& a) {
  int k = 0;
  for (int o = 0; o < a.ti.nops; ++o) {
    const int kind = a.ops[o].kind;
    if ((kind == GBQ_OP_RDENSE || kind == GBQ_OP_RPROBE) && a.ops[o].k > k) k = a.ops[o].k;
  }
  return k;
}

template <int LT, int KMAX, bool DUAL>
int launch_tile_pass(Ctx* c, const PassArgs& a) {
  if constexpr (KMAX == 0 && !DUAL) {
    if (pass_rkmax(a) <= 2) {
      if constexpr (LT == 12) {
        if (ws_enabled() && a.ti.m >= 5) return launch_tile_ws<LT>(c, a);
      }
      return launch_tile_pass_stages<LT, 0, false, 2, 2>(c, a);
    }
  }
  if constexpr (KMAX == 0 && DUAL) {
    // two-state (adjoint) passes of width <= 2 register ops: the lean variant
    if (pass_rkmax(a) <= 2) return launch_tile_pass_stages<LT, 0, true, 2, 2>(c, a);
  }
  return launch_tile_pass_stages<LT, KMAX, DUAL, 2, 4>(c, a);
}

// Widest shared-memory dense (or dense-probe) op of a pass (0 if none).
inline int pass_kmax(const PassArgs& a) {
  int k = 0;
  for (int o = 0; o < a.ti.nops; ++o) {
    const int kind = a.ops[o].kind;
    if ((kind == GBQ_OP_DENSE || kind == GBQ_OP_PROBE) && a.ops[o].k > k) k = a.ops[o].k;
  }
  return k;
}

}  // namespace gbq
