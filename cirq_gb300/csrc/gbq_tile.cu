// Tile-pass kernels: the state-vector / density-matrix hot path.
//
// One launch = one pass over the state.  Each CTA owns one tile of 2^L
// amplitudes at a time: tile bits 0..m-1 are the global index bits 0..m-1
// (so every tile is read as 2^(L-m) contiguous runs of 2^m amplitudes with
// 128-bit loads), tile bits m..L-1 are arbitrary global bits chosen by the
// host planner.  The tile is staged in shared memory, every op of the pass
// is applied to it there, and it is written back in place: HBM traffic per
// pass is one read and one write of the state whatever the number of ops.
//
// Replaces the numpy passes of the reference, one per operation:
// linalg.targeted_left_multiply (cirq-core/cirq/linalg/transformations.py:105-172),
// linalg.apply_matrix_to_slices (transformations.py:310-380), the gates'
// own _apply_unitary_ (cirq-core/cirq/ops/common_gates.py:123-134, 658-669,
// 1072-1082) and the Kraus/unitary channel paths
// (cirq-core/cirq/protocols/apply_channel_protocol.py:274-356).
//
// Shared-memory layout: amplitude i of the tile lives at phys(i) =
// i ^ swz(i), where swz() XORs a distinct non-unit 4-bit vector per tile bit
// >= 4 into bits 0..3.  For any op the host picks 4 "lane" bits whose
// vectors are independent, so the 16 lanes of a half-warp always hit 16
// different 8-byte bank pairs.

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbq_internal.cuh"

namespace gbq {

// Columns (tile bits 4..13) of the swizzle: distinct, nonzero, non-unit.
// swz bit r = parity(i & kSwzRow[r]).  Must match cirq_gb300/planner.py.
constexpr uint32_t kSwzV[10] = {3, 5, 6, 9, 10, 12, 7, 11, 13, 14};
constexpr uint32_t swz_row(int r) {
  uint32_t m = 0;
  for (int b = 0; b < 10; ++b)
    if ((kSwzV[b] >> r) & 1) m |= 1u << (b + 4);
  return m;
}
constexpr uint32_t kRow0 = swz_row(0), kRow1 = swz_row(1), kRow2 = swz_row(2), kRow3 = swz_row(3);

__device__ __forceinline__ uint32_t phys(uint32_t i) {
  uint32_t s = (__popc(i & kRow0) & 1) | ((__popc(i & kRow1) & 1) << 1) |
               ((__popc(i & kRow2) & 1) << 2) | ((__popc(i & kRow3) & 1) << 3);
  return i ^ s;
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

// Deposit the low `nb` bits of x at the tile positions pos[0..nb-1].
__device__ __forceinline__ uint32_t deposit(uint32_t x, const int8_t* pos, int nb) {
  uint32_t r = 0;
  for (int b = 0; b < nb; ++b) r |= ((x >> b) & 1u) << pos[b];
  return r;
}

__device__ __forceinline__ uint64_t hi_offset(const TileInfo& a, uint32_t x) {
  uint64_t r = 0;
  const int nh = a.L - a.m;
  for (int b = 0; b < nh; ++b) r |= (uint64_t)((x >> b) & 1u) << a.hi[b];
  return r;
}

__device__ __forceinline__ uint32_t code_bit(int8_t c, uint32_t tile_index, uint64_t gbase) {
  return c >= 0 ? ((tile_index >> c) & 1u) : (uint32_t)((gbase >> (-c - 1)) & 1u);
}

// ---- tile load / store ------------------------------------------------------
__device__ __forceinline__ void load_tile(const TileInfo& a, float2* sm, const float2* src,
                                          uint64_t gbase) {
  const uint32_t npairs = 1u << (a.L - 1);
  const uint32_t mmask = (1u << a.m) - 1u;
  for (uint32_t p = threadIdx.x; p < npairs; p += kThreads) {
    const uint32_t i = p << 1;
    const uint64_t off = gbase | (i & mmask) | hi_offset(a, i >> a.m);
    const float4 v = *reinterpret_cast<const float4*>(src + off);
    const uint32_t pi = phys(i);
    sm[pi] = make_float2(v.x, v.y);
    sm[pi ^ 1u] = make_float2(v.z, v.w);
  }
}

__device__ __forceinline__ void store_tile(const TileInfo& a, const float2* sm, float2* dst,
                                           uint64_t gbase) {
  const uint32_t npairs = 1u << (a.L - 1);
  const uint32_t mmask = (1u << a.m) - 1u;
  for (uint32_t p = threadIdx.x; p < npairs; p += kThreads) {
    const uint32_t i = p << 1;
    const uint64_t off = gbase | (i & mmask) | hi_offset(a, i >> a.m);
    const uint32_t pi = phys(i);
    const float2 x = sm[pi], y = sm[pi ^ 1u];
    *reinterpret_cast<float4*>(dst + off) = make_float4(x.x, x.y, y.x, y.y);
  }
}

// ---- CTA reduction (probes) -------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ void cta_sum_store(double v, double* out, double* red) {
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

// ---- dense k-qubit op (and dense probe) --------------------------------------
// Groups of 2^K amplitudes (the K target bits varying) are distributed over
// the CTA; when there are fewer groups than threads, the 2^K output rows of
// a group are split across R threads.
template <int K, int LTMAX, bool DUAL, bool PROBE>
__device__ __forceinline__ void op_dense(const TileInfo& a, const gbq_op& op, float2* smA,
                                         float2* smB, uint64_t gbase, int64_t tile, double* red) {
  constexpr int D = 1 << K;
  constexpr int WMAX = ((1 << LTMAX) >> K) / kThreads > 0 ? ((1 << LTMAX) >> K) / kThreads : 1;
  const int L = a.L;
  const uint32_t NG = 1u << (L - K);
  uint32_t R = NG >= (uint32_t)kThreads ? 1u : (uint32_t)kThreads / NG;
  if (R > (uint32_t)D) R = D;
  const uint32_t NW = NG * R;
  const int RPI = D / (int)R;

  uint32_t poff[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    uint32_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> b) & 1) o |= 1u << op.bits[b];
    poff[j] = phys(o);
  }

  float2 va[WMAX][D];
  float2 vb[DUAL ? WMAX : 1][DUAL ? D : 1];
  uint32_t pb[WMAX];
  const float2* mp[WMAX];
  int r0[WMAX];
  bool act[WMAX];
  // thread part of the group index (low 9 bits) deposited once
  const int ngb = L - K;
  const int nlo = ngb < 9 ? ngb : 9;
  const uint32_t tpart = deposit(threadIdx.x & ((1u << nlo) - 1u), op.gorder, nlo);
#pragma unroll
  for (int w = 0; w < WMAX; ++w) {
    const uint32_t id = threadIdx.x + (uint32_t)w * kThreads;
    act[w] = id < NW;
    const uint32_t g = id & (NG - 1u);
    const uint32_t rc = id >> (L - K);
    uint32_t base;
    if (NG >= (uint32_t)kThreads) {
      base = tpart | deposit(g >> 9, op.gorder + 9, ngb - 9);
    } else {
      base = deposit(g, op.gorder, ngb);
    }
    pb[w] = phys(base);
    uint32_t sel = 0;
    for (int s = 0; s < op.nsel; ++s) sel |= code_bit(op.sel[s], base, gbase) << s;
    mp[w] = a.mats + op.mat + (int64_t)sel * D * D;
    r0[w] = (int)rc * RPI;
    if (act[w]) {
#pragma unroll
      for (int j = 0; j < D; ++j) {
        va[w][j] = smA[pb[w] ^ poff[j]];
        if constexpr (DUAL) vb[w][j] = smB[pb[w] ^ poff[j]];
      }
    }
  }

  if constexpr (PROBE) {
    // Re <lam| D |psi> over this thread's rows; smA = psi, smB = lam.
    double accd = 0.0;
#pragma unroll
    for (int w = 0; w < WMAX; ++w) {
      if (!act[w]) continue;
      float part = 0.f;
#pragma unroll
      for (int r = 0; r < D; ++r) {
        if (r < r0[w] || r >= r0[w] + RPI) continue;
        const float2* row = mp[w] + r * D;
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; c += 2) {
          const float4 mm = __ldg(reinterpret_cast<const float4*>(row + c));
          cfma(acc, make_float2(mm.x, mm.y), va[w][c]);
          if (c + 1 < D) cfma(acc, make_float2(mm.z, mm.w), va[w][c + 1]);
        }
        // Re(conj(l) * acc)
        part = fmaf(vb[w][r].x, acc.x, part);
        part = fmaf(vb[w][r].y, acc.y, part);
      }
      accd += (double)part;
    }
    cta_sum_store(accd, a.partial + (int64_t)op.slot * a.ntiles + tile, red);
  } else {
    if (R > 1) __syncthreads();  // other threads still read this group's inputs
#pragma unroll
    for (int r = 0; r < D; ++r) {
      if constexpr (K <= 3) {
        // rows are short: load once, reuse for every group of this thread
        float2 row[D];
        const float2* rp = mp[0] + r * D;
#pragma unroll
        for (int c = 0; c < D; c += 2) {
          const float4 mm = __ldg(reinterpret_cast<const float4*>(rp + c));
          row[c] = make_float2(mm.x, mm.y);
          if (c + 1 < D) row[c + 1] = make_float2(mm.z, mm.w);
        }
#pragma unroll
        for (int w = 0; w < WMAX; ++w) {
          if (!act[w] || r < r0[w] || r >= r0[w] + RPI) continue;
          if (op.nsel && w > 0) {
            const float2* rq = mp[w] + r * D;
#pragma unroll
            for (int c = 0; c < D; c += 2) {
              const float4 mm = __ldg(reinterpret_cast<const float4*>(rq + c));
              row[c] = make_float2(mm.x, mm.y);
              if (c + 1 < D) row[c + 1] = make_float2(mm.z, mm.w);
            }
          }
          float2 acc = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; ++c) cfma(acc, row[c], va[w][c]);
          smA[pb[w] ^ poff[r]] = acc;
          if constexpr (DUAL) {
            float2 accb = make_float2(0.f, 0.f);
#pragma unroll
            for (int c = 0; c < D; ++c) cfma(accb, row[c], vb[w][c]);
            smB[pb[w] ^ poff[r]] = accb;
          }
        }
      } else {
#pragma unroll
        for (int w = 0; w < WMAX; ++w) {
          if (!act[w] || r < r0[w] || r >= r0[w] + RPI) continue;
          const float2* rp = mp[w] + r * D;
          float2 acc = make_float2(0.f, 0.f);
          float2 accb = make_float2(0.f, 0.f);
#pragma unroll
          for (int c = 0; c < D; c += 2) {
            const float4 mm = __ldg(reinterpret_cast<const float4*>(rp + c));
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

// ---- diagonal op (and diagonal probe) -----------------------------------------
template <bool DUAL, bool PROBE>
__device__ __forceinline__ void op_diag(const TileInfo& a, const gbq_op& op, float2* smA,
                                        float2* smB, uint64_t gbase, int64_t tile, double* red) {
  const int k = op.k;
  uint32_t ext = 0;
  for (int j = 0; j < k; ++j)
    if (op.bits[j] < 0) ext |= code_bit(op.bits[j], 0, gbase) << j;
  const float2* tab = a.mats + op.mat;
  const uint32_t n = 1u << a.L;
  float accf = 0.f;
  for (uint32_t i = threadIdx.x; i < n; i += kThreads) {
    uint32_t idx = ext;
    for (int j = 0; j < k; ++j) {
      const int8_t c = op.bits[j];
      if (c >= 0) idx |= ((i >> c) & 1u) << j;
    }
    const float2 d = __ldg(tab + idx);
    const uint32_t p = phys(i);
    if constexpr (PROBE) {
      const float2 y = cmul(d, smA[p]);
      const float2 l = smB[p];
      accf += fmaf(l.x, y.x, l.y * y.y);
    } else {
      smA[p] = cmul(d, smA[p]);
      if constexpr (DUAL) smB[p] = cmul(d, smB[p]);
    }
  }
  if constexpr (PROBE)
    cta_sum_store((double)accf, a.partial + (int64_t)op.slot * a.ntiles + tile, red);
}

template <int LTMAX, bool DUAL>
__device__ __forceinline__ void dispatch(const TileInfo& a, const gbq_op& op, float2* smA,
                                         float2* smB, uint64_t gbase, int64_t tile, double* red) {
  switch (op.kind) {
    case GBQ_OP_DENSE:
      switch (op.k) {
        case 1: op_dense<1, LTMAX, DUAL, false>(a, op, smA, smB, gbase, tile, red); break;
        case 2: op_dense<2, LTMAX, DUAL, false>(a, op, smA, smB, gbase, tile, red); break;
        case 3: op_dense<3, LTMAX, DUAL, false>(a, op, smA, smB, gbase, tile, red); break;
        case 4: op_dense<4, LTMAX, DUAL, false>(a, op, smA, smB, gbase, tile, red); break;
        case 5: op_dense<5, LTMAX, DUAL, false>(a, op, smA, smB, gbase, tile, red); break;
        default: break;
      }
      break;
    case GBQ_OP_DIAG:
      op_diag<DUAL, false>(a, op, smA, smB, gbase, tile, red);
      break;
    case GBQ_OP_PROBE:
      if constexpr (DUAL) {
        switch (op.k) {
          case 1: op_dense<1, LTMAX, true, true>(a, op, smA, smB, gbase, tile, red); break;
          case 2: op_dense<2, LTMAX, true, true>(a, op, smA, smB, gbase, tile, red); break;
          case 3: op_dense<3, LTMAX, true, true>(a, op, smA, smB, gbase, tile, red); break;
          default: break;
        }
      }
      break;
    case GBQ_OP_PROBE_DIAG:
      if constexpr (DUAL) op_diag<true, true>(a, op, smA, smB, gbase, tile, red);
      break;
    default:
      break;
  }
}

// Runs the ops of one pass on the tile whose global base index is gbase.
template <int LTMAX, bool DUAL>
__device__ __forceinline__ void run_tile(const TileInfo& ti, const gbq_op* ops, float2* psi,
                                         float2* lam, float2* smA, float2* smB, uint64_t gbase,
                                         int64_t tile, double* red) {
  load_tile(ti, smA, psi, gbase);
  if constexpr (DUAL) load_tile(ti, smB, lam, gbase);
  __syncthreads();
  for (int o = 0; o < ti.nops; ++o) {
    dispatch<LTMAX, DUAL>(ti, ops[o], smA, smB, gbase, tile, red);
    __syncthreads();
  }
  store_tile(ti, smA, psi, gbase);
  if constexpr (DUAL) store_tile(ti, smB, lam, gbase);
  __syncthreads();
}

__device__ __forceinline__ uint64_t tile_base(const TileInfo& ti, int64_t tile) {
  uint64_t gbase = 0;
  const int nnt = ti.nbits - ti.L;
  for (int j = 0; j < nnt; ++j) gbase |= (uint64_t)((tile >> j) & 1) << ti.nt[j];
  return gbase;
}

template <int LTMAX, bool DUAL>
__global__ void __launch_bounds__(kThreads) k_tile_pass(const __grid_constant__ PassArgs a) {
  extern __shared__ float4 smraw[];
  __shared__ double red[kThreads / 32];
  float2* smA = reinterpret_cast<float2*>(smraw);
  float2* smB = smA + (1u << a.ti.L);
  for (int64_t tile = blockIdx.x; tile < a.ti.ntiles; tile += gridDim.x) {
    run_tile<LTMAX, DUAL>(a.ti, a.ops, a.psi, a.lam, smA, smB, tile_base(a.ti, tile), tile, red);
  }
}

// ---- persistent batch kernel --------------------------------------------------
// Each CTA repeatedly claims the next parameter point (an atomic counter, no
// waiting on other CTAs), simulates it alone in its own scratch slot, and
// writes the point's expectation value.  Points may have different widths.
__global__ void __launch_bounds__(kThreads)
    k_batch(const gbq_point* __restrict__ points, int npoints, const gbq_pass* __restrict__ passes,
            const gbq_op* __restrict__ ops, const float2* __restrict__ mats,
            const gbq_pauli* __restrict__ terms, float2* slots, int64_t slot_stride, int* counter,
            double* out) {
  extern __shared__ float4 smraw[];
  __shared__ double red[kThreads / 32];
  __shared__ TileInfo ti;
  __shared__ gbq_op sops[GBQ_MAX_OPS_PER_PASS];
  __shared__ int s_point;
  float2* sm = reinterpret_cast<float2*>(smraw);
  float2* psi = slots + (int64_t)blockIdx.x * slot_stride;
  for (;;) {
    if (threadIdx.x == 0) s_point = atomicAdd(counter, 1);
    __syncthreads();
    const int p = s_point;
    __syncthreads();
    if (p >= npoints) break;
    const gbq_point pt = points[p];
    const uint64_t dim = 1ull << pt.nbits;
    for (uint64_t i = threadIdx.x; i < dim; i += kThreads)
      psi[i] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
    __syncthreads();
    for (int q = 0; q < pt.pass_count; ++q) {
      const gbq_pass& ps = passes[pt.pass_begin + q];
      if (threadIdx.x == 0) {
        ti.mats = mats + pt.mat_base;
        ti.partial = nullptr;
        ti.nbits = pt.nbits;
        ti.L = ps.L;
        ti.m = ps.m;
        ti.nops = ps.op_count;
        ti.ntiles = 1ll << (pt.nbits - ps.L);
        uint32_t inmask = (1u << ps.m) - 1u;
        for (int j = 0; j < 16; ++j) ti.hi[j] = ps.hi[j];
        for (int j = 0; j < ps.L - ps.m; ++j) inmask |= 1u << ps.hi[j];
        int c = 0;
        for (int b = 0; b < pt.nbits; ++b)
          if (!((inmask >> b) & 1u)) ti.nt[c++] = (int8_t)b;
      }
      for (int o = threadIdx.x; o < ps.op_count; o += kThreads) sops[o] = ops[ps.op_begin + o];
      __syncthreads();
      for (int64_t tile = 0; tile < ti.ntiles; ++tile)
        run_tile<13, false>(ti, sops, psi, nullptr, sm, nullptr, tile_base(ti, tile), tile, red);
    }
    // <psi| sum_t coef_t P_t |psi>, P_t = i^ny X^x Z^zy (phase on the input index)
    double re_acc = 0.0, im_acc = 0.0;
    for (int t = 0; t < pt.term_count; ++t) {
      const gbq_pauli tp = terms[pt.term_begin + t];
      float sre = 0.f, sim = 0.f;
      for (uint64_t i = threadIdx.x; i < dim; i += kThreads) {
        const uint64_t j = i ^ tp.x;
        const float2 a = psi[i], b = psi[j];
        const float sg = (__popcll(j & tp.zy) & 1) ? -1.f : 1.f;
        // conj(a) * b * sg
        sre += sg * fmaf(a.x, b.x, a.y * b.y);
        sim += sg * fmaf(a.x, b.y, -a.y * b.x);
      }
      // multiply by coef * i^ny
      double cr = tp.coef, ci = 0.0;
      const int ny = tp.ny & 3;
      if (ny == 1) { ci = cr; cr = 0.0; }
      else if (ny == 2) { cr = -cr; }
      else if (ny == 3) { ci = -cr; cr = 0.0; }
      re_acc += cr * sre - ci * sim;
      im_acc += cr * sim + ci * sre;
    }
    cta_sum_store(re_acc, out + 2 * p, red);
    cta_sum_store(im_acc, out + 2 * p + 1, red);
  }
}

int launch_batch(Ctx* c, const gbq_point* d_points, int npoints, const gbq_pass* d_passes,
                 const gbq_op* d_ops, const float2* mats, const gbq_pauli* d_terms, int max_nbits,
                 float2* slots, int nslots, int* d_counter, double* d_out) {
  const size_t smem = (size_t)(1 << 13) * sizeof(float2);
  static bool attr = false;
  cudaError_t e;
  if (!attr) {
    e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_batch)");
    attr = true;
  }
  k_batch<<<nslots, kThreads, smem, c->stream>>>(d_points, npoints, d_passes, d_ops, mats, d_terms,
                                                 slots, (int64_t)1 << max_nbits, d_counter, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_batch launch");
  c->launches += 1;
  return GBQ_OK;
}

int launch_pass(Ctx* c, const PassArgs& a, bool dual) {
  const size_t smem = (dual ? 2 : 1) * ((size_t)1 << a.ti.L) * sizeof(float2);
  const int64_t grid64 = a.ti.ntiles < (int64_t)0x7fffffff ? a.ti.ntiles : (int64_t)0x7fffffff;
  const unsigned grid = (unsigned)grid64;
  cudaError_t e;
  if (dual) {
    static bool attr = false;
    if (!attr) {
      e = cudaFuncSetAttribute(k_tile_pass<13, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               2 * (1 << 13) * (int)sizeof(float2));
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tile_pass dual)");
      attr = true;
    }
    k_tile_pass<13, true><<<grid, kThreads, smem, c->stream>>>(a);
  } else {
    static bool attr = false;
    if (!attr) {
      e = cudaFuncSetAttribute(k_tile_pass<13, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (1 << 13) * (int)sizeof(float2));
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_tile_pass)");
      attr = true;
    }
    k_tile_pass<13, false><<<grid, kThreads, smem, c->stream>>>(a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_tile_pass launch");
  c->launches += 1;
  return GBQ_OK;
}

}  // namespace gbq
