// Persistent batch kernel: many parameter points (possibly of different
// widths) in one launch.  Replaces the per-resolver loop of
// SimulatesIntermediateState.simulate_sweep_iter (cirq-core/cirq/sim/simulator.py:558-605)
// that feeds Simulator.simulate_expectation_values_sweep_iter
// (cirq-core/cirq/sim/sparse_simulator.py:193-218).
//
// Each CTA repeatedly claims the next point with an atomic counter (no CTA
// ever waits for another), simulates it alone in its own scratch slot with
// the same 12-bit tile code as the single-state kernels, and writes
// c_t <psi|P_t|psi> for each of the point's Pauli terms.

#include "gbq_tile.cuh"

namespace gbq {

constexpr int kBatchTile = 12;
constexpr int kTermGroup = 8;    // terms sharing one read of the state

template <int KMAX>
__global__ void __launch_bounds__(kThreads, 2)
    k_batch(const gbq_point* __restrict__ points, int npoints, const gbq_pass* __restrict__ passes,
            const OpDev* __restrict__ ops, const float2* __restrict__ mats,
            const gbq_pauli* __restrict__ terms, float2* slots, int64_t slot_stride, int* counter,
            double* out) {
  constexpr int LT = kBatchTile;
  extern __shared__ float4 smraw[];
  __shared__ double red[kThreads / 32];
  __shared__ TileInfo ti;
  __shared__ OpDev sops[GBQ_MAX_OPS_PER_PASS];
  __shared__ uint64_t ttab[3 * kTileTab];
  __shared__ int s_point;
  constexpr int TS = 1 << LT;
  float2* buf = reinterpret_cast<float2*>(smraw);  // [2][TS]
  float2* psi = slots + (int64_t)blockIdx.x * slot_stride;
  for (;;) {
    if (threadIdx.x == 0) s_point = atomicAdd(counter, 1);
    __syncthreads();
    const int p = s_point;
    __syncthreads();
    if (p >= npoints) break;
    const gbq_point pt = points[p];
    const uint64_t dim = 1ull << pt.nbits;
    for (uint64_t i = threadIdx.x; i < dim; i += kThreads) psi[i] = make_float2(i == 0 ? 1.f : 0.f, 0.f);
    __syncthreads();
    for (int q = 0; q < pt.pass_count; ++q) {
      const gbq_pass& ps = passes[pt.pass_begin + q];
      if (threadIdx.x == 0) {
        ti.mats = mats + pt.mat_base;
        ti.partial = nullptr;
        ti.pstride = 0;
        ti.pshift = 0;
        ti.nbits = pt.nbits;
        ti.L = ps.L;
        ti.m = ps.m;
        ti.nops = ps.op_count;
        ti.ntiles = 1ll << (pt.nbits - ps.L);
        uint64_t inmask = (1ull << ps.m) - 1ull;
        for (int b = 0; b < ps.m; ++b) ti.gw[b] = 1ull << b;
        for (int j = 0; j < ps.L - ps.m; ++j) {
          ti.gw[ps.m + j] = 1ull << ps.hi[j];
          inmask |= 1ull << ps.hi[j];
        }
        int c = 0;
        for (int b = 0; b < pt.nbits; ++b)
          if (!((inmask >> b) & 1ull)) ti.nt[c++] = (int8_t)b;
      }
      {
        const int nwords = ps.op_count * (int)(sizeof(OpDev) / 4);
        const uint32_t* src = reinterpret_cast<const uint32_t*>(ops + ps.op_begin);
        uint32_t* dst = reinterpret_cast<uint32_t*>(sops);
        for (int i = threadIdx.x; i < nwords; i += kThreads) dst[i] = src[i];
      }
      __syncthreads();
      tile_tables_build(ti, ttab);
      const TileSetup ts = tile_setup<LT>(ti);
      __syncthreads();
      // every global write of the previous pass is visible here: the whole
      // pass ran in this CTA and ended with __syncthreads()
      load_tile_async<LT>(ti, psi, buf, tile_base_fast(ttab, 0), ts.lo_t, ts.lp_t);
      cp_async_commit();
      int cur = 0;
      for (int64_t tile = 0; tile < ti.ntiles; ++tile) {
        if (tile + 1 < ti.ntiles)
          load_tile_async<LT>(ti, psi, buf + (cur ^ 1) * TS, tile_base_fast(ttab, tile + 1), ts.lo_t, ts.lp_t);
        cp_async_commit();
        cp_async_wait<1>();
        __syncthreads();
        const uint64_t gbase = tile_base_fast(ttab, tile);
        run_ops<LT, KMAX, false, 4>(ti, sops, buf + cur * TS, nullptr, gbase, tile, red);
        store_tile<LT>(ti, psi, buf + cur * TS, gbase, ts.off_t, ts.ph_t);
        __syncthreads();
        cur ^= 1;
      }
      cp_async_wait<0>();
      __syncthreads();
    }
    // per term: coef_t <psi|P_t|psi>, P_t = i^ny X^x Z^zy (sign on the input
    // index); consecutive terms with the same X mask (up to kTermGroup) share
    // one read of the state
    for (int t = 0; t < pt.term_count;) {
      const gbq_pauli* tb = terms + pt.term_begin + t;
      const uint64_t x = tb[0].x;
      int g = 1;
      while (t + g < pt.term_count && g < kTermGroup && tb[g].x == x) ++g;
      uint64_t zy[kTermGroup];
      float sre[kTermGroup], sim[kTermGroup];
#pragma unroll
      for (int u = 0; u < kTermGroup; ++u) {
        zy[u] = u < g ? tb[u].zy : 0ull;
        sre[u] = sim[u] = 0.f;
      }
      for (uint64_t i = threadIdx.x; i < dim; i += kThreads) {
        const uint64_t j = i ^ x;
        const float2 a = psi[i], b = psi[j];
        const float pr = fmaf(a.x, b.x, a.y * b.y), pi = fmaf(a.x, b.y, -a.y * b.x);
#pragma unroll
        for (int u = 0; u < kTermGroup; ++u) {
          const float sg = (__popcll(j & zy[u]) & 1) ? -1.f : 1.f;
          sre[u] = fmaf(sg, pr, sre[u]);
          sim[u] = fmaf(sg, pi, sim[u]);
        }
      }
      for (int u = 0; u < g; ++u) {
        double cr = tb[u].coef, ci = 0.0;
        const int ny = tb[u].ny & 3;
        if (ny == 1) { ci = cr; cr = 0.0; }
        else if (ny == 2) { cr = -cr; }
        else if (ny == 3) { ci = -cr; cr = 0.0; }
        const int64_t o = 2 * ((int64_t)pt.term_begin + t + u);
        cta_sum_store(cr * sre[u] - ci * sim[u], out + o, red);
        cta_sum_store(cr * sim[u] + ci * sre[u], out + o + 1, red);
      }
      t += g;
    }
  }
}

template <int KMAX>
static int launch_batch_k(Ctx* c, const gbq_point* d_points, int npoints, const gbq_pass* d_passes,
                          const OpDev* d_ops, const float2* mats, const gbq_pauli* d_terms,
                          int max_nbits, float2* slots, int nslots, int* d_counter, double* d_out) {
  const int smem = 2 * (1 << kBatchTile) * (int)sizeof(float2);
  static bool attr = false;
  cudaError_t e;
  if (!attr) {
    e = cudaFuncSetAttribute(k_batch<KMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_batch)");
    attr = true;
  }
  k_batch<KMAX><<<nslots, kThreads, smem, c->stream>>>(d_points, npoints, d_passes, d_ops, mats,
                                                       d_terms, slots, (int64_t)1 << max_nbits,
                                                       d_counter, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_batch launch");
  c->launches += 1;
  return GBQ_OK;
}

// kmax: widest shared-memory dense op of all points' passes (0: register
// phases only, which selects the lean kernel variant).
int launch_batch(Ctx* c, const gbq_point* d_points, int npoints, const gbq_pass* d_passes,
                 const OpDev* d_ops, const float2* mats, const gbq_pauli* d_terms, int max_nbits,
                 float2* slots, int nslots, int* d_counter, double* d_out, int kmax) {
  if (kmax == 0)
    return launch_batch_k<0>(c, d_points, npoints, d_passes, d_ops, mats, d_terms, max_nbits, slots,
                             nslots, d_counter, d_out);
  return launch_batch_k<5>(c, d_points, npoints, d_passes, d_ops, mats, d_terms, max_nbits, slots,
                           nslots, d_counter, d_out);
}

}  // namespace gbq
