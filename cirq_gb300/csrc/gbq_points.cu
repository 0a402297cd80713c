// Batched points: the states of many parameter points of one compiled circuit
// lie back to back (point p at states + p * 2^nbits) and are evolved pass by
// pass together -- one launch of the ordinary tile pass per pass covers every
// point (gbq_run_points in gbq_abi.cu) -- so a sweep streams through HBM as
// one large state instead of one CTA per point.  This file holds the two
// per-point kernels around it: |0...0> initialisation and Pauli-term sums.
//
// Replaces the per-resolver loop of SimulatesIntermediateState.simulate_sweep_iter
// (cirq-core/cirq/sim/simulator.py:558-605) feeding
// Simulator.simulate_expectation_values_sweep_iter
// (cirq-core/cirq/sim/sparse_simulator.py:193-218).

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbq_internal.cuh"

namespace gbq {

namespace {

constexpr int kPtThreads = 256;
constexpr int kPtGroup = 8;  // terms sharing one read of the state

__global__ void k_points_basis(float2* __restrict__ states, int nbits, int npoints) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npoints) states[(int64_t)p << nbits] = make_float2(1.f, 0.f);
}

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kPtThreads / 32; ++w) r += red[w];
  return r;
}

// Block (chunk c, point p) adds its part of <psi_p|P_t|psi_p> (unit
// coefficient, P_t = i^ny X^x Z^zy with the sign on the input index) to
// out[(p * nterms + t) * 2 + {re, im}].  Terms with equal X masks must be
// adjacent: up to kPtGroup of them share one read of the chunk.
__global__ void __launch_bounds__(kPtThreads) k_points_expect(const float2* __restrict__ states, int nbits,
                                                             int chunk_bits, const gbq_pauli* __restrict__ terms,
                                                             int nterms, double* __restrict__ out) {
  __shared__ double red[kPtThreads / 32];
  const int p = blockIdx.y;
  const float2* psi = states + ((int64_t)p << nbits);
  const uint64_t lo = (uint64_t)blockIdx.x << chunk_bits, hi = lo + (1ull << chunk_bits);
  for (int t = 0; t < nterms;) {
    const uint64_t x = terms[t].x;
    int g = 1;
    while (t + g < nterms && g < kPtGroup && terms[t + g].x == x) ++g;
    uint64_t zy[kPtGroup];
    float sre[kPtGroup], sim[kPtGroup];
#pragma unroll
    for (int u = 0; u < kPtGroup; ++u) {
      zy[u] = u < g ? terms[t + u].zy : 0ull;
      sre[u] = sim[u] = 0.f;
    }
    for (uint64_t i = lo + threadIdx.x; i < hi; i += kPtThreads) {
      const uint64_t j = i ^ x;
      const float2 a = psi[i], b = psi[j];
      const float pr = fmaf(a.x, b.x, a.y * b.y), pi = fmaf(a.x, b.y, -a.y * b.x);
#pragma unroll
      for (int u = 0; u < kPtGroup; ++u) {
        const float sg = (__popcll(j & zy[u]) & 1) ? -1.f : 1.f;
        sre[u] = fmaf(sg, pr, sre[u]);
        sim[u] = fmaf(sg, pi, sim[u]);
      }
    }
    for (int u = 0; u < g; ++u) {
      const double r = block_sum((double)sre[u], red);
      const double m = block_sum((double)sim[u], red);
      if (threadIdx.x == 0) {
        // i^ny phase of the term
        double re = r, im = m;
        const int ny = terms[t + u].ny & 3;
        if (ny == 1) { re = -m; im = r; }
        else if (ny == 2) { re = -r; im = -m; }
        else if (ny == 3) { re = m; im = -r; }
        double* o = out + ((int64_t)p * nterms + t + u) * 2;
        atomicAdd(o, re);
        atomicAdd(o + 1, im);
      }
    }
    t += g;
  }
}

// One CTA per point: draws out[p] from |psi_p|^2 with the uniform u[p]
// (inverse CDF in double: per-thread chunk sums, a block scan over the
// chunks, then the owning thread walks its chunk).
__global__ void __launch_bounds__(kPtThreads) k_points_sample(const float2* __restrict__ states, int nbits,
                                                             const double* __restrict__ u,
                                                             unsigned long long* __restrict__ out) {
  __shared__ double csum[kPtThreads];
  __shared__ int owner;
  const int p = blockIdx.x;
  const float2* psi = states + ((int64_t)p << nbits);
  const uint64_t dim = 1ull << nbits;
  const uint64_t per = (dim + kPtThreads - 1) / kPtThreads;
  const uint64_t lo = (uint64_t)threadIdx.x * per, hi = lo + per < dim ? lo + per : dim;
  double s = 0.0;
  for (uint64_t i = lo; i < hi; ++i) {
    const float2 a = psi[i];
    s += (double)a.x * a.x + (double)a.y * a.y;
  }
  csum[threadIdx.x] = s;
  if (threadIdx.x == 0) owner = -1;
  __syncthreads();
  // inclusive scan over the chunk sums (Hillis-Steele in shared memory)
  for (int o = 1; o < kPtThreads; o <<= 1) {
    const double v = threadIdx.x >= o ? csum[threadIdx.x - o] : 0.0;
    __syncthreads();
    csum[threadIdx.x] += v;
    __syncthreads();
  }
  const double total = csum[kPtThreads - 1];
  const double target = u[p] * total;
  const double before = threadIdx.x ? csum[threadIdx.x - 1] : 0.0;
  if (target >= before && (target < csum[threadIdx.x] || threadIdx.x == kPtThreads - 1)) atomicMax(&owner, (int)threadIdx.x);
  __syncthreads();
  if ((int)threadIdx.x == owner) {
    double acc = before;
    uint64_t pick = hi > lo ? hi - 1 : lo;
    for (uint64_t i = lo; i < hi; ++i) {
      const float2 a = psi[i];
      acc += (double)a.x * a.x + (double)a.y * a.y;
      if (acc > target) {
        pick = i;
        break;
      }
    }
    out[p] = pick;
  }
}

// Reduced density matrix of k <= 2 qubits for every point: block (chunk,
// point) sums psi[i(c, j)] conj(psi[i(c, l)]) over its share of the other
// index bits c and adds it to out[((p * D + j) * D + l) * 2 + {re, im}].
// Matrix index bit k-1-q <-> global bit g[q] (q = 0 is the first qubit of
// the channel, as in its Kraus matrices).
template <int K>
__global__ void __launch_bounds__(kPtThreads) k_points_rdm(const float2* __restrict__ states, int nbits, int g0,
                                                          int g1, int chunk_bits, double* __restrict__ out) {
  constexpr int D = 1 << K;
  __shared__ double red[kPtThreads / 32];
  const int p = blockIdx.y;
  const float2* psi = states + ((int64_t)p << nbits);
  const int glo = K == 1 ? g0 : (g0 < g1 ? g0 : g1), ghi = K == 1 ? g0 : (g0 < g1 ? g1 : g0);
  float re[D][D], im[D][D];
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int l = 0; l < D; ++l) re[j][l] = im[j][l] = 0.f;
  const uint64_t lo = (uint64_t)blockIdx.x << chunk_bits, hi = lo + (1ull << chunk_bits);
  for (uint64_t c = lo + threadIdx.x; c < hi; c += kPtThreads) {
    // insert zero bits at glo, then ghi
    uint64_t base = ((c >> glo) << (glo + 1)) | (c & ((1ull << glo) - 1));
    if (K == 2) base = ((base >> ghi) << (ghi + 1)) | (base & ((1ull << ghi) - 1));
    float2 a[D];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      uint64_t idx = base;
      if (K == 1) {
        if (j & 1) idx |= 1ull << g0;
      } else {
        if (j & 2) idx |= 1ull << g0;
        if (j & 1) idx |= 1ull << g1;
      }
      a[j] = psi[idx];
    }
#pragma unroll
    for (int j = 0; j < D; ++j)
#pragma unroll
      for (int l = 0; l < D; ++l) {
        re[j][l] = fmaf(a[j].x, a[l].x, fmaf(a[j].y, a[l].y, re[j][l]));
        im[j][l] = fmaf(a[j].y, a[l].x, fmaf(-a[j].x, a[l].y, im[j][l]));
      }
  }
#pragma unroll
  for (int j = 0; j < D; ++j)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      const double r = block_sum((double)re[j][l], red);
      const double m = block_sum((double)im[j][l], red);
      if (threadIdx.x == 0) {
        double* o = out + (((int64_t)p * D + j) * D + l) * 2;
        atomicAdd(o, r);
        atomicAdd(o + 1, m);
      }
    }
}

// Marginal distribution of m <= 5 measured qubits from the diagonal of every
// point's density matrix: rho_p = the 2nq-bit vector of point p (stride
// 2^nbits amplitudes; row index bits nq..2nq-1, column bits 0..nq-1), its
// diagonal entries at i (2^nq + 1).  Block (chunk, point) bins Re rho_p[i, i]
// of its share of the diagonal by the outcome sum_j bit(i, b_j) << j and adds
// the bins to out[p * 2^m + outcome].
__global__ void __launch_bounds__(kPtThreads) k_points_dm_marginal(const float2* __restrict__ states, int nbits,
                                                                  int nq, int m, int4 b03, int b4, int chunk_bits,
                                                                  double* __restrict__ out) {
  __shared__ double bins[32];
  const int p = blockIdx.y;
  const int nb = 1 << m;
  for (int j = threadIdx.x; j < nb; j += kPtThreads) bins[j] = 0.0;
  __syncthreads();
  const float2* rho = states + ((int64_t)p << nbits);
  const uint64_t step = (1ull << nq) + 1ull;
  const int bb[5] = {b03.x, b03.y, b03.z, b03.w, b4};
  const uint64_t lo = (uint64_t)blockIdx.x << chunk_bits, hi = lo + (1ull << chunk_bits);
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kPtThreads) {
    uint32_t o = 0;
#pragma unroll
    for (int j = 0; j < 5; ++j)
      if (j < m) o |= (uint32_t)((i >> bb[j]) & 1ull) << j;
    atomicAdd(&bins[o], (double)rho[i * step].x);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nb; j += kPtThreads) atomicAdd(out + (int64_t)p * nb + j, bins[j]);
}

}  // namespace

int points_dm_marginal(Ctx* c, const float2* states, int nbits, int nq, int npoints, int m, const int* bits,
                       double* d_out) {
  cudaError_t e = cudaMemsetAsync(d_out, 0, (size_t)npoints * (1u << m) * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(marginal out)");
  const int chunk_bits = nq < 16 ? nq : 16;
  dim3 grid((unsigned)(1u << (nq - chunk_bits)), (unsigned)npoints, 1);
  int b[5] = {0, 0, 0, 0, 0};
  for (int j = 0; j < m; ++j) b[j] = bits[j];
  k_points_dm_marginal<<<grid, kPtThreads, 0, c->stream>>>(states, nbits, nq, m, make_int4(b[0], b[1], b[2], b[3]),
                                                           b[4], chunk_bits, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_points_dm_marginal launch");
  c->launches += 1;
  return GBQ_OK;
}

int points_rdm(Ctx* c, const float2* states, int nbits, int npoints, int k, const int* g, double* d_out) {
  const int D = 1 << k;
  cudaError_t e = cudaMemsetAsync(d_out, 0, (size_t)npoints * D * D * 2 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(rdm out)");
  const int rest = nbits - k;
  const int chunk_bits = rest < 16 ? rest : 16;
  dim3 grid((unsigned)(1u << (rest - chunk_bits)), (unsigned)npoints, 1);
  if (k == 1)
    k_points_rdm<1><<<grid, kPtThreads, 0, c->stream>>>(states, nbits, g[0], g[0], chunk_bits, d_out);
  else
    k_points_rdm<2><<<grid, kPtThreads, 0, c->stream>>>(states, nbits, g[0], g[1], chunk_bits, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_points_rdm launch");
  c->launches += 1;
  return GBQ_OK;
}

int points_sample(Ctx* c, const float2* states, int nbits, int npoints, const double* d_u,
                  unsigned long long* d_out) {
  k_points_sample<<<npoints, kPtThreads, 0, c->stream>>>(states, nbits, d_u, d_out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_points_sample launch");
  c->launches += 1;
  return GBQ_OK;
}

int points_set_zero(Ctx* c, float2* states, int nbits, int npoints) {
  cudaError_t e = cudaMemsetAsync(states, 0, ((size_t)npoints << nbits) * sizeof(float2), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(points)");
  k_points_basis<<<(npoints + kPtThreads - 1) / kPtThreads, kPtThreads, 0, c->stream>>>(states, nbits, npoints);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_points_basis launch");
  c->launches += 1;
  return GBQ_OK;
}

int points_expect(Ctx* c, const float2* states, int nbits, int npoints, const gbq_pauli* d_terms, int nterms,
                  double* d_out) {
  cudaError_t e = cudaMemsetAsync(d_out, 0, (size_t)npoints * nterms * 2 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(points out)");
  if (nterms == 0) return GBQ_OK;
  const int chunk_bits = nbits < 16 ? nbits : 16;
  dim3 grid((unsigned)(1u << (nbits - chunk_bits)), (unsigned)npoints, 1);
  k_points_expect<<<grid, kPtThreads, 0, c->stream>>>(states, nbits, chunk_bits, d_terms, nterms, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_points_expect launch");
  c->launches += 1;
  return GBQ_OK;
}

}  // namespace gbq
