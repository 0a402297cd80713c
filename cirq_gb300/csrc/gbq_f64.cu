// Complex128 gate-by-gate passes: a double-precision state evolved one gate
// at a time, with no fusion and no tiles.
//
// This is the "complex128 GPU run" that the complex64 tile passes are
// checked against at sizes where the CPU oracle is too slow (a 30-qubit
// state is 16 GiB at complex128).  It shares nothing with the tile passes:
// each gate is one read and one write of the state by a plain grid-stride
// kernel that gathers the 2^k amplitudes of a group, multiplies them by the
// gate's matrix in double precision and scatters them back -- the
// arithmetic of linalg.targeted_left_multiply
// (cirq-core/cirq/linalg/transformations.py:105-172) on one group at a time.

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gbq_internal.cuh"

namespace gbq {
namespace {

constexpr int kF64Threads = 256;
constexpr int kF64MaxK = 3;

struct F64Gate {
  int k;
  int bits[kF64MaxK];         // matrix-index bit j <-> state index bit bits[j]
  int sorted[kF64MaxK];       // the same bits, ascending (for the group-index expansion)
  double2 m[1 << (2 * kF64MaxK)];  // row-major 2^k x 2^k
};

template <int K>
__global__ void k_f64_apply(double2* __restrict__ s, int64_t ngroups, const __grid_constant__ F64Gate g) {
  constexpr int D = 1 << K;
  uint64_t off[D];
#pragma unroll
  for (int j = 0; j < D; ++j) {
    uint64_t o = 0;
#pragma unroll
    for (int b = 0; b < K; ++b)
      if ((j >> b) & 1) o |= 1ull << g.bits[b];
    off[j] = o;
  }
  for (int64_t grp = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; grp < ngroups;
       grp += (int64_t)gridDim.x * blockDim.x) {
    // insert a zero at every target position (ascending) into the group index
    uint64_t base = (uint64_t)grp;
#pragma unroll
    for (int b = 0; b < K; ++b) {
      const int p = g.sorted[b];
      base = ((base >> p) << (p + 1)) | (base & ((1ull << p) - 1));
    }
    double2 a[D];
#pragma unroll
    for (int j = 0; j < D; ++j) a[j] = s[base | off[j]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      double re = 0.0, im = 0.0;
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const double2 m = g.m[r * D + c];
        re = fma(m.x, a[c].x, fma(-m.y, a[c].y, re));
        im = fma(m.x, a[c].y, fma(m.y, a[c].x, im));
      }
      s[base | off[r]] = make_double2(re, im);
    }
  }
}

__global__ void k_f64_basis(double2* __restrict__ s, int64_t n, uint64_t idx) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s[i] = make_double2((uint64_t)i == idx ? 1.0 : 0.0, 0.0);
}

// out[0] = max |a - b| (as the bit pattern of a non-negative double, whose
// integer order is its numeric order), out[1] = sum |a|^2, out[2] = sum |b|^2.
__global__ void k_f64_compare(const double2* __restrict__ a, const float2* __restrict__ b, int64_t n,
                              unsigned long long* dmax, double* sums) {
  double mx = 0.0, na = 0.0, nb = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = a[i];
    const float2 y = b[i];
    const double dx = x.x - (double)y.x, dy = x.y - (double)y.y;
    mx = fmax(mx, sqrt(dx * dx + dy * dy));
    na = fma(x.x, x.x, fma(x.y, x.y, na));
    nb = fma((double)y.x, (double)y.x, fma((double)y.y, (double)y.y, nb));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    na += __shfl_xor_sync(0xffffffffu, na, o);
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(dmax, (unsigned long long)__double_as_longlong(mx));
    atomicAdd(sums, na);
    atomicAdd(sums + 1, nb);
  }
}

int f64_grid(const Ctx* c, int64_t work) {
  int64_t g = (work + kF64Threads - 1) / kF64Threads;
  const int64_t cap = (int64_t)c->sm_count * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace gbq

using namespace gbq;

extern "C" {

int gbq_sv64_set_basis(gbq_ctx* c, void* state, int nbits, uint64_t index) {
  if (!c) {
    set_error("null context");
    return GBQ_ERR_ARG;
  }
  if (!state || nbits < 0 || nbits > 36 || (nbits < 64 && index >> nbits)) {
    set_error("gbq_sv64_set_basis: bad arguments");
    return GBQ_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  const int64_t n = (int64_t)1 << nbits;
  k_f64_basis<<<f64_grid(c, n), kF64Threads, 0, c->stream>>>(reinterpret_cast<double2*>(state), n, index);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_f64_basis launch");
  c->launches += 1;
  return GBQ_OK;
}

int gbq_sv64_apply(gbq_ctx* c, void* state, int nbits, int k, const int32_t* bits, const double* matrix) {
  if (!c) {
    set_error("null context");
    return GBQ_ERR_ARG;
  }
  if (!state || !bits || !matrix || nbits < 1 || nbits > 36 || k < 1 || k > kF64MaxK || k > nbits) {
    set_error("gbq_sv64_apply: bad arguments (k must be 1..3 and at most nbits)");
    return GBQ_ERR_ARG;
  }
  F64Gate g{};
  g.k = k;
  for (int j = 0; j < k; ++j) {
    if (bits[j] < 0 || bits[j] >= nbits) {
      set_error("gbq_sv64_apply: target bit out of range");
      return GBQ_ERR_ARG;
    }
    for (int i = 0; i < j; ++i)
      if (bits[i] == bits[j]) {
        set_error("gbq_sv64_apply: repeated target bit");
        return GBQ_ERR_ARG;
      }
    g.bits[j] = bits[j];
    g.sorted[j] = bits[j];
  }
  for (int i = 1; i < k; ++i)
    for (int j = i; j > 0 && g.sorted[j - 1] > g.sorted[j]; --j) {
      const int t = g.sorted[j];
      g.sorted[j] = g.sorted[j - 1];
      g.sorted[j - 1] = t;
    }
  const int d = 1 << k;
  for (int e2 = 0; e2 < d * d; ++e2) g.m[e2] = make_double2(matrix[2 * e2], matrix[2 * e2 + 1]);
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  const int64_t ngroups = (int64_t)1 << (nbits - k);
  double2* s = reinterpret_cast<double2*>(state);
  const int grid = f64_grid(c, ngroups);
  if (k == 1) k_f64_apply<1><<<grid, kF64Threads, 0, c->stream>>>(s, ngroups, g);
  else if (k == 2) k_f64_apply<2><<<grid, kF64Threads, 0, c->stream>>>(s, ngroups, g);
  else k_f64_apply<3><<<grid, kF64Threads, 0, c->stream>>>(s, ngroups, g);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_f64_apply launch");
  c->launches += 1;
  return GBQ_OK;
}

int gbq_sv64_compare(gbq_ctx* c, const void* state64, const gbq_c64* state32, int nbits, double* out) {
  if (!c) {
    set_error("null context");
    return GBQ_ERR_ARG;
  }
  if (!state64 || !state32 || !out || nbits < 0 || nbits > 36) {
    set_error("gbq_sv64_compare: bad arguments");
    return GBQ_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  int rc = ensure_scratch(c, 64);
  if (rc) return rc;
  unsigned long long* dmax = reinterpret_cast<unsigned long long*>(c->scratch);
  double* sums = reinterpret_cast<double*>(c->scratch) + 1;
  e = cudaMemsetAsync(c->scratch, 0, 3 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  const int64_t n = (int64_t)1 << nbits;
  k_f64_compare<<<f64_grid(c, n), kF64Threads, 0, c->stream>>>(
      reinterpret_cast<const double2*>(state64), reinterpret_cast<const float2*>(state32), n, dmax, sums);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_f64_compare launch");
  c->launches += 1;
  double h[3];
  e = cudaMemcpyAsync(h, c->scratch, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbq_sv64_compare");
  out[0] = h[0];  // the max's bit pattern is already a double
  out[1] = h[1];
  out[2] = h[2];
  return GBQ_OK;
}

}  // extern "C"
