// Reductions, sampling and Pauli-string kernels.
//
// Sampling replaces sample_state_vector (cirq-core/cirq/sim/state_vector.py:170-232)
// and sample_density_matrix (cirq-core/cirq/sim/density_matrix_utils.py:31-95):
// |psi|^2 (or diag rho) is summed per block of 4096 basis states, the block
// sums are prefix-summed in double, and every sample is drawn by one warp:
// binary search of the block CDF, then a warp-shuffle prefix sum over the
// block to locate the basis state (inverse-CDF sampling).
//
// Pauli kernels replace PauliString._expectation_from_state_vector_no_validation
// (cirq-core/cirq/ops/pauli_string.py:625-655): P = i^ny X^x Z^zy is applied
// by index arithmetic (partner index i ^ x, sign parity of (i ^ x) & zy),
// never materialising P psi.

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbq_internal.cuh"

namespace gbq {

namespace {

constexpr int kRedThreads = 256;
constexpr int kBlockBits = 12;  // sampling block = 4096 basis states

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide double sum; result valid in thread 0.
__device__ double block_sum(double v) {
  __shared__ double red[32];
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (warp == 0) {
    r = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    r = warp_sum_d(r);
  }
  return r;
}

__global__ void k_set_basis(float2* s, uint64_t n, uint64_t index) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    s[i] = make_float2(i == index ? 1.f : 0.f, 0.f);
}

// sum |s_i * scale|^2 with every scaled value rounded to float first.
// Pairs of amplitudes as 16-byte loads, four loads in flight per thread;
// float partial sums of at most 64 values go into a double.
__device__ __forceinline__ float norm_pair(float4 v, float scale, int use_scale) {
  if (use_scale) {
    v.x *= scale;
    v.y *= scale;
    v.z *= scale;
    v.w *= scale;
  }
  return fmaf(v.x, v.x, fmaf(v.y, v.y, fmaf(v.z, v.z, v.w * v.w)));
}
// Scalar form for states that do not start on a 16-byte boundary.
__global__ void k_norm2_scalar(const float2* s, uint64_t n, float scale, int use_scale, double* out) {
  double accd = 0.0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float2 v = s[i];
    if (use_scale) {
      v.x *= scale;
      v.y *= scale;
    }
    accd += fmaf(v.x, v.x, v.y * v.y);
  }
  const double r = block_sum(accd);
  if (threadIdx.x == 0) atomicAdd(out, r);
}

__global__ void k_norm2(const float2* s, uint64_t n, float scale, int use_scale, double* out) {
  const float4* s4 = reinterpret_cast<const float4*>(s);
  const uint64_t n4 = n / 2;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double accd = 0.0;
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n4; i += 4 * stride) {
    const float4 a = __ldcs(s4 + i), b = __ldcs(s4 + i + stride), c = __ldcs(s4 + i + 2 * stride),
                 d = __ldcs(s4 + i + 3 * stride);
    const float acc = norm_pair(a, scale, use_scale) + norm_pair(b, scale, use_scale) +
                      norm_pair(c, scale, use_scale) + norm_pair(d, scale, use_scale);
    accd += acc;
  }
  for (; i < n4; i += stride) accd += norm_pair(__ldcs(s4 + i), scale, use_scale);
  if (n & 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      float2 v = s[n - 1];
      if (use_scale) {
        v.x *= scale;
        v.y *= scale;
      }
      accd += fmaf(v.x, v.x, v.y * v.y);
    }
  }
  const double r = block_sum(accd);
  if (threadIdx.x == 0) atomicAdd(out, r);
}

__global__ void k_project(float2* s, uint64_t n, uint64_t mask, uint64_t value, float scale) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float2 v = s[i];
    const float f = ((i & mask) == value) ? scale : 0.f;
    s[i] = make_float2(v.x * f, v.y * f);
  }
}

__global__ void k_scale_scalar(float2* s, uint64_t n, float scale) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float2 v = s[i];
    s[i] = make_float2(v.x * scale, v.y * scale);
  }
}

__global__ void k_scale(float2* s, uint64_t n, float scale) {
  float4* s4 = reinterpret_cast<float4*>(s);
  const uint64_t n4 = n / 2;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (; i + stride < n4; i += 2 * stride) {
    float4 a = __ldcs(s4 + i), b = __ldcs(s4 + i + stride);
    a.x *= scale; a.y *= scale; a.z *= scale; a.w *= scale;
    b.x *= scale; b.y *= scale; b.z *= scale; b.w *= scale;
    __stcs(s4 + i, a);
    __stcs(s4 + i + stride, b);
  }
  for (; i < n4; i += stride) {
    float4 a = __ldcs(s4 + i);
    a.x *= scale; a.y *= scale; a.z *= scale; a.w *= scale;
    __stcs(s4 + i, a);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const float2 v = s[n - 1];
    s[n - 1] = make_float2(v.x * scale, v.y * scale);
  }
}

template <bool DM>
__device__ __forceinline__ float prob_at(const float2* s, uint64_t i, int nq) {
  if (DM) {
    const float2 v = s[i * ((1ull << nq) + 1ull)];
    return v.x;
  } else {
    const float2 v = s[i];
    return fmaf(v.x, v.x, v.y * v.y);
  }
}

template <bool DM>
__global__ void k_probs(const float2* s, int nq, float* out) {
  const uint64_t n = 1ull << nq;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = prob_at<DM>(s, i, nq);
}

// One CTA per sampling block: block_sums[b] = sum of probabilities in block b.
template <bool DM>
__global__ void k_block_probs(const float2* s, int nq, int bbits, double* block_sums) {
  const uint64_t b0 = (uint64_t)blockIdx.x << bbits;
  const uint32_t bn = 1u << bbits;
  float acc = 0.f;
  for (uint32_t j = threadIdx.x; j < bn; j += blockDim.x) acc += prob_at<DM>(s, b0 + j, nq);
  const double r = block_sum((double)acc);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = r;
}

// In-place inclusive prefix sum of n doubles by one CTA of 1024 threads.
__global__ void k_scan_inclusive(double* a, int64_t n) {
  __shared__ double tot[1024];
  const int t = threadIdx.x;
  const int64_t per = (n + 1023) / 1024;
  const int64_t lo = t * per, hi = lo + per < n ? lo + per : n;
  double s = 0.0;
  for (int64_t i = lo; i < hi; ++i) s += a[i];
  tot[t] = s;
  __syncthreads();
  if (t == 0) {
    double run = 0.0;
    for (int i = 0; i < 1024; ++i) {
      const double v = tot[i];
      tot[i] = run;
      run += v;
    }
  }
  __syncthreads();
  double run = tot[t];
  for (int64_t i = lo; i < hi; ++i) {
    run += a[i];
    a[i] = run;
  }
}

// One warp per sample.
template <bool DM>
__global__ void k_sample(const float2* s, int nq, int bbits, const double* cdf, int64_t nblocks,
                         const double* u, int64_t R, uint64_t* out) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  const double total = cdf[nblocks - 1];
  double target = u[r] * total;
  // first block with cdf > target
  int64_t lo = 0, hi = nblocks - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (cdf[mid] > target) hi = mid;
    else lo = mid + 1;
  }
  const int64_t b = lo;
  double resid = target - (b > 0 ? cdf[b - 1] : 0.0);
  const uint32_t bn = 1u << bbits;
  const uint32_t per = bn >= 32 ? bn / 32 : 1;
  const uint64_t base = ((uint64_t)b << bbits) + (uint64_t)lane * per;
  const bool has = (uint32_t)lane * per < bn;
  float part = 0.f;
  if (has)
    for (uint32_t j = 0; j < per; ++j) part += prob_at<DM>(s, base + j, nq);
  // inclusive warp scan in double
  double incl = (double)part;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const double excl = incl - (double)part;
  const unsigned hit = __ballot_sync(0xffffffffu, has && incl > resid);
  int owner;
  if (hit) owner = __ffs(hit) - 1;
  else {
    // rounding put the target past the block's last mass: take the last
    // lane holding nonzero probability
    const unsigned nz = __ballot_sync(0xffffffffu, has && part > 0.f);
    owner = nz ? 31 - __clz(nz) : 0;
    resid = 1e300;
  }
  if (lane == owner) {
    double run = excl;
    uint64_t pick = base + per - 1;
    uint64_t last_nz = base;
    for (uint32_t j = 0; j < per; ++j) {
      const float p = prob_at<DM>(s, base + j, nq);
      if (p > 0.f) last_nz = base + j;
      run += (double)p;
      if (run > resid) {
        pick = base + j;
        break;
      }
      if (j + 1 == per) pick = last_nz;
    }
    out[r] = pick;
  }
}

// ---- Pauli strings -------------------------------------------------------------
// partial[(t * nchunks + chunk) * 2 + {0,1}] = sum over the chunk of
// conj(psi_i) * sign * psi_{i^x}   (before coef * i^ny).
__global__ void k_expect_partial(const float2* psi, int nbits, const gbq_pauli* terms, int nterms,
                                 int cbits, double* partial) {
  __shared__ double red_re[kRedThreads / 32], red_im[kRedThreads / 32];
  const uint64_t c0 = (uint64_t)blockIdx.x << cbits;
  const uint32_t cn = 1u << cbits;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nchunks = gridDim.x;
  for (int t = 0; t < nterms; ++t) {
    const gbq_pauli tp = terms[t];
    float sre = 0.f, sim = 0.f;
    for (uint32_t j = threadIdx.x; j < cn; j += kRedThreads) {
      const uint64_t i = c0 + j;
      const uint64_t k = i ^ tp.x;
      const float2 a = psi[i];
      const float2 b = __ldg(psi + k);
      const float sg = (__popcll(k & tp.zy) & 1) ? -1.f : 1.f;
      sre += sg * fmaf(a.x, b.x, a.y * b.y);
      sim += sg * fmaf(a.x, b.y, -a.y * b.x);
    }
    sre = warp_sum_f(sre);
    sim = warp_sum_f(sim);
    if (lane == 0) {
      red_re[warp] = sre;
      red_im[warp] = sim;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0, i = 0.0;
      for (int w = 0; w < kRedThreads / 32; ++w) {
        r += red_re[w];
        i += red_im[w];
      }
      partial[((int64_t)t * nchunks + blockIdx.x) * 2] = r;
      partial[((int64_t)t * nchunks + blockIdx.x) * 2 + 1] = i;
    }
    __syncthreads();
  }
  (void)nbits;
}

// Tr(P rho) = sum_i phase(k) rho[k, i], k = i ^ x, for rho of nq qubits.
__global__ void k_dm_expect_partial(const float2* rho, int nq, const gbq_pauli* terms, int nterms,
                                    double* partial) {
  const uint64_t n = 1ull << nq;
  const int64_t nchunks = gridDim.x;
  for (int t = 0; t < nterms; ++t) {
    const gbq_pauli tp = terms[t];
    float sre = 0.f, sim = 0.f;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t k = i ^ tp.x;
      const float2 v = rho[k * n + i];
      const float sg = (__popcll(k & tp.zy) & 1) ? -1.f : 1.f;
      sre += sg * v.x;
      sim += sg * v.y;
    }
    const double r = block_sum((double)sre);
    const double im = block_sum((double)sim);
    if (threadIdx.x == 0) {
      partial[((int64_t)t * nchunks + blockIdx.x) * 2] = r;
      partial[((int64_t)t * nchunks + blockIdx.x) * 2 + 1] = im;
    }
  }
}

// out_i (+)= sum_t c_t * sign_t(i ^ x_t) * psi_{i ^ x_t},  c_t = coef_t * i^ny_t
// (terms sorted by x_t by the caller; accumulate: add to out)
__global__ void k_apply_paulisum(const float2* psi, int nbits, const gbq_pauli* terms, int nterms,
                                 float2* out, int accumulate) {
  extern __shared__ float4 sterm[];  // per term: (x lo/hi bits packed), zy, c.re, c.im
  for (int t = threadIdx.x; t < nterms; t += blockDim.x) {
    const gbq_pauli tp = terms[t];
    float cr = (float)tp.coef, ci = 0.f;
    const int ny = tp.ny & 3;
    if (ny == 1) { ci = cr; cr = 0.f; }
    else if (ny == 2) { cr = -cr; }
    else if (ny == 3) { ci = -cr; cr = 0.f; }
    sterm[2 * t] = make_float4(__uint_as_float((uint32_t)tp.x), __uint_as_float((uint32_t)(tp.x >> 32)),
                               __uint_as_float((uint32_t)tp.zy), __uint_as_float((uint32_t)(tp.zy >> 32)));
    sterm[2 * t + 1] = make_float4(cr, ci, 0.f, 0.f);
  }
  __syncthreads();
  const uint64_t n = 1ull << nbits;
  // terms come sorted by X mask: the coefficients of a run of equal masks
  // are summed (with their signs at this index) and the amplitude is read
  // once per run
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    float2 cf = make_float2(0.f, 0.f);
    uint64_t xcur = 0;
    for (int t = 0; t < nterms; ++t) {
      const float4 a = sterm[2 * t], c = sterm[2 * t + 1];
      const uint64_t x = (uint64_t)__float_as_uint(a.x) | ((uint64_t)__float_as_uint(a.y) << 32);
      const uint64_t zy = (uint64_t)__float_as_uint(a.z) | ((uint64_t)__float_as_uint(a.w) << 32);
      if (t > 0 && x != xcur) {
        const float2 v = __ldg(psi + (i ^ xcur));
        acc.x = fmaf(cf.x, v.x, fmaf(-cf.y, v.y, acc.x));
        acc.y = fmaf(cf.x, v.y, fmaf(cf.y, v.x, acc.y));
        cf = make_float2(0.f, 0.f);
      }
      xcur = x;
      const float sg = (__popcll((i ^ x) & zy) & 1) ? -1.f : 1.f;
      cf.x = fmaf(sg, c.x, cf.x);
      cf.y = fmaf(sg, c.y, cf.y);
    }
    if (nterms > 0) {
      const float2 v = __ldg(psi + (i ^ xcur));
      acc.x = fmaf(cf.x, v.x, fmaf(-cf.y, v.y, acc.x));
      acc.y = fmaf(cf.x, v.y, fmaf(cf.y, v.x, acc.y));
    }
    if (accumulate) {
      const float2 o = out[i];
      acc = make_float2(o.x + acc.x, o.y + acc.y);
    }
    out[i] = acc;
  }
}

__global__ void k_inner(const float2* a, const float2* b, uint64_t n, double* out) {
  float sr = 0.f, si = 0.f;
  double dr = 0.0, di = 0.0;
  int cnt = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const float2 x = a[i], y = b[i];
    sr = fmaf(x.x, y.x, fmaf(x.y, y.y, sr));
    si = fmaf(x.x, y.y, fmaf(-x.y, y.x, si));
    if (++cnt == 64) {
      dr += sr;
      di += si;
      sr = si = 0.f;
      cnt = 0;
    }
  }
  dr += sr;
  di += si;
  const double r = block_sum(dr);
  const double im = block_sum(di);
  if (threadIdx.x == 0) {
    atomicAdd(out, r);
    atomicAdd(out + 1, im);
  }
}

// out[s] = sum_t partial[s * ntiles + t]
__global__ void k_reduce_slots(const double* partial, int64_t ntiles, double* out, int stride2) {
  const int s = blockIdx.x;
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < ntiles; t += blockDim.x)
    acc += partial[(s * ntiles + t) * stride2];
  const double r = block_sum(acc);
  if (threadIdx.x == 0) out[s * stride2] = r;
}

int grid_for(Ctx* c, uint64_t n, int threads) {
  uint64_t g = (n + threads - 1) / threads;
  const uint64_t cap = (uint64_t)c->sm_count * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int check_launch(Ctx* c, const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  c->launches += 1;
  return GBQ_OK;
}

}  // namespace

// ---- entry points (called from gbq_abi.cu) -------------------------------------
int do_set_basis(Ctx* c, float2* s, int nbits, uint64_t index) {
  const uint64_t n = 1ull << nbits;
  k_set_basis<<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, n, index);
  return check_launch(c, "k_set_basis");
}

int do_norm2(Ctx* c, const float2* s, int nbits, float scale, int use_scale, double* d_out) {
  const uint64_t n = 1ull << nbits;
  cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "memset");
  if (reinterpret_cast<uintptr_t>(s) & 15)
    k_norm2_scalar<<<grid_for(c, n, kRedThreads), kRedThreads, 0, c->stream>>>(s, n, scale, use_scale, d_out);
  else
    k_norm2<<<grid_for(c, n, kRedThreads), kRedThreads, 0, c->stream>>>(s, n, scale, use_scale, d_out);
  return check_launch(c, "k_norm2");
}

int do_scale(Ctx* c, float2* s, int nbits, float scale) {
  const uint64_t n = 1ull << nbits;
  if (reinterpret_cast<uintptr_t>(s) & 15)
    k_scale_scalar<<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, n, scale);
  else
    k_scale<<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, n, scale);
  return check_launch(c, "k_scale");
}

int do_project(Ctx* c, float2* s, int nbits, uint64_t mask, uint64_t value, float scale) {
  const uint64_t n = 1ull << nbits;
  k_project<<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, n, mask, value, scale);
  return check_launch(c, "k_project");
}

int do_probs(Ctx* c, const float2* s, int nq, int dm, float* out) {
  const uint64_t n = 1ull << nq;
  if (dm) k_probs<true><<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, nq, out);
  else k_probs<false><<<grid_for(c, n, 256), 256, 0, c->stream>>>(s, nq, out);
  return check_launch(c, "k_probs");
}

// scratch layout: [block cdf: nblocks doubles][uniforms: R doubles][out: R uint64]
int do_sample(Ctx* c, const float2* s, int nq, int dm, const double* d_u, int64_t R,
              uint64_t* d_out, double* d_cdf) {
  const int bbits = nq < kBlockBits ? nq : kBlockBits;
  const int64_t nblocks = (int64_t)1 << (nq - bbits);
  if (dm) k_block_probs<true><<<(unsigned)nblocks, 256, 0, c->stream>>>(s, nq, bbits, d_cdf);
  else k_block_probs<false><<<(unsigned)nblocks, 256, 0, c->stream>>>(s, nq, bbits, d_cdf);
  int rc = check_launch(c, "k_block_probs");
  if (rc) return rc;
  k_scan_inclusive<<<1, 1024, 0, c->stream>>>(d_cdf, nblocks);
  rc = check_launch(c, "k_scan_inclusive");
  if (rc) return rc;
  const int64_t threads = R * 32;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  if (dm) k_sample<true><<<grid, 256, 0, c->stream>>>(s, nq, bbits, d_cdf, nblocks, d_u, R, d_out);
  else k_sample<false><<<grid, 256, 0, c->stream>>>(s, nq, bbits, d_cdf, nblocks, d_u, R, d_out);
  return check_launch(c, "k_sample");
}

int expect_chunk_bits(int nbits) { return nbits < 12 ? nbits : 12; }

int do_expect(Ctx* c, const float2* s, int nbits, const gbq_pauli* d_terms, int nterms,
              double* d_partial, double* d_out) {
  const int cbits = expect_chunk_bits(nbits);
  const int64_t nchunks = (int64_t)1 << (nbits - cbits);
  k_expect_partial<<<(unsigned)nchunks, kRedThreads, 0, c->stream>>>(s, nbits, d_terms, nterms,
                                                                      cbits, d_partial);
  int rc = check_launch(c, "k_expect_partial");
  if (rc) return rc;
  // reduce re and im separately (stride 2)
  k_reduce_slots<<<nterms, 256, 0, c->stream>>>(d_partial, nchunks, d_out, 2);
  rc = check_launch(c, "k_reduce_slots");
  if (rc) return rc;
  k_reduce_slots<<<nterms, 256, 0, c->stream>>>(d_partial + 1, nchunks, d_out + 1, 2);
  return check_launch(c, "k_reduce_slots");
}

int dm_expect_chunks(Ctx* c, int nq) { return grid_for(c, 1ull << nq, 256); }

int do_dm_expect(Ctx* c, const float2* rho, int nq, const gbq_pauli* d_terms, int nterms,
                 double* d_partial, double* d_out) {
  const int chunks = dm_expect_chunks(c, nq);
  k_dm_expect_partial<<<chunks, 256, 0, c->stream>>>(rho, nq, d_terms, nterms, d_partial);
  int rc = check_launch(c, "k_dm_expect_partial");
  if (rc) return rc;
  k_reduce_slots<<<nterms, 256, 0, c->stream>>>(d_partial, chunks, d_out, 2);
  rc = check_launch(c, "k_reduce_slots");
  if (rc) return rc;
  k_reduce_slots<<<nterms, 256, 0, c->stream>>>(d_partial + 1, chunks, d_out + 1, 2);
  return check_launch(c, "k_reduce_slots");
}

int do_apply_paulisum(Ctx* c, const float2* psi, int nbits, const gbq_pauli* d_terms, int nterms,
                      float2* out, int accumulate) {
  const uint64_t n = 1ull << nbits;
  const size_t smem = (size_t)nterms * 2 * sizeof(float4);
  if (smem > 200 * 1024) {
    set_error("gbq_sv_apply_paulisum: too many terms (max 6400)");
    return GBQ_ERR_ARG;
  }
  static size_t attr = 48 * 1024;
  if (smem > attr) {
    cudaError_t e = cudaFuncSetAttribute(k_apply_paulisum, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_apply_paulisum)");
    attr = smem;
  }
  k_apply_paulisum<<<grid_for(c, n, 256), 256, smem, c->stream>>>(psi, nbits, d_terms, nterms, out, accumulate);
  return check_launch(c, "k_apply_paulisum");
}

int do_inner(Ctx* c, const float2* a, const float2* b, int nbits, double* d_out) {
  const uint64_t n = 1ull << nbits;
  cudaError_t e = cudaMemsetAsync(d_out, 0, 2 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "memset");
  k_inner<<<grid_for(c, n, kRedThreads), kRedThreads, 0, c->stream>>>(a, b, n, d_out);
  return check_launch(c, "k_inner");
}

int do_reduce_slots(Ctx* c, const double* partial, int nslots, int64_t ntiles, double* out) {
  k_reduce_slots<<<nslots, 256, 0, c->stream>>>(partial, ntiles, out, 1);
  return check_launch(c, "k_reduce_slots");
}

}  // namespace gbq
