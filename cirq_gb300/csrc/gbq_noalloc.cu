// Pauli-string expectation values for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: services whose device memory is
// entirely owned by a host framework's pool, or latency-critical loops where
// cudaMalloc's implicit device synchronisation is not acceptable.  gbq_sv_expect_paulis
// needs scratch for the term list and per-block partial sums and takes it
// from the context's lazily grown cudaMalloc buffer; the entry point below
// computes the same values with its scratch in a fixed, file-scope device
// array instead, so it allocates nothing at all.
//
// The array (kNoAllocScratchBytes) is created when the library is loaded and
// lives on every GPU that loads it until the process exits.  Its address is
// looked up once per device with cudaGetSymbolAddress (in host code the
// symbol's name is only a host-side stand-in, not a device address).  Every
// call shares the array and it keeps the last call's contents; all of it
// that a call reads is written by that call first.  Calls whose work
// overlaps on the GPU (different streams, or different host threads without
// ordering) race on the array: serialise them.

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "gbq_internal.cuh"

namespace gbq {

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)4 << 20;  // GBQ_NOALLOC_SCRATCH_BYTES
constexpr int kNoAllocCtasPerSm = 4;                      // grid of the partial-sum pass
constexpr int kNoAllocThreads = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};
int g_grid_cap[kMaxDevices] = {};

// Device address of the scratch array on the current device and the widest
// grid of the partial-sum pass there (kNoAllocCtasPerSm per SM), both set up
// once per device.
int scratch_address(void** out, int* grid_cap) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("gbq_sv_expect_paulis_noalloc: device index too large");
    return GBQ_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute(multiprocessors)");
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[dev] = p;
    g_grid_cap[dev] = (sms > 0 ? sms : 1) * kNoAllocCtasPerSm;
  }
  *out = g_scratch_ptr[dev];
  *grid_cap = g_grid_cap[dev];
  return GBQ_OK;
}

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Scratch bytes of a call: [terms][partials: nterms x G x 2 doubles][out: nterms x 2 doubles],
// each part 256-byte aligned.
size_t scratch_need(int nterms, int G) {
  return al256((size_t)nterms * sizeof(gbq_pauli)) + al256((size_t)nterms * G * 2 * sizeof(double)) +
         al256((size_t)nterms * 2 * sizeof(double));
}

// Grid-stride variant of k_expect_partial: a fixed grid of G CTAs, CTA b
// covers amplitudes b*blockDim + i*G*blockDim; partial[(t*G + b)*2 + {0,1}].
__global__ void k_expect_partial_gs(const float2* __restrict__ psi, uint64_t n,
                                    const gbq_pauli* __restrict__ terms, int nterms,
                                    double* __restrict__ partial) {
  __shared__ double red_re[kNoAllocThreads / 32], red_im[kNoAllocThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (int t = 0; t < nterms; ++t) {
    const gbq_pauli tp = terms[t];
    double dre = 0.0, dim = 0.0;
    float sre = 0.f, sim = 0.f;
    int cnt = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
      const uint64_t k = i ^ tp.x;
      const float2 a = psi[i];
      const float2 b = __ldg(psi + k);
      const float sg = (__popcll(k & tp.zy) & 1) ? -1.f : 1.f;
      sre += sg * fmaf(a.x, b.x, a.y * b.y);
      sim += sg * fmaf(a.x, b.y, -a.y * b.x);
      if (++cnt == 32) {
        dre += sre;
        dim += sim;
        sre = sim = 0.f;
        cnt = 0;
      }
    }
    dre += sre;
    dim += sim;
    double wr = dre, wi = dim;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      wr += __shfl_xor_sync(0xffffffffu, wr, o);
      wi += __shfl_xor_sync(0xffffffffu, wi, o);
    }
    if (lane == 0) {
      red_re[warp] = wr;
      red_im[warp] = wi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = 0.0, im = 0.0;
      for (int w = 0; w < kNoAllocThreads / 32; ++w) {
        r += red_re[w];
        im += red_im[w];
      }
      partial[((int64_t)t * gridDim.x + blockIdx.x) * 2] = r;
      partial[((int64_t)t * gridDim.x + blockIdx.x) * 2 + 1] = im;
    }
    __syncthreads();
  }
}

// out[2t + c] = sum_b partial[(t*G + b)*2 + c]
__global__ void k_reduce_terms(const double* __restrict__ partial, int G, double* __restrict__ out) {
  __shared__ double red[2][kNoAllocThreads / 32];
  const int t = blockIdx.x;
  double r = 0.0, im = 0.0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) {
    r += partial[((int64_t)t * G + b) * 2];
    im += partial[((int64_t)t * G + b) * 2 + 1];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    r += __shfl_xor_sync(0xffffffffu, r, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = r;
    red[1][warp] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    out[2 * t] = a;
    out[2 * t + 1] = b;
  }
}

}  // namespace

}  // namespace gbq

using namespace gbq;

extern "C" int gbq_sv_expect_paulis_noalloc(void* stream, const gbq_c64* state, int nbits,
                                            const gbq_pauli* terms, int nterms, double* out) {
  if (!state || nbits < 0 || nbits > 40 || nterms < 0 || (nterms && (!terms || !out))) {
    set_error("gbq_sv_expect_paulis_noalloc: bad arguments");
    return GBQ_ERR_ARG;
  }
  if (nterms == 0) return GBQ_OK;
  const uint64_t mask = nbits >= 64 ? ~0ull : ((1ull << nbits) - 1ull);
  for (int t = 0; t < nterms; ++t)
    if ((terms[t].x & ~mask) || (terms[t].zy & ~mask)) {
      set_error("gbq_sv_expect_paulis_noalloc: pauli term acts on a qubit outside the state");
      return GBQ_ERR_ARG;
    }
  void* base = nullptr;
  int grid_cap = 0;
  int rc = scratch_address(&base, &grid_cap);
  if (rc) return rc;
  const uint64_t n = 1ull << nbits;
  uint64_t g64 = (n + kNoAllocThreads - 1) / kNoAllocThreads;
  const int G = (int)(g64 < (uint64_t)grid_cap ? g64 : (uint64_t)grid_cap);
  if (scratch_need(nterms, G) > kNoAllocScratchBytes) {
    int fit = (int)(kNoAllocScratchBytes / (sizeof(gbq_pauli) + (size_t)(G + 1) * 16));
    while (fit > 0 && scratch_need(fit, G) > kNoAllocScratchBytes) --fit;
    set_error("gbq_sv_expect_paulis_noalloc: " + std::to_string(nterms) +
              " terms need more than the fixed " + std::to_string(kNoAllocScratchBytes >> 20) +
              " MiB scratch (at most " + std::to_string(fit) + " terms fit for this state); split the term list");
    return GBQ_ERR_ARG;
  }
  const size_t b_terms = al256((size_t)nterms * sizeof(gbq_pauli));
  const size_t b_part = al256((size_t)nterms * G * 2 * sizeof(double));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  char* b = reinterpret_cast<char*>(base);
  gbq_pauli* d_terms = reinterpret_cast<gbq_pauli*>(b);
  double* d_part = reinterpret_cast<double*>(b + b_terms);
  double* d_out = reinterpret_cast<double*>(b + b_terms + b_part);
  cudaError_t e = cudaMemcpyAsync(d_terms, terms, (size_t)nterms * sizeof(gbq_pauli),
                                  cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(terms)");
  k_expect_partial_gs<<<G, kNoAllocThreads, 0, st>>>(reinterpret_cast<const float2*>(state), n,
                                                     d_terms, nterms, d_part);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_expect_partial_gs launch");
  k_reduce_terms<<<nterms, kNoAllocThreads, 0, st>>>(d_part, G, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_reduce_terms launch");
  e = cudaMemcpyAsync(out, d_out, (size_t)nterms * 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(out)");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  for (int t = 0; t < nterms; ++t) {
    const double re = out[2 * t], im = out[2 * t + 1];
    const int ny = terms[t].ny & 3;
    double r2 = re, i2 = im;
    if (ny == 1) { r2 = -im; i2 = re; }
    else if (ny == 2) { r2 = -re; i2 = -im; }
    else if (ny == 3) { r2 = im; i2 = -re; }
    out[2 * t] = terms[t].coef * r2;
    out[2 * t + 1] = terms[t].coef * i2;
  }
  return GBQ_OK;
}
