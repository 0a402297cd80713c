// Clifford circuits: one reference run on a stabilizer tableau and Pauli-frame
// sampling of many shots.
//
// Replaces the reference's per-repetition stabilizer simulation:
// StabilizerSampler._run (cirq-core/cirq/sim/clifford/stabilizer_sampler.py:52-70)
// re-runs the whole circuit on a CliffordTableau per repetition, and
// CliffordSimulator.run (cirq-core/cirq/sim/clifford/clifford_simulator.py via
// SimulatorBase._run, cirq-core/cirq/sim/simulator_base.py:225-273) measures a
// copy of the final CH-form state per repetition.
//
// Method (frame simulation, Aaronson-Gottesman tableau for the reference):
// * k_cliff_reference: a single CTA runs the circuit once on a tableau
//   (Aaronson & Gottesman, quant-ph/0406196; the reference's own tableau is
//   cirq-core/cirq/qis/clifford_tableau.py:457-560), taking outcome 0 for
//   every random measurement and ignoring noise.  Rows belong to threads
//   (row i to thread i mod blockDim), so gates need no barrier; a measurement
//   finds its pivot with a block reduction, multiplies rows in parallel, and
//   a deterministic outcome is the sign of a product of commuting
//   stabilizers, reduced as a tree over threads.
// * k_cliff_frames: one thread per 32 shots.  Every shot carries a Pauli
//   frame (X and Z bit per qubit, qubit-major words in HBM) relative to the
//   reference run.  Frames start with random Z parts (Z acts trivially on
//   |0>) and a measured or reset qubit gets a fresh random Z part; a gate
//   maps each frame by its symplectic matrix (signs do not matter for
//   frames); a measurement records reference bit ^ frame X bit; Pauli noise
//   XORs sampled Paulis into the frames; a Pauli conditioned on measurement
//   records is XORed in where the shot's condition differs from the
//   reference's.  The recorded outcomes then follow the circuit's exact
//   distribution.
// Random bits: SplitMix64 (Steele, Lea & Flood, OOPSLA 2014) of a per-launch
// seed and the (op, word) counters; noise draws one 32-bit value per shot
// from that with a 32-bit mixer.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <utility>
#include <string>
#include <vector>

#include "gbq_internal.cuh"

static_assert(sizeof(gbq_cliff_op) == 48, "gbq_cliff_op layout");

namespace gbq {

namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t rnd(uint64_t seed, uint64_t a, uint64_t b) {
  return mix64(seed ^ mix64(a * 0x100000001B3ull + b));
}

// Per-shot 32-bit draws for noise: one 64-bit hash per (op, word), then a
// 32-bit mixer per lane (Wellons' "lowbias32", x ^= x >> 16; x *= ...).
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}
// Pauli noise of one op on the 32 shots of word w: X with probability
// p[0], Y p[1], Z p[2], each shot independently (thresholds on 32-bit
// draws, single-precision probabilities).
// Pauli noise on the 32 shots of one word: each shot independently gets X,
// Y or Z with probabilities p[0], p[1], p[2].  The lanes with an error are
// found by geometric skipping: the gap to the next error is
// floor(ln U / ln(1 - p)) with p = p[0] + p[1] + p[2] and U uniform in
// (0, 1] (ln U taken as log1p(-V), V = 1 - U, so that small p keeps its
// resolution), and each error draws its type.  A word without an error
// costs one hash instead of one per shot.
__device__ __forceinline__ void noise_masks(const gbq_cliff_op& op, int o, int64_t w, uint64_t seed, uint32_t& mx,
                                            uint32_t& mz) {
  const float c1 = op.p[0], c2 = c1 + op.p[1], c3 = c2 + op.p[2];
  mx = 0u;
  mz = 0u;
  if (!(c3 > 0.f)) return;
  const float scale = 4294967296.0f;
  // error type given an error: X below s1, Y below s2, Z above
  const uint32_t s1 = c1 >= c3 ? 0xffffffffu : (uint32_t)((c1 / c3) * scale);
  const uint32_t s2 = c2 >= c3 ? 0xffffffffu : (uint32_t)((c2 / c3) * scale);
  const bool every = c3 >= 1.f;
  const float inv_lq = every ? 0.f : 1.f / log1pf(-c3);  // 1 / ln(1 - p) < 0
  const uint32_t base = (uint32_t)rnd(seed, (uint64_t)o, (uint64_t)w);
  int lane = -1;
  for (int it = 0; it < 32; ++it) {
    int gap = 0;
    if (!every) {
      const uint32_t u = mix32(base ^ (0x9E3779B9u * (uint32_t)(2 * it + 1)));
      const float g = log1pf(-(float)u * 2.3283064365386963e-10f) * inv_lq;  // >= 0, +inf for V = 1
      gap = g < 32.f ? (int)g : 32;
    }
    lane += 1 + gap;
    if (lane >= 32) break;
    const uint32_t v = mix32(base ^ (0x85EBCA6Bu * (uint32_t)(2 * it + 2)));
    const uint32_t bit = 1u << lane;
    if (v < s1) {
      mx |= bit;
    } else if (v < s2) {
      mx |= bit;
      mz |= bit;
    } else {
      mz |= bit;
    }
  }
}

// Frame map of a k-qubit op on one word: output bit o of (x_0..x_{k-1},
// z_0..z_{k-1}) is the XOR of the inputs in lin[o].  K is a compile-time
// width so the words stay in registers.
template <int K>
__device__ __forceinline__ void lin_map(const gbq_cliff_op& op, uint32_t* fx, uint32_t* fz, int64_t stride,
                                        int64_t j) {
  uint32_t in[2 * K], out[2 * K];
  int8_t lin[2 * K];
#pragma unroll
  for (int i = 0; i < 2 * K; ++i) lin[i] = op.lin[i];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    in[i] = fx[op.q[i] * stride + j];
    in[K + i] = fz[op.q[i] * stride + j];
  }
#pragma unroll
  for (int b = 0; b < 2 * K; ++b) {
    uint32_t v = 0;
#pragma unroll
    for (int c = 0; c < 2 * K; ++c) v ^= in[c] & (0u - (uint32_t)((lin[b] >> c) & 1));
    out[b] = v;
  }
#pragma unroll
  for (int i = 0; i < K; ++i) {
    fx[op.q[i] * stride + j] = out[i];
    fz[op.q[i] * stride + j] = out[K + i];
  }
}
__device__ __forceinline__ void apply_lin(const gbq_cliff_op& op, uint32_t* fx, uint32_t* fz, int64_t stride,
                                          int64_t j) {
  if (op.k == 1)
    lin_map<1>(op, fx, fz, stride, j);
  else if (op.k == 2)
    lin_map<2>(op, fx, fz, stride, j);
  else
    lin_map<3>(op, fx, fz, stride, j);
}

constexpr int kRefThreads = 1024;

// Bit j of a row half (words of 64 qubits).
__device__ __forceinline__ uint32_t bit_at(const uint64_t* row, int j) {
  return (uint32_t)((row[j >> 6] >> (j & 63)) & 1ull);
}
__device__ __forceinline__ void put_bit(uint64_t* row, int j, uint32_t v) {
  const uint64_t m = 1ull << (j & 63);
  row[j >> 6] = v ? (row[j >> 6] | m) : (row[j >> 6] & ~m);
}

// Exponent of i in P1 * P2 over one word of qubits (Hermitian Paulis with
// Y for x = z = 1): +1 and -1 contributions counted separately.
__device__ __forceinline__ int gsum(uint64_t x1, uint64_t z1, uint64_t x2, uint64_t z2) {
  const uint64_t y1 = x1 & z1, xo = x1 & ~z1, zo = ~x1 & z1;
  const uint64_t plus = (y1 & z2 & ~x2) | (xo & z2 & x2) | (zo & x2 & ~z2);
  const uint64_t minus = (y1 & x2 & ~z2) | (xo & z2 & ~x2) | (zo & x2 & z2);
  return __popcll(plus) - __popcll(minus);
}

// Tableau in device memory: rows 0..n-1 destabilizers, n..2n-1 stabilizers,
// row 2n and the per-thread accumulators are scratch.
struct Tab {
  uint64_t* x;   // [(2n + 1) * W]
  uint64_t* z;
  int* s;        // sign bits [2n + 1]
  uint64_t* ax;  // accumulators [kRefThreads * W]
  uint64_t* az;
  int* ae;       // accumulator phase exponents (of i, mod 4)
  int n, W;
};

// Applies a k-qubit table op (or a Pauli) to the rows owned by this thread.
__device__ void tab_apply(const Tab& T, const gbq_cliff_op& op, const uint32_t* tab) {
  const int k = op.k;
  for (int i = threadIdx.x; i < 2 * T.n; i += blockDim.x) {
    uint64_t* xr = T.x + (size_t)i * T.W;
    uint64_t* zr = T.z + (size_t)i * T.W;
    uint32_t idx = 0;
    for (int j = 0; j < k; ++j) idx |= (bit_at(xr, op.q[j]) << j) | (bit_at(zr, op.q[j]) << (k + j));
    const uint32_t e = tab[op.tab + idx];
    for (int j = 0; j < k; ++j) {
      put_bit(xr, op.q[j], (e >> j) & 1u);
      put_bit(zr, op.q[j], (e >> (k + j)) & 1u);
    }
    T.s[i] ^= (int)((e >> (2 * k)) & 1u);
  }
}

// Measures qubit q (outcome 0 when random); all threads call it.
__device__ int tab_measure(const Tab& T, int q, int* sh) {
  const int n = T.n, W = T.W;
  // sh[0]: pivot row; sh[1]: outcome
  if (threadIdx.x == 0) sh[0] = 2 * n;
  __syncthreads();
  for (int i = n + threadIdx.x; i < 2 * n; i += blockDim.x)
    if (bit_at(T.x + (size_t)i * W, q)) atomicMin(&sh[0], i);
  __syncthreads();
  const int p = sh[0];
  if (p < 2 * n) {
    const uint64_t* xp = T.x + (size_t)p * W;
    const uint64_t* zp = T.z + (size_t)p * W;
    for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
      if (i == p) continue;
      uint64_t* xi = T.x + (size_t)i * W;
      uint64_t* zi = T.z + (size_t)i * W;
      if (!bit_at(xi, q)) continue;
      int r = 2 * T.s[i] + 2 * T.s[p];
      for (int w = 0; w < W; ++w) r += gsum(xp[w], zp[w], xi[w], zi[w]);
      T.s[i] = (r & 3) != 0;
      for (int w = 0; w < W; ++w) {
        xi[w] ^= xp[w];
        zi[w] ^= zp[w];
      }
    }
    __syncthreads();
    for (int w = threadIdx.x; w < W; w += blockDim.x) {
      T.x[(size_t)(p - n) * W + w] = T.x[(size_t)p * W + w];
      T.z[(size_t)(p - n) * W + w] = T.z[(size_t)p * W + w];
      T.x[(size_t)p * W + w] = 0;
      T.z[(size_t)p * W + w] = (w == (q >> 6)) ? (1ull << (q & 63)) : 0ull;
    }
    if (threadIdx.x == 0) {
      T.s[p - n] = T.s[p];
      T.s[p] = 0;
    }
    __syncthreads();
    return 0;
  }
  // deterministic: the sign of the product of the stabilizers n + i whose
  // destabilizer i has an X on q (they commute: any order)
  const int t = threadIdx.x;
  uint64_t* ax = T.ax + (size_t)t * W;
  uint64_t* az = T.az + (size_t)t * W;
  for (int w = 0; w < W; ++w) ax[w] = az[w] = 0;
  int e = 0;
  for (int i = t; i < n; i += blockDim.x) {
    if (!bit_at(T.x + (size_t)i * W, q)) continue;
    const uint64_t* xr = T.x + (size_t)(n + i) * W;
    const uint64_t* zr = T.z + (size_t)(n + i) * W;
    e += 2 * T.s[n + i];
    for (int w = 0; w < W; ++w) {
      e += gsum(xr[w], zr[w], ax[w], az[w]);
      ax[w] ^= xr[w];
      az[w] ^= zr[w];
    }
    e &= 3;
  }
  T.ae[t] = e & 3;
  __syncthreads();
  for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
    if (t < stride) {
      const uint64_t* bx = T.ax + (size_t)(t + stride) * W;
      const uint64_t* bz = T.az + (size_t)(t + stride) * W;
      int r = T.ae[t] + T.ae[t + stride];
      for (int w = 0; w < W; ++w) {
        r += gsum(bx[w], bz[w], ax[w], az[w]);
        ax[w] ^= bx[w];
        az[w] ^= bz[w];
      }
      T.ae[t] = r & 3;
    }
    __syncthreads();
  }
  const int out = (T.ae[0] & 3) == 2;
  __syncthreads();
  return out;
}

__global__ void __launch_bounds__(kRefThreads) k_cliff_reference(Tab T, const gbq_cliff_op* __restrict__ ops, int nops,
                                                                  const uint32_t* __restrict__ tab,
                                                                  const int32_t* __restrict__ conds,
                                                                  uint8_t* __restrict__ ref) {
  __shared__ int sh[2];
  const int n = T.n, W = T.W;
  for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) {
    for (int w = 0; w < W; ++w) T.x[(size_t)i * W + w] = T.z[(size_t)i * W + w] = 0;
    if (i < n)
      T.x[(size_t)i * W + (i >> 6)] = 1ull << (i & 63);
    else
      T.z[(size_t)i * W + ((i - n) >> 6)] = 1ull << ((i - n) & 63);
    T.s[i] = 0;
  }
  __syncthreads();
  for (int o = 0; o < nops; ++o) {
    const gbq_cliff_op& op = ops[o];
    switch (op.kind) {
      case GBQ_CLIFF_UNITARY:
        tab_apply(T, op, tab);
        break;
      case GBQ_CLIFF_MEASURE: {
        const int m = tab_measure(T, op.q[0], sh);
        if (threadIdx.x == 0) ref[op.rec] = (uint8_t)(m ^ (op.lin[0] & 1));
        __syncthreads();
        break;
      }
      case GBQ_CLIFF_RESET: {
        const int m = tab_measure(T, op.q[0], sh);
        if (m) {
          // X on q: rows with a Z part on q change sign
          for (int i = threadIdx.x; i < 2 * n; i += blockDim.x)
            if (bit_at(T.z + (size_t)i * W, op.q[0])) T.s[i] ^= 1;
        }
        __syncthreads();
        break;
      }
      case GBQ_CLIFF_COND_PAULI: {
        int c = 0;
        for (int j = 0; j < op.cond_count; ++j) c |= ref[conds[op.cond_begin + j]];
        if (c) tab_apply(T, op, tab);
        break;
      }
      default:  // noise: the reference run is noiseless
        break;
    }
  }
}

// One thread per 32 shots; frames qubit-major: X[q * nw + w].
__global__ void k_cliff_frames(const gbq_cliff_op* __restrict__ ops, int nops, const int32_t* __restrict__ conds,
                               const uint8_t* __restrict__ ref, int nq, int64_t nw, uint32_t* __restrict__ fx,
                               uint32_t* __restrict__ fz, uint32_t* __restrict__ rec, uint64_t seed) {
  for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
    for (int q = 0; q < nq; ++q) {
      fx[(int64_t)q * nw + w] = 0u;
      fz[(int64_t)q * nw + w] = (uint32_t)rnd(seed, 0x7fffffffull + (uint64_t)q, (uint64_t)w);
    }
    for (int o = 0; o < nops; ++o) {
      const gbq_cliff_op& op = ops[o];
      switch (op.kind) {
        case GBQ_CLIFF_UNITARY:
          apply_lin(op, fx, fz, nw, w);
          break;
        case GBQ_CLIFF_MEASURE: {
          const int64_t a = (int64_t)op.q[0] * nw + w;
          rec[(int64_t)op.rec * nw + w] = fx[a] ^ (ref[op.rec] ? 0xffffffffu : 0u);
          fz[a] ^= (uint32_t)rnd(seed, (uint64_t)o, (uint64_t)w);
          break;
        }
        case GBQ_CLIFF_RESET: {
          const int64_t a = (int64_t)op.q[0] * nw + w;
          fx[a] = 0u;
          fz[a] = (uint32_t)rnd(seed, (uint64_t)o, (uint64_t)w);
          break;
        }
        case GBQ_CLIFF_NOISE: {
          uint32_t mx, mz;
          noise_masks(op, o, w, seed, mx, mz);
          const int64_t a = (int64_t)op.q[0] * nw + w;
          fx[a] ^= mx;
          fz[a] ^= mz;
          break;
        }
        case GBQ_CLIFF_COND_PAULI: {
          uint32_t c = 0;
          int cref = 0;
          for (int j = 0; j < op.cond_count; ++j) {
            const int r = conds[op.cond_begin + j];
            c |= rec[(int64_t)r * nw + w];
            cref |= ref[r];
          }
          const uint32_t d = c ^ (cref ? 0xffffffffu : 0u);
          // lin[j]: bit 0 = X part, bit 1 = Z part of the Pauli on q[j]
          for (int j = 0; j < op.k; ++j) {
            if (op.lin[j] & 1) fx[(int64_t)op.q[j] * nw + w] ^= d;
            if (op.lin[j] & 2) fz[(int64_t)op.q[j] * nw + w] ^= d;
          }
          break;
        }
        default:
          break;
      }
    }
  }
}

// Frames of a block of `wc` shot-words per CTA for all qubits in shared
// memory (fx[q * wc + j], fz likewise); the ops come in layers of ops on
// disjoint qubits (layer L = ops layer[L] .. layer[L + 1] - 1), and the CTA's
// threads apply every (op, word) pair of a layer at once, with a barrier
// between layers.  Records go to global memory, word index w0 + j.
__device__ __forceinline__ void frame_op(const gbq_cliff_op& op, int o, uint32_t* fx, uint32_t* fz, int wc, int j,
                                         int64_t w, int64_t nw, const int32_t* __restrict__ conds,
                                         const uint8_t* __restrict__ ref, uint32_t* __restrict__ rec,
                                         uint64_t seed) {
  switch (op.kind) {
    case GBQ_CLIFF_UNITARY:
      apply_lin(op, fx, fz, wc, j);
      break;
    case GBQ_CLIFF_MEASURE: {
      const int a = op.q[0] * wc + j;
      rec[(int64_t)op.rec * nw + w] = fx[a] ^ (ref[op.rec] ? 0xffffffffu : 0u);
      fz[a] ^= (uint32_t)rnd(seed, (uint64_t)o, (uint64_t)w);
      break;
    }
    case GBQ_CLIFF_RESET: {
      const int a = op.q[0] * wc + j;
      fx[a] = 0u;
      fz[a] = (uint32_t)rnd(seed, (uint64_t)o, (uint64_t)w);
      break;
    }
    case GBQ_CLIFF_NOISE: {
      uint32_t mx, mz;
      noise_masks(op, o, w, seed, mx, mz);
      const int a = op.q[0] * wc + j;
      fx[a] ^= mx;
      fz[a] ^= mz;
      break;
    }
    case GBQ_CLIFF_COND_PAULI: {
      uint32_t c = 0;
      int cref = 0;
      for (int i = 0; i < op.cond_count; ++i) {
        const int r = conds[op.cond_begin + i];
        c |= rec[(int64_t)r * nw + w];
        cref |= ref[r];
      }
      const uint32_t d = c ^ (cref ? 0xffffffffu : 0u);
      for (int i = 0; i < op.k; ++i) {
        if (op.lin[i] & 1) fx[op.q[i] * wc + j] ^= d;
        if (op.lin[i] & 2) fz[op.q[i] * wc + j] ^= d;
      }
      break;
    }
    default:
      break;
  }
}

__global__ void k_cliff_frames_layers(const gbq_cliff_op* __restrict__ ops, const int32_t* __restrict__ layer,
                                      int nlayers, const int32_t* __restrict__ conds,
                                      const uint8_t* __restrict__ ref, int nq, int64_t nw, int wc,
                                      uint32_t* __restrict__ rec, uint64_t seed) {
  extern __shared__ uint32_t fr[];
  uint32_t* fx = fr;
  uint32_t* fz = fr + (size_t)nq * wc;
  for (int64_t w0 = (int64_t)blockIdx.x * wc; w0 < nw; w0 += (int64_t)gridDim.x * wc) {
    const int nwc = (int)(nw - w0 < (int64_t)wc ? nw - w0 : (int64_t)wc);
    for (int e = threadIdx.x; e < nq * wc; e += blockDim.x) {
      const int q = e / wc, j = e % wc;
      fx[e] = 0u;
      fz[e] = j < nwc ? (uint32_t)rnd(seed, 0x7fffffffull + (uint64_t)q, (uint64_t)(w0 + j)) : 0u;
    }
    __syncthreads();
    for (int L = 0; L < nlayers; ++L) {
      const int first = layer[L], cnt = layer[L + 1] - first;
      for (int e = threadIdx.x; e < cnt * nwc; e += blockDim.x) {
        const int o = first + e / nwc, j = e % nwc;
        frame_op(ops[o], o, fx, fz, wc, j, w0 + j, nw, conds, ref, rec, seed);
      }
      __syncthreads();
    }
  }
}

// Records [nrec][nw] words -> bytes [shots][nrec] (shot-major, as the
// samplers return them), through 32 x 32-word shared tiles.
__global__ void k_cliff_transpose(const uint32_t* __restrict__ rec, int nrec, int64_t nw, int64_t shots,
                                  uint8_t* __restrict__ out) {
  __shared__ uint32_t tile[32][33];
  const int r0 = blockIdx.y * 32;
  for (int64_t w0 = (int64_t)blockIdx.x * 32; w0 < nw; w0 += (int64_t)gridDim.x * 32) {
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
      const int r = r0 + i;
      const int64_t w = w0 + threadIdx.x;
      tile[i][threadIdx.x] = (r < nrec && w < nw) ? rec[(int64_t)r * nw + w] : 0u;
    }
    __syncthreads();
    const int r = r0 + threadIdx.x;
    for (int s = threadIdx.y; s < 1024; s += blockDim.y) {
      const int64_t shot = w0 * 32 + s;
      if (r < nrec && shot < shots) out[shot * nrec + r] = (uint8_t)((tile[threadIdx.x][s >> 5] >> (s & 31)) & 1u);
    }
    __syncthreads();
  }
}

int check_cliff_program(int nq, const gbq_cliff_op* ops, int nops, int ntables, int nconds, int nrec) {
  for (int o = 0; o < nops; ++o) {
    const gbq_cliff_op& op = ops[o];
    const bool tabled = op.kind == GBQ_CLIFF_UNITARY || op.kind == GBQ_CLIFF_COND_PAULI;
    if (op.kind < GBQ_CLIFF_UNITARY || op.kind > GBQ_CLIFF_COND_PAULI) return -1;
    const int k = tabled ? op.k : 1;
    if (k < 1 || k > 3) return -1;
    for (int j = 0; j < k; ++j) {
      if (op.q[j] < 0 || op.q[j] >= nq) return -1;
      for (int i = 0; i < j; ++i)
        if (op.q[i] == op.q[j]) return -1;
    }
    if (tabled && (op.tab < 0 || (int64_t)op.tab + (1 << (2 * k)) > ntables)) return -1;
    if (op.kind == GBQ_CLIFF_MEASURE && (op.rec < 0 || op.rec >= nrec)) return -1;
    if (op.kind == GBQ_CLIFF_COND_PAULI &&
        (op.cond_begin < 0 || op.cond_count < 0 || op.cond_begin + op.cond_count > nconds))
      return -1;
    if (op.kind == GBQ_CLIFF_NOISE &&
        !(op.p[0] >= 0.f && op.p[1] >= 0.f && op.p[2] >= 0.f && op.p[0] + op.p[1] + op.p[2] <= 1.0001f))
      return -1;
  }
  return 0;
}

}  // namespace

int cliff_reference(Ctx* c, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables, int ntables,
                    const int32_t* conds, int nconds, int nrec, uint8_t* ref_out) {
  const int W = (nq + 63) / 64;
  const size_t rows = (size_t)(2 * nq + 1);
  const size_t bytes_ops = (size_t)nops * sizeof(gbq_cliff_op), bytes_tab = (size_t)ntables * 4,
               bytes_cond = (size_t)nconds * 4;
  const size_t bytes_rows = rows * W * 8, bytes_acc = (size_t)kRefThreads * W * 8;
  size_t off = 0;
  auto take = [&](size_t b) {
    const size_t at = off;
    off += (b + 255) / 256 * 256;
    return at;
  };
  const size_t o_ops = take(bytes_ops), o_tab = take(bytes_tab), o_cond = take(bytes_cond), o_x = take(bytes_rows),
               o_z = take(bytes_rows), o_s = take(rows * 4), o_ax = take(bytes_acc), o_az = take(bytes_acc),
               o_ae = take(kRefThreads * 4), o_ref = take((size_t)nrec + 1);
  int rc = ensure_scratch(c, off);
  if (rc) return rc;
  char* base = static_cast<char*>(c->scratch);
  cudaError_t e = cudaSuccess;
  if (bytes_ops) e = cudaMemcpyAsync(base + o_ops, ops, bytes_ops, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && bytes_tab) e = cudaMemcpyAsync(base + o_tab, tables, bytes_tab, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && bytes_cond) e = cudaMemcpyAsync(base + o_cond, conds, bytes_cond, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + o_ref, 0, (size_t)nrec + 1, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_reference upload");
  Tab T;
  T.x = reinterpret_cast<uint64_t*>(base + o_x);
  T.z = reinterpret_cast<uint64_t*>(base + o_z);
  T.s = reinterpret_cast<int*>(base + o_s);
  T.ax = reinterpret_cast<uint64_t*>(base + o_ax);
  T.az = reinterpret_cast<uint64_t*>(base + o_az);
  T.ae = reinterpret_cast<int*>(base + o_ae);
  T.n = nq;
  T.W = W;
  k_cliff_reference<<<1, kRefThreads, 0, c->stream>>>(
      T, reinterpret_cast<const gbq_cliff_op*>(base + o_ops), nops, reinterpret_cast<const uint32_t*>(base + o_tab),
      reinterpret_cast<const int32_t*>(base + o_cond), reinterpret_cast<uint8_t*>(base + o_ref));
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_cliff_reference launch");
  c->launches += 1;
  if (nrec) {
    e = cudaMemcpyAsync(ref_out, base + o_ref, (size_t)nrec, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_reference download");
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_reference");
  return GBQ_OK;
}

// Records to the host: packed words as they are, or (dev_bytes) transposed
// on the device into shot-major bytes first.
static int cliff_output(Ctx* c, char* rec, int nrec, int64_t nw, int64_t shots, char* dev_bytes, void* out,
                        size_t bytes_out) {
  cudaError_t e = cudaSuccess;
  const char* src = rec;
  if (dev_bytes && nrec) {
    const int64_t gx = std::min<int64_t>((nw + 31) / 32, 65535);
    const dim3 grid((unsigned)gx, (unsigned)((nrec + 31) / 32));
    k_cliff_transpose<<<grid, dim3(32, 8), 0, c->stream>>>(reinterpret_cast<const uint32_t*>(rec), nrec, nw, shots,
                                                          reinterpret_cast<uint8_t*>(dev_bytes));
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_cliff_transpose launch");
    c->launches += 1;
    src = dev_bytes;
  }
  if (bytes_out && nrec) {
    e = cudaMemcpyAsync(out, src, bytes_out, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_sample download");
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_sample");
  return GBQ_OK;
}

int cliff_sample(Ctx* c, int nq, const gbq_cliff_op* ops, int nops, const int32_t* conds, int nconds,
                 const uint8_t* ref, int nrec, int64_t shots, uint64_t seed, void* out,
                 const int32_t* layers, int nlayers, int out_bytes) {
  const int64_t nw = (shots + 31) / 32;
  // layered shared-memory path: as many shot-words per CTA as fit
  // (2 * nq words each) in kLayerSmem bytes, up to 32
  constexpr int kLayerSmem = 200 * 1024;
  int wc = 0;
  if (layers && nlayers > 0) {
    wc = 32;
    while (wc > 1 && (size_t)2 * nq * wc * 4 > (size_t)kLayerSmem) wc >>= 1;
    if ((size_t)2 * nq * wc * 4 > (size_t)kLayerSmem) wc = 0;
  }
  const bool layered = wc > 0;
  const size_t bytes_ops = (size_t)nops * sizeof(gbq_cliff_op), bytes_cond = (size_t)nconds * 4;
  const size_t bytes_frames = layered ? 0 : (size_t)nq * nw * 4, bytes_rec = (size_t)nrec * nw * 4;
  const size_t bytes_layers = layered ? (size_t)(nlayers + 1) * 4 : 0;
  const size_t bytes_out = out_bytes ? (size_t)shots * nrec : bytes_rec;
  size_t off = 0;
  auto take = [&](size_t b) {
    const size_t at = off;
    off += (b + 255) / 256 * 256;
    return at;
  };
  const size_t o_ops = take(bytes_ops), o_cond = take(bytes_cond), o_ref = take((size_t)nrec + 1),
               o_x = take(bytes_frames), o_z = take(bytes_frames), o_rec = take(bytes_rec),
               o_lay = take(bytes_layers), o_out = take(out_bytes ? bytes_out : 0);
  int rc = ensure_scratch(c, off);
  if (rc) return rc;
  char* base = static_cast<char*>(c->scratch);
  cudaError_t e = cudaSuccess;
  if (bytes_ops) e = cudaMemcpyAsync(base + o_ops, ops, bytes_ops, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && bytes_cond) e = cudaMemcpyAsync(base + o_cond, conds, bytes_cond, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && nrec) e = cudaMemcpyAsync(base + o_ref, ref, (size_t)nrec, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && layered)
    e = cudaMemcpyAsync(base + o_lay, layers, bytes_layers, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "gbq_cliff_sample upload");
  if (layered) {
    const int smem = 2 * nq * wc * 4;
    static int attr_set = 0;
    if (attr_set < smem) {
      e = cudaFuncSetAttribute(k_cliff_frames_layers, cudaFuncAttributeMaxDynamicSharedMemorySize, kLayerSmem);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_cliff_frames_layers)");
      attr_set = kLayerSmem;
    }
    const int64_t cblocks = (nw + wc - 1) / wc;
    int per_sm = 1;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cliff_frames_layers, 1024, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(cblocks, (int64_t)c->sm_count * std::max(per_sm, 1)));
    std::pair<cudaEvent_t, cudaEvent_t> ev{nullptr, nullptr};
    if (c->pass_timing && cudaEventCreate(&ev.first) == cudaSuccess && cudaEventCreate(&ev.second) == cudaSuccess)
      cudaEventRecord(ev.first, c->stream);
    k_cliff_frames_layers<<<(unsigned)blocks, 1024, smem, c->stream>>>(
        reinterpret_cast<const gbq_cliff_op*>(base + o_ops), reinterpret_cast<const int32_t*>(base + o_lay),
        nlayers, reinterpret_cast<const int32_t*>(base + o_cond), reinterpret_cast<const uint8_t*>(base + o_ref), nq,
        nw, wc, reinterpret_cast<uint32_t*>(base + o_rec), seed);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_cliff_frames_layers launch");
    c->launches += 1;
    if (ev.second) {
      cudaEventRecord(ev.second, c->stream);
      c->timed.push_back(ev);
    }
    return cliff_output(c, base + o_rec, nrec, nw, shots, out_bytes ? base + o_out : nullptr, out, bytes_out);
  }
  const int threads = 256;
  int64_t blocks = (nw + threads - 1) / threads;
  const int64_t cap = (int64_t)c->sm_count * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  k_cliff_frames<<<(unsigned)blocks, threads, 0, c->stream>>>(
      reinterpret_cast<const gbq_cliff_op*>(base + o_ops), nops, reinterpret_cast<const int32_t*>(base + o_cond),
      reinterpret_cast<const uint8_t*>(base + o_ref), nq, nw, reinterpret_cast<uint32_t*>(base + o_x),
      reinterpret_cast<uint32_t*>(base + o_z), reinterpret_cast<uint32_t*>(base + o_rec), seed);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_cliff_frames launch");
  c->launches += 1;
  return cliff_output(c, base + o_rec, nrec, nw, shots, out_bytes ? base + o_out : nullptr, out, bytes_out);
}

int cliff_check(int nq, const gbq_cliff_op* ops, int nops, int ntables, int nconds, int nrec) {
  return check_cliff_program(nq, ops, nops, ntables, nconds, nrec);
}

}  // namespace gbq
