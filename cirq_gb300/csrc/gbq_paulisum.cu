// out = H psi for H = sum_t c_t P_t, P = i^ny X^x Z^zy as in
// PauliString._expectation_from_state_vector_no_validation
// (cirq-core/cirq/ops/pauli_string.py:625-655):
//   out_i = sum_t c_t i^ny_t sign_t(i ^ x_t) psi_{i ^ x_t},  sign(j) = (-1)^{parity(j & zy)}.
//
// Tiled form.  The terms' X masks are covered by a few tile bit-sets B of
// |B| = 13 bits (the 4 lowest bits plus bits chosen greedily so that many
// masks fit).  One pass per bit-set: a CTA gathers the 2^13 amplitudes of
// one tile (fixed values g of the bits outside B) into shared memory and,
// for every term whose X mask lies inside B, adds
//   c_t * (-1)^{parity(x_t & zy_t)} * (-1)^{parity(g & zy_t)} * (-1)^{parity(l & zy_t|B)} * s[l ^ x_t|B]
// to the output amplitude of local index l (parity((i ^ x) & zy) splits
// into a per-term constant, a per-tile part and a per-amplitude part).  The
// first pass writes the output, later passes add to it.  HBM traffic is
// about three state transfers per pass, where the per-amplitude kernel
// reads the state once per distinct X mask.  Terms whose X mask has more
// high bits than a tile can hold go through that kernel (accumulate mode).

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "gbq_internal.cuh"

namespace gbq {

namespace {

constexpr int kPsThreads = 256;
constexpr int kPsTileBits = 13;   // 64 KB of amplitudes per CTA
constexpr int kPsLowFixed = 4;    // bits 0..3 always in the tile: 128-byte runs
constexpr int kPsMaxTerms = 1024; // terms per launch (shared table of 16 KB)
constexpr int kPsChunk = 8;       // amplitudes per thread held in registers

struct PsTerm {
  float cr, ci;     // c_t * i^ny * (-1)^{parity(x & zy)}
  uint32_t xloc;    // X mask in tile coordinates
  uint32_t zloc;    // Z mask in tile coordinates
  uint64_t zg;      // Z mask on the bits outside the tile
};
static_assert(sizeof(PsTerm) == 24, "PsTerm layout");

struct PsArgs {
  const float2* psi;
  float2* out;
  const PsTerm* terms;
  int lt, ng, nt, first;
  uint8_t bpos[16];  // tile bits, ascending
  uint8_t gpos[48];  // other bits, ascending
};

// FULL (tiles of 2^11 amplitudes or more): a thread's 8 amplitudes of a
// chunk are l = lb | k << 8 (k < 8, lb = thread index + chunk offset, bits
// 8..10 of lb clear), so parity(l & z) = parity(lb & z) ^ parity(k & z>>8):
// per term one popcount, and per amplitude the sign bits of bits 8..10 of z
// (precomputed per term, already at bit 31) are folded into the
// coefficient's sign; the shared index is (lb ^ x) ^ (k << 8).
template <bool FULL>
__global__ void __launch_bounds__(kPsThreads, 2) k_paulisum_tile(PsArgs a) {
  extern __shared__ float2 s[];                 // the tile's 2^lt amplitudes
  __shared__ float4 sc[kPsMaxTerms];            // signed coefficient, xloc, zloc
  __shared__ uint4 sz[FULL ? kPsMaxTerms : 1];  // sign bits of zloc bits 8, 9, 10 at bit 31
  __shared__ unsigned long long dep_lo[128], dep_hi[128];  // tile index -> state index bits
  constexpr uint32_t kSign = 0x80000000u;
  const int nl = 1 << a.lt;
  const int t = threadIdx.x;
  if (t < 128) {
    unsigned long long lo = 0, hi = 0;
    for (int j = 0; j < 7 && j < a.lt; ++j)
      if ((t >> j) & 1) lo |= 1ull << a.bpos[j];
    for (int j = 7; j < a.lt; ++j)
      if ((t >> (j - 7)) & 1) hi |= 1ull << a.bpos[j];
    dep_lo[t] = lo;
    dep_hi[t] = hi;
  }
  const int64_t ntiles = (int64_t)1 << a.ng;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    unsigned long long g = 0;
    for (int j = 0; j < a.ng; ++j) g |= (unsigned long long)((tile >> j) & 1) << a.gpos[j];
    __syncthreads();  // the previous tile's readers of s and sc are done; dep tables written
#pragma unroll 8
    for (int l = t; l < nl; l += kPsThreads) s[l] = __ldg(a.psi + (g | dep_lo[l & 127] | dep_hi[l >> 7]));
    for (int k = t; k < a.nt; k += kPsThreads) {
      const PsTerm tm = a.terms[k];
      const uint32_t sg = (uint32_t)(__popcll(g & tm.zg) & 1) << 31;
      sc[k] = make_float4(__uint_as_float(__float_as_uint(tm.cr) ^ sg), __uint_as_float(__float_as_uint(tm.ci) ^ sg),
                          __uint_as_float(tm.xloc), __uint_as_float(tm.zloc));
      if (FULL) sz[k] = make_uint4((tm.zloc << 23) & kSign, (tm.zloc << 22) & kSign, (tm.zloc << 21) & kSign, 0u);
    }
    __syncthreads();
    for (int l0 = t; l0 < nl; l0 += kPsThreads * kPsChunk) {
      // passes after the first add to out: its 8 old values are loaded
      // here, all in flight together, and land while the terms are summed
      // (loaded next to their stores, each would wait a full HBM round trip)
      float2 acc[kPsChunk];
#pragma unroll
      for (int k = 0; k < kPsChunk; ++k) {
        const int l = l0 + k * kPsThreads;
        acc[k] = (!a.first && l < nl) ? a.out[g | dep_lo[l & 127] | dep_hi[l >> 7]] : make_float2(0.f, 0.f);
      }
      if (FULL) {
        const uint32_t lb = (uint32_t)l0;
        for (int q = 0; q < a.nt; ++q) {
          const float4 c = sc[q];
          const uint4 zb = sz[q];
          const uint32_t x = __float_as_uint(c.z), z = __float_as_uint(c.w);
          const uint32_t p0 = (uint32_t)__popc(lb & z) << 31;
          const uint32_t crp = __float_as_uint(c.x) ^ p0, cip = __float_as_uint(c.y) ^ p0;
          const uint32_t base = lb ^ x;
#pragma unroll
          for (int k = 0; k < kPsChunk; ++k) {
            const uint32_t m = ((k & 1) ? zb.x : 0u) ^ ((k & 2) ? zb.y : 0u) ^ ((k & 4) ? zb.z : 0u);
            const float cr = __uint_as_float(crp ^ m), ci = __uint_as_float(cip ^ m);
            const float2 v = s[base ^ ((uint32_t)k << 8)];
            acc[k].x = fmaf(cr, v.x, fmaf(-ci, v.y, acc[k].x));
            acc[k].y = fmaf(cr, v.y, fmaf(ci, v.x, acc[k].y));
          }
        }
      } else {
        for (int q = 0; q < a.nt; ++q) {
          const float4 c = sc[q];
          const uint32_t x = __float_as_uint(c.z), z = __float_as_uint(c.w);
#pragma unroll
          for (int k = 0; k < kPsChunk; ++k) {
            const uint32_t l = (uint32_t)(l0 + k * kPsThreads);
            if (l < (uint32_t)nl) {
              const float2 v = s[l ^ x];
              const uint32_t sg = (uint32_t)(__popc(l & z) & 1) << 31;
              const float cr = __uint_as_float(__float_as_uint(c.x) ^ sg);
              const float ci = __uint_as_float(__float_as_uint(c.y) ^ sg);
              acc[k].x = fmaf(cr, v.x, fmaf(-ci, v.y, acc[k].x));
              acc[k].y = fmaf(cr, v.y, fmaf(ci, v.x, acc[k].y));
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < kPsChunk; ++k) {
        const int l = l0 + k * kPsThreads;
        if (l < nl) a.out[g | dep_lo[l & 127] | dep_hi[l >> 7]] = acc[k];
      }
    }
  }
}

uint32_t compress_bits(uint64_t v, const std::vector<int>& pos) {
  uint32_t r = 0;
  for (size_t j = 0; j < pos.size(); ++j)
    if ((v >> pos[j]) & 1) r |= 1u << j;
  return r;
}

int popc64(uint64_t v) { return __builtin_popcountll(v); }

struct PsPass {
  uint64_t bmask;
  std::vector<int> terms;
};
struct PsCover {
  int nbits;
  std::vector<uint64_t> xs;
  std::vector<PsPass> passes;
  std::vector<int> wide;  // terms for the per-amplitude kernel
};

// Greedy cover of the X masks by tile bit-sets (memoised per mask list).
PsCover make_cover(const gbq_pauli* terms, int nterms, int nbits) {
  PsCover cv;
  cv.nbits = nbits;
  cv.xs.resize(nterms);
  for (int t = 0; t < nterms; ++t) cv.xs[t] = terms[t].x;
  const uint64_t all = nbits >= 64 ? ~0ull : (1ull << nbits) - 1ull;
  if (nbits <= kPsTileBits) {
    PsPass p{all, {}};
    for (int t = 0; t < nterms; ++t) p.terms.push_back(t);
    if (nterms) cv.passes.push_back(std::move(p));
    return cv;
  }
  const uint64_t low = (1ull << kPsLowFixed) - 1ull;
  std::map<uint64_t, std::vector<int>> groups;  // high part of the X mask -> terms
  for (int t = 0; t < nterms; ++t) {
    const uint64_t h = cv.xs[t] & ~low;
    if (popc64(h) > kPsTileBits - kPsLowFixed)
      cv.wide.push_back(t);
    else
      groups[h].push_back(t);
  }
  std::vector<std::pair<uint64_t, std::vector<int>>> rem(groups.begin(), groups.end());
  // larger groups first (first-fit order for very many distinct masks)
  std::stable_sort(rem.begin(), rem.end(), [](const auto& a, const auto& b) { return a.second.size() > b.second.size(); });
  while (!rem.empty()) {
    uint64_t S = low;
    if (rem.size() > 1024) {
      for (const auto& g : rem)
        if (popc64(S | g.first) <= kPsTileBits) S |= g.first;
    } else {
      for (;;) {
        int best = -1;
        double best_score = 0.0;
        size_t best_gain = 0;
        for (size_t i = 0; i < rem.size(); ++i) {
          const uint64_t h = rem[i].first;
          const int nb = popc64(h & ~S);
          if (nb == 0 || popc64(S | h) > kPsTileBits) continue;
          const uint64_t U = S | h;
          size_t gain = 0;
          for (const auto& g : rem)
            if ((g.first & ~U) == 0 && (g.first & ~S) != 0) gain += g.second.size();
          const double score = (double)gain / nb;
          if (score > best_score || (score == best_score && gain > best_gain)) {
            best = (int)i;
            best_score = score;
            best_gain = gain;
          }
        }
        if (best < 0) break;
        S |= rem[best].first;
      }
    }
    for (int b = 0; b < nbits && popc64(S) < kPsTileBits; ++b) S |= 1ull << b;
    PsPass p{S, {}};
    std::vector<std::pair<uint64_t, std::vector<int>>> left;
    for (auto& g : rem) {
      if ((g.first & ~S) == 0)
        p.terms.insert(p.terms.end(), g.second.begin(), g.second.end());
      else
        left.push_back(std::move(g));
    }
    std::sort(p.terms.begin(), p.terms.end());
    cv.passes.push_back(std::move(p));
    rem.swap(left);
  }
  return cv;
}

std::mutex g_cover_mu;
std::vector<PsCover> g_covers;  // most recent last

PsCover cover_for(const gbq_pauli* terms, int nterms, int nbits) {
  std::lock_guard<std::mutex> lk(g_cover_mu);
  for (size_t i = 0; i < g_covers.size(); ++i) {
    const PsCover& c = g_covers[i];
    if (c.nbits != nbits || (int)c.xs.size() != nterms) continue;
    bool same = true;
    for (int t = 0; t < nterms && same; ++t) same = c.xs[t] == terms[t].x;
    if (same) return c;
  }
  PsCover c = make_cover(terms, nterms, nbits);
  if (g_covers.size() >= 8) g_covers.erase(g_covers.begin());
  g_covers.push_back(c);
  return c;
}

}  // namespace

int paulisum_cover_stats(const gbq_pauli* terms, int nterms, int nbits, int* npasses, int* nwide,
                         int* pass_terms, int max_passes) {
  const PsCover cv = cover_for(terms, nterms, nbits);
  *npasses = (int)cv.passes.size();
  *nwide = (int)cv.wide.size();
  for (int q = 0; q < max_passes && q < (int)cv.passes.size(); ++q) pass_terms[q] = (int)cv.passes[q].terms.size();
  return GBQ_OK;
}

int apply_paulisum(Ctx* c, const float2* psi, int nbits, const gbq_pauli* terms, int nterms, float2* out) {
  const PsCover cv = cover_for(terms, nterms, nbits);
  const int lt = std::min(nbits, kPsTileBits);
  size_t ntab = 0;
  for (const PsPass& p : cv.passes) ntab += p.terms.size();
  const size_t tab_bytes = (ntab ? ntab : 1) * sizeof(PsTerm);
  const size_t wide_off = (tab_bytes + 255) & ~(size_t)255;
  const size_t wide_bytes = cv.wide.size() * sizeof(gbq_pauli);
  int rc = ensure_scratch(c, wide_off + wide_bytes + 256);
  if (rc) return rc;
  rc = ensure_host_scratch(c, wide_off + wide_bytes + 256);
  if (rc) return rc;
  char* host = reinterpret_cast<char*>(c->host_scratch);
  PsTerm* tab = reinterpret_cast<PsTerm*>(host);
  size_t k = 0;
  std::vector<std::vector<int>> bpos(cv.passes.size()), gpos(cv.passes.size());
  for (size_t q = 0; q < cv.passes.size(); ++q) {
    const PsPass& p = cv.passes[q];
    for (int b = 0; b < nbits; ++b) ((p.bmask >> b) & 1 ? bpos[q] : gpos[q]).push_back(b);
    for (int t : p.terms) {
      const gbq_pauli& tm = terms[t];
      float cr = (float)tm.coef, ci = 0.f;
      const int ny = tm.ny & 3;
      if (ny == 1) { ci = cr; cr = 0.f; }
      else if (ny == 2) { cr = -cr; }
      else if (ny == 3) { ci = -cr; cr = 0.f; }
      if (popc64(tm.x & tm.zy) & 1) { cr = -cr; ci = -ci; }
      tab[k++] = PsTerm{cr, ci, compress_bits(tm.x, bpos[q]), compress_bits(tm.zy, bpos[q]), tm.zy & ~p.bmask};
    }
  }
  // the per-amplitude kernel reads an amplitude once per run of equal X masks
  std::vector<gbq_pauli> wide;
  for (int t : cv.wide) wide.push_back(terms[t]);
  std::stable_sort(wide.begin(), wide.end(), [](const gbq_pauli& a, const gbq_pauli& b) { return a.x < b.x; });
  if (!wide.empty()) memcpy(host + wide_off, wide.data(), wide_bytes);
  char* dev = reinterpret_cast<char*>(c->scratch);
  cudaError_t e = cudaMemcpyAsync(dev, host, wide_off + wide_bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(pauli tables)");

  // static (18 KB) + dynamic shared memory may pass the 48 KB default: allow
  // the largest tile (per call: the attribute belongs to the current device)
  const size_t smem = (size_t)8 << lt;
  const bool full = lt >= 11;
  auto kern = full ? k_paulisum_tile<true> : k_paulisum_tile<false>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 8 << kPsTileBits);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_paulisum_tile)");
  bool first = true;
  k = 0;
  for (size_t q = 0; q < cv.passes.size(); ++q) {
    const PsPass& p = cv.passes[q];
    PsArgs a{};
    a.psi = psi;
    a.out = out;
    a.lt = lt;
    a.ng = nbits - lt;
    for (int j = 0; j < lt; ++j) a.bpos[j] = (uint8_t)bpos[q][j];
    for (int j = 0; j < a.ng; ++j) a.gpos[j] = (uint8_t)gpos[q][j];
    const int64_t ntiles = (int64_t)1 << a.ng;
    const int grid = (int)std::min<int64_t>(ntiles, (int64_t)2 * c->sm_count);
    for (size_t t0 = 0; t0 < p.terms.size(); t0 += kPsMaxTerms) {
      a.terms = reinterpret_cast<const PsTerm*>(dev) + k + t0;
      a.nt = (int)std::min<size_t>(kPsMaxTerms, p.terms.size() - t0);
      a.first = first ? 1 : 0;
      kern<<<grid, kPsThreads, smem, c->stream>>>(a);
      e = cudaGetLastError();
      if (e != cudaSuccess) return cuda_fail(e, "k_paulisum_tile");
      c->launches += 1;
      first = false;
    }
    k += p.terms.size();
  }
  if (first || !wide.empty())
    return do_apply_paulisum(c, psi, nbits, reinterpret_cast<const gbq_pauli*>(dev + wide_off), (int)wide.size(),
                             out, first ? 0 : 1);
  return GBQ_OK;
}

}  // namespace gbq
