// Pass-specialised tile kernels, compiled at run time with NVRTC.
//
// The tile-pass interpreter (k_tile_ws, gbq_tile.cuh) decodes every op of a
// pass for every tile: op kind, register-position mask, selector bits, table
// columns and matrix offsets are read from the kernel parameters and turned
// into shared-memory indices and matrix pointers at run time.  Here one
// kernel is generated per pass structure instead: the same warp-specialised
// producer/consumer kernel, whose consumer body is straight-line code with
// every bit position, shared-memory offset and matrix-pool offset folded
// into constants.  The arithmetic of each op is the interpreter's (same
// packed FMA order), so results are bit-identical to the interpreter's.
//
// Only the pool offsets of the matrices are baked in, not their values: a
// kernel serves every parameter point of a structure (sweeps replay it with
// new pools).  Kernels are cached by the pass's converted op records.
//
// NVRTC is loaded with dlopen on first use, so the library has no link-time
// dependency on it; without it the interpreter runs.
//
// Replaces, like the interpreter, the per-operation numpy passes of the
// reference: linalg.targeted_left_multiply / apply_matrix_to_slices
// (cirq-core/cirq/linalg/transformations.py:105-172, 310-380) reached from
// protocols.apply_unitary (cirq-core/cirq/protocols/apply_unitary_protocol.py:306-418).

#include <dlfcn.h>
#include <nvrtc.h>

#include <atomic>
#include <chrono>
#include <cstdlib>
#include <condition_variable>
#include <deque>
#include <memory>
#include <cstring>
#include <mutex>
#include <sstream>
#include <thread>
#include <unordered_map>

#include "gbq_internal.cuh"

namespace gbq {

// ---- kernel skeleton ------------------------------------------------------------
// The producer side and the tile loop are those of k_tile_ws<12> (three
// 32 KB buffers, two producer warps with 8-byte cp.async loads and 16-byte
// streaming stores, eight consumer warps, bounded mbarrier waits with a
// consumer-wide vote).  @SETUP@ and @BODY@ are replaced by the generated
// per-thread setup and per-tile op code.
static const char kJitSkeleton[] = R"GBQJIT(
typedef unsigned int u32;
typedef unsigned long long u64;
typedef long long i64;
typedef unsigned short u16;

struct JitArgs {
  float2* psi;
  float2* lam;
  const float2* mats;
  double* partial;
  int* abort;
  i64 ntiles;
  int nbits;
  int L;
  u64 gw[13];
  signed char nt[64];
};

#define LT @LT@
#define DUAL @DUAL@
#define NSL (1 << (LT - 8))

__device__ __forceinline__ u32 phys_dev(u32 i) {
  u32 s = (__popc(i & @SWZ0@u) & 1) | ((__popc(i & @SWZ1@u) & 1) << 1) |
          ((__popc(i & @SWZ2@u) & 1) << 2) | ((__popc(i & @SWZ3@u) & 1) << 3);
  return i ^ s;
}
__device__ __forceinline__ u32 su32(const void* p) { return (u32)__cvta_generic_to_shared(p); }
__device__ __forceinline__ u64 lin_off(const JitArgs& a, u32 i) {
  u64 r = 0;
#pragma unroll
  for (int b = 0; b < LT; ++b)
    if ((i >> b) & 1u) r ^= a.gw[b];
  return r;
}
__device__ __forceinline__ u64 tile_base(const JitArgs& a, i64 tile) {
  u64 g = 0;
  const int nnt = a.nbits - a.L;
  for (int j = 0; j < nnt; ++j) g |= (u64)((tile >> j) & 1) << a.nt[j];
  return g;
}
__device__ __forceinline__ u64 tile_base_fast(const u64* tab, i64 tile) {
  return tab[tile & 255] | tab[256 + ((tile >> 8) & 255)] | tab[512 + ((tile >> 16) & 255)];
}
__device__ __forceinline__ void cp_async8(float2* sdst, const float2* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(su32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ bool ws_wait(u64* bar, u32 parity, volatile int* abort) {
  const u32 a = su32(bar);
  for (long it = 0; it < (1L << 26); ++it) {
    u32 done;
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
__device__ __forceinline__ bool consumers_any(bool v) {
  u32 r;
  asm volatile(
      "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, 1, 256, p;\n"
      "selp.u32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"((u32)v)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void ops_barrier() { asm volatile("bar.sync 1, 256;\n" ::: "memory"); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Per-thread probe accumulator over the CTA's tiles: a float-float pair
// (hi, lo) updated by Knuth's TwoSum, with the rounding errors summed in lo
// (Neumaier's compensated summation).  About 48 significant bits, like the
// double it replaces, in FP32 instructions: FP64 issues at a small fraction
// of the FP32 rate on this part, and a double add per probe per tile kept
// the FP64 pipe half busy.
struct ffacc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float b) {
    const float s = hi + b;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (b - bb);
    hi = s;
  }
};
// A probe's per-thread total over the CTA's tiles into its accumulator
// (once per CTA, in double).
__device__ __forceinline__ void probe_flush(const ffacc& f, int pidx, double* red) {
  double v = warp_sum((double)f.hi + (double)f.lo);
  if ((threadIdx.x & 31) == 0) atomicAdd(red + pidx, v);
}
__host__ __device__ constexpr int popc_c(int x) { return x ? (x & 1) + popc_c(x >> 1) : 0; }
__host__ __device__ constexpr int dep_c(int x, int mask) {
  int r = 0, i = 0;
  for (int b = 0; b < 8; ++b)
    if ((mask >> b) & 1) {
      if ((x >> i) & 1) r |= 1 << b;
      ++i;
    }
  return r;
}
template <bool SH>
__device__ __forceinline__ float4 mload(const float2* mp, int e) {
  return SH ? *reinterpret_cast<const float4*>(mp + e) : __ldg(reinterpret_cast<const float4*>(mp + e));
}
// Dense op on the register positions in MASK (width <= 2) of v (and, in
// two-state passes, of w with the same matrix): packed form
// acc += m * (a.x, a.x) + (i m) * (a.y, a.y), the interpreter's order.
template <int MASK, bool SH>
__device__ __forceinline__ void rdense(float2 (&v)[NSL], float2 (&w)[NSL], const float2* __restrict__ mp) {
  constexpr int K = popc_c(MASK);
  constexpr int D = 1 << K;
  constexpr int NG = NSL / D;
  constexpr int REST = (NSL - 1) & ~MASK;
  float2 m[D * D], im[D * D];
#pragma unroll
  for (int e = 0; e < D * D; e += 2) {
    const float4 mm = mload<SH>(mp, e);
    m[e] = make_float2(mm.x, mm.y);
    m[e + 1] = make_float2(mm.z, mm.w);
    im[e] = make_float2(-mm.y, mm.x);
    im[e + 1] = make_float2(-mm.w, mm.z);
  }
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    const int s0 = dep_c(g, REST);
    float2 ax[D], ay[D], bx[DUAL ? D : 1], by[DUAL ? D : 1];
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const float2 a = v[s0 | dep_c(j, MASK)];
      ax[j] = make_float2(a.x, a.x);
      ay[j] = make_float2(a.y, a.y);
      if (DUAL) {
        const float2 b = w[s0 | dep_c(j, MASK)];
        bx[j % (DUAL ? D : 1)] = make_float2(b.x, b.x);
        by[j % (DUAL ? D : 1)] = make_float2(b.y, b.y);
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
      v[s0 | dep_c(r, MASK)] = acc;
      if (DUAL) {
        float2 accb = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) {
          accb = __ffma2_rn(m[r * D + c], bx[c % (DUAL ? D : 1)], accb);
          accb = __ffma2_rn(im[r * D + c], by[c % (DUAL ? D : 1)], accb);
        }
        w[s0 | dep_c(r, MASK)] = accb;
      }
    }
  }
}
// Dense probe on the register positions in MASK: the thread's part of
// Re <w | M v> (the interpreter's scalar order; width 3 reads M row by row).
template <int MASK, bool SH>
__device__ __forceinline__ float rprobe(const float2 (&v)[NSL], const float2 (&w)[NSL], const float2* __restrict__ mp) {
  constexpr int K = popc_c(MASK);
  constexpr int D = 1 << K;
  constexpr int NG = NSL / D;
  constexpr int REST = (NSL - 1) & ~MASK;
  float part = 0.f;
  if (K <= 2) {
    float2 m[D * D];
#pragma unroll
    for (int e = 0; e < D * D; e += 2) {
      const float4 mm = mload<SH>(mp, e);
      m[e] = make_float2(mm.x, mm.y);
      m[e + 1] = make_float2(mm.z, mm.w);
    }
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int s0 = dep_c(g, REST);
      float2 in[D];
#pragma unroll
      for (int j = 0; j < D; ++j) in[j] = v[s0 | dep_c(j, MASK)];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; ++c) cfma(acc, m[r * D + c], in[c]);
        const float2 l = w[s0 | dep_c(r, MASK)];
        part = fmaf(l.x, acc.x, fmaf(l.y, acc.y, part));
      }
    }
  } else {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      const int s0 = dep_c(g, REST);
      float2 in[D];
#pragma unroll
      for (int j = 0; j < D; ++j) in[j] = v[s0 | dep_c(j, MASK)];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int c = 0; c < D; c += 2) {
          const float4 mm = mload<SH>(mp, r * D + c);
          cfma(acc, make_float2(mm.x, mm.y), in[c]);
          cfma(acc, make_float2(mm.z, mm.w), in[c + 1]);
        }
        const float2 l = w[s0 | dep_c(r, MASK)];
        part = fmaf(l.x, acc.x, fmaf(l.y, acc.y, part));
      }
    }
  }
  return part;
}

extern "C" __global__ void __launch_bounds__(320, 2) k_jit(const __grid_constant__ JitArgs a) {
  constexpr int TS = 1 << LT;
  constexpr int S = 3;
  constexpr int NH = TS >> 5;
  constexpr int NST = DUAL ? 2 : 1;  // states per tile buffer
  extern __shared__ float4 smraw[];
  __shared__ u64 ttab[768];
  __shared__ u64 hoff[NH];
  __shared__ u16 hphys[NH];
  __shared__ __align__(8) u64 full[S], empty[S];
  __shared__ int abort_flag;
  __shared__ u32 lent[@NL@ * 256];  // consumers' shared offsets of slot 0, per layout
  __shared__ __align__(16) float2 mtab[@NM@];  // the pass's dense matrices, staged once per CTA
  __shared__ double red[@NP@];  // probe accumulators of this CTA
  float2* buf = reinterpret_cast<float2*>(smraw);  // [S][NST][TS]
  const int t = threadIdx.x;
  for (int e = t; e < 768; e += 320) {
    const int part = e / 256;
    ttab[e] = tile_base(a, (i64)(e % 256) << (8 * part));
  }
  for (int j = t; j < NH; j += 320) {
    hoff[j] = lin_off(a, (u32)j << 5);
    hphys[j] = (u16)phys_dev((u32)j << 5);
  }
  for (int j = t; j < @NP@; j += 320) red[j] = 0.0;
@STAGE@
  if (t == 0) {
    abort_flag = 0;
    for (int b = 0; b < S; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 64;\n" ::"r"(su32(&full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 256;\n" ::"r"(su32(&empty[b])));
    }
  }
  __syncthreads();
  const i64 step = gridDim.x;
  const i64 count = blockIdx.x < a.ntiles ? (a.ntiles - 1 - blockIdx.x) / step + 1 : 0;
  volatile int* abort = &abort_flag;
  const int warp_u = __shfl_sync(0xffffffffu, t >> 5, 0);
  if (warp_u >= 8) {
    const int pt = t - 256;
    const int lane = pt & 31, pw = pt >> 5;
    const u64 lo_l = lin_off(a, (u32)lane);
    const u32 lp_l = phys_dev((u32)lane);
    const u64 so_l = lin_off(a, (u32)(2 * lane) & 31u);
    const u32 sp_l = phys_dev((u32)(2 * lane) & 31u);
    const int shalf = (2 * lane) >> 5;
    for (i64 i = 0; i < count + S; ++i) {
      const int b = (int)(i % S);
      float2* sb = buf + (size_t)b * NST * TS;
      if (i >= S) {
        if (!ws_wait(&empty[b], (u32)(((i - S) / S) & 1), abort)) break;
        const u64 gb = tile_base_fast(ttab, blockIdx.x + (i - S) * step);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          float2* g = (st ? a.lam : a.psi) + gb + so_l;
          const float2* sbs = sb + st * TS;
#pragma unroll 4
          for (int j = pw; j < NH / 2; j += 2) {
            const int h = 2 * j + shalf;
            const u32 p = sp_l ^ hphys[h];
            const float2 x = sbs[p], y = sbs[p ^ 1u];
            __stcs(reinterpret_cast<float4*>(g + hoff[h]), make_float4(x.x, x.y, y.x, y.y));
          }
        }
      }
      if (i < count) {
        const u64 gb = tile_base_fast(ttab, blockIdx.x + i * step);
#pragma unroll
        for (int st = 0; st < NST; ++st) {
          const float2* g = (st ? a.lam : a.psi) + gb + lo_l;
          float2* sbs = sb + st * TS;
#pragma unroll 4
          for (int jj = pw; jj < NH / 2; jj += 2) {
            cp_async8(sbs + (lp_l ^ hphys[2 * jj]), g + hoff[2 * jj]);
            cp_async8(sbs + (lp_l ^ hphys[2 * jj + 1]), g + hoff[2 * jj + 1]);
          }
        }
        asm volatile("cp.async.mbarrier.arrive.noinc.shared.b64 [%0];\n" ::"r"(su32(&full[b])) : "memory");
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  } else {
@SETUP@
    for (i64 i = 0; i < count; ++i) {
      const int b = (int)(i % S);
      const bool ok = ws_wait(&full[b], (u32)((i / S) & 1), abort);
      if (consumers_any(!ok)) break;
      char* sbb = reinterpret_cast<char*>(buf + (size_t)b * NST * TS);
      char* sbw = sbb + (size_t)TS * 8;
      const u64 gb = tile_base_fast(ttab, blockIdx.x + i * step);
      const float2* __restrict__ M = a.mats;
      float2 v[NSL];
      float2 w[NSL];
      (void)sbw;
      (void)w;
@BODY@
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(su32(&empty[b])) : "memory");
    }
@FLUSH@
  }
  if (t == 0 || t == 256) {
    if (*abort && a.abort) atomicExch(a.abort, 1);
  }
@EPILOGUE@
}
)GBQJIT";

struct JitArgs {
  float2* psi;
  float2* lam;
  const float2* mats;
  double* partial;
  int* abort;
  int64_t ntiles;
  int nbits;
  int L;
  uint64_t gw[13];
  int8_t nt[64];
};

// ---- NVRTC, loaded on first use -------------------------------------------------
struct Nvrtc {
  bool tried = false, ok = false;
  std::string why;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

static std::mutex g_nvrtc_mu;
static Nvrtc g_nvrtc;

static Nvrtc* nvrtc() {
  std::lock_guard<std::mutex> lk(g_nvrtc_mu);
  Nvrtc& n = g_nvrtc;
  if (n.tried) return n.ok ? &n : nullptr;
  n.tried = true;
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", nullptr, nullptr};
  std::string home = getenv("CUDA_HOME") ? getenv("CUDA_HOME") : "/usr/local/cuda";
  std::string abs = home + "/lib64/libnvrtc.so.13";
  names[2] = abs.c_str();
  void* h = nullptr;
  for (int i = 0; i < 3 && !h; ++i) h = dlopen(names[i], RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    n.why = "NVRTC library not found";
    return nullptr;
  }
  n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
  n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
  n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
  n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
  n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
  n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
  n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
  n.ok = n.create && n.compile && n.log_size && n.log && n.cubin_size && n.cubin && n.destroy;
  if (!n.ok) n.why = "NVRTC library lacks an entry point";
  return n.ok ? &n : nullptr;
}

// Compiles src for sm_103a; returns the CUBIN (empty on failure, with the
// compiler log in *log).
static std::string nvrtc_compile(const std::string& src, std::string* log) {
  Nvrtc* n = nvrtc();
  if (!n) {
    if (log) *log = g_nvrtc.why;
    return {};
  }
  nvrtcProgram prog;
  if (n->create(&prog, src.c_str(), "gbq_pass.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
    if (log) *log = "nvrtcCreateProgram failed";
    return {};
  }
  const bool verbose = getenv("GBQ_JIT_VERBOSE") != nullptr;
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-default-device",
                        "--ptxas-options=-v"};
  const nvrtcResult r = n->compile(prog, verbose ? 4 : 3, opts);
  size_t ls = 0;
  n->log_size(prog, &ls);
  std::string lg(ls, '\0');
  if (ls) n->log(prog, &lg[0]);
  if (log) *log = lg;
  if (verbose && ls > 1) fprintf(stderr, "gbq jit: %s\n", lg.c_str());
  std::string out;
  if (r == NVRTC_SUCCESS) {
    size_t cs = 0;
    n->cubin_size(prog, &cs);
    out.resize(cs);
    if (cs) n->cubin(prog, &out[0]);
  }
  n->destroy(&prog);
  return out;
}

// ---- source generation ----------------------------------------------------------
constexpr int kJitMaxLayouts = 8;  // per-thread layout table: 1 KB per layout
// Static shared memory per CTA that keeps two CTAs of three 32 KB tile
// buffers on an SM (228 KB per SM, 1 KB reserved per CTA).
constexpr int64_t kJitStaticSmem = 17 * 1024 - 256;

// Tile width of the specialised kernels: 12 bits for one state (16
// amplitudes per consumer thread), 11 bits for two states (8 + 8).
static int jit_tile_bits(bool dual) { return dual ? 11 : 12; }

static bool jit_op_ok(const OpDev& op, bool dual, int R) {
  if (op.kind == GBQ_OP_LAYOUT) return op.k == R;
  if (op.kind == GBQ_OP_RDENSE) return op.k >= 1 && op.k <= 2 && op.nsel <= 3;
  if (op.kind == GBQ_OP_RDIAG) return op.k >= 1 && op.k <= 8;
  if (!dual) return false;
  if (op.kind == GBQ_OP_RPROBE) return op.k >= 1 && op.k <= 3 && op.nsel <= 3;
  if (op.kind == GBQ_OP_RPROBE_DIAG) return op.k >= 1 && op.k <= 8;
  return false;
}

bool jit_eligible(const PassArgs& a, bool dual) {
  const TileInfo& ti = a.ti;
  if (ti.L != jit_tile_bits(dual) || ti.m < 5 || ti.pstride != 0 || ti.nops < 1 || ti.nbits - ti.L > 24)
    return false;
  if (dual && !ti.partial) {
    for (int o = 0; o < ti.nops; ++o)
      if (a.ops[o].kind == GBQ_OP_RPROBE || a.ops[o].kind == GBQ_OP_RPROBE_DIAG) return false;
  }
  if (a.ops[0].kind != GBQ_OP_LAYOUT) return false;
  int nl = 0;
  for (int o = 0; o < ti.nops; ++o) {
    if (!jit_op_ok(a.ops[o], dual, ti.L - 8)) return false;
    nl += a.ops[o].kind == GBQ_OP_LAYOUT;
  }
  return nl <= kJitMaxLayouts;
}

static std::string hex(uint32_t v) {
  char b[16];
  snprintf(b, sizeof(b), "0x%xu", v);
  return b;
}

// Shared byte offset (relative to the thread's slot 0) of register slot s.
static uint32_t slot_off(const OpDev& lay, int s, int R) {
  uint32_t p = 0;
  for (int b = 0; b < R; ++b)
    if ((s >> b) & 1) p ^= lay.pcol[b];
  return p * 8u;
}

std::string jit_source(const PassArgs& a, bool dual) {
  const TileInfo& ti = a.ti;
  const int L = ti.L, R = L - 8, NS = 1 << R;
  std::ostringstream setup, body, stage, epi;
  int nl = 0, np = 0;
  for (int o = 0; o < ti.nops; ++o) {
    nl += a.ops[o].kind == GBQ_OP_LAYOUT;
    if (a.ops[o].kind == GBQ_OP_RPROBE || a.ops[o].kind == GBQ_OP_RPROBE_DIAG) np = std::max(np, a.ops[o].pidx + 1);
  }
  // dense matrices staged in shared memory (as many ops as fit; the rest
  // are read through the read-only cache).  A family of 2^nsel selected
  // matrices is stored with a stride of dd + 2 entries, so the matrices
  // that the lanes of a quarter-warp select start in different banks.
  const int64_t nh = (int64_t)1 << (L - 5);
  const int64_t fixed = 768 * 8 + nh * 8 + nh * 2 + 6 * 8 + 16 + 8 * std::max(np, 1);
  const int64_t budget = (kJitStaticSmem - fixed - 1024 * (int64_t)nl) / 8;  // float2 entries
  int64_t staged = 0;
  std::vector<int64_t> soff(ti.nops, -1);
  for (int o = 0; o < ti.nops; ++o) {
    const OpDev& op = a.ops[o];
    if (op.kind != GBQ_OP_RDENSE && op.kind != GBQ_OP_RPROBE) continue;
    const int lg = 2 * op.k;
    const int64_t dd = (int64_t)1 << lg, stride = op.nsel ? dd + 2 : dd;
    const int64_t cnt = dd << op.nsel;
    if (staged + (stride << op.nsel) > budget) continue;
    soff[o] = staged;
    stage << "  for (int e = t; e < " << cnt << "; e += 320) mtab[" << staged << " + (e >> " << lg << ") * " << stride
          << " + (e & " << dd - 1 << ")] = a.mats[" << (long long)op.mat << "ll + e];\n";
    staged += stride << op.nsel;
  }
  // then the diagonal tables (2^k entries), read per tile with plain shared
  // loads instead of read-only-cache loads that each gate the ops after them
  for (int o = 0; o < ti.nops; ++o) {
    const OpDev& op = a.ops[o];
    if (op.kind != GBQ_OP_RDIAG && op.kind != GBQ_OP_RPROBE_DIAG) continue;
    const int64_t cnt = (int64_t)1 << op.k;
    if (staged + cnt > budget) continue;
    soff[o] = staged;
    stage << "  for (int e = t; e < " << cnt << "; e += 320) mtab[" << staged << " + e] = a.mats["
          << (long long)op.mat << "ll + e];\n";
    staged += cnt;
  }
  int q = -1;  // current layout index
  const OpDev* lay = nullptr;
  int tbit[13];  // thread bit carrying tile bit c in the current layout, or -1
  auto exit_layout = [&]() {
    for (int s = 0; s < NS; ++s) {
      body << "      *reinterpret_cast<float2*>(sbb + (P" << q << " ^ " << hex(slot_off(*lay, s, R)) << ")) = v[" << s
           << "];\n";
      if (dual)
        body << "      *reinterpret_cast<float2*>(sbw + (P" << q << " ^ " << hex(slot_off(*lay, s, R)) << ")) = w["
             << s << "];\n";
    }
    body << "      ops_barrier();\n";
  };
  auto matrix_ptr = [&](int o, const OpDev& op) {
    const int dd = 1 << (2 * op.k);
    const int stride = soff[o] >= 0 && op.nsel ? dd + 2 : dd;
    std::ostringstream sel;
    for (int s = 0; s < op.nsel; ++s) {
      const int c = op.selg[s];
      if (c >= 0)
        sel << " + (((u32)t >> " << tbit[c] << ") & 1u) * " << (stride << s) << "u";
      else
        sel << " + ((u32)(gb >> " << (-c - 1) << ") & 1u) * " << (stride << s) << "u";
    }
    std::ostringstream out;
    if (soff[o] >= 0)
      out << "true>(v, w, mtab + (" << soff[o] << sel.str() << "))";
    else
      out << "false>(v, w, M + (" << (long long)op.mat << "ll" << sel.str() << "))";
    return out.str();
  };
  for (int o = 0; o < ti.nops; ++o) {
    const OpDev& op = a.ops[o];
    if (op.kind == GBQ_OP_LAYOUT) {
      if (lay) exit_layout();
      ++q;
      lay = &op;
      for (int c = 0; c < 13; ++c) tbit[c] = -1;
      for (int j = 0; j < 8; ++j)
        for (int c = 0; c < L; ++c)
          if (op.tcol[j] == (1u << c)) tbit[c] = j;
      // per-thread shared byte offset of slot 0, kept in shared memory
      setup << "    {\n      u32 p = 0u;\n";
      for (int j = 0; j < 8; ++j)
        setup << "      if ((t >> " << j << ") & 1) p ^= " << hex(op.gcol[j] * 8u) << ";\n";
      setup << "      lent[" << q * 256 << " + t] = p;\n    }\n";
      body << "      const u32 P" << q << " = lent[" << q * 256 << " + t];\n";
      for (int s = 0; s < NS; ++s) {
        body << "      v[" << s << "] = *reinterpret_cast<const float2*>(sbb + (P" << q << " ^ "
             << hex(slot_off(op, s, R)) << "));\n";
        if (dual)
          body << "      w[" << s << "] = *reinterpret_cast<const float2*>(sbw + (P" << q << " ^ "
               << hex(slot_off(op, s, R)) << "));\n";
      }
      continue;
    }
    if (op.kind == GBQ_OP_RDENSE) {
      body << "      rdense<" << (int)op.rmask << ", " << matrix_ptr(o, op) << ";\n";
      continue;
    }
    if (op.kind == GBQ_OP_RPROBE) {
      body << "      pacc" << op.pidx << ".add(rprobe<" << (int)op.rmask << ", " << matrix_ptr(o, op) << ");\n";
      continue;
    }
    // RDIAG / RPROBE_DIAG: table index = thread part ^ global part ^ register-slot part
    const bool probe = op.kind == GBQ_OP_RPROBE_DIAG;
    body << "      {\n        u32 base = 0u;\n";
    for (int c = 0; c < L; ++c)
      if (op.dcol[c] && tbit[c] >= 0)
        body << "        if ((t >> " << tbit[c] << ") & 1) base ^= " << hex(op.dcol[c]) << ";\n";
    for (int j = 0; j < op.k && j < 8; ++j)
      if (op.dext[j] >= 0) body << "        base |= ((u32)(gb >> " << (int)op.dext[j] << ") & 1u) << " << j << ";\n";
    const bool sh = soff[o] >= 0;
    if (sh)
      body << "        const float2* tab = mtab + " << soff[o] << ";\n";
    else
      body << "        const float2* __restrict__ tab = M + " << (long long)op.mat << "ll;\n";
    auto tload = [&](uint32_t x) {
      return sh ? "tab[base ^ " + hex(x) + "]" : "__ldg(tab + (base ^ " + hex(x) + "))";
    };
    if (probe) body << "        float part = 0.f;\n";
    uint32_t rc[5];
    for (int p = 0; p < R; ++p) rc[p] = op.dcol[lay->rbits[p]];
    for (int s = 0; s < NS; ++s) {
      uint32_t x = 0;
      for (int p = 0; p < R; ++p)
        if ((s >> p) & 1) x ^= rc[p];
      if (probe) {
        body << "        {\n          const float2 y = cmul(" << tload(x) << ", v[" << s
             << "]);\n          part = fmaf(w[" << s << "].x, y.x, fmaf(w[" << s << "].y, y.y, part));\n        }\n";
      } else {
        body << "        {\n          const float2 d = " << tload(x) << ";\n          v[" << s
             << "] = cmul(d, v[" << s << "]);\n";
        if (dual) body << "          w[" << s << "] = cmul(d, w[" << s << "]);\n";
        body << "        }\n";
      }
    }
    if (probe) body << "        pacc" << op.pidx << ".add(part);\n";
    body << "      }\n";
  }
  if (lay) exit_layout();
  std::ostringstream flush;
  for (int i = 0; i < np; ++i) {
    setup << "    ffacc pacc" << i << ";\n";
    flush << "    probe_flush(pacc" << i << ", " << i << ", red);\n";
  }
  if (np) {
    // probe totals of this CTA: into the partial of its first tile, zeros into
    // those of its other tiles (the host sums over all tiles)
    epi << "  __syncthreads();\n";
    for (int o = 0; o < ti.nops; ++o) {
      const OpDev& op = a.ops[o];
      if (op.kind != GBQ_OP_RPROBE && op.kind != GBQ_OP_RPROBE_DIAG) continue;
      epi << "  for (i64 tile = blockIdx.x + (i64)t * step; tile < a.ntiles; tile += 320 * step)\n"
          << "    a.partial[(i64)" << op.slot << " * a.ntiles + tile] = tile == (i64)blockIdx.x ? red[" << op.pidx
          << "] : 0.0;\n";
    }
  }
  std::string src(kJitSkeleton);
  auto put = [&](const char* key, const std::string& val) {
    size_t at;
    while ((at = src.find(key)) != std::string::npos) src.replace(at, strlen(key), val);
  };
  put("@SWZ0@", std::to_string(kSwzRow0));
  put("@SWZ1@", std::to_string(kSwzRow1));
  put("@SWZ2@", std::to_string(kSwzRow2));
  put("@SWZ3@", std::to_string(kSwzRow3));
  put("@LT@", std::to_string(L));
  put("@DUAL@", dual ? "1" : "0");
  put("@NL@", std::to_string(q + 1));
  put("@NM@", std::to_string(std::max<int64_t>(staged, 2)));
  put("@NP@", std::to_string(std::max(np, 1)));
  put("@STAGE@", stage.str());
  put("@SETUP@", setup.str());
  put("@BODY@", body.str());
  put("@EPILOGUE@", epi.str());
  put("@FLUSH@", flush.str());
  return src;
}

// ---- kernel cache ---------------------------------------------------------------
struct JitKernel {
  int state = 0;  // 0 compiling, 1 ready, -1 failed
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kern = nullptr;
  int blocks_per_sm = 0;
  std::string log;
};

// Cache and compile queue.  Heap-allocated and never destroyed, so worker
// threads still compiling when the process exits touch no destroyed state.
struct JitJob {
  std::string key;
  std::unique_ptr<PassArgs> args;
  int device;
  bool dual;
};
struct JitState {
  std::mutex mu;
  std::condition_variable cv;       // a kernel became ready or failed
  std::condition_variable work_cv;  // a job was queued
  std::unordered_map<std::string, JitKernel> cache;
  std::deque<JitJob> queue;
  int workers = 0;
  int busy = 0;          // workers compiling now
  bool stopping = false;  // process exit: take no new job
  bool exit_hook = false;
  std::atomic<int64_t> compiles{0};
  std::atomic<int64_t> launches{0};
};
static JitState& jst() {
  static JitState* s = new JitState();
  return *s;
}

constexpr int kJitThreads = 320;
constexpr int kJitSmem = 3 * 4096 * 8;

// Loads a CUBIN into the current device's context.
static void jit_load(JitKernel& k, const std::string& cubin) {
  if (cubin.empty()) {
    k.state = -1;
    return;
  }
  cudaError_t e = cudaLibraryLoadData(&k.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&k.kern, k.lib, "k_jit");
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute((const void*)k.kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kJitSmem);
  int nb = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k.kern, kJitThreads, kJitSmem);
  if (e != cudaSuccess) {
    k.log = std::string("loading the specialised pass failed: ") + cudaGetErrorString(e);
    k.state = -1;
    return;
  }
  k.blocks_per_sm = nb > 0 ? nb : 1;
  k.state = 1;
}

// Cache key of a pass: its converted op records (zero-padded by
// convert_op), which fix the generated source completely, and the device.
std::string jit_key(const PassArgs& a, const Ctx* c, bool dual) {
  std::string k(reinterpret_cast<const char*>(&c->device), sizeof(c->device));
  k.push_back(dual ? 'D' : 'S');
  k.append(reinterpret_cast<const char*>(a.ops), (size_t)a.ti.nops * sizeof(OpDev));
  return k;
}

// Compiles and loads one queued pass (outside the lock).
static void jit_build(JitJob& job) {
  JitState& S = jst();
  std::string log;
  const std::string cubin = nvrtc_compile(jit_source(*job.args, job.dual), &log);
  S.compiles.fetch_add(1);
  JitKernel k;
  k.log = log;
  cudaSetDevice(job.device);
  jit_load(k, cubin);
  if (k.state != 1 && getenv("GBQ_DEBUG")) fprintf(stderr, "gbq jit: %s\n", k.log.c_str());
  std::lock_guard<std::mutex> lk(S.mu);
  S.cache[job.key] = k;
  S.cv.notify_all();
}

static void jit_worker() {
  JitState& S = jst();
  for (;;) {
    JitJob job;
    {
      std::unique_lock<std::mutex> lk(S.mu);
      S.work_cv.wait(lk, [&] { return S.stopping || !S.queue.empty(); });
      // at process exit a worker never returns: a thread that exits while the
      // process shuts down would run its CUDA runtime thread-exit handlers
      // against a runtime already torn down
      if (S.stopping) {
        S.cv.notify_all();
        for (;;) S.work_cv.wait(lk);
      }
      job = std::move(S.queue.front());
      S.queue.pop_front();
      ++S.busy;
    }
    jit_build(job);
    std::lock_guard<std::mutex> lk(S.mu);
    --S.busy;
    S.cv.notify_all();
  }
}

// At process exit: drop the queued jobs and wait (bounded) for the ones
// being compiled, so no worker is inside NVRTC or the CUDA runtime while
// they shut down.  Registered when the first worker starts, i.e. after the
// CUDA runtime, so it runs before the runtime's own exit handlers.
// Stops the compile workers: drops the queued jobs and waits (bounded) for
// the ones being compiled.  Returns true if none is left running.
static bool jit_stop(double timeout_s) {
  JitState& S = jst();
  std::unique_lock<std::mutex> lk(S.mu);
  S.stopping = true;
  for (auto& j : S.queue) S.cache.erase(j.key);
  S.queue.clear();
  S.work_cv.notify_all();
  return S.cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return S.busy == 0; });
}

static void jit_at_exit() { jit_stop(30.0); }

bool jit_enabled(Ctx* c) {
  if (c->jit < 0) {
    const char* e = getenv("GBQ_JIT");
    c->jit = e ? std::max(0, std::min(2, atoi(e))) : 2;
  }
  return c->jit > 0 && nvrtc() != nullptr;
}

// Queues the passes whose kernels are not cached (entry state 0 until a
// worker has built them).  With wait, returns once every kernel of `passes`
// is ready or has failed.
void jit_prepare(Ctx* c, std::vector<std::pair<std::string, PassArgs*>>& passes, bool dual, bool wait) {
  JitState& S = jst();
  std::unique_lock<std::mutex> lk(S.mu);
  if (S.stopping) return;
  size_t queued = 0;
  for (auto& p : passes) {
    if (S.cache.count(p.first)) continue;
    S.cache.emplace(p.first, JitKernel());
    JitJob job;
    job.key = p.first;
    job.args.reset(new PassArgs(*p.second));
    job.device = c->device;
    job.dual = dual;
    S.queue.push_back(std::move(job));
    ++queued;
  }
  if (queued) {
    const unsigned hw = std::thread::hardware_concurrency();
    const int want = (int)std::min<unsigned>(hw ? hw : 4, 16);
    const int target = std::min<int>(want, (int)S.queue.size());
    if (!S.exit_hook) {
      S.exit_hook = true;
      std::atexit(jit_at_exit);
    }
    while (S.workers < target) {
      std::thread(jit_worker).detach();
      ++S.workers;
    }
    S.work_cv.notify_all();
  }
  if (!wait) return;
  // bounded: a pass whose kernel is still not built then runs the interpreter
  const auto until = std::chrono::steady_clock::now() + std::chrono::seconds(600);
  for (auto& p : passes)
    S.cv.wait_until(lk, until, [&] {
      auto it = S.cache.find(p.first);
      return it == S.cache.end() || it->second.state != 0;
    });
}

// The ready kernel of a key, or nullptr (not queued, still compiling, failed).
static JitKernel* jit_ready(const std::string& key) {
  JitState& S = jst();
  std::lock_guard<std::mutex> lk(S.mu);
  auto it = S.cache.find(key);
  return it != S.cache.end() && it->second.state == 1 ? &it->second : nullptr;
}

// Launches the specialised kernel of a pass; launched = false when the pass
// is not eligible or its kernel is unavailable (the interpreter then runs).
int jit_launch(Ctx* c, const PassArgs& a, const std::string& key, bool& launched) {
  // the kernel's own state count is part of its key
  launched = false;
  JitKernel* k = jit_ready(key);
  if (!k) return GBQ_OK;
  JitArgs j;
  memset(&j, 0, sizeof(j));
  j.psi = a.psi;
  j.lam = a.lam;
  j.partial = a.ti.partial;
  j.mats = a.ti.mats;
  j.abort = a.abort;
  j.ntiles = a.ti.ntiles;
  j.nbits = a.ti.nbits;
  j.L = a.ti.L;
  for (int b = 0; b < 13; ++b) j.gw[b] = a.ti.gw[b];
  memcpy(j.nt, a.ti.nt, sizeof(j.nt));
  int64_t grid = (int64_t)c->sm_count * k->blocks_per_sm;
  if (grid > a.ti.ntiles) grid = a.ti.ntiles;
  void* args[] = {&j};
  cudaError_t e = cudaLaunchKernel((const void*)k->kern, dim3((unsigned)grid), dim3(kJitThreads), args,
                                   kJitSmem, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "specialised pass launch");
  c->launches += 1;
  jst().launches.fetch_add(1);
  launched = true;
  return GBQ_OK;
}

int64_t jit_compile_count() { return jst().compiles.load(); }
int64_t jit_launch_count() { return jst().launches.load(); }

int64_t jit_pending() {
  JitState& S = jst();
  std::lock_guard<std::mutex> lk(S.mu);
  int64_t n = 0;
  for (const auto& e : S.cache) n += e.second.state == 0;
  return n;
}

}  // namespace gbq

using namespace gbq;

extern "C" {

// Stops background compilation for good (the process is about to exit):
// queued passes are dropped and running compiles are awaited, at most
// timeout_s seconds.  Passes whose kernel is not built keep running on the
// interpreter.
int gbq_jit_shutdown(double timeout_s) {
  return jit_stop(timeout_s > 0 ? timeout_s : 0.0) ? GBQ_OK : GBQ_ERR_UNSUPPORTED;
}

// Test hook: compiles a source with NVRTC for sm_103a (no GPU needed).
// Returns 0 and the CUBIN size, or an error with the compiler log.
int gbq_jit_compile_check(const char* src, size_t* cubin_bytes) {
  if (!src) return GBQ_ERR_ARG;
  std::string log;
  const std::string cubin = nvrtc_compile(src, &log);
  if (cubin_bytes) *cubin_bytes = cubin.size();
  if (cubin.empty()) {
    set_error("specialised pass compile failed: " + log);
    return GBQ_ERR_UNSUPPORTED;
  }
  return GBQ_OK;
}

}  // extern "C"
