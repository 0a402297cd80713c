// C ABI of cirq_gb300 (declared in include/cirq_gb300.h).
//
// Host-side validation happens here, before any launch: every pass's tile
// geometry and every op's bit positions are checked against the state width
// so that no kernel can index outside its tile or its state.

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <stdlib.h>
#include <sys/mman.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "gbq_internal.cuh"

namespace gbq {

// implemented in gbq_kernels.cu
int do_set_basis(Ctx* c, float2* s, int nbits, uint64_t index);
int do_norm2(Ctx* c, const float2* s, int nbits, float scale, int use_scale, double* d_out);
int do_scale(Ctx* c, float2* s, int nbits, float scale);
int do_project(Ctx* c, float2* s, int nbits, uint64_t mask, uint64_t value, float scale);
int do_probs(Ctx* c, const float2* s, int nq, int dm, float* out);
int do_sample(Ctx* c, const float2* s, int nq, int dm, const double* d_u, int64_t R,
              uint64_t* d_out, double* d_cdf);
int do_expect(Ctx* c, const float2* s, int nbits, const gbq_pauli* d_terms, int nterms,
              double* d_partial, double* d_out);
int expect_chunk_bits(int nbits);
int dm_expect_chunks(Ctx* c, int nq);
int do_dm_expect(Ctx* c, const float2* rho, int nq, const gbq_pauli* d_terms, int nterms,
                 double* d_partial, double* d_out);
int do_inner(Ctx* c, const float2* a, const float2* b, int nbits, double* d_out);
int do_reduce_slots(Ctx* c, const double* partial, int nslots, int64_t ntiles, double* out);

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return e == cudaErrorMemoryAllocation ? GBQ_ERR_OOM : GBQ_ERR_CUDA;
}

static int arg_fail(const std::string& msg) {
  g_err = msg;
  return GBQ_ERR_ARG;
}

int ensure_scratch(Ctx* c, size_t bytes) {
  if (c->scratch_bytes >= bytes) return GBQ_OK;
  if (c->scratch) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
  }
  const size_t want = bytes < 4096 ? 4096 : bytes;
  cudaError_t e = cudaMalloc(&c->scratch, want);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
  c->scratch_bytes = want;
  return GBQ_OK;
}

int ensure_host_scratch(Ctx* c, size_t bytes) {
  if (c->host_scratch_bytes >= bytes) return GBQ_OK;
  if (c->host_scratch) {
    cudaStreamSynchronize(c->stream);
    cudaFreeHost(c->host_scratch);
    c->host_scratch = nullptr;
    c->host_scratch_bytes = 0;
  }
  const size_t want = bytes < 4096 ? 4096 : bytes;
  cudaError_t e = cudaMallocHost(&c->host_scratch, want);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocHost(scratch)");
  c->host_scratch_bytes = want;
  return GBQ_OK;
}

static int set_device(Ctx* c) {
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return GBQ_OK;
}

static int sync(Ctx* c, const char* what) {
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail(e, what);
  if (c->abort_armed && c->d_abort) {
    int flag = 0;
    e = cudaMemcpy(&flag, c->d_abort, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (flag) {
      cudaMemset(c->d_abort, 0, sizeof(int));
      set_error(std::string(what) + ": a pass gave up a bounded wait (state invalid)");
      return GBQ_ERR_CUDA;
    }
  }
  return GBQ_OK;
}

// Bank-pair column (shared index mod 16) of tile bit b.
static uint32_t bank_col(int b) { return phys_const(1u << b) & 15u; }

// Converts one public op into its device form for a pass whose tile bits
// are described by `inmask` (global bits in the tile).  The group index of a
// dense op enumerates its non-target tile bits in this order: 4 bits whose
// bank columns are independent (conflict-free half-warps), the other free
// bits, then the tile bits used as selectors (so a selector is uniform over
// a warp and the matrix loads do not diverge).
// Register layout in force while converting the ops of one pass:
// reg[p] = tile bit of register position p, nreg = 0 outside a phase.
struct LayoutState {
  int nreg = 0;
  int reg[5] = {0, 0, 0, 0, 0};
  int nprobe = 0;  // probe ops of the pass so far (their accumulator index)
};

// Thread-bit order of a layout: 4 bank-independent bits first.
static void thread_bit_order(int L, uint32_t regmask, int* order, int& no) {
  no = 0;
  uint32_t basis[4] = {0, 0, 0, 0};
  int nbasis = 0;
  uint32_t used = regmask;
  for (int b = 0; b < L && nbasis < 4; ++b) {
    if ((used >> b) & 1u) continue;
    uint32_t v = phys_const(1u << b) & 15u;
    for (int i = 0; i < nbasis; ++i)
      if ((v ^ basis[i]) < v) v ^= basis[i];
    if (!v) continue;
    basis[nbasis++] = v;
    for (int i = nbasis - 1; i > 0 && basis[i] > basis[i - 1]; --i) {
      const uint32_t t = basis[i];
      basis[i] = basis[i - 1];
      basis[i - 1] = t;
    }
    order[no++] = b;
    used |= 1u << b;
  }
  for (int b = 0; b < L; ++b)
    if (!((used >> b) & 1u)) order[no++] = b;
}

static int convert_op(const gbq_op& op, int L, int nbits, uint64_t inmask, bool dual, OpDev& d,
                      LayoutState& lay) {
  memset(&d, 0, sizeof(d));
  const int kind = op.kind;
  const bool reg = kind == GBQ_OP_RDENSE || kind == GBQ_OP_RDIAG || kind == GBQ_OP_RPROBE ||
                   kind == GBQ_OP_RPROBE_DIAG;
  if (kind == GBQ_OP_LAYOUT) {
    const int R = L - 8;
    if (L > 12) return arg_fail("op: register layouts need tile widths 10..12");
    if (op.k != R) return arg_fail("op: a layout names exactly L - 8 register bits");
    uint32_t regmask = 0;
    for (int p = 0; p < R; ++p) {
      const int b = op.bits[p];
      if (b < 0 || b >= L || ((regmask >> b) & 1u)) return arg_fail("op: layout bit invalid");
      regmask |= 1u << b;
      d.pcol[p] = phys_const(1u << b);
      d.rbits[p] = (int8_t)b;
      lay.reg[p] = b;
    }
    lay.nreg = R;
    int order[GBQ_MAX_TILE_BITS];
    int no = 0;
    thread_bit_order(L, regmask, order, no);
    if (no != 8) return arg_fail("op: internal layout error");
    for (int j = 0; j < 8; ++j) {
      d.gcol[j] = phys_const(1u << order[j]);
      d.tcol[j] = (uint16_t)(1u << order[j]);
    }
    d.kind = (int8_t)kind;
    d.k = (int8_t)R;
    return GBQ_OK;
  }
  if (reg && lay.nreg == 0) return arg_fail("op: register op outside a register layout");
  if (!reg) lay.nreg = 0;  // a plain op ends the phase
  const bool dense = kind == GBQ_OP_DENSE || kind == GBQ_OP_PROBE;
  const bool diag = kind == GBQ_OP_DIAG || kind == GBQ_OP_PROBE_DIAG;
  const bool rdense = kind == GBQ_OP_RDENSE || kind == GBQ_OP_RPROBE;
  const bool rdiag = kind == GBQ_OP_RDIAG || kind == GBQ_OP_RPROBE_DIAG;
  const bool probe = kind == GBQ_OP_PROBE || kind == GBQ_OP_PROBE_DIAG || kind == GBQ_OP_RPROBE ||
                     kind == GBQ_OP_RPROBE_DIAG;
  if (!dense && !diag && !rdense && !rdiag) return arg_fail("op: unknown kind");
  if (probe && !dual) return arg_fail("op: probe ops need a two-state pass");
  if (probe && op.slot < 0) return arg_fail("op: probe slot < 0");
  if (op.mat < 0 || (op.mat & 1)) return arg_fail("op: matrix offset must be even and >= 0");
  d.kind = op.kind;
  d.k = op.k;
  d.slot = op.slot;
  d.mat = op.mat;
  if (probe) d.pidx = lay.nprobe++;
  for (int p = 0; p < lay.nreg; ++p) d.rbits[p] = (int8_t)lay.reg[p];
  if (rdense) {
    const int kmax = kind == GBQ_OP_RPROBE ? 3 : 4;
    if (op.k < 1 || op.k > kmax || op.k > lay.nreg) return arg_fail("op: register dense k out of range");
    if (op.nsel < 0 || op.nsel > 3) return arg_fail("op: nsel out of range");
    int mask = 0, lastpos = -1;
    for (int j = 0; j < op.k; ++j) {
      int pos = -1;
      for (int p = 0; p < lay.nreg; ++p)
        if (lay.reg[p] == op.bits[j]) pos = p;
      if (pos < 0) return arg_fail("op: register op target is not a register bit");
      if (pos <= lastpos) return arg_fail("op: register op targets must ascend in register position");
      lastpos = pos;
      mask |= 1 << pos;
    }
    d.rmask = (int8_t)mask;
    d.nsel = op.nsel;
    for (int j = 0; j < op.nsel; ++j) {
      const int sb = op.sel[j];
      if (sb >= 0) {
        if (sb >= L) return arg_fail("op: selector tile bit out of range");
        for (int p = 0; p < lay.nreg; ++p)
          if (lay.reg[p] == sb) return arg_fail("op: register op selector is a register bit");
      } else {
        const int gb = -sb - 1;
        if (gb >= nbits || ((inmask >> gb) & 1ull))
          return arg_fail("op: selector global bit invalid (must be outside the tile)");
      }
      d.selg[j] = (int8_t)sb;
    }
    return GBQ_OK;
  }
  if (dense) {
    const int kmax = op.kind == GBQ_OP_PROBE ? 3 : GBQ_MAX_DENSE_K;
    if (op.k < 1 || op.k > kmax || op.k > L) return arg_fail("op: dense k out of range");
    if (op.nsel < 0 || op.nsel > 3) return arg_fail("op: nsel out of range");
    uint32_t tmask = 0;
    for (int j = 0; j < op.k; ++j) {
      const int b = op.bits[j];
      if (b < 0 || b >= L || ((tmask >> b) & 1u)) return arg_fail("op: dense target bit invalid");
      tmask |= 1u << b;
      d.pcol[j] = phys_const(1u << b);
    }
    uint32_t smask = 0;
    for (int j = 0; j < op.nsel; ++j) {
      const int s = op.sel[j];
      if (s >= 0) {
        if (s >= L) return arg_fail("op: selector tile bit out of range");
        if ((tmask >> s) & 1u) return arg_fail("op: selector bit is a target");
        if ((smask >> s) & 1u) return arg_fail("op: duplicate selector bit");
        smask |= 1u << s;
      } else {
        const int gb = -s - 1;
        if (gb >= nbits || ((inmask >> gb) & 1ull))
          return arg_fail("op: selector global bit invalid (must be outside the tile)");
      }
    }
    int order[GBQ_MAX_TILE_BITS];
    int no = 0;
    uint32_t basis[4] = {0, 0, 0, 0};
    int nbasis = 0;
    uint32_t used = tmask | smask;
    for (int b = 0; b < L && nbasis < 4; ++b) {
      if ((used >> b) & 1u) continue;
      uint32_t v = bank_col(b);
      for (int i = 0; i < nbasis; ++i)
        if ((v ^ basis[i]) < v) v ^= basis[i];
      if (!v) continue;
      basis[nbasis++] = v;
      // keep the basis sorted descending so the reduction above is valid
      for (int i = nbasis - 1; i > 0 && basis[i] > basis[i - 1]; --i) {
        const uint32_t t = basis[i];
        basis[i] = basis[i - 1];
        basis[i - 1] = t;
      }
      order[no++] = b;
      used |= 1u << b;
    }
    for (int b = 0; b < L; ++b)
      if (!((used >> b) & 1u)) order[no++] = b;
    for (int j = 0; j < op.nsel; ++j)
      if (op.sel[j] >= 0) order[no++] = op.sel[j];
    if (no != L - op.k) return arg_fail("op: internal group order error");
    for (int i = 0; i < no; ++i) d.gcol[i] = phys_const(1u << order[i]);
    d.nsel = op.nsel;
    for (int j = 0; j < op.nsel; ++j) {
      const int s = op.sel[j];
      if (s >= 0) {
        int pos = -1;
        for (int i = 0; i < no; ++i)
          if (order[i] == s) pos = i;
        d.selg[j] = (int8_t)pos;
      } else {
        d.selg[j] = (int8_t)s;
      }
    }
  } else {
    // plain and register diagonal ops share the table encoding
    if (op.k < 1 || op.k > GBQ_MAX_DIAG_K) return arg_fail("op: diag k out of range");
    for (int j = 0; j < 8; ++j) d.dext[j] = -1;
    for (int j = 0; j < op.k; ++j) {
      const int s = op.bits[j];
      if (s >= 0) {
        if (s >= L) return arg_fail("op: diag tile bit out of range");
        if (d.dcol[s]) return arg_fail("op: duplicate diag bit");
        d.dcol[s] = (uint16_t)(1u << j);
      } else {
        const int gb = -s - 1;
        if (gb >= nbits || ((inmask >> gb) & 1ull)) return arg_fail("op: diag global bit invalid");
        d.dext[j] = (int8_t)gb;
      }
    }
  }
  return GBQ_OK;
}

// Validates one pass against a state of nbits bits; fills `ti` (not the
// pointers) and the tile-membership mask.
static int pass_geometry(const gbq_pass& p, int nops, int nbits, TileInfo& ti, uint64_t& inmask) {
  if (p.L < GBQ_MIN_TILE_BITS || p.L > GBQ_MAX_TILE_BITS || p.L > nbits)
    return arg_fail("pass: tile bits L=" + std::to_string(p.L) + " invalid for a " +
                    std::to_string(nbits) + "-bit state (need 10 <= L <= min(13, nbits))");
  if (p.m < 1 || p.m > p.L) return arg_fail("pass: contiguous bits m out of range");
  if (p.op_count < 0 || p.op_count > GBQ_MAX_OPS_PER_PASS)
    return arg_fail("pass: op_count out of range (max 64)");
  if (p.op_begin < 0 || p.op_begin + p.op_count > nops) return arg_fail("pass: ops out of range");
  inmask = (1ull << p.m) - 1ull;
  memset(&ti, 0, sizeof(ti));
  for (int b = 0; b < p.m; ++b) ti.gw[b] = 1ull << b;
  for (int j = 0; j < p.L - p.m; ++j) {
    const int b = p.hi[j];
    if (b < p.m || b >= nbits) return arg_fail("pass: tile high bit out of range");
    if ((inmask >> b) & 1ull) return arg_fail("pass: duplicate tile bit");
    inmask |= 1ull << b;
    ti.gw[p.m + j] = 1ull << b;
  }
  ti.nbits = nbits;
  ti.L = p.L;
  ti.m = p.m;
  ti.nops = p.op_count;
  ti.ntiles = (int64_t)1 << (nbits - p.L);
  int c = 0;
  for (int b = 0; b < nbits; ++b)
    if (!((inmask >> b) & 1ull)) ti.nt[c++] = (int8_t)b;
  return GBQ_OK;
}

static int launch_pass(Ctx* c, const PassArgs& a, bool dual) {
  switch (a.ti.L) {
    case 10: return launch_pass_l10(c, a, dual);
    case 11: return launch_pass_l11(c, a, dual);
    case 12: return launch_pass_l12(c, a, dual);
    case 13: return launch_pass_l13(c, a, dual);
    default: return arg_fail("pass: unsupported tile width");
  }
}

static int timed_pair(Ctx* c, std::pair<cudaEvent_t, cudaEvent_t>& ev) {
  if (!c->event_pool.empty()) {
    ev = c->event_pool.back();
    c->event_pool.pop_back();
    return GBQ_OK;
  }
  cudaError_t e = cudaEventCreate(&ev.first);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  e = cudaEventCreate(&ev.second);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  return GBQ_OK;
}

static bool is_mma_pass(const gbq_pass& p, const gbq_op* ops) {
  for (int o = 0; o < p.op_count; ++o)
    if (ops[p.op_begin + o].kind == GBQ_OP_MMA) return true;
  return false;
}

// Checks one pass (and fills the kernel arguments of its kind).
// mma: 0 = CUDA-core pass (PassArgs), 1 = 11-bit tensor-core pass (MmaArgs),
// 2 = pipelined 12-bit tensor-core pass (TcArgs).
static int convert_pass(const gbq_pass& p, const gbq_op* ops, int nops, int nbits, bool dual, PassArgs& a,
                        MmaArgs& ma, TcArgs& ta, int& mma) {
  memset(&a, 0, sizeof(a));
  uint64_t inmask = 0;
  int rc = pass_geometry(p, nops, nbits, a.ti, inmask);
  if (rc) return rc;
  mma = is_mma_pass(p, ops) ? (p.L == GBQ_TC_TILE_BITS ? 2 : 1) : 0;
  if (mma) {
    if (dual) return arg_fail("pass: tensor-core passes run on one state only");
    if (mma == 2) return build_tc_args(p, ops, nbits, a.ti, inmask, ta);
    return build_mma_args(p, ops, nbits, a.ti, inmask, ma);
  }
  LayoutState lay;
  for (int o = 0; o < p.op_count; ++o) {
    rc = convert_op(ops[p.op_begin + o], p.L, nbits, inmask, dual, a.ops[o], lay);
    if (rc) return rc;
  }
  return GBQ_OK;
}

static int run_passes(Ctx* c, float2* psi, float2* lam, int nbits, const gbq_pass* passes,
                      int npasses, const gbq_op* ops, int nops, const float2* mats,
                      double* partial) {
  const bool dual = lam != nullptr;
  PassArgs a;
  MmaArgs ma;
  TcArgs ta;
  // pass-specialised kernels: queue the new ones of this program (compiled
  // in parallel by worker threads); mode 1 waits for them
  // background mode only for states of >= kJitAutoMinBits bits: below, a
  // pass takes microseconds and the interpreter is as fast
  const bool jit = jit_enabled(c) && (c->jit == 1 || nbits >= kJitAutoMinBits);
  if (jit) {
    std::vector<std::pair<std::string, PassArgs*>> todo;
    int rc = GBQ_OK;
    for (int q = 0; q < npasses && !rc; ++q) {
      int mma = 0;
      rc = convert_pass(passes[q], ops, nops, nbits, dual, a, ma, ta, mma);
      if (rc || mma) continue;
      a.ti.partial = partial;
      if (!jit_eligible(a, dual)) continue;
      todo.emplace_back(jit_key(a, c, dual), new PassArgs(a));
    }
    if (!rc) jit_prepare(c, todo, dual, c->jit == 1);
    for (auto& t : todo) delete t.second;
    if (rc) return rc;
  }
  for (int q = 0; q < npasses; ++q) {
    int mma = 0;
    int rc = convert_pass(passes[q], ops, nops, nbits, dual, a, ma, ta, mma);
    if (rc) return rc;
    a.psi = psi;
    a.lam = lam;
    a.abort = c->d_abort;
    a.ti.mats = mats;
    a.ti.partial = partial;
    c->abort_armed = true;
    std::pair<cudaEvent_t, cudaEvent_t> ev;
    if (c->pass_timing) {
      rc = timed_pair(c, ev);
      if (rc) return rc;
      cudaEventRecord(ev.first, c->stream);
    }
    if (mma == 2) {
      ta.psi = psi;
      ta.ti.mats = mats;
      ta.abort = c->d_abort;
      rc = launch_tc_pass(c, ta);
    } else if (mma == 1) {
      ma.psi = psi;
      ma.ti.mats = mats;
      ma.abort = c->d_abort;
      rc = launch_mma_pass(c, ma);
    } else {
      bool launched = false;
      if (jit && jit_eligible(a, dual)) rc = jit_launch(c, a, jit_key(a, c, dual), launched);
      if (!rc && !launched) rc = launch_pass(c, a, dual);
    }
    if (rc) return rc;
    if (c->pass_timing) {
      cudaEventRecord(ev.second, c->stream);
      c->timed.push_back(ev);
    }
  }
  return GBQ_OK;
}

}  // namespace gbq

using namespace gbq;

#define CHECK_CTX(c)                                   \
  do {                                                 \
    if (!(c)) return arg_fail("null context");         \
    int _rc = set_device(c);                           \
    if (_rc) return _rc;                               \
  } while (0)

extern "C" {

const char* gbq_last_error(void) { return g_err.c_str(); }

int gbq_version(void) { return 1; }

int gbq_struct_sizes(int* op, int* pass, int* pauli, int* point) {
  if (op) *op = (int)sizeof(gbq_op);
  if (pass) *pass = (int)sizeof(gbq_pass);
  if (pauli) *pauli = (int)sizeof(gbq_pauli);
  if (point) *point = (int)sizeof(gbq_point);
  return GBQ_OK;
}

int gbq_ctx_create(int device, gbq_ctx** out) {
  if (!out) return arg_fail("null output pointer");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
  if (device < 0 || device >= ndev) return arg_fail("device index out of range");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  gbq_ctx* c = new gbq_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_abort, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(c->d_abort, 0, sizeof(int));
  if (e != cudaSuccess) {
    if (c->d_abort) cudaFree(c->d_abort);
    cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(e, "gbq_ctx_create");
  }
  *out = c;
  return GBQ_OK;
}

int gbq_ctx_destroy(gbq_ctx* c) {
  if (!c) return GBQ_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  if (c->scratch) cudaFree(c->scratch);
  if (c->d_abort) cudaFree(c->d_abort);
  if (c->host_scratch) cudaFreeHost(c->host_scratch);
  for (auto& ev : c->timed) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  for (auto& ev : c->event_pool) {
    cudaEventDestroy(ev.first);
    cudaEventDestroy(ev.second);
  }
  for (auto& ev : c->events)
    if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(c->stream);
  delete c;
  return GBQ_OK;
}

int gbq_ctx_sync(gbq_ctx* c) {
  CHECK_CTX(c);
  return sync(c, "gbq_ctx_sync");
}

int gbq_device_info(gbq_ctx* c, int* sm_count, size_t* free_bytes, size_t* total_bytes) {
  CHECK_CTX(c);
  if (sm_count) *sm_count = c->sm_count;
  size_t f = 0, t = 0;
  cudaError_t e = cudaMemGetInfo(&f, &t);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return GBQ_OK;
}

int gbq_device_name(gbq_ctx* c, char* buf, int len) {
  CHECK_CTX(c);
  if (!buf || len < 1) return arg_fail("gbq_device_name: bad buffer");
  cudaDeviceProp p;
  cudaError_t e = cudaGetDeviceProperties(&p, c->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  strncpy(buf, p.name, (size_t)len - 1);
  buf[len - 1] = 0;
  return GBQ_OK;
}

int gbq_set_graphs(gbq_ctx* c, int enable) {
  if (!c) return arg_fail("null context");
  c->use_graphs = enable != 0;
  return GBQ_OK;
}

int gbq_cliff_validate(int nq, const gbq_cliff_op* ops, int nops, int ntables, int nconds, int nrec) {
  if (nq < 1 || nq > (1 << 20) || nops < 0 || (nops && !ops) || ntables < 0 || nconds < 0 || nrec < 0)
    return arg_fail("gbq_cliff_validate: bad sizes");
  if (cliff_check(nq, ops, nops, ntables, nconds, nrec)) return arg_fail("gbq_cliff_validate: invalid op");
  return GBQ_OK;
}

int gbq_cliff_reference(gbq_ctx* c, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables,
                        int ntables, const int32_t* conds, int nconds, int nrec, uint8_t* ref_out) {
  CHECK_CTX(c);
  int rc = gbq_cliff_validate(nq, ops, nops, ntables, nconds, nrec);
  if (rc) return rc;
  if ((ntables && !tables) || (nconds && !conds) || (nrec && !ref_out)) return arg_fail("gbq_cliff_reference: null array");
  for (int i = 0; i < nconds; ++i)
    if (conds[i] < 0 || conds[i] >= nrec) return arg_fail("gbq_cliff_reference: condition record out of range");
  return cliff_reference(c, nq, ops, nops, tables, ntables, conds, nconds, nrec, ref_out);
}

int gbq_cliff_sample(gbq_ctx* c, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables, int ntables,
                     const int32_t* conds, int nconds, const uint8_t* ref, int nrec, int64_t shots, uint64_t seed,
                     void* out, const int32_t* layers, int nlayers, int out_bytes) {
  CHECK_CTX(c);
  int rc = gbq_cliff_validate(nq, ops, nops, ntables, nconds, nrec);
  if (rc) return rc;
  if (shots < 1 || shots > ((int64_t)1 << 40)) return arg_fail("gbq_cliff_sample: shots out of range");
  if (out_bytes && nrec > (1 << 21)) return arg_fail("gbq_cliff_sample: byte output takes at most 2^21 records");
  if ((nconds && !conds) || (nrec && (!ref || !out))) return arg_fail("gbq_cliff_sample: null array");
  for (int i = 0; i < nconds; ++i)
    if (conds[i] < 0 || conds[i] >= nrec) return arg_fail("gbq_cliff_sample: condition record out of range");
  (void)tables;
  if (layers) {
    if (nlayers < 0 || layers[0] != 0 || layers[nlayers] != nops) return arg_fail("gbq_cliff_sample: bad layers");
    std::vector<int> last(nq, -1), rec_layer(nrec, INT32_MAX);
    for (int L = 0; L < nlayers; ++L) {
      if (layers[L + 1] < layers[L]) return arg_fail("gbq_cliff_sample: layers must not decrease");
      for (int o = layers[L]; o < layers[L + 1]; ++o) {
        const gbq_cliff_op& op = ops[o];
        if (op.kind == GBQ_CLIFF_MEASURE) rec_layer[op.rec] = L;
        if (op.kind == GBQ_CLIFF_COND_PAULI)
          for (int i = 0; i < op.cond_count; ++i)
            if (rec_layer[conds[op.cond_begin + i]] >= L)
              return arg_fail("gbq_cliff_sample: a condition must come after its measurement's layer");
        const int k = (op.kind == GBQ_CLIFF_UNITARY || op.kind == GBQ_CLIFF_COND_PAULI) ? op.k : 1;
        for (int j = 0; j < k; ++j) {
          if (last[op.q[j]] == L) return arg_fail("gbq_cliff_sample: a layer acts twice on one qubit");
          last[op.q[j]] = L;
        }
      }
    }
  }
  return cliff_sample(c, nq, ops, nops, conds, nconds, ref, nrec, shots, seed, out, layers, layers ? nlayers : 0,
                      out_bytes != 0);
}

int gbq_set_jit(gbq_ctx* c, int mode) {
  if (!c) return arg_fail("null context");
  if (mode < 0 || mode > 2) return arg_fail("gbq_set_jit: mode must be 0, 1 or 2");
  c->jit = mode;
  return GBQ_OK;
}

int gbq_jit_stats(int64_t* compiles, int64_t* pending, int64_t* launches) {
  if (!compiles) return arg_fail("null argument");
  *compiles = jit_compile_count();
  if (pending) *pending = jit_pending();
  if (launches) *launches = jit_launch_count();
  return GBQ_OK;
}

int gbq_jit_source(int nbits, const gbq_pass* pass, const gbq_op* ops, int nops, int dual, char* buf, size_t len,
                   size_t* needed) {
  if (!pass || !ops || !needed) return arg_fail("gbq_jit_source: null argument");
  PassArgs* a = new PassArgs();
  MmaArgs* ma = new MmaArgs();
  TcArgs* ta = new TcArgs();
  int mma = 0;
  int rc = convert_pass(*pass, ops, nops, nbits, dual != 0, *a, *ma, *ta, mma);
  static double probe_sink;  // probes need a partial buffer to be eligible; only its presence is checked
  a->ti.partial = dual ? &probe_sink : nullptr;
  if (!rc && (mma || !jit_eligible(*a, dual != 0))) rc = GBQ_ERR_UNSUPPORTED;
  if (rc == GBQ_ERR_UNSUPPORTED) set_error("gbq_jit_source: the pass has no specialised form");
  if (!rc) {
    const std::string src = jit_source(*a, dual != 0);
    *needed = src.size() + 1;
    if (buf && len) {
      const size_t n = std::min(len - 1, src.size());
      memcpy(buf, src.data(), n);
      buf[n] = '\0';
    }
  }
  delete a;
  delete ma;
  delete ta;
  return rc;
}

int gbq_launch_count(gbq_ctx* c, int64_t* out) {
  if (!c || !out) return arg_fail("null argument");
  *out = c->launches;
  return GBQ_OK;
}

int gbq_event_record(gbq_ctx* c, int slot) {
  CHECK_CTX(c);
  if (slot < 0 || slot >= 16) return arg_fail("event slot out of range (0..15)");
  cudaError_t e;
  if (!c->events[slot]) {
    e = cudaEventCreate(&c->events[slot]);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  }
  e = cudaEventRecord(c->events[slot], c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
  return GBQ_OK;
}

int gbq_event_elapsed(gbq_ctx* c, int a, int b, float* ms) {
  CHECK_CTX(c);
  if (a < 0 || a >= 16 || b < 0 || b >= 16 || !c->events[a] || !c->events[b] || !ms)
    return arg_fail("gbq_event_elapsed: events not recorded");
  cudaError_t e = cudaEventSynchronize(c->events[b]);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize");
  e = cudaEventElapsedTime(ms, c->events[a], c->events[b]);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
  return GBQ_OK;
}

int gbq_pass_timing(gbq_ctx* c, double* total_ms, int64_t* launches) {
  CHECK_CTX(c);
  for (auto& ev : c->timed) {
    cudaError_t e = cudaEventSynchronize(ev.second);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize");
    float ms = 0.f;
    e = cudaEventElapsedTime(&ms, ev.first, ev.second);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
    c->timed_ms += ms;
    c->timed_launches += 1;
    c->event_pool.push_back(ev);
  }
  c->timed.clear();
  if (total_ms) *total_ms = c->timed_ms;
  if (launches) *launches = c->timed_launches;
  return GBQ_OK;
}

int gbq_set_pass_timing(gbq_ctx* c, int enable) {
  CHECK_CTX(c);
  int rc = gbq_pass_timing(c, nullptr, nullptr);  // drain pending events
  if (rc) return rc;
  c->pass_timing = enable != 0;
  c->timed_ms = 0.0;
  c->timed_launches = 0;
  return GBQ_OK;
}

int gbq_alloc(gbq_ctx* c, size_t bytes, void** dptr) {
  CHECK_CTX(c);
  if (!dptr) return arg_fail("null output pointer");
  cudaError_t e = cudaMalloc(dptr, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *dptr = nullptr;
    return cuda_fail(e, "cudaMalloc");
  }
  return GBQ_OK;
}

int gbq_free(gbq_ctx* c, void* dptr) {
  CHECK_CTX(c);
  if (!dptr) return GBQ_OK;
  cudaStreamSynchronize(c->stream);
  cudaError_t e = cudaFree(dptr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree");
  return GBQ_OK;
}

// Large pinned buffers are 2 MiB-aligned host memory advised for
// transparent huge pages, each huge page touched once, then registered with
// cudaHostRegister.  Measured on a GB300 host whose memory earlier processes
// had used: 8 GiB device-to-host copies into cudaMallocHost memory took
// 0.27-0.34 s in three of four tries, into this memory 0.0445 s every time
// (the same as either on a fresh host).  Anything that fails falls back to
// cudaMallocHost.
static std::mutex g_host_mu;
static std::unordered_map<void*, size_t> g_host_registered;
static constexpr size_t kHugePage = 2u << 20;
static constexpr size_t kHugeMin = 4u << 20;

static void* host_alloc_huge(size_t n) {
  const size_t len = (n + kHugePage - 1) & ~(kHugePage - 1);
  void* p = nullptr;
  if (posix_memalign(&p, kHugePage, len) != 0) return nullptr;
  madvise(p, len, MADV_HUGEPAGE);  // advisory; small pages where none is free
  for (size_t off = 0; off < len; off += kHugePage) static_cast<volatile char*>(p)[off] = 0;
  if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    free(p);
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_host_mu);
  g_host_registered[p] = len;
  return p;
}

int gbq_host_alloc(size_t bytes, void** hptr) {
  if (!hptr) return arg_fail("null output pointer");
  const size_t n = bytes ? bytes : 16;
  if (n >= kHugeMin) {
    *hptr = host_alloc_huge(n);
    if (*hptr) return GBQ_OK;
  }
  cudaError_t e = cudaMallocHost(hptr, n);
  if (e != cudaSuccess) {
    *hptr = nullptr;
    return cuda_fail(e, "cudaMallocHost");
  }
  return GBQ_OK;
}

int gbq_host_free(void* hptr) {
  if (!hptr) return GBQ_OK;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    auto it = g_host_registered.find(hptr);
    if (it != g_host_registered.end()) {
      g_host_registered.erase(it);
      cudaError_t e = cudaHostUnregister(hptr);
      free(hptr);
      if (e != cudaSuccess) return cuda_fail(e, "cudaHostUnregister");
      return GBQ_OK;
    }
  }
  cudaError_t e = cudaFreeHost(hptr);
  if (e != cudaSuccess) return cuda_fail(e, "cudaFreeHost");
  return GBQ_OK;
}

int gbq_h2d(gbq_ctx* c, void* dst, const void* src, size_t bytes) {
  CHECK_CTX(c);
  if (!bytes) return GBQ_OK;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(H2D)");
  // the caller may free or reuse `src` as soon as we return
  return sync(c, "gbq_h2d");
}

int gbq_d2h(gbq_ctx* c, void* dst, const void* src, size_t bytes) {
  CHECK_CTX(c);
  if (!bytes) return GBQ_OK;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(D2H)");
  return sync(c, "gbq_d2h");
}

int gbq_sv_set_basis(gbq_ctx* c, gbq_c64* state, int nbits, uint64_t index) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_set_basis: bad state");
  if (nbits < 64 && index >= (1ull << nbits)) return arg_fail("gbq_sv_set_basis: index out of range");
  return do_set_basis(c, reinterpret_cast<float2*>(state), nbits, index);
}

int gbq_validate_program(int nbits, const gbq_pass* passes, int npasses, const gbq_op* ops,
                         int nops, int dual) {
  if (nbits < 1 || nbits > 40) return arg_fail("gbq_validate_program: bad width");
  if (npasses < 0 || (npasses && (!passes || !ops))) return arg_fail("gbq_validate_program: null program");
  PassArgs* a = new PassArgs();
  MmaArgs* ma = new MmaArgs();
  TcArgs* ta = new TcArgs();
  int rc = GBQ_OK;
  for (int q = 0; q < npasses && rc == GBQ_OK; ++q) {
    int mma = 0;
    rc = convert_pass(passes[q], ops, nops, nbits, dual != 0, *a, *ma, *ta, mma);
  }
  delete a;
  delete ma;
  delete ta;
  return rc;
}

struct gbq_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
  int64_t launches = 0;  // kernels per replay
};

int gbq_graph_create(gbq_ctx* c, gbq_c64* state, int nbits, const gbq_pass* passes,
                     int npasses, const gbq_op* ops, int nops, const gbq_c64* mats,
                     gbq_graph** out) {
  CHECK_CTX(c);
  if (!out) return arg_fail("gbq_graph_create: null output");
  if (!state || nbits < 1 || nbits > 40) return arg_fail("gbq_graph_create: bad state");
  if (npasses < 0 || (npasses && (!passes || !ops || !mats))) return arg_fail("gbq_graph_create: null program");
  // validate (and set kernel attributes) before capturing
  int rc = gbq_validate_program(nbits, passes, npasses, ops, nops, 0);
  if (rc) return rc;
  const bool timing = c->pass_timing;
  c->pass_timing = false;
  const int64_t l0 = c->launches;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    c->pass_timing = timing;
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  rc = run_passes(c, reinterpret_cast<float2*>(state), nullptr, nbits, passes, npasses, ops, nops,
                  reinterpret_cast<const float2*>(mats), nullptr);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(c->stream, &g);
  c->pass_timing = timing;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  gbq_graph* gr = new gbq_graph();
  gr->graph = g;
  gr->exec = x;
  gr->device = c->device;
  gr->launches = c->launches - l0;
  c->launches = l0;  // captured, not launched
  *out = gr;
  return GBQ_OK;
}

int gbq_graph_launch(gbq_ctx* c, gbq_graph* g) {
  CHECK_CTX(c);
  if (!g || !g->exec) return arg_fail("gbq_graph_launch: null graph");
  if (g->device != c->device) return arg_fail("gbq_graph_launch: graph belongs to another device");
  cudaError_t e = cudaGraphLaunch(g->exec, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  c->launches += g->launches;
  return GBQ_OK;
}

int gbq_graph_destroy(gbq_graph* g) {
  if (!g) return GBQ_OK;
  cudaSetDevice(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return GBQ_OK;
}

int gbq_run(gbq_ctx* c, gbq_c64* state, int nbits, const gbq_pass* passes, int npasses,
            const gbq_op* ops, int nops, const gbq_c64* mats) {
  CHECK_CTX(c);
  if (!state || nbits < 1 || nbits > 40) return arg_fail("gbq_run: bad state");
  if (npasses < 0 || (npasses && (!passes || !ops || !mats))) return arg_fail("gbq_run: null program");
  return run_passes(c, reinterpret_cast<float2*>(state), nullptr, nbits, passes, npasses, ops, nops,
                    reinterpret_cast<const float2*>(mats), nullptr);
}

int gbq_run_dual(gbq_ctx* c, gbq_c64* psi, gbq_c64* lam, int nbits, const gbq_pass* passes,
                 int npasses, const gbq_op* ops, int nops, const gbq_c64* mats, double* partial) {
  CHECK_CTX(c);
  if (!psi || !lam || nbits < 1 || nbits > 40) return arg_fail("gbq_run_dual: bad states");
  if (npasses < 0 || (npasses && (!passes || !ops || !mats))) return arg_fail("gbq_run_dual: null program");
  for (int q = 0; q < npasses; ++q)
    for (int o = 0; o < passes[q].op_count; ++o) {
      const int idx = passes[q].op_begin + o;
      if (idx < 0 || idx >= nops) return arg_fail("gbq_run_dual: op index out of range");
      const int k = ops[idx].kind;
      if ((k == GBQ_OP_PROBE || k == GBQ_OP_PROBE_DIAG) && !partial)
        return arg_fail("gbq_run_dual: probe ops need a partial buffer");
    }
  return run_passes(c, reinterpret_cast<float2*>(psi), reinterpret_cast<float2*>(lam), nbits,
                    passes, npasses, ops, nops, reinterpret_cast<const float2*>(mats), partial);
}

int gbq_adjoint(gbq_ctx* c, int nq, int nbits, const gbq_pass* fpasses, int nfpasses, const gbq_op* fops,
                int nfops, const gbq_c64* fmats, const gbq_pauli* terms, int nterms, const gbq_pass* rpasses,
                int nrpasses, const gbq_op* rops, int nrops, const gbq_c64* rmats, int nslots, double* value,
                double* slot_values) {
  CHECK_CTX(c);
  if (nq < 1 || nbits < nq || nbits > 36 || !value || nslots < 0 || (nslots && !slot_values))
    return arg_fail("gbq_adjoint: bad arguments");
  if (nfpasses < 0 || (nfpasses && (!fpasses || !fops || !fmats))) return arg_fail("gbq_adjoint: null forward program");
  if (nrpasses < 0 || (nrpasses && (!rpasses || !rops || !rmats))) return arg_fail("gbq_adjoint: null reverse program");
  int rc = gbq_validate_program(nbits, fpasses, nfpasses, fops, nfops, 0);
  if (rc) return rc;
  rc = gbq_validate_program(nbits, rpasses, nrpasses, rops, nrops, 1);
  if (rc) return rc;
  int rl = 0;
  for (int q = 0; q < nrpasses; ++q) {
    if (rl && rpasses[q].L != rl) return arg_fail("gbq_adjoint: reverse passes must share one tile width");
    rl = rpasses[q].L;
  }
  for (int q = 0; q < nrpasses; ++q)
    for (int o = 0; o < rpasses[q].op_count; ++o) {
      const gbq_op& op = rops[rpasses[q].op_begin + o];
      const bool probe = op.kind == GBQ_OP_PROBE || op.kind == GBQ_OP_PROBE_DIAG || op.kind == GBQ_OP_RPROBE ||
                         op.kind == GBQ_OP_RPROBE_DIAG;
      if (probe && (op.slot < 0 || op.slot >= nslots)) return arg_fail("gbq_adjoint: probe slot out of range");
    }
  const int64_t ntiles = rl ? (int64_t)1 << (nbits - rl) : 1;
  const size_t sbytes = (size_t)8 << nbits;
  const size_t pbytes = (size_t)8 * (nslots ? nslots : 1) * ntiles;
  float2 *psi = nullptr, *lam = nullptr;
  double *partial = nullptr, *d_slots = nullptr;
  auto release = [&]() {
    cudaStreamSynchronize(c->stream);
    cudaFree(psi);
    cudaFree(lam);
    cudaFree(partial);
    cudaFree(d_slots);
  };
  cudaError_t e = cudaMalloc(&psi, sbytes);
  if (e == cudaSuccess) e = cudaMalloc(&lam, sbytes);
  if (e == cudaSuccess) e = cudaMalloc(&partial, pbytes);
  if (e == cudaSuccess) e = cudaMalloc(&d_slots, 8 * (size_t)(nslots ? nslots : 1));
  if (e != cudaSuccess) {
    release();
    return cuda_fail(e, "gbq_adjoint: cudaMalloc");
  }
  // forward: psi = U(theta)|0>, lam = H psi (padding amplitudes stay zero), E = <psi|lam>
  rc = do_set_basis(c, psi, nbits, 0);
  if (!rc && nfpasses)
    rc = run_passes(c, psi, nullptr, nbits, fpasses, nfpasses, fops, nfops, reinterpret_cast<const float2*>(fmats),
                    nullptr);
  if (!rc) {
    e = cudaMemsetAsync(lam, 0, sbytes, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "gbq_adjoint: cudaMemsetAsync");
  }
  if (!rc)
    rc = gbq_sv_apply_paulisum(c, reinterpret_cast<const gbq_c64*>(psi), nq, terms, nterms,
                               reinterpret_cast<gbq_c64*>(lam));
  double ip[2] = {0.0, 0.0};
  if (!rc) rc = gbq_sv_inner(c, reinterpret_cast<const gbq_c64*>(psi), reinterpret_cast<const gbq_c64*>(lam), nq, ip);
  // reverse sweep: probes add Re<lam|D|psi> per slot
  if (!rc && nrpasses)
    rc = run_passes(c, psi, lam, nbits, rpasses, nrpasses, rops, nrops, reinterpret_cast<const float2*>(rmats),
                    partial);
  if (!rc && nslots) rc = do_reduce_slots(c, partial, nslots, ntiles, d_slots);
  if (!rc && nslots) {
    e = cudaMemcpyAsync(slot_values, d_slots, 8 * (size_t)nslots, cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "gbq_adjoint: cudaMemcpyAsync");
  }
  if (!rc) rc = sync(c, "gbq_adjoint");
  release();
  if (!rc) *value = ip[0];
  return rc;
}

int gbq_reduce_slots(gbq_ctx* c, const double* partial, int nslots, int64_t ntiles, double* out) {
  CHECK_CTX(c);
  if (nslots <= 0) return GBQ_OK;
  if (!partial || !out || ntiles < 1) return arg_fail("gbq_reduce_slots: bad arguments");
  return do_reduce_slots(c, partial, nslots, ntiles, out);
}

int gbq_sv_norm2(gbq_ctx* c, const gbq_c64* state, int nbits, double* out) {
  CHECK_CTX(c);
  if (!state || !out || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_norm2: bad arguments");
  int rc = ensure_scratch(c, 64);
  if (rc) return rc;
  double* d = reinterpret_cast<double*>(c->scratch);
  rc = do_norm2(c, reinterpret_cast<const float2*>(state), nbits, 1.f, 0, d);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(out, d, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  return sync(c, "gbq_sv_norm2");
}

int gbq_sv_scale(gbq_ctx* c, gbq_c64* state, int nbits, float scale) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_scale: bad arguments");
  return do_scale(c, reinterpret_cast<float2*>(state), nbits, scale);
}

int gbq_sv_project(gbq_ctx* c, gbq_c64* state, int nbits, uint64_t mask, uint64_t value,
                   float scale) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_project: bad arguments");
  return do_project(c, reinterpret_cast<float2*>(state), nbits, mask, value, scale);
}

int gbq_sv_final_renormalize(gbq_ctx* c, gbq_c64* state, int nbits, int* applied, double* norm_out) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_final_renormalize: bad arguments");
  if (applied) *applied = 0;
  double n2 = 0.0;
  int rc = gbq_sv_norm2(c, state, nbits, &n2);
  if (rc) return rc;
  const double norm = sqrt(n2);
  if (norm_out) *norm_out = norm;
  const double tol = 3.4526698e-4;  // sqrt(float32 eps), the reference's threshold
  if (fabs(norm - 1.0) > tol || norm == 0.0) return GBQ_OK;
  const float inv = (float)(1.0 / norm);
  double* d = reinterpret_cast<double*>(c->scratch);
  rc = do_norm2(c, reinterpret_cast<const float2*>(state), nbits, inv, 1, d);
  if (rc) return rc;
  double n2s = 0.0;
  cudaError_t e = cudaMemcpyAsync(&n2s, d, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  rc = sync(c, "gbq_sv_final_renormalize");
  if (rc) return rc;
  if (fabs(n2s - 1.0) - fabs(n2 - 1.0) < 0) {
    rc = do_scale(c, reinterpret_cast<float2*>(state), nbits, inv);
    if (rc) return rc;
    if (applied) *applied = 1;
  }
  return GBQ_OK;
}

int gbq_probabilities(gbq_ctx* c, const gbq_c64* state, int nbits, int dm, float* out) {
  CHECK_CTX(c);
  if (!state || !out || nbits < 0 || nbits > 40) return arg_fail("gbq_probabilities: bad arguments");
  return do_probs(c, reinterpret_cast<const float2*>(state), nbits, dm, out);
}

int gbq_sample(gbq_ctx* c, const gbq_c64* state, int nbits, int dm, const double* u, int64_t R,
               uint64_t* out) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40 || R < 0 || (R && (!u || !out)))
    return arg_fail("gbq_sample: bad arguments");
  if (R == 0) return GBQ_OK;
  const int bbits = nbits < 12 ? nbits : 12;
  const int64_t nblocks = (int64_t)1 << (nbits - bbits);
  const size_t need = (size_t)nblocks * 8 + (size_t)R * 8 + (size_t)R * 8 + 256;
  int rc = ensure_scratch(c, need);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  double* d_cdf = reinterpret_cast<double*>(base);
  double* d_u = reinterpret_cast<double*>(base + (size_t)nblocks * 8);
  uint64_t* d_out = reinterpret_cast<uint64_t*>(base + (size_t)nblocks * 8 + (size_t)R * 8);
  cudaError_t e = cudaMemcpyAsync(d_u, u, (size_t)R * 8, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(uniforms)");
  rc = do_sample(c, reinterpret_cast<const float2*>(state), nbits, dm, d_u, R, d_out, d_cdf);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, (size_t)R * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(samples)");
  return sync(c, "gbq_sample");
}

static int validate_terms(const gbq_pauli* terms, int nterms, int nbits) {
  if (nterms < 0 || (nterms && !terms)) return arg_fail("pauli terms: bad arguments");
  const uint64_t mask = nbits >= 64 ? ~0ull : ((1ull << nbits) - 1ull);
  for (int t = 0; t < nterms; ++t)
    if ((terms[t].x & ~mask) || (terms[t].zy & ~mask))
      return arg_fail("pauli term acts on a qubit outside the state");
  return GBQ_OK;
}

int gbq_sv_expect_paulis(gbq_ctx* c, const gbq_c64* state, int nbits, const gbq_pauli* terms,
                         int nterms, double* out) {
  CHECK_CTX(c);
  if (!state || nbits < 0 || nbits > 40 || (nterms && !out)) return arg_fail("gbq_sv_expect_paulis: bad arguments");
  int rc = validate_terms(terms, nterms, nbits);
  if (rc || nterms == 0) return rc;
  const int cbits = expect_chunk_bits(nbits);
  const int64_t nchunks = (int64_t)1 << (nbits - cbits);
  const size_t tbytes = (size_t)nterms * sizeof(gbq_pauli);
  const size_t pbytes = (size_t)nterms * nchunks * 2 * sizeof(double);
  const size_t obytes = (size_t)nterms * 2 * sizeof(double);
  rc = ensure_scratch(c, tbytes + pbytes + obytes + 512);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  gbq_pauli* d_terms = reinterpret_cast<gbq_pauli*>(base);
  double* d_partial = reinterpret_cast<double*>(base + ((tbytes + 255) & ~(size_t)255));
  double* d_out = reinterpret_cast<double*>(base + ((tbytes + 255) & ~(size_t)255) + pbytes);
  cudaError_t e = cudaMemcpyAsync(d_terms, terms, tbytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(terms)");
  rc = do_expect(c, reinterpret_cast<const float2*>(state), nbits, d_terms, nterms, d_partial, d_out);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, obytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(expectations)");
  rc = sync(c, "gbq_sv_expect_paulis");
  if (rc) return rc;
  for (int t = 0; t < nterms; ++t) {
    // multiply by coef * i^ny
    double re = out[2 * t], im = out[2 * t + 1];
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

int gbq_dm_expect_paulis(gbq_ctx* c, const gbq_c64* rho, int nbits, const gbq_pauli* terms,
                         int nterms, double* out) {
  CHECK_CTX(c);
  if (!rho || nbits < 0 || nbits > 20 || (nterms && !out)) return arg_fail("gbq_dm_expect_paulis: bad arguments");
  int rc = validate_terms(terms, nterms, nbits);
  if (rc || nterms == 0) return rc;
  const int chunks = dm_expect_chunks(c, nbits);
  const size_t tbytes = (size_t)nterms * sizeof(gbq_pauli);
  const size_t pbytes = (size_t)nterms * chunks * 2 * sizeof(double);
  const size_t obytes = (size_t)nterms * 2 * sizeof(double);
  rc = ensure_scratch(c, tbytes + pbytes + obytes + 512);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  gbq_pauli* d_terms = reinterpret_cast<gbq_pauli*>(base);
  double* d_partial = reinterpret_cast<double*>(base + ((tbytes + 255) & ~(size_t)255));
  double* d_out = reinterpret_cast<double*>(base + ((tbytes + 255) & ~(size_t)255) + pbytes);
  cudaError_t e = cudaMemcpyAsync(d_terms, terms, tbytes, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(terms)");
  rc = do_dm_expect(c, reinterpret_cast<const float2*>(rho), nbits, d_terms, nterms, d_partial, d_out);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, obytes, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(expectations)");
  rc = sync(c, "gbq_dm_expect_paulis");
  if (rc) return rc;
  for (int t = 0; t < nterms; ++t) {
    double re = out[2 * t], im = out[2 * t + 1];
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

int gbq_sv_apply_paulisum(gbq_ctx* c, const gbq_c64* psi, int nbits, const gbq_pauli* terms,
                          int nterms, gbq_c64* out) {
  CHECK_CTX(c);
  if (!psi || !out || psi == out || nbits < 0 || nbits > 40)
    return arg_fail("gbq_sv_apply_paulisum: bad arguments (out must differ from psi)");
  int rc = validate_terms(terms, nterms, nbits);
  if (rc) return rc;
  rc = apply_paulisum(c, reinterpret_cast<const float2*>(psi), nbits, terms, nterms, reinterpret_cast<float2*>(out));
  if (rc) return rc;
  // the term tables live in the shared scratch buffers: finish before they can be reused
  return sync(c, "gbq_sv_apply_paulisum");
}

int gbq_paulisum_cover(const gbq_pauli* terms, int nterms, int nbits, int* npasses, int* nwide, int* pass_terms,
                       int max_passes) {
  if (!npasses || !nwide || nbits < 0 || nbits > 40 || max_passes < 0 || (max_passes && !pass_terms))
    return arg_fail("gbq_paulisum_cover: bad arguments");
  const int rc = validate_terms(terms, nterms, nbits);
  if (rc) return rc;
  return paulisum_cover_stats(terms, nterms, nbits, npasses, nwide, pass_terms, max_passes);
}

int gbq_points_set_zero(gbq_ctx* c, gbq_c64* states, int nbits, int npoints) {
  CHECK_CTX(c);
  if (!states || nbits < 1 || nbits > 34 || npoints < 1) return arg_fail("gbq_points_set_zero: bad arguments");
  return points_set_zero(c, reinterpret_cast<float2*>(states), nbits, npoints);
}

int gbq_run_points(gbq_ctx* c, gbq_c64* states, int nbits, int npoints, const gbq_pass* passes, int npasses,
                   const gbq_op* ops, int nops, const gbq_c64* mats, int64_t pool_stride) {
  CHECK_CTX(c);
  if (!states || nbits < 1 || nbits > 34 || npoints < 1) return arg_fail("gbq_run_points: bad states");
  if (npasses < 0 || (npasses && (!passes || !ops || !mats))) return arg_fail("gbq_run_points: null program");
  if (pool_stride < 0 || (pool_stride & 1)) return arg_fail("gbq_run_points: pool_stride must be even and >= 0");
  int pbits = 0;
  while ((1 << pbits) < npoints) ++pbits;
  PassArgs a;
  MmaArgs ma;
  TcArgs ta;
  for (int q = 0; q < npasses; ++q) {
    int mma = 0;
    int rc = convert_pass(passes[q], ops, nops, nbits, false, a, ma, ta, mma);
    if (rc) return rc;
    if (mma) return arg_fail("gbq_run_points: tensor-core passes run on one state only");
    const int L = passes[q].L;
    if (((int64_t)npoints << (nbits - L)) > ((int64_t)1 << 24))
      return arg_fail("gbq_run_points: more than 2^24 tiles per pass; split the points");
    // widen the pass to the index space of all points: the point index is
    // the top global bits, above the state's own nbits
    const int nnt = nbits - L;
    for (int b = 0; b < pbits; ++b) a.ti.nt[nnt + b] = (int8_t)(nbits + b);
    a.ti.nbits = nbits + pbits;
    a.ti.ntiles = (int64_t)npoints << nnt;
    a.ti.pshift = nbits;
    a.ti.pstride = pool_stride;
    a.ti.mats = reinterpret_cast<const float2*>(mats);
    a.ti.partial = nullptr;
    a.psi = reinterpret_cast<float2*>(states);
    a.lam = nullptr;
    a.abort = c->d_abort;
    c->abort_armed = true;
    rc = launch_pass(c, a, false);
    if (rc) return rc;
  }
  return GBQ_OK;
}

int gbq_points_rdm(gbq_ctx* c, const gbq_c64* states, int nbits, int npoints, int k, const int* bits,
                   double* out) {
  CHECK_CTX(c);
  if (!states || nbits < 2 || nbits > 34 || npoints < 1 || npoints > 65535 || k < 1 || k > 2 || !bits || !out)
    return arg_fail("gbq_points_rdm: bad arguments");
  for (int q = 0; q < k; ++q)
    if (bits[q] < 0 || bits[q] >= nbits) return arg_fail("gbq_points_rdm: bit out of range");
  if (k == 2 && bits[0] == bits[1]) return arg_fail("gbq_points_rdm: bits must differ");
  const size_t b = (size_t)npoints * (1u << (2 * k)) * 2 * sizeof(double);
  int rc = ensure_scratch(c, b);
  if (rc) return rc;
  double* d_out = reinterpret_cast<double*>(c->scratch);
  rc = points_rdm(c, reinterpret_cast<const float2*>(states), nbits, npoints, k, bits, d_out);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(out, d_out, b, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(rdm)");
  return sync(c, "gbq_points_rdm");
}

int gbq_points_dm_marginal(gbq_ctx* c, const gbq_c64* states, int nbits, int nq, int npoints, int m,
                           const int* bits, double* out) {
  CHECK_CTX(c);
  if (!states || nq < 1 || 2 * nq > nbits || nbits > 34 || npoints < 1 || npoints > 65535 || m < 1 || m > 5 ||
      !bits || !out)
    return arg_fail("gbq_points_dm_marginal: bad arguments");
  for (int j = 0; j < m; ++j)
    if (bits[j] < 0 || bits[j] >= nq) return arg_fail("gbq_points_dm_marginal: bit out of range");
  const size_t b = (size_t)npoints * (1u << m) * sizeof(double);
  int rc = ensure_scratch(c, b);
  if (rc) return rc;
  double* d_out = reinterpret_cast<double*>(c->scratch);
  rc = points_dm_marginal(c, reinterpret_cast<const float2*>(states), nbits, nq, npoints, m, bits, d_out);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(out, d_out, b, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(marginal)");
  return sync(c, "gbq_points_dm_marginal");
}

int gbq_points_sample(gbq_ctx* c, const gbq_c64* states, int nbits, int npoints, const double* u,
                      uint64_t* out) {
  CHECK_CTX(c);
  if (!states || nbits < 1 || nbits > 34 || npoints < 1 || !u || !out)
    return arg_fail("gbq_points_sample: bad arguments");
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b = al((size_t)npoints * 8);
  int rc = ensure_scratch(c, 2 * b);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  double* d_u = reinterpret_cast<double*>(base);
  unsigned long long* d_out = reinterpret_cast<unsigned long long*>(base + b);
  cudaError_t e = cudaMemcpyAsync(d_u, u, (size_t)npoints * 8, cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(u)");
  rc = points_sample(c, reinterpret_cast<const float2*>(states), nbits, npoints, d_u, d_out);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, (size_t)npoints * 8, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(out)");
  return sync(c, "gbq_points_sample");
}

int gbq_points_expect(gbq_ctx* c, const gbq_c64* states, int nbits, int npoints, const gbq_pauli* terms,
                      int nterms, double* out) {
  CHECK_CTX(c);
  if (!states || nbits < 1 || nbits > 34 || npoints < 1 || npoints > 65535 || nterms < 0 ||
      (nterms && (!terms || !out)))
    return arg_fail("gbq_points_expect: bad arguments");
  if (nterms == 0) return GBQ_OK;
  int rc = validate_terms(terms, nterms, nbits);
  if (rc) return rc;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_terms = al((size_t)nterms * sizeof(gbq_pauli));
  const size_t b_out = (size_t)npoints * nterms * 2 * sizeof(double);
  rc = ensure_scratch(c, b_terms + b_out);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  gbq_pauli* d_terms = reinterpret_cast<gbq_pauli*>(base);
  double* d_out = reinterpret_cast<double*>(base + b_terms);
  cudaError_t e = cudaMemcpyAsync(d_terms, terms, (size_t)nterms * sizeof(gbq_pauli), cudaMemcpyHostToDevice,
                                  c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(terms)");
  rc = points_expect(c, reinterpret_cast<const float2*>(states), nbits, npoints, d_terms, nterms, d_out);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(out)");
  return sync(c, "gbq_points_expect");
}

int gbq_sv_inner(gbq_ctx* c, const gbq_c64* a, const gbq_c64* b, int nbits, double* out) {
  CHECK_CTX(c);
  if (!a || !b || !out || nbits < 0 || nbits > 40) return arg_fail("gbq_sv_inner: bad arguments");
  int rc = ensure_scratch(c, 64);
  if (rc) return rc;
  double* d = reinterpret_cast<double*>(c->scratch);
  rc = do_inner(c, reinterpret_cast<const float2*>(a), reinterpret_cast<const float2*>(b), nbits, d);
  if (rc) return rc;
  cudaError_t e = cudaMemcpyAsync(out, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
  return sync(c, "gbq_sv_inner");
}

int gbq_batch_expect(gbq_ctx* c, const gbq_point* points, int npoints, const gbq_pass* passes,
                     int npasses, const gbq_op* ops, int nops, const gbq_c64* mats,
                     const gbq_pauli* terms, int nterms, int max_nbits, double* out) {
  CHECK_CTX(c);
  if (npoints < 0 || (npoints && (!points || !out))) return arg_fail("gbq_batch_expect: bad arguments");
  if (npoints == 0) return GBQ_OK;
  if (max_nbits < 1 || max_nbits > 30) return arg_fail("gbq_batch_expect: max_nbits out of range (1..30)");
  if (!mats) return arg_fail("gbq_batch_expect: null matrix pool");
  // validate every point's program on the host and convert each pass's ops
  std::vector<OpDev> dops((size_t)(nops ? nops : 1));
  int smem_kmax = 0;  // widest shared-memory dense op (0: register phases only)
  std::vector<char> converted((size_t)(npasses ? npasses : 1), 0);
  TileInfo ti;
  for (int p = 0; p < npoints; ++p) {
    const gbq_point& pt = points[p];
    if (pt.nbits < 12 || pt.nbits > max_nbits)
      return arg_fail("gbq_batch_expect: point width out of range (12 <= nbits <= max_nbits)");
    if (pt.pass_begin < 0 || pt.pass_count < 0 || pt.pass_begin + pt.pass_count > npasses)
      return arg_fail("gbq_batch_expect: point passes out of range");
    if (pt.term_begin < 0 || pt.term_count < 0 || pt.term_begin + pt.term_count > nterms)
      return arg_fail("gbq_batch_expect: point terms out of range");
    if (pt.mat_base < 0 || (pt.mat_base & 1)) return arg_fail("gbq_batch_expect: mat_base must be even");
    for (int q = 0; q < pt.pass_count; ++q) {
      const gbq_pass& ps = passes[pt.pass_begin + q];
      if (ps.L != 12) return arg_fail("gbq_batch_expect: batch passes must use 12-bit tiles");
      uint64_t inmask = 0;
      int rc = pass_geometry(ps, nops, pt.nbits, ti, inmask);
      if (rc) return rc;
      LayoutState lay;
      for (int o = 0; o < ps.op_count; ++o) {
        OpDev d;
        rc = convert_op(ops[ps.op_begin + o], ps.L, pt.nbits, inmask, false, d, lay);
        if (rc) return rc;
        if (!converted[pt.pass_begin + q]) dops[ps.op_begin + o] = d;
        if ((d.kind == GBQ_OP_DENSE || d.kind == GBQ_OP_PROBE) && d.k > smem_kmax) smem_kmax = d.k;
      }
      converted[pt.pass_begin + q] = 1;
    }
    int rc = validate_terms(terms + pt.term_begin, pt.term_count, pt.nbits);
    if (rc) return rc;
  }
  int nslots = c->sm_count * 2;
  if (nslots > npoints) nslots = npoints;
  const size_t slot_bytes = ((size_t)1 << max_nbits) * sizeof(float2);
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_points = al((size_t)npoints * sizeof(gbq_point));
  const size_t b_passes = al((size_t)(npasses ? npasses : 1) * sizeof(gbq_pass));
  const size_t b_ops = al((size_t)(nops ? nops : 1) * sizeof(OpDev));
  const size_t b_terms = al((size_t)(nterms ? nterms : 1) * sizeof(gbq_pauli));
  const size_t b_out = al((size_t)(nterms ? nterms : 1) * 2 * sizeof(double));
  const size_t b_counter = 256;
  const size_t head = b_points + b_passes + b_ops + b_terms + b_out + b_counter;
  int rc = ensure_scratch(c, head + slot_bytes * nslots);
  if (rc) return rc;
  char* base = reinterpret_cast<char*>(c->scratch);
  gbq_point* d_points = reinterpret_cast<gbq_point*>(base);
  gbq_pass* d_passes = reinterpret_cast<gbq_pass*>(base + b_points);
  OpDev* d_ops = reinterpret_cast<OpDev*>(base + b_points + b_passes);
  gbq_pauli* d_terms = reinterpret_cast<gbq_pauli*>(base + b_points + b_passes + b_ops);
  double* d_out = reinterpret_cast<double*>(base + b_points + b_passes + b_ops + b_terms);
  int* d_counter = reinterpret_cast<int*>(base + b_points + b_passes + b_ops + b_terms + b_out);
  float2* slots = reinterpret_cast<float2*>(base + head);
  cudaError_t e;
  e = cudaMemcpyAsync(d_points, points, (size_t)npoints * sizeof(gbq_point), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(points)");
  if (npasses) {
    e = cudaMemcpyAsync(d_passes, passes, (size_t)npasses * sizeof(gbq_pass), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(passes)");
  }
  if (nops) {
    e = cudaMemcpyAsync(d_ops, dops.data(), (size_t)nops * sizeof(OpDev), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(ops)");
  }
  if (nterms) {
    e = cudaMemcpyAsync(d_terms, terms, (size_t)nterms * sizeof(gbq_pauli), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(terms)");
  }
  e = cudaMemsetAsync(d_counter, 0, sizeof(int), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(counter)");
  e = cudaMemsetAsync(d_out, 0, (size_t)(nterms ? nterms : 1) * 2 * sizeof(double), c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(out)");
  rc = launch_batch(c, d_points, npoints, d_passes, d_ops, reinterpret_cast<const float2*>(mats),
                    d_terms, max_nbits, slots, nslots, d_counter, d_out, smem_kmax);
  if (rc) return rc;
  e = cudaMemcpyAsync(out, d_out, (size_t)nterms * 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync(out)");
  return sync(c, "gbq_batch_expect");
}

}  // extern "C"
