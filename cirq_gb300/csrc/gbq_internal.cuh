// Internal declarations shared by the CUDA translation units of cirq_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/cirq_gb300.h"

namespace gbq {

constexpr int kThreads = 256;  // threads per tile CTA (8 warps)
constexpr int kMinTile = GBQ_MIN_TILE_BITS;
constexpr int kMaxTile = GBQ_MAX_TILE_BITS;

// ---- shared-memory swizzle ------------------------------------------------------
// Tile amplitude i is stored at phys(i) = i ^ swz(i).  swz XORs one 4-bit
// column vector per tile bit >= 4 into bits 0..3; the columns below are
// distinct, nonzero and not unit vectors, so for any op there are 4 group
// bits whose columns (together with the unit columns of tile bits 0..3) are
// independent -- a half-warp spread over them hits 16 distinct bank pairs.
constexpr uint32_t kSwzV[10] = {3, 5, 6, 9, 10, 12, 7, 11, 13, 14};
__host__ __device__ constexpr uint32_t swz_row(int r) {
  uint32_t m = 0;
  for (int b = 0; b < 10; ++b)
    if ((kSwzV[b] >> r) & 1) m |= 1u << (b + 4);
  return m;
}
constexpr uint32_t kSwzRow0 = swz_row(0), kSwzRow1 = swz_row(1), kSwzRow2 = swz_row(2),
                   kSwzRow3 = swz_row(3);

__host__ __device__ constexpr uint32_t parity_const(uint32_t x) {
  uint32_t p = 0;
  while (x) {
    p ^= x & 1u;
    x >>= 1;
  }
  return p;
}

// phys() for constants and host code (no intrinsics, folds at compile time)
__host__ __device__ constexpr uint32_t phys_const(uint32_t i) {
  return i ^ (parity_const(i & kSwzRow0) | (parity_const(i & kSwzRow1) << 1) |
              (parity_const(i & kSwzRow2) << 2) | (parity_const(i & kSwzRow3) << 3));
}

// Device form of one op, derived on the host from the public gbq_op.
struct OpDev {
  int8_t kind, k, nsel, rmask;  // rmask: register-op target positions
  int8_t selg[4];     // selector s: group-index bit (dense) or tile bit (register
                      // ops), >= 0; or -(global bit)-1
  uint32_t pcol[5];   // shared-index column of each target / register bit
  uint32_t gcol[13];  // shared-index column of each group-index / thread bit
  uint16_t dcol[13];  // diag: table-index contribution of each tile bit
  uint16_t tcol[8];   // layout: tile-index column of each thread bit
  int8_t dext[8];     // diag: global bit feeding table bit j, or -1
  int8_t rbits[5];    // layout: tile bit of each register position
  int8_t pad2[3];
  int32_t slot;
  int32_t pidx;       // probe: accumulator index within the pass
  int64_t mat;
};

// Tile geometry of one pass.
struct TileInfo {
  const float2* mats;  // matrix / table pool (op.mat is relative to it)
  double* partial;     // probe partials [slot][tile]
  int64_t ntiles;      // 2^(nbits - L)
  int32_t nbits;
  int32_t L;
  int32_t m;
  int32_t nops;
  uint64_t gw[GBQ_MAX_TILE_BITS];  // global weight (1 << global bit) of each tile bit
  int8_t nt[64];                   // global bits not in the tile, ascending
  // Batched points (gbq_run_points): the states of several points lie back
  // to back as one wider index space; point (global index >> pshift) uses
  // the matrices at mats + point * pstride.  pstride = 0: a single state.
  int64_t pstride;
  int32_t pshift;
  int32_t pad;
};

// Kernel arguments of one tile pass, passed by value (__grid_constant__).
struct PassArgs {
  float2* psi;
  float2* lam;  // second state (two-state passes only)
  int* abort;   // set to 1 by a pass that gave up a bounded wait
  TileInfo ti;
  OpDev ops[GBQ_MAX_OPS_PER_PASS];
};

// Tensor-core pass (gbq_mma.cu): per MMA op, the amplitude-position columns
// of its result in the next op's layout (or the final natural layout).
struct MmaOpDev {
  int64_t mat;         // pool offset of the first matrix
  uint16_t tnext[4];   // next-layout position column of target bit p
  uint16_t rnext[7];   // ... of row bit q (row bits 0..4 are the lane bits)
  int8_t nsel;
  int8_t selg[3];      // global bit of selector s
  int16_t bslot;       // first B-operand slot in shared memory
  int8_t ndiag;        // diagonal ops applied to this op's result
  int8_t diag0;
};

struct MmaDiagDev {
  int64_t mat;
  uint16_t trow[7];  // table-index bits contributed by row bit q of the MMA op
  uint16_t ttgt[4];  // ... by target bit p
  int8_t k;
  int8_t dext[8];    // table bit j <- global bit dext[j] (-1: a tile bit)
  int8_t pad[5];
};

struct MmaArgs {
  float2* psi;
  int* abort;        // set to 1 when an MMA wait gives up
  TileInfo ti;
  int32_t nops, ndiag, nmats, pad;
  uint16_t lcol[GBQ_MMA_TILE_BITS];  // position column of tile bit b in op 0's layout
  uint16_t pad2;
  MmaOpDev ops[GBQ_MAX_MMA_OPS];
  MmaDiagDev diags[GBQ_MAX_OPS_PER_PASS];
};

// Pipelined tensor-core pass (gbq_tc.cu): 12-bit tiles, 4-bit MMA ops.
struct TcOpDev {
  int64_t mat;         // pool offset of the first matrix
  uint16_t tnext[4];   // next layout's pair-index column of target bit p
  uint16_t rnext[8];   // ... of row bit q (0..4: lanes, 5..6: warps, 7: half)
  int8_t nsel;
  int8_t selg[3];      // global bit of selector s
  int16_t bslot;       // first B-operand slot in shared memory
  int8_t ndiag;        // diagonal ops applied to this op's result
  int8_t diag0;
};

struct TcDiagDev {
  int64_t mat;
  uint16_t trow[8];  // table-index bits contributed by row bit q of the MMA op
  uint16_t ttgt[4];  // ... by target bit p
  int8_t k;
  int8_t dext[8];    // table bit j <- global bit dext[j] (-1: a tile bit)
  int8_t pad[7];
};

struct TcArgs {
  float2* psi;
  int* abort;        // set to 1 when a wait gives up
  TileInfo ti;
  int32_t nops, ndiag, nmats, pad;
  uint16_t lcol[GBQ_TC_TILE_BITS];  // first op's layout pair-index column of tile bit b
  TcOpDev ops[GBQ_MAX_MMA_OPS];
  TcDiagDev diags[GBQ_MAX_OPS_PER_PASS];
};

// Error plumbing (gbq_abi.cu).
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int sm_count = 0;
  bool use_graphs = false;
  int64_t launches = 0;
  void* scratch = nullptr;  // device scratch, grown on demand
  size_t scratch_bytes = 0;
  void* host_scratch = nullptr;  // pinned
  size_t host_scratch_bytes = 0;
  cudaEvent_t events[16] = {};
  bool pass_timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;  // pending (start, stop)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> event_pool;
  double timed_ms = 0.0;
  int64_t timed_launches = 0;
  int* d_abort = nullptr;  // device flag set by a pass that gave up a bounded wait
  bool abort_armed = false;  // a kernel that can set d_abort has been launched
  // pass-specialised kernels: 0 off, 1 compiled before a program's first
  // launch, 2 compiled in the background (the interpreter runs passes whose
  // kernel is not ready); -1 not decided yet (environment variable GBQ_JIT)
  int jit = -1;
};

int ensure_scratch(Ctx* c, size_t bytes);
int ensure_host_scratch(Ctx* c, size_t bytes);

// out (+)= H psi by the per-amplitude kernel (d_terms on the device, sorted by X mask)
int do_apply_paulisum(Ctx* c, const float2* psi, int nbits, const gbq_pauli* d_terms, int nterms,
                      float2* out, int accumulate);
// out = H psi: tiled passes over a cover of the X masks (host terms; uses both scratch buffers)
int apply_paulisum(Ctx* c, const float2* psi, int nbits, const gbq_pauli* terms, int nterms, float2* out);
int paulisum_cover_stats(const gbq_pauli* terms, int nterms, int nbits, int* npasses, int* nwide,
                         int* pass_terms, int max_passes);

// Launchers (one translation unit per tile width; the 11- and 12-bit
// two-state passes, and for 12 bits those with shared-memory dense ops, have
// units of their own so the widest units compile in parallel).
int launch_pass_l10(Ctx* c, const PassArgs& a, bool dual);
int launch_pass_l11(Ctx* c, const PassArgs& a, bool dual);
int launch_pass_l11_dual(Ctx* c, const PassArgs& a);
int launch_pass_l12(Ctx* c, const PassArgs& a, bool dual);
int launch_pass_l12_dual(Ctx* c, const PassArgs& a);
int launch_pass_l12_dual_dense(Ctx* c, const PassArgs& a);
int launch_pass_l13(Ctx* c, const PassArgs& a, bool dual);
int build_mma_args(const gbq_pass& p, const gbq_op* ops, int nbits, const TileInfo& ti, uint64_t inmask,
                   MmaArgs& A);
int launch_mma_pass(Ctx* c, const MmaArgs& a);
int build_tc_args(const gbq_pass& p, const gbq_op* ops, int nbits, const TileInfo& ti, uint64_t inmask,
                  TcArgs& A);
int launch_tc_pass(Ctx* c, const TcArgs& a);
int points_set_zero(Ctx* c, float2* states, int nbits, int npoints);
// Clifford circuits (gbq_clifford.cu).
int cliff_reference(Ctx* c, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables, int ntables,
                    const int32_t* conds, int nconds, int nrec, uint8_t* ref_out);
int cliff_sample(Ctx* c, int nq, const gbq_cliff_op* ops, int nops, const int32_t* conds, int nconds,
                 const uint8_t* ref, int nrec, int64_t shots, uint64_t seed, void* out,
                 const int32_t* layers, int nlayers, int out_bytes);
int cliff_check(int nq, const gbq_cliff_op* ops, int nops, int ntables, int nconds, int nrec);

// Pass-specialised kernels (gbq_jit.cu).
constexpr int kJitAutoMinBits = 20;
bool jit_enabled(Ctx* c);
bool jit_eligible(const PassArgs& a, bool dual);
std::string jit_key(const PassArgs& a, const Ctx* c, bool dual);
std::string jit_source(const PassArgs& a, bool dual);
void jit_prepare(Ctx* c, std::vector<std::pair<std::string, PassArgs*>>& passes, bool dual, bool wait);
int jit_launch(Ctx* c, const PassArgs& a, const std::string& key, bool& launched);
int64_t jit_compile_count();
int64_t jit_launch_count();
int64_t jit_pending();
int points_rdm(Ctx* c, const float2* states, int nbits, int npoints, int k, const int* g, double* d_out);
int points_dm_marginal(Ctx* c, const float2* states, int nbits, int nq, int npoints, int m, const int* bits,
                       double* d_out);
int points_sample(Ctx* c, const float2* states, int nbits, int npoints, const double* d_u,
                  unsigned long long* d_out);
int points_expect(Ctx* c, const float2* states, int nbits, int npoints, const gbq_pauli* d_terms, int nterms,
                  double* d_out);
int launch_batch(Ctx* c, const gbq_point* d_points, int npoints, const gbq_pass* d_passes,
                 const OpDev* d_ops, const float2* mats, const gbq_pauli* d_terms, int max_nbits,
                 float2* slots, int nslots, int* d_counter, double* d_out, int kmax);

}  // namespace gbq

struct gbq_ctx : gbq::Ctx {};
