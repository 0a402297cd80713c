// Internal declarations shared by the CUDA translation units of cirq_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/cirq_gb300.h"

namespace gbq {

constexpr int kThreads = 512;  // threads per tile CTA (16 warps)

// Tile geometry of one pass (shared by the per-pass and the batch kernels).
struct TileInfo {
  const float2* mats;     // matrix / table pool (op.mat is relative to it)
  double* partial;        // probe partials [slot][tile]
  int64_t ntiles;         // 2^(nbits - L)
  int32_t nbits;
  int32_t L;
  int32_t m;
  int32_t nops;
  int8_t hi[16];          // global bit of tile bit m + j
  int8_t nt[64];          // global bits NOT in the tile, ascending (nbits - L entries)
};

// Kernel arguments of one tile pass, passed by value (__grid_constant__).
struct PassArgs {
  float2* psi;
  float2* lam;            // second state (two-state passes only)
  TileInfo ti;
  gbq_op ops[GBQ_MAX_OPS_PER_PASS];
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
  // scratch buffers owned by the context (grown on demand)
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  void* host_scratch = nullptr;  // pinned
  size_t host_scratch_bytes = 0;
  cudaEvent_t events[16] = {};
  // per-launch tile-pass timing
  bool pass_timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> timed;  // pending (start, stop)
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> event_pool;
  double timed_ms = 0.0;
  int64_t timed_launches = 0;
};

int ensure_scratch(Ctx* c, size_t bytes);
int ensure_host_scratch(Ctx* c, size_t bytes);

// Launchers implemented in the .cu files.
int launch_pass(Ctx* c, const PassArgs& a, bool dual);
int launch_batch(Ctx* c, const gbq_point* d_points, int npoints, const gbq_pass* d_passes,
                 const gbq_op* d_ops, const float2* mats, const gbq_pauli* d_terms, int max_nbits,
                 float2* slots, int nslots, int* d_counter, double* d_out);

}  // namespace gbq

struct gbq_ctx : gbq::Ctx {};
