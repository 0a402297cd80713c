/*
 * cirq_gb300 -- C ABI of the GB300 (sm_103a) circuit-simulation engine.
 *
 * This is the device boundary under the Python drop-in simulators
 * (cirq_gb300.Simulator / cirq_gb300.DensityMatrixSimulator).  The reference
 * (quantumlib/Cirq) has no FFI: its simulators call numpy in-process.  Each
 * entry point below replaces one numpy site of the reference's simulation
 * path, cited as file:line relative to the Cirq repository.
 *
 * Conventions
 *  - Amplitudes are complex64 (gbq_c64, interleaved float re/im), the layout
 *    of numpy.complex64.  A state of n qubits is 2^n amplitudes; index bit b
 *    belongs to the qubit at position n-1-b of the qubit order (Cirq's
 *    big-endian order, cirq-core/cirq/sim/state_vector.py:81-112).
 *  - A density matrix of n qubits is handled as a 2n-bit vector: index
 *    row*2^n + col, exactly the reference's (2,)*2n tensor flattened
 *    (cirq-core/cirq/sim/density_matrix_simulation_state.py:178).
 *  - Every function returns 0 on success and a negative GBQ_ERR_* code on
 *    failure; gbq_last_error() then returns a message (thread-local).
 *  - All device work is ordered on the context's stream.  Functions that
 *    return host data synchronise that stream before returning.
 *  - Device pointers come from gbq_alloc; host pointers are caller-owned.
 *  - A context is not thread-safe: use one context per thread.
 */
#ifndef CIRQ_GB300_H
#define CIRQ_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBQ_OK 0
#define GBQ_ERR_ARG -1     /* invalid argument (maps to ValueError) */
#define GBQ_ERR_CUDA -2    /* CUDA runtime error */
#define GBQ_ERR_OOM -3     /* device allocation failed (maps to MemoryError) */
#define GBQ_ERR_UNSUPPORTED -4

typedef struct gbq_c64 {
  float re, im;
} gbq_c64;

typedef struct gbq_ctx gbq_ctx;

/* ---- operation program ------------------------------------------------
 * A program is a list of passes.  One pass streams the state once through
 * HBM in tiles of 2^L amplitudes: tile bits 0..m-1 are the global index bits
 * 0..m-1 (contiguous runs of 2^m amplitudes) and tile bits m..L-1 are the
 * global bits hi[0..L-m-1].  Inside a tile the pass applies its ops in
 * order.  Bit codes: a value c >= 0 names tile bit c; c < 0 names global
 * index bit (-c - 1), which is constant over one tile.
 */
#define GBQ_OP_DENSE 0      /* 2^k x 2^k matrix on k tile bits                */
#define GBQ_OP_DIAG 1       /* 2^k-entry diagonal on k bit codes               */
#define GBQ_OP_PROBE 2      /* two-state passes: Re<lam|D|psi> on k tile bits  */
#define GBQ_OP_PROBE_DIAG 3 /* two-state passes: Re<lam|diag(d)|psi>, bit codes */
/* Register phases.  A LAYOUT op makes bits[0..R-1] (R = L - 8) the
 * "register bits" of the tile: every thread then holds the 2^R amplitudes
 * that differ only in those bits in registers, and the R* ops that follow
 * act on registers without shared-memory traffic or barriers, until the
 * next LAYOUT or a plain (shared-memory) op.  R* ops compute exactly what
 * their plain counterparts compute; their extra constraints: RDENSE/RPROBE
 * targets are register bits listed in ascending register position (bits[j]
 * is register bit number <= bits[j+1]'s), selectors are not register bits. */
#define GBQ_OP_LAYOUT 4
#define GBQ_OP_RDENSE 5
#define GBQ_OP_RDIAG 6
#define GBQ_OP_RPROBE 7
#define GBQ_OP_RPROBE_DIAG 8
/* Tensor-core op: a 16 x 16 matrix on exactly 4 tile bits (bits[0..3]),
 * applied with tcgen05 MMAs in a three-term TF32 split (fp32-level
 * accuracy); selectors, if any, are global bit codes (< 0).  A pass that
 * holds an MMA op is a tensor-core pass: its first op is MMA, every other op
 * is MMA or DIAG (a DIAG applies to the result of the MMA op before it), at
 * most GBQ_MAX_MMA_OPS MMA ops; single-state runs only (gbq_run,
 * gbq_graph_create).  Two tile widths:
 *   L = GBQ_MMA_TILE_BITS (11), m >= 1: one tile at a time per CTA, MMA
 *     matrices (2^nsel each) at most GBQ_MAX_MMA_MATS per pass;
 *   L = GBQ_TC_TILE_BITS (12), m >= 5: the pipelined pass (two tiles in
 *     flight per CTA, loads, MMAs and read-backs overlapped), matrices at
 *     most GBQ_TC_MAX_MATS per pass. */
#define GBQ_OP_MMA 9
#define GBQ_MMA_TILE_BITS 11
#define GBQ_MAX_MMA_OPS 8
#define GBQ_MAX_MMA_MATS 6
#define GBQ_TC_TILE_BITS 12
#define GBQ_TC_MAX_MATS 10

#define GBQ_MAX_OPS_PER_PASS 64
#define GBQ_MAX_TILE_BITS 13
#define GBQ_MIN_TILE_BITS 10 /* states narrower than this are padded with |0> bits */
#define GBQ_MAX_DENSE_K 5
#define GBQ_MAX_DIAG_K 8

typedef struct gbq_op {
  int8_t kind;       /* GBQ_OP_*                                              */
  int8_t k;          /* dense/probe: number of target bits; diag: number of bits */
  int8_t nsel;       /* dense/probe: selector bits (0..3), 2^nsel matrices     */
  int8_t pad0;
  int8_t bits[8];    /* dense/probe: tile bit of matrix-index bit j; diag: bit codes */
  int8_t sel[4];     /* selector bit codes; matrix number = sum sel_j << j       */
  int32_t slot;      /* probe: output slot                                       */
  int32_t pad1;
  int64_t mat;       /* offset (in gbq_c64) of the first matrix/table in the pool */
} gbq_op;

typedef struct gbq_pass {
  int32_t L;         /* tile bits (<= GBQ_MAX_TILE_BITS, <= state bits)          */
  int32_t m;         /* contiguous low bits (1..L)                               */
  int32_t op_begin;  /* first op of this pass in the op array                    */
  int32_t op_count;  /* <= GBQ_MAX_OPS_PER_PASS                                  */
  int8_t hi[16];     /* global bits of tile bits m..L-1                          */
} gbq_pass;

/* Pauli string for expectation values: P = coef * i^{ny} X^{x} Z^{z} form
 * with x = bits carrying X or Y, zy = bits carrying Z or Y, ny = #Y. */
typedef struct gbq_pauli {
  uint64_t x;
  uint64_t zy;
  int32_t ny;
  int32_t pad;
  double coef;
} gbq_pauli;

/* ---- context and memory ---------------------------------------------- */
const char* gbq_last_error(void);
int gbq_version(void);
/* sizeof(gbq_op), sizeof(gbq_pass), sizeof(gbq_pauli), sizeof(gbq_point): lets
 * a binding check its struct mirrors without touching a GPU. */
int gbq_struct_sizes(int* op, int* pass, int* pauli, int* point);
int gbq_ctx_create(int device, gbq_ctx** out);
int gbq_ctx_destroy(gbq_ctx* ctx);
int gbq_ctx_sync(gbq_ctx* ctx);
int gbq_device_info(gbq_ctx* ctx, int* sm_count, size_t* free_bytes, size_t* total_bytes);
int gbq_set_graphs(gbq_ctx* ctx, int enable);
/* Name of the context's GPU (NUL-terminated, truncated to len - 1 bytes). */
int gbq_device_name(gbq_ctx* ctx, char* buf, int len);
/* Number of kernels this context has launched (for launch accounting). */
int gbq_launch_count(gbq_ctx* ctx, int64_t* out);

/* Matrix pool of one parameter point from a plan's fused-op recipes (host
 * only, no GPU): `prog` is the plan's int32 recipe program (layout of
 * cirq_gb300/csrc/gbq_pool.cu), `gates` the point's gate matrices as
 * complex128 (gate g at element gate_off[g], gate_dim[g] x gate_dim[g],
 * row-major).  out receives pool_len complex64 entries (zero where no op
 * writes; real and imaginary parts below 1e-12 in magnitude stored as 0).  Replaces the per-point replay of the planner's fusion recipes;
 * the fused ops themselves replace the reference's per-gate
 * apply_unitary calls (cirq-core/cirq/protocols/apply_unitary_protocol.py:306-418). */
int gbq_pool_build(const int32_t* prog, int64_t prog_len, const double* gates, const int64_t* gate_off,
                   const int32_t* gate_dim, int ngates, gbq_c64* out, int64_t pool_len);
/* gbq_pool_build for npoints points: point p's gates start gate_stride
 * complex128 elements after point p-1's (same gate_off / gate_dim), its pool
 * at out + p * pool_len.  Points run on nthreads host threads (0: one per
 * hardware thread); the first error code is returned. */
int gbq_pool_build_points(const int32_t* prog, int64_t prog_len, const double* gates, int64_t gate_stride,
                          const int64_t* gate_off, const int32_t* gate_dim, int ngates, int npoints,
                          gbq_c64* out, int64_t pool_len, int nthreads);

/* ---- Clifford circuits: reference tableau run + Pauli-frame shots ---------
 * Replaces the reference's per-repetition stabilizer simulation
 * (StabilizerSampler._run, cirq-core/cirq/sim/clifford/stabilizer_sampler.py:52-70;
 * CliffordSimulator.run through SimulatorBase._run,
 * cirq-core/cirq/sim/simulator_base.py:225-273).
 * Program: ops in circuit order; qubits 0..nq-1; measurement records
 * 0..nrec-1 (one per measured qubit and measurement).
 *   UNITARY (k = 1..3 qubits q[0..k)): tables[tab + idx] for idx = x bits |
 *     z bits << k of a Pauli on those qubits gives its image x' | z' << k |
 *     sign << 2k; lin[o] (o < 2k) gives output bit o of the frame map as an
 *     XOR of input bits (x_0..x_{k-1}, z_0..z_{k-1}).
 *   MEASURE (q[0] in the Z basis into record rec; lin[0] = 1 inverts).
 *   RESET (q[0] to |0>).
 *   NOISE (q[0]): Pauli X, Y, Z with probabilities p[0], p[1], p[2].
 *   COND_PAULI (k qubits): the Pauli of tables[tab ...] (lin[j]: bit 0 = X,
 *     bit 1 = Z part on q[j]) applied when any of the records
 *     conds[cond_begin .. cond_begin + cond_count) is 1. */
#define GBQ_CLIFF_UNITARY 0
#define GBQ_CLIFF_MEASURE 1
#define GBQ_CLIFF_RESET 2
#define GBQ_CLIFF_NOISE 3
#define GBQ_CLIFF_COND_PAULI 4
typedef struct gbq_cliff_op {
  int8_t kind;
  int8_t k;
  int8_t lin[6];
  int32_t q[3];
  int32_t tab;
  int32_t rec;
  int32_t cond_begin;
  int32_t cond_count;
  float p[3];
} gbq_cliff_op;

/* Runs the program once on a stabilizer tableau on the GPU (one CTA): every
 * random measurement takes outcome 0, noise is skipped.  ref_out[nrec]
 * receives the records.  Host arrays. */
int gbq_cliff_reference(gbq_ctx* ctx, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables,
                        int ntables, const int32_t* conds, int nconds, int nrec, uint8_t* ref_out);
/* Samples `shots` runs by Pauli frames relative to the reference records
 * `ref` (from gbq_cliff_reference).  out (host): with out_bytes = 0, nrec *
 * ceil(shots/32) words, record r's bit of shot j at
 * out[r * ceil(shots/32) + j / 32] bit j % 32; with out_bytes != 0, shots *
 * nrec bytes, out[j * nrec + r] (transposed on the device).  The same seed
 * gives the same samples.
 * layers (optional, nlayers + 1 entries): the ops in layers of ops on
 * disjoint qubits, layer L = ops layers[L] .. layers[L + 1] - 1
 * (layers[0] = 0, layers[nlayers] = nops).  With layers, each CTA keeps the
 * frames of up to 1024 shots in shared memory and applies a layer's ops in
 * parallel (when 2 * nq words per 32 shots fit; otherwise the frames stay
 * in device memory and every thread walks the ops in order). */
int gbq_cliff_sample(gbq_ctx* ctx, int nq, const gbq_cliff_op* ops, int nops, const uint32_t* tables, int ntables,
                     const int32_t* conds, int nconds, const uint8_t* ref, int nrec, int64_t shots, uint64_t seed,
                     void* out, const int32_t* layers, int nlayers, int out_bytes);
/* Checks a Clifford program without a GPU (GBQ_ERR_ARG if invalid). */
int gbq_cliff_validate(int nq, const gbq_cliff_op* ops, int nops, int ntables, int nconds, int nrec);

/* Pass-specialised kernels.  Every single-state pass of 12-bit tiles whose
 * ops are register layouts, register dense ops of width <= 2 and register
 * diagonals, and every two-state pass (gbq_run_dual) of 11-bit tiles whose
 * ops are those and register probes, can run a kernel generated for its op
 * records and compiled at run time with NVRTC (cached per op-record
 * sequence and device; worker threads compile the new passes of a program
 * in parallel).  The generated kernel computes exactly what the interpreter
 * computes, in the same order, so states are bit-identical whichever kernel
 * runs a pass (probe sums are reduced with atomics in either kernel, so
 * they agree to rounding).
 * mode 0: off.  mode 1: a program's new kernels are compiled before its
 * first launch.  mode 2: they are compiled in the background and the
 * interpreter runs each pass until its kernel is ready (states of 20 or
 * more bits only; smaller passes take microseconds).  Default: the value of
 * the environment variable GBQ_JIT, else 2. */
int gbq_set_jit(gbq_ctx* ctx, int mode);
/* Specialised kernels compiled by this process so far and (optional) those
 * queued or being compiled now, and the launches of specialised kernels. */
int gbq_jit_stats(int64_t* compiles, int64_t* pending, int64_t* launches);
/* Stops background compilation for good: queued passes are dropped and
 * running compiles awaited (at most timeout_s seconds; GBQ_ERR_UNSUPPORTED
 * if some are still running then).  A host calls it before it exits (the
 * Python package does so from its atexit handler); passes whose kernel is
 * not built run on the interpreter. */
int gbq_jit_shutdown(double timeout_s);
/* The generated CUDA source of one pass (test and inspection hook; no GPU
 * needed); dual != 0 for a two-state pass as gbq_run_dual runs it.  *needed
 * receives the size including the terminating zero; GBQ_ERR_UNSUPPORTED if
 * the pass has no specialised form. */
int gbq_jit_source(int nbits, const gbq_pass* pass, const gbq_op* ops, int nops, int dual, char* buf, size_t len,
                   size_t* needed);
/* Compiles a source with NVRTC for sm_103a (no GPU needed); *cubin_bytes
 * receives the size of the result.  GBQ_ERR_UNSUPPORTED with the compiler
 * log as the error message if it does not compile or NVRTC is absent. */
int gbq_jit_compile_check(const char* src, size_t* cubin_bytes);
/* Stream-ordered timing: records CUDA event `slot` (0..15) on the context's
 * stream; gbq_event_elapsed waits for event b and returns the ms from a to b. */
int gbq_event_record(gbq_ctx* ctx, int slot);
int gbq_event_elapsed(gbq_ctx* ctx, int a, int b, float* ms);
/* Per-launch timing of tile passes: when enabled, every tile-pass launch is
 * bracketed by CUDA events on the context's stream and its duration added to
 * a running total (read with gbq_pass_timing, which synchronises). */
int gbq_set_pass_timing(gbq_ctx* ctx, int enable);
int gbq_pass_timing(gbq_ctx* ctx, double* total_ms, int64_t* launches);

int gbq_alloc(gbq_ctx* ctx, size_t bytes, void** dptr);
int gbq_free(gbq_ctx* ctx, void* dptr);
/* Pinned host memory.  From 4 MiB up: 2 MiB-aligned memory advised for
 * transparent huge pages and registered with cudaHostRegister (copies keep
 * full speed on a host whose memory is fragmented); cudaMallocHost below
 * that or when registration fails.  Free with gbq_host_free. */
int gbq_host_alloc(size_t bytes, void** hptr);
int gbq_host_free(void* hptr);
int gbq_h2d(gbq_ctx* ctx, void* dst, const void* src, size_t bytes);
int gbq_d2h(gbq_ctx* ctx, void* dst, const void* src, size_t bytes);

/* ---- state vectors ------------------------------------------------------
 * Replaces StateVectorSimulationState construction
 * (cirq-core/cirq/sim/state_vector_simulation_state.py:321-358): |index>. */
int gbq_sv_set_basis(gbq_ctx* ctx, gbq_c64* state, int nbits, uint64_t index);

/* Runs a program over one state, in place.
 * Replaces the per-operation loop SimulatorBase._core_iterator
 * (cirq-core/cirq/sim/simulator_base.py:169-214) -> protocols.apply_unitary
 * (cirq-core/cirq/protocols/apply_unitary_protocol.py:306-418) ->
 * linalg.targeted_left_multiply / apply_matrix_to_slices
 * (cirq-core/cirq/linalg/transformations.py:105-172, 310-380), and for
 * density matrices protocols.apply_channel
 * (cirq-core/cirq/protocols/apply_channel_protocol.py:168-356).
 * mats is a device pool of matrices/tables referenced by gbq_op.mat.
 * Every pass has GBQ_MIN_TILE_BITS <= L <= min(nbits, GBQ_MAX_TILE_BITS), so
 * nbits >= GBQ_MIN_TILE_BITS: narrower registers are simulated inside a
 * 2^GBQ_MIN_TILE_BITS buffer whose extra (high) bits stay |0>. */
int gbq_run(gbq_ctx* ctx, gbq_c64* state, int nbits, const gbq_pass* passes, int npasses,
            const gbq_op* ops, int nops, const gbq_c64* mats);

/* CUDA-graph capture of a program: gbq_graph_create records the launches
 * gbq_run would make for (state, program, mats) into a graph (stream capture
 * on the context's stream; nothing runs); gbq_graph_launch replays it.  The
 * state and pool pointers are baked in -- their contents may change between
 * launches (new parameter values, a new initial state), their addresses not.
 * Replaces one host launch per pass with one graph launch per simulation of
 * a circuit (the per-point loop of cirq-core/cirq/sim/simulator.py:558-605). */
typedef struct gbq_graph gbq_graph;
int gbq_graph_create(gbq_ctx* ctx, gbq_c64* state, int nbits, const gbq_pass* passes,
                     int npasses, const gbq_op* ops, int nops, const gbq_c64* mats,
                     gbq_graph** out);
int gbq_graph_launch(gbq_ctx* ctx, gbq_graph* graph);
int gbq_graph_destroy(gbq_graph* graph);

/* Checks a program against a state of nbits bits exactly as gbq_run /
 * gbq_run_dual (dual != 0) do before launching, without touching a GPU. */
int gbq_validate_program(int nbits, const gbq_pass* passes, int npasses, const gbq_op* ops,
                         int nops, int dual);

/* Two-state reverse sweep for adjoint differentiation (no reference
 * counterpart: the reference has no gradient code).  Dense/diag ops are
 * applied to both psi and lam; probe ops add Re<lam|D|psi> of each tile to
 * partial[slot * ntiles + tile] where ntiles = 2^(nbits - L) of that pass. */
int gbq_run_dual(gbq_ctx* ctx, gbq_c64* psi, gbq_c64* lam, int nbits, const gbq_pass* passes,
                 int npasses, const gbq_op* ops, int nops, const gbq_c64* mats, double* partial);
/* out[s] = sum_t partial[s * ntiles + t] for s < nslots (device arrays). */
int gbq_reduce_slots(gbq_ctx* ctx, const double* partial, int nslots, int64_t ntiles, double* out);
/* One-call adjoint gradient of <H> (no reference counterpart: the reference
 * has no gradient code; its gradients come from parameter shift through
 * Simulator.simulate_expectation_values, cirq-core/cirq/sim/sparse_simulator.py:193-218).
 * Runs the forward program (fpasses/fops, matrices fmats on the device) on
 * |0...0> of nbits bits (nq qubits; nbits > nq pads with |0> high bits),
 * forms lam = H psi from the nterms Pauli terms (real coefficients) over the
 * nq qubits, *value = <psi|H|psi>, then the two-state reverse program
 * (rpasses/rops, device matrices rmats; every pass the same tile width),
 * whose probe ops add Re<lam|D_s|psi> into slot s < nslots:
 * slot_values[s] (host array) receives each slot's total.  A parameter's
 * derivative is 2 x the sum of its slots.  Device buffers for psi, lam and
 * the per-tile partial sums are allocated and freed by the call. */
int gbq_adjoint(gbq_ctx* ctx, int nq, int nbits, const gbq_pass* fpasses, int nfpasses, const gbq_op* fops,
                int nfops, const gbq_c64* fmats, const gbq_pauli* terms, int nterms, const gbq_pass* rpasses,
                int nrpasses, const gbq_op* rops, int nrops, const gbq_c64* rmats, int nslots, double* value,
                double* slot_values);

/* Sum of |psi_i|^2 in double (host result).
 * Replaces np.linalg.norm in StateVectorTrialResult.final_state_vector
 * (cirq-core/cirq/sim/state_vector_simulator.py:131-146). */
int gbq_sv_norm2(gbq_ctx* ctx, const gbq_c64* state, int nbits, double* out);
/* Keeps the amplitudes whose index satisfies (index & mask) == value, scaled
 * by `scale`, and zeroes the rest: the collapse step of measure_state_vector
 * (cirq-core/cirq/sim/state_vector.py:235-322) and, on a 2n-bit density
 * vector, of measure_density_matrix (cirq-core/cirq/sim/density_matrix_utils.py:97-183). */
int gbq_sv_project(gbq_ctx* ctx, gbq_c64* state, int nbits, uint64_t mask, uint64_t value,
                   float scale);
/* state *= scale (device, in place). */
int gbq_sv_scale(gbq_ctx* ctx, gbq_c64* state, int nbits, float scale);
/* Final-state renormalisation rule of state_vector_simulator.py:131-146,
 * evaluated on the device: renormalises in place only when the norm is
 * within sqrt(float32 eps) of 1 and dividing by it reduces the round-off of
 * the total probability.  *applied = 1 when it did; *norm (optional)
 * receives the norm before the call (the reference warns when it is too far
 * from 1). */
int gbq_sv_final_renormalize(gbq_ctx* ctx, gbq_c64* state, int nbits, int* applied, double* norm);

/* Inverse-CDF sampling of R basis indices from |psi|^2 (dm = 0) or from the
 * diagonal of a density matrix of nbits qubits (dm = 1).  u[r] in [0, 1) are
 * host uniforms; out[r] receives the sampled index.
 * Replaces sample_state_vector (cirq-core/cirq/sim/state_vector.py:170-232),
 * state_probabilities_by_indices (cirq-core/cirq/sim/simulation_utils.py:24-65)
 * and sample_density_matrix (cirq-core/cirq/sim/density_matrix_utils.py:31-95). */
int gbq_sample(gbq_ctx* ctx, const gbq_c64* state, int nbits, int dm, const double* u, int64_t R,
               uint64_t* out);

/* Probabilities |psi_i|^2 (dm = 0) or diag(rho) (dm = 1) as float32 into a
 * device array of 2^nbits entries. */
int gbq_probabilities(gbq_ctx* ctx, const gbq_c64* state, int nbits, int dm, float* out);

/* Expectation values out[2t], out[2t+1] = (re, im) of coef_t <psi|P_t|psi>.
 * Replaces PauliString._expectation_from_state_vector_no_validation
 * (cirq-core/cirq/ops/pauli_string.py:625-655) summed by
 * PauliSum.expectation_from_state_vector (cirq-core/cirq/ops/linear_combinations.py:659-718). */
int gbq_sv_expect_paulis(gbq_ctx* ctx, const gbq_c64* state, int nbits, const gbq_pauli* terms,
                         int nterms, double* out);
/* Same values as gbq_sv_expect_paulis, for callers that cannot allocate
 * device memory (no counterpart in the reference: Cirq's simulators run in
 * host memory).  Such callers include services whose device memory belongs
 * to a host framework's pool, and loops that cannot afford cudaMalloc's
 * implicit device synchronisation.  This entry point allocates nothing: its scratch
 * is a fixed GBQ_NOALLOC_SCRATCH_BYTES array in the library's device image,
 * present on every GPU that loads the library until the process exits, and
 * found with cudaGetSymbolAddress the first time it is called on a device.
 * `state` is a device
 * array, `terms` and `out` are host arrays (2 doubles per term, as for
 * gbq_sv_expect_paulis); work is ordered on `stream` (a cudaStream_t, NULL
 * for the default stream) and the call returns after it finished.  Term lists
 * too long for the scratch (about 400 terms for states of 18 or more qubits on a
 * 152-SM GPU, more for smaller states) are rejected with GBQ_ERR_ARG.
 * All calls share the scratch: calls that overlap on the GPU race and must
 * be serialised by the caller. */
#define GBQ_NOALLOC_SCRATCH_BYTES (4u << 20)
int gbq_sv_expect_paulis_noalloc(void* stream, const gbq_c64* state, int nbits,
                                 const gbq_pauli* terms, int nterms, double* out);
/* Complex128 gate-by-gate passes (no counterpart in the reference's
 * complex64 path; they restate linalg.targeted_left_multiply,
 * cirq-core/cirq/linalg/transformations.py:105-172, in double precision,
 * one gate per pass, no fusion, no tiles).  They evolve an independent
 * double-precision copy of a circuit's state on the GPU, against which the
 * complex64 tile passes are checked at widths the CPU oracle cannot reach.
 * `state` is a device array of 2^nbits (re, im) double pairs (nbits <= 36). */
int gbq_sv64_set_basis(gbq_ctx* ctx, void* state, int nbits, uint64_t index);
/* Applies a 2^k x 2^k complex matrix (row-major (re, im) doubles, host
 * array; matrix-index bit j <-> state index bit bits[j]) for 1 <= k <= 3. */
int gbq_sv64_apply(gbq_ctx* ctx, void* state, int nbits, int k, const int32_t* bits,
                   const double* matrix);
/* out[0] = max_i |state64_i - state32_i|, out[1] = sum |state64_i|^2,
 * out[2] = sum |state32_i|^2 (host array of 3 doubles). */
int gbq_sv64_compare(gbq_ctx* ctx, const void* state64, const gbq_c64* state32, int nbits,
                     double* out);
/* Density-matrix counterpart: coef_t Tr(P_t rho) for rho of nbits qubits
 * (cirq-core/cirq/ops/pauli_string.py:734-760). */
int gbq_dm_expect_paulis(gbq_ctx* ctx, const gbq_c64* rho, int nbits, const gbq_pauli* terms,
                         int nterms, double* out);
/* out = sum_t coef_t P_t psi (a new state; used for lam = H psi).  The X
 * masks are covered by tile bit-sets of 13 bits (bits 0..3 and nine more);
 * one pass per bit-set applies every term whose X mask lies in it to tiles
 * of the state held in shared memory.  Terms with more than nine X/Y factors
 * on qubits 4 and up go through a per-amplitude kernel. */
int gbq_sv_apply_paulisum(gbq_ctx* ctx, const gbq_c64* psi, int nbits, const gbq_pauli* terms,
                          int nterms, gbq_c64* out);
/* The cover gbq_sv_apply_paulisum uses for these terms: number of tiled
 * passes, of terms left to the per-amplitude kernel, and (pass_terms, up to
 * max_passes entries; may be NULL when max_passes is 0) the terms of each
 * pass.  Host only. */
int gbq_paulisum_cover(const gbq_pauli* terms, int nterms, int nbits, int* npasses, int* nwide, int* pass_terms,
                       int max_passes);
/* out[j] = <a|b> as (re, im) in double. */
int gbq_sv_inner(gbq_ctx* ctx, const gbq_c64* a, const gbq_c64* b, int nbits, double* out);

/* ---- batched sweeps -----------------------------------------------------
 * One persistent launch over many parameter points of possibly different
 * widths.  Replaces the per-resolver loop of
 * SimulatesIntermediateState.simulate_sweep_iter (cirq-core/cirq/sim/simulator.py:558-605)
 * feeding Simulator.simulate_expectation_values_sweep_iter
 * (cirq-core/cirq/sim/sparse_simulator.py:193-218).
 * Point p runs passes [pass_begin, pass_begin+pass_count) of `passes`, with
 * op.mat offsets relative to mat_base, on a 2^nbits state held in one CTA's
 * scratch slot (all passes use 12-bit tiles, so nbits >= 12), then writes
 * out[2j], out[2j+1] = (re, im) of coef_j <psi|P_j|psi> for each of its terms
 * j in [term_begin, term_begin+term_count).  Terms of different points must
 * not overlap.  Host arrays: points, passes, ops, terms.  Device array: mats.
 */
typedef struct gbq_point {
  int32_t nbits;
  int32_t pass_begin;
  int32_t pass_count;
  int32_t term_begin;
  int32_t term_count;
  int32_t pad;
  int64_t mat_base;
} gbq_point;

int gbq_batch_expect(gbq_ctx* ctx, const gbq_point* points, int npoints, const gbq_pass* passes,
                     int npasses, const gbq_op* ops, int nops, const gbq_c64* mats,
                     const gbq_pauli* terms, int nterms, int max_nbits, double* out);

/* Batched points of one compiled circuit, evolved together (no reference
 * counterpart; same role as gbq_batch_expect: replaces the per-resolver loop
 * of simulate_sweep_iter, cirq-core/cirq/sim/simulator.py:558-605).  The
 * states of npoints points lie back to back in device memory, point p at
 * states + p * 2^nbits.
 * gbq_points_set_zero: every point's state to |0...0>.
 * gbq_run_points: runs the program on every point; each pass is one launch
 *   over all points, point p reading its matrices at mats + p * pool_stride
 *   (op.mat offsets relative to that; pool_stride even).  Single-state pass
 *   kinds only (no MMA ops), states of nbits <= 34, npoints * 2^(nbits - L)
 *   <= 2^24 tiles per pass.
 * gbq_points_expect: out[(p * nterms + t) * 2 + {0, 1}] = (re, im) of
 *   <psi_p| i^ny X^x Z^zy |psi_p> (unit coefficients) for every point p and
 *   term t; terms with equal x should be adjacent (they share one read of
 *   the state); npoints <= 65535.  Host arrays: terms, out. */
int gbq_points_set_zero(gbq_ctx* ctx, gbq_c64* states, int nbits, int npoints);
int gbq_run_points(gbq_ctx* ctx, gbq_c64* states, int nbits, int npoints, const gbq_pass* passes,
                   int npasses, const gbq_op* ops, int nops, const gbq_c64* mats, int64_t pool_stride);
int gbq_points_expect(gbq_ctx* ctx, const gbq_c64* states, int nbits, int npoints,
                      const gbq_pauli* terms, int nterms, double* out);
/* One draw per point from |psi_p|^2: out[p] = the basis index where the
 * cumulative probability first exceeds u[p] * sum |psi_p|^2 (the state's own
 * norm; u in [0, 1)).  Batched trajectories: one sample per trajectory,
 * the inverse-CDF rule of gbq_sample.  Host arrays: u, out. */
int gbq_points_sample(gbq_ctx* ctx, const gbq_c64* states, int nbits, int npoints, const double* u,
                      uint64_t* out);
/* Reduced density matrix of k = 1 or 2 qubits (global index bits bits[0..k-1];
 * bits[0] is the most significant matrix index bit) for every point:
 * out[((p * D + j) * D + l) * 2 + {0, 1}] = sum_c psi_p[i(c, j)] conj(psi_p[i(c, l)]),
 * D = 2^k, npoints <= 65535.  Trajectory Kraus weights Tr(K^dagger K rho) read it (the weights
 * ||K psi||^2 of cirq-core/cirq/sim/state_vector_simulation_state.py:206-257). */
int gbq_points_rdm(gbq_ctx* ctx, const gbq_c64* states, int nbits, int npoints, int k, const int* bits,
                   double* out);
/* Marginal distribution of m <= 5 measured qubits for every point's density
 * matrix: the states are npoints density matrices of nq qubits, each the
 * 2nq-bit vector of the reference's (2,)*2nq tensor (index row * 2^nq + col)
 * in a 2^nbits slot (nbits >= 2 nq).  out[p * 2^m + o] (host array) =
 * sum of rho_p[i, i] over the row indices i whose bit bits[j] is bit j of o
 * (bits[j] < nq: qubit position nq-1-bits[j]).  The outcome probabilities of
 * a measurement in the reference's measure_density_matrix
 * (cirq-core/cirq/sim/density_matrix_utils.py:97-183), for all trajectories
 * of a batch at once; npoints <= 65535. */
int gbq_points_dm_marginal(gbq_ctx* ctx, const gbq_c64* states, int nbits, int nq, int npoints, int m,
                           const int* bits, double* out);

#ifdef __cplusplus
}
#endif
#endif /* CIRQ_GB300_H */
