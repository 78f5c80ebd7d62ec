/*
 * qibojit_gb300.h -- C ABI of the GB300 state-vector engine.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (SV_OK = 0).  State vectors, probability and frequency arrays are DEVICE
 * pointers owned by the caller (torch, cupy or cudaMalloc'd memory); the engine
 * mutates states in place and never frees caller memory.  Gate operands (2x2,
 * 4x4, 2^k x 2^k row-major matrices, the U1 phase scalar, the 5-entry fSim
 * vector) and qubit lists are HOST pointers, read before the call returns.
 * Work is enqueued on the context's stream and is asynchronous unless the entry
 * point says otherwise; sv_sync() waits for it.
 *
 * Conventions (qibojit src/qibojit/backends/cpu.py:565-635):
 *   - qubit q of an n-qubit state is bit n-q-1 of the amplitude index;
 *   - `qubits` lists (the reference's "qubits tensor") are the SORTED bit
 *     positions n-q-1 of all controls and targets of a gate, int32;
 *   - a two-target gate's row index is 2*bit(target1) + bit(target2) in the
 *     order the targets are given; a k-target gate's row index has target[0]
 *     as its most significant bit.
 *
 * Status codes map to the reference's Python exceptions in the Python layer:
 * SV_ERR_ARG -> ValueError, SV_ERR_OOM -> RuntimeError (gpu.py:733-739),
 * SV_ERR_NO_DEVICE -> ImportError (gpu.py:85-91), others -> RuntimeError.
 */
#ifndef QIBOJIT_GB300_H
#define QIBOJIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum sv_status {
  SV_OK = 0,
  SV_ERR_ARG = 1,         /* bad argument (qubit out of range, duplicate qubit, k too large) */
  SV_ERR_OOM = 2,         /* device allocation failed */
  SV_ERR_CUDA = 3,        /* CUDA runtime error */
  SV_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  SV_ERR_UNSUPPORTED = 5, /* kernel/dtype combination not supported (e.g. Y on a real state) */
  SV_ERR_NO_DEVICE = 6    /* no usable CUDA device */
};

/* Amplitude types, as CupyBackend compiles its kernels for (gpu.py:107-112). */
enum sv_dtype { SV_C128 = 0, SV_C64 = 1, SV_F64 = 2, SV_F32 = 3 };

/* One-target kernel families, GATE_OPS (cpu.py:23-36) plus the default "apply_gate". */
enum sv_one_kind { SV_APPLY_GATE = 0, SV_APPLY_X = 1, SV_APPLY_Y = 2, SV_APPLY_Z = 3, SV_APPLY_Z_POW = 4 };
/* Two-target kernel families (cpu.py:23-36) plus the default "apply_two_qubit_gate". */
enum sv_two_kind { SV_APPLY_TWO_QUBIT_GATE = 0, SV_APPLY_SWAP = 1, SV_APPLY_FSIM = 2 };

typedef struct sv_context sv_context;

/* ---------------------------------------------------------------- context */
/* Library version (major*10000 + minor*100 + patch). */
int sv_version(void);
/* Message of the last failed call on this host thread ("" if none). */
const char* sv_last_error(void);
/* Number of CUDA devices visible, or -1 if the runtime cannot be queried. */
int sv_device_count(void);
/* Creates an engine context on `device` (CupyBackend.__init__, gpu.py:50-143,
 * without the runtime compilation: kernels are prebuilt for sm_103a). */
int sv_context_create(int device, sv_context** out);
int sv_context_destroy(sv_context* ctx);
/* Sets the cudaStream_t (as void*) later calls enqueue on; NULL = legacy default stream. */
int sv_context_set_stream(sv_context* ctx, void* stream);
/* Blocks until all work enqueued on the context's stream is done (the reference's
 * stream.synchronize() after each kernel, gpu.py:598, 638, 1006, 1035, 1075).
 * Returns SV_ERR_TIMEOUT if a kernel with bounded waits (the tensor-core dense
 * gates) gave up since the last sv_sync. */
int sv_sync(sv_context* ctx);

/* How sv_apply_multi_qubit applies dense gates: SV_DENSE_AUTO (default) runs
 * complex64 gates with 5 or 6 targets on the tensor cores and everything else on the
 * CUDA cores; SV_DENSE_SIMT uses the CUDA-core kernels only; SV_DENSE_TENSOR
 * requires the tensor-core kernel, which takes complex64 gates with 4..6 targets
 * (SV_ERR_UNSUPPORTED for others).
 * The reference has one fixed kernel per target count (gpu.py:975-1007). */
enum sv_dense_mode { SV_DENSE_AUTO = 0, SV_DENSE_SIMT = 1, SV_DENSE_TENSOR = 2 };
int sv_context_set_dense_mode(sv_context* ctx, int mode);

/* Arithmetic of the complex128 one- and two-target dense gates (apply_gate,
 * apply_z_pow, apply_two_qubit_gate, apply_fsim): SV_C128_DOUBLE_WORD (default)
 * carries every double as a pair of floats and computes on the FP32 pipe (GB300's
 * FP64 rate is 1/56 of FP32), about 2^-45 relative to the summed magnitudes of a
 * gate row, a few 1e-15 absolute for amplitudes <= 1; SV_C128_FP64 uses FP64
 * instructions.  The reference computes in FP64 (gates.py:15-254). */
enum sv_c128_arithmetic { SV_C128_DOUBLE_WORD = 0, SV_C128_FP64 = 1 };
int sv_context_set_c128_arithmetic(sv_context* ctx, int mode);

/* ---------------------------------------------------------- state creation */
/* |0...0>: state[0] = 1, all others 0.  Replaces ops.initial_state_vector
 * (custom_operators/ops.py:10-18) / CupyBackend.zero_state (gpu.py:584-600). */
int sv_zero_state(sv_context* ctx, void* state, int dtype, int nqubits);

/* ------------------------------------------------------------ gate kernels */
/* One target, any number of controls.  Replaces NumbaBackend._one_qubit_base
 * (cpu.py:606-616) and CupyBackend._one_qubit_base (gpu.py:1009-1036), i.e. the
 * {multicontrol_}apply_{gate,x,y,z,z_pow}_kernel family (gates.py:15-114).
 * gate: 4 values (2x2 row-major) for SV_APPLY_GATE, 1 value (the U1 phase) for
 * SV_APPLY_Z_POW, ignored (may be NULL) otherwise; same dtype as the state.
 * qubits: sorted bit positions of controls and target (nq = ncontrols + 1), or
 * NULL / nq = 0 for an uncontrolled gate. */
int sv_apply_one_qubit(sv_context* ctx, void* state, int dtype, int nqubits, int kind,
                       const void* gate, int target, const int32_t* qubits, int nq);

/* Two targets, any number of controls.  Replaces _two_qubit_base (cpu.py:618-635,
 * gpu.py:1038-1076): {multicontrol_}apply_{two_qubit_gate,swap,fsim}_kernel
 * (gates.py:117-254).  gate: 16 values for SV_APPLY_TWO_QUBIT_GATE, the 5-entry
 * fSim operand (matrices.py:62-70) for SV_APPLY_FSIM, ignored for SV_APPLY_SWAP.
 * qubits: as above with nq = ncontrols + 2, or NULL / 0. */
int sv_apply_two_qubit(sv_context* ctx, void* state, int dtype, int nqubits, int kind,
                       const void* gate, int target1, int target2, const int32_t* qubits, int nq);

/* k = ntargets targets (1 <= k <= 10), any number of controls.  Replaces
 * _multi_qubit_base (cpu.py:581-604, gpu.py:975-1007) and the
 * apply_{three,four,five,multi}_qubit_gate kernels (gates.py:265-424).
 * targets: qubit indices in gate order; gate: 4^k values row-major.
 * qubits: sorted bit positions of controls and targets, or NULL / 0.
 * complex64 gates with 5 or 6 targets run on the tensor cores (tcgen05, TF32
 * operands split in two, FP32 accumulation: about 2^-21 relative error per gate)
 * unless sv_context_set_dense_mode says otherwise. */
int sv_apply_multi_qubit(sv_context* ctx, void* state, int dtype, int nqubits,
                         const void* gate, const int32_t* targets, int ntargets,
                         const int32_t* qubits, int nq);

/* ---------------------------------------------------------------- collapse */
/* Zeroes the amplitudes whose measured bits differ from `result` and, when
 * `normalize`, divides the kept ones by their FP64 (compensated) norm.
 * `qubits`: the measured qubit indices in the order given (the reference maps
 * them to reversed bit positions, cpu.py:548-552); bit j of `result` (counting
 * from the most significant) is the outcome of qubits[j].  Replaces
 * NumbaBackend._collapse_statevector (cpu.py:541-563) -> ops.collapse_state /
 * collapse_state_normalized (ops.py:43-79), and CupyBackend.collapse_state
 * (gpu.py:616-644).  Uses context scratch for the norm partials. */
int sv_collapse_state(sv_context* ctx, void* state, int dtype, int nqubits,
                      const int32_t* qubits, int nq, int64_t result, int normalize);

/* Same collapse as sv_collapse_state, for callers that cannot allocate device
 * memory: code running inside a host framework that owns every device byte through
 * its own pool allocator, or a latency-critical loop that cannot afford a cudaMalloc
 * or the device synchronisation of a later cudaFree.  It takes no context and calls
 * no cudaMalloc, cudaFree or allocating library routine; the caller passes the
 * state (device pointer) and the measured qubits/outcome (host), and the work is
 * enqueued on `stream` (a cudaStream_t as void*, NULL = legacy default stream) on
 * the current device.  The norm reduction uses a fixed file-scope device array of
 * 4096 doubles (32 KiB), held by every GPU that loads the library until the process
 * exits; a call whose reduction would need more (more than 4094 partial sums, i.e.
 * a GPU with more than 511 SMs) is rejected with SV_ERR_ARG.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress) with the
 * device current, so make that first call before any stream capture.  The address is
 * kept for the life of the process: it does not survive cudaDeviceReset or any other
 * teardown of the device's primary context, after which this entry point must not be
 * called again in that process.  All calls
 * share the array and it keeps the last call's contents (every call overwrites what
 * it reads, nothing needs to start at zero); calls that overlap on the GPU (different
 * streams, or different host threads on one device) race on it.
 * This entry point has no counterpart in the reference. */
int sv_collapse_state_noalloc(void* stream, void* state, int dtype, int nqubits,
                              const int32_t* qubits, int nq, int64_t result, int normalize);

/* ----------------------------------------------------------- probabilities */
/* out[o] = sum of |amp|^2 over amplitudes whose measured bits spell o, with
 * qubits[0] the most significant bit of o (qibo Backend.calculate_probabilities,
 * wrapped by CupyBackend at gpu.py:751-768).  Accumulates in FP64; out_dtype is
 * SV_F64 or SV_F32 (rounded from the FP64 sums).  `out` has 2^nq entries. */
int sv_probabilities(sv_context* ctx, const void* state, int dtype, int nqubits,
                     const int32_t* qubits, int nq, void* out, int out_dtype);

/* ------------------------------------------------------- density matrices */
/* Marginal probabilities of an n-qubit density matrix `rho` (row-major
 * 2^n x 2^n, 2n <= 40): out[o] = sum of Re rho_ii over the basis states i whose
 * measured bits read o, qubits ordered as given (qibo's density-matrix
 * calculate_probabilities, the branch CupyBackend.calculate_probabilities
 * forwards at gpu.py:751-768).  Same output rules as sv_probabilities. */
int sv_density_probabilities(sv_context* ctx, const void* rho, int dtype, int nqubits,
                             const int32_t* qubits, int nq, void* out, int out_dtype);

/* y <- a x + b y over n elements of `dtype` (complex coefficients for complex
 * arrays; a_im = b_im = 0 for real ones).  With b = 0 y is only written.  x and
 * y may be the same array.  The accumulation of NumbaBackend
 * _apply_channel_density_matrix (cpu.py:400-415):
 * new = (1 - sum c) rho + sum_k c_k U_k rho U_k^dagger. */
int sv_axpby(sv_context* ctx, int dtype, int64_t n, const void* x, double a_re,
             double a_im, void* y, double b_re, double b_im);

/* ------------------------------------------------------------- sampling */
/* Metropolis sampling of `nshots` outcomes from `probs` (2^nbits entries,
 * SV_F64 or SV_F32), `nchains` independent chains, accumulated into the int64
 * device array `frequencies`.  Reproduces ops.measure_frequencies
 * (ops.py:82-108) exactly: chain seeds are NumPy-legacy randint(0, 1e8) draws
 * after seeding with `seed`; every chain starts at the first argmax of probs,
 * proposes (shot + randint(0, N)) % N and accepts when
 * probs[new] / probs[shot] > random(), with NumPy's legacy MT19937 streams. */
int sv_measure_frequencies(sv_context* ctx, int64_t* frequencies, const void* probs,
                           int prob_dtype, int nbits, int64_t nshots, uint32_t seed,
                           int nchains);

/* Direct sampling, the reference's branch below SHOT_METROPOLIS_THRESHOLD
 * (cpu.py:384-385 -> qibo Backend.sample_shots = numpy.random.choice(N, nshots, p)):
 * for each of the nshots uniforms in [0, 1) (host array, the caller's random_sample
 * stream) the outcome is the first index whose FP64 cumulative probability exceeds
 * u times the total.  `frequencies` (device int64, 2^nbits, added to) and `samples`
 * (device int64, nshots) may each be NULL.  Synchronises the context's stream. */
int sv_sample_cdf(sv_context* ctx, const void* probs, int prob_dtype, int nbits, const double* uniforms,
                  int64_t nshots, int64_t* frequencies, int64_t* samples);

/* -------------------------------------------------------------- reductions */
/* The precision mode keeps bulk gate arithmetic in complex64 and every reduction in
 * FP64 (Neumaier-compensated per thread, fixed-order final sums).  These return
 * their result to the host and synchronise the context's stream.  States may have
 * different dtypes (e.g. a complex64 state against a complex128 one).  They extend
 * the reference, whose norms and expectations are NumPy/CuPy sums on the host side
 * (e.g. the collapse norm, gpu.py:640-642). */
/* out_re_im[0] + i out_re_im[1] = <a|b> = sum_i conj(a_i) b_i */
int sv_inner_product(sv_context* ctx, const void* a, int dtype_a, const void* b, int dtype_b, int nqubits,
                     double* out_re_im);
/* out[0] = max_i |a_i - b_i| */
int sv_max_abs_diff(sv_context* ctx, const void* a, int dtype_a, const void* b, int dtype_b, int nqubits,
                    double* out);
/* out[0] = <Z_{q1} Z_{q2} ...> over the listed qubits (nq = 0: the norm squared) */
int sv_expectation_z(sv_context* ctx, const void* state, int dtype, int nqubits, const int32_t* qubits, int nq,
                     double* out);

/* ------------------------------------------------------------ fused programs */
/* Gate fusion.  The reference fuses with qibo's Circuit.fuse (FusedGate, applied
 * as one dense 2^k x 2^k multi-qubit kernel: cpu.py:535-537, gpu.py:929-930); the
 * engine instead compiles a gate list once into HBM passes (a native planner picks,
 * per pass, a tile of `tile_bits` bit positions and every gate whose dense targets
 * lie in it) and runs each pass as one cache-blocked kernel: one read and one write
 * of the state for many gates. */
enum sv_op_kind { SV_OP_DENSE = 0, SV_OP_DIAG = 1 };

typedef struct sv_gate_op {
  int32_t kind;          /* SV_OP_DENSE: 2^k x 2^k matrix on the targets;
                            SV_OP_DIAG: its 2^k diagonal entries */
  int32_t ntargets;      /* 1..10 (dense ops with more than 2 targets and diagonal ops
                            with more than 3 run unfused, as separate kernels) */
  int32_t ncontrols;     /* 0..16: the op acts where every control qubit is 1 */
  int32_t targets[10];   /* qubit indices; targets[0] is the most significant bit of
                            the row (dense) or table (diagonal) index */
  int32_t controls[16];  /* qubit indices */
  const double* matrix;  /* host: complex entries as (re, im) pairs, row-major */
} sv_gate_op;

typedef struct sv_program sv_program;

/* Plans and uploads a program for states of `nqubits` qubits and type `dtype`
 * (SV_C128 or SV_C64).  tile_bits <= 0 picks the default (12: 2^12 amplitudes per
 * tile).  The op list is read before the call returns.  Each pass's ops are grouped
 * into register phases by dependency, so a block of qubits runs several layers per
 * shared-memory exchange.  Complex128 programs (and complex64 programs once
 * specialised) are also phase-folded: each uncontrolled one-qubit gate becomes
 * diag * real 2x2 * diag with the diagonals carried to the next gate on their qubit
 * and folded per phase into one table, the same unitary with fewer multiply-adds. */
int sv_program_create(sv_context* ctx, int dtype, int nqubits, const sv_gate_op* ops, int nops,
                       int tile_bits, sv_program** out);
/* Applies the program to `state` (device, 2^nqubits amplitudes) on the context's stream. */
int sv_program_run(sv_context* ctx, const sv_program* prog, void* state);
/* Plan statistics: HBM passes, unfused ops, planned ops inside passes (after one-qubit
 * gate merging and phase folding), tile bits (any may be NULL). */
int sv_program_stats(const sv_program* prog, int* npasses, int* nunfused, int* nfused_gates,
                     int* tile_bits);
int sv_program_destroy(sv_program* prog);
/* Compiles, once per program structure, one kernel per pass in which the pass's tile
 * and register bit positions, op order, control masks and sign tables are literals
 * (the CUDA runtime compiler, libnvrtc, is loaded at run time); later sv_program_run
 * calls launch those kernels instead of the interpreting tile kernel.  The result is
 * the same computation (tests compare both); compilation takes seconds, so this pays
 * off for programs run many times.  No reference counterpart: qibojit compiles its
 * fixed kernel set once at import (gpu.py:76-107).  SV_ERR_UNSUPPORTED when libnvrtc
 * is absent. */
int sv_program_specialize(sv_context* ctx, sv_program* prog);

/* Introspection of a planned program, for tests that check the planner on the host:
 * the host copy of pass `pass`'s parameter block (what the pass kernel receives) and
 * its size, valid while the program lives. */
int sv_program_pass_params(const sv_program* prog, int pass, const void** params, size_t* bytes);
/* Arithmetic instructions per amplitude of one run of the program as planned (every
 * pass touches every amplitude once): lane instructions of the pass kernels' register
 * ops (FFMA and FMUL; FP32 for complex64, FP64 or their double-word expansion for
 * complex128), with controlled ops counted for the amplitudes they select.  Times 2^n
 * and divided by a run's duration it gives the rate to set against the FP32 issue peak:
 * the bound of the fused complex64 passes.  No reference counterpart. */
int sv_program_arith_per_amplitude(const sv_program* prog, double* out);
/* Byte layout of a pass block for `dtype` (SV_C128 / SV_C64): 32 entries, in order
 * sizeof(block) and the offsets of n, kt, nphases, nops, ntiles, tile_pos, coef_goff,
 * phases, ops, coef; sizeof(phase), offsets of rb, op_begin, op_end; sizeof(op), offsets
 * of type, u0, u1, nd, tb, ob, jmask, tmask, coef, omask, rpart, neg, flags, nrun, ru;
 * sizeof(coefficient). */
int sv_pass_layout(int dtype, int64_t* offsets, int n);

/* ---------------------------------------------------------- batched circuits */
/* Many circuits of uneven size (8..34 qubits) in one job, for variational workloads
 * (the reference runs circuits one at a time through execute_circuit).  Circuits with
 * the same gate structure share one plan; each run zeroes every state and applies
 * every circuit as batched fused-pass launches spread over several streams; the
 * first run also records them as a CUDA graph that later runs replay.  States live
 * in one device buffer owned by the batch. */
typedef struct sv_batch sv_batch;
int sv_batch_create(sv_context* ctx, int dtype, int ncirc, const int32_t* nqubits, const sv_gate_op* const* ops,
                    const int32_t* nops, int tile_bits, sv_batch** out);
/* |0...0> then every circuit; asynchronous on the context stream. */
int sv_batch_run(sv_context* ctx, sv_batch* b);
/* Compiles one kernel per pass of every group with the group's structure as literals
 * (as sv_program_specialize, on the unfolded plan: each circuit keeps its own
 * coefficient block); later sv_batch_run calls launch them and record a new graph.
 * Synchronises the device first.  SV_ERR_UNSUPPORTED when libnvrtc is absent. */
int sv_batch_specialize(sv_context* ctx, sv_batch* b);
/* How sv_batch_run executes the batch.  SV_BATCH_GRAPH (the default): one launch per
 * group and pass (interpreting, or the kernels of sv_batch_specialize) spread over four
 * streams and recorded as one CUDA graph.  SV_BATCH_PERSISTENT: every pass of every
 * group in one cooperative launch of an interpreting kernel whose blocks take work
 * tickets in order (each circuit's pass r after its pass r - 1, tracked per circuit in
 * device counters); recorded as a graph where the driver allows, eager otherwise.  Its
 * waits are bounded: a wait that runs out stops the launch and the next sv_sync or
 * sv_batch_tfim_energy returns SV_ERR_TIMEOUT.  Synchronises the batch's streams. */
enum sv_batch_executor { SV_BATCH_GRAPH = 0, SV_BATCH_PERSISTENT = 1 };
int sv_batch_set_executor(sv_context* ctx, sv_batch* b, int executor);
/* Transverse-field Ising energies E_c = -sum_i <Z_i Z_{i+1}> - h sum_i <X_i> (open chain),
 * FP64 accumulation; `energies` (host) receives ncirc values; synchronises. */
int sv_batch_tfim_energy(sv_context* ctx, sv_batch* b, double h, double* energies);
/* Device pointer and qubit count of one circuit's state. */
int sv_batch_state(const sv_batch* b, int circuit, void** state, int* nqubits);
int sv_batch_stats(const sv_batch* b, int* ngroups, int* npasses, size_t* state_bytes);
/* Algorithmic HBM bytes of one run's gate passes: for every circuit, its plan's pass
 * count times one read and one write of its state (the |0...0> fill excluded). */
int sv_batch_pass_bytes(const sv_batch* b, double* bytes);
/* Arithmetic lane instructions of one run's gate passes: for every circuit, its plan's
 * sv_program_arith_per_amplitude times its 2^n amplitudes. */
int sv_batch_arith(const sv_batch* b, double* instructions);
int sv_batch_destroy(sv_batch* b);

/* ---------------------------------------------------------- adjoint gradients */
/* Gradients of the transverse-field Ising energy E = <psi|H|psi>,
 * H = -sum_i Z_i Z_{i+1} - h sum_i X_i, for `ncirc` circuits of one structure (same
 * gates on the same qubits, different parameters) by the adjoint method.  Gate j is a
 * fixed gate (generators[j] = 0) or exp(-i t G / 2) with G = X, Y, Z (generators[j] =
 * 1, 2, 3) on one qubit, t = parameter params[j] in [0, nparams).  The forward state is
 * checkpointed after segment_ends[0..nsegments-2] and restored during the reverse
 * sweep (bounds complex64 drift); inner products accumulate in FP64.  The reference
 * has no gradient path; this extends it for variational workloads. */
typedef struct sv_adjoint sv_adjoint;
int sv_adjoint_create(sv_context* ctx, int dtype, int ncirc, int nqubits, const sv_gate_op* const* ops, int nops,
                      const int8_t* generators, const int32_t* params, int nparams, const int32_t* segment_ends,
                      int nsegments, int tile_bits, sv_adjoint** out);
/* New parameters for the same structure: re-gathers coefficients, keeps plans and memory. */
int sv_adjoint_update(sv_context* ctx, sv_adjoint* A, const sv_gate_op* const* ops, int nops,
                      const int8_t* generators, const int32_t* params);
/* Forward + reverse sweep: energies (host, ncirc) and gradients (host, ncirc x nparams,
 * row-major); either may be NULL.  Synchronises. */
int sv_adjoint_run(sv_context* ctx, sv_adjoint* A, double h, double* energies, double* grads);
/* Compiles the forward passes (as sv_batch_specialize) and the reverse-sweep passes
 * (psi and lambda tiles, every gradient marker as literals) of every segment with the
 * structure fixed in the source; later runs launch them, and sv_adjoint_update keeps
 * them (coefficients stay in device arrays).  SV_ERR_UNSUPPORTED when libnvrtc is
 * absent. */
int sv_adjoint_specialize(sv_context* ctx, sv_adjoint* A);
/* Device pointer of a circuit's final forward state (valid after a run, until the next). */
int sv_adjoint_state(const sv_adjoint* A, int circuit, void** psi);
int sv_adjoint_destroy(sv_adjoint* A);

#ifdef __cplusplus
}
#endif

#endif /* QIBOJIT_GB300_H */
