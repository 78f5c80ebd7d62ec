// sv_plan.cuh -- the fused-pass program: op records, phases, pass parameters and the
// host-side program object shared by the planner (sv_fused.cu) and the run-time
// specialiser of pass kernels (sv_specialize.cu).
#pragma once

#include <stdint.h>

#include <vector>

#include "sv_common.cuh"

namespace sv {

constexpr int kRB = 4;            // register bits per phase (16 amplitudes per thread)
constexpr int kMaxTile = 14;      // tile bits
constexpr int kLowBits = 4;       // lowest bits always in a tile (contiguous runs)
constexpr int kMaxPassOps = 192;  // ops (and phases) per pass: capacity of the pass parameters
constexpr int kMaxPassOpsRefill = 128;  // ops per pass of programs refilled per circuit (batches, adjoint)
constexpr int kCoefBytes = 12288; // coefficient bytes per pass

enum : uint8_t {
  FOP_DENSE1 = 0,   // complex 2x2
  FOP_DENSE2 = 1,   // complex 4x4
  FOP_DIAG = 2,     // diagonal phases on up to 3 bits
  FOP_SIGN = 3,     // diagonal with entries +-1 (CZ, Z, CCZ): folded into a negate mask
  FOP_D1RUN = 4,    // up to 4 uncontrolled complex 2x2 on distinct register bits
  FOP_X1 = 5,       // X (CNOT, Toffoli targets): a register swap, no arithmetic
  FOP_DENSE1R = 6,  // real 2x2 (RY, H): half the flops of a complex one
  FOP_SWAP2 = 7,    // SWAP: exchange of |01> and |10>, no arithmetic
  FOP_GRADX = 8,    // adjoint sweep: Im<lambda|X_q|psi> on a register bit (coef = parameter index)
  FOP_GRADY = 9,    //                Im<lambda|Y_q|psi>
  FOP_GRADZ = 10,   //                Im<lambda|Z_q|psi>, any bit (diagonal)
  FOP_DIAGR = 11,   // diagonal over the 4 register bits: amplitude j times coefficient j
  FOP_D1RUNR = 12,  // FOP_D1RUN of real 2x2 gates
  FOP_DENSE1P = 13  // real 2x2 with a unit entry in each row (u1 bit i: row i's unit is in column 1)
};
// internal op kind of the adjoint planner: a gradient marker (no matrix)
constexpr int OP_GRAD = 2;
enum : uint8_t { FLAG_OMASK = 1, FLAG_TMASK = 2 };

// One op in phase-local form (64 bytes).
struct FOp {
  uint8_t type, u0, u1, nd;  // dense: register positions of the targets (u0 = row MSB); diag: #bits
  int8_t tb[3];              // diag bit i read from the thread's local index bit tb[i] (or -1)
  int8_t ob[3];              // diag bit i read from the tile's outer global bit ob[i] (or -1)
  uint8_t pad0[2];
  uint16_t jmask;            // register-level controls: amplitudes / pair bases j allowed
  uint16_t pad1;
  uint32_t tmask;            // thread-level controls: local non-register bits that must be 1
  uint32_t coef;             // first coefficient of this op in the pass's coefficient array
  uint64_t omask;            // tile-level controls: outer global bits that must be 1
  uint64_t rpart;            // diag: table-index part from register bits, 4 bits per amplitude j
  uint16_t neg[8];           // sign diag: negate-mask over j for each non-register index part
  uint8_t flags;             // FLAG_OMASK / FLAG_TMASK: which control checks apply
  uint8_t nrun;              // FOP_D1RUN: number of uncontrolled one-target gates (1..4)
  uint8_t ru[4];             // FOP_D1RUN: their register positions; matrices at coef + 4k
  uint8_t pad2[2];
};
static_assert(sizeof(FOp) == 64, "FOp layout");

struct Phase {
  uint8_t rb[kRB];           // local tile bits held in registers, ascending (j bit u <-> rb[u])
  uint16_t op_begin, op_end;
  uint16_t soff[16];         // shared-memory offset of register j: smem_pos(register bits of j)
};

template <typename T>
struct PassParams {
  int32_t n, kt, nphases, nops;
  int64_t ntiles;
  int32_t tile_pos[kMaxTile];  // global bit positions of the tile bits, ascending
  int32_t coef_goff;           // batched runs: this pass's first coefficient in a circuit's block
  Phase phases[kMaxPassOps];
  FOp ops[kMaxPassOps];
  T coef[kCoefBytes / sizeof(T)];
};

struct HostOp {
  int kind;                 // SV_OP_DENSE / SV_OP_DIAG
  int nt;                   // targets
  int tpos[kMaxTargets];    // global bit positions of the targets, gate order
  int nc;
  int cpos[16];
  std::vector<double> m;    // complex entries (re, im) pairs
  bool sign_only = false;   // diagonal with entries in {+1, -1}
  int sign_mask = 0;        // bit i set: entry i is -1
  bool is_x = false;        // dense one-target [[0, 1], [1, 0]]
  bool is_real = false;     // dense with all-real entries
  bool is_swap = false;     // dense two-target SWAP
  int unit_cols = -1;       // pivoted real 2x2 (phase folding): bit i = column of row i's unit entry
  int gen = 0;              // OP_GRAD: generator 1 = X, 2 = Y, 3 = Z
  int param = -1;           // OP_GRAD: parameter index
};

// ops that need their target bit in the tile and in the phase's registers
static inline bool dense_like(const HostOp& h) { return h.kind == SV_OP_DENSE || (h.kind == OP_GRAD && h.gen != 3); }

// run-time compiled kernels of a program's passes
struct Specialized;

struct Segment {
  bool fused = false;
  int pass = -1;            // index into the program's pass parameter blocks
  int host_op = -1;         // unfused op
};

}  // namespace sv

struct sv_program {
  int dtype, nqubits, kt;
  std::vector<sv::HostOp> ops;
  std::vector<sv::Segment> segments;
  std::vector<unsigned char> passes;  // PassParams<T> blocks, back to back
  size_t pass_bytes = 0;
  // complex128 programs: the same blocks with every coefficient split into float pairs
  // (PassParams<cw>, read by the double-word pass kernels)
  std::vector<unsigned char> passes_dw;
  // coefficient sources of all passes, back to back: (op index, entry) per slot
  std::vector<int32_t> coef_src;
  std::vector<size_t> pass_coef_off;
  size_t coef_total = 0;
  int npasses = 0, nunfused = 0, nfused_gates = 0, nphases = 0;
  // the encoder may fold a phase's one-bit register diagonals into one FOP_DIAGR table;
  // its coefficients are products of several ops' entries, so programs whose
  // coefficients are refilled per circuit (batches, adjoint sweeps) keep this off
  bool fold_diagonals = false;
  // group a pass's ops into phases by dependency (several layers per tile exchange)
  // rather than in program order; adjoint sweeps keep program order around their
  // gradient markers
  bool pack_phases = false;
  // pass kernels compiled for this program's structure (sv_program_specialize), or null
  sv::Specialized* spec = nullptr;
  // batched pass kernels for a group of circuits of this structure (sv_batch_specialize)
  sv::Specialized* bspec = nullptr;
  sv::Specialized* aspec = nullptr;   // adjoint-sweep kernels of a backward program
};


namespace sv {

// shared memory of a fused pass: two tiles (double buffering) and the tile-bit deposit table
template <typename T>
inline size_t pass_smem(int kt) {
  const int tsize = 1 << kt;
  return 2 * sizeof(T) * tile_stride(tsize) + sizeof(int64_t) * (1 << (kt - kLowBits));
}

// re-plans a program with phase folding (sv_fused.cu) unless it already has it
int refold_program(sv_program* prog);
// launches pass `pass` of a specialised program on the context stream
int specialized_launch(Context* ctx, const sv_program* prog, int pass, void* state);
// whether a specialised program's kernels compute in double-word arithmetic (cw)
bool specialized_is_dw(const Specialized* s);
// compiles the batched pass kernels of an (unfolded) program into prog->bspec; dw:
// complex128 kernels in double-word arithmetic (coefficients passed as cw)
int specialize_batched(Context* ctx, sv_program* prog, bool dw);
// launches batched pass `pass` over ncirc circuits: state pointer table, coefficient blocks
int specialized_launch_batched(Context* ctx, const sv_program* prog, int pass, cudaStream_t stream, void* states,
                               const void* coef, int64_t coef_stride, int ncirc);
// compiles the adjoint-sweep kernels of a backward program (psi and lambda, gradient
// markers) into prog->aspec
int specialize_adjoint(Context* ctx, sv_program* prog);
// launches adjoint pass `pass` over ncirc circuits: psi and lambda pointer tables,
// coefficient blocks, per-block gradient partials gpart[circuit][parameter][gstride]
int specialized_launch_adjoint(Context* ctx, const sv_program* prog, int pass, void* psis, void* lams,
                               const void* coef, int64_t coef_stride, int ncirc, double* gpart, int nparams,
                               int gstride);
void specialized_free(Specialized* s);

}  // namespace sv
