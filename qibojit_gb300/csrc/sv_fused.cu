// sv_fused.cu -- gate fusion: a native pass planner and the cache-blocked tile kernel.
//
// A circuit is compiled once into a program of HBM passes.  Each pass owns a set S of
// kt "tile" bit positions (always containing the 4 lowest bits, so a tile is read as
// runs of 16 contiguous amplitudes); a CTA loads the 2^kt amplitudes of one tile (one
// fixed value of the other bits) into shared memory, applies every gate the pass
// holds, and writes the tile back: one read and one write of the state for many
// gates.  A gate joins a pass when its dense target bits lie in S; diagonal gates and
// control qubits may sit on any bit (outside S they are constant over a tile).
//
// Inside a tile, gates run in register-blocked phases: each thread holds the 16
// amplitudes that differ in the 4 local bits of the phase, applies all gates of the
// phase in registers, and exchanges through shared memory between phases.  The
// planner precomputes everything that depends only on the gate and the phase (which
// registers a control or a diagonal bit selects, sign masks), so the kernel's inner
// loops are FMAs and constant-shift bit tests.  A pass's ops and coefficients ride in
// the kernel parameters (constant bank); tiles are double-buffered with cp.async so
// the next tile's HBM read overlaps this tile's arithmetic.
//
// Phases are packed by dependency (pack_phases), so a block of qubits runs several
// layers per tile exchange.  Programs can also be phase-folded (fold_phases,
// fold_register_diagonals): every one-qubit gate becomes diag * pivoted real 2x2 *
// diag, and diagonals are carried to the next gate on their qubit and folded per phase
// into one register table.  Complex128 programs always fold; complex64 programs fold
// when their passes are compiled into specialised kernels (sv_specialize.cu), because
// this interpreting kernel pays a decode cost per op.
//
// This replaces the reference's fusion path (qibo Circuit.fuse -> FusedGate, applied
// by qibojit as one dense 2^k x 2^k multi-qubit kernel, cpu.py:535-537,
// gpu.py:929-930) with a schedule that needs no dense products of gate matrices.
#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <type_traits>
#include <vector>

#include "sv_plan.cuh"
#include "sv_persist_queue.h"

namespace sv {

// ------------------------------------------------- register ops at run-time positions
template <typename T>
__device__ __forceinline__ void dense1_dispatch(T (&v)[16], const T* m, int u, unsigned jm) {
  // jm == 0xffff marks an op without register-level controls: no per-pair tests
  if (jm == 0xffffu) {
    switch (u) {
      case 0: dense1_regs<T, 0>(v, m, 0xffffu); break;
      case 1: dense1_regs<T, 1>(v, m, 0xffffu); break;
      case 2: dense1_regs<T, 2>(v, m, 0xffffu); break;
      default: dense1_regs<T, 3>(v, m, 0xffffu); break;
    }
    return;
  }
  switch (u) {
    case 0: dense1_regs<T, 0>(v, m, jm); break;
    case 1: dense1_regs<T, 1>(v, m, jm); break;
    case 2: dense1_regs<T, 2>(v, m, jm); break;
    default: dense1_regs<T, 3>(v, m, jm); break;
  }
}

template <typename T>
__device__ __forceinline__ void pivot1_dispatch(T (&v)[16], const T* m, int u, int form, unsigned jm) {
#define SV_P1(U, F) \
  if (u == U && form == F) { pivot1_regs<T, U, F>(v, m, jm); return; }
  SV_P1(0, 0) SV_P1(0, 1) SV_P1(0, 2) SV_P1(0, 3) SV_P1(1, 0) SV_P1(1, 1) SV_P1(1, 2) SV_P1(1, 3)
  SV_P1(2, 0) SV_P1(2, 1) SV_P1(2, 2) SV_P1(2, 3) SV_P1(3, 0) SV_P1(3, 1) SV_P1(3, 2) SV_P1(3, 3)
#undef SV_P1
}

template <typename T>
__device__ __forceinline__ void x1_dispatch(T (&v)[16], int u, unsigned jm) {
  switch (u) {
    case 0: x1_regs<T, 0>(v, jm); break;
    case 1: x1_regs<T, 1>(v, jm); break;
    case 2: x1_regs<T, 2>(v, jm); break;
    default: x1_regs<T, 3>(v, jm); break;
  }
}

template <typename T>
__device__ __forceinline__ void dense1r_dispatch(T (&v)[16], const T* m, int u, unsigned jm) {
  switch (u) {
    case 0: dense1r_regs<T, 0>(v, m, jm); break;
    case 1: dense1r_regs<T, 1>(v, m, jm); break;
    case 2: dense1r_regs<T, 2>(v, m, jm); break;
    default: dense1r_regs<T, 3>(v, m, jm); break;
  }
}

template <typename T>
__device__ __forceinline__ void swap2_dispatch(T (&v)[16], int u0, int u1, unsigned jm) {
  const int a = u0 < u1 ? u0 : u1, b = u0 < u1 ? u1 : u0;  // symmetric in its two targets
#define SV_S2(A, B) \
  if (a == A && b == B) { swap2_regs<T, A, B>(v, jm); return; }
  SV_S2(0, 1) SV_S2(0, 2) SV_S2(0, 3) SV_S2(1, 2) SV_S2(1, 3) SV_S2(2, 3)
#undef SV_S2
}

template <typename T>
__device__ __forceinline__ void dense2_dispatch(T (&v)[16], const T* m, int u0, int u1, unsigned jm) {
#define SV_D2(A, B) \
  if (u0 == A && u1 == B) { dense2_regs<T, A, B>(v, m, jm); return; }
  SV_D2(0, 1) SV_D2(0, 2) SV_D2(0, 3) SV_D2(1, 0) SV_D2(1, 2) SV_D2(1, 3)
  SV_D2(2, 0) SV_D2(2, 1) SV_D2(2, 3) SV_D2(3, 0) SV_D2(3, 1) SV_D2(3, 2)
#undef SV_D2
}

// threads per CTA = 2^(kt - 4): at most 512 (complex64, kt <= 13) or 256 (complex128, kt <= 12)
template <typename T>
constexpr int fused_max_threads() { return sizeof(T) >= 16 ? 256 : 512; }

__device__ __forceinline__ int64_t tile_origin(int64_t t, const int32_t* pos, int kt) {
  int64_t base = t;  // insert zeros at the ascending tile bit positions
  for (int b = 0; b < kt; b++) {
    const int p = pos[b];
    base = ((base >> p) << (p + 1)) | (base & (((int64_t)1 << p) - 1));
  }
  return base;
}

// ------------------------------------------------------------------ tile kernel
// MAXT/MINB: threads per CTA and CTAs per SM the register allocation is sized for.
// complex64 tiles of up to 2^12 amplitudes run three 256-thread CTAs per SM (80
// registers); larger complex64 tiles and complex128 tiles (FP64-bound) run with the
// whole register file.
// Batched runs: many circuits with the same pass structure (same gates on the same
// qubits, different parameters) share one launch; work item = (circuit, tile), each
// circuit has its own state and its own coefficient block in global memory.
template <typename T>
struct BatchArgs {
  T* const* states;        // device array of per-circuit state pointers
  const T* coef;           // per-circuit coefficient blocks, coef_stride apart
  int64_t coef_stride;
  int32_t ncirc;
  int32_t pad;
};

// the ops of one pass on one tile in shared memory, phase by phase (a barrier after
// each); `active`: this thread holds registers in this tile (threads beyond the tile's
// 2^(kt-4) only take part in the barriers)
template <typename T>
__device__ __forceinline__ void tile_phases(const PassParams<T>& p, T* tile, const T* cbase, int64_t base,
                                            bool active) {
  for (int ph = 0; ph < p.nphases; ph++) {
    // one barrier instruction for every thread (an aligned barrier must not be reached
    // by the lanes of one warp at different call sites)
    if (active) {
      const Phase& P = p.phases[ph];
      const int r0 = P.rb[0], r1 = P.rb[1], r2 = P.rb[2], r3 = P.rb[3];
      // thread bits deposited into the non-register local bits (register bits ascending)
      int lbase = threadIdx.x;
      lbase = ((lbase >> r0) << (r0 + 1)) | (lbase & ((1 << r0) - 1));
      lbase = ((lbase >> r1) << (r1 + 1)) | (lbase & ((1 << r1) - 1));
      lbase = ((lbase >> r2) << (r2 + 1)) | (lbase & ((1 << r2) - 1));
      lbase = ((lbase >> r3) << (r3 + 1)) | (lbase & ((1 << r3) - 1));
      // lbase and the register bits are disjoint, so smem_pos splits into a sum
      T* const tp_base = tile + smem_pos(lbase);
      T v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = tp_base[P.soff[j]];
      unsigned pending_neg = 0;  // sign-only diagonals commute: collect them, apply before mixing
      for (int o = P.op_begin; o < P.op_end; o++) {
        const FOp& op = p.ops[o];
        const int type = op.type;
        if (type == FOP_D1RUN) {
          if (pending_neg) {
            apply_negations(v, pending_neg);
            pending_neg = 0;
          }
          const int nr = op.nrun;
          const T* c = cbase + op.coef;
          if (nr == 4) {
            // the planner sorts a run of four gates on distinct bits into register order
            dense1_regs<T, 0>(v, c, 0xffffu);
            dense1_regs<T, 1>(v, c + 4, 0xffffu);
            dense1_regs<T, 2>(v, c + 8, 0xffffu);
            dense1_regs<T, 3>(v, c + 12, 0xffffu);
          } else {
#pragma unroll 1
            for (int k = 0; k < nr; k++) dense1_dispatch(v, c + 4 * k, op.ru[k], 0xffffu);
          }
          continue;
        }
        if (type == FOP_D1RUNR) {
          if (pending_neg) {
            apply_negations(v, pending_neg);
            pending_neg = 0;
          }
          const int nr = op.nrun;
          const T* c = cbase + op.coef;
          if (nr == 4) {
            dense1r_regs<T, 0>(v, c, 0xffffu);
            dense1r_regs<T, 1>(v, c + 4, 0xffffu);
            dense1r_regs<T, 2>(v, c + 8, 0xffffu);
            dense1r_regs<T, 3>(v, c + 12, 0xffffu);
          } else {
#pragma unroll 1
            for (int k = 0; k < nr; k++) dense1r_dispatch(v, c + 4 * k, op.ru[k], 0xffffu);
          }
          continue;
        }
        if (type == FOP_DIAGR) {  // commutes with the pending sign flips
          const T* c = cbase + op.coef;
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = tmul(c[j], v[j]);
          continue;
        }
        const int flags = op.flags;
        if ((flags & FLAG_OMASK) && ((base & (int64_t)op.omask) != (int64_t)op.omask)) continue;
        if ((flags & FLAG_TMASK) && (((unsigned)lbase & op.tmask) != op.tmask)) continue;
        if (type == FOP_DENSE1 || type == FOP_DENSE1R || type == FOP_DENSE1P || type == FOP_X1 ||
            type == FOP_SWAP2) {
          if (pending_neg) {
            apply_negations(v, pending_neg);
            pending_neg = 0;
          }
          if (type == FOP_DENSE1) dense1_dispatch(v, cbase + op.coef, op.u0, op.jmask);
          else if (type == FOP_DENSE1R) dense1r_dispatch(v, cbase + op.coef, op.u0, op.jmask);
          else if (type == FOP_DENSE1P) pivot1_dispatch(v, cbase + op.coef, op.u0, op.u1, op.jmask);
          else if (type == FOP_X1) x1_dispatch(v, op.u0, op.jmask);
          else swap2_dispatch(v, op.u0, op.u1, op.jmask);
        } else if (type == FOP_DENSE2) {
          if (pending_neg) {
            apply_negations(v, pending_neg);
            pending_neg = 0;
          }
          dense2_dispatch(v, cbase + op.coef, op.u0, op.u1, op.jmask);
        } else {
          const int nd = op.nd;
          int tp = 0;
#pragma unroll
          for (int i = 0; i < 3; i++) {
            if (i >= nd) break;
            if (op.tb[i] >= 0) tp |= ((lbase >> op.tb[i]) & 1) << (nd - 1 - i);
            else if (op.ob[i] >= 0) tp |= (int)((base >> op.ob[i]) & 1) << (nd - 1 - i);
          }
          if (type == FOP_SIGN) {
            pending_neg ^= op.neg[tp];
          } else {
            const unsigned jm = op.jmask;
            const uint64_t rp = op.rpart;
            const T* c = cbase + op.coef;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              if (!((jm >> j) & 1u)) continue;
              const int idx = (int)((rp >> (4 * j)) & 15) | tp;
              v[j] = tmul(c[idx], v[j]);
            }
          }
        }
      }
      if (pending_neg) apply_negations(v, pending_neg);
#pragma unroll
      for (int j = 0; j < 16; j++) tp_base[P.soff[j]] = v[j];
    }
    __syncthreads();
  }
}

template <typename T, int MAXT, int MINB, bool BATCHED>
__global__ void __launch_bounds__(MAXT, MINB) k_fused_pass(T* __restrict__ state,
                                                         const __grid_constant__ PassParams<T> p,
                                                         const __grid_constant__ BatchArgs<T> batch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int kt = p.kt;
  const int tsize = 1 << kt;
  const int tstride = tile_stride(tsize);
  T* const buf0 = reinterpret_cast<T*>(smem_raw);  // two tiles, tstride apart
  int64_t* dep_hi = reinterpret_cast<int64_t*>(buf0 + 2 * tstride);
  const int nhi = kt - kLowBits;
  for (int h = threadIdx.x; h < (1 << nhi); h += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < nhi; b++)
      if ((h >> b) & 1) o |= (int64_t)1 << p.tile_pos[kLowBits + b];
    dep_hi[h] = o;
  }
  __syncthreads();
  const int nthreads = blockDim.x;
  auto issue_load = [&](T* buf, const T* st, int64_t base) {
    for (int e = threadIdx.x; e < tsize; e += nthreads)
      cp_async<sizeof(T)>(buf + smem_pos(e), st + (base | dep_hi[e >> kLowBits] | (e & ((1 << kLowBits) - 1))));
    cp_async_commit();
  };
  // items: (circuit, tile) for batched runs, tiles of the one state otherwise
  const int64_t nitems = BATCHED ? p.ntiles * batch.ncirc : p.ntiles;
  const int tshift = p.n - kt;  // ntiles = 2^tshift
  auto item_state = [&](int64_t it) -> T* {
    if constexpr (BATCHED) return batch.states[it >> tshift];
    else return state;
  };
  auto item_tile = [&](int64_t it) -> int64_t { return BATCHED ? (it & (p.ntiles - 1)) : it; };
  int64_t t = blockIdx.x;
  if (t < nitems) issue_load(buf0, item_state(t), tile_origin(item_tile(t), p.tile_pos, kt));
  int cur = 0;
  for (; t < nitems; t += gridDim.x, cur ^= 1) {
    T* tile = buf0 + cur * tstride;
    T* const st = item_state(t);
    const int64_t base = tile_origin(item_tile(t), p.tile_pos, kt);
    const T* cbase;
    if constexpr (BATCHED) cbase = batch.coef + (t >> tshift) * batch.coef_stride + p.coef_goff;
    else cbase = p.coef;
    const int64_t tn = t + gridDim.x;
    if (tn < nitems) {
      issue_load(buf0 + (cur ^ 1) * tstride, item_state(tn), tile_origin(item_tile(tn), p.tile_pos, kt));
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    if constexpr (stored_as_double_pairs<T>::value) {
      // the tile arrived as complex128 bytes: convert it to float pairs in place, once
      // per pass (the final stores convert back)
      for (int e = threadIdx.x; e < tsize; e += nthreads) cw_from_stored(tile + smem_pos(e));
      __syncthreads();
    }
    tile_phases(p, tile, cbase, base, true);
    for (int e = threadIdx.x; e < tsize; e += nthreads)
      stg_stream(st + (base | dep_hi[e >> kLowBits] | (e & ((1 << kLowBits) - 1))), tile[smem_pos(e)]);
    __syncthreads();  // this buffer is refilled by the prefetch two tiles later
  }
}

// =================================================================== planner
template <typename T>
static T to_elem(const double* re_im) {
  if constexpr (is_complex<T>::value) {
    using R = typename real_of<T>::type;
    return T{(R)re_im[0], (R)re_im[1]};
  } else {
    return (T)re_im[0];
  }
}

static int coef_cost(const HostOp& h) {
  if (h.kind == OP_GRAD) return 0;
  if (h.kind == SV_OP_DENSE) {
    if (h.is_x || (h.nt == 2 && h.is_swap)) return 0;
    if (h.nt == 1 && h.unit_cols >= 0) return 2;  // the two row ratios of a pivoted real 2x2
    return h.nt == 1 ? 4 : 16;
  }
  return h.sign_only ? 0 : (1 << h.nt);
}

// Builds the phase-local form of the scheduled ops of one pass.
// Every coefficient slot of a pass records where it came from (op index, entry), so a
// circuit with the same structure and other parameters can refill the slots.
// Consecutive sign diagonals of one phase commute and act as one: merge each run of
// them (without thread or tile controls) into a single FOP_SIGN whose negate table is
// indexed by the union of their non-register bits, while that union has <= 3 bits.
static void merge_signs(FOp* ops, int begin, int* end) {
  auto descs = [](const FOp& f, int (*d)[2], int* slot) {  // non-register bits and their table slots
    int k = 0;
    for (int i = 0; i < f.nd; i++) {
      if (f.tb[i] < 0 && f.ob[i] < 0) continue;
      d[k][0] = f.tb[i];
      d[k][1] = f.ob[i];
      slot[k] = f.nd - 1 - i;
      k++;
    }
    return k;
  };
  int w = begin;
  for (int r = begin; r < *end; r++) {
    FOp f = ops[r];
    const bool plain_sign = f.type == FOP_SIGN && f.omask == 0 && f.tmask == 0;
    if (plain_sign && w > begin) {
      FOp& g = ops[w - 1];
      if (g.type == FOP_SIGN && g.omask == 0 && g.tmask == 0) {
        int dg[3][2], sg[3], df[3][2], sf[3];
        const int ng = descs(g, dg, sg), nf = descs(f, df, sf);
        int du[3][2], nu = 0, mapg[3], mapf[3];
        bool fits = true;
        for (int a = 0; a < ng + nf && fits; a++) {
          const int* d = a < ng ? dg[a] : df[a - ng];
          int u = 0;
          while (u < nu && !(du[u][0] == d[0] && du[u][1] == d[1])) u++;
          if (u == nu) {
            if (nu == 3) {
              fits = false;
              break;
            }
            du[nu][0] = d[0];
            du[nu][1] = d[1];
            nu++;
          }
          (a < ng ? mapg[a] : mapf[a - ng]) = u;
        }
        if (fits) {
          FOp m;
          memset(&m, 0, sizeof(m));
          m.type = FOP_SIGN;
          m.nd = (uint8_t)nu;
          m.jmask = 0xffffu;
          for (int i = 0; i < 3; i++) {
            m.tb[i] = i < nu ? (int8_t)du[i][0] : (int8_t)-1;
            m.ob[i] = i < nu ? (int8_t)du[i][1] : (int8_t)-1;
          }
          // union entry u sits at table bit nu - 1 - u
          for (int t = 0; t < (1 << nu); t++) {
            int tg = 0, tf = 0;
            for (int a = 0; a < ng; a++) tg |= ((t >> (nu - 1 - mapg[a])) & 1) << sg[a];
            for (int a = 0; a < nf; a++) tf |= ((t >> (nu - 1 - mapf[a])) & 1) << sf[a];
            m.neg[t] = (uint16_t)(g.neg[tg] ^ f.neg[tf]);
          }
          g = m;
          continue;
        }
      }
    }
    ops[w++] = f;
  }
  *end = w;
}

// Folds runs of register-only diagonals of a phase (diagonals and sign diagonals whose
// table bits and controls are all register bits) into one FOP_DIAGR table of 16
// complex factors, one multiply per amplitude for the whole run.  These foldable
// diagonals are first regrouped: each may sit anywhere between the mixing ops on its
// own slots before and after it (it commutes with the rest, diagonals included), and
// the fewest common positions that hold every one of them are chosen greedily (interval
// stabbing: each position is the right end of the earliest-ending interval not yet
// held).  Table entries are products of the ops' FP64 entries.
template <typename T>
static void fold_register_diagonals(const sv_program* prog, PassParams<T>* pp, int begin, int* end, int* ncoef,
                                    int* slack, std::vector<int32_t>* src) {
  // a diagonal whose table bits and controls are all register bits
  auto reg_diag = [](const FOp& f) {
    if (f.type != FOP_DIAG || f.omask || f.tmask) return false;
    for (int i = 0; i < f.nd; i++)
      if (f.tb[i] >= 0 || f.ob[i] >= 0) return false;
    return true;
  };
  auto reg_sign = [](const FOp& f) {
    if (f.type != FOP_SIGN || f.omask || f.tmask) return false;
    for (int i = 0; i < f.nd; i++)
      if (f.tb[i] >= 0 || f.ob[i] >= 0) return false;
    return true;
  };
  auto rpart_of = [](const FOp& f, int j) { return (int)((f.rpart >> (4 * j)) & 15); };
  // register slots a foldable diagonal depends on
  auto fold_slots = [&](const FOp& f) -> unsigned {
    unsigned m = 0;
    for (int v = 0; v < kRB; v++)
      for (int j = 0; j < 16; j++) {
        const int k = j ^ (1 << v);
        if (reg_diag(f)) {
          const bool a = (f.jmask >> j) & 1, b = (f.jmask >> k) & 1;
          if (a != b || (a && rpart_of(f, j) != rpart_of(f, k))) m |= 1u << v;
        } else if (((f.neg[0] >> j) & 1) != ((f.neg[0] >> k) & 1)) {
          m |= 1u << v;
        }
      }
    return m;
  };
  // register slots whose diagonals a fixed op does not commute with (all 4: unknown kind)
  auto mixing_slots = [](const FOp& g) -> unsigned {
    switch (g.type) {
      case FOP_DENSE1: case FOP_DENSE1R: case FOP_DENSE1P: case FOP_X1: return 1u << g.u0;
      case FOP_DENSE2: case FOP_SWAP2: return (1u << g.u0) | (1u << g.u1);
      case FOP_D1RUN: case FOP_D1RUNR: {
        unsigned m = 0;
        for (int k = 0; k < g.nrun; k++) m |= 1u << g.ru[k];
        return m;
      }
      case FOP_DIAG: case FOP_SIGN: case FOP_DIAGR: return 0u;
      default: return 0xfu;
    }
  };
  {
    std::vector<FOp> fixed, fold;
    std::vector<int> gap, lo, hi;  // per foldable: fixed ops before it, interval of gaps
    for (int r = begin; r < *end; r++) {
      const FOp& f = pp->ops[r];
      if (reg_diag(f) || reg_sign(f)) {
        fold.push_back(f);
        gap.push_back((int)fixed.size());
      } else {
        fixed.push_back(f);
      }
    }
    const int nf = (int)fold.size(), m = (int)fixed.size();
    if (nf > 1) {
      lo.resize(nf);
      hi.resize(nf);
      for (int i = 0; i < nf; i++) {
        const unsigned sl = fold_slots(fold[i]);
        int a = gap[i];
        while (a > 0 && !(mixing_slots(fixed[a - 1]) & sl)) a--;
        int b = gap[i];
        while (b < m && !(mixing_slots(fixed[b]) & sl)) b++;
        lo[i] = a;
        hi[i] = b;
      }
      std::vector<int> order(nf), at(nf, -1);
      for (int i = 0; i < nf; i++) order[i] = i;
      std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hi[x] < hi[y]; });
      for (int k = 0; k < nf; k++) {
        const int i = order[k];
        if (at[i] >= 0) continue;
        const int pnt = hi[i];
        for (int j = 0; j < nf; j++)
          if (at[j] < 0 && lo[j] <= pnt && pnt <= hi[j]) at[j] = pnt;
      }
      int w = begin;
      for (int g = 0; g <= m; g++) {
        for (int i = 0; i < nf; i++)
          if (at[i] == g) pp->ops[w++] = fold[i];
        if (g < m) pp->ops[w++] = fixed[g];
      }
    }
  }
  int w = begin;
  for (int r = begin; r < *end;) {
    if (!reg_diag(pp->ops[r]) && !reg_sign(pp->ops[r])) {
      pp->ops[w++] = pp->ops[r++];
      continue;
    }
    int e = r, ndiag = 0;
    while (e < *end && (reg_diag(pp->ops[e]) || reg_sign(pp->ops[e]))) ndiag += reg_diag(pp->ops[e++]);
    if (ndiag == 0 || e - r < 2 || *slack < 16) {
      while (r < e) pp->ops[w++] = pp->ops[r++];
      continue;
    }
    std::complex<double> tab[16];
    for (int j = 0; j < 16; j++) tab[j] = 1.0;
    for (int q = r; q < e; q++) {
      const FOp& f = pp->ops[q];
      if (!reg_diag(f)) {
        for (int j = 0; j < 16; j++)
          if ((f.neg[0] >> j) & 1) tab[j] = -tab[j];
        continue;
      }
      for (int j = 0; j < 16; j++) {
        if (!((f.jmask >> j) & 1)) continue;  // register controls: the entry is 1 elsewhere
        const int c = (int)f.coef + rpart_of(f, j);
        const HostOp& h = prog->ops[(*src)[2 * c]];
        const int ent = (*src)[2 * c + 1];
        tab[j] *= std::complex<double>(h.m[2 * ent], h.m[2 * ent + 1]);
      }
    }
    FOp m;
    memset(&m, 0, sizeof(m));
    m.type = FOP_DIAGR;
    m.jmask = 0xffffu;
    m.coef = (uint32_t)*ncoef;
    for (int j = 0; j < 16; j++) {
      const double re_im[2] = {tab[j].real(), tab[j].imag()};
      pp->coef[(*ncoef)++] = to_elem<T>(re_im);
      src->push_back(-1);  // a product of several ops' entries: not refillable per circuit
      src->push_back(j);
    }
    *slack -= 16;
    pp->ops[w++] = m;
    r = e;
  }
  *end = w;
}

// one op of a phase: its program index and the local tile bits of its dense targets
struct Pending {
  int op;
  int lt[2];
};

// Phase packing: ops are placed by their dependencies rather than
// in program order.  An op depends on the earlier ops of the pass it does not commute
// with (two diagonals commute; a diagonal and a dense op commute unless the dense op
// targets one of the diagonal's bits; dense ops commute when they share no qubit).  A
// phase takes its register bits from the first ready dense ops and then every ready
// op whose dense targets fit them, in program order, so a block of qubits runs as many
// layers as its light cone allows before the tile is exchanged.  One-qubit diagonals
// wait for a phase holding their qubit in the registers (where they fold into the
// phase's diagonal table) and join just before the first gate that needs them.
static void pack_phases(const sv_program* prog, const std::vector<int>& sched, const int* local_of,
                        std::vector<std::vector<Pending>>* groups, std::vector<std::vector<int>>* group_bits) {
  const int m = (int)sched.size();
  std::vector<uint64_t> tbits(m), allbits(m);
  std::vector<char> diag(m), one_diag(m);
  for (int i = 0; i < m; i++) {
    const HostOp& h = prog->ops[sched[i]];
    uint64_t t = 0, a = 0;
    for (int k = 0; k < h.nt; k++) t |= 1ull << h.tpos[k];
    a = t;
    for (int k = 0; k < h.nc; k++) a |= 1ull << h.cpos[k];
    tbits[i] = t;
    allbits[i] = a;
    diag[i] = !dense_like(h) && h.kind != OP_GRAD;
    one_diag[i] = diag[i] && h.nt == 1 && h.nc == 0;
  }
  auto commute = [&](int i, int j) {
    if (diag[i] && diag[j]) return true;
    if (diag[i]) return (tbits[j] & allbits[i]) == 0;
    if (diag[j]) return (tbits[i] & allbits[j]) == 0;
    return (allbits[i] & allbits[j]) == 0;
  };
  std::vector<std::vector<int>> preds(m);
  for (int i = 0; i < m; i++)
    for (int j = 0; j < i; j++)
      if (!commute(i, j)) preds[i].push_back(j);
  std::vector<char> done(m, 0);
  int left = m;
  while (left > 0) {
    std::vector<Pending> cur;
    std::vector<int> bits;
    auto ready = [&](int i) {
      for (int j : preds[i])
        if (!done[j]) return false;
      return true;
    };
    auto place = [&](int i) {
      Pending pd{sched[i], {-1, -1}};
      const HostOp& h = prog->ops[sched[i]];
      if (!diag[i])
        for (int k = 0; k < h.nt; k++) pd.lt[k] = local_of[h.tpos[k]];
      cur.push_back(pd);
      done[i] = 1;
      left--;
    };
    for (int i = 0; i < m; i++) {
      if (done[i]) continue;
      if (diag[i]) {
        // a one-qubit diagonal goes with the first dense op on its qubit (below), in the
        // phase that op runs in, or to the last phase when no later op needs it
        if (one_diag[i]) continue;
        if (ready(i)) place(i);
        continue;
      }
      // a dense op: its one-qubit diagonal predecessors on its own targets join first
      bool ok = true;
      for (int j : preds[i])
        if (!done[j] && !(one_diag[j] && (tbits[j] & tbits[i]) && ready(j))) ok = false;
      if (!ok) continue;
      const HostOp& h = prog->ops[sched[i]];
      std::vector<int> nb = bits;
      for (int k = 0; k < h.nt; k++) {
        const int lb = local_of[h.tpos[k]];
        if (std::find(nb.begin(), nb.end(), lb) == nb.end()) nb.push_back(lb);
      }
      if ((int)nb.size() > kRB) continue;
      bits = nb;
      for (int j : preds[i])
        if (!done[j]) place(j);
      place(i);
    }
    if (cur.empty()) {
      // only one-qubit diagonals whose qubit no later phase holds are left (they commute
      // with each other): they join the last phase
      for (int i = 0; i < m; i++)
        if (!done[i]) place(i);
      if (!groups->empty()) {
        groups->back().insert(groups->back().end(), cur.begin(), cur.end());
        continue;
      }
    }
    groups->push_back(cur);
    group_bits->push_back(bits);
  }
}

template <typename T>
static void encode_pass(const sv_program* prog, const std::vector<int>& sched, uint64_t S, PassParams<T>* pp,
                        int* nphases_out, std::vector<int32_t>* src) {
  const int n = prog->nqubits, kt = prog->kt;
  memset(pp, 0, sizeof(*pp));
  pp->n = n;
  pp->kt = kt;
  pp->ntiles = (int64_t)1 << (n - kt);
  int local_of[64];
  for (int b = 0, k = 0; b < 64; b++) {
    local_of[b] = -1;
    if (b < n && ((S >> b) & 1)) {
      pp->tile_pos[k] = b;
      local_of[b] = k++;
    }
  }
  // group ops into phases by register bits (order preserved)
  std::vector<std::vector<Pending>> groups;
  std::vector<std::vector<int>> group_bits;
  std::vector<int> cur_bits;
  std::vector<Pending> cur;
  auto flush = [&]() {
    if (cur.empty()) return;
    groups.push_back(cur);
    group_bits.push_back(cur_bits);
    cur.clear();
    cur_bits.clear();
  };
  if (prog->pack_phases) {
    pack_phases(prog, sched, local_of, &groups, &group_bits);
  } else {
  // diagonal ops wait for the next dense op and join its phase: a diagonal emitted just
  // before a gate on its qubit then finds that qubit in the registers
  std::vector<Pending> held;
  for (int oi : sched) {
    const HostOp& h = prog->ops[oi];
    Pending pd{oi, {-1, -1}};
    if (!dense_like(h)) {
      held.push_back(pd);
      continue;
    }
    for (int i = 0; i < h.nt; i++) pd.lt[i] = local_of[h.tpos[i]];
    int need = 0;
    for (int i = 0; i < h.nt; i++)
      if (std::find(cur_bits.begin(), cur_bits.end(), pd.lt[i]) == cur_bits.end()) need++;
    if ((int)cur_bits.size() + need > kRB) flush();
    for (int i = 0; i < h.nt; i++)
      if (std::find(cur_bits.begin(), cur_bits.end(), pd.lt[i]) == cur_bits.end()) cur_bits.push_back(pd.lt[i]);
    cur.insert(cur.end(), held.begin(), held.end());
    held.clear();
    cur.push_back(pd);
  }
  cur.insert(cur.end(), held.begin(), held.end());
  flush();
  }
  int nops = 0, ncoef = 0, ngrad = 0;
  // coefficient slots left beyond those the scheduled ops need: room for the copies and
  // tables that run merging and diagonal folding add
  int slack = kCoefBytes / (int)sizeof(T);
  for (int oi : sched) slack -= coef_cost(prog->ops[oi]);
  for (size_t g = 0; g < groups.size(); g++) {
    std::vector<int> rb = group_bits[g];
    for (int b = kt - 1; b >= 0 && (int)rb.size() < kRB; b--)
      if (std::find(rb.begin(), rb.end(), b) == rb.end()) rb.push_back(b);
    std::sort(rb.begin(), rb.end());
    int regpos[kMaxTile];
    for (int b = 0; b < kt; b++) regpos[b] = -1;
    for (int u = 0; u < kRB; u++) regpos[rb[u]] = u;
    Phase& P = pp->phases[g];
    for (int u = 0; u < kRB; u++) P.rb[u] = (uint8_t)rb[u];
    for (int j = 0; j < 16; j++) {
      int off = 0;
      for (int u = 0; u < kRB; u++)
        if ((j >> u) & 1) off |= 1 << rb[u];
      P.soff[j] = (uint16_t)smem_pos(off);
    }
    P.op_begin = (uint16_t)nops;
    for (const Pending& pd : groups[g]) {
      const HostOp& h = prog->ops[pd.op];
      FOp& f = pp->ops[nops++];
      memset(&f, 0, sizeof(f));
      // controls: register-level (reg_c), thread-level (tmask), tile-level (omask)
      unsigned reg_c = 0;
      for (int i = 0; i < h.nc; i++) {
        const int lc = local_of[h.cpos[i]];
        if (lc < 0) f.omask |= 1ull << h.cpos[i];
        else if (regpos[lc] >= 0) reg_c |= 1u << regpos[lc];
        else f.tmask |= 1u << lc;
      }
      unsigned jm = 0;
      unsigned tbits = 0;  // register bits that are targets of a dense op
      if (h.kind == OP_GRAD && h.gen != 3) {
        f.type = h.gen == 1 ? FOP_GRADX : FOP_GRADY;
        f.u0 = (uint8_t)regpos[pd.lt[0]];
        f.u1 = (uint8_t)(ngrad++);  // shared-memory accumulator slot
        f.coef = (uint32_t)h.param;
        f.jmask = 0xffffu;
      } else if (h.kind == OP_GRAD) {
        // Z generator: a one-bit "diagonal" read like FOP_DIAG's index bits
        f.type = FOP_GRADZ;
        f.u1 = (uint8_t)(ngrad++);
        f.coef = (uint32_t)h.param;
        f.nd = 1;
        f.jmask = 0xffffu;
        for (int i = 0; i < 3; i++) {
          f.tb[i] = -1;
          f.ob[i] = -1;
        }
        const int lb = local_of[h.tpos[0]];
        uint64_t rpart = 0;
        if (lb >= 0 && regpos[lb] >= 0) {
          for (int j = 0; j < 16; j++)
            if ((j >> regpos[lb]) & 1) rpart |= (uint64_t)1 << (4 * j);
        } else if (lb >= 0) {
          f.tb[0] = (int8_t)lb;
        } else {
          f.ob[0] = (int8_t)h.tpos[0];
        }
        f.rpart = rpart;
      } else if (h.kind == SV_OP_DENSE) {
        if (h.nt == 1)
          f.type = h.is_x ? FOP_X1 : (h.unit_cols >= 0 ? FOP_DENSE1P : (h.is_real ? FOP_DENSE1R : FOP_DENSE1));
        else
          f.type = h.is_swap ? FOP_SWAP2 : FOP_DENSE2;
        f.u0 = (uint8_t)regpos[pd.lt[0]];
        tbits = 1u << f.u0;
        if (h.nt == 2) {
          f.u1 = (uint8_t)regpos[pd.lt[1]];
          tbits |= 1u << f.u1;
        }
        for (int j = 0; j < 16; j++)
          if (!(j & tbits) && (j & reg_c) == reg_c) jm |= 1u << j;
        if (reg_c == 0) jm = 0xffffu;  // no register-level controls: kernel skips the tests
        f.jmask = (uint16_t)jm;
        f.coef = (uint32_t)ncoef;
        if (f.type == FOP_DENSE1P) {
          // coefficients: row i's ratio, the entry beside its unit
          f.u1 = (uint8_t)h.unit_cols;
          for (int i = 0; i < 2; i++) {
            const int e = 2 * i + (((h.unit_cols >> i) & 1) ? 0 : 1);
            src->push_back(pd.op);
            src->push_back(e);
            pp->coef[ncoef++] = to_elem<T>(&h.m[2 * e]);
          }
        } else {
          const int ne = coef_cost(h);
          for (int i = 0; i < ne; i++) {
            src->push_back(pd.op);
            src->push_back(i);
            pp->coef[ncoef++] = to_elem<T>(&h.m[2 * i]);
          }
        }
      } else {
        f.nd = (uint8_t)h.nt;
        for (int j = 0; j < 16; j++)
          if ((j & reg_c) == reg_c) jm |= 1u << j;
        f.jmask = (uint16_t)jm;
        uint64_t rpart = 0;
        unsigned nonreg_bits = 0;  // table-index bits fed by thread or outer bits
        for (int i = 0; i < 3; i++) {
          f.tb[i] = -1;
          f.ob[i] = -1;
        }
        for (int i = 0; i < h.nt; i++) {
          const int sh = h.nt - 1 - i;
          const int lb = local_of[h.tpos[i]];
          if (lb >= 0 && regpos[lb] >= 0) {
            for (int j = 0; j < 16; j++)
              if ((j >> regpos[lb]) & 1) rpart |= (uint64_t)1 << (4 * j + sh);
          } else if (lb >= 0) {
            f.tb[i] = (int8_t)lb;
            nonreg_bits |= 1u << sh;
          } else {
            f.ob[i] = (int8_t)h.tpos[i];
            nonreg_bits |= 1u << sh;
          }
        }
        f.rpart = rpart;
        if (h.sign_only) {
          f.type = FOP_SIGN;
          for (int tp = 0; tp < 8; tp++) {
            if (tp & ~nonreg_bits) continue;
            unsigned nm = 0;
            for (int j = 0; j < 16; j++) {
              const int idx = (int)((rpart >> (4 * j)) & 15) | tp;
              if (((jm >> j) & 1) && ((h.sign_mask >> idx) & 1)) nm |= 1u << j;
            }
            f.neg[tp] = (uint16_t)nm;
          }
        } else {
          f.type = FOP_DIAG;
          f.coef = (uint32_t)ncoef;
          for (int i = 0; i < (1 << h.nt); i++) {
            src->push_back(pd.op);
            src->push_back(i);
            pp->coef[ncoef++] = to_elem<T>(&h.m[2 * i]);
          }
        }
      }
    }
    if (prog->fold_diagonals) fold_register_diagonals<T>(prog, pp, P.op_begin, &nops, &ncoef, &slack, src);
    merge_signs(pp->ops, P.op_begin, &nops);
    // merge runs of uncontrolled one-target dense ops into FOP_D1RUN / FOP_D1RUNR records
    {
      int w = P.op_begin;
      for (int r = P.op_begin; r < nops;) {
        FOp f = pp->ops[r];
        const bool plain1 = (f.type == FOP_DENSE1 || f.type == FOP_DENSE1R) && f.omask == 0 && f.tmask == 0 &&
                            f.jmask == 0xffffu;
        if (!plain1) {
          pp->ops[w++] = f;
          r++;
          continue;
        }
        FOp run;
        memset(&run, 0, sizeof(run));
        run.type = f.type == FOP_DENSE1 ? FOP_D1RUN : FOP_D1RUNR;
        int k = 0;
        unsigned used = 0;
        uint32_t gcoef[4];
        bool contiguous = true;
        // a run holds gates on distinct register bits, which commute
        while (r < nops && k < 4) {
          const FOp& g2 = pp->ops[r];
          const bool ok = g2.type == f.type && g2.omask == 0 && g2.tmask == 0 && g2.jmask == 0xffffu &&
                          !((used >> g2.u0) & 1u);
          if (!ok) break;
          used |= 1u << g2.u0;
          gcoef[k] = g2.coef;
          contiguous &= g2.coef == f.coef + 4u * (unsigned)k;
          run.ru[k++] = g2.u0;
          r++;
        }
        run.nrun = (uint8_t)k;
        // the run's matrices back to back (four entries each): in place when the gates'
        // coefficients already are, else copied to the end of the pass's array; four
        // gates are sorted into register order 0..3
        const bool sort4 = k == 4;
        if (contiguous && !sort4) {
          run.coef = f.coef;
        } else if (!contiguous && slack < 4 * k) {
          // no room for a copy: leave the gates as single-gate runs in place
          for (int q = 0; q < k; q++) {
            FOp one = run;
            one.nrun = 1;
            one.ru[0] = run.ru[q];
            one.coef = gcoef[q];
            pp->ops[w++] = one;
          }
          continue;
        } else {
          T tmp[16];
          int32_t tsrc[32];
          for (int q = 0; q < k; q++) {
            const int to_gate = sort4 ? run.ru[q] : q;
            for (int e = 0; e < 4; e++) {
              const int from = (int)gcoef[q] + e, to = 4 * to_gate + e;
              tmp[to] = pp->coef[from];
              tsrc[2 * to] = (*src)[2 * from];
              tsrc[2 * to + 1] = (*src)[2 * from + 1];
            }
          }
          run.coef = contiguous ? f.coef : (uint32_t)ncoef;
          if (!contiguous) {
            ncoef += 4 * k;
            slack -= 4 * k;
            src->resize(2 * (size_t)ncoef);
          }
          for (int e = 0; e < 4 * k; e++) {
            pp->coef[run.coef + e] = tmp[e];
            (*src)[2 * (run.coef + e)] = tsrc[2 * e];
            (*src)[2 * (run.coef + e) + 1] = tsrc[2 * e + 1];
          }
          if (sort4)
            for (int q = 0; q < 4; q++) run.ru[q] = (uint8_t)q;
        }
        pp->ops[w++] = run;
      }
      nops = w;
    }
    for (int q = P.op_begin; q < nops; q++) {
      FOp& f = pp->ops[q];
      f.flags = (uint8_t)((f.omask ? FLAG_OMASK : 0) | (f.tmask ? FLAG_TMASK : 0));
    }
    P.op_end = (uint16_t)nops;
  }
  pp->nphases = (int)groups.size();
  pp->nops = nops;
  *nphases_out = (int)groups.size();
}

template <typename T>
static int build_program(sv_program* prog) {
  const int n = prog->nqubits;
  const int kt = prog->kt;
  // folded programs leave a quarter of the coefficient slots for the encoder's run copies
  // and register-diagonal tables (about 24 slots per phase)
  const int coef_cap = (kCoefBytes / (int)sizeof(T)) * (prog->fold_diagonals ? 3 : 4) / 4;
  // folded programs encode more, smaller ops; the adjoint sweep keeps one shared-memory
  // gradient slot per op of a pass, so refilled programs stay at the smaller bound
  const int max_ops = prog->fold_diagonals ? kMaxPassOps : kMaxPassOpsRefill;
  prog->pass_bytes = sizeof(PassParams<T>);
  // split at unfusable ops (dense on more than 2 targets, diagonal on more than 3)
  std::vector<std::vector<int>> runs(1);
  std::vector<int> barriers;
  for (size_t i = 0; i < prog->ops.size(); i++) {
    const HostOp& h = prog->ops[i];
    const bool fusable =
        (h.kind == SV_OP_DIAG && h.nt <= 3) || (h.kind == SV_OP_DENSE && h.nt <= 2) || h.kind == OP_GRAD;
    if (fusable) {
      runs.back().push_back((int)i);
    } else {
      barriers.push_back((int)i);
      runs.emplace_back();
    }
  }
  for (size_t r = 0; r < runs.size(); r++) {
    std::vector<int> rem = runs[r];
    while (!rem.empty()) {
      // greedy in gate order: a gate joins while its dense targets fit in the tile
      // and none of its qubits is held back by an earlier gate left for later
      uint64_t S = (1ull << kLowBits) - 1;
      int ssize = kLowBits;
      uint64_t blocked = 0;
      int nops = 0, ncoef = 0;
      bool full = false;
      std::vector<int> sched, next;
      // would op h join now, with `extra_ops` / `extra_coef` taken by ops joining before it
      auto fits = [&](const HostOp& h, int extra_ops, int extra_coef, bool* fills) {
        uint64_t tbits = 0, bits = 0;
        for (int i = 0; i < h.nt; i++) tbits |= 1ull << h.tpos[i];
        bits = tbits;
        for (int i = 0; i < h.nc; i++) bits |= 1ull << h.cpos[i];
        const bool over = nops + extra_ops + 1 > max_ops || ncoef + extra_coef + coef_cost(h) > coef_cap;
        *fills = over;
        if (full || (bits & blocked) || over) return false;
        return !dense_like(h) || ssize + __builtin_popcountll(tbits & ~S) <= kt;
      };
      auto take = [&](int oi) {
        const HostOp& h = prog->ops[oi];
        if (dense_like(h))
          for (int i = 0; i < h.nt; i++)
            if (!((S >> h.tpos[i]) & 1)) {
              S |= 1ull << h.tpos[i];
              ssize++;
            }
        sched.push_back(oi);
        nops++;
        ncoef += coef_cost(h);
      };
      auto leave = [&](int oi, bool fills) {
        const HostOp& h = prog->ops[oi];
        if (fills) full = true;
        for (int i = 0; i < h.nt; i++) blocked |= 1ull << h.tpos[i];
        for (int i = 0; i < h.nc; i++) blocked |= 1ull << h.cpos[i];
        next.push_back(oi);
      };
      for (size_t k = 0; k < rem.size(); k++) {
        const int oi = rem[k];
        const HostOp& h = prog->ops[oi];
        bool fills = false;
        // a one-bit diagonal directly before a dense op on the same bit (the phases that
        // fold_phases carries to the next dense op) goes with that op: left behind alone,
        // it would cost a full complex multiply here instead of joining the next pass's
        // register-diagonal table
        if (h.kind == SV_OP_DIAG && h.nt == 1 && h.nc == 0 && k + 1 < rem.size()) {
          const HostOp& nx = prog->ops[rem[k + 1]];
          if (dense_like(nx) && nx.nt == 1 && nx.tpos[0] == h.tpos[0]) {
            bool fd = false, fn = false;
            if (fits(h, 0, 0, &fd) && fits(nx, 1, coef_cost(h), &fn)) {
              take(oi);
              take(rem[k + 1]);
            } else {
              leave(oi, fd || fn);
              leave(rem[k + 1], false);
            }
            k++;
            continue;
          }
        }
        if (fits(h, 0, 0, &fills)) take(oi);
        else leave(oi, fills);
      }
      for (int b = 0; b < n && ssize < kt; b++)
        if (!((S >> b) & 1)) {
          S |= 1ull << b;
          ssize++;
        }
      const size_t off = prog->passes.size();
      prog->passes.resize(off + sizeof(PassParams<T>));
      int nph = 0;
      std::vector<int32_t> src;
      encode_pass<T>(prog, sched, S, reinterpret_cast<PassParams<T>*>(prog->passes.data() + off), &nph, &src);
      reinterpret_cast<PassParams<T>*>(prog->passes.data() + off)->coef_goff = (int32_t)prog->coef_total;
      prog->pass_coef_off.push_back(prog->coef_total);
      prog->coef_total += src.size() / 2;
      prog->coef_src.insert(prog->coef_src.end(), src.begin(), src.end());
      Segment seg;
      seg.fused = true;
      seg.pass = prog->npasses;
      prog->segments.push_back(seg);
      prog->npasses++;
      prog->nphases += nph;
      prog->nfused_gates += (int)sched.size();
      rem.swap(next);
    }
    if (r < barriers.size()) {
      Segment seg;
      seg.host_op = barriers[r];
      prog->segments.push_back(seg);
      prog->nunfused++;
    }
  }
  return SV_OK;
}


template <typename T, int MAXT, int MINB, bool BATCHED>
static int launch_variant(Context* ctx, cudaStream_t stream, const PassParams<T>& p, void* state, int threads,
                          size_t smem, int64_t nitems, const BatchArgs<T>& batch) {
  auto kern = k_fused_pass<T, MAXT, MINB, BATCHED>;
  // the attribute is one value per kernel: raise it to the largest tile ever run
  static size_t attr_bytes = 0;
  if (smem > attr_bytes) {
    SV_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                      "fused pass smem attribute"));
    attr_bytes = smem;
  }
  static int per_sm_cache[kMaxTile + 1] = {0};
  int& per_sm = per_sm_cache[p.kt];
  if (per_sm == 0) {
    SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem),
                      "fused pass occupancy"));
    if (per_sm < 1) return set_error(SV_ERR_ARG, "tile of 2^%d amplitudes does not fit on an SM", p.kt);
  }
  int64_t grid = (int64_t)per_sm * ctx->num_sms;
  if (grid > nitems) grid = nitems;
  kern<<<(unsigned)grid, threads, smem, stream>>>((T*)state, p, batch);
  SV_LAUNCH_CHECK("fused pass launch");
  return SV_OK;
}

template <typename T, bool BATCHED = false>
static int launch_pass(Context* ctx, const PassParams<T>& p, void* state, int threads, size_t smem, int64_t nitems,
                       cudaStream_t stream, const BatchArgs<T>& batch = BatchArgs<T>{}) {
  if constexpr (stored_as_double_pairs<T>::value) {
    // double-word tiles of up to 2^11 amplitudes: three 128-thread CTAs fit an SM's shared
    // memory, so the registers are sized for three (the whole file would allow two)
    if (threads <= 128) return launch_variant<T, 128, 3, BATCHED>(ctx, stream, p, state, threads, smem, nitems, batch);
    return launch_variant<T, 256, 1, BATCHED>(ctx, stream, p, state, threads, smem, nitems, batch);
  } else if constexpr (sizeof(T) >= 16) {
    return launch_variant<T, 256, 1, BATCHED>(ctx, stream, p, state, threads, smem, nitems, batch);
  } else {
    if (threads <= 256) return launch_variant<T, 256, 3, BATCHED>(ctx, stream, p, state, threads, smem, nitems, batch);
    return launch_variant<T, 512, 1, BATCHED>(ctx, stream, p, state, threads, smem, nitems, batch);
  }
}

template <typename T>
static int run_program(Context* ctx, const sv_program* prog, void* state) {
  constexpr bool kDW = stored_as_double_pairs<T>::value;
  const std::vector<unsigned char>& blocks = kDW ? prog->passes_dw : prog->passes;
  const bool spec = prog->spec && specialized_is_dw(prog->spec) == kDW;
  const int n = prog->nqubits, kt = prog->kt;
  const size_t smem = pass_smem<T>(kt);
  const int threads = 1 << (kt - kRB);
  if (threads > fused_max_threads<T>())
    return set_error(SV_ERR_ARG, "tile_bits %d too large for this dtype (at most %d)", kt,
                     kRB + (sizeof(T) >= 16 ? 8 : 9));
  const int64_t ntiles = (int64_t)1 << (n - kt);
  for (const Segment& s : prog->segments) {
    if (s.fused) {
      const PassParams<T>& p =
          *reinterpret_cast<const PassParams<T>*>(blocks.data() + (size_t)s.pass * prog->pass_bytes);
      if (spec) SV_TRY(specialized_launch(ctx, prog, s.pass, state));
      else SV_TRY(launch_pass<T>(ctx, p, state, threads, smem, ntiles, ctx->stream));
    } else {
      const HostOp& h = prog->ops[s.host_op];
      std::vector<int32_t> targets(h.nt), qubits;
      for (int i = 0; i < h.nt; i++) {
        targets[i] = n - 1 - h.tpos[i];
        qubits.push_back(h.tpos[i]);
      }
      for (int i = 0; i < h.nc; i++) qubits.push_back(h.cpos[i]);
      std::sort(qubits.begin(), qubits.end());
      const size_t d = (size_t)1 << h.nt;
      using E = typename std::conditional<kDW, c128, T>::type;  // the operand in the state's dtype
      std::vector<E> dense(d * d);
      if (h.kind == SV_OP_DIAG) {  // a diagonal on more than 3 bits: apply as a dense matrix
        const double zero[2] = {0.0, 0.0};
        for (size_t i = 0; i < d * d; i++) dense[i] = to_elem<E>(zero);
        for (size_t i = 0; i < d; i++) dense[i * d + i] = to_elem<E>(&h.m[2 * i]);
      } else {
        for (size_t i = 0; i < d * d; i++) dense[i] = to_elem<E>(&h.m[2 * i]);
      }
      SV_TRY(sv_apply_multi_qubit(static_cast<sv_context*>(ctx), state, prog->dtype, n, dense.data(), targets.data(),
                                  h.nt, qubits.data(), (int)qubits.size()));
    }
  }
  return SV_OK;
}

static void classify(HostOp& h) {
  const size_t ne = h.kind == SV_OP_DENSE ? ((size_t)1 << (2 * h.nt)) : ((size_t)1 << h.nt);
  h.sign_only = false;
  h.sign_mask = 0;
  h.is_x = h.is_real = h.is_swap = false;
  if (h.kind == SV_OP_DIAG) {
    h.sign_only = true;
    for (size_t e = 0; e < ne; e++) {
      const double re = h.m[2 * e], im = h.m[2 * e + 1];
      if (im != 0.0 || (re != 1.0 && re != -1.0)) h.sign_only = false;
      if (re == -1.0 && im == 0.0) h.sign_mask |= 1 << e;
    }
    return;
  }
  h.is_real = true;
  for (size_t e = 0; e < ne; e++)
    if (h.m[2 * e + 1] != 0.0) h.is_real = false;
  auto is = [&](const double* want, size_t n) {
    for (size_t e = 0; e < n; e++)
      if (h.m[2 * e] != want[e] || h.m[2 * e + 1] != 0.0) return false;
    return true;
  };
  static const double X[4] = {0, 1, 1, 0};
  static const double SW[16] = {1, 0, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, 1};
  if (h.nt == 1) h.is_x = is(X, 4);
  if (h.nt == 2) h.is_swap = is(SW, 16);
}

// 2x2 of a one-target op (diagonal ops expanded), complex (re, im) pairs
static void as_dense2x2(const HostOp& h, double out[8]) {
  if (h.kind == SV_OP_DENSE) {
    for (int i = 0; i < 8; i++) out[i] = h.m[i];
  } else {
    const double d[8] = {h.m[0], h.m[1], 0, 0, 0, 0, h.m[2], h.m[3]};
    for (int i = 0; i < 8; i++) out[i] = d[i];
  }
}

// Consecutive uncontrolled one-target gates on the same qubit (no other gate touching
// that qubit in between) are multiplied into one 2x2: fewer ops, same result.
static void merge_single_qubit(std::vector<HostOp>& ops, int nqubits) {
  std::vector<HostOp> out;
  std::vector<int> last(64, -1);  // index in `out` of the last op touching each bit
  for (HostOp& h : ops) {
    const bool single = h.nt == 1 && h.nc == 0;
    const int t = h.tpos[0];
    if (single && last[t] >= 0) {
      HostOp& p = out[last[t]];
      if (p.nt == 1 && p.nc == 0 && p.tpos[0] == t) {
        if (p.kind == SV_OP_DIAG && h.kind == SV_OP_DIAG) {
          for (int e = 0; e < 2; e++) {
            const double ar = h.m[2 * e], ai = h.m[2 * e + 1], br = p.m[2 * e], bi = p.m[2 * e + 1];
            p.m[2 * e] = ar * br - ai * bi;
            p.m[2 * e + 1] = ar * bi + ai * br;
          }
        } else {
          double A[8], B[8], C[8];
          as_dense2x2(h, A);  // applied second
          as_dense2x2(p, B);
          for (int r = 0; r < 2; r++)
            for (int c = 0; c < 2; c++) {
              double re = 0, im = 0;
              for (int k = 0; k < 2; k++) {
                const double ar = A[2 * (2 * r + k)], ai = A[2 * (2 * r + k) + 1];
                const double br = B[2 * (2 * k + c)], bi = B[2 * (2 * k + c) + 1];
                re += ar * br - ai * bi;
                im += ar * bi + ai * br;
              }
              C[2 * (2 * r + c)] = re;
              C[2 * (2 * r + c) + 1] = im;
            }
          p.kind = SV_OP_DENSE;
          p.m.assign(C, C + 8);
        }
        classify(p);
        continue;
      }
    }
    out.push_back(h);
    const int idx = (int)out.size() - 1;
    for (int i = 0; i < h.nt; i++) last[h.tpos[i]] = idx;
    for (int i = 0; i < h.nc; i++) last[h.cpos[i]] = idx;
  }
  (void)nqubits;
  ops.swap(out);
}

// Phase folding (programs run through sv_program_create only).  Every uncontrolled
// one-qubit gate with complex entries is written as D1 R D2: two diagonal phases and a
// real 2x2 (a unitary 2x2 always separates so: |U_ij| e^{i(a_i + b_j)} up to signs).
// A real 2x2 costs half the multiply-adds of a complex one, and the diagonals of all
// gates commute with every diagonal gate (CZ, CU1, ...) and with gates on other qubits,
// so they are carried along per qubit, multiplied together, and emitted only before
// the next non-diagonal gate on their qubit.  For a layer of arbitrary one-qubit gates
// between entangling diagonal layers this leaves one real 2x2 and one diagonal per
// qubit and layer, and the encoder folds the diagonals of a phase's register bits into
// one 16-entry table (FOP_DIAGR): about 5 instead of 8 FP multiply-adds per amplitude
// and gate.
static bool phase_separate(const HostOp& h, double d1[4], double r[4], double d2[4]) {
  typedef std::complex<double> cd;
  const cd a(h.m[0], h.m[1]), b(h.m[2], h.m[3]), c(h.m[4], h.m[5]), d(h.m[6], h.m[7]);
  auto unit = [](cd z) { return std::abs(z) > 0 ? z / std::abs(z) : cd(1, 0); };
  cd p0, p1, q0, q1;
  if (std::abs(a) >= std::abs(b)) {
    p0 = unit(a);
    q0 = 1;
    q1 = unit(b) / p0;
  } else {
    p0 = unit(b);
    q1 = 1;
    q0 = unit(a) / p0;
  }
  p1 = std::abs(c) >= std::abs(d) ? unit(c) / q0 : unit(d) / q1;
  const cd m[4] = {a, b, c, d}, p[2] = {p0, p1}, q[2] = {q0, q1};
  double err = 0;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      const cd rij = std::conj(p[i]) * m[2 * i + j] * std::conj(q[j]);
      r[2 * i + j] = rij.real();
      err = std::max(err, std::abs(p[i] * rij.real() * q[j] - m[2 * i + j]));
    }
  if (err > 1e-13) return false;
  d1[0] = p0.real(), d1[1] = p0.imag(), d1[2] = p1.real(), d1[3] = p1.imag();
  d2[0] = q0.real(), d2[1] = q0.imag(), d2[2] = q1.real(), d2[3] = q1.imag();
  return true;
}

static void fold_phases(std::vector<HostOp>& ops) {
  typedef std::complex<double> cd;
  std::vector<HostOp> out;
  std::vector<cd> pend0(64, cd(1, 0)), pend1(64, cd(1, 0));
  std::vector<bool> pending(64, false);
  auto flush = [&](int t) {
    if (!pending[t]) return;
    pending[t] = false;
    const cd z0 = pend0[t], z1 = pend1[t];
    pend0[t] = pend1[t] = cd(1, 0);
    if (z0 == cd(1, 0) && z1 == cd(1, 0)) return;
    HostOp g;
    g.kind = SV_OP_DIAG;
    g.nt = 1;
    g.nc = 0;
    g.tpos[0] = t;
    g.m = {z0.real(), z0.imag(), z1.real(), z1.imag()};
    classify(g);
    out.push_back(std::move(g));
  };
  auto absorb = [&](int t, const double* dg) {  // pending diagonal of bit t times diag(dg)
    pend0[t] *= cd(dg[0], dg[1]);
    pend1[t] *= cd(dg[2], dg[3]);
    pending[t] = true;
  };
  for (HostOp& h : ops) {
    const bool one = h.nt == 1 && h.nc == 0;
    if (one && h.kind == SV_OP_DIAG) {
      absorb(h.tpos[0], h.m.data());
      continue;
    }
    double d1[4], r[4], d2[4];
    const bool real1 = one && h.kind == SV_OP_DENSE && h.is_real && !h.is_x;
    if (real1) {  // already real: no phases to separate
      for (int i = 0; i < 4; i++) r[i] = h.m[2 * i];
      d1[0] = d1[2] = d2[0] = d2[2] = 1.0;
      d1[1] = d1[3] = d2[1] = d2[3] = 0.0;
    }
    if (real1 || (one && h.kind == SV_OP_DENSE && !h.is_real && !h.is_x && phase_separate(h, d1, r, d2))) {
      const int t = h.tpos[0];
      absorb(t, d2);  // applied first
      flush(t);
      // R = diag(p0, p1) P: each row divided by its larger entry (|ratio| <= 1), the row
      // scales joining the diagonal that follows
      double pm[4], piv[2];
      int cols = 0;
      bool ok = true;
      for (int i = 0; i < 2 && ok; i++) {
        const double a = r[2 * i], b = r[2 * i + 1];
        if (a == 0.0 && b == 0.0) ok = false;
        else if (std::fabs(a) >= std::fabs(b)) {
          piv[i] = a;
          pm[2 * i] = 1.0;
          pm[2 * i + 1] = b / a;
        } else {
          piv[i] = b;
          pm[2 * i] = a / b;
          pm[2 * i + 1] = 1.0;
          cols |= 1 << i;
        }
      }
      HostOp g = h;
      if (ok) {
        g.m = {pm[0], 0.0, pm[1], 0.0, pm[2], 0.0, pm[3], 0.0};
        g.unit_cols = cols;
        const double dp[4] = {d1[0] * piv[0], d1[1] * piv[0], d1[2] * piv[1], d1[3] * piv[1]};
        for (int i = 0; i < 4; i++) d1[i] = dp[i];
      } else {
        g.m = {r[0], 0.0, r[1], 0.0, r[2], 0.0, r[3], 0.0};
      }
      classify(g);
      out.push_back(std::move(g));
      absorb(t, d1);
      continue;
    }
    // diagonal gates commute with the pending diagonals; other gates meet them on their targets
    if (h.kind != SV_OP_DIAG)
      for (int i = 0; i < h.nt; i++) flush(h.tpos[i]);
    out.push_back(h);
  }
  for (int t = 0; t < 64; t++) flush(t);
  ops.swap(out);
}

static int parse_ops(int nqubits, const sv_gate_op* ops, int nops, std::vector<HostOp>* out) {
  out->clear();
  for (int i = 0; i < nops; i++) {
    const sv_gate_op& g = ops[i];
    HostOp h;
    h.kind = g.kind;
    h.nt = g.ntargets;
    h.nc = g.ncontrols;
    const bool ok_kind = g.kind == SV_OP_DENSE || g.kind == SV_OP_DIAG;
    if (!ok_kind || g.ntargets < 1 || g.ntargets > kMaxTargets || g.ncontrols < 0 || g.ncontrols > 16 || !g.matrix)
      return set_error(SV_ERR_ARG, "op %d: bad kind, target count, control count or matrix", i);
    uint64_t seen = 0;
    for (int k = 0; k < g.ntargets + g.ncontrols; k++) {
      const int q = k < g.ntargets ? g.targets[k] : g.controls[k - g.ntargets];
      if (q < 0 || q >= nqubits || ((seen >> q) & 1))
        return set_error(SV_ERR_ARG, "op %d: qubit %d out of range or repeated", i, q);
      seen |= 1ull << q;
      if (k < g.ntargets) h.tpos[k] = nqubits - 1 - q;
      else h.cpos[k - g.ntargets] = nqubits - 1 - q;
    }
    const size_t ne = g.kind == SV_OP_DENSE ? ((size_t)1 << (2 * g.ntargets)) : ((size_t)1 << g.ntargets);
    h.m.assign(g.matrix, g.matrix + 2 * ne);
    classify(h);
    out->push_back(std::move(h));
  }
  merge_single_qubit(*out, nqubits);
  return SV_OK;
}

static int check_tile_bits(int dtype, int nqubits, int tile_bits, int* kt_out) {
  int kt = tile_bits;
  if (kt <= 0) kt = dtype == SV_C128 ? 11 : 12;
  if (kt > nqubits) kt = nqubits;
  const int kt_max = kRB + (dtype == SV_C128 ? 8 : 9);
  if (kt < kLowBits + kRB || kt > kt_max)
    return set_error(SV_ERR_ARG, "tile_bits must be in [%d, %d]", kLowBits + kRB, kt_max);
  *kt_out = kt;
  return SV_OK;
}

// complex128 programs also keep their pass blocks with every coefficient split into the
// nearest float pair (round to nearest, then the remainder), for the double-word kernels
static void make_dw_blocks(sv_program* prog) {
  static_assert(sizeof(PassParams<cw>) == sizeof(PassParams<c128>), "double-word blocks mirror complex128 ones");
  static_assert(offsetof(PassParams<cw>, coef) == offsetof(PassParams<c128>, coef), "same coefficient offset");
  prog->passes_dw = prog->passes;
  constexpr size_t ncoef = sizeof(PassParams<c128>::coef) / sizeof(c128);
  for (int i = 0; i < prog->npasses; i++) {
    const auto* src = reinterpret_cast<const PassParams<c128>*>(prog->passes.data() + (size_t)i * prog->pass_bytes);
    auto* dst = reinterpret_cast<PassParams<cw>*>(prog->passes_dw.data() + (size_t)i * prog->pass_bytes);
    for (size_t k = 0; k < ncoef; k++) dst->coef[k] = cw(src->coef[k].re, src->coef[k].im);
  }
}

static int plan(int dtype, int nqubits, int kt, std::vector<HostOp>&& ops, sv_program** out,
                bool fold_diagonals = false, bool pack = true) {
  if (kt > nqubits || kt < kLowBits + kRB) return set_error(SV_ERR_ARG, "tile of %d bits for %d qubits", kt, nqubits);
  sv_program* prog = new sv_program();
  prog->fold_diagonals = fold_diagonals;
  prog->pack_phases = pack;
  prog->dtype = dtype;
  prog->nqubits = nqubits;
  prog->kt = kt;
  prog->ops = std::move(ops);
  const int rc = dtype == SV_C128 ? build_program<c128>(prog) : build_program<c64>(prog);
  if (rc != SV_OK) {
    delete prog;
    return rc;
  }
  if (dtype == SV_C128) make_dw_blocks(prog);
  *out = prog;
  return SV_OK;
}

int refold_program(sv_program* prog) {
  if (prog->fold_diagonals) return SV_OK;
  fold_phases(prog->ops);
  prog->fold_diagonals = true;
  prog->segments.clear();
  prog->passes.clear();
  prog->coef_src.clear();
  prog->pass_coef_off.clear();
  prog->coef_total = 0;
  prog->npasses = prog->nunfused = prog->nfused_gates = prog->nphases = 0;
  if (prog->dtype != SV_C128) return build_program<c64>(prog);
  SV_TRY(build_program<c128>(prog));
  make_dw_blocks(prog);
  return SV_OK;
}

}  // namespace sv

using namespace sv;

extern "C" {

int sv_program_create(sv_context* ctx, int dtype, int nqubits, const sv_gate_op* ops, int nops, int tile_bits,
                      sv_program** out) {
  if (!ctx || !out) return set_error(SV_ERR_ARG, "null context or output");
  *out = nullptr;
  if (dtype != SV_C128 && dtype != SV_C64) return set_error(SV_ERR_UNSUPPORTED, "fused programs need a complex dtype");
  if (nqubits < kLowBits + kRB || nqubits > kMaxQubits)
    return set_error(SV_ERR_ARG, "fused programs need %d..%d qubits", kLowBits + kRB, kMaxQubits);
  if (nops < 0 || (nops > 0 && !ops)) return set_error(SV_ERR_ARG, "bad op list");
  int kt = 0;
  // complex128 passes are arithmetic-bound: phase folding (fewer multiply-adds) pays on
  // the interpreting kernel; in double-word arithmetic 2^11-amplitude tiles run fastest
  // (three CTAs per SM: 429 against 399 gates/s on the n=30 brickwork), in FP64 2^12.
  // Complex64 programs are folded when their passes are specialised (the interpreter
  // runs the unfolded plan faster)
  const bool fold = dtype == SV_C128;
  const int c128_default = ctx->c128_fp64 ? 12 : 11;
  SV_TRY(check_tile_bits(dtype, nqubits, tile_bits > 0 ? tile_bits : (fold ? c128_default : 0), &kt));
  std::vector<HostOp> hops;
  SV_TRY(parse_ops(nqubits, ops, nops, &hops));
  if (fold) fold_phases(hops);
  return plan(dtype, nqubits, kt, std::move(hops), out, fold);
}

int sv_program_run(sv_context* ctx, const sv_program* prog, void* state) {
  if (!ctx || !prog || !state) return set_error(SV_ERR_ARG, "null context, program or state");
  if (((uintptr_t)state) % 16) return set_error(SV_ERR_ARG, "state must be 16-byte aligned");
  if (prog->dtype == SV_C128)  // double-word arithmetic unless the context asks for FP64
    return ctx->c128_fp64 ? run_program<c128>(ctx, prog, state) : run_program<cw>(ctx, prog, state);
  return run_program<c64>(ctx, prog, state);
}

int sv_program_stats(const sv_program* prog, int* npasses, int* nunfused, int* nfused_gates, int* tile_bits) {
  if (!prog) return set_error(SV_ERR_ARG, "null program");
  if (npasses) *npasses = prog->npasses;
  if (nunfused) *nunfused = prog->nunfused;
  if (nfused_gates) *nfused_gates = prog->nfused_gates;
  if (tile_bits) *tile_bits = prog->kt;
  return SV_OK;
}

}  // extern "C"

namespace sv {
// arithmetic instructions per amplitude of one pass block under the pass kernels'
// register ops (lane instructions, FMUL and FFMA alike): complex 2x2 8 per amplitude it
// touches, real 2x2 4, pivoted real 2x2 2, complex 4x4 16, a diagonal or a diagonal
// table one complex multiply (4); sign flips, X and SWAP are register moves (0).  Ops
// under tile-level or thread-level controls count for the fraction of amplitudes their
// masks select; a dense op's register-level mask selects pair (or quadruple) bases.
template <typename T>
static double pass_arith_per_amplitude(const PassParams<T>& p) {
  double total = 0.0;
  for (int q = 0; q < p.nops; q++) {
    const FOp& f = p.ops[q];
    double cost = 0.0;
    // the register-level mask's bases: amplitudes for a diagonal, pair (quadruple) bases
    // with the target bit(s) clear for a dense op
    auto bases = [&](unsigned targets) {
      int c = 0;
      for (int j = 0; j < 16; j++)
        if (!(j & targets) && ((f.jmask >> j) & 1u)) c++;
      return (double)c;
    };
    switch (f.type) {
      case FOP_D1RUN: cost = 8.0 * f.nrun; break;
      case FOP_D1RUNR: cost = 4.0 * f.nrun; break;
      case FOP_DIAGR: cost = 4.0; break;
      case FOP_DENSE1: cost = 8.0 * bases(1u << f.u0) / 8.0; break;
      case FOP_DENSE1R: cost = 4.0 * bases(1u << f.u0) / 8.0; break;
      case FOP_DENSE1P: cost = 2.0 * bases(1u << f.u0) / 8.0; break;
      case FOP_DENSE2: cost = 16.0 * bases((1u << f.u0) | (1u << f.u1)) / 4.0; break;
      case FOP_DIAG: cost = 4.0 * bases(0) / 16.0; break;
      default: cost = 0.0; break;  // sign flips, register swaps, gradient markers
    }
    if (f.type != FOP_D1RUN && f.type != FOP_D1RUNR && f.type != FOP_DIAGR) {
      if (f.flags & FLAG_OMASK) cost /= (double)(1ull << __builtin_popcountll((unsigned long long)f.omask));
      if (f.flags & FLAG_TMASK) cost /= (double)(1u << __builtin_popcount(f.tmask));
    }
    total += cost;
  }
  return total;
}
static double program_arith_per_amplitude(const sv_program* prog) {
  double total = 0.0;
  for (int i = 0; i < prog->npasses; i++) {
    const unsigned char* b = prog->passes.data() + (size_t)i * prog->pass_bytes;
    total += prog->dtype == SV_C128 ? pass_arith_per_amplitude(*reinterpret_cast<const PassParams<c128>*>(b))
                                    : pass_arith_per_amplitude(*reinterpret_cast<const PassParams<c64>*>(b));
  }
  return total;
}
}  // namespace sv

extern "C" {

int sv_program_arith_per_amplitude(const sv_program* prog, double* out) {
  if (!prog || !out) return set_error(SV_ERR_ARG, "null argument");
  *out = program_arith_per_amplitude(prog);
  return SV_OK;
}

int sv_program_pass_params(const sv_program* prog, int pass, const void** params, size_t* bytes) {
  if (!prog || !params || !bytes) return set_error(SV_ERR_ARG, "null argument");
  if (pass < 0 || pass >= prog->npasses) return set_error(SV_ERR_ARG, "pass %d out of range", pass);
  *params = prog->passes.data() + (size_t)pass * prog->pass_bytes;
  *bytes = prog->pass_bytes;
  return SV_OK;
}

int sv_pass_layout(int dtype, int64_t* offsets, int n) {
  if (!offsets || n < 32) return set_error(SV_ERR_ARG, "the layout has 32 entries");
  if (dtype != SV_C128 && dtype != SV_C64) return set_error(SV_ERR_ARG, "pass blocks exist for complex dtypes");
  auto fill = [&](auto tag) {
    using P = decltype(tag);
    const int64_t o[32] = {
        (int64_t)sizeof(P), (int64_t)offsetof(P, n), (int64_t)offsetof(P, kt), (int64_t)offsetof(P, nphases),
        (int64_t)offsetof(P, nops), (int64_t)offsetof(P, ntiles), (int64_t)offsetof(P, tile_pos),
        (int64_t)offsetof(P, coef_goff), (int64_t)offsetof(P, phases), (int64_t)offsetof(P, ops),
        (int64_t)offsetof(P, coef), (int64_t)sizeof(Phase), (int64_t)offsetof(Phase, rb),
        (int64_t)offsetof(Phase, op_begin), (int64_t)offsetof(Phase, op_end), (int64_t)sizeof(FOp),
        (int64_t)offsetof(FOp, type), (int64_t)offsetof(FOp, u0), (int64_t)offsetof(FOp, u1),
        (int64_t)offsetof(FOp, nd), (int64_t)offsetof(FOp, tb), (int64_t)offsetof(FOp, ob),
        (int64_t)offsetof(FOp, jmask), (int64_t)offsetof(FOp, tmask), (int64_t)offsetof(FOp, coef),
        (int64_t)offsetof(FOp, omask), (int64_t)offsetof(FOp, rpart), (int64_t)offsetof(FOp, neg),
        (int64_t)offsetof(FOp, flags), (int64_t)offsetof(FOp, nrun), (int64_t)offsetof(FOp, ru),
        (int64_t)sizeof(P::coef[0])};
    for (int i = 0; i < 32; i++) offsets[i] = o[i];
  };
  if (dtype == SV_C128) fill(PassParams<c128>{});
  else fill(PassParams<c64>{});
  return SV_OK;
}

int sv_program_destroy(sv_program* prog) {
  if (prog && prog->spec) specialized_free(prog->spec);
  if (prog && prog->bspec) specialized_free(prog->bspec);
  if (prog && prog->aspec) specialized_free(prog->aspec);
  delete prog;
  return SV_OK;
}

}  // extern "C"

// ============================================================ batched circuits
// Thousands of circuits of uneven size run together: circuits with the same gate
// structure (same qubit count, same gates on the same qubits) form a group that is
// planned once; each circuit gets its own coefficient block gathered through the
// plan's coefficient-source map.  One run = zero all states, then every pass of every
// group as one batched launch (circuits x tiles), groups spread over several streams.
// The first run executes eagerly and records a CUDA graph of the same launches;
// later runs replay the graph.
namespace sv {

constexpr int kBatchStreams = 4;

struct BatchGroup {
  sv_program* prog = nullptr;
  std::vector<int> circuits;
  void* d_coef = nullptr;      // ncirc x coef_total elements
  void* d_coef_dw = nullptr;   // complex128 batches: the same, split into float pairs (cw)
  void* d_states = nullptr;    // ncirc device pointers
};

}  // namespace sv

struct sv_batch {
  int dtype = 0, ncirc = 0, kt = 0;
  bool dw = false;                     // complex128 passes in double-word arithmetic
  std::vector<int> nq;
  std::vector<size_t> off;             // element offset of each circuit's state
  size_t total = 0;                    // elements
  void* d_buf = nullptr;
  void* d_ptrs = nullptr;              // ncirc state pointers (for the ones kernel / energies)
  std::vector<std::vector<sv::HostOp>> ops;
  std::vector<sv::BatchGroup> groups;
  cudaStream_t streams[sv::kBatchStreams] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[sv::kBatchStreams] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // executor: SV_BATCH_GRAPH (a launch per group and pass, four streams, one graph) or
  // SV_BATCH_PERSISTENT (one cooperative launch); eager: the runs are not recorded
  int executor = 0;
  bool eager = false;
  void* d_pparams = nullptr;           // persistent: every group's pass blocks
  void* d_plaunch = nullptr;           // persistent: the (group, pass) queue
  int* d_pcnt = nullptr;               // persistent: per-circuit tile counters, ticket, abort flag
  int p_nl = 0, p_ncnt = 0, p_threads = 0;
  int64_t p_ntickets = 0;
  size_t p_smem = 0;
  // energies
  int nblocks = 0;
  void* d_blocks = nullptr;            // int2 (circuit, block index within circuit) per energy block
  void* d_nb = nullptr;                // blocks per circuit
  double* d_partials = nullptr;
  double* d_energy = nullptr;
  double* h_energy = nullptr;          // pinned
};

namespace sv {

template <typename T>
__global__ void k_batch_ones(T* const* states, int ncirc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncirc) return;
  if constexpr (is_complex<T>::value) {
    using R = typename real_of<T>::type;
    states[c][0] = T{(R)1, (R)0};
  } else {
    states[c][0] = (T)1;
  }
}

// TFIM energy E = -sum_i <Z_i Z_{i+1}> - h sum_i <X_i> (open chain), per circuit.
// Amplitude k contributes -(n-1-2*popc((k ^ k>>1) & (2^(n-1)-1))) |a_k|^2 for the ZZ
// terms and -2h sum_{b: bit b of k is 0} Re(conj(a_k) a_{k | 2^b}) for the X terms.
template <typename T>
__global__ void __launch_bounds__(256) k_tfim_partials(T* const* states, const int* nqs, const int2* blocks,
                                                      const int* nb, double h, double* partials) {
  const int2 bi = blocks[blockIdx.x];
  const int c = bi.x;
  const int n = nqs[c];
  const T* s = states[c];
  const int64_t N = (int64_t)1 << n;
  const int64_t stride = (int64_t)nb[c] * blockDim.x;
  const int64_t zzmask = (N >> 1) - 1;
  double acc = 0.0;
  for (int64_t k = (int64_t)bi.y * blockDim.x + threadIdx.x; k < N; k += stride) {
    const T a = s[k];
    double ar, ai;
    if constexpr (is_complex<T>::value) { ar = (double)a.re; ai = (double)a.im; } else { ar = (double)a; ai = 0.0; }
    using R = typename real_of<T>::type;
    R xs = 0;
    for (int b = 0; b < n; b++) {
      const int64_t kb = k | ((int64_t)1 << b);
      if (kb == k) continue;
      const T q = s[kb];
      if constexpr (is_complex<T>::value) xs += a.re * q.re + a.im * q.im;
      else xs += a * q;
    }
    const int zz = (n - 1) - 2 * __popcll((unsigned long long)((k ^ (k >> 1)) & zzmask));
    acc += -(double)zz * (ar * ar + ai * ai) - 2.0 * h * (double)xs;
  }
  // block sum (fixed order)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += part[w];
    partials[blockIdx.x] = r;
  }
}

__global__ void k_tfim_finish(const double* partials, const int* nb, const int* first, int ncirc, double* energy) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncirc) return;
  double s = 0.0, comp = 0.0;
  for (int i = 0; i < nb[c]; i++) {
    const double x = partials[first[c] + i];
    const double t = s + x;
    comp += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  energy[c] = s + comp;
}

// ------------------------------------------------- persistent batched executor
// One cooperative launch runs every pass of every group.  Work comes as tickets in
// queue order -- round r holds every group's pass r, largest states first -- and a
// ticket is a run of 2^cshift tiles of one circuit in one pass.  A ticket of pass
// r > 0 waits until its circuit's pass r - 1 has finished all its tiles (per-circuit
// tile counters, released with a fence, read with acquire loads).  Every ticket's
// dependencies precede it in the queue and the blocks, all resident, take tickets in
// order, so the earliest unfinished ticket can always proceed; a wait that exceeds its
// time limit raises the abort flag for every block and leaves status 2.
struct PLaunch {
  int64_t first;          // first ticket of this (group, pass)
  const void* params;     // the pass's PassParams block (device copy)
  const void* states;     // the group's state pointer table
  const void* coef;       // the group's coefficient blocks
  int64_t coef_stride;
  int32_t tshift;         // log2 tiles per circuit
  int32_t cshift;         // log2 tiles per ticket
  int32_t cnt;            // this pass's per-circuit counters (offset)
  int32_t prev;           // the previous pass's counters (offset), -1 for a group's first pass
};

constexpr unsigned long long kPersistWaitNs = 2000000000ull;  // 2 s; a ticket takes microseconds

__device__ __forceinline__ unsigned long long persist_clock() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// loads that bypass L1 (the previous pass was written by other SMs during this launch)
template <typename T> __device__ __forceinline__ T ld_l2(const T* p);
template <> __device__ __forceinline__ c64 ld_l2<c64>(const c64* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return c64{v.x, v.y};
}
template <> __device__ __forceinline__ c128 ld_l2<c128>(const c128* p) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return c128{v.x, v.y};
}
template <> __device__ __forceinline__ cw ld_l2<cw>(const cw* p) {  // stored as complex128
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return cw(dw_from_double(v.x), dw_from_double(v.y));
}
// plain stores (the next pass may read them from L2)
template <typename T> __device__ __forceinline__ void st_plain(T* p, T v) { *p = v; }
template <> __device__ __forceinline__ void st_plain<cw>(cw* p, cw v) {
  *reinterpret_cast<double2*>(p) = make_double2(dw_to_double(v.re), dw_to_double(v.im));
}

template <typename T, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_batch_persistent(const PLaunch* __restrict__ L, int nl,
                                                               int64_t ntickets, unsigned long long* ticket,
                                                               int* cnt, int* abort_flag, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ long long s_t;
  __shared__ int s_l, s_go;
  T* const tile = reinterpret_cast<T*>(smem_raw);
  // the largest tile (2^kRB amplitudes per thread), then its outer-bit deposit table
  int64_t* const dep_hi = reinterpret_cast<int64_t*>(smem_raw + sizeof(T) * (size_t)tile_stride(blockDim.x << kRB));
  int cur_l = -1;
  for (;;) {
    if (threadIdx.x == 0) {
      const long long t = (long long)atomicAdd(ticket, 1ull);
      int go = t < ntickets && !*(volatile int*)abort_flag;
      int l = 0;
      if (go) {
        // the last (group, pass) whose first ticket is <= t: a block's tickets increase,
        // so the search starts at its previous one and gallops forward
        int lo = cur_l < 0 ? 0 : cur_l, hi = lo + 1, step = 1;  // L[lo].first <= t
        while (hi < nl && L[hi].first <= t) {
          lo = hi;
          hi += step;
          step <<= 1;
        }
        if (hi > nl - 1) hi = nl - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (L[mid].first <= t) lo = mid;
          else hi = mid - 1;
        }
        l = lo;
        const PLaunch& la = L[l];
        if (la.prev >= 0) {
          const int c = (int)(((t - la.first) << la.cshift) >> la.tshift);
          const int need = 1 << la.tshift;
          const unsigned long long t0 = persist_clock();
          while (ld_acquire_gpu(cnt + la.prev + c) < need) {
            if (*(volatile int*)abort_flag) {
              go = 0;
              break;
            }
            if (persist_clock() - t0 > kPersistWaitNs) {
              atomicExch(abort_flag, 1);
              atomicExch(status, 2);
              go = 0;
              break;
            }
            __nanosleep(128);
          }
        }
      }
      s_t = t;
      s_l = l;
      s_go = go;
    }
    __syncthreads();
    if (!s_go) break;
    const long long t = s_t;
    const int l = s_l;
    const PLaunch& la = L[l];
    const PassParams<T>& p = *reinterpret_cast<const PassParams<T>*>(la.params);
    const int kt = p.kt;
    const int tsize = 1 << kt;
    if (l != cur_l) {  // this pass's tile map
      const int nhi = kt - kLowBits;
      for (int h = threadIdx.x; h < (1 << nhi); h += blockDim.x) {
        int64_t o = 0;
        for (int b = 0; b < nhi; b++)
          if ((h >> b) & 1) o |= (int64_t)1 << p.tile_pos[kLowBits + b];
        dep_hi[h] = o;
      }
      cur_l = l;
      __syncthreads();
    }
    const int64_t first_tile = (int64_t)(t - la.first) << la.cshift;
    const int c = (int)(first_tile >> la.tshift);
    T* const st = reinterpret_cast<T* const*>(la.states)[c];
    const T* const cbase = reinterpret_cast<const T*>(la.coef) + (int64_t)c * la.coef_stride + p.coef_goff;
    const bool active = (int)threadIdx.x < (tsize >> kRB);
    auto gofs = [&](int e) { return dep_hi[e >> kLowBits] | (e & ((1 << kLowBits) - 1)); };
    for (int k = 0; k < (1 << la.cshift); k++) {
      const int64_t base = tile_origin((first_tile + k) & ((1ll << la.tshift) - 1), p.tile_pos, kt);
      // element threadIdx.x + i * blockDim.x, i < 2^kRB: all of a thread's loads in flight
      T r[1 << kRB];
#pragma unroll
      for (int i = 0; i < (1 << kRB); i++) {
        const int e = threadIdx.x + i * blockDim.x;
        if (e < tsize) r[i] = ld_l2(st + (base | gofs(e)));
      }
#pragma unroll
      for (int i = 0; i < (1 << kRB); i++) {
        const int e = threadIdx.x + i * blockDim.x;
        if (e < tsize) tile[smem_pos(e)] = r[i];
      }
      __syncthreads();
      tile_phases(p, tile, cbase, base, active);
#pragma unroll
      for (int i = 0; i < (1 << kRB); i++) {
        const int e = threadIdx.x + i * blockDim.x;
        if (e < tsize) st_plain(st + (base | gofs(e)), tile[smem_pos(e)]);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {  // release: the block's stores before the count
      __threadfence();
      atomicAdd(cnt + la.cnt + c, 1 << la.cshift);
    }
  }
}

static bool same_structure(const std::vector<HostOp>& a, const std::vector<HostOp>& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); i++) {
    const HostOp& x = a[i];
    const HostOp& y = b[i];
    if (x.kind != y.kind || x.nt != y.nt || x.nc != y.nc || x.sign_only != y.sign_only ||
        (x.sign_only && x.sign_mask != y.sign_mask) || x.is_x != y.is_x || x.is_real != y.is_real ||
        x.is_swap != y.is_swap)
      return false;
    for (int k = 0; k < x.nt; k++)
      if (x.tpos[k] != y.tpos[k]) return false;
    for (int k = 0; k < x.nc; k++)
      if (x.cpos[k] != y.cpos[k]) return false;
  }
  return true;
}

template <typename T>
static int batch_build(sv_batch* b) {
  // coefficient blocks and state pointer tables per group
  for (auto& g : b->groups) {
    const sv_program* prog = g.prog;
    const size_t nc = g.circuits.size(), ct = prog->coef_total;
    std::vector<T> coef(nc * ct);
    std::vector<T*> ptrs(nc);
    for (size_t i = 0; i < nc; i++) {
      const int c = g.circuits[i];
      const std::vector<HostOp>& ops = b->ops[c];
      for (size_t sl = 0; sl < ct; sl++) {
        const int op = prog->coef_src[2 * sl], e = prog->coef_src[2 * sl + 1];
        coef[i * ct + sl] = to_elem<T>(&ops[op].m[2 * e]);
      }
      ptrs[i] = (T*)b->d_buf + b->off[c];
    }
    if (ct) {
      SV_TRY(check_cuda(cudaMalloc(&g.d_coef, nc * ct * sizeof(T)), "batch coefficients"));
      SV_TRY(check_cuda(cudaMemcpy(g.d_coef, coef.data(), nc * ct * sizeof(T), cudaMemcpyHostToDevice), "coef upload"));
      if constexpr (std::is_same<T, c128>::value) {
        if (b->dw) {
          std::vector<cw> split(nc * ct);
          for (size_t k = 0; k < nc * ct; k++) split[k] = cw(coef[k].re, coef[k].im);
          SV_TRY(check_cuda(cudaMalloc(&g.d_coef_dw, nc * ct * sizeof(cw)), "batch coefficients"));
          SV_TRY(check_cuda(cudaMemcpy(g.d_coef_dw, split.data(), nc * ct * sizeof(cw), cudaMemcpyHostToDevice),
                            "coef upload"));
        }
      }
    }
    SV_TRY(check_cuda(cudaMalloc(&g.d_states, nc * sizeof(T*)), "batch pointers"));
    SV_TRY(check_cuda(cudaMemcpy(g.d_states, ptrs.data(), nc * sizeof(T*), cudaMemcpyHostToDevice), "pointer upload"));
  }
  std::vector<T*> all(b->ncirc);
  for (int c = 0; c < b->ncirc; c++) all[c] = (T*)b->d_buf + b->off[c];
  SV_TRY(check_cuda(cudaMalloc(&b->d_ptrs, b->ncirc * sizeof(T*)), "batch pointers"));
  SV_TRY(check_cuda(cudaMemcpy(b->d_ptrs, all.data(), b->ncirc * sizeof(T*), cudaMemcpyHostToDevice), "pointer upload"));
  return SV_OK;
}

// the persistent executor's queue (persist_queue, sv_persist_queue.h) with device
// pointers: pass blocks copied to the device once, the groups' state tables and
// coefficient blocks
template <typename T>
static int persist_build(Context* ctx, sv_batch* b) {
  std::vector<PLaunch> ls;
  std::vector<size_t> pofs;  // each group's first pass block in the device copy
  size_t pbytes = 0;
  int ktmax = kRB + 1;
  for (const BatchGroup& g : b->groups) {
    for (const Segment& s : g.prog->segments)
      if (!s.fused) return set_error(SV_ERR_UNSUPPORTED, "the persistent executor runs fused passes only");
    pofs.push_back(pbytes);
    pbytes += g.prog->passes.size();
    ktmax = std::max(ktmax, g.prog->kt);
  }
  if (pbytes == 0) return set_error(SV_ERR_ARG, "the batch has no passes");
  std::vector<unsigned char> blocks(pbytes);
  for (size_t gi = 0; gi < b->groups.size(); gi++) {
    const sv_program* prog = b->groups[gi].prog;
    const std::vector<unsigned char>& src = b->dw ? prog->passes_dw : prog->passes;
    memcpy(blocks.data() + pofs[gi], src.data(), src.size());
  }
  SV_TRY(check_cuda(cudaMalloc(&b->d_pparams, pbytes), "persistent pass blocks"));
  SV_TRY(check_cuda(cudaMemcpy(b->d_pparams, blocks.data(), pbytes, cudaMemcpyHostToDevice), "pass block upload"));
  std::vector<PersistGroup> shape;
  for (const BatchGroup& g : b->groups)
    shape.push_back({(int)g.prog->segments.size(), (int)g.circuits.size(), g.prog->nqubits - g.prog->kt});
  int counters = 0;
  const std::vector<PersistEntry> queue = persist_queue(shape, &counters);
  int64_t tickets = 0;
  for (const PersistEntry& e : queue) {
    const BatchGroup& g = b->groups[e.group];
    const sv_program* prog = g.prog;
    PLaunch x;
    memset(&x, 0, sizeof(x));
    x.first = e.first;
    x.params = (const char*)b->d_pparams + pofs[e.group] + (size_t)prog->segments[e.pass].pass * prog->pass_bytes;
    x.states = g.d_states;
    x.coef = b->dw ? g.d_coef_dw : g.d_coef;
    x.coef_stride = (int64_t)prog->coef_total;
    x.tshift = e.tshift;
    x.cshift = e.cshift;
    x.cnt = e.cnt;
    x.prev = e.prev;
    tickets = e.first + e.ntickets;
    ls.push_back(x);
  }
  SV_TRY(check_cuda(cudaMalloc(&b->d_plaunch, ls.size() * sizeof(PLaunch)), "persistent queue"));
  SV_TRY(check_cuda(cudaMemcpy(b->d_plaunch, ls.data(), ls.size() * sizeof(PLaunch), cudaMemcpyHostToDevice),
                    "queue upload"));
  SV_TRY(check_cuda(cudaMalloc(&b->d_pcnt, sizeof(int) * (size_t)counters + 16), "persistent counters"));
  b->p_nl = (int)ls.size();
  b->p_ncnt = counters;
  b->p_ntickets = tickets;
  b->p_threads = 1 << (ktmax - kRB);
  b->p_smem = sizeof(T) * (size_t)tile_stride(1 << ktmax) + sizeof(int64_t) * ((size_t)1 << (ktmax - kLowBits));
  (void)ctx;
  return SV_OK;
}

template <typename T, int MAXT, int MINB>
static int persist_launch_variant(Context* ctx, sv_batch* b, cudaStream_t st) {
  auto kern = k_batch_persistent<T, MAXT, MINB>;
  SV_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->p_smem),
                    "persistent executor smem attribute"));
  int per_sm = 0;
  SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, b->p_threads, b->p_smem),
                    "persistent executor occupancy"));
  if (per_sm < 1) return set_error(SV_ERR_ARG, "the persistent executor's tile does not fit on an SM");
  int64_t grid = (int64_t)per_sm * ctx->num_sms;  // all blocks resident (cooperative launch)
  if (grid > b->p_ntickets) grid = b->p_ntickets;
  const PLaunch* dl = (const PLaunch*)b->d_plaunch;
  int nl = b->p_nl;
  int64_t nt = b->p_ntickets;
  int* cnt = b->d_pcnt;
  unsigned long long* ticket = (unsigned long long*)(cnt + b->p_ncnt + (b->p_ncnt & 1));  // 8-byte aligned
  int* abort_flag = (int*)(ticket + 1);
  int* status = ctx->device_status;
  SV_TRY(check_cuda(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)b->p_ncnt + 16, st), "counter reset"));
  void* args[] = {&dl, &nl, &nt, &ticket, &cnt, &abort_flag, &status};
  SV_TRY(check_cuda(cudaLaunchCooperativeKernel((const void*)kern, dim3((unsigned)grid), dim3(b->p_threads), args,
                                                b->p_smem, st),
                    "persistent executor launch"));
  return SV_OK;
}

// |0...0> for every circuit, then the whole batch in one cooperative launch
template <typename T>
static int persist_launches(Context* ctx, sv_batch* b) {
  cudaStream_t st = b->streams[0];
  const size_t es = b->dtype == SV_C128 ? sizeof(c128) : sizeof(c64);
  SV_TRY(check_cuda(cudaMemsetAsync(b->d_buf, 0, b->total * es, st), "batch zero"));
  if (b->dtype == SV_C128) k_batch_ones<c128><<<grid_for(b->ncirc, 256), 256, 0, st>>>((c128* const*)b->d_ptrs, b->ncirc);
  else k_batch_ones<c64><<<grid_for(b->ncirc, 256), 256, 0, st>>>((c64* const*)b->d_ptrs, b->ncirc);
  SV_LAUNCH_CHECK("batch ones");
  if constexpr (sizeof(T) >= 16) return persist_launch_variant<T, 256, 1>(ctx, b, st);
  else if (b->p_threads <= 256) return persist_launch_variant<T, 256, 2>(ctx, b, st);
  else return persist_launch_variant<T, 512, 1>(ctx, b, st);
}

template <typename T>
static int batch_launches(Context* ctx, sv_batch* b) {
  if (b->executor == SV_BATCH_PERSISTENT) return b->dw ? persist_launches<cw>(ctx, b) : persist_launches<T>(ctx, b);
  const size_t bytes = b->total * sizeof(T);
  SV_TRY(check_cuda(cudaMemsetAsync(b->d_buf, 0, bytes, b->streams[0]), "batch zero"));
  k_batch_ones<T><<<grid_for(b->ncirc, 256), 256, 0, b->streams[0]>>>((T* const*)b->d_ptrs, b->ncirc);
  SV_LAUNCH_CHECK("batch ones");
  SV_TRY(check_cuda(cudaEventRecord(b->ev_fork, b->streams[0]), "fork"));
  for (int k = 1; k < kBatchStreams; k++)
    SV_TRY(check_cuda(cudaStreamWaitEvent(b->streams[k], b->ev_fork, 0), "fork wait"));
  // largest groups first, round-robin over the streams
  for (size_t gi = 0; gi < b->groups.size(); gi++) {
    const BatchGroup& g = b->groups[gi];
    const sv_program* prog = g.prog;
    cudaStream_t st = b->streams[gi % kBatchStreams];
    const int kt = prog->kt;
    const int threads = 1 << (kt - kRB);
    const size_t smem = pass_smem<T>(kt);
    BatchArgs<T> args;
    memset(&args, 0, sizeof(args));
    args.states = (T* const*)g.d_states;
    args.coef = (const T*)g.d_coef;
    args.coef_stride = (int64_t)prog->coef_total;
    args.ncirc = (int32_t)g.circuits.size();
    for (const Segment& s : prog->segments) {
      if (prog->bspec) {
        SV_TRY(specialized_launch_batched(ctx, prog, s.pass, st, g.d_states, b->dw ? g.d_coef_dw : g.d_coef,
                                          (int64_t)prog->coef_total,
                                          args.ncirc));
        continue;
      }
      if constexpr (std::is_same<T, c128>::value) {
        if (b->dw) {  // double-word kernels on the pre-split blocks and coefficients
          BatchArgs<cw> a;
          memset(&a, 0, sizeof(a));
          a.states = (cw* const*)g.d_states;
          a.coef = (const cw*)g.d_coef_dw;
          a.coef_stride = args.coef_stride;
          a.ncirc = args.ncirc;
          const PassParams<cw>& p =
              *reinterpret_cast<const PassParams<cw>*>(prog->passes_dw.data() + (size_t)s.pass * prog->pass_bytes);
          SV_TRY(launch_pass<cw, true>(ctx, p, nullptr, threads, smem, p.ntiles * a.ncirc, st, a));
          continue;
        }
      }
      const PassParams<T>& p =
          *reinterpret_cast<const PassParams<T>*>(prog->passes.data() + (size_t)s.pass * prog->pass_bytes);
      SV_TRY(launch_pass<T, true>(ctx, p, nullptr, threads, smem, p.ntiles * args.ncirc, st, args));
    }
  }
  for (int k = 1; k < kBatchStreams; k++) {
    SV_TRY(check_cuda(cudaEventRecord(b->ev_join[k], b->streams[k]), "join"));
    SV_TRY(check_cuda(cudaStreamWaitEvent(b->streams[0], b->ev_join[k], 0), "join wait"));
  }
  return SV_OK;
}

static void batch_free(sv_batch* b) {
  if (!b) return;
  if (b->d_pparams) cudaFree(b->d_pparams);
  if (b->d_plaunch) cudaFree(b->d_plaunch);
  if (b->d_pcnt) cudaFree(b->d_pcnt);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto& g : b->groups) {
    if (g.d_coef) cudaFree(g.d_coef);
    if (g.d_coef_dw) cudaFree(g.d_coef_dw);
    if (g.d_states) cudaFree(g.d_states);
    sv_program_destroy(g.prog);
  }
  for (int k = 0; k < kBatchStreams; k++) {
    if (b->streams[k]) cudaStreamDestroy(b->streams[k]);
    if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
  }
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->d_buf) cudaFree(b->d_buf);
  if (b->d_ptrs) cudaFree(b->d_ptrs);
  if (b->d_blocks) cudaFree(b->d_blocks);
  if (b->d_nb) cudaFree(b->d_nb);
  if (b->d_partials) cudaFree(b->d_partials);
  if (b->d_energy) cudaFree(b->d_energy);
  if (b->h_energy) cudaFreeHost(b->h_energy);
  delete b;
}

}  // namespace sv

extern "C" {

int sv_batch_create(sv_context* ctx, int dtype, int ncirc, const int32_t* nqubits, const sv_gate_op* const* ops,
                    const int32_t* nops, int tile_bits, sv_batch** out) {
  if (!ctx || !out || !nqubits || !ops || !nops || ncirc < 1) return set_error(SV_ERR_ARG, "bad batch arguments");
  *out = nullptr;
  if (dtype != SV_C128 && dtype != SV_C64) return set_error(SV_ERR_UNSUPPORTED, "batches need a complex dtype");
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  sv_batch* b = new sv_batch();
  b->dtype = dtype;
  // complex128 batches compute in double-word arithmetic unless the context asks for
  // FP64 when the batch is created (fixed for its life: its runs replay one graph)
  b->dw = dtype == SV_C128 && !ctx->c128_fp64;
  b->ncirc = ncirc;
  const size_t es = dtype_size(dtype);
  // parse every circuit through the program front end (validation included)
  std::vector<sv_program*> progs(ncirc, nullptr);
  for (int c = 0; c < ncirc; c++) {
    const int n = nqubits[c];
    if (n < kLowBits + kRB || n > 34) {
      batch_free(b);
      return set_error(SV_ERR_ARG, "circuit %d: %d qubits outside [%d, 34]", c, n, kLowBits + kRB);
    }
    b->nq.push_back(n);
    b->off.push_back(b->total);
    b->total += ((((size_t)1 << n) * es + 255) / 256) * 256 / es;
  }
  // groups: identical structure (after single-qubit merging); plan one circuit per group
  for (int c = 0; c < ncirc; c++) {
    std::vector<HostOp> hops;
    int rc = parse_ops(nqubits[c], ops[c], nops[c], &hops);
    int kt = 0;
    if (rc == SV_OK) rc = check_tile_bits(dtype, nqubits[c], tile_bits, &kt);
    if (rc != SV_OK) {
      batch_free(b);
      return rc;
    }
    bool found = false;
    for (auto& g : b->groups) {
      if (g.prog->nqubits == nqubits[c] && g.prog->kt == kt && same_structure(g.prog->ops, hops)) {
        g.circuits.push_back(c);
        found = true;
        break;
      }
    }
    b->ops.push_back(hops);
    if (!found) {
      sv_program* p = nullptr;
      rc = plan(dtype, nqubits[c], kt, std::move(hops), &p);
      if (rc == SV_OK && p->nunfused) {
        sv_program_destroy(p);
        rc = set_error(SV_ERR_UNSUPPORTED, "circuit %d has gates on more than 2 targets; batches need fusable gates", c);
      }
      if (rc != SV_OK) {
        batch_free(b);
        return rc;
      }
      BatchGroup g;
      g.prog = p;
      g.circuits.push_back(c);
      b->groups.push_back(g);
    }
  }
  // largest states first so the big groups start early on every stream
  std::stable_sort(b->groups.begin(), b->groups.end(), [](const BatchGroup& x, const BatchGroup& y) {
    return ((size_t)x.circuits.size() << x.prog->nqubits) > ((size_t)y.circuits.size() << y.prog->nqubits);
  });
  int rc = check_cuda(cudaMalloc(&b->d_buf, b->total * es), "batch states");
  if (rc == SV_OK) rc = dtype == SV_C128 ? batch_build<c128>(b) : batch_build<c64>(b);
  for (int k = 0; k < kBatchStreams && rc == SV_OK; k++) {
    rc = check_cuda(cudaStreamCreateWithFlags(&b->streams[k], cudaStreamNonBlocking), "batch stream");
    if (rc == SV_OK) rc = check_cuda(cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming), "event");
  }
  if (rc == SV_OK) rc = check_cuda(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming), "event");
  // energy block table: up to 64 blocks of 256 threads per circuit
  if (rc == SV_OK) {
    std::vector<int2> blocks;
    std::vector<int> nb(ncirc), first(ncirc);
    for (int c = 0; c < ncirc; c++) {
      int64_t want = ((int64_t)1 << b->nq[c]) / 4096;
      if (want < 1) want = 1;
      if (want > 64) want = 64;
      nb[c] = (int)want;
      first[c] = (int)blocks.size();
      for (int k = 0; k < nb[c]; k++) blocks.push_back(make_int2(c, k));
    }
    b->nblocks = (int)blocks.size();
    rc = check_cuda(cudaMalloc(&b->d_blocks, blocks.size() * sizeof(int2)), "energy table");
    if (rc == SV_OK) rc = check_cuda(cudaMalloc(&b->d_nb, 3 * ncirc * sizeof(int)), "energy table");
    if (rc == SV_OK) rc = check_cuda(cudaMalloc(&b->d_partials, blocks.size() * sizeof(double)), "energy partials");
    if (rc == SV_OK) rc = check_cuda(cudaMalloc(&b->d_energy, ncirc * sizeof(double)), "energies");
    if (rc == SV_OK) rc = check_cuda(cudaMallocHost(&b->h_energy, ncirc * sizeof(double)), "energies (host)");
    if (rc == SV_OK)
      rc = check_cuda(cudaMemcpy(b->d_blocks, blocks.data(), blocks.size() * sizeof(int2), cudaMemcpyHostToDevice),
                      "energy table upload");
    if (rc == SV_OK) {
      std::vector<int> nbf(nb);  // [blocks per circuit | first block | qubits]
      nbf.insert(nbf.end(), first.begin(), first.end());
      nbf.insert(nbf.end(), b->nq.begin(), b->nq.end());
      rc = check_cuda(cudaMemcpy(b->d_nb, nbf.data(), nbf.size() * sizeof(int), cudaMemcpyHostToDevice), "upload");
    }
  }
  if (rc != SV_OK) {
    batch_free(b);
    return rc;
  }
  *out = b;
  return SV_OK;
}

int sv_batch_set_executor(sv_context* ctx, sv_batch* b, int executor) {
  if (!ctx || !b) return set_error(SV_ERR_ARG, "null context or batch");
  if (executor != SV_BATCH_GRAPH && executor != SV_BATCH_PERSISTENT)
    return set_error(SV_ERR_ARG, "executor must be SV_BATCH_GRAPH or SV_BATCH_PERSISTENT");
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  SV_TRY(check_cuda(cudaStreamSynchronize(b->streams[0]), "batch sync"));
  if (executor == SV_BATCH_PERSISTENT && !b->d_plaunch) {
    SV_TRY(ensure_device_status(ctx));
    int rc = b->dw ? persist_build<cw>(ctx, b) : b->dtype == SV_C128 ? persist_build<c128>(ctx, b)
                                                                     : persist_build<c64>(ctx, b);
    if (rc != SV_OK) {
      if (b->d_pparams) cudaFree(b->d_pparams);
      if (b->d_plaunch) cudaFree(b->d_plaunch);
      if (b->d_pcnt) cudaFree(b->d_pcnt);
      b->d_pparams = b->d_plaunch = nullptr;
      b->d_pcnt = nullptr;
      return rc;
    }
  }
  if (executor != b->executor) {  // record the new launches on the next run
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->eager = false;
    b->executor = executor;
  }
  return SV_OK;
}

int sv_batch_specialize(sv_context* ctx, sv_batch* b) {
  if (!ctx || !b) return set_error(SV_ERR_ARG, "null context or batch");
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  SV_TRY(check_cuda(cudaDeviceSynchronize(), "batch specialise sync"));
  for (auto& g : b->groups) SV_TRY(specialize_batched(ctx, g.prog, b->dw));
  // the recorded graph holds the interpreting launches: record again on the next run
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  return SV_OK;
}

int sv_batch_run(sv_context* ctx, sv_batch* b) {
  if (!ctx || !b) return set_error(SV_ERR_ARG, "null context or batch");
  cudaEvent_t ev;
  SV_TRY(check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event"));
  // order after earlier work on the context stream
  SV_TRY(check_cuda(cudaEventRecord(ev, ctx->stream), "event"));
  SV_TRY(check_cuda(cudaStreamWaitEvent(b->streams[0], ev, 0), "wait"));
  int rc = SV_OK;
  if (b->executor == SV_BATCH_PERSISTENT) ctx->status_pending = true;  // its waits are bounded
  if (b->exec) {
    rc = check_cuda(cudaGraphLaunch(b->exec, b->streams[0]), "graph launch");
  } else if (b->eager) {
    rc = b->dtype == SV_C128 ? batch_launches<c128>(ctx, b) : batch_launches<c64>(ctx, b);
  } else {
    // first run: eager (sets kernel attributes), then record the same launches as a graph
    rc = b->dtype == SV_C128 ? batch_launches<c128>(ctx, b) : batch_launches<c64>(ctx, b);
    if (rc == SV_OK) rc = check_cuda(cudaStreamSynchronize(b->streams[0]), "batch sync");
    if (rc == SV_OK) rc = check_cuda(cudaStreamBeginCapture(b->streams[0], cudaStreamCaptureModeThreadLocal), "capture");
    if (rc == SV_OK) {
      const int rc2 = b->dtype == SV_C128 ? batch_launches<c128>(ctx, b) : batch_launches<c64>(ctx, b);
      cudaGraph_t g = nullptr;
      const int rc3 = check_cuda(cudaStreamEndCapture(b->streams[0], &g), "end capture");
      rc = rc2 != SV_OK ? rc2 : rc3;
      if (rc == SV_OK) {
        b->graph = g;
        rc = check_cuda(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate");
      } else if (g) {
        cudaGraphDestroy(g);
      }
      if (rc != SV_OK && b->executor == SV_BATCH_PERSISTENT) {
        // a cooperative launch that cannot be recorded runs eagerly on later runs
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        (void)cudaGetLastError();
        b->eager = true;
        rc = SV_OK;
      }
    }
    // the eager run already produced the states; the graph is for later runs
  }
  if (rc == SV_OK) rc = check_cuda(cudaEventRecord(ev, b->streams[0]), "event");
  if (rc == SV_OK) rc = check_cuda(cudaStreamWaitEvent(ctx->stream, ev, 0), "wait");
  cudaEventDestroy(ev);
  return rc;
}

int sv_batch_tfim_energy(sv_context* ctx, sv_batch* b, double h, double* energies) {
  if (!ctx || !b || !energies) return set_error(SV_ERR_ARG, "null argument");
  const int* nb = (const int*)b->d_nb;
  const int* first = nb + b->ncirc;
  const int* nqs = nb + 2 * b->ncirc;
  if (b->dtype == SV_C128)
    k_tfim_partials<c128><<<b->nblocks, 256, 0, ctx->stream>>>((c128* const*)b->d_ptrs, nqs, (const int2*)b->d_blocks,
                                                               nb, h, b->d_partials);
  else
    k_tfim_partials<c64><<<b->nblocks, 256, 0, ctx->stream>>>((c64* const*)b->d_ptrs, nqs, (const int2*)b->d_blocks,
                                                              nb, h, b->d_partials);
  SV_LAUNCH_CHECK("tfim energy launch");
  k_tfim_finish<<<grid_for(b->ncirc, 128), 128, 0, ctx->stream>>>(b->d_partials, nb, first, b->ncirc, b->d_energy);
  SV_LAUNCH_CHECK("tfim finish launch");
  SV_TRY(check_cuda(cudaMemcpyAsync(b->h_energy, b->d_energy, b->ncirc * sizeof(double), cudaMemcpyDeviceToHost,
                                    ctx->stream), "energy copy"));
  SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "energy sync"));
  memcpy(energies, b->h_energy, b->ncirc * sizeof(double));
  return take_device_status(ctx);  // a persistent run that gave up waiting reports here
}

int sv_batch_state(const sv_batch* b, int circuit, void** state, int* nqubits) {
  if (!b || circuit < 0 || circuit >= b->ncirc || !state) return set_error(SV_ERR_ARG, "bad batch query");
  *state = (unsigned char*)b->d_buf + b->off[circuit] * dtype_size(b->dtype);
  if (nqubits) *nqubits = b->nq[circuit];
  return SV_OK;
}

int sv_batch_stats(const sv_batch* b, int* ngroups, int* npasses, size_t* state_bytes) {
  if (!b) return set_error(SV_ERR_ARG, "null batch");
  int np = 0;
  for (auto& g : b->groups) np += g.prog->npasses;
  if (ngroups) *ngroups = (int)b->groups.size();
  if (npasses) *npasses = np;
  if (state_bytes) *state_bytes = b->total * dtype_size(b->dtype);
  return SV_OK;
}

int sv_batch_arith(const sv_batch* b, double* instructions) {
  if (!b || !instructions) return set_error(SV_ERR_ARG, "bad batch query");
  double total = 0.0;
  for (auto& g : b->groups) {
    const double per_amp = program_arith_per_amplitude(g.prog);
    for (int c : g.circuits) total += per_amp * (double)((int64_t)1 << b->nq[c]);
  }
  *instructions = total;
  return SV_OK;
}

int sv_batch_pass_bytes(const sv_batch* b, double* bytes) {
  if (!b || !bytes) return set_error(SV_ERR_ARG, "bad batch query");
  double total = 0.0;
  for (auto& g : b->groups)
    for (int c : g.circuits)
      total += (double)g.prog->npasses * 2.0 * (double)dtype_size(b->dtype) * (double)((size_t)1 << b->nq[c]);
  *bytes = total;
  return SV_OK;
}

int sv_batch_destroy(sv_batch* b) {
  batch_free(b);
  return SV_OK;
}

}  // extern "C"

// ============================================================ adjoint gradients
// Gradients of E = <psi|H|psi> for circuits of gates exp(-i t G / 2) (G = X, Y, Z on
// one qubit) plus fixed gates, by the adjoint method: forward, lambda = H psi, then a
// reverse sweep that for every gate j (last to first) takes
//   dE/dt_j = Im <lambda|G_j|psi>     (psi, lambda after gate j)
// and then un-applies gate j from both psi and lambda.  The sweep is planned like any
// program (gradient markers before each U^dagger) and runs as tile passes that keep
// the psi and lambda tiles side by side in shared memory.  Inner products are reduced
// per warp in FP32, then in FP64 per block into per-(circuit, parameter, block) slots
// (fixed order: deterministic).  Forward states are checkpointed at segment
// boundaries and restored during the sweep, which bounds complex64 drift.
namespace sv {

constexpr int kAdjMaxGrad = 128;  // gradient markers per pass

template <typename T>
struct AdjArgs {
  T* const* psi;
  T* const* lam;
  const T* coef;
  int64_t coef_stride;
  double* gpart;        // [circuit][parameter][gstride]
  int32_t ncirc, nparams, gstride, pad;
};
static_assert(kAdjMaxGrad >= kMaxPassOpsRefill, "one gradient slot per op of an adjoint pass");
// kernel parameters are limited to 32764 bytes
static_assert(sizeof(PassParams<c128>) + sizeof(AdjArgs<c128>) <= 32764, "adjoint pass parameters");
static_assert(sizeof(PassParams<c128>) + sizeof(BatchArgs<c128>) + sizeof(void*) <= 32764, "pass parameters");

template <typename T, int GEN>
__device__ __forceinline__ typename real_of<T>::type grad_dispatch(const T (&v)[16], const T (&w)[16], int u) {
  switch (u) {
    case 0: return grad_pairs<T, 0, GEN>(v, w);
    case 1: return grad_pairs<T, 1, GEN>(v, w);
    case 2: return grad_pairs<T, 2, GEN>(v, w);
    default: return grad_pairs<T, 3, GEN>(v, w);
  }
}

template <typename T, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_adjoint_pass(const __grid_constant__ PassParams<T> p,
                                                           const __grid_constant__ AdjArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int kt = p.kt;
  const int tsize = 1 << kt;
  const int tstride = tile_stride(tsize);
  T* const bpsi = reinterpret_cast<T*>(smem_raw);      // two psi tiles
  T* const blam = bpsi + 2 * tstride;                   // two lambda tiles
  int64_t* dep_hi = reinterpret_cast<int64_t*>(blam + 2 * tstride);
  const int nwarps = blockDim.x >> 5;
  double* gacc = reinterpret_cast<double*>(dep_hi + (1 << (kt - kLowBits)));  // [slot][warp]
  const int nhi = kt - kLowBits;
  for (int h = threadIdx.x; h < (1 << nhi); h += blockDim.x) {
    int64_t o = 0;
    for (int b = 0; b < nhi; b++)
      if ((h >> b) & 1) o |= (int64_t)1 << p.tile_pos[kLowBits + b];
    dep_hi[h] = o;
  }
  for (int i = threadIdx.x; i < kAdjMaxGrad * nwarps; i += blockDim.x) gacc[i] = 0.0;
  __syncthreads();
  const int nthreads = blockDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto issue_load = [&](int slot, int64_t it) {
    const int64_t base = tile_origin(it & (p.ntiles - 1), p.tile_pos, kt);
    const T* sp = a.psi[it >> (p.n - kt)];
    const T* sl = a.lam[it >> (p.n - kt)];
    for (int e = threadIdx.x; e < tsize; e += nthreads) {
      const int64_t g = base | dep_hi[e >> kLowBits] | (e & ((1 << kLowBits) - 1));
      cp_async<sizeof(T)>(bpsi + slot * tstride + smem_pos(e), sp + g);
      cp_async<sizeof(T)>(blam + slot * tstride + smem_pos(e), sl + g);
    }
    cp_async_commit();
  };
  // write this block's accumulated gradients of one circuit and clear the slots
  auto flush = [&](int circ) {
    __syncthreads();
    for (int o = threadIdx.x; o < p.nops; o += blockDim.x) {
      const FOp& op = p.ops[o];
      if (op.type != FOP_GRADX && op.type != FOP_GRADY && op.type != FOP_GRADZ) continue;
      double sum = 0.0;
      for (int w = 0; w < nwarps; w++) {
        sum += gacc[op.u1 * nwarps + w];
        gacc[op.u1 * nwarps + w] = 0.0;
      }
      a.gpart[((int64_t)circ * a.nparams + op.coef) * a.gstride + blockIdx.x] = sum;
    }
    __syncthreads();
  };
  const int64_t nitems = p.ntiles * a.ncirc;
  const int tshift = p.n - kt;
  int64_t t = blockIdx.x;
  if (t < nitems) issue_load(0, t);
  int cur = 0;
  int cur_circ = -1;
  for (; t < nitems; t += gridDim.x, cur ^= 1) {
    const int circ = (int)(t >> tshift);
    if (circ != cur_circ) {
      if (cur_circ >= 0) flush(cur_circ);
      cur_circ = circ;
    }
    T* tp = bpsi + cur * tstride;
    T* tl = blam + cur * tstride;
    const int64_t base = tile_origin(t & (p.ntiles - 1), p.tile_pos, kt);
    const T* cbase = a.coef + (int64_t)circ * a.coef_stride + p.coef_goff;
    const int64_t tn = t + gridDim.x;
    if (tn < nitems) {
      issue_load(cur ^ 1, tn);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    for (int ph = 0; ph < p.nphases; ph++) {
      const Phase& P = p.phases[ph];
      const int r0 = P.rb[0], r1 = P.rb[1], r2 = P.rb[2], r3 = P.rb[3];
      int lbase = threadIdx.x;
      lbase = ((lbase >> r0) << (r0 + 1)) | (lbase & ((1 << r0) - 1));
      lbase = ((lbase >> r1) << (r1 + 1)) | (lbase & ((1 << r1) - 1));
      lbase = ((lbase >> r2) << (r2 + 1)) | (lbase & ((1 << r2) - 1));
      lbase = ((lbase >> r3) << (r3 + 1)) | (lbase & ((1 << r3) - 1));
      const int sb = smem_pos(lbase);
      T v[16], w[16];
#pragma unroll
      for (int j = 0; j < 16; j++) {
        v[j] = tp[sb + P.soff[j]];
        w[j] = tl[sb + P.soff[j]];
      }
      unsigned pending_neg = 0;
      for (int o = P.op_begin; o < P.op_end; o++) {
        const FOp& op = p.ops[o];
        const int type = op.type;
        if (type == FOP_GRADZ) {
          // sign of each amplitude from its bit; invariant under pending negations
          int tpb = 0;
          if (op.tb[0] >= 0) tpb = (lbase >> op.tb[0]) & 1;
          else if (op.ob[0] >= 0) tpb = (int)((base >> op.ob[0]) & 1);
          typename real_of<T>::type acc = 0;
#pragma unroll
          for (int j = 0; j < 16; j++) {
            const int bit = (int)((op.rpart >> (4 * j)) & 1) | tpb;
            const auto x = im_cdot(w[j], v[j]);
            acc += bit ? -x : x;
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
          if (lane == 0) gacc[op.u1 * nwarps + warp] += (double)acc;
          continue;
        }
        if (pending_neg && type != FOP_SIGN && type != FOP_DIAG) {
          apply_negations(v, pending_neg);
          apply_negations(w, pending_neg);
          pending_neg = 0;
        }
        if (type == FOP_GRADX || type == FOP_GRADY) {
          auto acc = type == FOP_GRADX ? grad_dispatch<T, 1>(v, w, op.u0) : grad_dispatch<T, 2>(v, w, op.u0);
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
          if (lane == 0) gacc[op.u1 * nwarps + warp] += (double)acc;
          continue;
        }
        if (type == FOP_D1RUN || type == FOP_D1RUNR) {
          // uncontrolled 2x2 gates on distinct register bits (complex, or real such as RY)
          const T* c = cbase + op.coef;
#pragma unroll 1
          for (int k = 0; k < op.nrun; k++) {
            if (type == FOP_D1RUN) {
              dense1_dispatch(v, c + 4 * k, op.ru[k], 0xffffu);
              dense1_dispatch(w, c + 4 * k, op.ru[k], 0xffffu);
            } else {
              dense1r_dispatch(v, c + 4 * k, op.ru[k], 0xffffu);
              dense1r_dispatch(w, c + 4 * k, op.ru[k], 0xffffu);
            }
          }
          continue;
        }
        const int flags = op.flags;
        if ((flags & FLAG_OMASK) && ((base & (int64_t)op.omask) != (int64_t)op.omask)) continue;
        if ((flags & FLAG_TMASK) && (((unsigned)lbase & op.tmask) != op.tmask)) continue;
        if (type == FOP_DENSE1) {
          dense1_dispatch(v, cbase + op.coef, op.u0, op.jmask);
          dense1_dispatch(w, cbase + op.coef, op.u0, op.jmask);
        } else if (type == FOP_DENSE1R) {
          dense1r_dispatch(v, cbase + op.coef, op.u0, op.jmask);
          dense1r_dispatch(w, cbase + op.coef, op.u0, op.jmask);
        } else if (type == FOP_X1) {
          x1_dispatch(v, op.u0, op.jmask);
          x1_dispatch(w, op.u0, op.jmask);
        } else if (type == FOP_SWAP2) {
          swap2_dispatch(v, op.u0, op.u1, op.jmask);
          swap2_dispatch(w, op.u0, op.u1, op.jmask);
        } else if (type == FOP_DENSE2) {
          dense2_dispatch(v, cbase + op.coef, op.u0, op.u1, op.jmask);
          dense2_dispatch(w, cbase + op.coef, op.u0, op.u1, op.jmask);
        } else {
          const int nd = op.nd;
          int tpx = 0;
#pragma unroll
          for (int i = 0; i < 3; i++) {
            if (i >= nd) break;
            if (op.tb[i] >= 0) tpx |= ((lbase >> op.tb[i]) & 1) << (nd - 1 - i);
            else if (op.ob[i] >= 0) tpx |= (int)((base >> op.ob[i]) & 1) << (nd - 1 - i);
          }
          if (type == FOP_SIGN) {
            pending_neg ^= op.neg[tpx];
          } else {
            const unsigned jm = op.jmask;
            const uint64_t rp = op.rpart;
            const T* c = cbase + op.coef;
#pragma unroll
            for (int j = 0; j < 16; j++) {
              if (!((jm >> j) & 1u)) continue;
              const int idx = (int)((rp >> (4 * j)) & 15) | tpx;
              v[j] = tmul(c[idx], v[j]);
              w[j] = tmul(c[idx], w[j]);
            }
          }
        }
      }
      if (pending_neg) {
        apply_negations(v, pending_neg);
        apply_negations(w, pending_neg);
      }
#pragma unroll
      for (int j = 0; j < 16; j++) {
        tp[sb + P.soff[j]] = v[j];
        tl[sb + P.soff[j]] = w[j];
      }
      __syncthreads();
    }
    T* const sp = a.psi[circ];
    T* const sl = a.lam[circ];
    for (int e = threadIdx.x; e < tsize; e += nthreads) {
      const int64_t g = base | dep_hi[e >> kLowBits] | (e & ((1 << kLowBits) - 1));
      stg_stream(sp + g, tp[smem_pos(e)]);
      stg_stream(sl + g, tl[smem_pos(e)]);
    }
    __syncthreads();
  }
  if (cur_circ >= 0) flush(cur_circ);
}

template <typename T>
static size_t adjoint_smem(int kt, int threads) {
  const int tsize = 1 << kt;
  return 4 * sizeof(T) * tile_stride(tsize) + sizeof(int64_t) * (1 << (kt - kLowBits)) +
         sizeof(double) * kAdjMaxGrad * (threads / 32);
}

// lambda = H psi for H = -sum_i Z_i Z_{i+1} - h sum_i X_i (open chain), all circuits
template <typename T>
__global__ void __launch_bounds__(256) k_tfim_apply(T* const* psi, T* const* lam, int n, int ncirc, double h) {
  const int64_t N = (int64_t)1 << n;
  const int64_t total = N * ncirc;
  const int64_t zzmask = (N >> 1) - 1;
  using R = typename real_of<T>::type;
  const R hh = (R)h;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(idx >> n);
    const int64_t k = idx & (N - 1);
    const T* s = psi[c];
    const T a = s[k];
    const int zz = (n - 1) - 2 * __popcll((unsigned long long)((k ^ (k >> 1)) & zzmask));
    T out;
    if constexpr (is_complex<T>::value) {
      R re = -(R)zz * a.re, im = -(R)zz * a.im;
      for (int b = 0; b < n; b++) {
        const T q = s[k ^ ((int64_t)1 << b)];
        re -= hh * q.re;
        im -= hh * q.im;
      }
      out = T{re, im};
    } else {
      R re = -(R)zz * a;
      for (int b = 0; b < n; b++) re -= hh * s[k ^ ((int64_t)1 << b)];
      out = re;
    }
    lam[c][k] = out;
  }
}

// per-circuit <psi|lambda> real part, FP64 (block partials, then a fixed-order finish)
template <typename T>
__global__ void __launch_bounds__(256) k_batch_dot_partials(T* const* psi, T* const* lam, int n, int nb,
                                                           double* partials) {
  const int c = blockIdx.y;
  const int64_t N = (int64_t)1 << n;
  double acc = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < N; k += (int64_t)nb * blockDim.x)
    acc += (double)re_cdot(psi[c][k], lam[c][k]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += part[w];
    partials[(int64_t)c * nb + blockIdx.x] = r;
  }
}

__global__ void k_rows_sum(const double* in, int64_t rows, int cols, double* out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0, comp = 0.0;
  for (int i = 0; i < cols; i++) {
    const double x = in[r * cols + i];
    const double t = s + x;
    comp += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  out[r] = s + comp;
}

struct AdjSegment {
  sv_program* fwd = nullptr;
  sv_program* bwd = nullptr;
  void* d_fcoef = nullptr;
  void* d_bcoef = nullptr;
};

}  // namespace sv

struct sv_adjoint {
  int dtype = 0, ncirc = 0, n = 0, nparams = 0, kt = 0;
  std::vector<sv::AdjSegment> segs;
  std::vector<std::vector<sv::HostOp>> fops;      // per circuit, forward (after parsing, no merging)
  std::vector<std::vector<sv::HostOp>> bops;      // per circuit per segment, backward lists (concatenated)
  std::vector<int> seg_begin;                     // op index where each segment starts (+ end)
  void* d_psi = nullptr;
  void* d_lam = nullptr;
  void* d_cp = nullptr;                           // (nseg - 1) checkpoints per circuit
  void* d_ptrs = nullptr;                         // [psi ptrs | lam ptrs]
  size_t stride = 0;                              // elements per state
  double* d_gpart = nullptr;
  double* d_grad = nullptr;
  double* d_epart = nullptr;
  double* d_energy = nullptr;
  int gstride = 0;
  int enb = 0;
};

namespace sv {

static std::vector<HostOp> backward_list(const std::vector<HostOp>& fwd, int b, int e, const int8_t* gens,
                                         const int32_t* params) {
  std::vector<HostOp> out;
  for (int j = e - 1; j >= b; j--) {
    const HostOp& h = fwd[j];
    if (gens && gens[j] > 0) {
      HostOp g;
      g.kind = OP_GRAD;
      g.nt = 1;
      g.tpos[0] = h.tpos[0];
      g.nc = 0;
      g.gen = gens[j];
      g.param = params[j];
      out.push_back(g);
    }
    // the inverse: conjugate transpose (diagonal: conjugate)
    HostOp inv = h;
    if (h.kind == SV_OP_DIAG) {
      for (size_t k = 1; k < inv.m.size(); k += 2) inv.m[k] = -inv.m[k];
    } else {
      const int d = 1 << h.nt;
      for (int r = 0; r < d; r++)
        for (int c = 0; c < d; c++) {
          inv.m[2 * (r * d + c)] = h.m[2 * (c * d + r)];
          inv.m[2 * (r * d + c) + 1] = -h.m[2 * (c * d + r) + 1];
        }
    }
    classify(inv);
    out.push_back(inv);
  }
  return out;
}

template <typename T>
static int gather_coef(const sv_program* prog, const std::vector<std::vector<HostOp>>& per_circ, void** d) {
  const size_t nc = per_circ.size(), ct = prog->coef_total;
  if (ct == 0) return SV_OK;
  std::vector<T> coef(nc * ct);
  for (size_t i = 0; i < nc; i++)
    for (size_t sl = 0; sl < ct; sl++) {
      const int op = prog->coef_src[2 * sl], e = prog->coef_src[2 * sl + 1];
      coef[i * ct + sl] = to_elem<T>(&per_circ[i][op].m[2 * e]);
    }
  if (!*d) SV_TRY(check_cuda(cudaMalloc(d, nc * ct * sizeof(T)), "adjoint coefficients"));
  return check_cuda(cudaMemcpy(*d, coef.data(), nc * ct * sizeof(T), cudaMemcpyHostToDevice), "coef upload");
}

template <typename T, int MAXT, int MINB>
static int launch_adj(Context* ctx, const PassParams<T>& p, const AdjArgs<T>& a, int threads) {
  if (threads < 32 || threads % 32) return set_error(SV_ERR_ARG, "adjoint passes need whole warps");
  auto kern = k_adjoint_pass<T, MAXT, MINB>;
  const size_t smem = adjoint_smem<T>(p.kt, threads);
  static size_t attr = 0;
  if (smem > attr) {
    SV_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr"));
    attr = smem;
  }
  int per_sm = 0;
  SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem), "occupancy"));
  if (per_sm < 1) return set_error(SV_ERR_ARG, "adjoint tile does not fit on an SM");
  int64_t grid = (int64_t)per_sm * ctx->num_sms;
  const int64_t nitems = p.ntiles * a.ncirc;
  if (grid > nitems) grid = nitems;
  if (grid > a.gstride) grid = a.gstride;
  kern<<<(unsigned)grid, threads, smem, ctx->stream>>>(p, a);
  SV_LAUNCH_CHECK("adjoint pass launch");
  return SV_OK;
}

template <typename T>
static int adjoint_run_typed(Context* ctx, sv_adjoint* A, double h, double* energies, double* grads) {
  const int n = A->n, nc = A->ncirc;
  T* const* psi = (T* const*)A->d_ptrs;
  T* const* lam = psi + nc;
  const size_t sbytes = A->stride * sizeof(T);
  cudaStream_t st = ctx->stream;
  // forward from |0...0>, checkpointing psi after every segment but the last
  SV_TRY(check_cuda(cudaMemsetAsync(A->d_psi, 0, sbytes * nc, st), "zero"));
  k_batch_ones<T><<<grid_for(nc, 256), 256, 0, st>>>(psi, nc);
  SV_LAUNCH_CHECK("ones");
  const int nseg = (int)A->segs.size();
  for (int s = 0; s < nseg; s++) {
    const AdjSegment& sg = A->segs[s];
    BatchArgs<T> args;
    memset(&args, 0, sizeof(args));
    args.states = psi;
    args.coef = (const T*)sg.d_fcoef;
    args.coef_stride = (int64_t)sg.fwd->coef_total;
    args.ncirc = nc;
    const int threads = 1 << (sg.fwd->kt - kRB);
    for (const Segment& seg : sg.fwd->segments) {
      if (sg.fwd->bspec) {
        SV_TRY(specialized_launch_batched(ctx, sg.fwd, seg.pass, st, (void*)psi, sg.d_fcoef, args.coef_stride, nc));
        continue;
      }
      const PassParams<T>& p =
          *reinterpret_cast<const PassParams<T>*>(sg.fwd->passes.data() + (size_t)seg.pass * sg.fwd->pass_bytes);
      SV_TRY(launch_pass<T, true>(ctx, p, nullptr, threads, pass_smem<T>(sg.fwd->kt), p.ntiles * nc, st, args));
    }
    if (s < nseg - 1)
      SV_TRY(check_cuda(cudaMemcpyAsync((char*)A->d_cp + (size_t)s * sbytes * nc, A->d_psi, sbytes * nc,
                                        cudaMemcpyDeviceToDevice, st), "checkpoint"));
  }
  // lambda = H psi, energies = Re <psi|lambda>
  {
    const int64_t total = ((int64_t)1 << n) * nc;
    int64_t g = (total + 255) / 256;
    if (g > (int64_t)ctx->num_sms * 16) g = (int64_t)ctx->num_sms * 16;
    k_tfim_apply<T><<<(unsigned)g, 256, 0, st>>>(psi, (T* const*)lam, n, nc, h);
    SV_LAUNCH_CHECK("tfim apply");
    dim3 grid(A->enb, nc);
    k_batch_dot_partials<T><<<grid, 256, 0, st>>>(psi, lam, n, A->enb, A->d_epart);
    SV_LAUNCH_CHECK("energy partials");
    k_rows_sum<<<grid_for(nc, 128), 128, 0, st>>>(A->d_epart, nc, A->enb, A->d_energy);
    SV_LAUNCH_CHECK("energy finish");
  }
  // reverse sweep
  SV_TRY(check_cuda(cudaMemsetAsync(A->d_gpart, 0, sizeof(double) * (size_t)nc * A->nparams * A->gstride, st),
                    "zero gradients"));
  for (int s = nseg - 1; s >= 0; s--) {
    if (s < nseg - 1)  // restore the exact forward state at this segment's end
      SV_TRY(check_cuda(cudaMemcpyAsync(A->d_psi, (char*)A->d_cp + (size_t)s * sbytes * nc, sbytes * nc,
                                        cudaMemcpyDeviceToDevice, st), "restore"));
    const AdjSegment& sg = A->segs[s];
    AdjArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.psi = psi;
    a.lam = lam;
    a.coef = (const T*)sg.d_bcoef;
    a.coef_stride = (int64_t)sg.bwd->coef_total;
    a.gpart = A->d_gpart;
    a.ncirc = nc;
    a.nparams = A->nparams;
    a.gstride = A->gstride;
    const int threads = 1 << (sg.bwd->kt - kRB);
    for (const Segment& seg : sg.bwd->segments) {
      if (sg.bwd->aspec) {
        SV_TRY(specialized_launch_adjoint(ctx, sg.bwd, seg.pass, (void*)psi, (void*)lam, sg.d_bcoef, a.coef_stride, nc,
                                          A->d_gpart, A->nparams, A->gstride));
        continue;
      }
      const PassParams<T>& p =
          *reinterpret_cast<const PassParams<T>*>(sg.bwd->passes.data() + (size_t)seg.pass * sg.bwd->pass_bytes);
      if constexpr (sizeof(T) >= 16) SV_TRY(launch_adj<T, 256, 1>(ctx, p, a, threads));
      else SV_TRY(launch_adj<T, 256, 2>(ctx, p, a, threads));
    }
  }
  k_rows_sum<<<grid_for((int64_t)nc * A->nparams, 128), 128, 0, st>>>(A->d_gpart, (int64_t)nc * A->nparams,
                                                                      A->gstride, A->d_grad);
  SV_LAUNCH_CHECK("gradient finish");
  if (energies)
    SV_TRY(check_cuda(cudaMemcpyAsync(energies, A->d_energy, nc * sizeof(double), cudaMemcpyDeviceToHost, st), "E"));
  if (grads)
    SV_TRY(check_cuda(cudaMemcpyAsync(grads, A->d_grad, (size_t)nc * A->nparams * sizeof(double),
                                      cudaMemcpyDeviceToHost, st), "grad"));
  return check_cuda(cudaStreamSynchronize(st), "adjoint sync");
}

static void adjoint_free(sv_adjoint* A) {
  if (!A) return;
  for (auto& s : A->segs) {
    delete s.fwd;
    delete s.bwd;
    if (s.d_fcoef) cudaFree(s.d_fcoef);
    if (s.d_bcoef) cudaFree(s.d_bcoef);
  }
  for (void* p : {A->d_psi, A->d_lam, A->d_cp, A->d_ptrs, (void*)A->d_gpart, (void*)A->d_grad, (void*)A->d_epart,
                  (void*)A->d_energy})
    if (p) cudaFree(p);
  delete A;
}

}  // namespace sv

extern "C" {

int sv_adjoint_create(sv_context* ctx, int dtype, int ncirc, int nqubits, const sv_gate_op* const* ops, int nops,
                      const int8_t* generators, const int32_t* params, int nparams, const int32_t* segment_ends,
                      int nsegments, int tile_bits, sv_adjoint** out) {
  if (!ctx || !out || !ops || !generators || !params || ncirc < 1 || nops < 1 || nparams < 1 || !segment_ends ||
      nsegments < 1)
    return set_error(SV_ERR_ARG, "bad adjoint arguments");
  *out = nullptr;
  if (dtype != SV_C128 && dtype != SV_C64) return set_error(SV_ERR_UNSUPPORTED, "adjoint needs a complex dtype");
  if (nqubits < kRB + 5 || nqubits > 34) return set_error(SV_ERR_ARG, "adjoint needs 9..34 qubits");
  for (int j = 0; j < nops; j++) {
    if (generators[j] < 0 || generators[j] > 3) return set_error(SV_ERR_ARG, "op %d: generator must be 0..3", j);
    if (generators[j] > 0) {
      if (params[j] < 0 || params[j] >= nparams) return set_error(SV_ERR_ARG, "op %d: parameter out of range", j);
      if (ops[0][j].ntargets != 1 || ops[0][j].ncontrols != 0)
        return set_error(SV_ERR_UNSUPPORTED, "op %d: parametrised gates must act on one qubit without controls", j);
    }
  }
  for (int s = 0; s < nsegments; s++)
    if (segment_ends[s] < 1 || segment_ends[s] > nops || (s > 0 && segment_ends[s] <= segment_ends[s - 1]) ||
        (s == nsegments - 1 && segment_ends[s] != nops))
      return set_error(SV_ERR_ARG, "segment ends must increase and end at nops");
  int kt = 0;
  // two states per tile: default one bit smaller than a forward tile
  SV_TRY(check_tile_bits(dtype, nqubits, tile_bits > 0 ? tile_bits : (dtype == SV_C128 ? 10 : 11), &kt));
  // the reverse sweep reduces with whole-warp shuffles: a tile needs >= 32 threads (2^(kt-4))
  if (kt < kRB + 5)
    return set_error(SV_ERR_ARG, "adjoint gradients need tiles of >= %d bits (circuits of >= %d qubits)", kRB + 5,
                     kRB + 5);
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  sv_adjoint* A = new sv_adjoint();
  A->dtype = dtype;
  A->ncirc = ncirc;
  A->n = nqubits;
  A->nparams = nparams;
  A->kt = kt;
  // parse every circuit (no merging: gradients sit between gates), check one structure
  for (int c = 0; c < ncirc; c++) {
    std::vector<HostOp> h;
    int rc = SV_OK;
    for (int j = 0; j < nops && rc == SV_OK; j++) {
      std::vector<HostOp> one;
      rc = parse_ops(nqubits, &ops[c][j], 1, &one);  // one op: merging cannot apply
      if (rc == SV_OK) h.push_back(one[0]);
    }
    if (rc == SV_OK && c > 0 && !same_structure(A->fops[0], h))
      rc = set_error(SV_ERR_ARG, "circuit %d differs in structure from circuit 0", c);
    if (rc != SV_OK) {
      adjoint_free(A);
      return rc;
    }
    A->fops.push_back(std::move(h));
  }
  int rc = SV_OK;
  int b0 = 0;
  for (int s = 0; s < nsegments && rc == SV_OK; s++) {
    const int e0 = segment_ends[s];
    AdjSegment sg;
    std::vector<std::vector<HostOp>> fper(ncirc), bper(ncirc);
    for (int c = 0; c < ncirc; c++) {
      fper[c].assign(A->fops[c].begin() + b0, A->fops[c].begin() + e0);
      bper[c] = backward_list(A->fops[c], b0, e0, generators, params);
    }
    std::vector<HostOp> f0 = fper[0], bw0 = bper[0];
    // forward passes hold one state per tile: one bit more than the backward tiles
    int ktf = kt + 1;
    if (ktf > nqubits) ktf = nqubits;
    if (ktf > (dtype == SV_C128 ? 12 : 13)) ktf = kt;
    rc = plan(dtype, nqubits, ktf, std::move(f0), &sg.fwd, false, false);
    if (rc == SV_OK) rc = plan(dtype, nqubits, kt, std::move(bw0), &sg.bwd, false, false);
    if (rc == SV_OK && (sg.fwd->nunfused || sg.bwd->nunfused))
      rc = set_error(SV_ERR_UNSUPPORTED, "adjoint circuits need gates on at most 2 targets");
    if (rc == SV_OK)
      rc = dtype == SV_C128 ? gather_coef<c128>(sg.fwd, fper, &sg.d_fcoef) : gather_coef<c64>(sg.fwd, fper, &sg.d_fcoef);
    if (rc == SV_OK)
      rc = dtype == SV_C128 ? gather_coef<c128>(sg.bwd, bper, &sg.d_bcoef) : gather_coef<c64>(sg.bwd, bper, &sg.d_bcoef);
    A->segs.push_back(sg);
    b0 = e0;
  }
  const size_t es = dtype_size(dtype);
  A->stride = ((((size_t)1 << nqubits) * es + 255) / 256) * 256 / es;
  const size_t sbytes = A->stride * es;
  A->gstride = ctx->num_sms * 4;
  A->enb = 64;
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_psi, sbytes * ncirc), "psi");
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_lam, sbytes * ncirc), "lambda");
  if (rc == SV_OK && nsegments > 1)
    rc = check_cuda(cudaMalloc(&A->d_cp, sbytes * ncirc * (nsegments - 1)), "checkpoints");
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_gpart, sizeof(double) * (size_t)ncirc * nparams * A->gstride), "g");
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_grad, sizeof(double) * (size_t)ncirc * nparams), "grad");
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_epart, sizeof(double) * (size_t)ncirc * A->enb), "e");
  if (rc == SV_OK) rc = check_cuda(cudaMalloc(&A->d_energy, sizeof(double) * ncirc), "energy");
  if (rc == SV_OK) {
    std::vector<void*> ptrs(2 * ncirc);
    for (int c = 0; c < ncirc; c++) {
      ptrs[c] = (char*)A->d_psi + c * sbytes;
      ptrs[ncirc + c] = (char*)A->d_lam + c * sbytes;
    }
    rc = check_cuda(cudaMalloc(&A->d_ptrs, ptrs.size() * sizeof(void*)), "pointers");
    if (rc == SV_OK)
      rc = check_cuda(cudaMemcpy(A->d_ptrs, ptrs.data(), ptrs.size() * sizeof(void*), cudaMemcpyHostToDevice), "ptrs");
  }
  if (rc != SV_OK) {
    adjoint_free(A);
    return rc;
  }
  *out = A;
  return SV_OK;
}

int sv_adjoint_update(sv_context* ctx, sv_adjoint* A, const sv_gate_op* const* ops, int nops,
                      const int8_t* generators, const int32_t* params) {
  if (!ctx || !A || !ops || !generators || !params) return set_error(SV_ERR_ARG, "bad adjoint update");
  if (nops != (int)A->fops[0].size()) return set_error(SV_ERR_ARG, "op count differs from the planned circuits");
  for (int c = 0; c < A->ncirc; c++) {
    std::vector<HostOp> h;
    for (int j = 0; j < nops; j++) {
      std::vector<HostOp> one;
      SV_TRY(parse_ops(A->n, &ops[c][j], 1, &one));
      h.push_back(one[0]);
    }
    if (!same_structure(A->fops[0], h)) return set_error(SV_ERR_ARG, "circuit %d changed structure", c);
    A->fops[c] = std::move(h);
  }
  int b0 = 0;
  for (auto& sg : A->segs) {
    const int e0 = b0 + (int)sg.fwd->ops.size();
    std::vector<std::vector<HostOp>> fper(A->ncirc), bper(A->ncirc);
    for (int c = 0; c < A->ncirc; c++) {
      fper[c].assign(A->fops[c].begin() + b0, A->fops[c].begin() + e0);
      bper[c] = backward_list(A->fops[c], b0, e0, generators, params);
    }
    if (A->dtype == SV_C128) {
      SV_TRY(gather_coef<c128>(sg.fwd, fper, &sg.d_fcoef));
      SV_TRY(gather_coef<c128>(sg.bwd, bper, &sg.d_bcoef));
    } else {
      SV_TRY(gather_coef<c64>(sg.fwd, fper, &sg.d_fcoef));
      SV_TRY(gather_coef<c64>(sg.bwd, bper, &sg.d_bcoef));
    }
    b0 = e0;
  }
  return SV_OK;
}

int sv_adjoint_run(sv_context* ctx, sv_adjoint* A, double h, double* energies, double* grads) {
  if (!ctx || !A) return set_error(SV_ERR_ARG, "null context or adjoint");
  return A->dtype == SV_C128 ? adjoint_run_typed<c128>(ctx, A, h, energies, grads)
                             : adjoint_run_typed<c64>(ctx, A, h, energies, grads);
}

int sv_adjoint_specialize(sv_context* ctx, sv_adjoint* A) {
  if (!ctx || !A) return set_error(SV_ERR_ARG, "null context or adjoint");
  SV_TRY(check_cuda(cudaSetDevice(ctx->device), "cudaSetDevice"));
  for (auto& sg : A->segs) {
    SV_TRY(specialize_batched(ctx, sg.fwd, false));
    SV_TRY(specialize_adjoint(ctx, sg.bwd));
  }
  return SV_OK;
}

int sv_adjoint_state(const sv_adjoint* A, int circuit, void** psi) {
  if (!A || circuit < 0 || circuit >= A->ncirc || !psi) return set_error(SV_ERR_ARG, "bad adjoint query");
  *psi = (char*)A->d_psi + (size_t)circuit * A->stride * dtype_size(A->dtype);
  return SV_OK;
}

int sv_adjoint_destroy(sv_adjoint* A) {
  adjoint_free(A);
  return SV_OK;
}

}  // extern "C"
