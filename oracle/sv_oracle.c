/*
 * sv_oracle.c -- CPU restatement of qibojit's Numba state-vector kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA engine in
 * qibojit_gb300/ is compared against, and the CPU baseline that bench.py times
 * beside it.  Nothing in the product path links, loads or calls it.
 *
 * Every routine follows one function of the reference (paths are relative to
 * the qibojit project root) with the same index maps and the same arithmetic
 * order, so that for a single thread the results are bit-identical to the
 * reference run in NUMBA_DISABLE_JIT mode (plain Python complex arithmetic:
 * (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re), no fused multiply-add).
 * Build with -ffp-contract=off -fcx-limited-range to keep that property.
 *
 *   oracle_multicontrol_index   src/qibojit/custom_operators/gates.py:5-12
 *   oracle_one_qubit            gates.py:15-114  (apply_gate/x/y/z/z_pow, +multicontrol)
 *   oracle_two_qubit            gates.py:117-254 (two_qubit_gate/swap/fsim, +multicontrol)
 *   oracle_multi_qubit          gates.py:257-424 (three/four/five/generic)
 *   oracle_initial_state        src/qibojit/custom_operators/ops.py:10-18
 *   oracle_collapse_state       ops.py:33-79 (collapse_index, collapse_state(_normalized))
 *   oracle_measure_frequencies  ops.py:82-108 (Metropolis chains, NumPy legacy RNG)
 *   oracle_probabilities        qibo Backend.calculate_probabilities (restated from its
 *                               published semantics: |psi|^2 marginalised, ordered as `qubits`)
 *
 * The random number streams reproduce NumPy's legacy RandomState (the generator the
 * reference's known-answer test tests/test_ops.py:236-256 was produced with):
 * MT19937 (Matsumoto & Nishimura 1998) seeded with init_genrand, randint(0, n) as a
 * masked draw of the low bits of one 32-bit word with rejection, and random() as the
 * 53-bit double (a>>5)*2^26 + (b>>6) over 2^53.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { DT_C128 = 0, DT_C64 = 1, DT_F64 = 2, DT_F32 = 3 };
enum { K_GATE = 0, K_X = 1, K_Y = 2, K_Z = 3, K_ZPOW = 4 };
enum { K2_GATE = 0, K2_SWAP = 1, K2_FSIM = 2 };

typedef double _Complex c128;
typedef float _Complex c64;

int64_t oracle_multicontrol_index(int64_t g, const int32_t *qubits, int nq) {
  int64_t i = g;
  for (int j = 0; j < nq; j++) {
    const int n = qubits[j];
    const int64_t k = (int64_t)1 << n;
    i = ((i >> n) << (n + 1)) + (i & (k - 1)) + k;
  }
  return i;
}

static int64_t multitarget_index(int64_t i, const int64_t *targets, int nt) {
  int64_t t = 0;
  for (int u = 0; u < nt; u++) t += ((i >> u) & 1) * targets[u];
  return t;
}

static int64_t collapse_index(int64_t g, int64_t h, const int32_t *qubits, int nq) {
  int64_t i = g;
  for (int j = 0; j < nq; j++) {
    const int n = qubits[j];
    const int64_t k = (int64_t)1 << n;
    i = ((i >> n) << (n + 1)) + (i & (k - 1)) + ((h >> j) % 2) * k;
  }
  return i;
}

/* ---------------------------------------------------------------- one qubit */
#define ONE_QUBIT(T, NAME)                                                        \
  static void NAME(T *state, const T *gate, const int32_t *qubits, int nq,        \
                   int64_t nstates, int m, int kind) {                            \
    const int64_t tk = (int64_t)1 << m;                                           \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (int64_t g = 0; g < nstates; g++) {                                       \
      int64_t i1, i2;                                                             \
      if (nq) {                                                                   \
        const int64_t i = oracle_multicontrol_index(g, qubits, nq);               \
        i1 = i - tk;                                                              \
        i2 = i;                                                                   \
      } else {                                                                    \
        i1 = ((g >> m) << (m + 1)) + (g & (tk - 1));                              \
        i2 = i1 + tk;                                                             \
      }                                                                           \
      switch (kind) {                                                             \
        case K_GATE: {                                                            \
          const T a = state[i1], b = state[i2];                                   \
          state[i1] = gate[0] * a + gate[1] * b;                                  \
          state[i2] = gate[2] * a + gate[3] * b;                                  \
        } break;                                                                  \
        case K_X: {                                                               \
          const T a = state[i1];                                                  \
          state[i1] = state[i2];                                                  \
          state[i2] = a;                                                          \
        } break;                                                                  \
        case K_Z: state[i2] *= -1; break;                                         \
        case K_ZPOW: state[i2] = gate[0] * state[i2]; break;                      \
        default: break;                                                           \
      }                                                                           \
    }                                                                             \
  }
ONE_QUBIT(c128, one_c128)
ONE_QUBIT(c64, one_c64)
ONE_QUBIT(double, one_f64)
ONE_QUBIT(float, one_f32)

/* Y is complex only: (a, b) <- (-i b, i a), gates.py:61-78.  The reference
 * multiplies by the complex scalars -1j / 1j, i.e. (0-1i)*(br+bi i) with the
 * plain complex product, which is (0*br - (-1)*bi) + (0*bi + (-1)*br) i.       */
#define Y_QUBIT(T, R, NAME)                                                       \
  static void NAME(T *state, const int32_t *qubits, int nq, int64_t nstates,      \
                   int m) {                                                       \
    const int64_t tk = (int64_t)1 << m;                                           \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (int64_t g = 0; g < nstates; g++) {                                       \
      int64_t i1, i2;                                                             \
      if (nq) {                                                                   \
        const int64_t i = oracle_multicontrol_index(g, qubits, nq);               \
        i1 = i - tk;                                                              \
        i2 = i;                                                                   \
      } else {                                                                    \
        i1 = ((g >> m) << (m + 1)) + (g & (tk - 1));                              \
        i2 = i1 + tk;                                                             \
      }                                                                           \
      const T a = state[i1], b = state[i2];                                       \
      const T mi = (T)(-1.0 * I), pi = (T)(1.0 * I);                              \
      state[i1] = mi * b;                                                         \
      state[i2] = pi * a;                                                         \
    }                                                                             \
  }
Y_QUBIT(c128, double, y_c128)
Y_QUBIT(c64, float, y_c64)

int oracle_one_qubit(int dtype, int kind, void *state, const void *gate,
                     const int32_t *qubits, int nq, int64_t nstates, int m) {
  if (kind == K_Y) {
    if (dtype == DT_C128) y_c128((c128 *)state, qubits, nq, nstates, m);
    else if (dtype == DT_C64) y_c64((c64 *)state, qubits, nq, nstates, m);
    else return 1;
    return 0;
  }
  switch (dtype) {
    case DT_C128: one_c128((c128 *)state, (const c128 *)gate, qubits, nq, nstates, m, kind); break;
    case DT_C64: one_c64((c64 *)state, (const c64 *)gate, qubits, nq, nstates, m, kind); break;
    case DT_F64: one_f64((double *)state, (const double *)gate, qubits, nq, nstates, m, kind); break;
    case DT_F32: one_f32((float *)state, (const float *)gate, qubits, nq, nstates, m, kind); break;
    default: return 1;
  }
  return 0;
}

/* ---------------------------------------------------------------- two qubits */
/* Quad ordering, gates.py:117-193: plain kernels insert zeros at m1 < m2 and use
 * (i, i+uk1, i+uk2, i+tk1+tk2); multicontrol kernels start from the all-ones index
 * and use (i-uk1-uk2, i-uk2, i-uk1, i).  uk1, uk2 = tk1, tk2, swapped when
 * swap_targets.  The 4x4 update reads the three partially-updated buffers the
 * same way the reference does.                                                 */
#define TWO_QUBIT(T, NAME)                                                        \
  static void NAME(T *state, const T *gate, const int32_t *qubits, int nq,        \
                   int64_t nstates, int m1, int m2, int swap_targets, int kind) { \
    const int64_t tk1 = (int64_t)1 << m1, tk2 = (int64_t)1 << m2;                 \
    int64_t uk1 = tk1, uk2 = tk2;                                                 \
    if (swap_targets) { uk1 = tk2; uk2 = tk1; }                                   \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (int64_t g = 0; g < nstates; g++) {                                       \
      int64_t i0, i1, i2, i3;                                                     \
      if (nq) {                                                                   \
        i3 = oracle_multicontrol_index(g, qubits, nq);                            \
        if (kind == K2_SWAP) {                                                    \
          i1 = i3 - tk2; i2 = i3 - tk1;                                           \
        } else {                                                                  \
          i1 = i3 - uk2; i2 = i3 - uk1;                                           \
        }                                                                         \
        i0 = i1 - uk1;                                                            \
      } else {                                                                    \
        int64_t i = ((g >> m1) << (m1 + 1)) + (g & (tk1 - 1));                    \
        i = ((i >> m2) << (m2 + 1)) + (i & (tk2 - 1));                            \
        i0 = i;                                                                   \
        if (kind == K2_SWAP) { i1 = i + tk1; i2 = i + tk2; }                      \
        else { i1 = i + uk1; i2 = i + uk2; }                                      \
        i3 = i + tk1 + tk2;                                                       \
      }                                                                           \
      if (kind == K2_GATE) {                                                      \
        const T b0 = state[i0], b1 = state[i1], b2 = state[i2];                   \
        state[i0] = gate[0] * state[i0] + gate[1] * state[i1] +                   \
                    gate[2] * state[i2] + gate[3] * state[i3];                    \
        state[i1] = gate[4] * b0 + gate[5] * state[i1] + gate[6] * state[i2] +    \
                    gate[7] * state[i3];                                          \
        state[i2] = gate[8] * b0 + gate[9] * b1 + gate[10] * state[i2] +          \
                    gate[11] * state[i3];                                         \
        state[i3] = gate[12] * b0 + gate[13] * b1 + gate[14] * b2 +               \
                    gate[15] * state[i3];                                         \
      } else if (kind == K2_SWAP) {                                               \
        const T a = state[i1];                                                    \
        state[i1] = state[i2];                                                    \
        state[i2] = a;                                                            \
      } else {                                                                    \
        const T a = state[i1], b = state[i2];                                     \
        state[i1] = gate[0] * a + gate[1] * b;                                    \
        state[i2] = gate[2] * a + gate[3] * b;                                    \
        state[i3] *= gate[4];                                                     \
      }                                                                           \
    }                                                                             \
  }
TWO_QUBIT(c128, two_c128)
TWO_QUBIT(c64, two_c64)
TWO_QUBIT(double, two_f64)
TWO_QUBIT(float, two_f32)

int oracle_two_qubit(int dtype, int kind, void *state, const void *gate,
                     const int32_t *qubits, int nq, int64_t nstates, int m1, int m2,
                     int swap_targets) {
  switch (dtype) {
    case DT_C128: two_c128((c128 *)state, (const c128 *)gate, qubits, nq, nstates, m1, m2, swap_targets, kind); break;
    case DT_C64: two_c64((c64 *)state, (const c64 *)gate, qubits, nq, nstates, m1, m2, swap_targets, kind); break;
    case DT_F64: two_f64((double *)state, (const double *)gate, qubits, nq, nstates, m1, m2, swap_targets, kind); break;
    case DT_F32: two_f32((float *)state, (const float *)gate, qubits, nq, nstates, m1, m2, swap_targets, kind); break;
    default: return 1;
  }
  return 0;
}

/* -------------------------------------------------------------- multi qubit */
/* gates.py:412-424 (and the unrolled 3/4/5-target versions :265-409, which compute
 * the same sums): buffer[i] = state[ig - multitarget_index(N-1-i)], then
 * state[ig - multitarget_index(N-1-i)] = sum_j gate[i, j] * buffer[j],
 * summed left to right.                                                        */
#define MULTI_QUBIT(T, NAME)                                                      \
  static void NAME(T *state, const T *gate, const int32_t *qubits, int nq,        \
                   int64_t nstates, const int64_t *targets, int nt) {             \
    const int64_t ns = (int64_t)1 << nt;                                          \
    _Pragma("omp parallel")                                                       \
    {                                                                             \
      T *buffer = (T *)malloc(sizeof(T) * ns);                                    \
      _Pragma("omp for schedule(static)")                                         \
      for (int64_t g = 0; g < nstates; g++) {                                     \
        const int64_t ig = oracle_multicontrol_index(g, qubits, nq);              \
        for (int64_t i = 0; i < ns; i++)                                          \
          buffer[i] = state[ig - multitarget_index(ns - i - 1, targets, nt)];     \
        for (int64_t i = 0; i < ns; i++) {                                        \
          T acc = gate[i * ns] * buffer[0];                                       \
          for (int64_t j = 1; j < ns; j++) acc = acc + gate[i * ns + j] * buffer[j]; \
          state[ig - multitarget_index(ns - i - 1, targets, nt)] = acc;           \
        }                                                                         \
      }                                                                           \
      free(buffer);                                                               \
    }                                                                             \
  }
MULTI_QUBIT(c128, multi_c128)
MULTI_QUBIT(c64, multi_c64)
MULTI_QUBIT(double, multi_f64)
MULTI_QUBIT(float, multi_f32)

int oracle_multi_qubit(int dtype, void *state, const void *gate, const int32_t *qubits,
                       int nq, int64_t nstates, const int64_t *targets, int nt) {
  switch (dtype) {
    case DT_C128: multi_c128((c128 *)state, (const c128 *)gate, qubits, nq, nstates, targets, nt); break;
    case DT_C64: multi_c64((c64 *)state, (const c64 *)gate, qubits, nq, nstates, targets, nt); break;
    case DT_F64: multi_f64((double *)state, (const double *)gate, qubits, nq, nstates, targets, nt); break;
    case DT_F32: multi_f32((float *)state, (const float *)gate, qubits, nq, nstates, targets, nt); break;
    default: return 1;
  }
  return 0;
}

/* ------------------------------------------------------------ initial state */
int oracle_initial_state(int dtype, void *state, int64_t n) {
  static const size_t width[4] = {16, 8, 8, 4};
  if (dtype < 0 || dtype > 3) return 1;
  memset(state, 0, width[dtype] * (size_t)n);
  switch (dtype) {
    case DT_C128: ((c128 *)state)[0] = 1; break;
    case DT_C64: ((c64 *)state)[0] = 1; break;
    case DT_F64: ((double *)state)[0] = 1; break;
    case DT_F32: ((float *)state)[0] = 1; break;
  }
  return 0;
}

/* ----------------------------------------------------------------- collapse */
/* ops.py:43-79.  `qubits` are the reversed bit positions the backend passes
 * (cpu.py:550-552).  The normalised version accumulates |kept|^2 in double for
 * complex128 (np.abs(c128)**2 is float64) and in float for complex64 (np.abs of a
 * complex64 is float32 and `norms` is promoted to its type), then divides.      */
#define COLLAPSE(T, R, ABS, SQRT, NAME)                                           \
  static void NAME(T *state, const int32_t *qubits, int nq, int64_t result,       \
                   int nqubits, int normalize) {                                  \
    const int64_t nstates = (int64_t)1 << (nqubits - nq);                         \
    const int64_t nsub = (int64_t)1 << nq;                                        \
    R norms = 0;                                                                  \
    _Pragma("omp parallel for schedule(static) reduction(+:norms)")               \
    for (int64_t g = 0; g < nstates; g++) {                                       \
      for (int64_t h = 0; h < result; h++) state[collapse_index(g, h, qubits, nq)] = 0; \
      if (normalize) {                                                            \
        const R a = ABS(state[collapse_index(g, result, qubits, nq)]);            \
        norms += a * a;                                                           \
      }                                                                           \
      for (int64_t h = result + 1; h < nsub; h++)                                 \
        state[collapse_index(g, h, qubits, nq)] = 0;                              \
    }                                                                             \
    if (!normalize) return;                                                       \
    const R norm = SQRT(norms);                                                   \
    _Pragma("omp parallel for schedule(static)")                                  \
    for (int64_t g = 0; g < nstates; g++) {                                       \
      const int64_t i = collapse_index(g, result, qubits, nq);                    \
      state[i] = DIV(state[i], norm);                                             \
    }                                                                             \
  }
/* NumPy divides a complex scalar by a real one as a complex division with
 * Smith's scaling, which for a zero imaginary part is a product with 1/norm. */
#define CDIV(a, n) ((a) * (1 / (n)))
#define RDIV(a, n) ((a) / (n))
#define DIV CDIV
COLLAPSE(c128, double, cabs, sqrt, collapse_c128)
COLLAPSE(c64, float, cabsf, sqrtf, collapse_c64)
#undef DIV
#define DIV RDIV
COLLAPSE(double, double, fabs, sqrt, collapse_f64)
COLLAPSE(float, float, fabsf, sqrtf, collapse_f32)
#undef DIV

int oracle_collapse_state(int dtype, void *state, const int32_t *qubits, int nq,
                          int64_t result, int nqubits, int normalize) {
  switch (dtype) {
    case DT_C128: collapse_c128((c128 *)state, qubits, nq, result, nqubits, normalize); break;
    case DT_C64: collapse_c64((c64 *)state, qubits, nq, result, nqubits, normalize); break;
    case DT_F64: collapse_f64((double *)state, qubits, nq, result, nqubits, normalize); break;
    case DT_F32: collapse_f32((float *)state, qubits, nq, result, nqubits, normalize); break;
    default: return 1;
  }
  return 0;
}

/* ------------------------------------------------------------ probabilities */
/* |psi|^2 summed over the qubits not in `qubits`; output index bit for qubits[j]
 * is bit (nm-1-j), i.e. qubits[0] is the most significant, in the order given.
 * Accumulates in double.  `out` has 2^nm doubles.                              */
int oracle_probabilities(int dtype, const void *state, int nqubits, const int32_t *qubits,
                         int nm, double *out) {
  const int64_t n = (int64_t)1 << nqubits;
  const int64_t nout = (int64_t)1 << nm;
  memset(out, 0, sizeof(double) * (size_t)nout);
  for (int64_t i = 0; i < n; i++) {
    double p;
    switch (dtype) {
      case DT_C128: { const c128 a = ((const c128 *)state)[i]; p = creal(a) * creal(a) + cimag(a) * cimag(a); } break;
      case DT_C64: { const c64 a = ((const c64 *)state)[i]; const float pf = crealf(a) * crealf(a) + cimagf(a) * cimagf(a); p = pf; } break;
      case DT_F64: { const double a = ((const double *)state)[i]; p = a * a; } break;
      case DT_F32: { const float a = ((const float *)state)[i]; p = (double)(a * a); } break;
      default: return 1;
    }
    int64_t o = 0;
    for (int j = 0; j < nm; j++) {
      const int bit = nqubits - 1 - qubits[j];
      o |= ((i >> bit) & 1) << (nm - 1 - j);
    }
    out[o] += p;
  }
  return 0;
}

/* --------------------------------------------------- NumPy legacy MT19937 */
typedef struct {
  uint32_t mt[624];
  int pos;
} mt_state;

static void mt_seed(mt_state *s, uint32_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->pos = 624;
}

static uint32_t mt_next(mt_state *s) {
  if (s->pos >= 624) {
    for (int k = 0; k < 624; k++) {
      const uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7fffffffu);
      s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    s->pos = 0;
  }
  uint32_t y = s->mt[s->pos++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

/* randint(0, high) for 1 <= high <= 2^32: masked rejection on one word. */
static uint32_t mt_randint(mt_state *s, uint64_t high) {
  const uint64_t rng = high - 1;
  if (rng == 0) return 0;
  uint64_t mask = rng;
  mask |= mask >> 1; mask |= mask >> 2; mask |= mask >> 4;
  mask |= mask >> 8; mask |= mask >> 16;
  uint64_t v;
  do { v = mt_next(s) & mask; } while (v > rng);
  return (uint32_t)v;
}

static double mt_random(mt_state *s) {
  const uint32_t a = mt_next(s) >> 5, b = mt_next(s) >> 6;
  return (a * 67108864.0 + b) / 9007199254740992.0;
}

/* Raw legacy stream for tests: `out` receives `count` values of kind
 * 0 = next 32-bit word, 1 = randint(0, high), 2 = random().                    */
int oracle_mt_stream(uint32_t seed, int kind, uint64_t high, int64_t count, double *out) {
  mt_state s;
  mt_seed(&s, seed);
  for (int64_t i = 0; i < count; i++) {
    if (kind == 0) out[i] = (double)mt_next(&s);
    else if (kind == 1) out[i] = (double)mt_randint(&s, high);
    else out[i] = mt_random(&s);
  }
  return 0;
}

/* ops.py:82-108.  probs are float64 (realtype 0) or float32 (realtype 1).  For
 * float32 the reference, run as plain NumPy 2 code, forms the ratio in float32 and
 * compares it with random() rounded to float32 (NEP 50 weak-scalar rule).
 * `thread_seeds_out` (nthreads entries, may be NULL) receives the chain seeds.  */
int oracle_measure_frequencies(int64_t *frequencies, const void *probs, int realtype,
                               int64_t nstates, int64_t nshots, uint32_t seed,
                               int nthreads, uint32_t *thread_seeds_out) {
  if (nthreads < 1 || nstates < 1 || nstates > ((int64_t)1 << 32)) return 1;
  int64_t *tshots = (int64_t *)malloc(sizeof(int64_t) * nthreads);
  uint32_t *tseed = (uint32_t *)malloc(sizeof(uint32_t) * nthreads);
  for (int t = 0; t < nthreads; t++) tshots[t] = nshots / nthreads;
  tshots[nthreads - 1] += nshots % nthreads;
  mt_state s0;
  mt_seed(&s0, seed);
  for (int t = 0; t < nthreads; t++) tseed[t] = mt_randint(&s0, 100000000u);
  if (thread_seeds_out)
    for (int t = 0; t < nthreads; t++) thread_seeds_out[t] = tseed[t];

  const double *pd = (const double *)probs;
  const float *pf = (const float *)probs;
  /* argmax, first index of the maximum */
  int64_t start = 0;
  for (int64_t i = 1; i < nstates; i++) {
    if (realtype == 0 ? (pd[i] > pd[start]) : (pf[i] > pf[start])) start = i;
  }
  int64_t *priv = (int64_t *)calloc((size_t)nthreads * (size_t)nstates, sizeof(int64_t));
  if (!priv) { free(tshots); free(tseed); return 2; }

#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < nthreads; t++) {
    mt_state s;
    mt_seed(&s, tseed[t]);
    int64_t *fp = priv + (size_t)t * (size_t)nstates;
    int64_t shot = start;
    for (int64_t i = 0; i < tshots[t]; i++) {
      const int64_t new_shot = (shot + (int64_t)mt_randint(&s, (uint64_t)nstates)) % nstates;
      const double r = mt_random(&s);
      int accept;
      if (realtype == 0) accept = (pd[new_shot] / pd[shot]) > r;
      else accept = (pf[new_shot] / pf[shot]) > (float)r;
      if (accept) shot = new_shot;
      fp[shot] += 1;
    }
  }
  for (int t = 0; t < nthreads; t++)
    for (int64_t i = 0; i < nstates; i++) frequencies[i] += priv[(size_t)t * (size_t)nstates + i];
  free(priv);
  free(tshots);
  free(tseed);
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
