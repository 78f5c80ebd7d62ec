// sv_gates.cu -- per-gate state-vector kernels (the "plain method") and their C ABI.
//
// One kernel launch is one read-modify-write pass over the amplitudes a gate touches.
// Thread t of block b handles ITEMS index groups b*256*ITEMS + t + j*256: all loads of
// a thread are issued before any arithmetic, so every thread keeps ITEMS independent
// 16/8-byte requests in flight, and consecutive threads touch consecutive amplitudes
// for every target position (two coalesced streams 2^m apart for a target at bit m).
//
// Index maps follow the reference kernels (qibojit src/qibojit/custom_operators/
// gates.py): an uncontrolled gate inserts a 0 at the target bit(s); a controlled gate
// inserts a 1 at every sorted control/target bit (multicontrol_index, gates.py:5-12)
// and steps back from that all-ones index.  Arithmetic uses fused multiply-adds, so
// results match the reference to rounding (<= a few ulp per gate), not bit for bit.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "sv_common.cuh"
#include "sv_dense_tc.cuh"
#include "sv_dw.cuh"

namespace sv {

constexpr int kBlock = 256;

template <typename T, int N>
struct Mat {
  T g[N];
};

// ------------------------------------------------------------------ one target
template <typename T, int KIND, bool CTRL, int ITEMS>
__global__ void __launch_bounds__(kBlock) k_one_qubit(T* __restrict__ s, int64_t nstates, int m,
                                                      Mat<T, 4> g, const __grid_constant__ BitList q) {
  const int64_t tk = (int64_t)1 << m;
  const int64_t base = (int64_t)blockIdx.x * (kBlock * ITEMS) + threadIdx.x;
  int64_t i1[ITEMS];
  T a[ITEMS], b[ITEMS];
  constexpr bool kReadsLow = (KIND == SV_APPLY_GATE || KIND == SV_APPLY_X || KIND == SV_APPLY_Y);
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    const int64_t gi = base + (int64_t)j * kBlock;
    i1[j] = -1;
    if (gi < nstates) {
      if (CTRL) i1[j] = insert_ones(gi, q) - tk;
      else i1[j] = insert_zero(gi, m);
      if (kReadsLow) a[j] = ldg_stream(s + i1[j]);
      b[j] = ldg_stream(s + i1[j] + tk);
    }
  }
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    if (i1[j] < 0) continue;
    T* p = s + i1[j];
    if constexpr (KIND == SV_APPLY_GATE) {
      T x, y;
      if constexpr (is_complex<T>::value) {
        x = cmad2(g.g[0], a[j], g.g[1], b[j]);
        y = cmad2(g.g[2], a[j], g.g[3], b[j]);
      } else {
        x = fma(g.g[0], a[j], g.g[1] * b[j]);
        y = fma(g.g[2], a[j], g.g[3] * b[j]);
      }
      stg_stream(p, x);
      stg_stream(p + tk, y);
    } else if constexpr (KIND == SV_APPLY_X) {
      stg_stream(p, b[j]);
      stg_stream(p + tk, a[j]);
    } else if constexpr (KIND == SV_APPLY_Y) {
      if constexpr (is_complex<T>::value) {
        // (a, b) <- (-i b, i a)
        T x, y;
        x.re = b[j].im; x.im = -b[j].re;
        y.re = -a[j].im; y.im = a[j].re;
        stg_stream(p, x);
        stg_stream(p + tk, y);
      }
    } else if constexpr (KIND == SV_APPLY_Z) {
      stg_stream(p + tk, tneg(b[j]));
    } else {  // SV_APPLY_Z_POW
      stg_stream(p + tk, tmul(g.g[0], b[j]));
    }
  }
}

// ------------------------------------------------------------------ two targets
template <typename T, int KIND, bool CTRL, int ITEMS>
__global__ void __launch_bounds__(kBlock) k_two_qubit(T* __restrict__ s, int64_t nstates, int m1,
                                                      int m2, int swap_targets, Mat<T, 16> g,
                                                      const __grid_constant__ BitList q) {
  const int64_t tk1 = (int64_t)1 << m1, tk2 = (int64_t)1 << m2;
  const int64_t uk1 = swap_targets ? tk2 : tk1;
  const int64_t uk2 = swap_targets ? tk1 : tk2;
  const int64_t base = (int64_t)blockIdx.x * (kBlock * ITEMS) + threadIdx.x;
  int64_t i0[ITEMS];
  T v[ITEMS][4];
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    const int64_t gi = base + (int64_t)j * kBlock;
    i0[j] = -1;
    if (gi < nstates) {
      if (CTRL) i0[j] = insert_ones(gi, q) - tk1 - tk2;
      else i0[j] = insert_zero(insert_zero(gi, m1), m2);
      if constexpr (KIND == SV_APPLY_TWO_QUBIT_GATE) {
        v[j][0] = ldg_stream(s + i0[j]);
        v[j][3] = ldg_stream(s + i0[j] + tk1 + tk2);
      }
      if constexpr (KIND == SV_APPLY_FSIM) v[j][3] = ldg_stream(s + i0[j] + tk1 + tk2);
      v[j][1] = ldg_stream(s + i0[j] + uk1);
      v[j][2] = ldg_stream(s + i0[j] + uk2);
    }
  }
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    if (i0[j] < 0) continue;
    T* p = s + i0[j];
    if constexpr (KIND == SV_APPLY_TWO_QUBIT_GATE) {
      T o[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        T acc = tmul(g.g[4 * r + 3], v[j][3]);
        acc = tfma(g.g[4 * r + 2], v[j][2], acc);
        acc = tfma(g.g[4 * r + 1], v[j][1], acc);
        o[r] = tfma(g.g[4 * r + 0], v[j][0], acc);
      }
      stg_stream(p, o[0]);
      stg_stream(p + uk1, o[1]);
      stg_stream(p + uk2, o[2]);
      stg_stream(p + tk1 + tk2, o[3]);
    } else if constexpr (KIND == SV_APPLY_SWAP) {
      stg_stream(p + uk1, v[j][2]);
      stg_stream(p + uk2, v[j][1]);
    } else {  // fSim: 2x2 on (|01>, |10>) and a phase on |11>
      const T x = tfma(g.g[0], v[j][1], tmul(g.g[1], v[j][2]));
      const T y = tfma(g.g[2], v[j][1], tmul(g.g[3], v[j][2]));
      stg_stream(p + uk1, x);
      stg_stream(p + uk2, y);
      stg_stream(p + tk1 + tk2, tmul(g.g[4], v[j][3]));
    }
  }
}

// ------------------------------------------------------------ k targets, registers
// One thread per group of 2^K amplitudes; the 4^K matrix rides in the kernel
// parameters (4 KB for K = 4, complex128).  Local row index bit u <-> stride ts[u].
struct Strides {
  int64_t ts[kMaxTargets];
  int64_t zero_off;  // sum of the target strides: all-ones index -> group origin
};

template <typename T, int K>
__global__ void __launch_bounds__(kBlock) k_multi_reg(T* __restrict__ s, int64_t ngroups,
                                                      Mat<T, (1 << (2 * K))> g, const __grid_constant__ BitList q,
                                                      const __grid_constant__ Strides st) {
  constexpr int N = 1 << K;
  const int64_t gi = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (gi >= ngroups) return;
  const int64_t i0 = insert_ones(gi, q) - st.zero_off;
  int64_t off[N];
  T in[N];
#pragma unroll
  for (int i = 0; i < N; i++) {
    int64_t o = 0;
#pragma unroll
    for (int u = 0; u < K; u++)
      if ((i >> u) & 1) o += st.ts[u];
    off[i] = o;
    in[i] = ldg_stream(s + i0 + o);
  }
#pragma unroll
  for (int r = 0; r < N; r++) {
    T acc = tmul(g.g[r * N], in[0]);
#pragma unroll
    for (int c = 1; c < N; c++) acc = tfma(g.g[r * N + c], in[c], acc);
    stg_stream(s + i0 + off[r], acc);
  }
}

// ------------------------------------------ k targets on the lowest k bits, coalesced
// Without controls and with the targets on bits 0..k-1 (any order), group gi is the
// 2^k consecutive amplitudes from gi * 2^k: a thread reading its own group would touch
// one 2^k-element run per lane, 2^k * sizeof(T) bytes apart.  Here a warp takes 32
// consecutive groups, loads and stores them coalesced (lane + 32 j) and regroups them
// in its own shared-memory slice (one padding slot every 16 elements, every 8 for
// 16-byte elements, so neither access pattern conflicts on banks).
template <typename T, int K>
__global__ void __launch_bounds__(kBlock) k_multi_low(T* __restrict__ s, int64_t nchunks,
                                                      Mat<T, (1 << (2 * K))> g, const __grid_constant__ Strides st) {
  constexpr int N = 1 << K;
  constexpr int CH = 32 * N;                       // amplitudes per warp
  constexpr int PS = sizeof(T) >= 16 ? 3 : 4;      // padding: one slot per 2^PS elements
  constexpr int PADDED = CH + (CH >> PS);
  __shared__ T buf[kBlock / 32][PADDED];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t chunk = (int64_t)blockIdx.x * (kBlock / 32) + warp;
  if (chunk >= nchunks) return;  // whole warps only: the kernel synchronises warps, not blocks
  T* const base = s + chunk * CH;
  T* const b = buf[warp];
#pragma unroll
  for (int j = 0; j < N; j++) {
    const int e = lane + 32 * j;
    b[e + (e >> PS)] = ldg_stream(base + e);
  }
  __syncwarp();
  int off[N];
  T in[N];
#pragma unroll
  for (int i = 0; i < N; i++) {
    int o = 0;
#pragma unroll
    for (int u = 0; u < K; u++)
      if ((i >> u) & 1) o += (int)st.ts[u];
    const int e = lane * N + o;
    off[i] = e + (e >> PS);
    in[i] = b[off[i]];
  }
  // every lane rewrites only the slots it read
#pragma unroll
  for (int r = 0; r < N; r++) {
    T acc = tmul(g.g[r * N], in[0]);
#pragma unroll
    for (int c = 1; c < N; c++) acc = tfma(g.g[r * N + c], in[c], acc);
    b[off[r]] = acc;
  }
  __syncwarp();
#pragma unroll
  for (int j = 0; j < N; j++) {
    const int e = lane + 32 * j;
    stg_stream(base + e, b[e + (e >> PS)]);
  }
}

// ------------------------------------------ k targets, complex128 in double-word arithmetic
// As k_multi_reg, each output a double-word dot product of a matrix row (split into
// float pairs on the host) with the group's 2^K amplitudes (cdw_dot, sv_dw.cuh).
template <int K>
__global__ void __launch_bounds__(kBlock) k_multi_dw(c128* __restrict__ s, int64_t ngroups,
                                                     Mat<cdw, (1 << (2 * K))> g, const __grid_constant__ BitList q,
                                                     const __grid_constant__ Strides st) {
  constexpr int N = 1 << K;
  const int64_t gi = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (gi >= ngroups) return;
  const int64_t i0 = insert_ones(gi, q) - st.zero_off;
  auto offset = [&](int i) {
    int64_t o = 0;
#pragma unroll
    for (int u = 0; u < K; u++)
      if ((i >> u) & 1) o += st.ts[u];
    return o;
  };
  double2 raw[N];
#pragma unroll
  for (int i = 0; i < N; i++) raw[i] = __ldcs(reinterpret_cast<const double2*>(s + i0 + offset(i)));
  cdw in[N];
#pragma unroll
  for (int i = 0; i < N; i++) in[i] = cdw_load(raw[i]);
  // one row per iteration, not unrolled: N unrolled double-word rows overflow the
  // instruction cache (the matrix row is read from the parameters at a run-time offset)
#pragma unroll 1
  for (int r = 0; r < N; r++)
    __stcs(reinterpret_cast<double2*>(s + i0 + offset(r)), cdw_store(cdw_dot<N>(&g.g[r * N], in)));
}

// ------------------------------------------------- k targets, shared-memory groups
// A block stages NG groups (NG * 2^k amplitudes, <= 32 KB) in shared memory, laid
// out [row][group] so that consecutive threads read consecutive groups, then every
// thread forms some outputs as dot products with a matrix row read from global
// memory (L1-resident, warp-uniform).  Outputs go straight back to HBM.
constexpr int kSmemBytes = 32 * 1024;

template <typename T>
__global__ void __launch_bounds__(kBlock) k_multi_smem(T* __restrict__ s, int64_t ngroups, int k,
                                                       const T* __restrict__ gmat, const __grid_constant__ BitList q,
                                                       const __grid_constant__ Strides st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* buf = reinterpret_cast<T*>(smem_raw);
  const int N = 1 << k;
  const int NG = (int)(kSmemBytes / sizeof(T)) / N;  // groups per block (>= 1)
  const int64_t g0 = (int64_t)blockIdx.x * NG;
  const int total = NG * N;
  for (int e = threadIdx.x; e < total; e += kBlock) {
    const int i = e / NG, gg = e - i * NG;
    const int64_t gi = g0 + gg;
    if (gi < ngroups) {
      int64_t o = 0;
      for (int u = 0; u < k; u++)
        if ((i >> u) & 1) o += st.ts[u];
      buf[e] = ldg_stream(s + insert_ones(gi, q) - st.zero_off + o);
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < total; e += kBlock) {
    const int r = e / NG, gg = e - r * NG;
    const int64_t gi = g0 + gg;
    if (gi >= ngroups) continue;
    const T* row = gmat + (size_t)r * N;
    T acc = tzero<T>();
    for (int c = 0; c < N; c++) acc = tfma(ldg_ro(row + c), buf[c * NG + gg], acc);
    int64_t o = 0;
    for (int u = 0; u < k; u++)
      if ((r >> u) & 1) o += st.ts[u];
    stg_stream(s + insert_ones(gi, q) - st.zero_off + o, acc);
  }
}

// k_multi_smem for complex128 in double-word arithmetic: groups staged as float pairs,
// each output a double-word dot product with a matrix row split on the host
__device__ __forceinline__ cdw ldg_cdw(const cdw* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return cdw(dw{v.x, v.y}, dw{v.z, v.w});
}

__global__ void __launch_bounds__(kBlock) k_multi_smem_dw(c128* __restrict__ s, int64_t ngroups, int k,
                                                          const cdw* __restrict__ gmat,
                                                          const __grid_constant__ BitList q,
                                                          const __grid_constant__ Strides st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cdw* buf = reinterpret_cast<cdw*>(smem_raw);
  const int N = 1 << k;
  const int NG = (int)(kSmemBytes / sizeof(cdw)) / N;  // groups per block (>= 1)
  const int64_t g0 = (int64_t)blockIdx.x * NG;
  const int total = NG * N;
  for (int e = threadIdx.x; e < total; e += kBlock) {
    const int i = e / NG, gg = e - i * NG;
    const int64_t gi = g0 + gg;
    if (gi < ngroups) {
      int64_t o = 0;
      for (int u = 0; u < k; u++)
        if ((i >> u) & 1) o += st.ts[u];
      buf[e] = cdw_load(__ldcs(reinterpret_cast<const double2*>(s + insert_ones(gi, q) - st.zero_off + o)));
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < total; e += kBlock) {
    const int r = e / NG, gg = e - r * NG;
    const int64_t gi = g0 + gg;
    if (gi >= ngroups) continue;
    const cdw* row = gmat + (size_t)r * N;
    dwacc re{0.0f, 0.0f}, im{0.0f, 0.0f};
    for (int c = 0; c < N; c++) {
      const cdw m = ldg_cdw(row + c), v = buf[c * NG + gg];
      dw_fma(re, m.re, v.re);
      dw_fma(re, dw_neg(m.im), v.im);
      dw_fma(im, m.re, v.im);
      dw_fma(im, m.im, v.re);
    }
    int64_t o = 0;
    for (int u = 0; u < k; u++)
      if ((r >> u) & 1) o += st.ts[u];
    __stcs(reinterpret_cast<double2*>(s + insert_ones(gi, q) - st.zero_off + o),
           cdw_store(cdw(dwacc_result(re), dwacc_result(im))));
  }
}

// ------------------------------------------------- complex128 in double-word arithmetic
// The same index maps and load/store pattern as k_one_qubit / k_two_qubit; every
// amplitude is converted to a (hi, lo) float pair on load and back on store, and each
// output is a double-word dot product (sv_dw.cuh), so the arithmetic runs on the FP32
// pipe instead of GB300's FP64 pipe.  Operands arrive already split on the host.
template <int KIND, bool CTRL, int ITEMS>
__global__ void __launch_bounds__(kBlock) k_one_qubit_dw(c128* __restrict__ s, int64_t nstates, int m,
                                                         Mat<cdw, 4> g, const __grid_constant__ BitList q) {
  const int64_t tk = (int64_t)1 << m;
  const int64_t base = (int64_t)blockIdx.x * (kBlock * ITEMS) + threadIdx.x;
  int64_t i1[ITEMS];
  double2 a[ITEMS], b[ITEMS];
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    const int64_t gi = base + (int64_t)j * kBlock;
    i1[j] = -1;
    if (gi < nstates) {
      i1[j] = CTRL ? insert_ones(gi, q) - tk : insert_zero(gi, m);
      if (KIND == SV_APPLY_GATE) a[j] = __ldcs(reinterpret_cast<const double2*>(s + i1[j]));
      b[j] = __ldcs(reinterpret_cast<const double2*>(s + i1[j] + tk));
    }
  }
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    if (i1[j] < 0) continue;
    double2* p = reinterpret_cast<double2*>(s + i1[j]);
    if constexpr (KIND == SV_APPLY_GATE) {
      const cdw v[2] = {cdw_load(a[j]), cdw_load(b[j])};
      __stcs(p, cdw_store(cdw_dot<2>(&g.g[0], v)));
      __stcs(p + tk, cdw_store(cdw_dot<2>(&g.g[2], v)));
    } else {  // SV_APPLY_Z_POW: the phase on the target-1 amplitude
      const cdw v = cdw_load(b[j]);
      __stcs(p + tk, cdw_store(cdw_dot<1>(&g.g[0], &v)));
    }
  }
}

template <int KIND, bool CTRL, int ITEMS>
__global__ void __launch_bounds__(kBlock) k_two_qubit_dw(c128* __restrict__ s, int64_t nstates, int m1, int m2,
                                                         int swap_targets, Mat<cdw, 16> g,
                                                         const __grid_constant__ BitList q) {
  const int64_t tk1 = (int64_t)1 << m1, tk2 = (int64_t)1 << m2;
  const int64_t uk1 = swap_targets ? tk2 : tk1;
  const int64_t uk2 = swap_targets ? tk1 : tk2;
  const int64_t base = (int64_t)blockIdx.x * (kBlock * ITEMS) + threadIdx.x;
  int64_t i0[ITEMS];
  double2 v[ITEMS][4];
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    const int64_t gi = base + (int64_t)j * kBlock;
    i0[j] = -1;
    if (gi < nstates) {
      i0[j] = CTRL ? insert_ones(gi, q) - tk1 - tk2 : insert_zero(insert_zero(gi, m1), m2);
      const double2* p = reinterpret_cast<const double2*>(s + i0[j]);
      if (KIND == SV_APPLY_TWO_QUBIT_GATE) v[j][0] = __ldcs(p);
      v[j][1] = __ldcs(p + uk1);
      v[j][2] = __ldcs(p + uk2);
      v[j][3] = __ldcs(p + tk1 + tk2);
    }
  }
#pragma unroll
  for (int j = 0; j < ITEMS; j++) {
    if (i0[j] < 0) continue;
    double2* p = reinterpret_cast<double2*>(s + i0[j]);
    if constexpr (KIND == SV_APPLY_TWO_QUBIT_GATE) {
      const cdw x[4] = {cdw_load(v[j][0]), cdw_load(v[j][1]), cdw_load(v[j][2]), cdw_load(v[j][3])};
      __stcs(p, cdw_store(cdw_dot<4>(&g.g[0], x)));
      __stcs(p + uk1, cdw_store(cdw_dot<4>(&g.g[4], x)));
      __stcs(p + uk2, cdw_store(cdw_dot<4>(&g.g[8], x)));
      __stcs(p + tk1 + tk2, cdw_store(cdw_dot<4>(&g.g[12], x)));
    } else {  // fSim: 2x2 on (|01>, |10>) and a phase on |11>
      const cdw x[2] = {cdw_load(v[j][1]), cdw_load(v[j][2])};
      const cdw w = cdw_load(v[j][3]);
      __stcs(p + uk1, cdw_store(cdw_dot<2>(&g.g[0], x)));
      __stcs(p + uk2, cdw_store(cdw_dot<2>(&g.g[2], x)));
      __stcs(p + tk1 + tk2, cdw_store(cdw_dot<1>(&g.g[4], &w)));
    }
  }
}

template <int N>
static void split_operand(Mat<cdw, N>& out, const c128* in, int count) {
  memset(&out, 0, sizeof(out));
  for (int i = 0; i < count; i++) {
    sv_dw_split_host(in[i].re, &out.g[i].re.h, &out.g[i].re.l);
    sv_dw_split_host(in[i].im, &out.g[i].im.h, &out.g[i].im.l);
  }
}

// =============================================================== host side
static int check_state_args(const void* state, int dtype, int nqubits) {
  if (!state) return set_error(SV_ERR_ARG, "state pointer is NULL");
  if (dtype < SV_C128 || dtype > SV_F32) return set_error(SV_ERR_ARG, "unknown dtype %d", dtype);
  if (nqubits < 1 || nqubits > kMaxQubits)
    return set_error(SV_ERR_ARG, "nqubits = %d out of range [1, %d]", nqubits, kMaxQubits);
  if (((uintptr_t)state) % dtype_size(dtype))
    return set_error(SV_ERR_ARG, "state pointer is not aligned to its element size");
  return SV_OK;
}

// Builds the sorted bit list of a gate.  `qubits` (if given) must be sorted, unique,
// in range, and contain every target bit; otherwise the target bits alone are used.
static int make_bitlist(BitList* out, int nqubits, const int* target_bits, int ntargets,
                        const int32_t* qubits, int nq) {
  std::vector<int> bits;
  if (qubits && nq > 0) {
    bits.assign(qubits, qubits + nq);
  } else {
    bits.assign(target_bits, target_bits + ntargets);
    std::sort(bits.begin(), bits.end());
  }
  if ((int)bits.size() > nqubits || (int)bits.size() > kMaxQubits)
    return set_error(SV_ERR_ARG, "gate acts on %d qubits of a %d-qubit state", (int)bits.size(), nqubits);
  for (size_t j = 0; j < bits.size(); j++) {
    if (bits[j] < 0 || bits[j] >= nqubits)
      return set_error(SV_ERR_ARG, "qubit bit position %d out of range for %d qubits", bits[j], nqubits);
    if (j > 0 && bits[j] <= bits[j - 1])
      return set_error(SV_ERR_ARG, "qubits tensor must be sorted and free of duplicates");
  }
  for (int t = 0; t < ntargets; t++)
    if (!std::binary_search(bits.begin(), bits.end(), target_bits[t]))
      return set_error(SV_ERR_ARG, "target bit %d missing from the qubits tensor", target_bits[t]);
  out->n = (int)bits.size();
  for (size_t j = 0; j < bits.size(); j++) out->pos[j] = bits[j];
  return SV_OK;
}

template <typename T, int KIND, bool CTRL>
static int launch_one(Context* ctx, void* state, int64_t nstates, int m, const Mat<T, 4>& g,
                      const BitList& q) {
  constexpr int ITEMS = 4;
  const unsigned grid = grid_for(nstates, kBlock * ITEMS);
  k_one_qubit<T, KIND, CTRL, ITEMS><<<grid, kBlock, 0, ctx->stream>>>((T*)state, nstates, m, g, q);
  SV_LAUNCH_CHECK("one-qubit kernel launch");
  return SV_OK;
}

template <typename T>
static int one_qubit_typed(Context* ctx, void* state, int nqubits, int kind, const void* gate,
                           int target, const BitList& q, bool ctrl) {
  Mat<T, 4> g;
  memset(&g, 0, sizeof(g));
  if (kind == SV_APPLY_GATE) {
    if (!gate) return set_error(SV_ERR_ARG, "apply_gate needs a 2x2 operand");
    memcpy(g.g, gate, 4 * sizeof(T));
  } else if (kind == SV_APPLY_Z_POW) {
    if (!gate) return set_error(SV_ERR_ARG, "apply_z_pow needs its phase operand");
    memcpy(g.g, gate, sizeof(T));
  }
  const int m = nqubits - target - 1;
  const int ncontrols = q.n - 1;
  const int64_t nstates = (int64_t)1 << (nqubits - ncontrols - 1);
  if constexpr (std::is_same<T, c128>::value) {
    if (!ctx->c128_fp64 && (kind == SV_APPLY_GATE || kind == SV_APPLY_Z_POW)) {
      Mat<cdw, 4> gd;
      split_operand(gd, g.g, kind == SV_APPLY_GATE ? 4 : 1);
      constexpr int ITEMS = 4;
      const unsigned grid = grid_for(nstates, kBlock * ITEMS);
      c128* st = (c128*)state;
      if (kind == SV_APPLY_GATE) {
        if (ctrl) k_one_qubit_dw<SV_APPLY_GATE, true, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m, gd, q);
        else k_one_qubit_dw<SV_APPLY_GATE, false, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m, gd, q);
      } else {
        if (ctrl) k_one_qubit_dw<SV_APPLY_Z_POW, true, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m, gd, q);
        else k_one_qubit_dw<SV_APPLY_Z_POW, false, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m, gd, q);
      }
      SV_LAUNCH_CHECK("one-qubit double-word kernel launch");
      return SV_OK;
    }
  }
#define SV_ONE_CASE(KIND)                                                   \
  case KIND:                                                                \
    return ctrl ? launch_one<T, KIND, true>(ctx, state, nstates, m, g, q)   \
                : launch_one<T, KIND, false>(ctx, state, nstates, m, g, q);
  switch (kind) {
    SV_ONE_CASE(SV_APPLY_GATE)
    SV_ONE_CASE(SV_APPLY_X)
    SV_ONE_CASE(SV_APPLY_Z)
    SV_ONE_CASE(SV_APPLY_Z_POW)
    case SV_APPLY_Y:
      if constexpr (is_complex<T>::value) {
        return ctrl ? launch_one<T, SV_APPLY_Y, true>(ctx, state, nstates, m, g, q)
                    : launch_one<T, SV_APPLY_Y, false>(ctx, state, nstates, m, g, q);
      } else {
        return set_error(SV_ERR_UNSUPPORTED, "apply_y needs a complex state");
      }
    default:
      return set_error(SV_ERR_ARG, "unknown one-qubit kernel %d", kind);
  }
#undef SV_ONE_CASE
}

template <typename T, int KIND, bool CTRL>
static int launch_two(Context* ctx, void* state, int64_t nstates, int m1, int m2, int swap,
                      const Mat<T, 16>& g, const BitList& q) {
  constexpr int ITEMS = 2;
  const unsigned grid = grid_for(nstates, kBlock * ITEMS);
  k_two_qubit<T, KIND, CTRL, ITEMS><<<grid, kBlock, 0, ctx->stream>>>((T*)state, nstates, m1, m2,
                                                                      swap, g, q);
  SV_LAUNCH_CHECK("two-qubit kernel launch");
  return SV_OK;
}

template <typename T>
static int two_qubit_typed(Context* ctx, void* state, int nqubits, int kind, const void* gate,
                           int target1, int target2, const BitList& q, bool ctrl) {
  Mat<T, 16> g;
  memset(&g, 0, sizeof(g));
  if (kind == SV_APPLY_TWO_QUBIT_GATE) {
    if (!gate) return set_error(SV_ERR_ARG, "apply_two_qubit_gate needs a 4x4 operand");
    memcpy(g.g, gate, 16 * sizeof(T));
  } else if (kind == SV_APPLY_FSIM) {
    if (!gate) return set_error(SV_ERR_ARG, "apply_fsim needs its 5-entry operand");
    memcpy(g.g, gate, 5 * sizeof(T));
  }
  // cpu.py:618-635: m1 < m2 always; swap the row order when target1 > target2
  int m1, m2, swap;
  if (target1 > target2) {
    swap = 1;
    m1 = nqubits - target1 - 1;
    m2 = nqubits - target2 - 1;
  } else {
    swap = 0;
    m1 = nqubits - target2 - 1;
    m2 = nqubits - target1 - 1;
  }
  const int ncontrols = q.n - 2;
  const int64_t nstates = (int64_t)1 << (nqubits - 2 - ncontrols);
  if constexpr (std::is_same<T, c128>::value) {
    if (!ctx->c128_fp64 && (kind == SV_APPLY_TWO_QUBIT_GATE || kind == SV_APPLY_FSIM)) {
      Mat<cdw, 16> gd;
      split_operand(gd, g.g, kind == SV_APPLY_FSIM ? 5 : 16);
      constexpr int ITEMS = 2;
      const unsigned grid = grid_for(nstates, kBlock * ITEMS);
      c128* st = (c128*)state;
      if (kind == SV_APPLY_TWO_QUBIT_GATE) {
        if (ctrl)
          k_two_qubit_dw<SV_APPLY_TWO_QUBIT_GATE, true, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m1, m2,
                                                                                              swap, gd, q);
        else
          k_two_qubit_dw<SV_APPLY_TWO_QUBIT_GATE, false, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m1,
                                                                                               m2, swap, gd, q);
      } else {
        if (ctrl)
          k_two_qubit_dw<SV_APPLY_FSIM, true, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m1, m2, swap, gd, q);
        else
          k_two_qubit_dw<SV_APPLY_FSIM, false, ITEMS><<<grid, kBlock, 0, ctx->stream>>>(st, nstates, m1, m2, swap, gd,
                                                                                     q);
      }
      SV_LAUNCH_CHECK("two-qubit double-word kernel launch");
      return SV_OK;
    }
  }
#define SV_TWO_CASE(KIND)                                                             \
  case KIND:                                                                          \
    return ctrl ? launch_two<T, KIND, true>(ctx, state, nstates, m1, m2, swap, g, q)  \
                : launch_two<T, KIND, false>(ctx, state, nstates, m1, m2, swap, g, q);
  switch (kind) {
    SV_TWO_CASE(SV_APPLY_TWO_QUBIT_GATE)
    SV_TWO_CASE(SV_APPLY_SWAP)
    SV_TWO_CASE(SV_APPLY_FSIM)
    default:
      return set_error(SV_ERR_ARG, "unknown two-qubit kernel %d", kind);
  }
#undef SV_TWO_CASE
}

template <typename T, int K>
static int launch_multi_reg(Context* ctx, void* state, int64_t ngroups, const void* gate,
                            const BitList& q, const Strides& st) {
  Mat<T, (1 << (2 * K))> g;
  memcpy(g.g, gate, sizeof(g.g));
  k_multi_reg<T, K><<<grid_for(ngroups, kBlock), kBlock, 0, ctx->stream>>>((T*)state, ngroups, g, q, st);
  SV_LAUNCH_CHECK("multi-qubit kernel launch");
  return SV_OK;
}

template <typename T, int K>
static int launch_multi_low(Context* ctx, void* state, int64_t ngroups, const void* gate, const Strides& st) {
  Mat<T, (1 << (2 * K))> g;
  memcpy(g.g, gate, sizeof(g.g));
  const int64_t nchunks = ngroups / 32;  // 32 groups per warp
  k_multi_low<T, K><<<grid_for(nchunks, kBlock / 32), kBlock, 0, ctx->stream>>>((T*)state, nchunks, g, st);
  SV_LAUNCH_CHECK("multi-qubit (low targets) kernel launch");
  return SV_OK;
}

template <int K>
static int launch_multi_dw(Context* ctx, void* state, int64_t ngroups, const void* gate, const BitList& q,
                           const Strides& st) {
  Mat<cdw, (1 << (2 * K))> g;
  split_operand(g, (const c128*)gate, 1 << (2 * K));
  k_multi_dw<K><<<grid_for(ngroups, kBlock), kBlock, 0, ctx->stream>>>((c128*)state, ngroups, g, q, st);
  SV_LAUNCH_CHECK("multi-qubit double-word kernel launch");
  return SV_OK;
}

template <typename T>
static int multi_qubit_typed(Context* ctx, void* state, int nqubits, const void* gate,
                             const int32_t* targets, int k, const BitList& q) {
  Strides st;
  memset(&st, 0, sizeof(st));
  for (int u = 0; u < k; u++) {
    st.ts[u] = (int64_t)1 << (nqubits - targets[k - 1 - u] - 1);
    st.zero_off += st.ts[u];
  }
  const int64_t ngroups = (int64_t)1 << (nqubits - q.n);
  if constexpr (std::is_same<T, c128>::value) {
    // complex128 in double-word arithmetic unless the context asks for FP64
    if (!ctx->c128_fp64 && k == 3) return launch_multi_dw<3>(ctx, state, ngroups, gate, q, st);
    if (!ctx->c128_fp64 && k == 4) return launch_multi_dw<4>(ctx, state, ngroups, gate, q, st);
    if (!ctx->c128_fp64 && k >= 5) {
      const int n2 = 1 << (2 * k);
      std::vector<cdw> split(n2);
      const c128* m = (const c128*)gate;
      for (int i = 0; i < n2; i++) {
        sv_dw_split_host(m[i].re, &split[i].re.h, &split[i].re.l);
        sv_dw_split_host(m[i].im, &split[i].im.h, &split[i].im.l);
      }
      const size_t mbytes = sizeof(cdw) * (size_t)n2;
      SV_TRY(ensure_operand(ctx, mbytes));
      // from pageable memory the copy is staged before the call returns, so the
      // temporary may go out of scope
      SV_TRY(check_cuda(cudaMemcpyAsync(ctx->operand, split.data(), mbytes, cudaMemcpyHostToDevice, ctx->stream),
                        "gate operand upload"));
      const int NG = (int)(kSmemBytes / sizeof(cdw)) >> k;
      if (NG < 1) return set_error(SV_ERR_ARG, "%d targets exceed the shared-memory group size", k);
      const int64_t nblocks = (ngroups + NG - 1) / NG;
      k_multi_smem_dw<<<(unsigned)nblocks, kBlock, kSmemBytes, ctx->stream>>>((c128*)state, ngroups, k,
                                                                              (const cdw*)ctx->operand, q, st);
      SV_LAUNCH_CHECK("multi-qubit double-word (shared) kernel launch");
      return SV_OK;
    }
  }
  // no controls, targets on bits 0..k-1 in any order, at least one warp of groups
  int64_t low_mask = 0;
  for (int u = 0; u < k; u++) low_mask |= st.ts[u];
  if (q.n == k && low_mask == ((int64_t)1 << k) - 1 && ngroups >= 32) {
    if (k == 3) return launch_multi_low<T, 3>(ctx, state, ngroups, gate, st);
    if (k == 4 && sizeof(T) <= 8) return launch_multi_low<T, 4>(ctx, state, ngroups, gate, st);
  }
  switch (k) {
    case 1: return launch_multi_reg<T, 1>(ctx, state, ngroups, gate, q, st);
    case 2: return launch_multi_reg<T, 2>(ctx, state, ngroups, gate, q, st);
    case 3: return launch_multi_reg<T, 3>(ctx, state, ngroups, gate, q, st);
    case 4:
      if (sizeof(T) <= 8) return launch_multi_reg<T, 4>(ctx, state, ngroups, gate, q, st);
      break;
    default: break;
  }
  const size_t mbytes = sizeof(T) << (2 * k);
  SV_TRY(ensure_operand(ctx, mbytes));
  SV_TRY(check_cuda(cudaMemcpyAsync(ctx->operand, gate, mbytes, cudaMemcpyHostToDevice, ctx->stream),
                    "gate operand upload"));
  const int NG = (int)(kSmemBytes / sizeof(T)) >> k;
  if (NG < 1) return set_error(SV_ERR_ARG, "%d targets exceed the shared-memory group size", k);
  const int64_t nblocks = (ngroups + NG - 1) / NG;
  k_multi_smem<T><<<(unsigned)nblocks, kBlock, kSmemBytes, ctx->stream>>>(
      (T*)state, ngroups, k, (const T*)ctx->operand, q, st);
  SV_LAUNCH_CHECK("multi-qubit (shared) kernel launch");
  return SV_OK;
}

}  // namespace sv

using namespace sv;

extern "C" {

int sv_apply_one_qubit(sv_context* ctx, void* state, int dtype, int nqubits, int kind,
                       const void* gate, int target, const int32_t* qubits, int nq) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  SV_TRY(check_state_args(state, dtype, nqubits));
  if (target < 0 || target >= nqubits)
    return set_error(SV_ERR_ARG, "target %d out of range for %d qubits", target, nqubits);
  const int tbit = nqubits - target - 1;
  BitList q;
  SV_TRY(make_bitlist(&q, nqubits, &tbit, 1, qubits, nq));
  const bool ctrl = q.n > 1;
  Context* c = ctx;
  switch (dtype) {
    case SV_C128: return one_qubit_typed<c128>(c, state, nqubits, kind, gate, target, q, ctrl);
    case SV_C64: return one_qubit_typed<c64>(c, state, nqubits, kind, gate, target, q, ctrl);
    case SV_F64: return one_qubit_typed<double>(c, state, nqubits, kind, gate, target, q, ctrl);
    default: return one_qubit_typed<float>(c, state, nqubits, kind, gate, target, q, ctrl);
  }
}

int sv_apply_two_qubit(sv_context* ctx, void* state, int dtype, int nqubits, int kind,
                       const void* gate, int target1, int target2, const int32_t* qubits, int nq) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  SV_TRY(check_state_args(state, dtype, nqubits));
  if (target1 < 0 || target1 >= nqubits || target2 < 0 || target2 >= nqubits || target1 == target2)
    return set_error(SV_ERR_ARG, "targets (%d, %d) invalid for %d qubits", target1, target2, nqubits);
  if (kind == SV_APPLY_FSIM && (dtype == SV_F64 || dtype == SV_F32))
    return set_error(SV_ERR_UNSUPPORTED, "apply_fsim needs a complex state");
  const int tb[2] = {nqubits - target1 - 1, nqubits - target2 - 1};
  BitList q;
  SV_TRY(make_bitlist(&q, nqubits, tb, 2, qubits, nq));
  const bool ctrl = q.n > 2;
  Context* c = ctx;
  switch (dtype) {
    case SV_C128: return two_qubit_typed<c128>(c, state, nqubits, kind, gate, target1, target2, q, ctrl);
    case SV_C64: return two_qubit_typed<c64>(c, state, nqubits, kind, gate, target1, target2, q, ctrl);
    case SV_F64: return two_qubit_typed<double>(c, state, nqubits, kind, gate, target1, target2, q, ctrl);
    default: return two_qubit_typed<float>(c, state, nqubits, kind, gate, target1, target2, q, ctrl);
  }
}

int sv_apply_multi_qubit(sv_context* ctx, void* state, int dtype, int nqubits, const void* gate,
                         const int32_t* targets, int ntargets, const int32_t* qubits, int nq) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  SV_TRY(check_state_args(state, dtype, nqubits));
  if (!gate || !targets) return set_error(SV_ERR_ARG, "gate and targets are required");
  if (ntargets < 1 || ntargets > kMaxTargets || ntargets > nqubits)
    return set_error(SV_ERR_ARG, "Number of target qubits must be <= %d but is %d.", kMaxTargets, ntargets);
  int tb[kMaxTargets];
  for (int t = 0; t < ntargets; t++) {
    if (targets[t] < 0 || targets[t] >= nqubits)
      return set_error(SV_ERR_ARG, "target %d out of range for %d qubits", targets[t], nqubits);
    for (int u = 0; u < t; u++)
      if (targets[u] == targets[t]) return set_error(SV_ERR_ARG, "duplicate target %d", targets[t]);
    tb[t] = nqubits - targets[t] - 1;
  }
  BitList q;
  SV_TRY(make_bitlist(&q, nqubits, tb, ntargets, qubits, nq));
  Context* c = ctx;
  const bool tc_ok = dense_tc_eligible(dtype, ntargets);
  if (c->dense_mode == SV_DENSE_TENSOR && !tc_ok)
    return set_error(SV_ERR_UNSUPPORTED, "the tensor-core kernel takes complex64 gates with 4..6 targets");
  // auto: 5 and 6 targets on the tensor cores; 4 targets stay on the register kernel,
  // which measured faster at n = 30 (0.83 against 0.51 of the HBM peak)
  if (tc_ok && c->dense_mode != SV_DENSE_SIMT &&
      (c->dense_mode == SV_DENSE_TENSOR || (ntargets >= 5 && nqubits - q.n >= 10)))
    return dense_tc_apply(c, state, nqubits, gate, targets, ntargets, q);
  switch (dtype) {
    case SV_C128: return multi_qubit_typed<c128>(c, state, nqubits, gate, targets, ntargets, q);
    case SV_C64: return multi_qubit_typed<c64>(c, state, nqubits, gate, targets, ntargets, q);
    case SV_F64: return multi_qubit_typed<double>(c, state, nqubits, gate, targets, ntargets, q);
    default: return multi_qubit_typed<float>(c, state, nqubits, gate, targets, ntargets, q);
  }
}

}  // extern "C"
