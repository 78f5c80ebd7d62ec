// sv_ops.cu -- state creation, collapse, probabilities and Metropolis sampling.
//
// Everything stays on the device and on the context's stream: the collapse norm is
// reduced, square-rooted and inverted by kernels (no host round trip), and the
// sampler runs NumPy's legacy MT19937 streams on the GPU, one warp per chain.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "sv_common.cuh"

namespace sv {

constexpr int kOpsBlock = 256;

// ----------------------------------------------------------------- zero state
// |0...0>, ops.py:10-18: 16-byte stores of zeros, the first chunk holding 1.0.
__global__ void k_fill_zero_state(uint4* __restrict__ p, int64_t nchunks, uint4 first) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks; c += stride)
    __stcs(p + c, c == 0 ? first : make_uint4(0, 0, 0, 0));
}
__global__ void k_set_first(unsigned char* p, int bytes, uint4 first) {
  const unsigned char* f = reinterpret_cast<const unsigned char*>(&first);
  for (int b = threadIdx.x; b < bytes; b += blockDim.x) p[b] = b < 16 ? f[b] : 0;
}

// ------------------------------------------------------------ block reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Neumaier-compensated accumulation of one term.
struct KSum {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

// Block-wide sum of `v` in a fixed order; the result is valid in thread 0.
__device__ double block_sum(double v) {
  __shared__ double part[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) part[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// ------------------------------------------------------------------ collapse
// Measured bits: `mask` has a 1 at every measured bit position, `value` holds the
// outcome bits at those positions.  An amplitude is kept iff (i & mask) == value.
// kept_index(g) enumerates the kept amplitudes in increasing order by inserting the
// outcome bits at the sorted measured positions (ops.py:33-40, collapse_index).
struct Measured {
  int n;
  int pos[kMaxQubits];   // sorted ascending bit positions
  int bit[kMaxQubits];   // outcome bit at pos[j]
  int64_t mask, value;
};

__device__ __forceinline__ int64_t kept_index(int64_t g, const Measured& m) {
  int64_t i = g;
  for (int j = 0; j < m.n; j++) {
    const int p = m.pos[j];
    const int64_t k = (int64_t)1 << p;
    i = ((i >> p) << (p + 1)) + (i & (k - 1)) + (m.bit[j] ? k : 0);
  }
  return i;
}

// Pass 1 (normalize only): per-block compensated partial sums of |kept|^2.
// CONTIG: the measured qubits are the top bits of the index, so the kept amplitudes
// are one contiguous slice and kept_index(g) = g | value.
template <typename T, bool CONTIG = false>
__global__ void __launch_bounds__(kOpsBlock) k_collapse_norm_partials(
    const T* __restrict__ s, int64_t nkept, const __grid_constant__ Measured m,
    double* __restrict__ partials) {
  KSum acc;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // 8 independent loads per thread and iteration; a complex64 state's 8 squares are
  // summed in FP32 (to 2^-21 relative) and added to the compensated FP64 sum as one
  // term (FP64 per amplitude would bound the pass on this GPU)
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < nkept; g += 8 * stride) {
    T v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int64_t gk = g + k * stride;
      v[k] = gk < nkept ? ldg_stream(s + (CONTIG ? (gk | m.value) : kept_index(gk, m))) : tzero<T>();
    }
    if constexpr (std::is_same<T, c64>::value) {
      float part = 0.0f;
#pragma unroll
      for (int k = 0; k < 8; k++) part = fmaf(v[k].re, v[k].re, fmaf(v[k].im, v[k].im, part));
      acc.add((double)part);
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) acc.add(tnorm2(v[k]));
    }
  }
  const double r = block_sum(acc.value());
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

// Sums the partials in a fixed order (compensated) and stores 1/sqrt(sum).
__global__ void k_finish_inverse_norm(const double* __restrict__ partials, int np,
                                      double* __restrict__ out) {
  KSum acc;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc.add(partials[i]);
  __shared__ double sh_s[kOpsBlock], sh_c[kOpsBlock];
  sh_s[threadIdx.x] = acc.s;
  sh_c[threadIdx.x] = acc.c;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    for (int i = 0; i < (int)blockDim.x; i++) {
      t.add(sh_s[i]);
      t.add(sh_c[i]);
    }
    const double norm2 = t.value();
    out[0] = norm2;
    out[1] = 1.0 / sqrt(norm2);  // NumPy divides a complex by a real as a product with 1/x
  }
}

// Pass 2: zero the amplitudes of other outcomes (write-only) and, when normalizing,
// scale the kept ones by the inverse norm computed on the device.
template <typename T, bool NORMALIZE>
__global__ void __launch_bounds__(kOpsBlock) k_collapse_apply(T* __restrict__ s, int64_t n,
                                                             int64_t mask, int64_t value,
                                                             const double* __restrict__ inv) {
  using R = typename real_of<T>::type;
  const R scale = NORMALIZE ? (R)inv[1] : (R)1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // four independent elements per thread and iteration keep more stores in flight
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int64_t i = i0 + k * stride;
      if (i >= n) break;
      if ((i & mask) != value) {
        stg_stream(s + i, tzero<T>());
      } else if (NORMALIZE) {
        T a = ldg_stream(s + i);
        if constexpr (is_complex<T>::value) {
          a.re *= scale;
          a.im *= scale;
        } else {
          a *= scale;
        }
        stg_stream(s + i, a);
      }
    }
  }
}

// ------------------------------------------------------------- probabilities
struct ProbMap {
  int n, nq;
  int mpos[kMaxQubits];     // bit position feeding output bit (nq-1-j), j = 0..nq-1
  int sorted[kMaxQubits];   // measured bit positions, ascending (for inserting zeros)
};

// amplitude index of (output bin o, unmeasured index u)
__device__ __forceinline__ int64_t prob_index(int64_t o, int64_t u, const ProbMap& p) {
  int64_t i = u;
  for (int j = 0; j < p.nq; j++) {
    const int b = p.sorted[j];
    const int64_t k = (int64_t)1 << b;
    i = ((i >> b) << (b + 1)) + (i & (k - 1));
  }
  for (int j = 0; j < p.nq; j++)
    if ((o >> (p.nq - 1 - j)) & 1) i |= (int64_t)1 << p.mpos[j];
  return i;
}

// Probability carried by basis index i: |s_i|^2 for a state vector; for a density
// matrix (DM) the real part of its diagonal element rho_ii, at i * (2^n + 1) in the
// row-major 2^n x 2^n array (dstride = 2^n + 1).
template <typename T, bool DM>
__device__ __forceinline__ double prob_at(const T* __restrict__ s, int64_t i, int64_t dstride) {
  if constexpr (DM) {
    const T a = ldg_ro(s + i * dstride);
    if constexpr (is_complex<T>::value) return (double)a.re;
    else return (double)a;
  } else {
    return tnorm2(ldg_stream(s + i));
  }
}

// |s_i|^2 of a complex64 state in FP32 (one rounding more than the FP64 square
// rounded to float; FP64 per amplitude would bound the pass on this GPU)
__device__ __forceinline__ float norm2_f32(const c64* __restrict__ s, int64_t i) {
  const c64 a = ldg_stream(s + i);
  return fmaf(a.re, a.re, a.im * a.im);
}
// float32 output from a complex64 state: the square in FP32; otherwise FP64
template <typename T, typename O, bool DM>
__device__ __forceinline__ O prob_out(const T* __restrict__ s, int64_t i, int64_t dstride) {
  if constexpr (std::is_same<T, c64>::value && std::is_same<O, float>::value && !DM) return norm2_f32(s, i);
  else return (O)prob_at<T, DM>(s, i, dstride);
}

template <typename T, typename O, bool DM>
__global__ void __launch_bounds__(kOpsBlock) k_probs_full(const T* __restrict__ s, int64_t n, int64_t dstride,
                                                          O* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    __stcs(out + i, prob_out<T, O, DM>(s, i, dstride));
}

// all qubits measured in a permuted order: out[perm(i)] = p_i
template <typename T, typename O, bool DM>
__global__ void __launch_bounds__(kOpsBlock) k_probs_perm(const T* __restrict__ s, int64_t n, int64_t dstride,
                                                          const __grid_constant__ ProbMap p,
                                                          O* __restrict__ out) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int64_t o = 0;
    for (int j = 0; j < p.nq; j++) o |= ((i >> p.mpos[j]) & 1) << (p.nq - 1 - j);
    out[o] = prob_out<T, O, DM>(s, i, dstride);
  }
}

// few amplitudes per bin: one thread per bin, sequential sum
template <typename T, typename O, bool DM>
__global__ void __launch_bounds__(kOpsBlock) k_probs_thread_bins(const T* __restrict__ s, int64_t dstride,
                                                                 int64_t nbins, int64_t per_bin,
                                                                 const __grid_constant__ ProbMap p,
                                                                 O* __restrict__ out) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nbins) return;
  double acc = 0.0;
  for (int64_t u = 0; u < per_bin; u++) acc += prob_at<T, DM>(s, prob_index(o, u, p), dstride);
  out[o] = (O)acc;
}

// many amplitudes per bin: block (segment, bin) sums a contiguous range of u
// CONTIG: every measured bit lies above the unmeasured ones, so bin o is the
// contiguous range prob_index(o, 0) + u.
template <typename T, bool DM, bool CONTIG = false>
__global__ void __launch_bounds__(kOpsBlock) k_probs_segments(const T* __restrict__ s, int64_t dstride,
                                                              int64_t per_bin, int nseg,
                                                              const __grid_constant__ ProbMap p,
                                                              double* __restrict__ partials) {
  const int64_t o = blockIdx.y;
  const int seg = blockIdx.x;
  const int64_t len = per_bin / nseg;
  const int64_t u0 = (int64_t)seg * len;
  double acc = 0.0;
  const int64_t end = u0 + len;
  const int64_t bd = blockDim.x;
  const int64_t obase = CONTIG ? prob_index(o, 0, p) : 0;
  if constexpr (!DM) {
    // 8 independent loads per thread and iteration keep enough bytes in flight; a
    // complex64 state's 8 squares are summed in FP32 and added to the FP64 sum as one
    // term (FP64 per amplitude would bound the pass on this GPU)
    for (int64_t u = u0 + threadIdx.x; u < end; u += 8 * bd) {
      T v[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int64_t uk = u + k * bd;
        v[k] = uk < end ? ldg_stream(s + (CONTIG ? obase + uk : prob_index(o, uk, p))) : tzero<T>();
      }
      if constexpr (std::is_same<T, c64>::value) {
        float part = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; k++) part = fmaf(v[k].re, v[k].re, fmaf(v[k].im, v[k].im, part));
        acc += (double)part;
      } else {
#pragma unroll
        for (int k = 0; k < 8; k++) acc += tnorm2(v[k]);
      }
    }
  } else {
    for (int64_t u = u0 + threadIdx.x; u < end; u += bd) acc += prob_at<T, DM>(s, prob_index(o, u, p), dstride);
  }
  const double r = block_sum(acc);
  if (threadIdx.x == 0) partials[o * nseg + seg] = r;
}

template <typename O>
__global__ void k_probs_finish(const double* __restrict__ partials, int64_t nbins, int nseg,
                               O* __restrict__ out) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nbins) return;
  double acc = 0.0;
  for (int k = 0; k < nseg; k++) acc += partials[o * nseg + k];
  out[o] = (O)acc;
}

// ------------------------------------------------------------ Metropolis sampler
// NumPy legacy MT19937 (Matsumoto & Nishimura 1998): init_genrand seeding, the
// twist over 624 words, and tempering on output.
constexpr int kMT = 624;

__host__ __device__ inline uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
__host__ __device__ inline uint32_t mt_twist(uint32_t cur, uint32_t next, uint32_t src) {
  const uint32_t y = (cur & 0x80000000u) | (next & 0x7fffffffu);
  return src ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

struct HostMT {
  uint32_t mt[kMT];
  int pos;
  explicit HostMT(uint32_t seed) {
    mt[0] = seed;
    for (int i = 1; i < kMT; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    pos = kMT;
  }
  uint32_t next() {
    if (pos >= kMT) {
      for (int k = 0; k < kMT; k++) mt[k] = mt_twist(mt[k], mt[(k + 1) % kMT], mt[(k + 397) % kMT]);
      pos = 0;
    }
    return mt_temper(mt[pos++]);
  }
  // NumPy legacy randint(0, high): masked rejection on one 32-bit word
  uint32_t randint(uint64_t high) {
    const uint64_t rng = high - 1;
    if (rng == 0) return 0;
    uint64_t mask = rng;
    mask |= mask >> 1; mask |= mask >> 2; mask |= mask >> 4; mask |= mask >> 8; mask |= mask >> 16;
    uint64_t v;
    do { v = next() & mask; } while (v > rng);
    return (uint32_t)v;
  }
};

// One warp regenerates the 624-word block in place, 32 words at a time, in the
// sequential algorithm's order (words below 227 read the old word k+397, later words
// the new word k-227; each chunk reads before it writes).
__device__ void mt_regenerate_warp(uint32_t* mt, int lane) {
  for (int base = 0; base < kMT; base += 32) {
    const int k = base + lane;
    uint32_t nv = 0;
    if (k < kMT) {
      const uint32_t cur = mt[k];
      const uint32_t nxt = mt[(k + 1) % kMT];
      const uint32_t src = k < 227 ? mt[k + 397] : mt[k - 227];
      nv = mt_twist(cur, nxt, src);
    }
    __syncwarp();
    // (the last word pairs with word 0, already renewed by the first chunk)
    if (k < kMT) mt[k] = nv;
    __syncwarp();
  }
}

struct Chain {
  uint32_t seed;
  int64_t nshots;
};

constexpr int kChainWarps = 4;  // chains per block

// Every lane of the warp follows the chain (warp-uniform control flow); lane 0 keeps
// the histogram.  Each step draws randint(0, N) (one word, N = 2^nbits so the mask
// never rejects) and random() (two words), exactly as ops.py:100-106 consumes them.
template <typename P>
__global__ void __launch_bounds__(32 * kChainWarps) k_metropolis(
    const P* __restrict__ probs, uint32_t mask, const Chain* __restrict__ chains, int nchains,
    const int64_t* __restrict__ start, unsigned long long* __restrict__ freq) {
  __shared__ uint32_t mt_all[kChainWarps][kMT];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = blockIdx.x * kChainWarps + w;
  if (c >= nchains) return;
  uint32_t* mt = mt_all[w];
  if (lane == 0) {
    mt[0] = chains[c].seed;
    for (int i = 1; i < kMT; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  }
  __syncwarp();
  int pos = kMT;
  const int64_t nshots = chains[c].nshots;
  uint64_t shot = (uint64_t)start[0];
  P pshot = probs[shot];
  auto next_word = [&]() -> uint32_t {
    if (pos >= kMT) {
      mt_regenerate_warp(mt, lane);
      pos = 0;
    }
    return mt_temper(mt[pos++]);
  };
  for (int64_t i = 0; i < nshots; i++) {
    const uint32_t w0 = next_word();
    const uint32_t w1 = next_word();
    const uint32_t w2 = next_word();
    const uint64_t nshot = (shot + (uint64_t)(w0 & mask)) & (uint64_t)mask;
    const double r = ((double)(w1 >> 5) * 67108864.0 + (double)(w2 >> 6)) / 9007199254740992.0;
    const P pnew = probs[nshot];
    bool accept;
    if constexpr (sizeof(P) == 8) accept = (pnew / pshot) > r;
    else accept = (pnew / pshot) > __double2float_rn(r);
    if (accept) {
      shot = nshot;
      pshot = pnew;
    }
    if (lane == 0) atomicAdd(freq + shot, 1ull);
  }
}

// Chain seeds: np.random.seed(seed); [randint(0, 1e8) for each chain], ops.py:92-93.
// Shots: nshots // nchains each, the remainder on the last chain (ops.py:88-90).
static void make_chains(uint32_t seed, int64_t nshots, int nchains, std::vector<Chain>* out) {
  HostMT m(seed);
  out->resize(nchains);
  for (int c = 0; c < nchains; c++) {
    (*out)[c].seed = m.randint(100000000u);
    (*out)[c].nshots = nshots / nchains;
  }
  (*out)[nchains - 1].nshots += nshots % nchains;
}

// first index of the maximum: per-block (value, index) then one final block
template <typename P>
__global__ void k_argmax_partials(const P* __restrict__ p, int64_t n, P* __restrict__ bv,
                                  int64_t* __restrict__ bi) {
  P best = p[0];
  int64_t idx = 0;
  bool have = false;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const P v = p[i];
    if (!have || v > best) {  // strided in increasing order: keeps the first maximum
      best = v;
      idx = i;
      have = true;
    }
  }
  __shared__ P sv[kOpsBlock];
  __shared__ int64_t si[kOpsBlock];
  sv[threadIdx.x] = best;
  si[threadIdx.x] = have ? idx : INT64_MAX;
  __syncthreads();
  if (threadIdx.x == 0) {
    P b = sv[0];
    int64_t bidx = si[0];
    for (int t = 1; t < (int)blockDim.x; t++) {
      if (si[t] == INT64_MAX) continue;
      if (bidx == INT64_MAX || sv[t] > b || (sv[t] == b && si[t] < bidx)) {
        b = sv[t];
        bidx = si[t];
      }
    }
    bv[blockIdx.x] = b;
    bi[blockIdx.x] = bidx;
  }
}

template <typename P>
__global__ void k_argmax_finish(const P* __restrict__ bv, const int64_t* __restrict__ bi, int nb,
                                int64_t* __restrict__ out) {
  if (threadIdx.x != 0) return;
  P b = bv[0];
  int64_t idx = bi[0];
  for (int k = 1; k < nb; k++) {
    if (bi[k] == INT64_MAX) continue;
    if (idx == INT64_MAX || bv[k] > b || (bv[k] == b && bi[k] < idx)) {
      b = bv[k];
      idx = bi[k];
    }
  }
  out[0] = idx == INT64_MAX ? 0 : idx;
}

// =================================================================== host side
static int check_state(const void* state, int dtype, int nqubits) {
  if (!state) return set_error(SV_ERR_ARG, "state pointer is NULL");
  if (dtype < SV_C128 || dtype > SV_F32) return set_error(SV_ERR_ARG, "unknown dtype %d", dtype);
  if (nqubits < 1 || nqubits > kMaxQubits)
    return set_error(SV_ERR_ARG, "nqubits = %d out of range [1, %d]", nqubits, kMaxQubits);
  if (((uintptr_t)state) % dtype_size(dtype))
    return set_error(SV_ERR_ARG, "state pointer is not aligned to its element size");
  return SV_OK;
}

static unsigned stream_grid(const Context* ctx, int64_t work) {
  const int64_t cap = (int64_t)ctx->num_sms * 8;
  int64_t g = (work + kOpsBlock - 1) / kOpsBlock;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (unsigned)g;
}

static int zero_state_impl(Context* ctx, void* state, int dtype, int nqubits) {
  SV_TRY(check_state(state, dtype, nqubits));
  const size_t bytes = dtype_size(dtype) << nqubits;
  uint4 first = make_uint4(0, 0, 0, 0);
  if (dtype == SV_C128 || dtype == SV_F64) {
    const double one = 1.0;
    memcpy(&first, &one, sizeof(one));
  } else {
    const float one = 1.0f;
    memcpy(&first, &one, sizeof(one));
  }
  if (bytes >= 16 && ((uintptr_t)state % 16) == 0 && bytes % 16 == 0) {
    const int64_t nchunks = (int64_t)(bytes / 16);
    k_fill_zero_state<<<stream_grid(ctx, nchunks), kOpsBlock, 0, ctx->stream>>>((uint4*)state, nchunks, first);
  } else {
    k_set_first<<<1, 32, 0, ctx->stream>>>((unsigned char*)state, (int)bytes, first);
  }
  SV_LAUNCH_CHECK("zero_state launch");
  return SV_OK;
}

// Measured qubits and outcome of a collapse call (both collapse entry points): the
// reference maps qubit q to bit n-q-1 (cpu.py:548-552); bit j of `result`, counting
// from the most significant, is the outcome of qubits[j].  Positions are stored in
// ascending order with their outcome bits.
static int decode_measured(int nqubits, const int32_t* qubits, int nq, int64_t result, Measured* out) {
  if (!qubits || nq < 1 || nq > nqubits) return set_error(SV_ERR_ARG, "collapse needs 1..n measured qubits");
  if (result < 0 || result >= ((int64_t)1 << nq))
    return set_error(SV_ERR_ARG, "outcome %lld out of range for %d qubits", (long long)result, nq);
  Measured m;
  memset(&m, 0, sizeof(m));
  m.n = nq;
  for (int j = 0; j < nq; j++) {
    if (qubits[j] < 0 || qubits[j] >= nqubits)
      return set_error(SV_ERR_ARG, "measured qubit %d out of range", qubits[j]);
    const int pos = nqubits - qubits[j] - 1;
    if (m.mask & ((int64_t)1 << pos)) return set_error(SV_ERR_ARG, "duplicate measured qubit %d", qubits[j]);
    m.mask |= (int64_t)1 << pos;
    if ((result >> (nq - 1 - j)) & 1) m.value |= (int64_t)1 << pos;
  }
  int k = 0;
  for (int p = 0; p < nqubits; p++) {
    if (!(m.mask & ((int64_t)1 << p))) continue;
    m.pos[k] = p;
    m.bit[k] = (int)((m.value >> p) & 1);
    k++;
  }
  *out = m;
  return SV_OK;
}

template <typename T>
static int collapse_typed(Context* ctx, void* state, int nqubits, const Measured& m, int normalize) {
  const int64_t n = (int64_t)1 << nqubits;
  double* inv = nullptr;
  if (normalize) {
    const int64_t nkept = (int64_t)1 << (nqubits - m.n);
    const unsigned grid = stream_grid(ctx, nkept);
    SV_TRY(ensure_scratch(ctx, (grid + 2) * sizeof(double)));
    double* partials = (double*)ctx->scratch;
    inv = partials + grid;
    if (m.pos[0] >= nqubits - m.n)  // the measured qubits are the top bits
      k_collapse_norm_partials<T, true><<<grid, kOpsBlock, 0, ctx->stream>>>((const T*)state, nkept, m, partials);
    else
      k_collapse_norm_partials<T><<<grid, kOpsBlock, 0, ctx->stream>>>((const T*)state, nkept, m, partials);
    SV_LAUNCH_CHECK("collapse norm launch");
    k_finish_inverse_norm<<<1, kOpsBlock, 0, ctx->stream>>>(partials, (int)grid, inv);
    SV_LAUNCH_CHECK("collapse norm finish launch");
    k_collapse_apply<T, true><<<stream_grid(ctx, n), kOpsBlock, 0, ctx->stream>>>((T*)state, n, m.mask, m.value, inv);
  } else {
    k_collapse_apply<T, false><<<stream_grid(ctx, n), kOpsBlock, 0, ctx->stream>>>((T*)state, n, m.mask, m.value, nullptr);
  }
  SV_LAUNCH_CHECK("collapse launch");
  return SV_OK;
}

template <typename T, typename O, bool DM = false>
static int probs_typed(Context* ctx, const void* state, int nqubits, const ProbMap& p, void* out) {
  const int64_t n = (int64_t)1 << nqubits;
  const int64_t dstride = n + 1;
  const T* s = (const T*)state;
  if (p.nq == nqubits) {
    bool identity = true;
    for (int j = 0; j < p.nq; j++) identity &= (p.mpos[j] == nqubits - 1 - j);
    if (identity) k_probs_full<T, O, DM><<<stream_grid(ctx, n), kOpsBlock, 0, ctx->stream>>>(s, n, dstride, (O*)out);
    else k_probs_perm<T, O, DM><<<stream_grid(ctx, n), kOpsBlock, 0, ctx->stream>>>(s, n, dstride, p, (O*)out);
    SV_LAUNCH_CHECK("probabilities launch");
    return SV_OK;
  }
  const int64_t nbins = (int64_t)1 << p.nq;
  const int64_t per_bin = (int64_t)1 << (nqubits - p.nq);
  if (per_bin <= 64 || nbins > 65535 || nbins >= (int64_t)ctx->num_sms * 4 * kOpsBlock) {
    k_probs_thread_bins<T, O, DM><<<grid_for(nbins, kOpsBlock), kOpsBlock, 0, ctx->stream>>>(s, dstride, nbins, per_bin,
                                                                                              p, (O*)out);
    SV_LAUNCH_CHECK("probabilities launch");
    return SV_OK;
  }
  // segments per bin: enough blocks to fill the GPU, each summing >= 4096 amplitudes
  int64_t nseg = ((int64_t)ctx->num_sms * 8 + nbins - 1) / nbins;
  while (nseg > 1 && per_bin / nseg < 4096) nseg >>= 1;
  int64_t pow2 = 1;
  while (pow2 * 2 <= nseg) pow2 *= 2;
  nseg = pow2;  // per_bin is a power of two: segments divide it exactly
  SV_TRY(ensure_scratch(ctx, (size_t)(nbins * nseg) * sizeof(double)));
  double* partials = (double*)ctx->scratch;
  dim3 grid((unsigned)nseg, (unsigned)nbins);
  if (!DM && p.sorted[0] >= nqubits - p.nq)  // the measured qubits are the top bits
    k_probs_segments<T, DM, true><<<grid, kOpsBlock, 0, ctx->stream>>>(s, dstride, per_bin, (int)nseg, p, partials);
  else
    k_probs_segments<T, DM><<<grid, kOpsBlock, 0, ctx->stream>>>(s, dstride, per_bin, (int)nseg, p, partials);
  SV_LAUNCH_CHECK("probabilities launch");
  k_probs_finish<O><<<grid_for(nbins, kOpsBlock), kOpsBlock, 0, ctx->stream>>>(partials, nbins, (int)nseg, (O*)out);
  SV_LAUNCH_CHECK("probabilities finish launch");
  return SV_OK;
}

template <typename P>
static int sample_typed(Context* ctx, int64_t* freq, const void* probs, int nbits, int64_t nshots,
                        uint32_t seed, int nchains) {
  const int64_t n = (int64_t)1 << nbits;
  std::vector<Chain> chains;
  make_chains(seed, nshots, nchains, &chains);
  const unsigned gblocks = stream_grid(ctx, n);
  // scratch layout: [chains][argmax block values][argmax block indices][start]
  const size_t chain_bytes = ((sizeof(Chain) * nchains + 255) / 256) * 256;
  const size_t val_bytes = ((sizeof(P) * gblocks + 255) / 256) * 256;
  const size_t idx_bytes = ((sizeof(int64_t) * gblocks + 255) / 256) * 256;
  SV_TRY(ensure_scratch(ctx, chain_bytes + val_bytes + idx_bytes + 256));
  unsigned char* base = (unsigned char*)ctx->scratch;
  Chain* d_chains = (Chain*)base;
  P* d_bv = (P*)(base + chain_bytes);
  int64_t* d_bi = (int64_t*)(base + chain_bytes + val_bytes);
  int64_t* d_start = (int64_t*)(base + chain_bytes + val_bytes + idx_bytes);
  // the chain table is small; a synchronous copy keeps the host vector's lifetime simple
  SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "sampler (sync)"));
  SV_TRY(check_cuda(cudaMemcpy(d_chains, chains.data(), sizeof(Chain) * nchains, cudaMemcpyHostToDevice),
                    "sampler chain upload"));
  k_argmax_partials<P><<<gblocks, kOpsBlock, 0, ctx->stream>>>((const P*)probs, n, d_bv, d_bi);
  SV_LAUNCH_CHECK("argmax launch");
  k_argmax_finish<P><<<1, 32, 0, ctx->stream>>>(d_bv, d_bi, (int)gblocks, d_start);
  SV_LAUNCH_CHECK("argmax finish launch");
  const uint32_t mask = (uint32_t)(n - 1);
  k_metropolis<P><<<grid_for(nchains, kChainWarps), 32 * kChainWarps, 0, ctx->stream>>>(
      (const P*)probs, mask, d_chains, nchains, d_start, (unsigned long long*)freq);
  SV_LAUNCH_CHECK("metropolis launch");
  return SV_OK;
}

// ------------------------------------------------- direct sampling (inverse CDF)
// Below qibo's SHOT_METROPOLIS_THRESHOLD the reference samples with qibo's
// Backend.sample_shots, numpy.random.choice(N, nshots, p=probs) (the branch at
// cpu.py:384-385): cdf = cumsum(p) / cdf[-1] in FP64 and, for each uniform u of the
// global MT19937 stream (random_sample), the first index i with cdf[i] > u.  The
// engine takes the same uniforms from the caller and searches an FP64 CDF built on
// the device in two levels (sums of 4096-probability blocks, their prefix, then the
// crossing inside one block), so the probabilities never leave the device.
constexpr int kCdfBlock = 4096;                // probabilities per block
constexpr int kCdfSeg = kCdfBlock / 32;        // per lane when a warp scans one block

template <typename P>
__global__ void __launch_bounds__(256) k_cdf_block_sums(const P* __restrict__ p, int64_t n, double* bsum) {
  __shared__ double red[8];
  const int64_t b0 = (int64_t)blockIdx.x * kCdfBlock;
  double s = 0.0;
  for (int i = threadIdx.x; i < kCdfBlock; i += blockDim.x)
    if (b0 + i < n) s += (double)p[b0 + i];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

// exclusive prefix of the block sums, bpre[nb] = total; one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_cdf_prefix(const double* bsum, int64_t nb, double* bpre) {
  __shared__ double part[1024];
  const int64_t per = (nb + 1023) / 1024;
  const int64_t lo = threadIdx.x * per, hi = lo + per < nb ? lo + per : nb;
  double s = 0.0;
  for (int64_t i = lo; i < hi; i++) s += bsum[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {  // 1024 sequential adds: fixed order
    double c = 0.0;
    for (int t = 0; t < 1024; t++) {
      const double x = part[t];
      part[t] = c;
      c += x;
    }
    bpre[nb] = c;
  }
  __syncthreads();
  double c = part[threadIdx.x];
  for (int64_t i = lo; i < hi; i++) {
    bpre[i] = c;
    c += bsum[i];
  }
}

// largest index with a nonzero probability (the answer when u * total rounds up to total)
template <typename P>
__global__ void __launch_bounds__(256) k_last_nonzero(const P* __restrict__ p, int64_t n,
                                                      unsigned long long* out) {
  long long best = -1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (p[i] > (P)0) best = i;
  for (int off = 16; off > 0; off >>= 1) {
    const long long o = __shfl_xor_sync(0xffffffffu, best, off);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0 && best >= 0) atomicMax(out, (unsigned long long)best);
}

// one warp per shot: block by binary search over the prefix, then the lane segment whose
// running sum crosses u * total, then the element inside it
template <typename P>
__global__ void __launch_bounds__(256) k_cdf_sample(const P* __restrict__ p, int64_t n, const double* __restrict__ bpre,
                                                    int64_t nb, const double* __restrict__ u, int64_t nshots,
                                                    const unsigned long long* last, unsigned long long* freq,
                                                    int64_t* samples) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double total = bpre[nb];
  for (int64_t shot = (((int64_t)blockIdx.x * blockDim.x) >> 5) + (threadIdx.x >> 5); shot < nshots; shot += nwarps) {
    const double t = u[shot] * total;
    int64_t lo = 0, hi = nb - 1;  // last block whose prefix is <= t
    while (lo < hi) {
      const int64_t mid = (lo + hi + 1) >> 1;
      if (bpre[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const int64_t e0 = lo * kCdfBlock + (int64_t)lane * kCdfSeg;
    double seg = 0.0;
    long long seglast = -1;  // last nonzero probability of this lane's segment
    for (int i = 0; i < kCdfSeg; i++)
      if (e0 + i < n) {
        const double x = (double)p[e0 + i];
        seg += x;
        if (x > 0.0) seglast = e0 + i;
      }
    double inc = seg;  // inclusive warp scan of the segment sums
    for (int off = 1; off < 32; off <<= 1) {
      const double o = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += o;
    }
    const unsigned hit = __ballot_sync(0xffffffffu, bpre[lo] + inc > t);
    long long idx = -1;
    if (hit) {
      const int L = __ffs(hit) - 1;
      if (lane == L) {
        double c = bpre[lo] + inc - seg;
        long long lastpos = -1;
        for (int i = 0; i < kCdfSeg && e0 + i < n; i++) {
          const double x = (double)p[e0 + i];
          if (x > 0.0) lastpos = e0 + i;
          c += x;
          if (c > t && x > 0.0) {
            idx = e0 + i;
            break;
          }
        }
        if (idx < 0) idx = lastpos;  // rounding between the two running sums
      }
      idx = __shfl_sync(0xffffffffu, idx, L);
    }
    if (idx < 0) {
      // no crossing inside the block: u * total sits within rounding of the block's end
      // (or of the total); the last nonzero probability of the block, else of the state
      long long bl = seglast;
      for (int off = 16; off > 0; off >>= 1) {
        const long long o = __shfl_xor_sync(0xffffffffu, bl, off);
        bl = o > bl ? o : bl;
      }
      idx = bl >= 0 ? bl : (long long)*last;
    }
    if (lane == 0) {
      if (freq) atomicAdd(&freq[idx], 1ull);
      if (samples) samples[shot] = idx;
    }
  }
}

template <typename P>
static int sample_cdf_typed(Context* ctx, const void* probs, int nbits, const double* uniforms, int64_t nshots,
                            int64_t* freq, int64_t* samples) {
  const int64_t n = (int64_t)1 << nbits;
  const int64_t nb = (n + kCdfBlock - 1) / kCdfBlock;
  const size_t a = ((sizeof(double) * (size_t)nb + 255) / 256) * 256;
  const size_t b = ((sizeof(double) * (size_t)(nb + 1) + 255) / 256) * 256;
  const size_t c = ((sizeof(double) * (size_t)nshots + 255) / 256) * 256;
  SV_TRY(ensure_scratch(ctx, a + b + c + 256));
  unsigned char* base = (unsigned char*)ctx->scratch;
  double* bsum = (double*)base;
  double* bpre = (double*)(base + a);
  double* du = (double*)(base + a + b);
  unsigned long long* last = (unsigned long long*)(base + a + b + c);
  SV_TRY(check_cuda(cudaMemcpyAsync(du, uniforms, sizeof(double) * nshots, cudaMemcpyHostToDevice, ctx->stream),
                    "uniforms upload"));
  SV_TRY(check_cuda(cudaMemsetAsync(last, 0, sizeof(unsigned long long), ctx->stream), "last index"));
  k_cdf_block_sums<P><<<(unsigned)nb, 256, 0, ctx->stream>>>((const P*)probs, n, bsum);
  SV_LAUNCH_CHECK("cdf block sums launch");
  k_cdf_prefix<<<1, 1024, 0, ctx->stream>>>(bsum, nb, bpre);
  SV_LAUNCH_CHECK("cdf prefix launch");
  k_last_nonzero<P><<<stream_grid(ctx, n), 256, 0, ctx->stream>>>((const P*)probs, n, last);
  SV_LAUNCH_CHECK("last nonzero launch");
  const int64_t warps = nshots < (int64_t)ctx->num_sms * 64 ? nshots : (int64_t)ctx->num_sms * 64;
  k_cdf_sample<P><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, ctx->stream>>>(
      (const P*)probs, n, bpre, nb, du, nshots, last, (unsigned long long*)freq, samples);
  SV_LAUNCH_CHECK("cdf sample launch");
  // the uniforms came from pageable host memory: finish before the caller may reuse it
  SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "cdf sampling"));
  return SV_OK;
}

}  // namespace sv

using namespace sv;

template <bool DM>
static int probabilities_impl(sv_context* ctx, const void* state, int dtype, int nqubits, const int32_t* qubits,
                              int nq, void* out, int out_dtype) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  if (DM && (nqubits < 1 || 2 * nqubits > kMaxQubits))
    return set_error(SV_ERR_ARG, "density matrix of %d qubits out of range [1, %d]", nqubits, kMaxQubits / 2);
  SV_TRY(check_state(state, dtype, DM ? 2 * nqubits : nqubits));
  if (!out) return set_error(SV_ERR_ARG, "output pointer is NULL");
  if (out_dtype != SV_F64 && out_dtype != SV_F32) return set_error(SV_ERR_ARG, "out_dtype must be SV_F64 or SV_F32");
  if (!qubits || nq < 1 || nq > nqubits) return set_error(SV_ERR_ARG, "probabilities need 1..n qubits");
  ProbMap p;
  memset(&p, 0, sizeof(p));
  p.n = nqubits;
  p.nq = nq;
  std::vector<int> sorted;
  for (int j = 0; j < nq; j++) {
    if (qubits[j] < 0 || qubits[j] >= nqubits) return set_error(SV_ERR_ARG, "qubit %d out of range", qubits[j]);
    p.mpos[j] = nqubits - qubits[j] - 1;
    sorted.push_back(p.mpos[j]);
  }
  std::sort(sorted.begin(), sorted.end());
  for (int j = 0; j < nq; j++) {
    if (j > 0 && sorted[j] == sorted[j - 1]) return set_error(SV_ERR_ARG, "duplicate qubit in probabilities");
    p.sorted[j] = sorted[j];
  }
  const bool f64 = out_dtype == SV_F64;
  switch (dtype) {
    case SV_C128: return f64 ? probs_typed<c128, double, DM>(ctx, state, nqubits, p, out) : probs_typed<c128, float, DM>(ctx, state, nqubits, p, out);
    case SV_C64: return f64 ? probs_typed<c64, double, DM>(ctx, state, nqubits, p, out) : probs_typed<c64, float, DM>(ctx, state, nqubits, p, out);
    case SV_F64: return f64 ? probs_typed<double, double, DM>(ctx, state, nqubits, p, out) : probs_typed<double, float, DM>(ctx, state, nqubits, p, out);
    default: return f64 ? probs_typed<float, double, DM>(ctx, state, nqubits, p, out) : probs_typed<float, float, DM>(ctx, state, nqubits, p, out);
  }
}

// y <- a x + b y (b == 0: y is only written).  x and y may be the same array.
template <typename T>
__global__ void __launch_bounds__(kOpsBlock) k_axpby(const T* x, T* y, int64_t n, double are, double aim,
                                                     double bre, double bim, bool read_y) {
  using R = typename real_of<T>::type;
  const R ar = (R)are, ai = (R)aim, br = (R)bre, bi = (R)bim;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T u = x[i];
    if constexpr (is_complex<T>::value) {
      T r{ar * u.re - ai * u.im, ar * u.im + ai * u.re};
      if (read_y) {
        const T v = y[i];
        r.re += br * v.re - bi * v.im;
        r.im += br * v.im + bi * v.re;
      }
      y[i] = r;
    } else {
      R r = ar * u;
      if (read_y) r += br * y[i];
      y[i] = r;
    }
  }
}

template <typename T>
static int axpby_typed(Context* ctx, int64_t n, const void* x, double are, double aim, void* y, double bre,
                       double bim) {
  const bool read_y = bre != 0.0 || bim != 0.0;
  k_axpby<T><<<stream_grid(ctx, n), kOpsBlock, 0, ctx->stream>>>((const T*)x, (T*)y, n, are, aim, bre, bim, read_y);
  SV_LAUNCH_CHECK("axpby launch");
  return SV_OK;
}

extern "C" {

int sv_sample_cdf(sv_context* ctx, const void* probs, int prob_dtype, int nbits, const double* uniforms,
                  int64_t nshots, int64_t* frequencies, int64_t* samples) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  if (!probs || (nshots > 0 && !uniforms)) return set_error(SV_ERR_ARG, "probs and uniforms are required");
  if (nbits < 0 || nbits > 34) return set_error(SV_ERR_ARG, "nbits = %d out of range [0, 34]", nbits);
  if (nshots < 0) return set_error(SV_ERR_ARG, "nshots must be >= 0");
  if (nshots == 0) return SV_OK;
  for (int64_t i = 0; i < nshots; i++)
    if (!(uniforms[i] >= 0.0 && uniforms[i] < 1.0)) return set_error(SV_ERR_ARG, "uniforms must lie in [0, 1)");
  if (prob_dtype == SV_F64) return sample_cdf_typed<double>(ctx, probs, nbits, uniforms, nshots, frequencies, samples);
  if (prob_dtype == SV_F32) return sample_cdf_typed<float>(ctx, probs, nbits, uniforms, nshots, frequencies, samples);
  return set_error(SV_ERR_ARG, "prob_dtype must be SV_F64 or SV_F32");
}

int sv_zero_state(sv_context* ctx, void* state, int dtype, int nqubits) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  return zero_state_impl(ctx, state, dtype, nqubits);
}

int sv_collapse_state(sv_context* ctx, void* state, int dtype, int nqubits, const int32_t* qubits,
                      int nq, int64_t result, int normalize) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  SV_TRY(check_state(state, dtype, nqubits));
  Measured m;
  SV_TRY(decode_measured(nqubits, qubits, nq, result, &m));
  switch (dtype) {
    case SV_C128: return collapse_typed<c128>(ctx, state, nqubits, m, normalize);
    case SV_C64: return collapse_typed<c64>(ctx, state, nqubits, m, normalize);
    case SV_F64: return collapse_typed<double>(ctx, state, nqubits, m, normalize);
    default: return collapse_typed<float>(ctx, state, nqubits, m, normalize);
  }
}

int sv_probabilities(sv_context* ctx, const void* state, int dtype, int nqubits, const int32_t* qubits,
                     int nq, void* out, int out_dtype) {
  return probabilities_impl<false>(ctx, state, dtype, nqubits, qubits, nq, out, out_dtype);
}

int sv_density_probabilities(sv_context* ctx, const void* rho, int dtype, int nqubits, const int32_t* qubits,
                             int nq, void* out, int out_dtype) {
  return probabilities_impl<true>(ctx, rho, dtype, nqubits, qubits, nq, out, out_dtype);
}

int sv_axpby(sv_context* ctx, int dtype, int64_t n, const void* x, double a_re, double a_im, void* y, double b_re,
             double b_im) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  if (!x || !y) return set_error(SV_ERR_ARG, "x and y are required");
  if (dtype < SV_C128 || dtype > SV_F32) return set_error(SV_ERR_ARG, "unknown dtype %d", dtype);
  if (n < 0) return set_error(SV_ERR_ARG, "negative length");
  if (((uintptr_t)x) % dtype_size(dtype) || ((uintptr_t)y) % dtype_size(dtype))
    return set_error(SV_ERR_ARG, "arrays are not aligned to their element size");
  const bool real = dtype == SV_F64 || dtype == SV_F32;
  if (real && (a_im != 0.0 || b_im != 0.0)) return set_error(SV_ERR_ARG, "complex coefficients on a real array");
  if (n == 0) return SV_OK;
  switch (dtype) {
    case SV_C128: return axpby_typed<c128>(ctx, n, x, a_re, a_im, y, b_re, b_im);
    case SV_C64: return axpby_typed<c64>(ctx, n, x, a_re, a_im, y, b_re, b_im);
    case SV_F64: return axpby_typed<double>(ctx, n, x, a_re, a_im, y, b_re, b_im);
    default: return axpby_typed<float>(ctx, n, x, a_re, a_im, y, b_re, b_im);
  }
}

int sv_measure_frequencies(sv_context* ctx, int64_t* frequencies, const void* probs, int prob_dtype,
                           int nbits, int64_t nshots, uint32_t seed, int nchains) {
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  if (!frequencies || !probs) return set_error(SV_ERR_ARG, "frequencies and probs are required");
  if (nbits < 0 || nbits > 32) return set_error(SV_ERR_ARG, "nbits = %d out of range [0, 32]", nbits);
  if (nchains < 1 || nchains > (1 << 20)) return set_error(SV_ERR_ARG, "nchains = %d out of range", nchains);
  if (nshots < 0) return set_error(SV_ERR_ARG, "nshots must be >= 0");
  if (prob_dtype == SV_F64) return sample_typed<double>(ctx, frequencies, probs, nbits, nshots, seed, nchains);
  if (prob_dtype == SV_F32) return sample_typed<float>(ctx, frequencies, probs, nbits, nshots, seed, nchains);
  return set_error(SV_ERR_ARG, "prob_dtype must be SV_F64 or SV_F32");
}

}  // extern "C"

// ============================================== collapse without device allocation
// Callers that cannot call cudaMalloc (a host framework that owns every device byte
// through its own pool allocator, or a latency-critical loop where an allocation and
// the device synchronisation of a later cudaFree are not acceptable) use
// sv_collapse_state_noalloc.  Its reduction scratch is the file-scope array below,
// which every GPU that loads this library holds until the process exits.
#include <mutex>

#include "sv_noalloc_grid.h"

namespace sv {

constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_collapse_scratch[kNoAllocScratchDoubles];

struct NoAllocDevice {
  bool ready = false;
  double* scratch = nullptr;  // device address of g_noalloc_collapse_scratch on this device
  int num_sms = 0;
};
static NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];
static std::mutex g_noalloc_mutex;

// Once per device, with that device current: the array's name is only a host-side
// stand-in, so its device address must come from cudaGetSymbolAddress.
static int noalloc_setup(int device, NoAllocDevice** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocDevice& d = g_noalloc_devices[device];
  if (!d.ready) {
    void* ptr = nullptr;
    SV_TRY(check_cuda(cudaGetSymbolAddress(&ptr, g_noalloc_collapse_scratch),
                      "cudaGetSymbolAddress(no-alloc collapse scratch)"));
    int sms = 0;
    SV_TRY(check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
                      "cudaDeviceGetAttribute"));
    d.scratch = static_cast<double*>(ptr);
    d.num_sms = sms;
    d.ready = true;
  }
  *out = &d;
  return SV_OK;
}

template <typename T>
static int collapse_noalloc_typed(cudaStream_t stream, const NoAllocDevice& d, void* state, int nqubits,
                                  const Measured& m, int normalize) {
  const int64_t n = (int64_t)1 << nqubits;
  auto grid_of = [&d](int64_t work) { return noalloc_grid(work, d.num_sms, kOpsBlock); };
  if (!normalize) {
    k_collapse_apply<T, false><<<grid_of(n), kOpsBlock, 0, stream>>>((T*)state, n, m.mask, m.value, nullptr);
    SV_LAUNCH_CHECK("no-alloc collapse launch");
    return SV_OK;
  }
  const int64_t nkept = (int64_t)1 << (nqubits - m.n);
  const unsigned grid = grid_of(nkept);
  // every block writes its own partial and the finish kernel writes both results
  // before the apply pass reads them, so nothing left from an earlier call is read
  if (!noalloc_norm_fits(grid))
    return set_error(SV_ERR_ARG,
                     "no-alloc collapse needs %u doubles of scratch; its static array holds at most %d",
                     grid + 2, kNoAllocScratchDoubles);
  double* partials = d.scratch;
  double* inv = d.scratch + grid;
  k_collapse_norm_partials<T><<<grid, kOpsBlock, 0, stream>>>((const T*)state, nkept, m, partials);
  SV_LAUNCH_CHECK("no-alloc collapse norm launch");
  k_finish_inverse_norm<<<1, kOpsBlock, 0, stream>>>(partials, (int)grid, inv);
  SV_LAUNCH_CHECK("no-alloc collapse norm finish launch");
  k_collapse_apply<T, true><<<grid_of(n), kOpsBlock, 0, stream>>>((T*)state, n, m.mask, m.value, inv);
  SV_LAUNCH_CHECK("no-alloc collapse launch");
  return SV_OK;
}

}  // namespace sv

extern "C" int sv_collapse_state_noalloc(void* stream, void* state, int dtype, int nqubits,
                                         const int32_t* qubits, int nq, int64_t result, int normalize) {
  using namespace sv;
  SV_TRY(check_state(state, dtype, nqubits));
  Measured m;
  SV_TRY(decode_measured(nqubits, qubits, nq, result, &m));
  int device = 0;
  SV_TRY(check_cuda(cudaGetDevice(&device), "cudaGetDevice"));
  if (device < 0 || device >= kNoAllocMaxDevices)
    return set_error(SV_ERR_ARG, "device %d beyond the %d devices the no-alloc path tracks", device,
                     kNoAllocMaxDevices);
  NoAllocDevice* d = nullptr;
  SV_TRY(noalloc_setup(device, &d));
  cudaStream_t s = (cudaStream_t)stream;
  switch (dtype) {
    case SV_C128: return collapse_noalloc_typed<c128>(s, *d, state, nqubits, m, normalize);
    case SV_C64: return collapse_noalloc_typed<c64>(s, *d, state, nqubits, m, normalize);
    case SV_F64: return collapse_noalloc_typed<double>(s, *d, state, nqubits, m, normalize);
    default: return collapse_noalloc_typed<float>(s, *d, state, nqubits, m, normalize);
  }
}

// ===================================================================== reductions
// FP64 reductions over states of either precision (the precision mode keeps bulk
// arithmetic in complex64 and every reduction in FP64): <a|b>, max |a_i - b_i|, and
// <Z_mask> = sum_i (-1)^popcount(i & mask) |a_i|^2.  Per-thread Neumaier sums, fixed
// grid, fixed-order final sums: results are reproducible run to run.
namespace sv {

template <typename T>
__device__ __forceinline__ void as_f64(T a, double& re, double& im) {
  if constexpr (is_complex<T>::value) {
    re = (double)a.re;
    im = (double)a.im;
  } else {
    re = (double)a;
    im = 0.0;
  }
}

template <typename TA, typename TB>
__global__ void __launch_bounds__(kOpsBlock) k_dot_partials(const TA* __restrict__ a, const TB* __restrict__ b,
                                                           int64_t n, double* __restrict__ partials) {
  KSum sre, sim;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double ar, ai, br, bi;
    as_f64(ldg_stream(a + i), ar, ai);
    as_f64(ldg_stream(b + i), br, bi);
    sre.add(ar * br + ai * bi);  // conj(a) * b
    sim.add(ar * bi - ai * br);
  }
  const double r = block_sum(sre.value());
  const double m = block_sum(sim.value());
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = r;
    partials[2 * blockIdx.x + 1] = m;
  }
}

template <typename TA, typename TB>
__global__ void __launch_bounds__(kOpsBlock) k_maxdiff_partials(const TA* __restrict__ a, const TB* __restrict__ b,
                                                               int64_t n, double* __restrict__ partials) {
  double mx = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double ar, ai, br, bi;
    as_f64(ldg_stream(a + i), ar, ai);
    as_f64(ldg_stream(b + i), br, bi);
    mx = fmax(mx, hypot(ar - br, ai - bi));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __shared__ double part[32];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = fmax(r, part[w]);
    partials[blockIdx.x] = r;
  }
}

template <typename T>
__global__ void __launch_bounds__(kOpsBlock) k_zexp_partials(const T* __restrict__ s, int64_t n, int64_t mask,
                                                            double* __restrict__ partials) {
  KSum acc;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double p = tnorm2(ldg_stream(s + i));
    acc.add((__popcll((unsigned long long)(i & mask)) & 1) ? -p : p);
  }
  const double r = block_sum(acc.value());
  if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

// host: fixed-order compensated sum of the partials
static double host_ksum(const double* v, int n, int stride) {
  double s = 0.0, c = 0.0;
  for (int i = 0; i < n; i++) {
    const double x = v[(size_t)i * stride];
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  return s + c;
}

template <typename TA, typename TB>
static int dot_typed(Context* ctx, const void* a, const void* b, int64_t n, double* out, bool maxdiff) {
  const unsigned grid = stream_grid(ctx, n);
  const size_t bytes = sizeof(double) * 2 * grid;
  SV_TRY(ensure_scratch(ctx, bytes));
  SV_TRY(ensure_host_pinned(ctx, bytes));
  double* d = (double*)ctx->scratch;
  if (maxdiff) k_maxdiff_partials<TA, TB><<<grid, kOpsBlock, 0, ctx->stream>>>((const TA*)a, (const TB*)b, n, d);
  else k_dot_partials<TA, TB><<<grid, kOpsBlock, 0, ctx->stream>>>((const TA*)a, (const TB*)b, n, d);
  SV_LAUNCH_CHECK("reduction launch");
  SV_TRY(check_cuda(cudaMemcpyAsync(ctx->host_pinned, d, bytes, cudaMemcpyDeviceToHost, ctx->stream), "reduction copy"));
  SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "reduction sync"));
  const double* h = (const double*)ctx->host_pinned;
  if (maxdiff) {
    double m = 0.0;
    for (unsigned i = 0; i < grid; i++) m = fmax(m, h[i]);
    out[0] = m;
  } else {
    out[0] = host_ksum(h, (int)grid, 2);
    out[1] = host_ksum(h + 1, (int)grid, 2);
  }
  return SV_OK;
}

template <typename TA>
static int dot_dispatch_b(Context* ctx, const void* a, const void* b, int dtb, int64_t n, double* out, bool maxdiff) {
  switch (dtb) {
    case SV_C128: return dot_typed<TA, c128>(ctx, a, b, n, out, maxdiff);
    case SV_C64: return dot_typed<TA, c64>(ctx, a, b, n, out, maxdiff);
    case SV_F64: return dot_typed<TA, double>(ctx, a, b, n, out, maxdiff);
    default: return dot_typed<TA, float>(ctx, a, b, n, out, maxdiff);
  }
}

static int dot_dispatch(Context* ctx, const void* a, int dta, const void* b, int dtb, int nqubits, double* out,
                        bool maxdiff) {
  SV_TRY(check_state(a, dta, nqubits));
  SV_TRY(check_state(b, dtb, nqubits));
  if (!out) return set_error(SV_ERR_ARG, "output pointer is NULL");
  const int64_t n = (int64_t)1 << nqubits;
  switch (dta) {
    case SV_C128: return dot_dispatch_b<c128>(ctx, a, b, dtb, n, out, maxdiff);
    case SV_C64: return dot_dispatch_b<c64>(ctx, a, b, dtb, n, out, maxdiff);
    case SV_F64: return dot_dispatch_b<double>(ctx, a, b, dtb, n, out, maxdiff);
    default: return dot_dispatch_b<float>(ctx, a, b, dtb, n, out, maxdiff);
  }
}

template <typename T>
static int zexp_typed(Context* ctx, const void* s, int64_t n, int64_t mask, double* out) {
  const unsigned grid = stream_grid(ctx, n);
  const size_t bytes = sizeof(double) * grid;
  SV_TRY(ensure_scratch(ctx, bytes));
  SV_TRY(ensure_host_pinned(ctx, bytes));
  double* d = (double*)ctx->scratch;
  k_zexp_partials<T><<<grid, kOpsBlock, 0, ctx->stream>>>((const T*)s, n, mask, d);
  SV_LAUNCH_CHECK("expectation launch");
  SV_TRY(check_cuda(cudaMemcpyAsync(ctx->host_pinned, d, bytes, cudaMemcpyDeviceToHost, ctx->stream), "expectation copy"));
  SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "expectation sync"));
  out[0] = host_ksum((const double*)ctx->host_pinned, (int)grid, 1);
  return SV_OK;
}

}  // namespace sv

extern "C" int sv_inner_product(sv_context* ctx, const void* a, int dtype_a, const void* b, int dtype_b, int nqubits,
                                double* out_re_im) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  return sv::dot_dispatch(ctx, a, dtype_a, b, dtype_b, nqubits, out_re_im, false);
}

extern "C" int sv_max_abs_diff(sv_context* ctx, const void* a, int dtype_a, const void* b, int dtype_b, int nqubits,
                               double* out) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  return sv::dot_dispatch(ctx, a, dtype_a, b, dtype_b, nqubits, out, true);
}

extern "C" int sv_expectation_z(sv_context* ctx, const void* state, int dtype, int nqubits, const int32_t* qubits,
                                int nq, double* out) {
  using namespace sv;
  if (!ctx) return set_error(SV_ERR_ARG, "null context");
  SV_TRY(check_state(state, dtype, nqubits));
  if (!out || (nq > 0 && !qubits) || nq < 0) return set_error(SV_ERR_ARG, "bad qubit list or output");
  int64_t mask = 0;
  for (int j = 0; j < nq; j++) {
    if (qubits[j] < 0 || qubits[j] >= nqubits) return set_error(SV_ERR_ARG, "qubit %d out of range", qubits[j]);
    mask ^= (int64_t)1 << (nqubits - 1 - qubits[j]);
  }
  const int64_t n = (int64_t)1 << nqubits;
  switch (dtype) {
    case SV_C128: return zexp_typed<c128>(ctx, state, n, mask, out);
    case SV_C64: return zexp_typed<c64>(ctx, state, n, mask, out);
    case SV_F64: return zexp_typed<double>(ctx, state, n, mask, out);
    default: return zexp_typed<float>(ctx, state, n, mask, out);
  }
}
