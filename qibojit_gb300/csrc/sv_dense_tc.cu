// sv_dense_tc.cu -- dense k-target gates (k = 4, 5, 6) on complex64 states with the
// 5th-generation tensor cores (tcgen05.mma, kind::tf32, accumulators in tensor memory).
//
// The reference applies a k-target gate as a 2^k x 2^k complex matvec per index group
// (gates.py:265-424, raw_kernels.py:478-518, the operand of _multi_qubit_base at
// cpu.py:581-604).  A GPU tile of 128 consecutive index groups is a 128 x 2^k complex
// matrix X (row = group, column = local index), and the gate is Y = X U^T.  Written
// with real and imaginary parts side by side,
//
//   [Yr | Yi] = [Xr | Xi] . [[ Ur^T, Ui^T ], [ -Ui^T, Ur^T ]]
//
// one MMA of M = 128 (groups), N = 2^(k+1) (real outputs) per 8-wide K step, over
// K = 2^(k+1) real inputs.  The B operand (N x K, K-major) is stored once as the
// stacked rows [-Ui; Ur; Ui] (3 * 2^k rows, 2^k columns): the K steps over the real
// inputs read rows [2^k, 3 * 2^k) = [Ur; Ui], those over the imaginary inputs rows
// [0, 2^k) + [2^k, 2 * 2^k) = [-Ui; Ur].
//
// Precision: tf32 keeps 10 mantissa bits, so both operands are split as v = hi + lo
// (hi = v with its low 13 mantissa bits cleared, lo = v - hi, exact in FP32) and the
// products lo*hi + hi*lo + hi*hi accumulate in FP32 (the dropped lo*lo is below
// 2^-21 of the result): the complex64 gate to about 2^-21 relative, close to a plain
// FP32 matvec.  The engine's other complex64 kernels round at 2^-24.
//
// Shared-memory operands use the tcgen05 canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, K-adjacent core matrices 128 bytes apart (LBO),
// 8-row groups SBO bytes apart.  The state rows are written by the thread that owns
// the group (one 16-byte store per 4 inputs: the 8 rows of a quarter warp fill one
// 128-byte line, so the stores are conflict-free).
//
// Pipeline per CTA (persistent, one CTA per tile at a time): registers -> split ->
// A tiles in shared memory -> one thread issues 3 * 2^(k-2) MMAs and commits them to
// an mbarrier -> every thread loads the next tile's amplitudes from HBM while the
// MMAs run -> bounded wait on the mbarrier -> tcgen05.ld of the accumulator ->
// streaming stores of the outputs.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "sv_common.cuh"
#include "sv_dense_tc.cuh"

namespace sv {

namespace tc {

constexpr int kThreads = 256;  // 8 warps: warps w and w+4 share TMEM lane quadrant w % 4
constexpr int kRows = 128;     // index groups per tile = MMA M
constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s bound on any wait

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void tmem_alloc(uint32_t holder, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(holder), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// generic-proxy writes to shared memory become visible to the tensor cores (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of the mbarrier for at most kWaitNs; false on time-out.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity) {
  if (mbar_try_wait(mbar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  while (!mbar_try_wait(mbar, parity))
    if (globaltimer_ns() - t0 > kWaitNs) return false;
  return true;
}

// 8 consecutive accumulator columns of this warp's 32 lanes (one lane per thread),
// with the wait for the load in the same statement so the registers are defined
// when the statement ends.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 8; j++) v[j] = __uint_as_float(r[j]);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading (K-direction core
// matrix) byte offset, stride (8-row group) byte offset, all in 16-byte units; bits
// 46-47 hold the descriptor version 1; no swizzle, base offset 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// byte offset of element (row, k) in a K-major no-swizzle operand with `kchunks`
// 16-byte chunks (4 FP32 values) per row
__host__ __device__ constexpr uint32_t kmajor_offset(int row, int k, int kchunks) {
  return (uint32_t)((row >> 3) * (kchunks * 128) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

template <int KT>
struct Shape {
  static constexpr int NA = 1 << KT;                    // amplitudes per group
  static constexpr int N = 2 * NA;                      // MMA N: real outputs
  static constexpr int A_CHUNKS = 2 * NA / 4;           // 16-byte chunks per state row
  static constexpr int A_SBO = A_CHUNKS * 128;          // bytes per 8-row group of A
  static constexpr int A_BYTES = (kRows / 8) * A_SBO;   // one precision part of A
  static constexpr int B_ROWS = 3 * NA;
  static constexpr int B_CHUNKS = NA / 4;
  static constexpr int B_SBO = B_CHUNKS * 128;
  static constexpr int B_BYTES = (B_ROWS / 8) * B_SBO;  // one precision part of B
  static constexpr int SMEM = 2 * A_BYTES + 2 * B_BYTES + 64;
  static constexpr int TMEM_COLS = N < 32 ? 32 : N;     // power of two >= 32
  static constexpr int HALF = NA / 2;                   // inputs/outputs per thread
  static constexpr int KSTEPS = NA / 8;                 // 8-wide K steps per input half
  static constexpr int MIN_BLOCKS = KT == 6 ? 1 : (KT == 5 ? 2 : 3);  // resident CTAs per SM
};

struct DenseTCParams {
  float2* state;
  int64_t ngroups;
  int64_t zero_off;           // all-ones index of the targets -> group origin
  int64_t off[64];            // local index i -> offset of its amplitude from the origin
  const float* bimage;        // [hi | lo] B images in the shared-memory byte layout
  int* status;                // set to 1 when a wait times out
};

template <int KT>
__global__ void __launch_bounds__(kThreads, Shape<KT>::MIN_BLOCKS) k_dense_tc(const __grid_constant__ DenseTCParams p,
                                                          const __grid_constant__ BitList q) {
  using S = Shape<KT>;
  extern __shared__ __align__(128) unsigned char smem[];
  unsigned char* a_hi = smem;
  unsigned char* a_lo = smem + S::A_BYTES;
  unsigned char* b_hi = smem + 2 * S::A_BYTES;
  unsigned char* b_lo = b_hi + S::B_BYTES;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(b_lo + S::B_BYTES);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(mbar + 1);
  __shared__ int s_abort;
  __shared__ uint32_t s_abort_phase;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int row = tid & (kRows - 1);  // index group within the tile (TMEM lane)
  const int half = tid >> 7;          // which half of the local indices this thread owns

  // B images (both precision parts) from global memory (L2-resident, read once per CTA)
  {
    const int4* src = reinterpret_cast<const int4*>(p.bimage);
    int4* dst = reinterpret_cast<int4*>(b_hi);
    for (int i = tid; i < 2 * S::B_BYTES / 16; i += kThreads) dst[i] = src[i];
  }
  if (tid == 0) {
    mbar_init(smem_u32(mbar), 1);
    s_abort = 0;
  }
  if (warp == 0) tmem_alloc(smem_u32(tmem_holder), S::TMEM_COLS);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;

  const int64_t ntiles = (p.ngroups + kRows - 1) / kRows;
  constexpr uint32_t idesc = idesc_tf32(kRows, S::N);
  const uint32_t a_hi_u = smem_u32(a_hi), a_lo_u = smem_u32(a_lo);
  const uint32_t b_hi_u = smem_u32(b_hi), b_lo_u = smem_u32(b_lo);
  const int i0 = half * S::HALF;

  float2 x[S::HALF];
  auto load_tile = [&](int64_t tile) {
    const int64_t g = tile * kRows + row;
    if (g < p.ngroups) {
      const float2* base = p.state + (insert_ones(g, q) - p.zero_off);
#pragma unroll
      for (int j = 0; j < S::HALF; j++) x[j] = __ldcs(base + p.off[i0 + j]);
    } else {
#pragma unroll
      for (int j = 0; j < S::HALF; j++) x[j] = make_float2(0.f, 0.f);
    }
  };

  uint32_t phase = 0;
  int64_t tile = blockIdx.x;
  if (tile < ntiles) load_tile(tile);
  for (; tile < ntiles; tile += gridDim.x) {
    // split this thread's inputs into hi/lo and write them into its row of A:
    // real parts at columns [0, NA), imaginary parts at [NA, 2 NA)
#pragma unroll
    for (int c = 0; c < S::HALF / 4; c++) {
      float4 rh, rl, ih, il;
      float* prh = &rh.x; float* prl = &rl.x; float* pih = &ih.x; float* pil = &il.x;
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const float2 v = x[4 * c + e];
        prh[e] = tf32_hi(v.x);
        prl[e] = v.x - prh[e];
        pih[e] = tf32_hi(v.y);
        pil[e] = v.y - pih[e];
      }
      const int kr = i0 + 4 * c, ki = S::NA + i0 + 4 * c;
      *reinterpret_cast<float4*>(a_hi + kmajor_offset(row, kr, S::A_CHUNKS)) = rh;
      *reinterpret_cast<float4*>(a_lo + kmajor_offset(row, kr, S::A_CHUNKS)) = rl;
      *reinterpret_cast<float4*>(a_hi + kmajor_offset(row, ki, S::A_CHUNKS)) = ih;
      *reinterpret_cast<float4*>(a_lo + kmajor_offset(row, ki, S::A_CHUNKS)) = il;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      uint32_t acc = 0;
      // small products first: A_lo B_hi, A_hi B_lo, then A_hi B_hi
#pragma unroll
      for (int prod = 0; prod < 3; prod++) {
        const uint32_t au = prod == 0 ? a_lo_u : a_hi_u;
        const uint32_t bu = prod == 1 ? b_lo_u : b_hi_u;
#pragma unroll
        for (int s = 0; s < S::KSTEPS; s++) {
          // real inputs (A columns [8s, 8s+8)) against B rows [NA, 3 NA) = [Ur; Ui]
          mma_tf32(tmem, smem_desc(au + 2 * s * 128, 128, S::A_SBO),
                   smem_desc(bu + (S::NA / 8) * S::B_SBO + 2 * s * 128, 128, S::B_SBO), idesc, acc);
          acc = 1;
          // imaginary inputs (A columns NA + [8s, 8s+8)) against B rows [0, 2 NA) = [-Ui; Ur]
          mma_tf32(tmem, smem_desc(au + (S::A_CHUNKS / 2 + 2 * s) * 128, 128, S::A_SBO),
                   smem_desc(bu + 2 * s * 128, 128, S::B_SBO), idesc, 1);
        }
      }
      mma_commit(smem_u32(mbar));
    }
    const int64_t this_tile = tile;
    const int64_t next = tile + gridDim.x;
    if (next < ntiles) load_tile(next);  // HBM reads of the next tile overlap the MMAs
    if (!mbar_wait_bounded(smem_u32(mbar), phase)) {
      s_abort = 1;
      s_abort_phase = phase;
    }
    phase ^= 1;
    tc_fence_after();
    __syncthreads();
    if (s_abort) break;
    // accumulator row `row`: real outputs in columns [0, NA), imaginary in [NA, 2 NA)
    const int64_t g = this_tile * kRows + row;
    float2* base = p.state + (insert_ones(g < p.ngroups ? g : 0, q) - p.zero_off);
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
#pragma unroll
    for (int c = 0; c < S::HALF / 8; c++) {
      float re[8], im[8];
      tmem_ld8(lane_addr + (uint32_t)(i0 + 8 * c), re);
      tmem_ld8(lane_addr + (uint32_t)(S::NA + i0 + 8 * c), im);
      if (g < p.ngroups) {
#pragma unroll
        for (int e = 0; e < 8; e++) __stcs(base + p.off[i0 + 8 * c + e], make_float2(re[e], im[e]));
      }
    }
    tc_fence_before();
    __syncthreads();  // accumulator read and A free before the next tile's MMAs
  }
  if (s_abort && tid == 0) {
    atomicExch(p.status, 1);
    // give the MMAs still in flight one more bounded wait before their columns are freed
    mbar_wait_bounded(smem_u32(mbar), s_abort_phase);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, S::TMEM_COLS);
}

// ------------------------------------------------------------------ host side
// B image of one precision part: element (row, k) of the stacked [-Ui; Ur; Ui] at its
// canonical-layout byte offset.
template <int KT>
static void build_bimage(const float* gate, std::vector<float>& img) {
  using S = Shape<KT>;
  img.assign((size_t)2 * S::B_BYTES / 4, 0.0f);
  float* hi = img.data();
  float* lo = img.data() + S::B_BYTES / 4;
  for (int o = 0; o < S::NA; o++) {
    for (int j = 0; j < S::NA; j++) {
      const float ur = gate[2 * (o * S::NA + j)], ui = gate[2 * (o * S::NA + j) + 1];
      const float vals[3] = {-ui, ur, ui};
      for (int blk = 0; blk < 3; blk++) {
        const float v = vals[blk];
        uint32_t bits;
        memcpy(&bits, &v, 4);
        bits &= 0xFFFFE000u;
        float h;
        memcpy(&h, &bits, 4);
        const uint32_t off = kmajor_offset(blk * S::NA + o, j, S::B_CHUNKS) / 4;
        hi[off] = h;
        lo[off] = v - h;
      }
    }
  }
}

template <int KT>
static int launch(Context* ctx, void* state, int nqubits, const void* gate, const int32_t* targets,
                  const BitList& q) {
  using S = Shape<KT>;
  DenseTCParams p;
  memset(&p, 0, sizeof(p));
  for (int i = 0; i < S::NA; i++) {
    int64_t o = 0;
    for (int u = 0; u < KT; u++)
      if ((i >> u) & 1) o += (int64_t)1 << (nqubits - targets[KT - 1 - u] - 1);
    p.off[i] = o;
  }
  p.zero_off = p.off[S::NA - 1];
  p.state = (float2*)state;
  p.ngroups = (int64_t)1 << (nqubits - q.n);
  std::vector<float> img;
  build_bimage<KT>((const float*)gate, img);
  const size_t ibytes = img.size() * sizeof(float);
  SV_TRY(ensure_operand(ctx, ibytes));
  SV_TRY(ensure_device_status(ctx));
  SV_TRY(check_cuda(cudaMemcpyAsync(ctx->operand, img.data(), ibytes, cudaMemcpyHostToDevice, ctx->stream),
                    "tensor-core gate operand upload"));
  p.bimage = (const float*)ctx->operand;
  p.status = ctx->device_status;
  SV_TRY(check_cuda(cudaFuncSetAttribute(k_dense_tc<KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM),
                    "tensor-core kernel shared-memory attribute"));
  int per_sm = 0;
  SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dense_tc<KT>, kThreads, S::SMEM),
                    "tensor-core kernel occupancy"));
  if (per_sm < 1) return set_error(SV_ERR_UNSUPPORTED, "tensor-core kernel does not fit on an SM");
  if (per_sm * S::TMEM_COLS > 512) per_sm = 512 / S::TMEM_COLS;  // every resident CTA holds its columns
  const int64_t ntiles = (p.ngroups + kRows - 1) / kRows;
  int64_t grid = (int64_t)ctx->num_sms * per_sm;
  if (grid > ntiles) grid = ntiles;
  k_dense_tc<KT><<<(unsigned)grid, kThreads, S::SMEM, ctx->stream>>>(p, q);
  SV_LAUNCH_CHECK("tensor-core dense gate launch");
  ctx->status_pending = true;
  return SV_OK;
}

}  // namespace tc

bool dense_tc_eligible(int dtype, int k) { return dtype == SV_C64 && k >= 4 && k <= 6; }

int dense_tc_apply(Context* ctx, void* state, int nqubits, const void* gate, const int32_t* targets, int k,
                   const BitList& q) {
  if (((uintptr_t)state) % 8) return set_error(SV_ERR_ARG, "complex64 state must be 8-byte aligned");
  switch (k) {
    case 4: return tc::launch<4>(ctx, state, nqubits, gate, targets, q);
    case 5: return tc::launch<5>(ctx, state, nqubits, gate, targets, q);
    case 6: return tc::launch<6>(ctx, state, nqubits, gate, targets, q);
    default: return set_error(SV_ERR_UNSUPPORTED, "tensor-core dense gates take 4..6 targets, not %d", k);
  }
}

}  // namespace sv
