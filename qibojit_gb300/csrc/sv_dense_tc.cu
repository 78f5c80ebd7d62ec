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

#include <algorithm>
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

// 8 consecutive accumulator columns of this warp's 32 lanes (one lane per thread).
// The loads of a batch are issued back to back and waited for once (tmem_wait): the
// destination registers are only read after the wait statement.
__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
}
// Waits for this thread's outstanding tcgen05.ld; the registers are passed through the
// statement so the compiler cannot read them before it.
template <int N>
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[N]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < N; j++) asm volatile("" : "+r"(r[j]));
}

// Shared-memory matrix descriptors (tcgen05): start address, leading byte offset and
// stride byte offset in 16-byte units, descriptor version 1 at bits 46-47, base offset
// 0, layout type at bits 61-63.
//  * no swizzle (B operand): 8-row x 16-byte core matrices, K-adjacent ones `lbo`
//    bytes apart, 8-row groups `sbo` apart;
//  * 128-byte swizzle (A operand): rows of 128 bytes (32 FP32 values) in 1 KiB atoms
//    of 8 rows, 16-byte chunk c of row r stored at chunk c ^ (r % 8); 8-row groups
//    1 KiB apart; K steps inside an atom advance the start address by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_plain(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) |
         (2ull << 61);
}

// Instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// byte offset of element (row, k) in the no-swizzle K-major B operand with `kchunks`
// 16-byte chunks per row
__host__ __device__ constexpr uint32_t kmajor_offset(int row, int k, int kchunks) {
  return (uint32_t)((row >> 3) * (kchunks * 128) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}
// byte offset of the 16-byte chunk holding elements (row, 4c .. 4c+3) of the 128-byte
// swizzled A operand (128 rows per 32-column block)
__device__ __forceinline__ uint32_t sw128_chunk(int row, int c) {
  return (uint32_t)((c >> 3) * (kRows * 128) + (row >> 3) * 1024 + (row & 7) * 128 + (((c & 7) ^ (row & 7)) << 4));
}

template <int KT>
struct Shape {
  static constexpr int NA = 1 << KT;                    // amplitudes per group
  static constexpr int N = 2 * NA;                      // MMA N: real outputs
  static constexpr int A_BYTES = kRows * 2 * NA * 4;    // one precision part of A (128 rows x 2 NA)
  static constexpr int B_ROWS = 3 * NA;
  static constexpr int B_CHUNKS = NA / 4;
  static constexpr int B_SBO = B_CHUNKS * 128;
  static constexpr int B_BYTES = (B_ROWS / 8) * B_SBO;  // one precision part of B
  static constexpr int SMEM = 1024 + 2 * A_BYTES + 2 * B_BYTES + 64;  // + alignment slack
  static constexpr int TMEM_COLS = 2 * N < 32 ? 32 : 2 * N;  // two accumulators, power of two
  static constexpr int HALF = NA / 2;                   // inputs/outputs per thread (row mapping)
  static constexpr int ITEMS = kRows * NA / 4 / kThreads;  // 4-input chunks per thread (chunk mapping)
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
  int pairs;                  // local indices 2e, 2e+1 are adjacent amplitudes
};

// MAP 0: thread (row, half) loads half of its group's inputs with 8-byte loads; a
// warp's 32 lanes read 32 consecutive groups.  (Pairing lanes to move two adjacent
// groups with 16-byte accesses and a shuffle measured slower: 0.56 against 0.73 of
// the HBM peak for 6 targets.)  MAP 1 (the two lowest bits are targets, local index bits 0-1 = address bits 0-1):
// a thread loads chunks of 4 adjacent inputs (32 contiguous bytes), lanes running
// along the chunks of a group first.  All write 16-byte chunks of A, which the
// 128-byte swizzle spreads over all banks for every pattern.
template <int KT, int MAP>
__global__ void __launch_bounds__(kThreads, Shape<KT>::MIN_BLOCKS) k_dense_tc(const __grid_constant__ DenseTCParams p,
                                                                          const __grid_constant__ BitList q) {
  using S = Shape<KT>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);  // 1 KiB aligned
  unsigned char* a_hi = smem;
  unsigned char* a_lo = smem + S::A_BYTES;
  unsigned char* b_hi = smem + 2 * S::A_BYTES;
  unsigned char* b_lo = b_hi + S::B_BYTES;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(b_lo + S::B_BYTES);  // [2]
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(mbar + 2);
  __shared__ int s_abort;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int row = tid & (kRows - 1);  // TMEM lane of this thread in the epilogue
  const int half = tid >> 7;
  const int i0 = half * S::HALF;

  {
    const int4* src = reinterpret_cast<const int4*>(p.bimage);
    int4* dst = reinterpret_cast<int4*>(b_hi);
    for (int i = tid; i < 2 * S::B_BYTES / 16; i += kThreads) dst[i] = src[i];
  }
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
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

  // ---- tile loads into registers (8 or 4 inputs per 16-byte chunk of A)
  constexpr int NX = MAP == 0 ? S::HALF : 4 * S::ITEMS;
  float2 x[NX];
  auto load_tile = [&](int64_t tile) {
    if constexpr (MAP == 0) {
      const int64_t g = tile * kRows + row;
      if (g < p.ngroups) {
        const float2* base = p.state + (insert_ones(g, q) - p.zero_off);
#pragma unroll
        for (int j = 0; j < S::HALF; j++) x[j] = __ldcs(base + p.off[i0 + j]);
      } else {
#pragma unroll
        for (int j = 0; j < S::HALF; j++) x[j] = make_float2(0.f, 0.f);
      }
    } else {
#pragma unroll
      for (int it = 0; it < S::ITEMS; it++) {
        const int item = tid + it * kThreads;
        const int r = item / (S::NA / 4), c = item % (S::NA / 4);
        const int64_t g = tile * kRows + r;
        if (g < p.ngroups) {
          const float4* src =
              reinterpret_cast<const float4*>(p.state + (insert_ones(g, q) - p.zero_off) + p.off[4 * c]);
          const float4 v0 = __ldcs(src), v1 = __ldcs(src + 1);
          x[4 * it + 0] = make_float2(v0.x, v0.y);
          x[4 * it + 1] = make_float2(v0.z, v0.w);
          x[4 * it + 2] = make_float2(v1.x, v1.y);
          x[4 * it + 3] = make_float2(v1.z, v1.w);
        } else {
#pragma unroll
          for (int e = 0; e < 4; e++) x[4 * it + e] = make_float2(0.f, 0.f);
        }
      }
    }
  };
  // ---- split into hi/lo and store 16-byte chunks of A: real parts in columns
  //      [0, NA), imaginary parts in [NA, 2 NA)
  auto write_chunk = [&](int r, int c, const float2* v) {
    float4 rh, rl, ih, il;
    float* prh = &rh.x; float* prl = &rl.x; float* pih = &ih.x; float* pil = &il.x;
#pragma unroll
    for (int e = 0; e < 4; e++) {
      prh[e] = tf32_hi(v[e].x);
      prl[e] = v[e].x - prh[e];
      pih[e] = tf32_hi(v[e].y);
      pil[e] = v[e].y - pih[e];
    }
    const uint32_t ore = sw128_chunk(r, c), oim = sw128_chunk(r, S::NA / 4 + c);
    *reinterpret_cast<float4*>(a_hi + ore) = rh;
    *reinterpret_cast<float4*>(a_lo + ore) = rl;
    *reinterpret_cast<float4*>(a_hi + oim) = ih;
    *reinterpret_cast<float4*>(a_lo + oim) = il;
  };
  auto write_tile = [&]() {
    if constexpr (MAP == 0) {
#pragma unroll
      for (int c = 0; c < S::HALF / 4; c++) write_chunk(row, i0 / 4 + c, &x[4 * c]);
    } else {
#pragma unroll
      for (int it = 0; it < S::ITEMS; it++) {
        const int item = tid + it * kThreads;
        write_chunk(item / (S::NA / 4), item % (S::NA / 4), &x[4 * it]);
      }
    }
  };
  auto issue_mmas = [&](uint32_t d_tmem, uint32_t bar) {
    tc_fence_after();
    uint32_t acc = 0;
    // small products first: A_lo B_hi, A_hi B_lo, then A_hi B_hi
#pragma unroll
    for (int prod = 0; prod < 3; prod++) {
      const uint32_t au = prod == 0 ? a_lo_u : a_hi_u;
      const uint32_t bu = prod == 1 ? b_lo_u : b_hi_u;
#pragma unroll
      for (int s = 0; s < S::KSTEPS; s++) {
        const int kre = 8 * s, kim = S::NA + 8 * s;  // A columns of this K step
        // real inputs against B rows [NA, 3 NA) = [Ur; Ui]
        mma_tf32(d_tmem, smem_desc_sw128(au + (kre >> 5) * (kRows * 128) + (kre & 31) * 4),
                 smem_desc_plain(bu + (S::NA / 8) * S::B_SBO + 2 * s * 128, 128, S::B_SBO), idesc, acc);
        acc = 1;
        // imaginary inputs against B rows [0, 2 NA) = [-Ui; Ur]
        mma_tf32(d_tmem, smem_desc_sw128(au + (kim >> 5) * (kRows * 128) + (kim & 31) * 4),
                 smem_desc_plain(bu + 2 * s * 128, 128, S::B_SBO), idesc, 1);
      }
    }
    mma_commit(bar);
  };
  // ---- accumulator rows -> HBM; thread (row, half) stores half of its group's outputs
  auto epilogue = [&](int64_t tile, uint32_t dcol) {
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + dcol;
    uint32_t re[S::HALF], im[S::HALF];
#pragma unroll
    for (int c = 0; c < S::HALF / 8; c++) {
      tmem_ld8_nowait(lane_addr + (uint32_t)(i0 + 8 * c), *reinterpret_cast<uint32_t(*)[8]>(&re[8 * c]));
      tmem_ld8_nowait(lane_addr + (uint32_t)(S::NA + i0 + 8 * c), *reinterpret_cast<uint32_t(*)[8]>(&im[8 * c]));
    }
    tmem_wait(re);
    tmem_wait(im);
    {
      const int64_t g = tile * kRows + row;
      if (g >= p.ngroups) return;
      float2* base = p.state + (insert_ones(g, q) - p.zero_off);
      if (p.pairs) {
#pragma unroll
        for (int e = 0; e < S::HALF; e += 2)
          __stcs(reinterpret_cast<float4*>(base + p.off[i0 + e]),
                 make_float4(__uint_as_float(re[e]), __uint_as_float(im[e]), __uint_as_float(re[e + 1]),
                             __uint_as_float(im[e + 1])));
      } else {
#pragma unroll
        for (int e = 0; e < S::HALF; e++)
          __stcs(base + p.off[i0 + e], make_float2(__uint_as_float(re[e]), __uint_as_float(im[e])));
      }
    }
  };

  // Skewed pipeline: tile i's MMAs run while the threads load tile i+1 and drain tile
  // i-1's accumulator (two accumulators in TMEM); A is rewritten only after tile i's
  // MMAs have completed.
  uint32_t phases = 0;  // bit b: parity of the next completion of mbar[b]
  int64_t tile = blockIdx.x, prev = -1;
  int it = 0;
  if (tile < ntiles) load_tile(tile);
  for (; tile < ntiles; tile += gridDim.x, it++) {
    const int b = it & 1;
    if (prev >= 0) {  // A free and accumulator 1-b ready once tile i-1's MMAs complete
      if (!mbar_wait_bounded(smem_u32(&mbar[1 - b]), (phases >> (1 - b)) & 1)) s_abort = 1;
    }
    write_tile();
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (s_abort) break;
    if (tid == 0) issue_mmas(tmem + (uint32_t)(b * S::N), smem_u32(&mbar[b]));
    const int64_t next = tile + gridDim.x;
    if (next < ntiles) load_tile(next);
    if (prev >= 0) {
      tc_fence_after();
      epilogue(prev, (uint32_t)((1 - b) * S::N));
      phases ^= 1u << (1 - b);
    }
    tc_fence_before();
    prev = tile;
  }
  if (prev >= 0 && !s_abort) {
    const int b = (it - 1) & 1;
    if (mbar_wait_bounded(smem_u32(&mbar[b]), (phases >> b) & 1)) {
      tc_fence_after();
      epilogue(prev, (uint32_t)(b * S::N));
    } else {
      s_abort = 1;
    }
  }
  __syncthreads();
  if (s_abort && tid == 0) {
    atomicExch(p.status, 1);
    // the MMAs still in flight get one more bounded wait before their columns are freed
    mbar_wait_bounded(smem_u32(&mbar[0]), phases & 1);
    mbar_wait_bounded(smem_u32(&mbar[1]), (phases >> 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, S::TMEM_COLS);
}

// ------------------------------------------------------------------ host side
// B image of one precision part: element (row, k) of the stacked [-Ui; Ur; Ui] at its
// canonical-layout byte offset, for the gate U in the kernel's local index order.
template <int KT>
static void build_bimage(const std::vector<float>& u, std::vector<float>& img) {
  using S = Shape<KT>;
  img.assign((size_t)2 * S::B_BYTES / 4, 0.0f);
  float* hi = img.data();
  float* lo = img.data() + S::B_BYTES / 4;
  for (int o = 0; o < S::NA; o++) {
    for (int j = 0; j < S::NA; j++) {
      const float ur = u[2 * (o * S::NA + j)], ui = u[2 * (o * S::NA + j) + 1];
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
  // The kernel's local index bit v is the v-th lowest target bit position, so low
  // target bits are low local-index bits (contiguous amplitudes); the gate's row index
  // has targets[0] as its most significant bit, i.e. row bit u is targets[KT-1-u].
  int pos_of_u[KT], u_of_v[KT], sorted[KT];
  for (int u = 0; u < KT; u++) pos_of_u[u] = nqubits - targets[KT - 1 - u] - 1;
  for (int u = 0; u < KT; u++) sorted[u] = pos_of_u[u];
  std::sort(sorted, sorted + KT);
  for (int v = 0; v < KT; v++)
    for (int u = 0; u < KT; u++)
      if (pos_of_u[u] == sorted[v]) u_of_v[v] = u;
  std::vector<int> perm(S::NA);
  DenseTCParams p;
  memset(&p, 0, sizeof(p));
  for (int i = 0; i < S::NA; i++) {
    int64_t o = 0;
    int r = 0;
    for (int v = 0; v < KT; v++)
      if ((i >> v) & 1) {
        o += (int64_t)1 << sorted[v];
        r |= 1 << u_of_v[v];
      }
    p.off[i] = o;
    perm[i] = r;
  }
  const float* g = (const float*)gate;
  std::vector<float> u((size_t)2 * S::NA * S::NA);
  for (int o = 0; o < S::NA; o++)
    for (int j = 0; j < S::NA; j++) {
      const size_t src = 2 * ((size_t)perm[o] * S::NA + perm[j]), dst = 2 * ((size_t)o * S::NA + j);
      u[dst] = g[src];
      u[dst + 1] = g[src + 1];
    }
  p.zero_off = p.off[S::NA - 1];
  p.state = (float2*)state;
  p.ngroups = (int64_t)1 << (nqubits - q.n);
  const bool aligned16 = ((uintptr_t)state % 16) == 0;
  p.pairs = aligned16 && sorted[0] == 0;
  const bool chunked = aligned16 && sorted[0] == 0 && sorted[1] == 1;
  std::vector<float> img;
  build_bimage<KT>(u, img);
  const size_t ibytes = img.size() * sizeof(float);
  SV_TRY(ensure_operand(ctx, ibytes));
  SV_TRY(ensure_device_status(ctx));
  SV_TRY(check_cuda(cudaMemcpyAsync(ctx->operand, img.data(), ibytes, cudaMemcpyHostToDevice, ctx->stream),
                    "tensor-core gate operand upload"));
  p.bimage = (const float*)ctx->operand;
  p.status = ctx->device_status;
  auto kern = chunked ? k_dense_tc<KT, 1> : k_dense_tc<KT, 0>;
  SV_TRY(check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM),
                    "tensor-core kernel shared-memory attribute"));
  int per_sm = 0;
  SV_TRY(check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, S::SMEM),
                    "tensor-core kernel occupancy"));
  if (per_sm < 1) return set_error(SV_ERR_UNSUPPORTED, "tensor-core kernel does not fit on an SM");
  if (per_sm * S::TMEM_COLS > 512) per_sm = 512 / S::TMEM_COLS;  // every resident CTA holds its columns
  const int64_t ntiles = (p.ngroups + kRows - 1) / kRows;
  int64_t grid = (int64_t)ctx->num_sms * per_sm;
  if (grid > ntiles) grid = ntiles;
  kern<<<(unsigned)grid, kThreads, S::SMEM, ctx->stream>>>(p, q);
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
