// sv_common.cuh -- types, index maps and launch helpers shared by the engine's kernels.
//
// Amplitude layout: one contiguous 1-D array of 2^n amplitudes in HBM, complex values
// interleaved (re, im), so an amplitude is one naturally aligned 16-byte (complex128)
// or 8-byte (complex64) word.  Qubit q is bit n-q-1 of the amplitude index
// (qibojit src/qibojit/backends/cpu.py:565-569, 610).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "qibojit_gb300.h"

namespace sv {

// --------------------------------------------------------------- amplitude types
template <typename R>
struct alignas(2 * sizeof(R)) cplx {
  R re, im;
};

using c128 = cplx<double>;
using c64 = cplx<float>;

template <typename T> struct real_of { using type = T; };
template <typename R> struct real_of<cplx<R>> { using type = R; };

template <typename T> struct is_complex { static constexpr bool value = false; };
template <typename R> struct is_complex<cplx<R>> { static constexpr bool value = true; };

template <typename R>
__host__ __device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
__host__ __device__ __forceinline__ cplx<R> cadd(cplx<R> a, cplx<R> b) {
  return {a.re + b.re, a.im + b.im};
}
// a*x + b*y, the shape of every dense gate row
template <typename R>
__device__ __forceinline__ cplx<R> cmad2(cplx<R> a, cplx<R> x, cplx<R> b, cplx<R> y) {
  cplx<R> r;
  r.re = fma(a.re, x.re, fma(-a.im, x.im, fma(b.re, y.re, -b.im * y.im)));
  r.im = fma(a.re, x.im, fma(a.im, x.re, fma(b.re, y.im, b.im * y.re)));
  return r;
}
template <typename R>
__device__ __forceinline__ cplx<R> cfma(cplx<R> a, cplx<R> x, cplx<R> acc) {
  acc.re = fma(a.re, x.re, fma(-a.im, x.im, acc.re));
  acc.im = fma(a.re, x.im, fma(a.im, x.re, acc.im));
  return acc;
}
template <typename R> __device__ __forceinline__ R rmul(R a, R b) { return a * b; }

// generic helpers usable for both real and complex amplitude types
template <typename T> __device__ __forceinline__ T tmul(T a, T b) { return a * b; }
template <> __device__ __forceinline__ c128 tmul<c128>(c128 a, c128 b) { return cmul(a, b); }
template <> __device__ __forceinline__ c64 tmul<c64>(c64 a, c64 b) { return cmul(a, b); }
template <typename T> __device__ __forceinline__ T tfma(T a, T x, T acc) { return fma(a, x, acc); }
template <> __device__ __forceinline__ c128 tfma<c128>(c128 a, c128 x, c128 acc) { return cfma(a, x, acc); }
template <> __device__ __forceinline__ c64 tfma<c64>(c64 a, c64 x, c64 acc) { return cfma(a, x, acc); }
template <typename T> __device__ __forceinline__ T tzero() { return T(0); }
template <> __device__ __forceinline__ c128 tzero<c128>() { return {0.0, 0.0}; }
template <> __device__ __forceinline__ c64 tzero<c64>() { return {0.0f, 0.0f}; }
template <typename T> __device__ __forceinline__ T tneg(T a) { return -a; }
template <> __device__ __forceinline__ c128 tneg<c128>(c128 a) { return {-a.re, -a.im}; }
template <> __device__ __forceinline__ c64 tneg<c64>(c64 a) { return {-a.re, -a.im}; }
template <typename T> __device__ __forceinline__ double tnorm2(T a) { return (double)a * (double)a; }
template <> __device__ __forceinline__ double tnorm2<c128>(c128 a) { return a.re * a.re + a.im * a.im; }
template <> __device__ __forceinline__ double tnorm2<c64>(c64 a) {
  return (double)a.re * (double)a.re + (double)a.im * (double)a.im;
}

// streaming loads/stores: each amplitude is touched once per pass
template <typename T> __device__ __forceinline__ T ldg_stream(const T* p) { return __ldcs(p); }
template <> __device__ __forceinline__ c128 ldg_stream<c128>(const c128* p) {
  double2 v = __ldcs(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
template <> __device__ __forceinline__ c64 ldg_stream<c64>(const c64* p) {
  float2 v = __ldcs(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
// read-only cached load (operands reused by many threads)
template <typename T> __device__ __forceinline__ T ldg_ro(const T* p) { return __ldg(p); }
template <> __device__ __forceinline__ c128 ldg_ro<c128>(const c128* p) {
  double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
template <> __device__ __forceinline__ c64 ldg_ro<c64>(const c64* p) {
  float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
template <typename T> __device__ __forceinline__ void stg_stream(T* p, T v) { __stcs(p, v); }
template <> __device__ __forceinline__ void stg_stream<c128>(c128* p, c128 v) {
  __stcs(reinterpret_cast<double2*>(p), make_double2(v.re, v.im));
}
template <> __device__ __forceinline__ void stg_stream<c64>(c64* p, c64 v) {
  __stcs(reinterpret_cast<float2*>(p), make_float2(v.re, v.im));
}

// ----------------------------------------------------------------- index maps
constexpr int kMaxQubits = 40;     // largest state the engine addresses (2^40 amplitudes)
constexpr int kMaxTargets = 10;    // largest dense gate (2^10 x 2^10)

// Sorted bit positions of all qubits a gate touches (controls and targets), passed
// by value in the kernel parameters.
struct BitList {
  int n;
  int pos[kMaxQubits];
};

// Insert a 1 at every listed bit position (gates.py:5-12, multicontrol_index):
// maps a group index g to the amplitude with all listed bits set.
__device__ __forceinline__ int64_t insert_ones(int64_t g, const BitList& b) {
  int64_t i = g;
  for (int j = 0; j < b.n; j++) {
    const int p = b.pos[j];
    const int64_t k = (int64_t)1 << p;
    i = ((i >> p) << (p + 1)) + (i & (k - 1)) + k;
  }
  return i;
}
__device__ __forceinline__ int64_t insert_zero(int64_t g, int p) {
  const int64_t k = (int64_t)1 << p;
  return ((g >> p) << (p + 1)) + (g & (k - 1));
}

// ------------------------------------------------------------------- dtypes
inline size_t dtype_size(int dtype) {
  switch (dtype) {
    case SV_C128: return 16;
    case SV_C64: return 8;
    case SV_F64: return 8;
    case SV_F32: return 4;
    default: return 0;
  }
}

// ------------------------------------------------------------------- context
struct Context {
  int device = 0;
  cudaStream_t stream = 0;
  int num_sms = 0;
  // grow-only device scratch owned by the context (reduction partials, staged operands)
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // device copy of large gate operands (matrices of >= 6 targets)
  void* operand = nullptr;
  size_t operand_bytes = 0;
  // pinned host staging for reduction results read back by the host
  void* host_pinned = nullptr;
  size_t host_pinned_bytes = 0;
};

// error plumbing (thread-local last error string)
int set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
int ensure_scratch(Context* ctx, size_t bytes);
int ensure_host_pinned(Context* ctx, size_t bytes);
int ensure_operand(Context* ctx, size_t bytes);

#define SV_TRY(...)                  \
  do {                               \
    int _rc = (__VA_ARGS__);         \
    if (_rc != SV_OK) return _rc;    \
  } while (0)

#define SV_LAUNCH_CHECK(what) SV_TRY(::sv::check_cuda(cudaGetLastError(), what))

inline unsigned grid_for(int64_t work, int per_block) {
  int64_t g = (work + per_block - 1) / per_block;
  if (g < 1) g = 1;
  return (unsigned)g;
}

}  // namespace sv

// The opaque handle of the C ABI is the engine context.
struct sv_context : public sv::Context {};
