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
#include "sv_device.cuh"

namespace sv {

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
  // device status word set by kernels whose bounded waits gave up (read by sv_sync)
  int* device_status = nullptr;
  bool status_pending = false;
  // dense k-target gates: SV_DENSE_AUTO, SV_DENSE_SIMT or SV_DENSE_TENSOR
  int dense_mode = 0;
  // complex128 per-gate arithmetic: 0 = double-word on the FP32 pipe, 1 = FP64
  int c128_fp64 = 0;
};

// error plumbing (thread-local last error string)
int set_error(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* what);
int ensure_scratch(Context* ctx, size_t bytes);
int ensure_host_pinned(Context* ctx, size_t bytes);
int ensure_operand(Context* ctx, size_t bytes);
int ensure_device_status(Context* ctx);
// after the context stream has been synchronised: SV_ERR_TIMEOUT when a kernel with a
// bounded wait gave up since the last check (the status word is then cleared)
int take_device_status(Context* ctx);

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
