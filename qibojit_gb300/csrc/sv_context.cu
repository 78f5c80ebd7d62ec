// sv_context.cu -- engine context, error reporting and scratch management.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "sv_common.cuh"

namespace sv {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return SV_OK;
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return set_error(SV_ERR_OOM, "%s: out of device memory", what);
  }
  return set_error(SV_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int ensure_scratch(Context* ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return SV_OK;
  if (ctx->scratch) {
    // the old buffer may still be read by queued work on the stream
    SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "scratch resize (sync)"));
    cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
  }
  size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
  SV_TRY(check_cuda(cudaMalloc(&ctx->scratch, want), "scratch allocation"));
  ctx->scratch_bytes = want;
  return SV_OK;
}

int ensure_host_pinned(Context* ctx, size_t bytes) {
  if (bytes <= ctx->host_pinned_bytes) return SV_OK;
  if (ctx->host_pinned) {
    SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "pinned resize (sync)"));
    cudaFreeHost(ctx->host_pinned);
    ctx->host_pinned = nullptr;
    ctx->host_pinned_bytes = 0;
  }
  size_t want = bytes < 4096 ? 4096 : bytes;
  SV_TRY(check_cuda(cudaMallocHost(&ctx->host_pinned, want), "pinned host allocation"));
  ctx->host_pinned_bytes = want;
  return SV_OK;
}

int ensure_operand(Context* ctx, size_t bytes) {
  if (bytes <= ctx->operand_bytes) return SV_OK;
  if (ctx->operand) {
    SV_TRY(check_cuda(cudaStreamSynchronize(ctx->stream), "operand resize (sync)"));
    cudaFree(ctx->operand);
    ctx->operand = nullptr;
    ctx->operand_bytes = 0;
  }
  size_t want = bytes < (64u << 10) ? (64u << 10) : bytes;
  SV_TRY(check_cuda(cudaMalloc(&ctx->operand, want), "operand allocation"));
  ctx->operand_bytes = want;
  return SV_OK;
}

int take_device_status(Context* ctx) {
  if (!ctx->status_pending) return SV_OK;
  // kernels with bounded waits report a time-out in the status word: 1 from the
  // tensor-core gates, 2 from the persistent batch executor
  ctx->status_pending = false;
  int status = 0;
  SV_TRY(check_cuda(cudaMemcpy(&status, ctx->device_status, sizeof(int), cudaMemcpyDeviceToHost), "status word read"));
  if (status == 0) return SV_OK;
  SV_TRY(check_cuda(cudaMemset(ctx->device_status, 0, sizeof(int)), "status word reset"));
  if (status == 2)
    return set_error(SV_ERR_TIMEOUT, "the persistent batch executor gave up waiting for a circuit's previous pass");
  return set_error(SV_ERR_TIMEOUT, "a tensor-core gate kernel gave up waiting for its matrix operations");
}

int ensure_device_status(Context* ctx) {
  if (ctx->device_status) return SV_OK;
  SV_TRY(check_cuda(cudaMalloc(&ctx->device_status, sizeof(int)), "status word allocation"));
  SV_TRY(check_cuda(cudaMemsetAsync(ctx->device_status, 0, sizeof(int), ctx->stream), "status word reset"));
  return SV_OK;
}

}  // namespace sv

extern "C" {

int sv_version(void) { return 100; }

const char* sv_last_error(void) { return sv::g_last_error; }

int sv_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return n;
}

int sv_context_create(int device, sv_context** out) {
  if (!out) return sv::set_error(SV_ERR_ARG, "sv_context_create: out is NULL");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return sv::set_error(SV_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= n)
    return sv::set_error(SV_ERR_ARG, "device %d out of range (%d devices)", device, n);
  SV_TRY(sv::check_cuda(cudaSetDevice(device), "cudaSetDevice"));
  cudaDeviceProp prop;
  SV_TRY(sv::check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties"));
  if (prop.major * 10 + prop.minor < 100)
    return sv::set_error(SV_ERR_NO_DEVICE, "device %d is sm_%d%d; this build targets sm_103a",
                         device, prop.major, prop.minor);
  sv_context* ctx = new sv_context();
  ctx->device = device;
  ctx->stream = 0;
  ctx->num_sms = prop.multiProcessorCount;
  *out = ctx;
  return SV_OK;
}

int sv_context_destroy(sv_context* ctx) {
  if (!ctx) return SV_OK;
  cudaSetDevice(ctx->device);
  if (ctx->scratch || ctx->operand || ctx->host_pinned) cudaStreamSynchronize(ctx->stream);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->operand) cudaFree(ctx->operand);
  if (ctx->host_pinned) cudaFreeHost(ctx->host_pinned);
  if (ctx->device_status) cudaFree(ctx->device_status);
  delete ctx;
  return SV_OK;
}

int sv_context_set_stream(sv_context* ctx, void* stream) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  ctx->stream = (cudaStream_t)stream;
  return SV_OK;
}

int sv_context_set_dense_mode(sv_context* ctx, int mode) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  if (mode < SV_DENSE_AUTO || mode > SV_DENSE_TENSOR) return sv::set_error(SV_ERR_ARG, "unknown dense mode %d", mode);
  ctx->dense_mode = mode;
  return SV_OK;
}

int sv_context_set_c128_arithmetic(sv_context* ctx, int mode) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  if (mode != SV_C128_DOUBLE_WORD && mode != SV_C128_FP64)
    return sv::set_error(SV_ERR_ARG, "unknown complex128 arithmetic mode %d", mode);
  ctx->c128_fp64 = mode == SV_C128_FP64;
  return SV_OK;
}

int sv_sync(sv_context* ctx) {
  if (!ctx) return sv::set_error(SV_ERR_ARG, "null context");
  SV_TRY(sv::check_cuda(cudaStreamSynchronize(ctx->stream), "sv_sync"));
  return sv::take_device_status(ctx);
}

}  // extern "C"
