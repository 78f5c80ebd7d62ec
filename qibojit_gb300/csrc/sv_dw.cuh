// sv_dw.cuh -- double-word (float-float) arithmetic for complex128 gate application.
//
// GB300 runs FP64 at 1/56 of its FP32 rate, so a complex128 gate pass with 8 FP64
// multiply-adds per amplitude is FP64-bound three times over (16 ms against 5 ms of
// HBM time at n = 30).  The per-gate complex128 kernels therefore compute in
// double-word arithmetic on the FP32 pipe: a double d is carried as an unevaluated sum
// hi + lo of two floats, products use the error-free transformation p = a*b,
// e = fma(a, b, -p) (Dekker 1971; Joldes, Muller and Popescu 2017, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic"), sums use
// Knuth's TwoSum.  Each output is a sum of such products, accumulated as an
// unnormalised (sum, error) pair and normalised once: about 2^-45 relative to the
// summed magnitudes sum_j |g_ij| |x_j|, i.e. a few 1e-15 absolute for amplitudes <= 1.
//
// Conversions use integer operations only (the FP64 pipe would otherwise be the
// bottleneck again): double -> (hi, lo) truncates the 52-bit mantissa into 24 + 23
// bits; (hi, lo) -> double assembles each float's bits into a double and adds the two
// with one FP64 addition.  Range: |values| < 2^128; values below 2^-103 keep their
// leading 24 bits (an absolute error below 2^-127); NaN and infinity are not carried.
#pragma once

#include <stdint.h>

#include "sv_device.cuh"

namespace sv {

// the double-word complex type and its conversions live in sv_device.cuh (shared with
// the pass kernels); the per-gate kernels use the accumulator below
using cdw = cw;

__device__ __forceinline__ cdw cdw_load(const double2& v) { return cdw(dw_from_double(v.x), dw_from_double(v.y)); }
__device__ __forceinline__ double2 cdw_store(const cdw& a) { return make_double2(dw_to_double(a.re), dw_to_double(a.im)); }

// (sum, error) accumulator of products: value = s + e, normalised by dwacc_result
struct dwacc {
  float s, e;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
  s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
}

// acc = a * b (the dropped a.l * b.l is below 2^-46 of the product)
__device__ __forceinline__ dwacc dw_prod(dw a, dw b) {
  dwacc r;
  r.s = a.h * b.h;
  r.e = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -r.s)));
  return r;
}
// acc += a * b
__device__ __forceinline__ void dw_fma(dwacc& acc, dw a, dw b) {
  const float p = a.h * b.h;
  const float pe = fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
  float s, t;
  two_sum(acc.s, p, s, t);
  acc.s = s;
  acc.e += pe + t;
}
__device__ __forceinline__ dw dwacc_result(dwacc acc) {
  dw r;
  two_sum(acc.s, acc.e, r.h, r.l);
  return r;
}
__device__ __forceinline__ dw dw_neg(dw a) { return -a; }

// complex sum_k m_k * v_k over N terms
template <int N>
__device__ __forceinline__ cdw cdw_dot(const cdw* m, const cdw* v) {
  dwacc re = dw_prod(m[0].re, v[0].re), im = dw_prod(m[0].re, v[0].im);
  dw_fma(re, dw_neg(m[0].im), v[0].im);
  dw_fma(im, m[0].im, v[0].re);
#pragma unroll
  for (int k = 1; k < N; k++) {
    dw_fma(re, m[k].re, v[k].re);
    dw_fma(re, dw_neg(m[k].im), v[k].im);
    dw_fma(im, m[k].re, v[k].im);
    dw_fma(im, m[k].im, v[k].re);
  }
  return cdw(dwacc_result(re), dwacc_result(im));
}

}  // namespace sv

// host: round-to-nearest split of a double into hi + lo floats
inline void sv_dw_split_host(double d, float* hi, float* lo) {
  const float h = (float)d;
  *hi = h;
  *lo = (float)(d - (double)h);
}
