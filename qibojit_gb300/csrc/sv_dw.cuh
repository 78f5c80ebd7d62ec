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

namespace sv {

struct dw {
  float h, l;
};
struct cdw {
  dw re, im;
};

__device__ __forceinline__ dw dw_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const uint32_t hb = (uint32_t)(b >> 32), lb = (uint32_t)b;
  const uint32_t sign = hb & 0x80000000u;
  const uint32_t e = (hb >> 20) & 0x7ffu;
  const uint32_t m23 = __funnelshift_l(lb, hb, 3) & 0x7fffffu;  // mantissa bits 51..29
  const uint32_t r23 = (lb >> 6) & 0x7fffffu;                    // mantissa bits 28..6
  dw r;
  r.h = __uint_as_float(sign | ((e - 896u) << 23) | m23);
  // (1 + r23 / 2^23) * 2^E' - 2^E' = r23 * 2^(E' - 23), exact (E' = e - 919 biased)
  const uint32_t eb = sign | ((e - 919u) << 23);
  r.l = __uint_as_float(eb | r23) - __uint_as_float(eb);
  if (e < 920u) {
    r.l = __uint_as_float(sign);
    if (e < 897u) r.h = __uint_as_float(sign);
  }
  return r;
}

// exact float -> double by its bits (zero and subnormal floats give a signed zero)
__device__ __forceinline__ double double_of_float_bits(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t sign = u & 0x80000000u, E = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  const unsigned long long bits = E == 0 ? (unsigned long long)sign << 32
                                         : ((unsigned long long)(sign | ((E + 896u) << 20) | (m >> 3)) << 32) |
                                               (unsigned long long)(m << 29);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double dw_to_double(dw a) { return double_of_float_bits(a.h) + double_of_float_bits(a.l); }

__device__ __forceinline__ cdw cdw_load(const double2& v) { return {dw_from_double(v.x), dw_from_double(v.y)}; }
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
__device__ __forceinline__ dw dw_neg(dw a) { return {-a.h, -a.l}; }

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
  return {dwacc_result(re), dwacc_result(im)};
}

}  // namespace sv

// host: round-to-nearest split of a double into hi + lo floats
inline void sv_dw_split_host(double d, float* hi, float* lo) {
  const float h = (float)d;
  *hi = h;
  *lo = (float)(d - (double)h);
}
