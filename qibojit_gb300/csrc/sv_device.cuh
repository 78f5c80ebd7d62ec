// sv_device.cuh -- device code shared by the compiled kernels and by the pass
// kernels specialised at run time.
//
// Amplitude types and their arithmetic, the shared-memory tile index map, cp.async
// wrappers and the register-level gate ops (a thread's 16 amplitudes of one phase).
// The file is self-contained (no includes, no host-only types) so the engine can hand
// its text to the CUDA runtime compiler unchanged.
#pragma once

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

// ------------------------------------------------------ double-word complex128
// GB300 runs FP64 at 1/56 of its FP32 rate.  `cw` carries a complex128 amplitude as two
// unevaluated float pairs (hi + lo per component), 16 bytes like the complex128 it
// stands for, and computes on the FP32 pipe: products by the error-free transformation
// p = a*b, e = fma(a, b, -p) plus the cross terms (Dekker 1971; Joldes, Muller and
// Popescu 2017), sums by Knuth's TwoSum, one normalisation per result: about 2^-46
// relative per operation.  Memory keeps doubles: dw_from_double splits the 52-bit
// mantissa into 24 + 23 bits with integer operations only (values below 2^-103 keep 24
// bits), dw_to_double assembles both floats' bits into doubles and adds them with one
// FP64 addition.  Range: |values| < 2^128; NaN and infinity are not carried.
struct dw {
  float h, l;
};

struct alignas(16) cw {
  dw re, im;
  cw() = default;
  __host__ __device__ constexpr cw(dw r, dw i) : re(r), im(i) {}
  // constants such as {1, 0}: the nearest float pair of each double
  __host__ __device__ cw(double r, double i) : re(split(r)), im(split(i)) {}
  static __host__ __device__ dw split(double x) {
    dw d;
    d.h = (float)x;
    d.l = (float)(x - (double)d.h);
    return d;
  }
};

__device__ __forceinline__ dw dw_from_double(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hb = (unsigned)(b >> 32), lb = (unsigned)b;
  const unsigned sign = hb & 0x80000000u;
  const unsigned e = (hb >> 20) & 0x7ffu;
  const unsigned m23 = __funnelshift_l(lb, hb, 3) & 0x7fffffu;  // mantissa bits 51..29
  const unsigned r23 = (lb >> 6) & 0x7fffffu;                    // mantissa bits 28..6
  dw r;
  r.h = __uint_as_float(sign | ((e - 896u) << 23) | m23);
  // (1 + r23 / 2^23) * 2^E' - 2^E' = r23 * 2^(E' - 23), exact (E' = e - 919 biased)
  const unsigned eb = sign | ((e - 919u) << 23);
  r.l = __uint_as_float(eb | r23) - __uint_as_float(eb);
  if (e < 920u) {
    r.l = __uint_as_float(sign);
    if (e < 897u) r.h = __uint_as_float(sign);
  }
  return r;
}
// exact float -> double by its bits (zero and subnormal floats give a signed zero)
__device__ __forceinline__ double double_of_float_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u, E = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  const unsigned long long bits = E == 0 ? (unsigned long long)sign << 32
                                         : ((unsigned long long)(sign | ((E + 896u) << 20) | (m >> 3)) << 32) |
                                               (unsigned long long)(m << 29);
  return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ double dw_to_double(dw a) { return double_of_float_bits(a.h) + double_of_float_bits(a.l); }

__device__ __forceinline__ void dw_two_sum(float a, float b, float& s, float& err) {
  s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
}
// renormalises s + e where e is the rounding error of the operation that made s (|e|
// at most ulp-sized against the summed products): Dekker's fast two-sum, 3 operations;
// after cancellation, when |s| may drop below |e|, the pair still sums to s + e within
// ulp(e), far below the magnitudes summed
__device__ __forceinline__ dw dw_norm(float s, float e) {
  dw r;
  r.h = s + e;
  r.l = e - (r.h - s);
  return r;
}
// a.h * b exactly split: p + e = a*b up to the dropped a.l*b.l
__device__ __forceinline__ float dw_prod_err(dw a, dw b, float p) {
  return fmaf(a.h, b.l, fmaf(a.l, b.h, fmaf(a.h, b.h, -p)));
}
__device__ __forceinline__ dw operator-(dw a) {
  dw r;
  r.h = -a.h;
  r.l = -a.l;
  return r;
}
__device__ __forceinline__ dw operator+(dw a, dw b) {
  float s, e;
  dw_two_sum(a.h, b.h, s, e);
  return dw_norm(s, e + (a.l + b.l));
}
__device__ __forceinline__ dw operator-(dw a, dw b) { return a + (-b); }
__device__ __forceinline__ dw operator*(dw a, dw b) {
  const float p = a.h * b.h;
  return dw_norm(p, dw_prod_err(a, b, p));
}
// a1*b1 + a2*b2 (+ c), one normalisation
__device__ __forceinline__ dw dw_dot2(dw a1, dw b1, dw a2, dw b2) {
  const float p1 = a1.h * b1.h, p2 = a2.h * b2.h;
  float s, t;
  dw_two_sum(p1, p2, s, t);
  return dw_norm(s, t + (dw_prod_err(a1, b1, p1) + dw_prod_err(a2, b2, p2)));
}
__device__ __forceinline__ dw dw_dot2_add(dw a1, dw b1, dw a2, dw b2, dw c) {
  const float p1 = a1.h * b1.h, p2 = a2.h * b2.h;
  float s, t, s2, t2;
  dw_two_sum(p1, p2, s, t);
  dw_two_sum(s, c.h, s2, t2);
  return dw_norm(s2, t2 + t + c.l + (dw_prod_err(a1, b1, p1) + dw_prod_err(a2, b2, p2)));
}

// multiply-add on the real type of an amplitude: a * b + c
__device__ __forceinline__ float rfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ dw rfma(dw a, dw b, dw c) {
  const float p = a.h * b.h;
  float s, t;
  dw_two_sum(p, c.h, s, t);
  return dw_norm(s, t + (dw_prod_err(a, b, p) + c.l));
}

template <> struct real_of<cw> { using type = dw; };
template <> struct is_complex<cw> { static constexpr bool value = true; };
// amplitude types kept in memory as doubles and converted in registers or shared memory
template <typename T> struct stored_as_double_pairs { static constexpr bool value = false; };
template <> struct stored_as_double_pairs<cw> { static constexpr bool value = true; };
template <> __device__ __forceinline__ cw tmul<cw>(cw a, cw b) {
  return cw(dw_dot2(a.re, b.re, -a.im, b.im), dw_dot2(a.re, b.im, a.im, b.re));
}
template <> __device__ __forceinline__ cw tfma<cw>(cw a, cw x, cw acc) {
  return cw(dw_dot2_add(a.re, x.re, -a.im, x.im, acc.re), dw_dot2_add(a.re, x.im, a.im, x.re, acc.im));
}
template <> __device__ __forceinline__ cw tzero<cw>() { return cw(dw{0.0f, 0.0f}, dw{0.0f, 0.0f}); }
template <> __device__ __forceinline__ cw tneg<cw>(cw a) { return cw(-a.re, -a.im); }
// a tile element written by a raw 16-byte copy of a complex128 amplitude -> cw, in place
__device__ __forceinline__ void cw_from_stored(cw* p) {
  const double2 d = *reinterpret_cast<const double2*>(p);
  *p = cw(dw_from_double(d.x), dw_from_double(d.y));
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
// a cw amplitude goes back to memory as the complex128 it stands for
template <> __device__ __forceinline__ void stg_stream<cw>(cw* p, cw v) {
  __stcs(reinterpret_cast<double2*>(p), make_double2(dw_to_double(v.re), dw_to_double(v.im)));
}

// ------------------------------------------------------------ shared-memory tile
// element e of a tile sits at e + e/16 + e/256: one padding slot per 16 elements and
// one more per 256.  The map is additive over disjoint bits (a thread's base plus a
// register's offset), and tile bits 0-3, 4-7 and 8-11 weigh 1, 2, 4, 8 modulo the 16
// eight-byte bank slots, so a warp whose lanes take one bit of each weight class spreads
// its accesses over all banks (the pass generator picks such lane bits per phase).
__host__ __device__ __forceinline__ int smem_pos(int e) { return e + (e >> 4) + (e >> 8); }
// elements of shared memory one tile of `tsize` amplitudes occupies
__host__ __device__ __forceinline__ int tile_stride(int tsize) { return tsize + (tsize >> 4) + (tsize >> 8); }

// ------------------------------------------------------------------ cp.async
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gmem_src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  if constexpr (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem_src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ---------------------------------------------------------------- register ops
template <typename T, int U>
__device__ __forceinline__ void dense1_regs(T (&v)[16], const T* __restrict__ m, unsigned jm) {
  const T a = m[0], b = m[1], c = m[2], d = m[3];
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & (1 << U)) continue;
    if (!((jm >> j) & 1u)) continue;
    const int k = j | (1 << U);
    const T x = v[j], y = v[k];
    v[j] = tfma(a, x, tmul(b, y));
    v[k] = tfma(c, x, tmul(d, y));
  }
}

template <typename T, int U0, int U1>
__device__ __forceinline__ void dense2_regs(T (&v)[16], const T* __restrict__ m, unsigned jm) {
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & ((1 << U0) | (1 << U1))) continue;
    if (!((jm >> j) & 1u)) continue;
    const int i1 = j | (1 << U1), i2 = j | (1 << U0), i3 = j | (1 << U0) | (1 << U1);
    const T x0 = v[j], x1 = v[i1], x2 = v[i2], x3 = v[i3];
    T o[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      T acc = tmul(m[4 * r + 3], x3);
      acc = tfma(m[4 * r + 2], x2, acc);
      acc = tfma(m[4 * r + 1], x1, acc);
      o[r] = tfma(m[4 * r + 0], x0, acc);
    }
    v[j] = o[0];
    v[i1] = o[1];
    v[i2] = o[2];
    v[i3] = o[3];
  }
}

template <typename T, int U>
__device__ __forceinline__ void x1_regs(T (&v)[16], unsigned jm) {
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & (1 << U)) continue;
    if (!((jm >> j) & 1u)) continue;
    const T t = v[j];
    v[j] = v[j | (1 << U)];
    v[j | (1 << U)] = t;
  }
}

// real 2x2 on complex amplitudes: coefficients' imaginary parts are zero
template <typename T, int U>
__device__ __forceinline__ void dense1r_regs(T (&v)[16], const T* __restrict__ m, unsigned jm) {
  if constexpr (is_complex<T>::value) {
    const auto a = m[0].re, b = m[1].re, c = m[2].re, d = m[3].re;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      if (j & (1 << U)) continue;
      if (!((jm >> j) & 1u)) continue;
      const int k = j | (1 << U);
      const T x = v[j], y = v[k];
      v[j].re = rfma(a, x.re, b * y.re);
      v[j].im = rfma(a, x.im, b * y.im);
      v[k].re = rfma(c, x.re, d * y.re);
      v[k].im = rfma(c, x.im, d * y.im);
    }
  }
}

// real 2x2 with a unit entry in each row (the row scale folded into a diagonal):
// out_i = v_unit + r_i * v_other, one multiply-add per component; FORM bit i is the
// column of row i's unit entry
template <typename T>
__device__ __forceinline__ T axpy_real(typename real_of<T>::type r, T x, T y) {  // r * x + y
  if constexpr (is_complex<T>::value) return T{rfma(r, x.re, y.re), rfma(r, x.im, y.im)};
  else return rfma(r, x, y);
}
template <typename T, int U, int FORM>
__device__ __forceinline__ void pivot1_regs(T (&v)[16], const T* __restrict__ m, unsigned jm) {
  typename real_of<T>::type r0, r1;
  if constexpr (is_complex<T>::value) {
    r0 = m[0].re;
    r1 = m[1].re;
  } else {
    r0 = m[0];
    r1 = m[1];
  }
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & (1 << U)) continue;
    if (!((jm >> j) & 1u)) continue;
    const int k = j | (1 << U);
    const T x = v[j], y = v[k];
    v[j] = (FORM & 1) ? axpy_real(r0, x, y) : axpy_real(r0, y, x);
    v[k] = (FORM & 2) ? axpy_real(r1, x, y) : axpy_real(r1, y, x);
  }
}

template <typename T, int U0, int U1>
__device__ __forceinline__ void swap2_regs(T (&v)[16], unsigned jm) {
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & ((1 << U0) | (1 << U1))) continue;
    if (!((jm >> j) & 1u)) continue;
    const T t = v[j | (1 << U1)];
    v[j | (1 << U1)] = v[j | (1 << U0)];
    v[j | (1 << U0)] = t;
  }
}

template <typename T>
__device__ __forceinline__ void apply_negations(T (&v)[16], unsigned nm) {
#pragma unroll
  for (int j = 0; j < 16; j++)
    if ((nm >> j) & 1u) v[j] = tneg(v[j]);
}

// adjoint gradients: products in the state's own precision (FP32 for complex64, FP64
// for complex128); the callers sum warps and blocks in FP64
template <typename T>
__device__ __forceinline__ typename real_of<T>::type im_cdot(T a, T b) {  // Im(conj(a) b)
  if constexpr (is_complex<T>::value) return a.re * b.im - a.im * b.re;
  else return 0;
}
template <typename T>
__device__ __forceinline__ typename real_of<T>::type re_cdot(T a, T b) {  // Re(conj(a) b)
  if constexpr (is_complex<T>::value) return a.re * b.re + a.im * b.im;
  else return a * b;
}
// Im <w| G |v> over the register pairs of bit U for the generator G = X (GEN 1) or
// Y (GEN 2): the derivative of exp(-i t G / 2) is -i G / 2 times it
template <typename T, int U, int GEN>
__device__ __forceinline__ typename real_of<T>::type grad_pairs(const T (&v)[16], const T (&w)[16]) {
  typename real_of<T>::type acc = 0;
#pragma unroll
  for (int j = 0; j < 16; j++) {
    if (j & (1 << U)) continue;
    const int k = j | (1 << U);
    if (GEN == 1) acc += im_cdot(w[j], v[k]) + im_cdot(w[k], v[j]);   // X
    else acc += re_cdot(w[k], v[j]) - re_cdot(w[j], v[k]);            // Y
  }
  return acc;
}
// the same for G = Z: amplitude j counts with sign -1 when its target bit is set, that
// bit being bit j of `bits` (a register bit) or `tbit` for every j (a bit outside them)
template <typename T>
__device__ __forceinline__ typename real_of<T>::type grad_z(const T (&v)[16], const T (&w)[16], unsigned bits,
                                                           int tbit) {
  typename real_of<T>::type acc = 0;
#pragma unroll
  for (int j = 0; j < 16; j++) {
    const auto x = im_cdot(w[j], v[j]);
    acc += ((int)((bits >> j) & 1u) | tbit) ? -x : x;
  }
  return acc;
}

}  // namespace sv
