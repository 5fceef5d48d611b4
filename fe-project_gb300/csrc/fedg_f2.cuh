// fedg_f2.cuh -- unevaluated float pairs (hi + lo, about 48 significant bits) for the parts of the
// mixed-precision path that need more than FP32 but run on the FP32 pipe.
//
// The FP64 pipe of this part retires about 2 thread-operations per cycle per SM against 128
// for FP32 FMA.  A float pair built from error-free transformations costs 3 to 12 FP32
// instructions per operation:
//   - Knuth's two-sum;
//   - Dekker's fast two-sum;
//   - the FMA-based exact product.
// It is therefore several times cheaper than the FP64 instruction it replaces, at a relative
// precision of about 2^-47.  The intrinsics __fadd_rn/__fmul_rn/__fmaf_rn keep the compiler
// from contracting or reassociating the error terms.
#pragma once
#include <cuda_runtime.h>

namespace fedg {

struct f2 {
  float h, l;
};

__device__ __forceinline__ f2 f2_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ f2 f2_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  const f2 s = f2_two_sum(a.h, b.h);
  return f2_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ f2 f2_neg(f2 a) { return {-a.h, -a.l}; }
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) { return f2_add(a, f2_neg(b)); }
__device__ __forceinline__ f2 f2_add_f(f2 a, float b) {
  const f2 s = f2_two_sum(a.h, b);
  return f2_fast_two_sum(s.h, __fadd_rn(s.l, a.l));
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return f2_fast_two_sum(p, e);
}
__device__ __forceinline__ f2 f2_mul_f(f2 a, float b) {
  const float p = __fmul_rn(a.h, b);
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return f2_fast_two_sum(p, e);
}
// 1/d: the FP32 estimate y refined by one Newton step carried in pairs (y + y (1 - d y))
__device__ __forceinline__ f2 f2_recip(f2 d) {
  const float y = __fdividef(1.f, d.h);
  const f2 t = f2_mul_f(d, y);  // ~1
  const float e = __fsub_rn(__fsub_rn(1.f, t.h), t.l);
  return f2_fast_two_sum(y, __fmul_rn(y, e));
}
__device__ __forceinline__ float f2_to_f(f2 a) { return __fadd_rn(a.h, a.l); }
__device__ __forceinline__ f2 f2_of(float2 v) { return {v.x, v.y}; }
__device__ __forceinline__ float2 f2_pack(f2 a) { return make_float2(a.h, a.l); }

// Compensated dot-product accumulator: sum of exact products of pairs, the leading sum kept
// exact by two-sum and every rounding error collected in c.
struct f2acc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(f2 d, f2 x) {
    const float p = __fmul_rn(d.h, x.h);
    float e = __fmaf_rn(d.h, x.h, -p);
    e = __fmaf_rn(d.h, x.l, e);
    e = __fmaf_rn(d.l, x.h, e);
    const f2 t = f2_two_sum(s, p);
    s = t.h;
    c = __fadd_rn(c, __fadd_rn(t.l, e));
  }
  __device__ __forceinline__ f2 get() const { return f2_fast_two_sum(s, c); }
};

// Split of an FP64 value into a pair with integer instructions only: hi is x truncated to 24
// significant bits, lo the remaining 29 bits rounded to a float.  Zero, values below the
// smallest normal float (|x| < 2^-126) and values whose remainder would be subnormal
// (|x| < 2^-75, remainder dropped) give a zero or single-float pair.  Infinities and NaN give
// an infinite or NaN hi.
__device__ __forceinline__ f2 f2_split(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const unsigned sgn = hi32 & 0x80000000u;
  const int ex = (int)((hi32 >> 20) & 0x7ffu);
  const int fe = ex - 1023 + 127;
  const unsigned m23 = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
  unsigned hb;
  if (ex == 0x7ff) hb = sgn | 0x7f800000u | (((hi32 & 0xfffffu) | lo32) ? 0x400000u : 0u);
  else if (fe >= 255) hb = sgn | 0x7f800000u;
  else if (fe <= 0) hb = sgn;
  else hb = sgn | ((unsigned)fe << 23) | m23;
  float lo = 0.f;
  const int se = ex - 1075 + 127;  // exponent of the remainder's unit bit
  if (fe > 0 && fe < 255 && se > 0) {
    lo = __fmul_rn(__uint2float_rn(lo32 & 0x1fffffffu), __uint_as_float((unsigned)se << 23));
    if (sgn) lo = -lo;
  }
  return {__uint_as_float(hb), lo};
}

}  // namespace fedg
