// Double-float ("df64") complex arithmetic on the FP32 pipes, packed two lanes wide.
//
// A df64 number is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2, about 48
// significant bits.  A complex df64 value keeps its real and imaginary parts side by side,
//   hi = (re_hi, im_hi),  lo = (re_lo, im_lo),
// so every step of the error-free transformations acts on both parts with one packed FP32x2
// instruction (__fadd2_rn / __fmul2_rn / __ffma2_rn, sm_100 and later).
//
// Error-free transformations (Knuth's TwoSum, Dekker's Fast2Sum and the FMA form of Dekker's
// TwoProduct, as in Dekker 1971 and Shewchuk 1997):
//   two_sum(a, b):   s = a + b, t = s - a, e = (a - (s - t)) + (b - t)       a + b = s + e exactly
//   fast_two_sum:    s = a + b, e = b - (s - a)                             needs |a| >= |b|
//   two_prod(a, b):  p = a * b, e = fma(a, b, -p)                           a * b = p + e exactly
// The df64 sum adds the low parts to the TwoSum error before renormalising ("sloppy" sum): its
// error is bounded relative to |a| + |b|, which is what an FFT's error analysis needs.  Every
// operation is an explicit round-to-nearest intrinsic, so the compiler can neither contract nor
// reassociate them; subnormals are kept (no flush-to-zero in this build).
#pragma once
#include <cuda_runtime.h>

namespace fdfk {
namespace df64 {

struct C {
    float2 hi, lo;
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b, exactly rounded once (fma(b, -1, a))
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float2 a, float2 b, float2& s, float2& e)
{
    s = add(a, b);
    const float2 t = sub(s, a);
    e = add(sub(a, sub(s, t)), sub(b, t));
}

// (s, e) renormalised: hi + lo = s + e with |lo| <= ulp(hi)/2 (|s| >= |e| per lane)
__device__ __forceinline__ C renorm(float2 s, float2 e)
{
    C r;
    r.hi = add(s, e);
    r.lo = sub(e, sub(r.hi, s));
    return r;
}

__device__ __forceinline__ C zero()
{
    C r;
    r.hi = f2(0.f, 0.f);
    r.lo = f2(0.f, 0.f);
    return r;
}

__device__ __forceinline__ C cadd(const C& a, const C& b)
{
    float2 s, e;
    two_sum(a.hi, b.hi, s, e);
    e = add(add(e, a.lo), b.lo);
    return renorm(s, e);
}

__device__ __forceinline__ C csub(const C& a, const C& b)
{
    float2 s, e;
    two_sum(a.hi, f2(-b.hi.x, -b.hi.y), s, e);
    e = add(sub(e, b.lo), a.lo);
    return renorm(s, e);
}

// complex product: re = ar br - ai bi, im = ar bi + ai br, as (ar br, ar bi) + (-ai bi, ai br)
__device__ __forceinline__ C cmul(const C& a, const C& b)
{
    const float2 ar = f2(a.hi.x, a.hi.x), arl = f2(a.lo.x, a.lo.x);
    const float2 ai = f2(a.hi.y, a.hi.y), ail = f2(a.lo.y, a.lo.y);
    const float2 bsh = f2(-b.hi.y, b.hi.x), bsl = f2(-b.lo.y, b.lo.x);
    const float2 ph = mul(ar, b.hi);
    float2 pe = fma(ar, b.hi, f2(-ph.x, -ph.y));
    pe = fma(ar, b.lo, pe);
    pe = fma(arl, b.hi, pe);
    const float2 qh = mul(ai, bsh);
    float2 qe = fma(ai, bsh, f2(-qh.x, -qh.y));
    qe = fma(ai, bsl, qe);
    qe = fma(ail, bsh, qe);
    float2 s, e;
    two_sum(ph, qh, s, e);
    e = add(add(e, pe), qe);
    return renorm(s, e);
}

// (re, im) times the df64 real r = (rh, rl)
__device__ __forceinline__ C cscale(const C& a, float rh, float rl)
{
    const float2 r = f2(rh, rh), q = f2(rl, rl);
    const float2 ph = mul(a.hi, r);
    float2 pe = fma(a.hi, r, f2(-ph.x, -ph.y));
    pe = fma(a.lo, r, pe);
    pe = fma(a.hi, q, pe);
    return renorm(ph, pe);
}

__device__ __forceinline__ C conj(const C& a)
{
    C r;
    r.hi = f2(a.hi.x, -a.hi.y);
    r.lo = f2(a.lo.x, -a.lo.y);
    return r;
}

// i * a
__device__ __forceinline__ C times_i(const C& a)
{
    C r;
    r.hi = f2(-a.hi.y, a.hi.x);
    r.lo = f2(-a.lo.y, a.lo.x);
    return r;
}

__device__ __forceinline__ float4 pack(const C& a) { return make_float4(a.hi.x, a.hi.y, a.lo.x, a.lo.y); }
__device__ __forceinline__ C unpack(const float4& v)
{
    C r;
    r.hi = f2(v.x, v.y);
    r.lo = f2(v.z, v.w);
    return r;
}

// df64 split of a double: hi = nearest float, lo = nearest float to the remainder
__host__ __device__ __forceinline__ void split(double d, float& hi, float& lo)
{
    hi = (float)d;
    lo = (float)(d - (double)hi);
}

__device__ __forceinline__ float4 from_double(double re, double im)
{
    float rh, rl, ih, il;
    split(re, rh, rl);
    split(im, ih, il);
    return make_float4(rh, ih, rl, il);
}

__device__ __forceinline__ double re_double(const C& a) { return (double)a.hi.x + (double)a.lo.x; }
__device__ __forceinline__ double im_double(const C& a) { return (double)a.hi.y + (double)a.lo.y; }

}  // namespace df64
}  // namespace fdfk
