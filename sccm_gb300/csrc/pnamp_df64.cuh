// Double-float arithmetic: a value is the unevaluated sum hi + lo of two
// floats (|lo| <= ulp(hi)/2), about 48 significant bits. GB300 issues FP32
// FMAs at ~60x its FP64 rate, so the O(n^3) per-point algebra in this form
// runs on the FP32 pipes. Algorithms: Knuth's TwoSum, Dekker's FastTwoSum and
// the FMA-based TwoProduct (exact product error), combined as in the
// double-double literature (Hida, Li, Bailey, "Algorithms for quad-double
// precision floating point arithmetic", 2001) one level down.
// The _rn intrinsics keep the compiler from contracting or reassociating the
// error-free transformations.
#pragma once
#include <cuda_runtime.h>

#include "pnamp_device.cuh"

namespace pnamp {

struct dd {
    float hi, lo;
};

struct __align__(16) zd {
    dd x, y;
};

__device__ __forceinline__ dd dd_make(float h, float l) {
    dd r;
    r.hi = h;
    r.lo = l;
    return r;
}
__device__ __forceinline__ dd two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float v = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
    return dd_make(s, e);
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ dd quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return dd_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dd dd_add(dd a, dd b) {
    const dd s = two_sum(a.hi, b.hi);
    return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd dd_neg(dd a) { return dd_make(-a.hi, -a.lo); }
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}
// a * b + c
__device__ __forceinline__ dd dd_fma(dd a, dd b, dd c) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const dd s = two_sum(p, c.hi);
    return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}
// 1 / b: float reciprocal refined by one Newton step with a double-float residual
__device__ __forceinline__ dd dd_recip(dd b) {
    const float q = __frcp_rn(b.hi);
    const dd r = dd_fma(dd_neg(b), dd_make(q, 0.0f), dd_make(1.0f, 0.0f));
    return quick_two_sum(q, __fmul_rn(r.hi, q));
}
__device__ __forceinline__ dd dd_from(double x) {
    const float h = __double2float_rn(x);
    return dd_make(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ double dd_to(dd a) { return (double)a.hi + (double)a.lo; }

// ------------------------------------------------------------------ complex
__device__ __forceinline__ zd mkd(dd a, dd b) {
    zd r;
    r.x = a;
    r.y = b;
    return r;
}
__device__ __forceinline__ zd operator+(zd a, zd b) { return mkd(dd_add(a.x, b.x), dd_add(a.y, b.y)); }
__device__ __forceinline__ zd operator-(zd a) { return mkd(dd_neg(a.x), dd_neg(a.y)); }
__device__ __forceinline__ zd operator-(zd a, zd b) { return a + (-b); }
__device__ __forceinline__ zd operator*(zd a, zd b) {
    return mkd(dd_fma(a.x, b.x, dd_neg(dd_mul(a.y, b.y))), dd_fma(a.x, b.y, dd_mul(a.y, b.x)));
}
__device__ __forceinline__ zd operator*(dd s, zd a) { return mkd(dd_mul(s, a.x), dd_mul(s, a.y)); }
__device__ __forceinline__ zd zconj(zd a) { return mkd(a.x, dd_neg(a.y)); }
// c + a*b
__device__ __forceinline__ zd zfma(zd a, zd b, zd c) {
    return mkd(dd_fma(a.x, b.x, dd_fma(dd_neg(a.y), b.y, c.x)), dd_fma(a.x, b.y, dd_fma(a.y, b.x, c.y)));
}
// c - a*b
__device__ __forceinline__ zd zfms(zd a, zd b, zd c) {
    return mkd(dd_fma(dd_neg(a.x), b.x, dd_fma(a.y, b.y, c.x)),
               dd_fma(dd_neg(a.x), b.y, dd_fma(dd_neg(a.y), b.x, c.y)));
}
// c + r*a, r real
__device__ __forceinline__ zd rfma(dd r, zd a, zd c) { return mkd(dd_fma(r, a.x, c.x), dd_fma(r, a.y, c.y)); }
__device__ __forceinline__ zd zrecip(zd b) {
    const dd n2 = dd_fma(b.x, b.x, dd_mul(b.y, b.y));
    const dd inv = dd_recip(n2);
    return mkd(dd_mul(b.x, inv), dd_neg(dd_mul(b.y, inv)));
}
__device__ __forceinline__ bool zfinite(zd a) { return isfinite(a.x.hi) && isfinite(a.y.hi); }
__device__ __forceinline__ zd zd_from(zc a) { return mkd(dd_from(a.x), dd_from(a.y)); }
__device__ __forceinline__ zc zd_to(zd a) { return mk(dd_to(a.x), dd_to(a.y)); }

}  // namespace pnamp
