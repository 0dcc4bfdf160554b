// Number types of the device kernels: FP64 (double2), FP32 (float2) and FP32x2
// (pairs of FP32 numbers, float4 = re_hi, im_hi, re_lo, im_lo).
//
// FP32x2 arithmetic uses error-free transformations: the two-sum of Knuth (TAOCP
// vol. 2, 4.2.2) and the FMA-based exact product (p = a*b, e = fma(a, b, -p)),
// combined as in Dekker (Numer. Math. 18 (1971) 224) "double-length" arithmetic.
// A value is hi + lo, about 48 significant bits; all operations run on the FP32 pipe.
// Intermediate results are kept unnormalised (the sum and product skip the final
// renormalising fast-two-sum; the error terms collect in lo), and values are
// renormalised to |lo| <= ulp(hi)/2 when stored.  Over the few dozen operations of one
// apply this keeps the error near 2^-48 relative while cutting the instruction count
// of an add from 11 to 8 and of a product from 7 to 4.  The intrinsics __fadd_rn /
// __fmul_rn keep the compiler from contracting or reassociating the compensation terms.
#pragma once
#include <cuda_runtime.h>

namespace heom {

struct DF {};   // tag of the FP32x2 number type

template <typename T> struct Num;

template <> struct Num<double> {
    using V = double2;      // stored complex
    using A = double2;      // accumulator / arithmetic complex
    using S = double;       // real scalar used in arithmetic
    static __host__ __device__ __forceinline__ A load(const V &v) { return v; }
    static __host__ __device__ __forceinline__ V store(const A &a) { return a; }
    static __host__ __device__ __forceinline__ V store_host(const A &a) { return a; }
    static __device__ __forceinline__ V pack(const A &a) { return a; }
    static __device__ __forceinline__ A norm(A a) { return a; }
    static __host__ __device__ __forceinline__ A zero() { return make_double2(0, 0); }
    static __host__ __device__ __forceinline__ A from_d(double re, double im) { return make_double2(re, im); }
    static __device__ __forceinline__ A add(A a, A b) { return make_double2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ A sub(A a, A b) { return make_double2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ A mul(A a, A b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
    // a * (r real); sc converts an FP64 scalar once, outside element loops
    static __host__ __device__ __forceinline__ S sc(double r) { return r; }
    static __device__ __forceinline__ A scale(A a, S r) { return make_double2(a.x * r, a.y * r); }
    static __device__ __forceinline__ A half(A a) { return make_double2(0.5 * a.x, 0.5 * a.y); }
    static __device__ __forceinline__ S re_s(A a) { return a.x; }
    // i * a
    static __device__ __forceinline__ A mul_i(A a) { return make_double2(-a.y, a.x); }
    static __device__ __forceinline__ A neg(A a) { return make_double2(-a.x, -a.y); }
    static __device__ __forceinline__ A conj(A a) { return make_double2(a.x, -a.y); }
    // (-1)^ng a, conjugated when cj = 1 (ng, cj in {0, 1}): sign-bit flips, no branches
    static __device__ __forceinline__ A flip(A a, uint32_t ng, uint32_t cj)
    {
        const unsigned long long mr = (unsigned long long)ng << 63, mi = (unsigned long long)(ng ^ cj) << 63;
        return make_double2(__longlong_as_double(__double_as_longlong(a.x) ^ (long long)mr),
                            __longlong_as_double(__double_as_longlong(a.y) ^ (long long)mi));
    }
    static __device__ __forceinline__ double re(A a) { return a.x; }
    static __device__ __forceinline__ double im(A a) { return a.y; }
};

template <> struct Num<float> {
    using V = float2;
    using A = float2;
    using S = float;
    static __host__ __device__ __forceinline__ A load(const V &v) { return v; }
    static __host__ __device__ __forceinline__ V store(const A &a) { return a; }
    static __host__ __device__ __forceinline__ V store_host(const A &a) { return a; }
    static __device__ __forceinline__ V pack(const A &a) { return a; }
    static __device__ __forceinline__ A norm(A a) { return a; }
    static __host__ __device__ __forceinline__ A zero() { return make_float2(0, 0); }
    static __host__ __device__ __forceinline__ A from_d(double re, double im) { return make_float2((float)re, (float)im); }
    static __device__ __forceinline__ A add(A a, A b) { return make_float2(a.x + b.x, a.y + b.y); }
    static __device__ __forceinline__ A sub(A a, A b) { return make_float2(a.x - b.x, a.y - b.y); }
    static __device__ __forceinline__ A mul(A a, A b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
    static __host__ __device__ __forceinline__ S sc(double r) { return (float)r; }
    static __device__ __forceinline__ A scale(A a, S r) { return make_float2(a.x * r, a.y * r); }
    static __device__ __forceinline__ A half(A a) { return make_float2(0.5f * a.x, 0.5f * a.y); }
    static __device__ __forceinline__ S re_s(A a) { return a.x; }
    static __device__ __forceinline__ A mul_i(A a) { return make_float2(-a.y, a.x); }
    static __device__ __forceinline__ A neg(A a) { return make_float2(-a.x, -a.y); }
    static __device__ __forceinline__ A conj(A a) { return make_float2(a.x, -a.y); }
    static __device__ __forceinline__ A flip(A a, uint32_t ng, uint32_t cj)
    {
        const uint32_t mr = ng << 31, mi = (ng ^ cj) << 31;
        return make_float2(__uint_as_float(__float_as_uint(a.x) ^ mr), __uint_as_float(__float_as_uint(a.y) ^ mi));
    }
    static __device__ __forceinline__ double re(A a) { return a.x; }
    static __device__ __forceinline__ double im(A a) { return a.y; }
};

// ---- FP32x2 ----
struct f2r { float hi, lo; };   // real FP32x2
struct f2c { f2r re, im; };     // complex FP32x2

__host__ __device__ __forceinline__ f2r f2r_from_d(double d)
{
    float h = (float)d;
    return {h, (float)(d - (double)h)};
}
__device__ __forceinline__ f2r two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    float v = __fadd_rn(s, -a);
    float e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -v)), __fadd_rn(b, -v));
    return {s, e};
}
__device__ __forceinline__ f2r fast_two_sum(float a, float b)
{
    float s = __fadd_rn(a, b);
    return {s, __fadd_rn(b, -__fadd_rn(s, -a))};
}
// unnormalised sum: exact two-sum of the high parts, low parts and error added in FP32
__device__ __forceinline__ f2r f2r_add(f2r a, f2r b)
{
    f2r s = two_sum(a.hi, b.hi);
    return {s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ f2r f2r_neg(f2r a) { return {-a.hi, -a.lo}; }
// unnormalised product: exact product of the high parts plus the cross terms.  The lo x lo
// term is dropped, so at least one operand must be normalised (|lo| <= ulp(hi) / 2): a lazy
// sum after cancellation can carry |lo| >= |hi|, and its square would then lose its leading
// term (even turn negative).  Loaded values are normalised; lazy sums go through norm first.
__device__ __forceinline__ f2r f2r_mul(f2r a, f2r b)
{
    float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
}
// renormalise to |lo| <= ulp(hi)/2
__device__ __forceinline__ f2r f2r_norm(f2r a) { return two_sum(a.hi, a.lo); }

template <> struct Num<DF> {
    using V = float4;    // (re_hi, im_hi, re_lo, im_lo)
    using A = f2c;
    using S = f2r;
    static __host__ __device__ __forceinline__ A load(const V &v) { return {{v.x, v.z}, {v.y, v.w}}; }
    static __device__ __forceinline__ V store(const A &a)
    {
        const f2r r = f2r_norm(a.re), i = f2r_norm(a.im);
        return make_float4(r.hi, i.hi, r.lo, i.lo);
    }
    static __host__ __device__ __forceinline__ V store_host(const A &a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }
    // store of a value that is already normalised (the result of norm)
    static __device__ __forceinline__ V pack(const A &a) { return make_float4(a.re.hi, a.im.hi, a.re.lo, a.im.lo); }
    // renormalise an accumulator (keeps long sums near 2^-48 relative)
    static __device__ __forceinline__ A norm(A a) { return {two_sum(a.re.hi, a.re.lo), two_sum(a.im.hi, a.im.lo)}; }
    static __host__ __device__ __forceinline__ A zero() { return {{0.f, 0.f}, {0.f, 0.f}}; }
    static __host__ __device__ __forceinline__ A from_d(double re, double im) { return {f2r_from_d(re), f2r_from_d(im)}; }
    static __device__ __forceinline__ A add(A a, A b) { return {f2r_add(a.re, b.re), f2r_add(a.im, b.im)}; }
    static __device__ __forceinline__ A sub(A a, A b) { return {f2r_add(a.re, f2r_neg(b.re)), f2r_add(a.im, f2r_neg(b.im))}; }
    static __device__ __forceinline__ A mul(A a, A b)
    {
        return {f2r_add(f2r_mul(a.re, b.re), f2r_neg(f2r_mul(a.im, b.im))), f2r_add(f2r_mul(a.re, b.im), f2r_mul(a.im, b.re))};
    }
    static __host__ __device__ __forceinline__ S sc(double r) { return f2r_from_d(r); }
    static __device__ __forceinline__ A scale(A a, S r) { return {f2r_mul(a.re, r), f2r_mul(a.im, r)}; }
    // exact halving of both parts
    static __device__ __forceinline__ A half(A a)
    {
        return {{0.5f * a.re.hi, 0.5f * a.re.lo}, {0.5f * a.im.hi, 0.5f * a.im.lo}};
    }
    static __device__ __forceinline__ S re_s(A a) { return a.re; }
    static __device__ __forceinline__ A mul_i(A a) { return {f2r_neg(a.im), a.re}; }
    static __device__ __forceinline__ A neg(A a) { return {f2r_neg(a.re), f2r_neg(a.im)}; }
    static __device__ __forceinline__ A conj(A a) { return {a.re, f2r_neg(a.im)}; }
    static __device__ __forceinline__ A flip(A a, uint32_t ng, uint32_t cj)
    {
        const uint32_t mr = ng << 31, mi = (ng ^ cj) << 31;
        return {{__uint_as_float(__float_as_uint(a.re.hi) ^ mr), __uint_as_float(__float_as_uint(a.re.lo) ^ mr)},
                {__uint_as_float(__float_as_uint(a.im.hi) ^ mi), __uint_as_float(__float_as_uint(a.im.lo) ^ mi)}};
    }
    static __device__ __forceinline__ double re(A a) { return (double)a.re.hi + (double)a.re.lo; }
    static __device__ __forceinline__ double im(A a) { return (double)a.im.hi + (double)a.im.lo; }
};

}  // namespace heom
