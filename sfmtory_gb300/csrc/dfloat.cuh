// Double-float arithmetic for the FP32 path's cost evaluation.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2: about 48 significant bits, carried on the FP32 pipe
// (GB300 issues FP32 at 64x its FP64 rate). The error-free transformations
// are Knuth's TwoSum, Dekker's FastTwoSum and the FMA form of Dekker's
// exact product; the operations on pairs follow the double-double
// algorithms of Hida, Li and Bailey ("Library for double-double and
// quad-double arithmetic", 2000: accurate addition, product with FMA,
// division by one Newton correction of the leading quotient), restated
// here for float pairs. Each operation has a relative error of a few
// 2^-48; the cost's projection chain (~40 operations) stays ~1e-12 relative
// on the pixel coordinates.
#pragma once

#include <cuda_runtime.h>

#if !defined(__CUDA_ARCH__)
#include <cmath>
#endif

namespace sfmba {

// Correctly rounded single operations: the CUDA intrinsics on the device
// (never contracted into an FMA); on the host (the arithmetic's CPU test)
// plain IEEE single operations, built without FP contraction.
#if defined(__CUDA_ARCH__)
#define SFMBA_DF_ADD(a, b) __fadd_rn(a, b)
#define SFMBA_DF_SUB(a, b) __fsub_rn(a, b)
#define SFMBA_DF_MUL(a, b) __fmul_rn(a, b)
#define SFMBA_DF_FMA(a, b, c) __fmaf_rn(a, b, c)
#define SFMBA_DF_RCP(a) __frcp_rn(a)
#define SFMBA_DF_D2F(x) __double2float_rn(x)
#else
#define SFMBA_DF_ADD(a, b) ((float)((a) + (b)))
#define SFMBA_DF_SUB(a, b) ((float)((a) - (b)))
#define SFMBA_DF_MUL(a, b) ((float)((a) * (b)))
#define SFMBA_DF_FMA(a, b, c) std::fmaf(a, b, c)
#define SFMBA_DF_RCP(a) (1.0f / (a))
#define SFMBA_DF_D2F(x) ((float)(x))
#endif

struct dfl {
    float hi, lo;
};

__host__ __device__ __forceinline__ dfl df_make(float h) { return {h, 0.f}; }

// Split of an FP64 value: hi = nearest float, lo = nearest float of the rest.
__host__ __device__ __forceinline__ dfl df_from(double x) {
    const float h = SFMBA_DF_D2F(x);
    return {h, SFMBA_DF_D2F(x - (double)h)};
}

__host__ __device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// |a| >= |b| or a == 0: s + e == a + b exactly (Dekker).
__host__ __device__ __forceinline__ dfl fast_two_sum(float a, float b) {
    const float s = SFMBA_DF_ADD(a, b);
    return {s, SFMBA_DF_SUB(b, SFMBA_DF_SUB(s, a))};
}

// s + e == a + b exactly for any a, b (Knuth).
__host__ __device__ __forceinline__ dfl two_sum(float a, float b) {
    const float s = SFMBA_DF_ADD(a, b);
    const float bb = SFMBA_DF_SUB(s, a);
    return {s, SFMBA_DF_ADD(SFMBA_DF_SUB(a, SFMBA_DF_SUB(s, bb)), SFMBA_DF_SUB(b, bb))};
}

// p + e == a * b exactly (the FMA gives the product's rounding error).
__host__ __device__ __forceinline__ dfl two_prod(float a, float b) {
    const float p = SFMBA_DF_MUL(a, b);
    return {p, SFMBA_DF_FMA(a, b, -p)};
}

__host__ __device__ __forceinline__ dfl operator+(dfl a, dfl b) {
    dfl s = two_sum(a.hi, b.hi);
    const dfl t = two_sum(a.lo, b.lo);
    s.lo = SFMBA_DF_ADD(s.lo, t.hi);
    s = fast_two_sum(s.hi, s.lo);
    s.lo = SFMBA_DF_ADD(s.lo, t.lo);
    return fast_two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ dfl operator-(dfl a) { return {-a.hi, -a.lo}; }
__host__ __device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }

__host__ __device__ __forceinline__ dfl operator*(dfl a, dfl b) {
    dfl p = two_prod(a.hi, b.hi);
    p.lo = SFMBA_DF_FMA(a.hi, b.lo, p.lo);
    p.lo = SFMBA_DF_FMA(a.lo, b.hi, p.lo);
    return fast_two_sum(p.hi, p.lo);
}

// Exact scaling by a power of two.
__host__ __device__ __forceinline__ dfl df_scale2(dfl a, float two_pow) { return {a.hi * two_pow, a.lo * two_pow}; }

// 1 / a: q1 = the float quotient, then the remainder 1 - a q1 in pair
// arithmetic corrects it to a pair.
__host__ __device__ __forceinline__ dfl df_recip(dfl a) {
    const float q1 = SFMBA_DF_RCP(a.hi);
    const dfl r = df_make(1.f) - a * df_make(q1);
    const float q2 = SFMBA_DF_MUL(r.hi, q1);
    return fast_two_sum(q1, q2);
}

}  // namespace sfmba
