// dfloat.h -- compensated FP32 pairs (hi, lo) as the nzval accumulator, and their exact
// rounding to FP64 with integer operations (GB300's FP64 pipe is a small fraction of its
// FP32 rate, so the write-out path avoids it). Host+device so it is unit-tested on the CPU.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif

namespace fe {

__host__ __device__ __forceinline__ uint32_t f2u(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ double u2d(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}

// Round hi + lo to the nearest double (ties to even). After a TwoSum the pair (s, e) has
// |e| <= ulp(s)/2; the double of s is exact and e only touches the 29 mantissa bits below
// s's FP32 precision, so the result is an integer add/subtract on the bit pattern.
#ifdef __CUDA_ARCH__
__device__ __noinline__ double pair_to_double(float hi, float lo);
#endif
// (kept out of line on the device: the kernels call it only for the rare sums that
// pair2_to_double / pair1_to_double flag)
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
__host__ __forceinline__
#endif
double pair_to_double(float hi, float lo) {
    const float s = hi + lo;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (lo - bb);  // TwoSum: exact for any magnitudes
    if (s == 0.0f) return 0.0;
    const uint32_t bs = f2u(s), be = f2u(e);
    const uint32_t es = (bs >> 23) & 0xFF, ee = (be >> 23) & 0xFF;
    if (es == 0 || es == 0xFF || (e != 0.0f && ee == 0)) return (double)s + (double)e;  // subnormal / inf: rare
    const uint32_t ms = bs & 0x7FFFFF;
    uint64_t D = ((uint64_t)(bs >> 31) << 63) | ((uint64_t)(es + 896) << 52) | ((uint64_t)ms << 29);
    if (e == 0.0f) return u2d(D);
    const bool same = ((bs ^ be) >> 31) == 0;
    const uint32_t Me = (be & 0x7FFFFF) | 0x800000;
    int shift = (int)ee - (int)es + 29;  // |e| / ulp(double(s)) = Me * 2^shift, shift <= 5
    if (!same && ms == 0) shift += 1;    // s - |e| lies in the binade below: half the ulp
    uint64_t delta;
    if (shift >= 0) {
        delta = (uint64_t)Me << shift;
    } else if (shift > -26) {
        const int r = -shift;
        const uint64_t q = (uint64_t)Me >> r;
        const uint64_t rem = (uint64_t)Me & ((1ull << r) - 1);
        const uint64_t half = 1ull << (r - 1);
        delta = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    } else {
        delta = 0;
    }
    D = same ? D + delta : D - delta;
    return u2d(D);
}

__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
__host__ __device__ __forceinline__ int f2i_rn(float x) {
#ifdef __CUDA_ARCH__
    return __float2int_rn(x);
#else
    return (int)lrintf(x);
#endif
}

// packed FP32 helpers (FADD2 / FFMA2 / FMUL2 on the device)
#if !defined(__CUDACC__) && !defined(__VECTOR_TYPES_H__)
struct float2 {
    float x, y;
};
#endif
__host__ __device__ __forceinline__ float2 f2add(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fadd2_rn(a, b);
#else
    return float2{a.x + b.x, a.y + b.y};
#endif
}
__host__ __device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#else
    return float2{a.x - b.x, a.y - b.y};
#endif
}
__host__ __device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
    return __fmul2_rn(a, b);
#else
    return float2{a.x * b.x, a.y * b.y};
#endif
}
// bit pattern of double(s) plus d units of its last place (|d| < 2^29)
__host__ __device__ __forceinline__ uint64_t scaled_low_word_add(uint32_t bs, int d) {
    const uint32_t mag = bs & 0x7FFFFFFFu;
    const uint32_t dhi = (bs & 0x80000000u) | ((mag >> 3) + (896u << 20));
    const uint32_t dlo = mag << 29;
    return (((uint64_t)dhi << 32) | dlo) + (uint64_t)(int64_t)d;
}
// s zero or below 2^-67, infinite or NaN, or a power of two
__host__ __device__ __forceinline__ bool sum_needs_care(uint32_t bs) {
    const uint32_t mag = bs & 0x7FFFFFFFu;
    return (mag - (60u << 23)) >= (195u << 23) || (mag & 0x7FFFFFu) == 0u;
}
// Two entries at once, without a branch: o0, o1 = hi + lo rounded to the nearest double (ties
// to even), exactly as pair_to_double, unless an entry's sum s needs care. `rare` is set for
// those (s zero, below 2^-67, infinite or NaN, or a power of two, whose low word may point into
// the binade below) and the caller redoes them with pair_to_double. The TwoSum renormalisation
// runs packed on both entries (any magnitudes of hi and lo); the low word e, scaled by a power
// of two that carries the sign of s to units of the double's last place, is rounded to an
// integer (|e| <= ulp_f(s)/2 keeps it within +-2^28) and added to the bit pattern of double(s).
__host__ __device__ __forceinline__ void pair2_to_double(float2 hi, float2 lo, double& o0, double& o1, bool& rare) {
    const float2 s = f2add(hi, lo);
    const float2 bb = f2sub(s, hi);
    const float2 e = f2add(f2sub(hi, f2sub(s, bb)), f2sub(lo, bb));
    const uint32_t b0 = f2u(s.x), b1 = f2u(s.y);
    // 2^(179 - exponent(s)) with the sign of s: (306 << 23) - (sign | exponent field), mod 2^32
    const float2 sc = float2{u2f((306u << 23) - (b0 & 0xFF800000u)), u2f((306u << 23) - (b1 & 0xFF800000u))};
    const float2 q = f2mul(e, sc);
    o0 = u2d(scaled_low_word_add(b0, f2i_rn(q.x)));
    o1 = u2d(scaled_low_word_add(b1, f2i_rn(q.y)));
    rare |= sum_needs_care(b0) | sum_needs_care(b1);
}

// One entry, the same way (scalar TwoSum)
__host__ __device__ __forceinline__ double pair1_to_double(float hi, float lo, bool& rare) {
    const float s = hi + lo;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (lo - bb);
    const uint32_t b = f2u(s);
    rare |= sum_needs_care(b);
    return u2d(scaled_low_word_add(b, f2i_rn(e * u2f((306u << 23) - (b & 0xFF800000u)))));
}

__host__ __device__ __forceinline__ int clz32(uint32_t x) {  // x != 0
#ifdef __CUDA_ARCH__
    return __clz((int)x);
#else
    return __builtin_clz(x);
#endif
}

// Exact FP32 -> FP64 with integer operations only (GB300's FP64 pipe, which also runs the
// F2F conversion, issues at a small fraction of the integer rate). Every class is handled
// without it: normal numbers by rebasing the exponent, zero and subnormals by normalising
// the mantissa, infinities and NaNs (payload kept) by widening the field.
__host__ __device__ __forceinline__ double float_to_double(float v) {
    const uint32_t b = f2u(v);
    const uint32_t sign = b & 0x80000000u;
    const uint32_t mag = b & 0x7FFFFFFFu;
    const uint32_t ex = mag >> 23;
    uint32_t hi = sign | ((mag >> 3) + (896u << 20));
    uint32_t lo = mag << 29;
    if (ex == 0u) {
        hi = sign;
        lo = 0u;
        if (mag) {  // subnormal: mag * 2^-149 with the leading bit at position p
            const int p = 31 - clz32(mag);
            const uint64_t D = ((uint64_t)(p + 874) << 52) | (((uint64_t)mag << (52 - p)) & 0xFFFFFFFFFFFFFull);
            hi = sign | (uint32_t)(D >> 32);
            lo = (uint32_t)D;
        }
    } else if (ex == 0xFFu) {
        hi = sign | 0x7FF00000u | ((mag & 0x7FFFFFu) >> 3);
    }
    return u2d(((uint64_t)hi << 32) | lo);
}

}  // namespace fe
