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

// Round hi + lo to the nearest double (ties to even). After a Fast2Sum the pair (s, e) has
// |e| <= ulp(s)/2; the double of s is exact and e only touches the 29 mantissa bits below
// s's FP32 precision, so the result is an integer add/subtract on the bit pattern.
#ifdef __CUDA_ARCH__
__device__ __noinline__ double pair_to_double(float hi, float lo);
#endif
// (kept out of line on the device: the rare paths of pair_to_double_fast call it, and a call
// cannot be turned into predicated FP64 instructions on the common path)
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
__host__ __forceinline__
#endif
double pair_to_double(float hi, float lo) {
    const float s = hi + lo;
    const float e = lo - (s - hi);
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

// Same result as pair_to_double, fewer operations: the low word, scaled by a power of two
// to units of the double's last place, is rounded to an integer (ties to even) and added to
// the bit pattern of double(s). |e| <= ulp_f(s)/2 keeps that integer within +-2^28.
__host__ __device__ __forceinline__ double pair_to_double_fast(float hi, float lo) {
    const float s = hi + lo;
    const float e = lo - (s - hi);
    const uint32_t bs = f2u(s);
    const uint32_t mag = bs & 0x7FFFFFFFu;
    const uint32_t es = mag >> 23;
    if (es < 60u || es == 0xFFu) return pair_to_double(hi, lo);  // tiny / subnormal / inf: rare
    // double(s): same sign, exponent rebased by 1023-127, mantissa shifted up by 29
    const uint32_t dhi = (bs & 0x80000000u) | ((mag >> 3) + (896u << 20));
    const uint32_t dlo = mag << 29;
    // e in units of ulp(double(s)) = 2^(es-127-52); one more bit if s is a power of two and
    // e points into the binade below
    const bool down = ((bs ^ f2u(e)) & 0x80000000u) && (mag & 0x7FFFFFu) == 0u;
    const uint32_t sc = (uint32_t)(306 - (int)es + (down ? 1 : 0)) << 23;
    const int d = f2i_rn(e * u2f(sc));
    const uint64_t D = (((uint64_t)dhi << 32) | dlo) + (uint64_t)(int64_t)((bs & 0x80000000u) ? -d : d);
    return u2d(D);
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
