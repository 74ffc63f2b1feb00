// dfloat.h -- compensated FP32 pairs (hi, lo) as the nzval accumulator, and their exact
// rounding to FP64 with integer operations (GB300's FP64 pipe is a small fraction of its
// FP32 rate, so the write-out path avoids it). Host+device so it is unit-tested on the CPU.
#pragma once
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
__host__ __device__ __forceinline__ double pair_to_double(float hi, float lo) {
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

}  // namespace fe
