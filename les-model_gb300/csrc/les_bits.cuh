// les_bits.cuh -- FP64 <-> FP32 conversions as integer operations on the
// IEEE 754 bit patterns (binary64: 1 sign, 11 exponent bits biased by 1023,
// 52 fraction bits; binary32: 1, 8 biased by 127, 23).
//
// GB300 runs FP64 instructions, conversions included, at about 2 per SM and
// clock; the FP32 physics kernels convert every FP64 value they load, so they
// do it on the integer pipe instead.  Host-compilable (the CPU tests check
// the functions against IEEE round-to-nearest-even conversion).
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define LES_BITS_FN __host__ __device__ __forceinline__
#else
#define LES_BITS_FN inline
#endif

LES_BITS_FN uint64_t les_bits64(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, sizeof b);
    return b;
#endif
}

LES_BITS_FN double les_from_bits64(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
#endif
}

LES_BITS_FN uint32_t les_bits32(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
#endif
}

LES_BITS_FN float les_from_bits32(uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
#endif
}

// double -> float, rounded to nearest (ties to even).  Magnitudes below the
// FP32 normal range (2^-126) give a zero of the same sign; magnitudes that
// round past FP32's largest finite value give infinity; NaN stays NaN.
LES_BITS_FN float d2f_bits(double d)
{
    const uint64_t b = les_bits64(d);
    const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - (1023 - 127);   // binary32 exponent field
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);     // top 23 fraction bits
    const uint32_t rest = lo & 0x1fffffffu;                      // the 29 bits rounded off
    uint32_t f = ((uint32_t)e << 23) + m;                        // a carry out of m raises the exponent
    f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    if (e <= 0) f = 0u;
    if (e >= 255) f = 0x7f800000u;   // overflow -> infinity
    if (((hi >> 20) & 0x7ffu) == 0x7ffu) f = 0x7f800000u | (((hi & 0xfffffu) | lo) ? 0x400000u : 0u);
    return les_from_bits32((hi & 0x80000000u) | f);
}

// float -> double, exact for normal numbers, zeros, infinities and NaN;
// FP32 subnormals give a zero of the same sign.
LES_BITS_FN double f2d_bits(float x)
{
    const uint32_t u = les_bits32(x);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint32_t E = e == 0xffu ? 0x7ffu : e + (1023 - 127);
    const uint32_t hi = (u & 0x80000000u) | (e ? (E << 20) | ((u & 0x7fffffu) >> 3) : 0u);
    const uint32_t lo = e ? (u << 29) : 0u;
    return les_from_bits64(((uint64_t)hi << 32) | lo);
}
