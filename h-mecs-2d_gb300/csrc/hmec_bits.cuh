// hmec_bits.cuh -- bit-pattern helpers: the FP32 -> FP64 widening on the
// integer pipe (the conversion instruction runs at the FP64 rate on this GPU;
// the marker gathers and the Arnoldi step widen millions of FP32 values per
// step).  Host-compilable as plain C++ (a CPU test compares it with the
// compiler's own conversion).
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define HMEC_HD __host__ __device__ __forceinline__
#else
#define HMEC_HD inline
#endif

HMEC_HD uint64_t hmec_bits_of(double d) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}
HMEC_HD double hmec_double_of(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}
HMEC_HD uint32_t hmec_bits_of(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
HMEC_HD float hmec_float_of(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}

// FP32 -> FP64: exact for normal values, infinities and NaN; FP32
// subnormals (below 1.2e-38) give 0.
HMEC_HD double f2d_bits(float f) {
    const uint32_t u = hmec_bits_of(f);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e == 0) return 0.0;
    if (e == 0xFFu) return (double)f;
    const uint64_t b = ((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                       ((uint64_t)(u & 0x7FFFFFu) << 29);
    return hmec_double_of(b);
}
