// hmec_dfexp.cuh -- exp(x) as a double-float h + l (two FP32 numbers), for
// the marker-property kernel: the FP64 exp costs some twenty operations on
// the FP64 pipe (a small fraction of the FP32 rate on this GPU) per marker,
// this one two FP64 operations (the range reduction) and ~200 on the FP32
// pipe.  Host-compilable as plain C++ (a CPU test compares it with the
// long-double exp).
//
// Method: x = k ln2 + r with k = round(x / ln2) and r by two fused
// multiply-adds against ln2 split into a 40-bit high part and the rest
// (Cody and Waite), |r| <= ln2 / 2; exp(r) by its Taylor series to r^13/13!
// (truncation < 1e-17 relative) evaluated by Horner's rule in double-float
// arithmetic (Dekker's product, Knuth's TwoSum; coefficients 1/n! as
// double-float pairs); exp(x) = 2^k exp(r), the scaling exact.  Relative
// error below 2e-14 (the pairs carry ~48 bits; 1e-14 worst over [-60, 60]).
#pragma once

#include <math.h>
#include <stdint.h>

#include "hmec_bits.cuh"

#if defined(__CUDA_ARCH__)
#define HMEC_FMUL(a, b) __fmul_rn(a, b)
#define HMEC_FADD(a, b) __fadd_rn(a, b)
#define HMEC_FSUB(a, b) __fsub_rn(a, b)
#define HMEC_FFMA(a, b, c) fmaf(a, b, c)
#else
#define HMEC_FMUL(a, b) ((float)(a) * (float)(b))
#define HMEC_FADD(a, b) ((float)(a) + (float)(b))
#define HMEC_FSUB(a, b) ((float)(a) - (float)(b))
#define HMEC_FFMA(a, b, c) fmaf(a, b, c)
#endif

// (a + b) exactly as s + e (TwoSum)
HMEC_HD void dfx_two_sum(float a, float b, float& s, float& e) {
    s = HMEC_FADD(a, b);
    const float bb = HMEC_FSUB(s, a);
    e = HMEC_FADD(HMEC_FSUB(a, HMEC_FSUB(s, bb)), HMEC_FSUB(b, bb));
}

// (ah + al)(bh + bl) + (ch + cl) as a normalised pair
HMEC_HD void dfx_mul_add(float ah, float al, float bh, float bl, float ch, float cl, float& h, float& l) {
    const float p = HMEC_FMUL(ah, bh);
    float pe = HMEC_FFMA(ah, bh, -p);
    pe = HMEC_FFMA(ah, bl, pe);
    pe = HMEC_FFMA(al, bh, pe);
    float s, e;
    dfx_two_sum(p, ch, s, e);
    e = HMEC_FADD(e, HMEC_FADD(pe, cl));
    h = HMEC_FADD(s, e);
    l = HMEC_FSUB(e, HMEC_FSUB(h, s));
}

// exp(x) as h + l for x in [-60, 60] (outside: false, the caller uses exp).
HMEC_HD bool df_exp(double x, float& h, float& l) {
    if (!(x >= -60.0 && x <= 60.0)) return false;
    // 1/n!, n = 0..13, as (high, low) FP32 pairs
    const float cf[14][2] = {
        {1.0f, 0.0f},
        {1.0f, 0.0f},
        {0.5f, 0.0f},
        {0.1666666716337204f, -4.967053879312289e-09f},
        {0.0416666679084301f, -1.2417634698280722e-09f},
        {0.008333333767950535f, -4.34617203337595e-10f},
        {0.0013888889225199819f, -3.3631094437103215e-11f},
        {0.00019841270113829523f, -2.725596874933456e-12f},
        {2.4801587642286904e-05f, -3.40699609366682e-13f},
        {2.7557318844628753e-06f, 3.793571224297229e-14f},
        {2.755731998149713e-07f, -7.575112209051195e-15f},
        {2.5052107943679403e-08f, 4.4176230446483665e-16f},
        {2.0876755879584152e-09f, 1.1082839147459852e-16f},
        {1.6059044372074283e-10f, -5.352526511562726e-18f},
    };
    const double LN2_HI = 0.6931471805601177;      // ln 2 rounded to 40 bits: k LN2_HI is exact
    const double LN2_LO = -1.7239444525614835e-13;  // ln 2 - LN2_HI
    const double k = floor(x * 1.4426950408889634 + 0.5);
    double r = fma(-k, LN2_HI, x);
    r = fma(-k, LN2_LO, r);
    // r as a pair (|r| <= 0.35)
    const float rh = (float)r;
    const float rl = (float)(r - (double)rh);
    float ph = cf[13][0], pl = cf[13][1];
    for (int n = 12; n >= 0; n--) dfx_mul_add(ph, pl, rh, rl, cf[n][0], cf[n][1], ph, pl);
    // times 2^k, exactly (k in [-87, 87])
    const int ki = (int)k;
    const float sc = hmec_float_of((uint32_t)(127 + ki / 2) << 23);
    const float sc2 = hmec_float_of((uint32_t)(127 + (ki - ki / 2)) << 23);
    h = HMEC_FMUL(HMEC_FMUL(ph, sc), sc2);
    l = HMEC_FMUL(HMEC_FMUL(pl, sc), sc2);
    return true;
}
