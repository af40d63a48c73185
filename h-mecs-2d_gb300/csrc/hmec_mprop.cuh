// hmec_mprop.cuh -- the per-marker properties of the markers->nodes
// section (cpp/h_mec_rsf_v9.cpp:386-423), shared by the context path
// (k_p2g.cu: k_mprop) and the allocation-free entry point (k_p2g_static.cu),
// so that both round alike, with the double-float helpers they use.
#pragma once

#include "hmec_dfexp.cuh"
#include "hmec_internal.cuh"

namespace {

// x = h + l: h keeps the top 24 bits of the mantissa (truncated), l is the
// remaining 29 bits rounded to FP32 (|x - h - l| < 2^-47 |x|).  Zeros and
// FP64 subnormals give 0; |x| outside [2^-74, 2^127) (and inf/NaN) take the
// FP64 conversions.
__device__ __forceinline__ void split_df(double x, float& h, float& l) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
    const int E = (int)((hi32 >> 20) & 0x7FF);
    const unsigned sign = hi32 & 0x80000000u;
    if (E >= 949 && E <= 1150) {
        h = __uint_as_float(sign | ((unsigned)(E - 896) << 23) | ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29));
        // the 29 remaining bits R as FP32: 2^23 + v has v in its mantissa for
        // v < 2^23, so R = 64 (R >> 6) + (R & 63) converts exactly, one rounding
        const unsigned R = lo32 & 0x1FFFFFFFu;
        const float rh = __fsub_rn(__uint_as_float(0x4B000000u | (R >> 6)), 8388608.f);
        const float rl = __fsub_rn(__uint_as_float(0x4B000000u | (R & 63u)), 8388608.f);
        const float r = __fmul_rn(fmaf(rh, 64.f, rl), __uint_as_float((unsigned)(E - 948) << 23));
        l = sign ? -r : r;
    } else if (E == 0) {
        h = 0.f;
        l = 0.f;
    } else {
        h = __double2float_rn(x);
        l = __double2float_rn(x - (double)h);
    }
}

// (ah + al)(bh + bl) as t + e (al * bl dropped, < 2^-48 relative).
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& t, float& e) {
    t = __fmul_rn(ah, bh);
    e = fmaf(ah, bh, -t);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
}

// normalised double-float a + b (|a| >= |b|)
__device__ __forceinline__ void df_norm(float& a, float& b) {
    const float s = __fadd_rn(a, b);
    b = __fsub_rn(b, __fsub_rn(s, a));
    a = s;
}

// v < lo ? lo : (v > hi ? hi : v).  Non-negative finite doubles order like
// their bit patterns, so for those the compares run on the integer pipe.
__device__ __forceinline__ double enforce_bounds(double v, double lo, double hi) {
    const long long b = __double_as_longlong(v), bl = __double_as_longlong(lo), bh = __double_as_longlong(hi);
    constexpr long long INF = 0x7FF0000000000000LL;
    if (b >= 0 && b < INF && bl >= 0 && bl < INF && bh >= 0 && bh < INF) return b < bl ? lo : (b > bh ? hi : v);
    return v < lo ? lo : (v > hi ? hi : v);
}

// The FP64 properties of marker m (:389-423).  FP64 runs at a small
// fraction of the FP32 rate on this GPU, so the arithmetic is kept to what
// the values need: (por/POR0)^3 is two products with ipor0 = 1/POR0, and
// etas exp(-alpha por) is formed in double-float (df_exp; the FP64 exp
// outside its range).  M: any struct of the marker array pointers.
struct MarkerProps {
    double por, tm, kkk, cohc, coht, fric, dilc, frit, etas, eta0, eta, rho;
};

template <class M>
__device__ __forceinline__ MarkerProps marker_props(const M& mk, int m, const hmec_params& p, double ipor0) {
    MarkerProps q;
    const double por = mk.porm[m];
    const double pr = por * ipor0;  // por / POR0 to an ulp
    q.por = por;
    q.kkk = enforce_bounds(mk.kkkm[m] * (pr * pr * pr), p.kkkmin, p.kkkmax);
    q.tm = mk.t_marker[m];
    if ((__double_as_longlong(q.tm) << 1) != 0) {  // tm != 0 (either zero fails, NaN passes)
        q.cohc = mk.cohescm[m] * (1 - por);
        q.coht = mk.cohestm[m] * (1 - por);
        q.fric = mk.frictcm[m];
        q.dilc = mk.dilatcm[m];
        q.frit = mk.fricttm[m];
        q.etas = mk.etasm[m];
        // etas exp(-alpha por): the exponential in double-float (two FP64
        // operations of range reduction instead of the FP64 exp's ~20)
        const double xe = -p.alpha * por;
        float eh, el;
        if (df_exp(xe, eh, el)) {
            float sh, sl, t, e;
            split_df(q.etas, sh, sl);
            df_mul(sh, sl, eh, el, t, e);
            df_norm(t, e);
            q.eta0 = f2d_bits(t) + f2d_bits(e);
        } else {
            q.eta0 = q.etas * exp(xe);
        }
        q.eta = mk.etam[m];
        q.rho = mk.rhom[m] * (1 - por) + mk.rhofm[m] * por;
    } else {
        q.cohc = mk.cohescm[m];
        q.coht = mk.cohestm[m];
        q.fric = mk.frictcm[m];
        q.dilc = 0;
        q.frit = mk.fricttm[m];
        q.etas = mk.etasm[m];
        q.eta0 = mk.etasm[m];
        q.eta = mk.etam[m];
        q.rho = mk.rhom[m];
    }
    q.eta0 = enforce_bounds(q.eta0, p.etamin, p.etamax);
    q.eta = enforce_bounds(q.eta, p.etamin, p.etamax);
    return q;
}

}  // namespace
