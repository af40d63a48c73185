// k_p2g.cu -- markers -> nodes (sections a1-a4, cpp/h_mec_rsf_v9.cpp:376-583).
//
// The reference scatters every marker into four 2x2 node blocks with an
// OpenMP `+=` that races between threads (:384-528).  Here the scatter is
// turned into a deterministic gather:
//
//  1. keys: each marker's basic cell (ib, jb) and pressure cell (iP, jP) are
//     computed with the reference's integer arithmetic (fix + check_bounds,
//     IEEE division, no contraction), so they are bit-exact.  Because
//     iP - ib and jP - jb are always 0 or 1, the pair defines a "half cell"
//     (hr = 2*ib + (iP-ib), hc = 2*jb + (jP-jb)), and the cell of the
//     marker on each of the four grids (basic, P, Vx = (iP, jb),
//     Vy = (ib, jP)) is a function of its half cell.  One counting sort by
//     half cell therefore serves all four grids.
//  2. counting sort: warp-aggregated integer atomics for the histogram and
//     the scatter, a three-phase scan, then each half-cell segment is put in
//     marker-index order, so the permutation is deterministic.
//  3. per-marker properties (a1) and interpolation distances are computed
//     once, in sorted order, into structure-of-arrays buffers.
//  4. one thread per cell of each grid sums weight and weight * property per
//     corner node over the cell's markers (two contiguous sorted runs); one
//     thread per node adds its four cells' corner sums in a fixed order and
//     normalises in the epilogue (a4).  No float atomics.
#include "hmec_dfexp.cuh"
#include "hmec_internal.cuh"
#include "hmec_mprop.cuh"
#include "hmec_sort.cuh"

namespace {

constexpr int NPROP = 21;
// Per-marker records of each grid's gather, in sorted order: the two
// interpolation distances then the grid's properties, each a double-float
// (h, l) pair of FP32, padded to whole float4s.  One thread reads its
// marker's record with 16-byte loads, so a gather touches each sector once.
constexpr int REC_B = 24, REC_P = 16, REC_X = 12, REC_Y = 12;  // floats per record
constexpr int REC_ALL = REC_B + REC_P + REC_X + REC_Y;         // floats per marker
// sorted per-marker property rows
enum {
    MP_DXB, MP_DYB, MP_DXX, MP_DYY, MP_DXP, MP_DYP,  // interpolation distances
    MP_RHO, MP_KKK, MP_TTT, MP_INVG, MP_ETA0, MP_COHT, MP_FRIT, MP_COHC, MP_FRIC, MP_DILC,
    MP_ETAP, MP_POR, MP_ETAB0, MP_INVETAD, MP_RHOF
};
// Record contents (dx, dy, then the properties in the order the node
// kernels read them):
//   basic: DXB DYB | RHO KKK TTT INVG ETA0 COHT FRIT COHC FRIC DILC
//   P:     DXP DYP | ETAP POR ETAB0 ETA0 INVG (+ 2 floats of padding)
//   Vx:    DXX DYP | RHO INVETAD RHOF POR
//   Vy:    DXP DYY | RHO INVETAD RHOF POR

// ---------------------------------------------------------------- double-float
// The gathers' products and sums run in double-float: a value is the
// unevaluated sum h + l of two FP32 numbers (~48 bits), with the error-free
// transformations of Dekker and Knuth (TwoSum; the exact FP32 product error
// from one fmaf).  On this GPU the FP32 pipe issues ~60x the FP64 rate, and
// FP64<->FP32 conversions run at the FP64 rate, so FP64 values are split by
// their bit patterns.  Relative error of a sum of same-sign terms ~1e-14.

// (sh, sl) += t + e, with t + e already a double-float (|e| <= ulp(t)).
__device__ __forceinline__ void df_acc(float& sh, float& sl, float t, float e) {
    const float s = __fadd_rn(sh, t);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(t, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// h + l = 1 / a: the FP32 reciprocal refined by one Newton-Raphson step
// x + x (u + u^2), u = 1 - a x, evaluated in double-float (relative error
// < 3e-14).
// False when a is outside (1e-30, 1e30) in magnitude: the caller divides.
__device__ __forceinline__ bool df_rcp(double a, float& h, float& l) {
    float ah, al;
    split_df(a, ah, al);
    const float aa = fabsf(ah);
    if (!(aa > 1e-30f && aa < 1e30f)) return false;
    const float r = __frcp_rn(ah);
    const float t = __fmul_rn(ah, r);  // within 2^-23 of 1: 1 - t is exact
    const float e1 = fmaf(ah, r, -t);
    const float u = fmaf(-al, r, __fsub_rn(__fsub_rn(1.f, t), e1));  // 1 - a r
    const float ru = __fmul_rn(r, u);
    h = r;
    l = fmaf(ru, u, ru);  // r (u + u^2)
    df_norm(h, l);
    return true;
}

// a1 per marker (:389-423) in sorted order, plus interpolation distances.
struct MkPtrs {
    const double *xm, *ym, *t_marker, *rhom, *etasm, *etam, *cohescm, *cohestm, *frictcm, *dilatcm, *fricttm,
        *porm, *kkkm, *gm, *rhofm, *etafm;
};
struct Crd {
    const double *x, *y, *xvx, *yvx, *xvy, *yvy, *xp, *yp;
};

// FP64 runs at a small fraction of the FP32 rate on this GPU, so the
// arithmetic is kept to what the values need: the cells come from the sort
// key (no second set of divisions), (por/POR0)^3 is two products, the
// distances are products with 1/dx and 1/dy, and 1/etad = k/etaf is one
// division; each differs from the reference's expression by at most an ulp
// or two (the marker->node fields are tested to 1e-13).  Each row is stored
// as a double-float pair of FP32 rows for the gathers.
__global__ void k_mprop(MkPtrs mk, const int32_t* __restrict__ perm, const int32_t* __restrict__ key, int64_t n,
                        Geo g, Crd c, hmec_params p, double ipor0, float* __restrict__ out) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int m = perm[k];
    const MarkerProps q = marker_props(mk, m, p, ipor0);
    const double xmm = mk.xm[m], ymm = mk.ym[m];
    // half cell (hr, hc) = (2 ib + (iP - ib), 2 jb + (jP - jb)), key = hc * HR + hr
    const int HR = 2 * (g.Ny - 1), kk = key[m];
    const int hc = kk / HR, hr = kk - hc * HR;
    const int ib = hr >> 1, jb = hc >> 1, iP = ib + (hr & 1), jP = jb + (hc & 1);
    // v[2q], v[2q + 1]: property row q as a double-float
    float v[2 * NPROP];
    auto put_df = [&](int q, float h, float l) {
        v[2 * q] = h;
        v[2 * q + 1] = l;
    };
    auto put = [&](int q, double v) {
        float h, l;
        split_df(v, h, l);
        put_df(q, h, l);
    };
    // distances: the node offset exactly in FP64 (Sterbenz), then the
    // product with 1/dx or 1/dy in double-float
    float ixh, ixl, iyh, iyl;
    split_df(g.idx, ixh, ixl);
    split_df(g.idy, iyh, iyl);
    auto put_dist = [&](int q, double d, float ih, float il) {
        float dh, dl, t, e;
        split_df(d, dh, dl);
        df_mul(dh, dl, ih, il, t, e);
        df_norm(t, e);
        put_df(q, t, e);
    };
    put_dist(MP_DXB, xmm - c.x[jb], ixh, ixl);
    put_dist(MP_DYB, ymm - c.y[ib], iyh, iyl);
    put_dist(MP_DXX, xmm - c.xvx[jb], ixh, ixl);
    put_dist(MP_DYY, ymm - c.yvy[ib], iyh, iyl);
    put_dist(MP_DXP, xmm - c.xp[jP], ixh, ixl);
    put_dist(MP_DYP, ymm - c.yp[iP], iyh, iyl);
    put(MP_RHO, q.rho);
    put(MP_KKK, q.kkk);
    put(MP_TTT, q.tm);
    {
        float h, l;
        if (df_rcp(mk.gm[m], h, l))
            put_df(MP_INVG, h, l);
        else
            put(MP_INVG, 1. / mk.gm[m]);
    }
    put(MP_ETA0, q.eta0);
    put(MP_COHT, q.coht);
    put(MP_FRIT, q.frit);
    put(MP_COHC, q.cohc);
    put(MP_FRIC, q.fric);
    put(MP_DILC, q.dilc);
    put(MP_ETAP, q.eta);
    put(MP_POR, q.por);
    put(MP_ETAB0, q.etas);
    {
        // k / etaf as k * (1 / etaf) in double-float
        float rh, rl, kh, kl, t, e;
        if (df_rcp(mk.etafm[m], rh, rl)) {
            split_df(q.kkk, kh, kl);
            df_mul(kh, kl, rh, rl, t, e);
            df_norm(t, e);
            put_df(MP_INVETAD, t, e);
        } else {
            put(MP_INVETAD, q.kkk / mk.etafm[m]);
        }
    }
    put(MP_RHOF, mk.rhofm[m]);
    // the four grids' records (layout above), 16-byte stores
    auto f4 = [&](int a, int b) { return make_float4(v[2 * a], v[2 * a + 1], v[2 * b], v[2 * b + 1]); };
    const size_t n_ = (size_t)n;
    float4* rb = reinterpret_cast<float4*>(out + (size_t)k * REC_B);
    rb[0] = f4(MP_DXB, MP_DYB);
    rb[1] = f4(MP_RHO, MP_KKK);
    rb[2] = f4(MP_TTT, MP_INVG);
    rb[3] = f4(MP_ETA0, MP_COHT);
    rb[4] = f4(MP_FRIT, MP_COHC);
    rb[5] = f4(MP_FRIC, MP_DILC);
    float4* rp = reinterpret_cast<float4*>(out + n_ * REC_B + (size_t)k * REC_P);
    rp[0] = f4(MP_DXP, MP_DYP);
    rp[1] = f4(MP_ETAP, MP_POR);
    rp[2] = f4(MP_ETAB0, MP_ETA0);
    rp[3] = make_float4(v[2 * MP_INVG], v[2 * MP_INVG + 1], 0.f, 0.f);
    float4* rx = reinterpret_cast<float4*>(out + n_ * (REC_B + REC_P) + (size_t)k * REC_X);
    rx[0] = f4(MP_DXX, MP_DYP);
    rx[1] = f4(MP_RHO, MP_INVETAD);
    rx[2] = f4(MP_RHOF, MP_POR);
    float4* ry = reinterpret_cast<float4*>(out + n_ * (REC_B + REC_P + REC_X) + (size_t)k * REC_Y);
    ry[0] = f4(MP_DXP, MP_DYY);
    ry[1] = f4(MP_RHO, MP_INVETAD);
    ry[2] = f4(MP_RHOF, MP_POR);
}

// Gathers in two passes.  Every marker of one grid's cell (ci, cj) (cells
// indexed by their top-left node; all four grids have (Ny-1) x (Nx-1) cells
// after the reference's clamping) adds to the cell's four corner nodes with
// the bilinear weights (1-dx)(1-dy) to (ci, cj), (1-dx) dy to (ci+1, cj),
// dx (1-dy) to (ci, cj+1), dx dy to (ci+1, cj+1) -- the products fx * fy of
// :435-528.  Pass 1, one thread per cell, sums weight and weight * property
// per corner over the cell's markers (its half cells are two contiguous runs
// of the sorted order, markers in sorted order); pass 2, one thread per
// node, adds the corner sums of its four cells in a fixed order.  Each
// marker is read once per grid, not once per node.
//
// ROWP / COLP: the grid's cell rows / columns follow the pressure cell.
// Corner sums: cs[(s * 4 + corner) * ncell + cj * (Ny-1) + ci], s = 0 the
// weight, s = 1..NP the properties.
// rec: the grid's marker records (RW floats each: dx, dy, NP properties).
// One thread's share of cell (ci, cj): the weight sums when WT, and the
// sums of properties [Q0, Q1).  Every sum sees the same operations in the
// same order whichever thread holds it, so splitting a cell's properties
// over threads changes no result.
template <bool ROWP, bool COLP, int NP, int RW, int Q0, int Q1, bool WT>
__device__ __forceinline__ void cell_sums_part(const Geo& g, const int32_t* __restrict__ start,
                                               const float* __restrict__ rec, double* __restrict__ cs, int ci,
                                               int cj) {
    static_assert(RW % 4 == 0 && RW >= 4 + 2 * NP, "record layout");
    constexpr int NQ = Q1 - Q0;
    // the record's float4s this share reads: the distances (0) and those
    // holding properties Q0..Q1-1 (property q at floats 4 + 2q, 5 + 2q)
    constexpr int F0 = 1 + Q0 / 2, F1 = 1 + (Q1 - 1) / 2;
    const int NCI = g.Ny - 1, NCJ = g.Nx - 1;
    const int HR = 2 * (g.Ny - 1), HC = 2 * (g.Nx - 1);
    const int r0 = ROWP ? 2 * ci - 1 : 2 * ci, c0 = COLP ? 2 * cj - 1 : 2 * cj;
    const int rlo = r0 < 0 ? 0 : r0, rhi = r0 + 1 > HR - 1 ? HR - 1 : r0 + 1;
    // double-float accumulators: [c] weight, [q][c] weight * property
    float Wh[4] = {0, 0, 0, 0}, Wl[4] = {0, 0, 0, 0}, Sh[NQ][4], Sl[NQ][4];
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int c = 0; c < 4; c++) Sh[q][c] = Sl[q][c] = 0;
    // the low parts collect the high parts' rounding errors; folding them back
    // every 8 markers keeps the sums at double-float accuracy however many
    // markers a cell holds (markers that cluster)
    int since_norm = 0;
    for (int hc = c0 < 0 ? 0 : c0; hc <= c0 + 1 && hc < HC; hc++) {
        const int b = start[hc * HR + rlo], e = start[hc * HR + rhi + 1];
        for (int k = b; k < e; k++) {
            if (++since_norm == 8) {
                since_norm = 0;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    if (WT) df_norm(Wh[c], Wl[c]);
#pragma unroll
                    for (int q = 0; q < NQ; q++) df_norm(Sh[q][c], Sl[q][c]);
                }
            }
            float r[RW];
            const float4* r4 = reinterpret_cast<const float4*>(rec + (size_t)k * RW);
            {
                const float4 x = __ldg(r4);
                r[0] = x.x;
                r[1] = x.y;
                r[2] = x.z;
                r[3] = x.w;
            }
#pragma unroll
            for (int t = F0; t <= F1; t++) {
                const float4 x = __ldg(r4 + t);
                r[4 * t] = x.x;
                r[4 * t + 1] = x.y;
                r[4 * t + 2] = x.z;
                r[4 * t + 3] = x.w;
            }
            const float dxh = r[0], dxl = r[1], dyh = r[2], dyl = r[3];
            // 1 - dx and 1 - dy exactly as TwoSum pairs (plus the low parts)
            float axh = __fsub_rn(1.f, dxh), ayh = __fsub_rn(1.f, dyh);
            float axl, ayl;
            {
                float bb = __fsub_rn(axh, 1.f);
                axl = __fsub_rn(__fadd_rn(__fsub_rn(1.f, __fsub_rn(axh, bb)), __fsub_rn(-dxh, bb)), dxl);
                bb = __fsub_rn(ayh, 1.f);
                ayl = __fsub_rn(__fadd_rn(__fsub_rn(1.f, __fsub_rn(ayh, bb)), __fsub_rn(-dyh, bb)), dyl);
            }
            // the bilinear weights (1-dx)(1-dy), (1-dx) dy, dx (1-dy), dx dy
            float wh[4], wl[4];
            df_mul(axh, axl, ayh, ayl, wh[0], wl[0]);
            df_mul(axh, axl, dyh, dyl, wh[1], wl[1]);
            df_mul(dxh, dxl, ayh, ayl, wh[2], wl[2]);
            df_mul(dxh, dxl, dyh, dyl, wh[3], wl[3]);
#pragma unroll
            for (int c = 0; c < 4; c++) {
                df_norm(wh[c], wl[c]);
                if (WT) df_acc(Wh[c], Wl[c], wh[c], wl[c]);
            }
#pragma unroll
            for (int q = 0; q < NQ; q++) {
                const float ph = r[4 + 2 * (Q0 + q)], pl = r[5 + 2 * (Q0 + q)];
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    float t, er;
                    df_mul(wh[c], wl[c], ph, pl, t, er);
                    df_acc(Sh[q][c], Sl[q][c], t, er);
                }
            }
        }
    }
    const size_t ncell = (size_t)NCI * NCJ, cell = (size_t)cj * NCI + ci;
    if (WT) {
#pragma unroll
        for (int c = 0; c < 4; c++) cs[(size_t)c * ncell + cell] = f2d_bits(Wh[c]) + f2d_bits(Wl[c]);
    }
#pragma unroll
    for (int q = 0; q < NQ; q++)
#pragma unroll
        for (int c = 0; c < 4; c++)
            cs[((size_t)(1 + Q0 + q) * 4 + c) * ncell + cell] = f2d_bits(Sh[q][c]) + f2d_bits(Sl[q][c]);
}

// Grid (SPLIT, cell-row blocks, cell columns).  SPLIT = 2: blockIdx.x = 0
// sums the weights and the first half of the properties, 1 the second half
// (the basic grid's ten properties in one thread need 172 registers; halves
// keep twice the warps resident).  The half is the fastest grid index, so
// both halves of a cell range run together and the second one reads the
// records from L2, not DRAM again.
template <bool ROWP, bool COLP, int NP, int RW, int SPLIT>
__global__ void k_cell_sums(Geo g, const int32_t* __restrict__ start, const float* __restrict__ rec,
                            double* __restrict__ cs) {
    const int ci = blockIdx.y * blockDim.x + threadIdx.x, cj = blockIdx.z;
    if (ci >= g.Ny - 1) return;
    if (SPLIT == 1) {
        cell_sums_part<ROWP, COLP, NP, RW, 0, NP, true>(g, start, rec, cs, ci, cj);
    } else if (blockIdx.x == 0) {
        cell_sums_part<ROWP, COLP, NP, RW, 0, NP / 2, true>(g, start, rec, cs, ci, cj);
    } else {
        cell_sums_part<ROWP, COLP, NP, RW, NP / 2, NP, false>(g, start, rec, cs, ci, cj);
    }
}

// Node (i, j): cells (i-1, j-1), (i, j-1), (i-1, j), (i, j), of which it is
// corner 3, 2, 1, 0, in that order.
template <int NP>
__device__ __forceinline__ void node_sums(int i, int j, const Geo& g, const double* __restrict__ cs, double& wt,
                                          double (&acc)[NP]) {
    const int NCI = g.Ny - 1, NCJ = g.Nx - 1;
    const size_t ncell = (size_t)NCI * NCJ;
    wt = 0;
#pragma unroll
    for (int q = 0; q < NP; q++) acc[q] = 0;
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const int ci = i - 1 + (t & 1), cj = j - 1 + (t >> 1), corner = 3 - t;
        if (ci < 0 || ci >= NCI || cj < 0 || cj >= NCJ) continue;
        const size_t cell = (size_t)cj * NCI + ci;
        wt += cs[(size_t)corner * ncell + cell];
#pragma unroll
        for (int q = 0; q < NP; q++) acc[q] += cs[((size_t)(1 + q) * 4 + corner) * ncell + cell];
    }
}

__global__ void k_node_basic(Geo g, const double* __restrict__ cs, double* RHO, double* KKK, double* TTT,
                             double* GGG, double* ETA0, double* COHT, double* FRIT, double* COHC, double* FRIC,
                             double* DILC) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    double wt, a[10];
    node_sums<10>(i, j, g, cs, wt, a);
    if (wt > 0) {
        size_t o = (size_t)j * g.Ny + i;
        const double iw = 1. / wt;  // products instead of ten divisions (an ulp apart)
        RHO[o] = a[0] * iw;
        KKK[o] = a[1] * iw;
        TTT[o] = a[2] * iw;
        GGG[o] = 1. / (a[3] * iw);
        ETA0[o] = a[4] * iw;
        COHT[o] = a[5] * iw;
        FRIT[o] = a[6] * iw;
        COHC[o] = a[7] * iw;
        FRIC[o] = a[8] * iw;
        DILC[o] = a[9] * iw;
    }
}

__global__ void k_node_p(Geo g, const double* __restrict__ cs, double* ETAP, double* POR, double* ETAB0,
                         double* ETAP0, double* GGGP) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny1) return;
    double wt, a[5];
    node_sums<5>(i, j, g, cs, wt, a);
    if (wt > 0) {
        size_t o = (size_t)j * g.Ny1 + i;
        const double iw = 1. / wt;
        ETAP[o] = a[0] * iw;
        const double por = a[1] * iw;
        POR[o] = por;
        ETAB0[o] = a[2] * iw / por;
        ETAP0[o] = a[3] * iw;
        GGGP[o] = 1. / (a[4] * iw);
    }
}

// Vx nodes: rows follow the pressure cell, columns the basic cell.
__global__ void k_node_vx(Geo g, const double* __restrict__ cs, double* RHOX, double* ETADX, double* RHOFX,
                          double* PORX) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny1 || j >= g.Nx) return;
    double wt, a[4];
    node_sums<4>(i, j, g, cs, wt, a);
    if (wt > 0) {
        size_t o = (size_t)j * g.Ny1 + i;
        RHOX[o] = a[0] / wt;
        ETADX[o] = 1. / (a[1] / wt);
        RHOFX[o] = a[2] / wt;
        PORX[o] = a[3] / wt;
    }
}

// Vy nodes: rows follow the basic cell, columns the pressure cell.
__global__ void k_node_vy(Geo g, const double* __restrict__ cs, double* RHOY, double* ETADY, double* RHOFY,
                          double* PORY) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    double wt, a[4];
    node_sums<4>(i, j, g, cs, wt, a);
    if (wt > 0) {
        size_t o = (size_t)j * g.Ny1 + i;
        RHOY[o] = a[0] / wt;
        ETADY[o] = 1. / (a[1] / wt);
        RHOFY[o] = a[2] / wt;
        PORY[o] = a[3] / wt;
    }
}

// The cell-index rule of marker_cells on arbitrary coordinates.
__global__ void k_cell_index(const double* __restrict__ x, int64_t n, double d, int half, int32_t* out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fix_quot(x[i], d, rcp_f32(d), half != 0);
}

}  // namespace

extern "C" int32_t hmec_cell_index(const double* x, int64_t n, double d, int32_t half, int32_t* out) {
    if (n < 0 || (n > 0 && (!x || !out)) || !(d > 0)) return HMEC_ERR_ARG;
    if (n == 0) return HMEC_OK;
    double* dx = nullptr;
    int32_t* dout = nullptr;
    cudaError_t e = cudaMalloc(&dx, sizeof(double) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(int32_t) * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_cell_index<<<nblocks(n, 256), 256>>>(dx, n, d, half, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dout);
    return e == cudaSuccess ? HMEC_OK : HMEC_ERR_CUDA;
}

// ------------------------------------------------ marker storage order
// The library keeps the marker arrays on the device in half-cell order (the
// order of the sort below at upload time): the per-step gathers through the
// sort permutation then read consecutive markers instead of scattered ones.
// mord[k] is the caller's index of stored marker k; within a half cell the
// stored order keeps increasing caller index, so every per-step sort yields
// the same marker sequence -- and the same sums -- as caller order would.
__global__ void k_iota(int32_t* a, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (int32_t)i;
}
__global__ void k_gather_f64(const double* __restrict__ src, const int32_t* __restrict__ idx, int64_t n,
                             double* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}
__global__ void k_scatter_f64(const double* __restrict__ src, const int32_t* __restrict__ idx, int64_t n,
                              double* __restrict__ dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[idx[i]] = src[i];
}

int p2g_alloc(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    ctx->nhalf = 4 * (g.Nx - 1) * (g.Ny - 1);
    int64_t n = ctx->marknum;
    int nparts = (ctx->nhalf + 1 + 2047) / 2048;
    HMEC_CUDA(ctx, cudaMalloc(&ctx->mkey, sizeof(int32_t) * (size_t)n));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->perm, sizeof(int32_t) * (size_t)n));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->hc_count, sizeof(int32_t) * ((size_t)ctx->nhalf + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->hc_start, sizeof(int32_t) * ((size_t)ctx->nhalf + 2)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->hc_fill, sizeof(int32_t) * ((size_t)ctx->nhalf + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->scan_part, sizeof(int32_t) * ((size_t)nparts + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->sort_long, sizeof(int)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->mord, sizeof(int32_t) * (size_t)std::max<int64_t>(n, 1)));
    HMEC_LAUNCH(ctx, k_iota, nblocks(n, 256), 256, 0, ctx->mord, n);
    for (int k = 0; k < 4; k++) {
        HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->gs4[k], cudaStreamNonBlocking));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_g_done[k], cudaEventDisableTiming));
    }
    HMEC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_g_fork, cudaEventDisableTiming));
    // the marker records double as the radix sort's scratch (they are
    // written only after the sort); they hold 64 ints per marker, the sort
    // needs about 3.5
    int rgrid = 1;
    HMEC_CUDA(ctx, hsort::radix_grid(&rgrid));
    // ... and the marker transfers' staging (three FP64 arrays) past the sort's part
    const size_t rec = (size_t)REC_ALL * (size_t)n;
    const size_t need = hsort::radix_scratch_ints(n, rgrid);
    ctx->stage_off = (need + 3) / 4 * 4;  // floats; 16-byte aligned
    const size_t stage_end = ctx->stage_off + 6 * (size_t)n;
    HMEC_CUDA(ctx, cudaMalloc(&ctx->mprop, sizeof(float) * std::max(rec, stage_end)));
    // corner sums: (10 + 5 + 4 + 4 properties + 4 weights) x 4 corners per cell
    const size_t ncell = (size_t)(g.Ny - 1) * (g.Nx - 1);
    HMEC_CUDA(ctx, cudaMalloc(&ctx->cellsum, sizeof(double) * 27 * 4 * ncell));
    return HMEC_OK;
}

void p2g_free(hmec_inst* ctx) {
    cudaFree(ctx->mkey);
    cudaFree(ctx->perm);
    cudaFree(ctx->hc_count);
    cudaFree(ctx->hc_start);
    cudaFree(ctx->hc_fill);
    cudaFree(ctx->scan_part);
    cudaFree(ctx->sort_long);
    cudaFree(ctx->mord);
    for (int k = 0; k < 4; k++) {
        if (ctx->gs4[k]) cudaStreamDestroy(ctx->gs4[k]);
        if (ctx->ev_g_done[k]) cudaEventDestroy(ctx->ev_g_done[k]);
    }
    if (ctx->ev_g_fork) cudaEventDestroy(ctx->ev_g_fork);
    if (ctx->up_stream) {
        cudaStreamSynchronize(ctx->up_stream);
        cudaStreamDestroy(ctx->up_stream);
        cudaEventDestroy(ctx->ev_up_fork);
        cudaEventDestroy(ctx->ev_up_done);
    }
    cudaFree(ctx->mprop);
    cudaFree(ctx->cellsum);
}

// Staging buffers for the marker transfers: doubles of the marker-record
// region past the part the radix sort uses as scratch.
static double* stage_f64(hmec_inst* ctx, int k) {
    return reinterpret_cast<double*>(ctx->mprop + ctx->stage_off) + (size_t)k * (size_t)ctx->marknum;
}

int markers_stream_issue(hmec_inst* ctx) {
    if (!ctx->src_set) return HMEC_OK;
    if (!ctx->up_stream) {
        HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_up_fork, cudaEventDisableTiming));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_up_done, cudaEventDisableTiming));
    }
    // after the markers->nodes section nothing else in the step reads the
    // marker arrays (advection, which would, is refused at registration).
    // Streamed markers are stored in the caller's order: plain copies, no
    // kernel competes with the solve for the SMs (the next step's sort orders
    // them, as it does every step); the storage order becomes the identity.
    HMEC_CUDA(ctx, cudaEventRecord(ctx->ev_up_fork, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamWaitEvent(ctx->up_stream, ctx->ev_up_fork, 0));
    const int64_t n = ctx->marknum;
    for (int k = 0; k < HMEC_M_COUNT; k++)
        HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->mk[k], ctx->src_mk[k], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                       ctx->up_stream));
    {
        StreamScope scope(ctx, ctx->up_stream);
        HMEC_LAUNCH(ctx, k_iota, nblocks(n, 256), 256, 0, ctx->mord, n);
    }
    HMEC_CUDA(ctx, cudaEventRecord(ctx->ev_up_done, ctx->up_stream));
    return HMEC_OK;
}

int markers_stream_join(hmec_inst* ctx) {
    if (!ctx->src_set) return HMEC_OK;
    HMEC_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->ev_up_done, 0));
    return HMEC_OK;
}

int p2g_store_markers(hmec_inst* ctx, const double* const* fields) {
    const int64_t n = ctx->marknum;
    const Geo& g = ctx->g;
    double* tx = stage_f64(ctx, 0);
    double* ty = stage_f64(ctx, 1);
    double* tf = stage_f64(ctx, 2);
    HMEC_CUDA(ctx, cudaMemcpyAsync(tx, fields[HMEC_M_xm], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                   ctx->stream));
    HMEC_CUDA(ctx, cudaMemcpyAsync(ty, fields[HMEC_M_ym], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                   ctx->stream));
    // the half-cell order of the caller's markers (its index breaking ties)
    const int nh = ctx->nhalf;
    HMEC_CUDA(ctx, cudaMemsetAsync(ctx->hc_count, 0, sizeof(int32_t) * ((size_t)nh + 1), ctx->stream));
    HMEC_LAUNCH(ctx, hsort::k_keys, nblocks(n, ctx->bs_so), ctx->bs_so, 0, tx, ty, n, g, ctx->mkey, ctx->hc_count,
                &ctx->ds->status);
    hsort::SortBufs sb{ctx->mkey, ctx->hc_count, ctx->hc_start, ctx->hc_fill, ctx->scan_part, ctx->mord,
                       ctx->sort_long, reinterpret_cast<int32_t*>(ctx->mprop), ctx->bs_so};
    HMEC_CUDA(ctx, hsort::sort_by_half_cell(ctx->stream, sb, n, nh, &ctx->launches));
    for (int k = 0; k < HMEC_M_COUNT; k++) {
        const double* src = tx;
        if (k == HMEC_M_ym) src = ty;
        if (k != HMEC_M_xm && k != HMEC_M_ym) {
            HMEC_CUDA(ctx, cudaMemcpyAsync(tf, fields[k], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                           ctx->stream));
            src = tf;
        }
        HMEC_LAUNCH(ctx, k_gather_f64, nblocks(n, 256), 256, 0, src, ctx->mord, n, ctx->mk[k]);
    }
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

int p2g_load_markers(hmec_inst* ctx, double* const* fields) {
    const int64_t n = ctx->marknum;
    double* tf = stage_f64(ctx, 2);
    for (int k = 0; k < HMEC_M_COUNT; k++) {
        if (!fields[k]) continue;
        HMEC_LAUNCH(ctx, k_scatter_f64, nblocks(n, 256), 256, 0, ctx->mk[k], ctx->mord, n, tf);
        HMEC_CUDA(ctx, cudaMemcpyAsync(fields[k], tf, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    }
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

int p2g_run(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    const int64_t n = ctx->marknum;
    const int nh = ctx->nhalf;
    int* status = &ctx->ds->status;
    HMEC_CUDA(ctx, cudaMemsetAsync(ctx->hc_count, 0, sizeof(int32_t) * ((size_t)nh + 1), ctx->stream));
    HMEC_LAUNCH(ctx, hsort::k_keys, nblocks(n, ctx->bs_so), ctx->bs_so, 0, ctx->mk[HMEC_M_xm], ctx->mk[HMEC_M_ym], n, g, ctx->mkey,
                ctx->hc_count, status);
    // segment starts hc_start[0..nh], the scatter, the per-segment order
    hsort::SortBufs sb{ctx->mkey, ctx->hc_count, ctx->hc_start, ctx->hc_fill, ctx->scan_part, ctx->perm,
                       ctx->sort_long, reinterpret_cast<int32_t*>(ctx->mprop), ctx->bs_so};
    HMEC_CUDA(ctx, hsort::sort_by_half_cell(ctx->stream, sb, n, nh, &ctx->launches));
    MkPtrs mk;
    mk.xm = ctx->mk[HMEC_M_xm];
    mk.ym = ctx->mk[HMEC_M_ym];
    mk.t_marker = ctx->mk[HMEC_M_t_marker];
    mk.rhom = ctx->mk[HMEC_M_rhom];
    mk.etasm = ctx->mk[HMEC_M_etasm];
    mk.etam = ctx->mk[HMEC_M_etam];
    mk.cohescm = ctx->mk[HMEC_M_cohescm];
    mk.cohestm = ctx->mk[HMEC_M_cohestm];
    mk.frictcm = ctx->mk[HMEC_M_frictcm];
    mk.dilatcm = ctx->mk[HMEC_M_dilatcm];
    mk.fricttm = ctx->mk[HMEC_M_fricttm];
    mk.porm = ctx->mk[HMEC_M_porm];
    mk.kkkm = ctx->mk[HMEC_M_kkkm];
    mk.gm = ctx->mk[HMEC_M_gm];
    mk.rhofm = ctx->mk[HMEC_M_rhofm];
    mk.etafm = ctx->mk[HMEC_M_etafm];
    Crd c{ctx->crd[0], ctx->crd[1], ctx->crd[2], ctx->crd[3], ctx->crd[4], ctx->crd[5], ctx->crd[6], ctx->crd[7]};
    HMEC_LAUNCH(ctx, k_mprop, nblocks(n, ctx->bs_so), ctx->bs_so, 0, mk, ctx->perm, ctx->mkey, n, g, c, ctx->p, 1.0 / ctx->p.POR0,
                ctx->mprop);
    double* const* f = ctx->f;
    // pass 1: corner sums per cell of each grid; pass 2: node sums and the a4 epilogues
    const size_t ncell = (size_t)(g.Ny - 1) * (g.Nx - 1);
    double* cs_b = ctx->cellsum;
    double* cs_p = cs_b + 11 * 4 * ncell;
    double* cs_x = cs_p + 6 * 4 * ncell;
    double* cs_y = cs_x + 5 * 4 * ncell;
    const float* rec_b = ctx->mprop;
    const float* rec_p = rec_b + (size_t)n * REC_B;
    const float* rec_x = rec_p + (size_t)n * REC_P;
    const float* rec_y = rec_x + (size_t)n * REC_X;
    const int bs = ctx->bs_st;
    dim3 bb(bs), gc(1, nblocks(g.Ny - 1, bs), g.Nx - 1), gc2(2, nblocks(g.Ny - 1, bs), g.Nx - 1);
    dim3 gb(nblocks(g.Ny, bs), g.Nx), gs(nblocks(g.Ny1, bs), g.Nx1);
    // the four grids' gathers are independent: each pair (cell sums, node
    // sums) on a stream of its own (streams of this section only: the
    // solver's level streams join the capture of a global iteration's body
    // when the timestep is captured as a graph, and a stream belongs to one
    // capture at a time)
    const cudaStream_t main = ctx->stream;
    HMEC_CUDA(ctx, cudaEventRecord(ctx->ev_g_fork, main));
    cudaError_t fork_err = cudaSuccess;
    auto on = [&](int k) {
        const cudaError_t e = cudaStreamWaitEvent(ctx->gs4[k], ctx->ev_g_fork, 0);
        if (e != cudaSuccess) fork_err = e;
        return ctx->gs4[k];
    };
    {
        StreamScope scope(ctx, on(0));
        HMEC_LAUNCH(ctx, (k_cell_sums<false, false, 10, REC_B, 2>), gc2, bb, 0, g, ctx->hc_start, rec_b, cs_b);
        HMEC_LAUNCH(ctx, k_node_basic, gb, bb, 0, g, cs_b, f[HMEC_F_RHO], f[HMEC_F_KKK], f[HMEC_F_TTT], f[HMEC_F_GGG],
                    f[HMEC_F_ETA0], f[HMEC_F_COHT], f[HMEC_F_FRIT], f[HMEC_F_COHC], f[HMEC_F_FRIC], f[HMEC_F_DILC]);
    }
    {
        StreamScope scope(ctx, on(1));
        HMEC_LAUNCH(ctx, (k_cell_sums<true, true, 5, REC_P, 1>), gc, bb, 0, g, ctx->hc_start, rec_p, cs_p);
        HMEC_LAUNCH(ctx, k_node_p, gs, bb, 0, g, cs_p, f[HMEC_F_ETAP], f[HMEC_F_POR], f[HMEC_F_ETAB0],
                    f[HMEC_F_ETAP0], f[HMEC_F_GGGP]);
    }
    {
        StreamScope scope(ctx, on(2));
        HMEC_LAUNCH(ctx, (k_cell_sums<true, false, 4, REC_X, 1>), gc, bb, 0, g, ctx->hc_start, rec_x, cs_x);
        HMEC_LAUNCH(ctx, k_node_vx, gs, bb, 0, g, cs_x, f[HMEC_F_RHOX], f[HMEC_F_ETADX], f[HMEC_F_RHOFX],
                    f[HMEC_F_PORX]);
    }
    {
        StreamScope scope(ctx, on(3));
        HMEC_LAUNCH(ctx, (k_cell_sums<false, true, 4, REC_Y, 1>), gc, bb, 0, g, ctx->hc_start, rec_y, cs_y);
        HMEC_LAUNCH(ctx, k_node_vy, gs, bb, 0, g, cs_y, f[HMEC_F_RHOY], f[HMEC_F_ETADY], f[HMEC_F_RHOFY],
                    f[HMEC_F_PORY]);
    }
    HMEC_CUDA(ctx, fork_err);
    for (int k = 0; k < 4; k++) {
        HMEC_CUDA(ctx, cudaEventRecord(ctx->ev_g_done[k], ctx->gs4[k]));
        HMEC_CUDA(ctx, cudaStreamWaitEvent(main, ctx->ev_g_done[k], 0));
    }
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}
