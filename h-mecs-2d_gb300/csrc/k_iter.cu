// k_iter.cu -- the global (plastic) iteration and the timestep frame
// (sections a5-a17, a19 of cpp/h_mec_rsf_v9.cpp:585-1726).
//
// Every grid kernel maps the row index i to threadIdx.x and the column j to
// blockIdx.y, matching the column-major layout.  The control logic of the
// loop (error, adaptive dt, exit test; :1310-1456) runs in one device thread
// on the scalars block, so the loop never needs the host to decide anything.
// Sums whose order changes the last bits (the fault error `ddd`) are taken
// in the reference's j order by that single thread; min/max reductions are
// exact in any order.
#include "hmec_internal.cuh"

#include <cmath>

namespace {

#define IB(F, i, j) F[(size_t)(j) * g.Ny + (i)]
#define IS(F, i, j) F[(size_t)(j) * g.Ny1 + (i)]

// Column-major 2x2 block sum, (0,0)+(1,0)+(0,1)+(1,1).
__device__ __forceinline__ double bsum(const double* a, int rows, int i, int j) {
    const double* c0 = a + (size_t)j * rows + i;
    const double* c1 = c0 + rows;
    return ((c0[0] + c0[1]) + c1[0]) + c1[1];
}

// ---------------------------------------------------------------- a5 begin
__global__ void k_step_begin(Geo g, DevScalars* ds, hmec_params p, const double* __restrict__ ETA0,
                             const double* __restrict__ ETA00, const double* __restrict__ OM0, double* ETA1,
                             double* ETA, double* ETA50, double* OM) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < g.Ny) {
        size_t o = (size_t)j * g.Ny + i;
        const double e = (ds->timestep == 1) ? ETA0[o] : ETA00[o];  // :586-594
        ETA1[o] = e;
        ETA[o] = e;
        ETA50[o] = e;
        OM[o] = OM0[o];  // :596
    }
    if (i == 0 && j == 0) {  // :599-608
        double dt = ds->dt;
        if (!ds->yndtdecrease) dt = DMAX(DMIN(dt * p.dtkoefup, p.dtelastic0), p.dtmin);
        else dt = DMAX(DMIN(dt, p.dtelastic0), p.dtmin);
        ds->dt = dt;
        ds->yndtdecrease = 0;
        ds->dt00 = dt;
        ds->ynlast = 0;
        ds->iterstep = 0;
        ds->dsylsq = 0;
        ds->dsylsq_prev = 0;
        ds->stop = 0;
        ds->loop_done = 0;
        ds->krylov_total = 0;
        ds->krylov_maxrel = 0;
        ds->iters_in_step = 0;
        ds->krylov_cycles = 0;
    }
}

// ------------------------------------------------------ a6-a7 preparation
// External P nodes: symmetry (:616-617, copy_bounds on pt and pf): a ghost
// takes the value of the nearest interior node, corners the diagonal one.
__global__ void k_copy_bounds(Geo g, double* pt, double* pf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny1) return;
    if (i != 0 && i != g.Ny && j != 0 && j != g.Nx) return;
    int is = i < 1 ? 1 : (i > g.Ny - 1 ? g.Ny - 1 : i);
    int js = j < 1 ? 1 : (j > g.Nx - 1 ? g.Nx - 1 : j);
    IS(pt, i, j) = IS(pt, is, js);
    IS(pf, i, j) = IS(pf, is, js);
}

// :620-636
__global__ void k_prep_basic(Geo g, const DevScalars* ds, hmec_params p, double* ETA, const double* __restrict__ ETA0,
                             const double* __restrict__ SXX, const double* __restrict__ SYY,
                             const double* __restrict__ SXY, double* SIIB, double* IETAPLB, double* EIIB) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    const double etamincur = ds->dt * p.shearmod * 1e-4;
    size_t o = (size_t)j * g.Ny + i;
    double eta = ETA[o];
    if (eta < etamincur) {
        eta = etamincur;
        ETA[o] = eta;
    }
    const double eta0 = ETA0[o];
    if (eta < eta0) {
        const double sxx = bsum(SXX, g.Ny1, i, j), syy = bsum(SYY, g.Ny1, i, j);
        const double sxy = SXY[o];
        const double siib = sqrt(sxy * sxy + (sxx * sxx + syy * syy + (sxx + syy) * (sxx + syy)) / 32.);
        const double ietapl = (1. / eta - 1. / eta0);
        SIIB[o] = siib;
        IETAPLB[o] = ietapl;
        EIIB[o] = g.dy_faultw * siib * ietapl / 2.;
    } else {
        EIIB[o] = 0;
        IETAPLB[o] = 0;
    }
}

// :639-669
__global__ void k_prep_p(Geo g, const DevScalars* ds, hmec_params p, const double* __restrict__ IETAPLB,
                         const double* __restrict__ YNY0, const double* __restrict__ ETAP0,
                         const double* __restrict__ ETAB0, const double* __restrict__ POR,
                         const double* __restrict__ GGGP, double* ETAP, double* ETAB, double* GGGB, double* DILP) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < 1 || i >= g.Ny || j < 1 || j >= g.Nx) return;
    const double etamincur = ds->dt * p.shearmod * 1e-4;
    const double IETAPL = bsum(IETAPLB, g.Ny, i - 1, j - 1) / 4.;
    const double por = IS(POR, i, j);
    double etap, etab;
    if (IB(YNY0, i - 1, j - 1) > 0 || IB(YNY0, i, j - 1) > 0 || IB(YNY0, i - 1, j) > 0 || IB(YNY0, i, j) > 0) {
        etap = 1. / (1. / IS(ETAP0, i, j) + IETAPL);
        etab = 1. / (1. / IS(ETAB0, i, j) + g.dy_faultw * IETAPL * por);
    } else {
        etap = IS(ETAP0, i, j);
        etab = IS(ETAB0, i, j);
    }
    if (etap < etamincur) etap = etamincur;
    if (etab * por < etamincur) etab = etamincur / por;
    IS(ETAP, i, j) = etap;
    IS(ETAB, i, j) = etab;
    IS(GGGB, i, j) = IS(GGGP, i, j) / por;
    IS(DILP, i, j) = 0;
}

// :671-677 -- min(ETADX(1:Ny-1, 0:Nx-1)) in block partials, finished below.
__device__ __forceinline__ double block_min256(double* sh, double v) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = DMIN(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ void set_scales(const Geo& g, DevScalars* ds, double mn);

// min(ETADX) over rows 1..Ny-1 in block partials; the last block sets the
// pressure scales from it (block 256 threads).
__global__ void k_min_etadx(Geo g, const double* __restrict__ ETADX, double* part, DevScalars* ds,
                            unsigned* ticket) {
    __shared__ double sh[256];
    double mn = INFINITY;
    const int nrow = g.Ny - 1;
    const int tot = nrow * g.Nx;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += gridDim.x * blockDim.x) {
        int j = t / nrow, i = 1 + (t - j * nrow);
        mn = DMIN(mn, IS(ETADX, i, j));
    }
    mn = block_min256(sh, mn);
    if (threadIdx.x == 0) part[blockIdx.x] = mn;
    if (!arrive_last(ticket)) return;
    mn = INFINITY;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) mn = DMIN(mn, __ldcg(part + b));
    mn = block_min256(sh, mn);
    if (threadIdx.x == 0) set_scales(g, ds, mn);
}

__device__ void set_scales(const Geo& g, DevScalars* ds, double mn) {
    const double dt = ds->dt;
    double pf = (dt > 2e5) ? mn * g.dx * 1e17 / (dt * dt) : mn * g.dx;
    // The solution vector S holds pt/ptscale and pf/pfscale of the previous
    // solve; the ratio brings that warm start to the new scales.
    const double old = ds->ptscale;
    ds->guess_ratio = (old > 0.0 && isfinite(old) && isfinite(pf) && pf > 0.0) ? old / pf : 1.0;
    ds->pfscale = pf;
    ds->ptscale = pf;
}

// Warm start of the next solve in the new pressure scales (the Krylov
// solver's initial guess only; the converged solution does not depend on it).
__global__ void k_rescale_guess(Geo g, const DevScalars* ds, double* S) {
    const double r = ds->guess_ratio;
    if (r == 1.0) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= g.Ny1) return;
    const int kp = (j * g.Ny1 + i) * 6;
    S[kp] *= r;
    S[kp + 3] *= r;
}

// ------------------------------------------------------------- a9 assembly
// A row under construction: at most 11 distinct columns (the ELL width), in
// registers -- every index below is a compile-time constant after unrolling,
// so nothing goes to local memory.
constexpr int RB_CAP = 12;
struct RowB {
    int n;
    int c[RB_CAP];
    double v[RB_CAP];
    __device__ __forceinline__ void reset() {
        n = 0;
#pragma unroll
        for (int k = 0; k < RB_CAP; k++) {
            c[k] = 0;
            v[k] = 0.0;
        }
    }
    // an entry whose column the row does not hold yet (interior rows: their
    // stencil columns are distinct), appended without a search -- no FP64
    // operation, the arrays stay in registers
    __device__ __forceinline__ void put(int col, double val) {
#pragma unroll
        for (int k = 0; k < RB_CAP; k++) {
            const bool at = k == n;
            c[k] = at ? col : c[k];
            v[k] = at ? val : v[k];
        }
        n++;
    }
    // duplicates summed in insertion order (setFromTriplets; the boundary
    // rows' branches can add a column twice); branch-free, so the arrays stay
    // in registers
    __device__ __forceinline__ void add(int col, double val) {
        bool dup = false;
#pragma unroll
        for (int k = 0; k < RB_CAP; k++) {
            const bool hit = k < n && c[k] == col;
            v[k] = hit ? v[k] + val : v[k];
            dup = dup || hit;
        }
#pragma unroll
        for (int k = 0; k < RB_CAP; k++) {
            const bool put = !dup && k == n;
            c[k] = put ? col : c[k];
            v[k] = put ? val : v[k];
        }
        n += dup ? 0 : 1;
    }
};

// Write one row into the slot-major ELL arrays, sorted by column, padded
// with (row, 0); the row scale is the power of two that brings max|a| into
// [0.5, 1), so scaling is exact.
__device__ __forceinline__ void emit_row(RowB& rb, int row, int N, int32_t* col, double* val, double* dscale,
                                         double* rhs_scaled, double* rhs_raw, double rhs) {
    // frexp's exponent of max|a| from the largest biased exponent (integer
    // pipe); zeros, subnormals, infinities and NaN take the FP64 route
    int emax = 0;
#pragma unroll
    for (int k = 0; k < RB_CAP; k++)
        if (k < rb.n) emax = max(emax, (int)((__double_as_longlong(rb.v[k]) >> 52) & 0x7FF));
    double s = 1.0;
    if (emax >= 1 && emax <= 2044) {
        s = __longlong_as_double((long long)(2045 - emax) << 52);  // 2^-(emax - 1022)
    } else {
        double mx = 0;
#pragma unroll
        for (int k = 0; k < RB_CAP; k++)
            if (k < rb.n) mx = DMAX(mx, fabs(rb.v[k]));
        if (mx > 0 && isfinite(mx)) {
            int e;
            frexp(mx, &e);
            s = ldexp(1.0, -e);
        }
    }
    // sort by column: odd-even transposition over the fixed width, unused
    // entries last (columns are distinct, so the order is the sorted one)
#pragma unroll
    for (int k = 0; k < RB_CAP; k++)
        if (k >= rb.n) rb.c[k] = 0x7FFFFFFF;
#pragma unroll
    for (int pass = 0; pass < RB_CAP; pass++) {
#pragma unroll
        for (int k = pass & 1; k + 1 < RB_CAP; k += 2) {
            if (rb.c[k] > rb.c[k + 1]) {
                const int tc = rb.c[k];
                rb.c[k] = rb.c[k + 1];
                rb.c[k + 1] = tc;
                const double tv = rb.v[k];
                rb.v[k] = rb.v[k + 1];
                rb.v[k + 1] = tv;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < HMEC_W; k++) {
        const size_t o = (size_t)k * N + row;
        if (k < rb.n) {
            col[o] = rb.c[k];
            val[o] = rb.v[k] * s;
        } else {
            col[o] = row;
            val[o] = 0.0;
        }
    }
    dscale[row] = s;
    if (rhs_scaled) rhs_scaled[row] = rhs * s;
    if (rhs_raw) rhs_raw[row] = rhs;
}

// One thread per staggered cell (i, j): the six equations of :698-980.
__global__ void k_assemble(Geo g, AsmFields F, const DevScalars* ds, hmec_params p, int32_t* col, double* val,
                           double* dscale, double* rhs_scaled, double* rhs_raw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    // blockIdx.z: which of the cell's six rows this thread assembles (Pt,
    // vx, vy, Pf, vxD, vyD); the rows are independent.  (With the row kind
    // as the fastest grid index instead, the interleaved rows' sectors leave
    // L2 filled -- a quarter of the DRAM traffic -- but the kernel, bound by
    // the FP64 pipe, ran 8 % slower.)
    const int sec = blockIdx.z;
    if (i >= g.Ny1) return;
    const int Nx = g.Nx, Ny = g.Ny, Ny1 = g.Ny1, N = g.N;
    // the reference divides by the grid constants and dt; the matrix entries
    // multiply by their reciprocals instead (an ulp or two apart, ~40 FP64
    // divisions per cell saved), the right-hand sides, which can cancel
    // strongly, keep the reference's divisions
    const double idx = g.idx, idy = g.idy, idx2 = g.idx2, idy2 = g.idy2, idx_dy = g.idx_dy;
    const double dt = ds->dt, ptscale = ds->ptscale, pfscale = ds->pfscale;
    const double idt = 1. / dt;
    const double gx = p.gx, gy = p.gy, inertia = p.inertia;
    const int NV = 6, RS = Ny1 * 6;
    const int kp = (j * Ny1 + i) * NV;
    const int kx = kp + 1, ky = kp + 2, kpf = kp + 3, kxf = kp + 4, kyf = kp + 5;
    const bool want_rhs = rhs_raw != nullptr;
    RowB rb;
    double r;
    if (sec == 0) {
        // 5c) Pt  :842-862
        rb.reset();
        r = 0;
        if (i == 0 || j == 0 || i == Ny || j == Nx) {
            rb.add(kp, 1);
        } else {
            const double por = IS(F.POR, i, j);
            const double BETADRAINED = (1. / IS(F.GGGB, i, j) + p.BETASOLID) / (1 - por);
            const double KBW = 1 - p.BETASOLID / BETADRAINED;
            const double ietab = 1. / IS(F.ETAB, i, j) / (1 - por);
            rb.put(kx - RS, -idx);
            rb.put(kx, idx);
            rb.put(ky - NV, -idy);
            rb.put(ky, idy);
            rb.put(kp, ptscale * (ietab + BETADRAINED * idt));
            rb.put(kpf, -pfscale * (ietab + BETADRAINED * KBW * idt));
            if (want_rhs) r = BETADRAINED * (IS(F.PT0, i, j) - KBW * IS(F.PF0, i, j)) / dt + IS(F.DILP, i, j);
        }
        emit_row(rb, kp, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
    if (sec == 1) {
        // 5a) vxs  :698-768
        rb.reset();
        r = 0;
        if (i == 0 || i == Ny || j == 0 || j >= Nx - 1) {
            if (j == Nx) rb.add(kx, 1);
            if (i == 0 && j < Nx) {
                rb.add(kx, 1);
                rb.add(kx + NV, 1);
                r = 2 * p.bcupper;
            }
            if (i == Ny && j < Nx) {
                rb.add(kx, 1);
                rb.add(kx - NV, 1);
                r = 2 * p.bclower;
            }
            if (j == 0 && i > 0 && i < Ny) {
                rb.add(kx, 1);
                rb.add(kx + RS, -1);
            }
            if (j == Nx - 1 && i > 0 && i < Ny) {
                rb.add(kx, 1);
                rb.add(kx - RS, -1);
            }
        } else {
            double ETAXY1 = IB(F.ETA, i - 1, j), ETAXY2 = IB(F.ETA, i, j);
            double ETAXX1 = IS(F.ETAP, i, j), ETAXX2 = IS(F.ETAP, i, j + 1);
            const double GXY1 = IB(F.GGG, i - 1, j), GXY2 = IB(F.GGG, i, j);
            const double GXX1 = IS(F.GGGP, i, j), GXX2 = IS(F.GGGP, i, j + 1);
            const double KXY1 = divplus(dt * GXY1, ETAXY1), KXY2 = divplus(dt * GXY2, ETAXY2);
            const double KXX1 = divplus(dt * GXX1, ETAXX1), KXX2 = divplus(dt * GXX2, ETAXX2);
            ETAXY1 *= KXY1;
            ETAXY2 *= KXY2;
            ETAXX1 *= KXX1;
            ETAXX2 *= KXX2;
            const double dRHOdx = (IS(F.RHOX, i, j + 1) - IS(F.RHOX, i, j - 1)) * g.i2dx;
            const double dRHOdy = (IB(F.RHO, i, j) - IB(F.RHO, i - 1, j)) * idy;
            const double temp = gx * dt * dRHOdy / 4.;
            rb.put(kx, -(ETAXX1 + ETAXX2) * idx2 - (ETAXY1 + ETAXY2) * idy2 - gx * dt * dRHOdx - inertia * IS(F.RHOX, i, j) * idt);
            rb.put(kx - RS, ETAXX1 * idx2);
            rb.put(kx + RS, ETAXX2 * idx2);
            rb.put(kx - NV, ETAXY1 * idy2);
            rb.put(kx + NV, ETAXY2 * idy2);
            rb.put(ky - NV, (ETAXY1 - ETAXX1) * idx_dy - temp);
            rb.put(ky, (ETAXX1 - ETAXY2) * idx_dy - temp);
            rb.put(ky - NV + RS, (ETAXX2 - ETAXY1) * idx_dy - temp);
            rb.put(ky + RS, (ETAXY2 - ETAXX2) * idx_dy - temp);
            rb.put(kp, ptscale * idx);
            rb.put(kp + RS, -ptscale * idx);
            if (want_rhs) {
                const double SXY1 = IB(F.SXY0, i - 1, j) * (1 - KXY1), SXY2 = IB(F.SXY0, i, j) * (1 - KXY2);
                const double SXX1 = IS(F.SXX0, i, j) * (1 - KXX1), SXX2 = IS(F.SXX0, i, j + 1) * (1 - KXX2);
                r = -IS(F.RHOX, i, j) * (inertia * IS(F.VX0, i, j) / dt + gx) - (SXX2 - SXX1) / g.dx - (SXY2 - SXY1) / g.dy;
            }
        }
        emit_row(rb, kx, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
    if (sec == 2) {
        // 5b) vys  :770-840
        rb.reset();
        r = 0;
        if (j == 0 || j == Nx || i == 0 || i >= Ny - 1) {
            if (i == Ny) rb.add(ky, 1);
            if (j == 0) {
                rb.add(ky, 1);
                rb.add(ky + RS, 1);
            }
            if (j == Nx) {
                rb.add(ky, 1);
                rb.add(ky - RS, 1);
            }
            if (i == 0 && j > 0 && j < Nx) rb.add(ky, 1);
            if (i == Ny - 1 && j > 0 && j < Nx) rb.add(ky, 1);
        } else {
            double ETAXY1 = IB(F.ETA, i, j - 1), ETAXY2 = IB(F.ETA, i, j);
            double ETAYY1 = IS(F.ETAP, i, j), ETAYY2 = IS(F.ETAP, i + 1, j);
            const double GXY1 = IB(F.GGG, i, j - 1), GXY2 = IB(F.GGG, i, j);
            const double GYY1 = IS(F.GGGP, i, j), GYY2 = IS(F.GGGP, i + 1, j);
            const double KXY1 = divplus(dt * GXY1, ETAXY1), KXY2 = divplus(dt * GXY2, ETAXY2);
            const double KYY1 = divplus(dt * GYY1, ETAYY1), KYY2 = divplus(dt * GYY2, ETAYY2);
            ETAXY1 *= KXY1;
            ETAXY2 *= KXY2;
            ETAYY1 *= KYY1;
            ETAYY2 *= KYY2;
            const double dRHOdy = (IS(F.RHOY, i + 1, j) - IS(F.RHOY, i - 1, j)) * g.i2dy;
            const double dRHOdx = (IB(F.RHO, i, j) - IB(F.RHO, i, j - 1)) * idx;
            const double temp = gy * dt * dRHOdx / 4.;
            rb.put(ky, -(ETAYY1 + ETAYY2) * idy2 - (ETAXY1 + ETAXY2) * idx2 - gy * dt * dRHOdy - inertia * IS(F.RHOY, i, j) * idt);
            rb.put(ky - RS, ETAXY1 * idx2);
            rb.put(ky + RS, ETAXY2 * idx2);
            rb.put(ky - NV, ETAYY1 * idy2);
            rb.put(ky + NV, ETAYY2 * idy2);
            rb.put(kx - RS, (ETAXY1 - ETAYY1) * idx_dy - temp);
            rb.put(kx + NV - RS, (ETAYY2 - ETAXY1) * idx_dy - temp);
            rb.put(kx, (ETAYY1 - ETAXY2) * idx_dy - temp);
            rb.put(kx + NV, (ETAXY2 - ETAYY2) * idx_dy - temp);
            rb.put(kp, ptscale * idy);
            rb.put(kp + NV, -ptscale * idy);
            if (want_rhs) {
                const double SXY1 = IB(F.SXY0, i, j - 1) * (1 - KXY1), SXY2 = IB(F.SXY0, i, j) * (1 - KXY2);
                const double SYY1 = IS(F.SYY0, i, j) * (1 - KYY1), SYY2 = IS(F.SYY0, i + 1, j) * (1 - KYY2);
                r = -IS(F.RHOY, i, j) * (inertia * IS(F.VY0, i, j) / dt + gy) - (SYY2 - SYY1) / g.dy - (SXY2 - SXY1) / g.dx;
            }
        }
        emit_row(rb, ky, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
    if (sec == 3) {
        // 5f) Pf  :951-980
        rb.reset();
        r = 0;
        if (j == 0 || j == Nx || i <= 1 || i >= Ny - 1) {
            if (i == 1 || i == Ny - 1) {
                rb.add(kpf, pfscale);
                rb.add(kp, -ptscale);
                r = -p.PTFDIFF;
            } else {
                rb.add(kpf, 1);
            }
        } else {
            const double por = IS(F.POR, i, j);
            const double BETADRAINED = (1 / IS(F.GGGB, i, j) + p.BETASOLID) / (1 - por);
            const double KBW = 1 - p.BETASOLID / BETADRAINED;
            const double KSK = (BETADRAINED - p.BETASOLID) / (BETADRAINED - p.BETASOLID + por * (p.BETAFLUID - p.BETASOLID));
            const double ietab = 1 / IS(F.ETAB, i, j) / (1 - por);
            rb.put(kxf - RS, -idx);
            rb.put(kxf, idx);
            rb.put(kyf - NV, -idy);
            rb.put(kyf, idy);
            rb.put(kp, -ptscale * (ietab + BETADRAINED * KBW * idt));
            rb.put(kpf, pfscale * (ietab + BETADRAINED * KBW / KSK * idt));
            if (want_rhs) r = -BETADRAINED * KBW * (IS(F.PT0, i, j) - 1. / KSK * IS(F.PF0, i, j)) / dt - IS(F.DILP, i, j);
        }
        emit_row(rb, kpf, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
    if (sec == 4) {
        // 5d) vxD  :864-903
        rb.reset();
        r = 0;
        if (i == 0 || i == Ny || j == 0 || j >= Nx - 1) {
            if (j == Nx) rb.add(kxf, 1);
            if (i == 0 && j < Nx) {
                rb.add(kxf, 1);
                rb.add(kxf + NV, -1);
            }
            if (i == Ny && j < Nx) {
                rb.add(kxf, 1);
                rb.add(kxf - NV, -1);
            }
            if (j == 0) rb.add(kxf, 1);
            if (j == Nx - 1) rb.add(kxf, 1);
        } else {
            rb.put(kxf, -IS(F.ETADX, i, j) - IS(F.RHOFX, i, j) / IS(F.PORX, i, j) * inertia * idt);
            rb.put(kx, -IS(F.RHOFX, i, j) * inertia * idt);
            rb.put(kpf, pfscale * idx);
            rb.put(kpf + RS, -pfscale * idx);
            if (want_rhs) r = -IS(F.RHOFX, i, j) * (inertia * IS(F.VXF0, i, j) / dt + gx);
        }
        emit_row(rb, kxf, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
    if (sec == 5) {
        // 5e) vyD  :905-949
        rb.reset();
        r = 0;
        if (j == 0 || j == Nx || i == 0 || i >= Ny - 1) {
            if (i == Ny) rb.add(kyf, 1);
            if (j == 0 && i > 0 && i < Ny - 1) {
                rb.add(kyf, 1);
                rb.add(kyf + RS, -1);
            }
            if (j == Nx && i > 0 && i < Ny - 1) {
                rb.add(kyf, 1);
                rb.add(kyf - RS, -1);
            }
            if (i == 0) {
                rb.add(kyf, 1);
                r = p.bcvyflower;
            }
            if (i == Ny - 1) {
                rb.add(kyf, 1);
                r = p.bcvyflower;
            }
        } else {
            rb.put(kyf, -IS(F.ETADY, i, j) - IS(F.RHOFY, i, j) / IS(F.PORY, i, j) * inertia * idt);
            rb.put(ky, -IS(F.RHOFY, i, j) * inertia * idt);
            rb.put(kpf, pfscale * idy);
            rb.put(kpf + NV, -pfscale * idy);
            if (want_rhs) r = -IS(F.RHOFY, i, j) * (inertia * IS(F.VYF0, i, j) / dt + gy);
        }
        emit_row(rb, kyf, N, col, val, dscale, rhs_scaled, rhs_raw, r);
    }
}

// --------------------------------------------------------- a11 reload
// :1060-1075, and Vmax = max(VSLIPB) (:1077) in block partials.
__global__ void k_reload(Geo g, const DevScalars* ds, const double* __restrict__ S, double* pt, double* vxs,
                         double* vys, double* pf, double* vxD, double* vyD, int* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny1) return;
    const int kp = (j * g.Ny1 + i) * 6;
    size_t o = (size_t)j * g.Ny1 + i;
    double s0 = S[kp], s1 = S[kp + 1], s2 = S[kp + 2], s3 = S[kp + 3], s4 = S[kp + 4], s5 = S[kp + 5];
    if (!isfinite(s0) || !isfinite(s1) || !isfinite(s2) || !isfinite(s3) || !isfinite(s4) || !isfinite(s5))
        atomicOr(status, HMEC_DEV_NAN);
    pt[o] = s0 * ds->ptscale;
    vxs[o] = s1;
    vys[o] = s2;
    pf[o] = s3 * ds->pfscale;
    vxD[o] = s4;
    vyD[o] = s5;
}

__device__ __forceinline__ double block_max256(double* sh, double v) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] = DMAX(sh[threadIdx.x], sh[threadIdx.x + s]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Vmax = max(VSLIPB) (:1077): block partials, the last block finishes (256 threads).
__global__ void k_vmax(Geo g, const double* __restrict__ VSLIPB, DevScalars* ds, double* part, unsigned* ticket) {
    __shared__ double sh[256];
    double mx = -INFINITY;
    const int nb = g.Nx * g.Ny;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x) mx = DMAX(mx, VSLIPB[t]);
    mx = block_max256(sh, mx);
    if (threadIdx.x == 0) part[blockIdx.x] = mx;
    if (!arrive_last(ticket)) return;
    mx = -INFINITY;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) mx = DMAX(mx, __ldcg(part + b));
    mx = block_max256(sh, mx);
    if (threadIdx.x == 0) ds->Vmax = mx;
}

// ---------------------------------------------------------- a12 stress
// Basic nodes :1102-1107, fused with the RSF resets of :1154-1163.
__global__ void k_stress_basic(Geo g, const DevScalars* ds, const double* __restrict__ vxs,
                               const double* __restrict__ vys, const double* __restrict__ GGG,
                               const double* __restrict__ ETA, const double* __restrict__ SXY0, double* EXY,
                               double* SXY, const double* __restrict__ ETA0, double* ETA5, double* DSY, double* YNY,
                               double* SigmaY, double* SII_fault, const double* __restrict__ OM, double* OM5) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    size_t o = (size_t)j * g.Ny + i;
    const double dt = ds->dt;
    const double exy = .5 * ((IS(vxs, i + 1, j) - IS(vxs, i, j)) / g.dy + (IS(vys, i, j + 1) - IS(vys, i, j)) / g.dx);
    const double KXY = divplus(dt * GGG[o], ETA[o]);
    EXY[o] = exy;
    SXY[o] = 2 * ETA[o] * exy * KXY + SXY0[o] * (1 - KXY);
    ETA5[o] = ETA0[o];
    DSY[o] = 0;
    YNY[o] = 0;
    SigmaY[o] = 0;
    SII_fault[o] = 0;
    OM5[o] = OM[o];
}

// Pressure cells :1118-1127 (ghost rows/cols of SXX, SYY untouched: Q2).
__global__ void k_stress_p(Geo g, const DevScalars* ds, const double* __restrict__ vxs, const double* __restrict__ vys,
                           const double* __restrict__ GGGP, const double* __restrict__ ETAP,
                           const double* __restrict__ SXX0, const double* __restrict__ SYY0, double* EXX, double* EYY,
                           double* SXX, double* SYY) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < 1 || i >= g.Ny || j < 1 || j >= g.Nx) return;
    const double dt = ds->dt;
    const double dvx = IS(vxs, i, j) - IS(vxs, i, j - 1), dvy = IS(vys, i, j) - IS(vys, i - 1, j);
    const double exx = (2 * dvx / g.dx - dvy / g.dy) / 3.;
    const double eyy = (2 * dvy / g.dy - dvx / g.dx) / 3.;
    const double etap = IS(ETAP, i, j);
    const double KXX = divplus(dt * IS(GGGP, i, j), etap);
    IS(EXX, i, j) = exx;
    IS(EYY, i, j) = eyy;
    IS(SXX, i, j) = 2 * etap * exx * KXX + IS(SXX0, i, j) * (1 - KXX);
    IS(SYY, i, j) = 2 * etap * eyy * KXX + IS(SYY0, i, j) * (1 - KXX);
}

// ------------------------------------------------------------ a13 RSF
struct RsfIn {
    const double *ARSF, *BRSF, *LRSF, *FRIC, *ETA0, *SXX, *SYY, *SXY, *GGG, *ETA, *OM, *OM0, *pt, *pf, *YNY0;
};
struct RsfOut {
    double *SIIB, *OM5, *SigmaY, *VSLIPB, *SII_fault, *DSY, *YNY, *ETA5;
    double* buf;  // [3][Nx]: counted?, DSY^2, dt candidate
};

// One thread per node of the fault row i = line_fault (:1169-1305).
__global__ void k_rsf(Geo g, const DevScalars* ds, hmec_params p, RsfIn in, RsfOut out, int* status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.Nx) return;
    double* cnt = out.buf;
    double* dd = out.buf + g.Nx;
    double* dtl = out.buf + 2 * g.Nx;
    if (!(ds->timestep > p.tyield)) {
        cnt[j] = 0;
        dd[j] = 0;
        dtl[j] = 1e7;
        return;
    }
    const int i = g.line_fault;
    const size_t o = (size_t)j * g.Ny + i;
    const double dt = ds->dt, dx = g.dx, V0 = p.V0;
    const double arsf = in.ARSF[o], brsf = in.BRSF[o], lrsf = in.LRSF[o], fric = in.FRIC[o], eta0 = in.ETA0[o];
    const double sxx = bsum(in.SXX, g.Ny1, i, j), syy = bsum(in.SYY, g.Ny1, i, j), sxy = in.SXY[o];
    const double siib = sqrt(sxy * sxy + (sxx * sxx + syy * syy + (sxx + syy) * (sxx + syy)) / 32.);
    out.SIIB[o] = siib;
    const double G = in.GGG[o], ETAij = in.ETA[o], OMij = in.OM[o];
    const double siiel = siib / (ETAij / (G * dt + ETAij));
    const double prB_temp = (bsum(in.pt, g.Ny1, i, j) - bsum(in.pf, g.Ny1, i, j)) / 4.;
    double prB = prB_temp;
    if (prB < 1e3) prB = 1e3;
    double SIIB1 = siib;
    const double eom = exp(-(brsf * OMij + fric) / arsf);
    double EIISLIP = V0 * sinh(DMAX(SIIB1, 0.) / arsf / prB) * eom / dx;
    double ETAPL = SIIB1 / 2. / EIISLIP;
    double ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
    double SIIB2 = siiel * ETAVP / (G * dt + ETAVP);
    const double DSIIB1 = SIIB2 - SIIB1;
    double V = 2 * V0 * sinh(DMAX(SIIB2, 0.) / arsf / prB) * eom;
    EIISLIP = V / dx / 2.;
    ETAPL = SIIB2 / 2. / EIISLIP;
    ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
    const double DSIIB2 = siiel * ETAVP / (G * dt + ETAVP) - SIIB2;
    double SIIB4 = 0.;
    if ((DSIIB1 >= 0 && DSIIB2 <= 0) || (DSIIB1 <= 0 && DSIIB2 >= 0)) {  // :1221-1243
        double DSIIB = 1e9;
        int it = 0;
        while (fabs(DSIIB) > 1e-3) {
            if (it++ >= p.rsf_maxit) {  // the reference loops without a cap
                atomicOr(status, HMEC_DEV_RSF_NOCONV);
                break;
            }
            SIIB4 = (SIIB1 + SIIB2) / 2.;
            V = 2 * V0 * sinh(DMAX(SIIB4, 0.) / arsf / prB) * eom;
            EIISLIP = V / dx / 2.;
            ETAPL = SIIB4 / 2. / EIISLIP;
            ETAVP = 1. / (1. / eta0 + 1. / ETAPL);
            DSIIB = siiel * ETAVP / (G * dt + ETAVP) - SIIB4;
            if ((DSIIB >= 0 && DSIIB1 >= 0) || (DSIIB <= 0 && DSIIB1 <= 0)) SIIB1 = SIIB4;
            else SIIB2 = SIIB4;
        }
    }
    double om5;  // aging law :1245-1249
    if (V * dt / lrsf > 1e-6) om5 = log(V0 / V + (exp(in.OM0[o]) - V0 / V) * exp(-V * dt / lrsf));
    else om5 = log(exp(in.OM0[o]) * (1 - V * dt / lrsf) + V0 * dt / lrsf);
    out.OM5[o] = om5;
    const double syield = DMAX(p.syieldmin, prB_temp * arsf * asinh(V / 2. / V0 * exp((brsf * om5 + fric) / arsf)));
    out.SigmaY[o] = syield;
    out.VSLIPB[o] = V;
    out.SII_fault[o] = SIIB4;
    const double g_temp = 2 * G;  // Lapusta timestep :1263-1273
    const double k = g_temp / (M_PI * (1 - ((3. / p.BETASOLID - g_temp) / (6. / p.BETASOLID + g_temp))) * dx);
    double dTETAmax;
    const double q = (k * lrsf / prB - brsf) / arsf - 1;
    if ((q * q / 4. - k * lrsf / arsf / prB) < 0) dTETAmax = DMIN(1. - (brsf - arsf) * prB / (k * lrsf), .2);
    else dTETAmax = DMIN(arsf * prB / (k * lrsf - (brsf - arsf) * prB), .2);
    dtl[j] = dTETAmax * lrsf / V;
    double counted = 0, dsy2 = 0;
    bool ynn = false;
    if (in.YNY0[o] > 0) {  // :1276-1282
        ynn = true;
        const double dsy = siib - syield;
        out.DSY[o] = dsy;
        dsy2 = dsy * dsy;
        counted = 1;
    }
    const double A = syield / siiel;  // :1285-1304
    double eta5 = eta0;
    if (A < 1) {
        const double etapl = dt * G * A / (1 - A);
        if (etapl < eta0) {
            eta5 = pow(etapl, 1 - p.etawt) * pow(ETAij, p.etawt);
            out.YNY[o] = 1;
            if (!ynn) {
                const double dsy = siib - syield;
                out.DSY[o] = dsy;
                dsy2 = dsy * dsy;
                counted = 1;
            }
        }
    }
    out.ETA5[o] = eta5;
    cnt[j] = counted;
    dd[j] = dsy2;
}

// ------------------------------------------------ a14 reductions + control
// Block partials over the staggered grid: max/min of vxs, vys, the
// fault-band maxima of |vxs|, |vys|, and min dx*stpmax/VSLIPB over the basic grid.
constexpr int NRED = 7;
__device__ void control_update(const Geo& g, DevScalars* ds, const hmec_params& p, const double* red, int ynpl,
                               double ddd, double dtlapusta);

// Velocity extrema and the slip-limited dt over the grid in block partials
// (256 threads); the last block finishes them and runs the timestep control.
__global__ void k_reduce_vel(Geo g, hmec_params p, const double* __restrict__ yvx, const double* __restrict__ yvy,
                             const double* __restrict__ vxs, const double* __restrict__ vys,
                             const double* __restrict__ VSLIPB, double* part, const double* __restrict__ rsfbuf,
                             DevScalars* ds, unsigned* ticket) {
    __shared__ double sh[NRED][256];
    double a[NRED] = {-INFINITY, INFINITY, -INFINITY, INFINITY, 0.0, 0.0, 1e30};
    const int ns = g.Nx1 * g.Ny1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ns; t += gridDim.x * blockDim.x) {
        const int i = t - (t / g.Ny1) * g.Ny1;
        const double vx = vxs[t], vy = vys[t];
        a[0] = DMAX(a[0], vx);
        a[1] = DMIN(a[1], vx);
        a[2] = DMAX(a[2], vy);
        a[3] = DMIN(a[3], vy);
        if (yvx[i] >= g.upper_block && yvx[i] <= g.lower_block) a[4] = DMAX(a[4], fabs(vx));
        if (yvy[i] >= g.upper_block && yvy[i] <= g.lower_block) a[5] = DMAX(a[5], fabs(vy));
    }
    const long long nb = (long long)g.Nx * g.Ny;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += (long long)gridDim.x * blockDim.x) {
        const double v = VSLIPB[t];
        if (v > 0) a[6] = DMIN(a[6], g.dx * p.stpmax / v);
    }
    for (int q = 0; q < NRED; q++) sh[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sh[0][threadIdx.x] = DMAX(sh[0][threadIdx.x], sh[0][threadIdx.x + s]);
            sh[1][threadIdx.x] = DMIN(sh[1][threadIdx.x], sh[1][threadIdx.x + s]);
            sh[2][threadIdx.x] = DMAX(sh[2][threadIdx.x], sh[2][threadIdx.x + s]);
            sh[3][threadIdx.x] = DMIN(sh[3][threadIdx.x], sh[3][threadIdx.x + s]);
            sh[4][threadIdx.x] = DMAX(sh[4][threadIdx.x], sh[4][threadIdx.x + s]);
            sh[5][threadIdx.x] = DMAX(sh[5][threadIdx.x], sh[5][threadIdx.x + s]);
            sh[6][threadIdx.x] = DMIN(sh[6][threadIdx.x], sh[6][threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < NRED; q++) part[blockIdx.x * NRED + q] = sh[q][0];
    if (!arrive_last(ticket)) return;
    // last block: combine the partials, then the fault bookkeeping and the
    // timestep control (one thread)
    a[0] = -INFINITY, a[1] = INFINITY, a[2] = -INFINITY, a[3] = INFINITY, a[4] = 0.0, a[5] = 0.0, a[6] = 1e30;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        double v[NRED];
        for (int q = 0; q < NRED; q++) v[q] = __ldcg(part + b * NRED + q);
        a[0] = DMAX(a[0], v[0]);
        a[1] = DMIN(a[1], v[1]);
        a[2] = DMAX(a[2], v[2]);
        a[3] = DMIN(a[3], v[3]);
        a[4] = DMAX(a[4], v[4]);
        a[5] = DMAX(a[5], v[5]);
        a[6] = DMIN(a[6], v[6]);
    }
    int cnt = 0;
    double dtl = 1e7;
    for (int j = threadIdx.x; j < g.Nx; j += blockDim.x) {
        if (rsfbuf[j] != 0) cnt++;
        dtl = DMIN(dtl, rsfbuf[2 * g.Nx + j]);
    }
    __syncthreads();
    for (int q = 0; q < NRED; q++) sh[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sh[0][threadIdx.x] = DMAX(sh[0][threadIdx.x], sh[0][threadIdx.x + s]);
            sh[1][threadIdx.x] = DMIN(sh[1][threadIdx.x], sh[1][threadIdx.x + s]);
            sh[2][threadIdx.x] = DMAX(sh[2][threadIdx.x], sh[2][threadIdx.x + s]);
            sh[3][threadIdx.x] = DMIN(sh[3][threadIdx.x], sh[3][threadIdx.x + s]);
            sh[4][threadIdx.x] = DMAX(sh[4][threadIdx.x], sh[4][threadIdx.x + s]);
            sh[5][threadIdx.x] = DMAX(sh[5][threadIdx.x], sh[5][threadIdx.x + s]);
            sh[6][threadIdx.x] = DMIN(sh[6][threadIdx.x], sh[6][threadIdx.x + s]);
        }
        __syncthreads();
    }
    double red[NRED];
    for (int q = 0; q < NRED; q++) red[q] = sh[q][0];
    __syncthreads();
    __shared__ int s_cnt;
    if (threadIdx.x == 0) s_cnt = 0;
    sh[0][threadIdx.x] = dtl;
    __syncthreads();
    atomicAdd(&s_cnt, cnt);
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[0][threadIdx.x] = DMIN(sh[0][threadIdx.x], sh[0][threadIdx.x + s]);
        __syncthreads();
    }
    const double dtlapusta = sh[0][0];
    const int ynpl = s_cnt;
    __syncthreads();
    // ddd: sequential sum in j order, staged through shared memory in chunks
    double* stage = &sh[0][0];
    const int CHUNK = NRED * 256;
    double ddd = 0;
    for (int j0 = 0; j0 < g.Nx; j0 += CHUNK) {
        const int n = g.Nx - j0 < CHUNK ? g.Nx - j0 : CHUNK;
        for (int t = threadIdx.x; t < n; t += blockDim.x)
            stage[t] = rsfbuf[j0 + t] != 0 ? rsfbuf[g.Nx + j0 + t] : 0.0;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int t = 0; t < n; t++) ddd += stage[t];
        __syncthreads();
    }
    if (threadIdx.x == 0) control_update(g, ds, p, red, ynpl, ddd, dtlapusta);
}

// :1310-1456 on one thread, from the reduced velocity extrema red[NRED] and
// the fault bookkeeping (ynpl, ddd summed in the reference's j order,
// dtlapusta).
__device__ void control_update(const Geo& g, DevScalars* ds, const hmec_params& p, const double* red, int ynpl,
                               double ddd, double dtlapusta) {
    const double vxmax = red[0], vxmin = red[1], vymax = red[2], vymin = red[3], bx = red[4], by = red[5];
    double dtslip = red[6];
    const int iterstep = ds->iterstep;
    int ynlast = ds->ynlast;
    double dt = ds->dt;
    double dsylsq = 0;
    if (ynpl > 0) dsylsq = sqrt(ddd / ynpl);
    const double D_iter = dsylsq;
    double D_iter_quot = 0;
    if (iterstep != 0) D_iter_quot = D_iter / ds->dsylsq_prev;
    bool yn = false;
    double dtpl = dt;
    if (ynpl > 0 && iterstep < p.niterglobal && ynlast >= p.dtstep &&
        (ynlast > p.ynlastmax || log10(D_iter_quot) >= 0 ||
         log10(D_iter_quot) > log10(p.errmin / D_iter) / (double)(p.ynlastmax - ynlast))) {
        dtpl = dt / p.dtkoef;
        yn = true;
    }
    if (iterstep > 0) ds->maxvxy0 = ds->maxvxy;
    double maxvxs = DMAX(vxmax, fabs(vxmin));
    double maxvys = DMAX(vymax, fabs(vymin));
    const double maxvxy = sqrt((vxmax - vxmin) * (vxmax - vxmin) + (vymax - vymin) * (vymax - vymin));
    ds->maxvxy = maxvxy;
    double stpmaxcur = p.stpmax1;
    double dtx = dt;
    if (dt > g.dx * stpmaxcur / maxvxs) {
        dtx = g.dx / p.dtkoefv * stpmaxcur / maxvxs;
        yn = true;
    }
    double dty = dt;
    if (dt > g.dy * stpmaxcur / maxvys) {
        dty = g.dy / p.dtkoefv * stpmaxcur / maxvys;
        yn = true;
    }
    maxvxs = bx;
    maxvys = by;
    stpmaxcur = p.stpmax;
    if (dt > g.dx * stpmaxcur / maxvxs) {
        dtx = g.dx / p.dtkoefv * stpmaxcur / maxvxs;
        yn = true;
    }
    if (dt > g.dy * stpmaxcur / maxvys) {
        dty = g.dy / p.dtkoefv * stpmaxcur / maxvys;
        yn = true;
    }
    if (ynpl > 0 && dtslip < dt) {
        yn = true;
        dtslip = dtslip / p.dtkoefv;
    }
    if (yn && dt > p.dtmin) {
        const double dtold = dt;
        dt = DMAX(DMIN(DMIN(dtx, dty), DMIN(DMIN(dtpl, dtslip), dtlapusta)), p.dtmin);
        if (dt < dtold) ynlast = 0;
    } else {
        yn = false;
    }
    double vratio = 0;
    if (iterstep > 0) vratio = log10(maxvxy / ds->maxvxy0);
    const bool stop = !yn && (ynpl == 0 || (dsylsq < p.errmin && iterstep > 0 && fabs(vratio) < p.vratiomax));
    ds->dt = dt;
    ds->dtx = dtx;
    ds->dty = dty;
    ds->dtlapusta = dtlapusta;
    ds->ynpl = ynpl;
    ds->dsylsq = dsylsq;
    ds->dsylsq_prev = dsylsq;
    ds->stop = stop ? 1 : 0;
    ds->iters_in_step += 1;
    if (!stop) {
        ynlast++;
        ds->iterstep = iterstep + 1;
    }
    ds->ynlast = ynlast;
    if (stop || ds->iterstep >= p.niterglobal) ds->loop_done = 1;
}

// :1315-1317 and :1440-1448
__global__ void k_eta_update(Geo g, const DevScalars* ds, hmec_params p, double* ETA, const double* __restrict__ ETA5,
                             const double* __restrict__ ETA0, double* ETA50, double* YNY0,
                             const double* __restrict__ YNY, double* OM, const double* __restrict__ OM5) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    size_t o = (size_t)j * g.Ny + i;
    if (!ds->stop) {
        const double e = DMAX(DMIN(ETA5[o], ETA0[o]), p.etamin);
        ETA[o] = e;
        ETA50[o] = e;
        YNY0[o] = YNY[o];
        OM[o] = OM5[o];
    } else if (ds->ynpl == 0) {
        ETA[o] = ETA0[o];
    }
}

// ------------------------------------------------------ a16 end of step
__global__ void k_end_scalars(DevScalars* ds) {
    if (ds->dt00 > ds->dt) ds->yndtdecrease = 1;  // :1464-1466
    ds->dt = DMIN(DMIN(ds->dtx, ds->dty), DMIN(ds->dt, ds->dtlapusta));  // :1472
    ds->timesum += ds->dt;  // :1661
    ds->iterstep = ds->stop ? ds->iterstep : ds->iterstep;
}

// a17 basic nodes :1480-1495 (with ETA00 = ETA50, OM0 = OM of :1469-1470)
__global__ void k_post_basic(Geo g, const DevScalars* ds, const double* __restrict__ vxs, const double* __restrict__ vys,
                             const double* __restrict__ GGG, const double* __restrict__ ETA,
                             const double* __restrict__ SXY0, double* ESP, double* EXY, double* SXY,
                             const double* __restrict__ ETA50, double* ETA00, const double* __restrict__ OM, double* OM0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i >= g.Ny) return;
    size_t o = (size_t)j * g.Ny + i;
    const double dt = ds->dt;
    const double dvyx = (IS(vys, i, j + 1) - IS(vys, i, j)) / g.dx, dvxy = (IS(vxs, i + 1, j) - IS(vxs, i, j)) / g.dy;
    ESP[o] = .5 * (dvyx - dvxy);
    const double exy = .5 * (dvxy + dvyx);
    EXY[o] = exy;
    const double KXY = divplus(dt * GGG[o], ETA[o]);
    SXY[o] = 2 * ETA[o] * exy * KXY + SXY0[o] * (1 - KXY);
    ETA00[o] = ETA50[o];
    OM0[o] = OM[o];
}

struct PostP {
    const double *vxs, *vys, *GGGP, *ETAP, *SXX0, *SYY0, *SXY, *EXY, *ETA, *pt, *pf, *PT0, *PF0, *ETAB, *POR, *GGGB;
    double *EXX, *EYY, *SXX, *SYY, *EII, *EIIVP, *SII, *DIS, *pt_ave, *pf_ave, *VIS_COMP, *EL_DECOM;
};

__device__ __forceinline__ double sq4(double a, double b, double c, double d) {
    return ((a * a + b * b) + c * c) + d * d;
}

// a17 pressure cells :1499-1559 (invariants and compaction are output fields)
__global__ void k_post_p(Geo g, const DevScalars* ds, hmec_params p, PostP P) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < 1 || i >= g.Ny || j < 1 || j >= g.Nx) return;
    const double dt = ds->dt;
    const double dvx = IS(P.vxs, i, j) - IS(P.vxs, i, j - 1), dvy = IS(P.vys, i, j) - IS(P.vys, i - 1, j);
    const double exx = (2 * dvx / g.dx - dvy / g.dy) / 3.;
    const double eyy = (2 * dvy / g.dy - dvx / g.dx) / 3.;
    const double etap = IS(P.ETAP, i, j);
    const double KXX = divplus(dt * IS(P.GGGP, i, j), etap);
    const double sxx = 2 * etap * exx * KXX + IS(P.SXX0, i, j) * (1 - KXX);
    const double syy = 2 * etap * eyy * KXX + IS(P.SYY0, i, j) * (1 - KXX);
    IS(P.EXX, i, j) = exx;
    IS(P.EYY, i, j) = eyy;
    IS(P.SXX, i, j) = sxx;
    IS(P.SYY, i, j) = syy;
    // the rest are output fields: with invariants_every = k > 1 the steps
    // between multiples of k write only the fault-line row
    if (p.invariants_every > 1 && ds->timestep % p.invariants_every != 0 && i != g.line_fault) return;
    const double s00 = IB(P.SXY, i - 1, j - 1), s01 = IB(P.SXY, i - 1, j), s10 = IB(P.SXY, i, j - 1), s11 = IB(P.SXY, i, j);
    const double e00 = IB(P.ETA, i - 1, j - 1), e01 = IB(P.ETA, i - 1, j), e10 = IB(P.ETA, i, j - 1), e11 = IB(P.ETA, i, j);
    IS(P.EII, i, j) = sqrt(exx * exx + sq4(IB(P.EXY, i - 1, j - 1), IB(P.EXY, i - 1, j), IB(P.EXY, i, j - 1), IB(P.EXY, i, j)) / 4.);
    const double a = sxx / (2 * etap), b = syy / (2 * etap);
    IS(P.EIIVP, i, j) = sqrt(.5 * (a * a + b * b) + sq4(s00 / e00, s01 / e01, s10 / e10, s11 / e11) / 16.);
    IS(P.SII, i, j) = sqrt(.5 * (sxx * sxx + syy * syy) + sq4(s00, s01, s10, s11) / 4.);
    const double DISXY = (s11 * s11 / e11 + s01 * s01 / e01 + s10 * s10 / e10 + s00 * s00 / e00) / 2.;
    IS(P.DIS, i, j) = sxx * sxx / (2 * etap) + syy * syy / (2 * etap) + DISXY;
    double pta, pfa, PT0a, PF0a;
    if (i < g.Ny - 1) {
        pta = (IS(P.pt, i, j) + IS(P.pt, i + 1, j)) / 2.;
        pfa = (IS(P.pf, i, j) + IS(P.pf, i + 1, j)) / 2.;
        PT0a = (IS(P.PT0, i, j) + IS(P.PT0, i + 1, j)) / 2.;
        PF0a = (IS(P.PF0, i, j) + IS(P.PF0, i + 1, j)) / 2.;
    } else {
        pta = IS(P.pt, i, j);
        pfa = IS(P.pf, i, j);
        PT0a = IS(P.PT0, i, j);
        PF0a = IS(P.PF0, i, j);
    }
    IS(P.pt_ave, i, j) = pta;
    IS(P.pf_ave, i, j) = pfa;
    const double por = IS(P.POR, i, j);
    IS(P.VIS_COMP, i, j) = (pta - pfa) / (IS(P.ETAB, i, j) * (1 - por));
    const double BETADRAINED = (1 / IS(P.GGGB, i, j) + p.BETASOLID) / (1 - por);
    const double KBW = 1 - p.BETASOLID / BETADRAINED;
    IS(P.EL_DECOM, i, j) = BETADRAINED * (pta - PT0a - KBW * pfa + KBW * PF0a) / dt;
}

// a19 rollover monitors :1665-1696 (over i < Ny, j < Nx): block partials, the
// last block finishes (256 threads).
__global__ void k_monitors(Geo g, DevScalars* ds, const double* __restrict__ RHOX, const double* __restrict__ RHOY,
                           const double* __restrict__ vxs, const double* __restrict__ vys, double* part,
                           unsigned* ticket) {
    __shared__ double sh[4][256];
    double a0 = -1e30, a1 = 1e30, a2 = -1e30, a3 = 1e30;
    const int nb = g.Nx * g.Ny;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nb; t += gridDim.x * blockDim.x) {
        const int j = t / g.Ny, i = t - j * g.Ny;
        if (IS(RHOX, i, j) > 2000 && i != 0) {
            a0 = DMAX(a0, IS(vxs, i, j));
            a1 = DMIN(a1, IS(vxs, i, j));
        }
        if (IS(RHOY, i, j) > 2000 && j != 0) {
            a2 = DMAX(a2, IS(vys, i, j));
            a3 = DMIN(a3, IS(vys, i, j));
        }
    }
    sh[0][threadIdx.x] = a0;
    sh[1][threadIdx.x] = a1;
    sh[2][threadIdx.x] = a2;
    sh[3][threadIdx.x] = a3;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sh[0][threadIdx.x] = DMAX(sh[0][threadIdx.x], sh[0][threadIdx.x + s]);
            sh[1][threadIdx.x] = DMIN(sh[1][threadIdx.x], sh[1][threadIdx.x + s]);
            sh[2][threadIdx.x] = DMAX(sh[2][threadIdx.x], sh[2][threadIdx.x + s]);
            sh[3][threadIdx.x] = DMIN(sh[3][threadIdx.x], sh[3][threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; q++) part[blockIdx.x * 4 + q] = sh[q][0];
    if (!arrive_last(ticket)) return;
    a0 = -1e30, a1 = 1e30, a2 = -1e30, a3 = 1e30;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        a0 = DMAX(a0, __ldcg(part + b * 4));
        a1 = DMIN(a1, __ldcg(part + b * 4 + 1));
        a2 = DMAX(a2, __ldcg(part + b * 4 + 2));
        a3 = DMIN(a3, __ldcg(part + b * 4 + 3));
    }
    a0 = block_max256(sh[0], a0);
    a1 = block_min256(sh[1], a1);
    a2 = block_max256(sh[2], a2);
    a3 = block_min256(sh[3], a3);
    if (threadIdx.x == 0) {
        ds->maxvxsmod = a0;
        ds->minvxsmod = a1;
        ds->maxvysmod = a2;
        ds->minvysmod = a3;
    }
}

struct Roll {
    const double *vxs, *vys, *vxD, *vyD, *PORX, *PORY, *SXX, *SYY, *SXY, *pt, *pf;
    double *VX0, *VY0, *VXF0, *VYF0, *SXX0, *SYY0, *SXY0, *PTF0, *PT0, *PF0;
};

// a19 copies :1672-1726
__global__ void k_rollover(Geo g, Roll R) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (i < g.Ny1) {
        size_t o = (size_t)j * g.Ny1 + i;
        const double vx = R.vxs[o], vy = R.vys[o];
        R.VX0[o] = vx;
        R.VY0[o] = vy;
        if (R.PORX[o] > 0) R.VXF0[o] = vx + R.vxD[o] / R.PORX[o];
        if (R.PORY[o] > 0) R.VYF0[o] = vy + R.vyD[o] / R.PORY[o];
        R.SXX0[o] = R.SXX[o];
        R.SYY0[o] = R.SYY[o];
        const double pt = R.pt[o], pf = R.pf[o];
        R.PTF0[o] = pt - pf;
        R.PT0[o] = pt;
        R.PF0[o] = pf;
    }
    if (i < g.Ny && j < g.Nx) {
        size_t o = (size_t)j * g.Ny + i;
        R.SXY0[o] = R.SXY[o];
    }
}

__global__ void k_next_step(DevScalars* ds) { ds->timestep += 1; }

}  // namespace

// =================================================================== host

static inline dim3 grid_b(const Geo& g, int bs) { return dim3(nblocks(g.Ny, bs), g.Nx); }
static inline dim3 grid_s(const Geo& g, int bs) { return dim3(nblocks(g.Ny1, bs), g.Nx1); }

int step_begin(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    double* const* f = ctx->f;
    HMEC_LAUNCH(ctx, k_step_begin, grid_b(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->p, f[HMEC_F_ETA0], f[HMEC_F_ETA00],
                f[HMEC_F_OM0], f[HMEC_F_ETA1], f[HMEC_F_ETA], f[HMEC_F_ETA50], f[HMEC_F_OM]);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

int iter_prepare(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    double* const* f = ctx->f;
    HMEC_LAUNCH(ctx, k_copy_bounds, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, f[HMEC_F_pt], f[HMEC_F_pf]);
    HMEC_LAUNCH(ctx, k_prep_basic, grid_b(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->p, f[HMEC_F_ETA], f[HMEC_F_ETA0],
                f[HMEC_F_SXX], f[HMEC_F_SYY], f[HMEC_F_SXY], f[HMEC_F_SIIB], f[HMEC_F_IETAPLB], f[HMEC_F_EIIB]);
    HMEC_LAUNCH(ctx, k_prep_p, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->p, f[HMEC_F_IETAPLB], f[HMEC_F_YNY0],
                f[HMEC_F_ETAP0], f[HMEC_F_ETAB0], f[HMEC_F_POR], f[HMEC_F_GGGP], f[HMEC_F_ETAP], f[HMEC_F_ETAB],
                f[HMEC_F_GGGB], f[HMEC_F_DILP]);
    const int nb = 152;
    HMEC_LAUNCH(ctx, k_min_etadx, nb, 256, 0, g, f[HMEC_F_ETADX], ctx->red, ctx->ds, ctx->ticket);
    HMEC_LAUNCH(ctx, k_rescale_guess, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->S);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

void launch_assemble(hmec_inst* ctx, const Geo& g, const AsmFields& af, int32_t* col, double* val, double* dscale,
                     double* rhs_scaled, double* rhs_raw, const double*) {
    const dim3 grid(nblocks(g.Ny1, ctx->bs_st), g.Nx1, 6);  // z: the six rows of a cell
    HMEC_LAUNCH(ctx, k_assemble, grid, ctx->bs_st, 0, g, af, ctx->ds, ctx->p, col, val, dscale, rhs_scaled, rhs_raw);
}

int iter_assemble(hmec_inst* ctx) {
    Level& L = ctx->sv.lv[0];
    launch_assemble(ctx, ctx->g, L.af, L.col, L.val, L.dscale, L.db, ctx->R, nullptr);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

int iter_finish(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    double* const* f = ctx->f;
    int* status = &ctx->ds->status;
    HMEC_LAUNCH(ctx, k_reload, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->S, f[HMEC_F_pt], f[HMEC_F_vxs], f[HMEC_F_vys],
                f[HMEC_F_pf], f[HMEC_F_vxD], f[HMEC_F_vyD], status);
    HMEC_LAUNCH(ctx, k_vmax, 152, 256, 0, g, f[HMEC_F_VSLIPB], ctx->ds, ctx->red + 2048, ctx->ticket + 1);
    HMEC_LAUNCH(ctx, k_stress_basic, grid_b(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_GGG],
                f[HMEC_F_ETA], f[HMEC_F_SXY0], f[HMEC_F_EXY], f[HMEC_F_SXY], f[HMEC_F_ETA0], f[HMEC_F_ETA5],
                f[HMEC_F_DSY], f[HMEC_F_YNY], f[HMEC_F_SigmaY], f[HMEC_F_SII_fault], f[HMEC_F_OM], f[HMEC_F_OM5]);
    HMEC_LAUNCH(ctx, k_stress_p, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_GGGP],
                f[HMEC_F_ETAP], f[HMEC_F_SXX0], f[HMEC_F_SYY0], f[HMEC_F_EXX], f[HMEC_F_EYY], f[HMEC_F_SXX],
                f[HMEC_F_SYY]);
    RsfIn in{f[HMEC_F_ARSF], f[HMEC_F_BRSF], f[HMEC_F_LRSF], f[HMEC_F_FRIC], f[HMEC_F_ETA0], f[HMEC_F_SXX],
             f[HMEC_F_SYY], f[HMEC_F_SXY], f[HMEC_F_GGG], f[HMEC_F_ETA], f[HMEC_F_OM], f[HMEC_F_OM0], f[HMEC_F_pt],
             f[HMEC_F_pf], f[HMEC_F_YNY0]};
    double* rsfbuf = ctx->red + 4096;
    RsfOut out{f[HMEC_F_SIIB], f[HMEC_F_OM5], f[HMEC_F_SigmaY], f[HMEC_F_VSLIPB], f[HMEC_F_SII_fault], f[HMEC_F_DSY],
               f[HMEC_F_YNY], f[HMEC_F_ETA5], rsfbuf};
    HMEC_LAUNCH(ctx, k_rsf, nblocks(g.Nx, 128), 128, 0, g, ctx->ds, ctx->p, in, out, status);
    const int nb = 152;
    HMEC_LAUNCH(ctx, k_reduce_vel, nb, 256, 0, g, ctx->p, ctx->crd[3], ctx->crd[5], f[HMEC_F_vxs], f[HMEC_F_vys],
                f[HMEC_F_VSLIPB], ctx->red, rsfbuf, ctx->ds, ctx->ticket + 2);
    HMEC_LAUNCH(ctx, k_eta_update, grid_b(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->p, f[HMEC_F_ETA], f[HMEC_F_ETA5],
                f[HMEC_F_ETA0], f[HMEC_F_ETA50], f[HMEC_F_YNY0], f[HMEC_F_YNY], f[HMEC_F_OM], f[HMEC_F_OM5]);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

int step_end(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    double* const* f = ctx->f;
    HMEC_LAUNCH(ctx, k_end_scalars, 1, 1, 0, ctx->ds);
    HMEC_LAUNCH(ctx, k_post_basic, grid_b(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_GGG],
                f[HMEC_F_ETA], f[HMEC_F_SXY0], f[HMEC_F_ESP], f[HMEC_F_EXY], f[HMEC_F_SXY], f[HMEC_F_ETA50],
                f[HMEC_F_ETA00], f[HMEC_F_OM], f[HMEC_F_OM0]);
    PostP P{f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_GGGP], f[HMEC_F_ETAP], f[HMEC_F_SXX0], f[HMEC_F_SYY0],
            f[HMEC_F_SXY], f[HMEC_F_EXY], f[HMEC_F_ETA], f[HMEC_F_pt], f[HMEC_F_pf], f[HMEC_F_PT0], f[HMEC_F_PF0],
            f[HMEC_F_ETAB], f[HMEC_F_POR], f[HMEC_F_GGGB], f[HMEC_F_EXX], f[HMEC_F_EYY], f[HMEC_F_SXX],
            f[HMEC_F_SYY], f[HMEC_F_EII], f[HMEC_F_EIIVP], f[HMEC_F_SII], f[HMEC_F_DIS], f[HMEC_F_pt_ave],
            f[HMEC_F_pf_ave], f[HMEC_F_VIS_COMP], f[HMEC_F_EL_DECOM]};
    HMEC_LAUNCH(ctx, k_post_p, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, ctx->ds, ctx->p, P);
    HMEC_LAUNCH(ctx, k_monitors, 152, 256, 0, g, ctx->ds, f[HMEC_F_RHOX], f[HMEC_F_RHOY], f[HMEC_F_vxs], f[HMEC_F_vys],
                ctx->red + 2048, ctx->ticket + 3);
    Roll R{f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_vxD], f[HMEC_F_vyD], f[HMEC_F_PORX], f[HMEC_F_PORY],
           f[HMEC_F_SXX], f[HMEC_F_SYY], f[HMEC_F_SXY], f[HMEC_F_pt], f[HMEC_F_pf], f[HMEC_F_VX0], f[HMEC_F_VY0],
           f[HMEC_F_VXF0], f[HMEC_F_VYF0], f[HMEC_F_SXX0], f[HMEC_F_SYY0], f[HMEC_F_SXY0], f[HMEC_F_PTF0],
           f[HMEC_F_PT0], f[HMEC_F_PF0]};
    HMEC_LAUNCH(ctx, k_rollover, grid_s(g, ctx->bs_st), ctx->bs_st, 0, g, R);
    HMEC_LAUNCH(ctx, k_next_step, 1, 1, 0, ctx->ds);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}
