// k_solver.cu -- solution of the assembled system (section a10), in place of
// the Pardiso analyse/factorise/solve of cpp/h_mec_rsf_v9.cpp:1046-1052.
//
// Outer: FGMRES(m) in FP64 on the row-equilibrated system D A x = D b
// (D a power of two per row, so the scaling is exact).  Orthogonalisation is
// classical Gram-Schmidt applied twice (CGS2) so the m dot products of a
// step are one batched kernel; all reductions are block partials summed in a
// fixed order (deterministic, no atomics).  The Hessenberg/Givens update runs
// in one device thread; kernels of a converged solve return immediately, so
// the host only looks at the convergence flag every few steps.
//
// Preconditioner: one geometric-multigrid V-cycle.  Coarse operators are
// rediscretised: the node coefficients that enter the assembly are
// restricted from the fine grid and the same assembly kernel builds the
// coarse matrix.  The smoother is a multiplicative Vanka smoother on the
// staggered cell patch {Pt, Pf, 2 vx, 2 vy, 2 vxD, 2 vyD} (10 unknowns), with
// the 10x10 patch inverses formed once per solve.  Patches are applied in nine
// colour classes (same-class patches neither share unknowns nor read each
// other's), then a two-phase Jacobi pass covers the boundary rows no patch
// contains.  A whole smoothing pass -- every sweep, colour and boundary phase
// -- is ONE cooperative kernel with grid-wide barriers between phases (a
// single block with __syncthreads on small levels), and half a warp works on
// one patch (a lane per patch row, shuffles for the 10x10 product), so a
// V-cycle is about three launches per level.  The V-cycle runs in FP64
// (HMEC_FORM_FP64) or entirely in FP32 (HMEC_FORM_MIXED); FGMRES stays FP64.
#include <cooperative_groups.h>

#include "hmec_internal.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace cg = cooperative_groups;

namespace {

constexpr int PB = 10;   // patch size
constexpr int RED_BS = 256;
constexpr int SM_BS = 256;  // block size of the smoothing kernels

__device__ __forceinline__ int kp_of(int i, int j, int Ny1) { return (j * Ny1 + i) * 6; }

// Global index of unknown q of the patch of P cell (i, j).
__device__ __forceinline__ int patch_unknown(int i, int j, int Ny1, int q) {
    switch (q) {
        case 0: return kp_of(i, j, Ny1) + 0;      // Pt
        case 1: return kp_of(i, j, Ny1) + 3;      // Pf
        case 2: return kp_of(i, j - 1, Ny1) + 1;  // vx left face
        case 3: return kp_of(i, j, Ny1) + 1;      // vx right face
        case 4: return kp_of(i - 1, j, Ny1) + 2;  // vy top face
        case 5: return kp_of(i, j, Ny1) + 2;      // vy bottom face
        case 6: return kp_of(i, j - 1, Ny1) + 4;  // vxD left
        case 7: return kp_of(i, j, Ny1) + 4;      // vxD right
        case 8: return kp_of(i - 1, j, Ny1) + 5;  // vyD top
        default: return kp_of(i, j, Ny1) + 5;     // vyD bottom
    }
}

// ------------------------------------------------------------ Vanka setup
// Gauss-Jordan with partial pivoting on the 10x10 patch block of D A, in the
// smoother's precision T (FP64 form: FP64; mixed form: FP32, the inverses
// being used in FP32 anyway -- and FP64 arithmetic runs at a small fraction
// of the FP32 rate on this GPU); inverses stored patch-major,
// pinv[p*100 + r*10 + c].  Half a warp per patch, lane r holding row r of
// [A | I] in registers.  Pivoting is implicit: column c's pivot is the
// largest |a| among the lanes not yet used as pivots, its normalised row is
// broadcast through shared memory and eliminated from the other lanes; at the end the
// pivot lane of column c holds row c of the inverse.
constexpr int VS_BS = 128;
template <typename T>
__global__ void __launch_bounds__(VS_BS) k_vanka_setup(Geo g, const int32_t* __restrict__ col,
                                                       const double* __restrict__ val, T* pinv, int* status) {
    const int lane = threadIdx.x & 31, q = lane & 15;
    const int pi = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    const int np = (g.Ny - 1) * (g.Nx - 1);
    const bool live = pi < np;
    const int pc = live ? pi : np - 1;  // spare half-warps repeat a patch (uniform shuffles)
    const int i = 1 + pc % (g.Ny - 1), j = 1 + pc / (g.Ny - 1);
    int u[PB];
#pragma unroll
    for (int c = 0; c < PB; c++) u[c] = patch_unknown(i, j, g.Ny1, c);
    T a[PB], b[PB];
#pragma unroll
    for (int c = 0; c < PB; c++) {
        a[c] = 0;
        b[c] = (q == c) ? (T)1 : (T)0;
    }
    if (q < PB) {
        int row = u[0];
#pragma unroll
        for (int c = 1; c < PB; c++)
            if (q == c) row = u[c];
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * g.N + row;
            const int cc = col[o];
            const T v = (T)val[o];
#pragma unroll
            for (int c = 0; c < PB; c++)
                if (u[c] == cc) a[c] += v;
        }
    }
    bool used = q >= PB;
    bool singular = false;
    int my_row = 0;
    // the pivot row of this half-warp's patch, written by the pivot lane and
    // read by the others: a[c+1..PB-1] at [k], b at [PB + k] (vector loads
    // instead of one shuffle per value)
    __shared__ __align__(16) T srow[VS_BS / 16][2 * PB];
    T* const prow = srow[threadIdx.x >> 4];
#pragma unroll
    for (int c = 0; c < PB; c++) {
        T best = used ? (T)-1 : (T)fabs(a[c]);
        int bl = q;
#pragma unroll
        for (int m = 8; m >= 1; m >>= 1) {
            const T ob = __shfl_xor_sync(0xffffffffu, best, m);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, m);
            if (ob > best || (ob == best && ol < bl)) {
                best = ob;
                bl = ol;
            }
        }
        if (!(best > 0)) singular = true;
        if (q == bl) {
            const T inv = (T)1 / a[c];
#pragma unroll
            for (int k = c; k < PB; k++) a[k] *= inv;
#pragma unroll
            for (int k = 0; k < PB; k++) b[k] *= inv;
            used = true;
            my_row = c;
#pragma unroll
            for (int k = c + 1; k < PB; k++) prow[k] = a[k];
#pragma unroll
            for (int k = 0; k < PB; k++) prow[PB + k] = b[k];
        }
        __syncwarp();
        if (q != bl) {
            const T f = a[c];
#pragma unroll
            for (int k = c + 1; k < PB; k++) a[k] -= f * prow[k];
            a[c] = 0;
#pragma unroll
            for (int k = 0; k < PB; k++) b[k] -= f * prow[PB + k];
        }
        __syncwarp();  // the row is read before the next pivot writes it
    }
    if (!live || q >= PB) return;
    if (singular) {
        if (q == 0) atomicOr(status, HMEC_DEV_NAN);
#pragma unroll
        for (int k = 0; k < PB; k++) b[k] = 0;
    }
    const size_t o = (size_t)pi * 100 + my_row * PB;
#pragma unroll
    for (int k = 0; k < PB; k++) pinv[o + k] = b[k];
}

// ---------------------------------------------------- smoothing kernel
template <typename T>
struct SmoothArgs {
    Geo g;
    const int32_t* col;
    const T* val;
    const T* pinv;
    const T* b;
    T* x;
    T* tmp;               // boundary deltas (>= nbnd)
    const int32_t* bnd;
    int nbnd;
    Geo gc;               // coarse level of the prolongation (post-smoothing)
    const T* xc;
    const XferEnt *pmx, *pmy;  // this level's prolongation tables
};

template <bool COOP>
__device__ __forceinline__ void phase_sync() {
    if (COOP) cg::this_grid().sync();
    else __syncthreads();
}

// One colour class (ri, rj) of the multiplicative Vanka sweep.  Half a warp
// per patch: lane q < 10 forms the residual of patch row q, the 10x10
// inverse is applied with shuffles, lane q updates unknown q.  Every lane of
// a warp runs the same number of loop trips (the shuffles need them all).
template <typename T>
__device__ __forceinline__ void vanka_colour(const SmoothArgs<T>& a, int ri, int rj, int gwarp, int nwarps) {
    const Geo& g = a.g;
    const int fi = ri == 0 ? 3 : ri, fj = rj == 0 ? 3 : rj;  // first i >= 1 with i % 3 == ri
    const int ni = (g.Ny - 1 - fi) >= 0 ? (g.Ny - 1 - fi) / 3 + 1 : 0;
    const int nj = (g.Nx - 1 - fj) >= 0 ? (g.Nx - 1 - fj) / 3 + 1 : 0;
    const int npc = ni * nj;
    const int lane = threadIdx.x & 31, q = lane & 15, half = lane >> 4;
    for (int pair = gwarp; 2 * pair < npc; pair += nwarps) {
        const int pidx = 2 * pair + half;
        const bool valid = pidx < npc;
        int i = 1, j = 1, row = 0;
        T r = 0;
        if (valid) {
            i = fi + 3 * (pidx % ni);
            j = fj + 3 * (pidx / ni);
        }
        // this lane's row of the patch inverse, loaded before the residual so
        // its latency overlaps the residual's gathers
        T pr[PB];
        {
            const T* P = a.pinv + (size_t)((j - 1) * (g.Ny - 1) + (i - 1)) * 100 + (q < PB ? q : 0) * PB;
#pragma unroll
            for (int c = 0; c < PB; c++) pr[c] = (valid && q < PB) ? P[c] : (T)0;
        }
        if (valid) {
            if (q < PB) {
                row = patch_unknown(i, j, g.Ny1, q);
                T acc = a.b[row];
#pragma unroll
                for (int s = 0; s < HMEC_W; s++) {
                    const size_t o = (size_t)s * g.N + row;
                    acc -= a.val[o] * a.x[a.col[o]];
                }
                r = acc;
            }
        }
        T d = 0;
#pragma unroll
        for (int c = 0; c < PB; c++) {
            const T rc = __shfl_sync(0xffffffffu, r, (lane & 16) + c);
            d += pr[c] * rc;
        }
        if (valid && q < PB) a.x[row] += d;
    }
}

template <typename T>
__device__ __forceinline__ void bnd_delta(const SmoothArgs<T>& a, int tid, int nth) {
    for (int t = tid; t < a.nbnd; t += nth) {
        const int row = a.bnd[t];
        T acc = a.b[row], diag = 0;
#pragma unroll
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * a.g.N + row;
            const int c = a.col[o];
            const T v = a.val[o];
            acc -= v * a.x[c];
            if (c == row) diag += v;
        }
        a.tmp[t] = diag != 0 ? acc / diag : (T)0;
    }
}

// ------------------------------------------------ 1D grid transfer maps
// A coarse level has ceil(n/2) cells where its fine level has n, over the
// same length, so coarse and fine points align only when n is even.  The
// transfers are separable; in each direction there are two point families:
//   node points j in [0, nf+1] at j*hf (nf+1: the ghost beyond the end), and
//   cell points k in [0, nf+1] centred at (k-1/2)*hf (0, nf+1: ghosts).
// Cell points transfer piecewise-constant (a fine cell to the coarse cell
// containing its centre), node points by linear (hat) interpolation.  All
// positions are compared in exact integer arithmetic (hf/hc = nc/nf).  For
// even n these are the 2:1 operators: cells {2K-1, 2K} -> K; node 2J -> J,
// node 2J+1 -> halves of J and J+1.
struct Map1D {
    int nf, nc;
    double inv;  // 1 / nf
};

__host__ __device__ __forceinline__ int m_cell(const Map1D& m, int k) {
    if (k <= 0) return 0;
    if (k >= m.nf + 1) return m.nc + 1;
    const long long num = (long long)(2 * k - 1) * m.nc;
    // 32-bit division where the operands fit (64-bit division is emulated)
    if (num < 0x7FFFFFFFLL && m.nf < 0x3FFFFFFF) return (int)((unsigned)num / (unsigned)(2 * m.nf)) + 1;
    return (int)(num / (2LL * m.nf)) + 1;
}

// hat weight of coarse node K at fine node j: 1 - |j nc - K nf| / nf (the
// quotient as a product with 1/nf; these weights only shape the
// preconditioner)
__host__ __device__ __forceinline__ double m_hat(const Map1D& m, int j, int K) {
    long long d = (long long)j * m.nc - (long long)K * m.nf;
    if (d < 0) d = -d;
    return d >= m.nf ? 0.0 : (double)(m.nf - d) * m.inv;
}

// fine nodes that can have a nonzero hat weight for coarse node K
__host__ __device__ __forceinline__ void m_hat_range(const Map1D& m, int K, int& j0, int& j1) {
    const int a = (int)(((long long)(K - 1) * m.nf) / m.nc);
    const int b = (int)(((long long)(K + 1) * m.nf + m.nc - 1) / m.nc);
    j0 = a > 0 ? a : 0;
    j1 = b < m.nf + 1 ? b : m.nf + 1;
}

// fine cells that can map to coarse cell K (filter with m_cell(k) == K)
__host__ __device__ __forceinline__ void m_cell_range(const Map1D& m, int K, int& k0, int& k1) {
    if (K <= 0) {
        k0 = k1 = 0;
    } else if (K >= m.nc + 1) {
        k0 = k1 = m.nf + 1;
    } else {
        const int a = (int)(((long long)(K - 1) * m.nf) / m.nc);
        const int b = (int)(((long long)K * m.nf) / m.nc) + 1;
        k0 = a > 1 ? a : 1;
        k1 = b < m.nf ? b : m.nf;
    }
}

__host__ __device__ __forceinline__ Map1D mapx(const Geo& gf, const Geo& gc) {
    return Map1D{gf.Nx - 1, gc.Nx - 1, 1.0 / (gf.Nx - 1)};
}
__host__ __device__ __forceinline__ Map1D mapy(const Geo& gf, const Geo& gc) {
    return Map1D{gf.Ny - 1, gc.Ny - 1, 1.0 / (gf.Ny - 1)};
}

// The transfer table of one direction: entry k for fine index k in [0, nf+1].
static inline std::vector<XferEnt> xfer_table(const Map1D& m) {
    std::vector<XferEnt> t(m.nf + 2);
    for (int k = 0; k <= m.nf + 1; k++) {
        const int n0 = (int)(((long long)k * m.nc) / m.nf);
        t[k] = XferEnt{m_cell(m, k), n0, m_hat(m, k, n0), m_hat(m, k, n0 + 1)};
    }
    return t;
}

// The prolongation of unknown v at fine cell (i, j): cell-centred unknowns
// piecewise constant (interior cells only), face unknowns linear along the
// face normal and constant across it (ghost rows map to ghost rows, which
// keeps the homogeneous boundary relations of the coarse correction).
// mx / my: the transfer tables of the fine level (xfer_table).
template <typename T>
__device__ __forceinline__ T prolong_one(const Geo& gf, const Geo& gc, const XferEnt* __restrict__ mx,
                                         const XferEnt* __restrict__ my, const T* __restrict__ xc, int i, int j,
                                         int v) {
    auto xcv = [&](int I, int J) -> T {
        if (I < 0 || I > gc.Ny || J < 0 || J > gc.Nx) return (T)0;
        return xc[kp_of(I, J, gc.Ny1) + v];
    };
    const XferEnt ex = mx[j], ey = my[i];
    if (v == 0 || v == 3)
        return (i >= 1 && i <= gf.Ny - 1 && j >= 1 && j <= gf.Nx - 1) ? xcv(ey.cell, ex.cell) : (T)0;
    if (v == 1 || v == 4) return (T)ex.w0 * xcv(ey.cell, ex.node0) + (T)ex.w1 * xcv(ey.cell, ex.node0 + 1);
    return (T)ey.w0 * xcv(ey.node0, ex.cell) + (T)ey.w1 * xcv(ey.node0 + 1, ex.cell);
}

// x_f += P x_c over the whole level.
template <typename T>
__device__ __forceinline__ void prolong_add(const Geo& gf, const Geo& gc, const XferEnt* __restrict__ mx,
                                            const XferEnt* __restrict__ my, const T* __restrict__ xc, T* xf,
                                            int tid, int nth) {
    for (int t = tid; t < gf.N; t += nth) {
        const int v = t % 6, cell = t / 6;
        xf[t] += prolong_one(gf, gc, mx, my, xc, cell % gf.Ny1, cell / gf.Ny1, v);
    }
}

// A whole smoothing pass.  mode 0: x = 0 first; mode 1: x += P xc first.
// COOP: launched cooperatively (grid-wide barriers); otherwise one block.
template <typename T, bool COOP>
__global__ void __launch_bounds__(SM_BS) k_smooth(SmoothArgs<T> a, int nsweeps, int mode) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int gwarp = tid >> 5, nwarps = nth >> 5;
    if (mode == 0) {
        for (int t = tid; t < a.g.N; t += nth) a.x[t] = (T)0;
    } else {
        prolong_add(a.g, a.gc, a.pmx, a.pmy, a.xc, a.x, tid, nth);
    }
    phase_sync<COOP>();
    for (int s = 0; s < nsweeps; s++) {
        for (int c = 0; c < 9; c++) {
            vanka_colour(a, c / 3, c % 3, gwarp, nwarps);
            phase_sync<COOP>();
        }
        bnd_delta(a, tid, nth);
        phase_sync<COOP>();
        for (int t = tid; t < a.nbnd; t += nth) a.x[a.bnd[t]] += a.tmp[t];
        phase_sync<COOP>();
    }
}

// The same pass for a small level on one 1024-thread block, with the level's
// x, b and boundary deltas in shared memory: block barriers instead of grid
// barriers and the x gathers of every residual served from shared memory.
// The matrix rows and inverses still come from L2 through the read-only path.
constexpr int SMEM_BS = 1024;
template <typename T>
__global__ void __launch_bounds__(SMEM_BS) k_smooth_smem(SmoothArgs<T> a, int nsweeps, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* xs = reinterpret_cast<T*>(smem_raw);
    T* bs = xs + a.g.N;
    T* ts = bs + a.g.N;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int t = tid; t < a.g.N; t += nth) {
        bs[t] = a.b[t];
        xs[t] = (mode == 0) ? (T)0 : a.x[t];
    }
    __syncthreads();
    if (mode == 1) {
        prolong_add(a.g, a.gc, a.pmx, a.pmy, a.xc, xs, tid, nth);
        __syncthreads();
    }
    SmoothArgs<T> s = a;
    s.x = xs;
    s.b = bs;
    s.tmp = ts;
    for (int k = 0; k < nsweeps; k++) {
        for (int c = 0; c < 9; c++) {
            vanka_colour(s, c / 3, c % 3, tid >> 5, nth >> 5);
            __syncthreads();
        }
        bnd_delta(s, tid, nth);
        __syncthreads();
        for (int t = tid; t < s.nbnd; t += nth) xs[s.bnd[t]] += ts[t];
        __syncthreads();
    }
    for (int t = tid; t < a.g.N; t += nth) a.x[t] = xs[t];
}

// ------------------------------------------------ tiled smoothing pass
// Each block owns tiles of TILE x TILE patches.  Every unknown has exactly one
// owning tile (its cell's patch, a shared face going to the patch on its right
// or below, a boundary row to the adjacent patch).  During a sweep a tile reads
// the unknowns it owns from the live buffer Q and all others from the
// snapshot P, and writes only its own unknowns to Q; so tiles are independent
// within a sweep (deterministic, no races) and only one grid-wide barrier per
// sweep is needed.  Inside a tile the 9 colour classes and the boundary rows
// run in sequence with block barriers: a multiplicative Vanka sweep per tile,
// additive across tile borders.
constexpr int TILE = 12;
constexpr int TILE_BS = 256;  // 16 lanes x at most 16 patches of one colour in a tile

// The window of a tile: the cells its patch rows and boundary rows can read
// (the tile's patches extended by two cells up/left and one down/right).
constexpr int WIN_MAX = (TILE + 3) * (TILE + 3) * 6;

// ------------------------------------------------ staged tiled smoothing pass
// Everything a tile's sweep reads is held in shared memory, so the nine colour
// phases and the boundary phase touch no global memory.  Staged once per tile
// (once per launch when a block keeps one tile for all sweeps, which every
// level with at most one tile per co-resident block does):
//  - the ELL rows of the tile's patches (cells [i0-1, i1) x [j0-1, j1), all
//    six unknowns: (TILE+1)^2 * 6 rows), their rhs, and their columns as
//    int16 offsets in the x window, by LDGSTS (cp.async) runs of 8/16 bytes;
//  - the 10x10 inverses of the tile's patches by TMA bulk copies
//    (cp.async.bulk, one per patch column) completing on an mbarrier -- for
//    FP64 they do not fit beside the rows, and one colour's inverses are
//    streamed per colour instead, double buffered so colour c+1's load while
//    colour c computes;
//  - the tile's boundary rows (values, offsets, rhs, diagonal).
// The x window is reloaded every sweep.  It has a fixed stride (TILE+3 cells
// per window column, starting two cells before the tile), so a column's
// window offset depends only on its offset to the row and is precomputed
// once per assembly (k_stage_prep).  The first sweep of a pre-smoothing pass
// needs no grid barrier before it (its window is zero); a post-smoothing pass
// first adds the prolonged coarse correction to x in one streaming pass over
// the level and a grid barrier.  After the last sweep the residual of the
// fine rows each coarse row needs is formed on the fly and restricted
// (pre-smoothing), again without another barrier.
constexpr int WSTR = TILE + 3;                                    // window cells per window column
constexpr int RSTR = ((TILE + 1) * 6 + 7) / 8 * 8;                // staged rows per staged column (padded)
constexpr int ROWS_MAX = (TILE + 1) * RSTR;                       // staged rows of a tile
constexpr int PV_MAX = ((TILE + 2) / 3) * ((TILE + 2) / 3);       // patches of one colour in a tile
constexpr int TB_MAX = 320;                                       // boundary rows of a tile
constexpr int OWN_BYTES = (WIN_MAX + 127) / 128 * 16;             // a tile's window ownership bits (16-byte multiple)
constexpr int META_BYTES = 9 * TILE_BS * 4;                       // a tile's per-lane colour table
static_assert(WIN_MAX == WSTR * WSTR * 6, "window size");
static_assert(PV_MAX * 16 <= TILE_BS, "a colour's patches fit the block");
static_assert((TILE * 6 * 4) % 16 == 0, "a tile's first staged row starts on 16 bytes in the padded layout");

// Tile owning the unknown v of staggered cell (i, j): a boundary row (outside
// every patch) goes to the adjacent patch, a cell unknown to its own patch,
// an x face to the patch on its right, a y face to the patch below (the
// patch on the other side at the domain edge).
__host__ __device__ __forceinline__ int unknown_tile(const Geo& g, int ntile_i, int i, int j, int v) {
    const bool pin = i >= 1 && i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 1;
    const bool vxin = i >= 1 && i <= g.Ny - 1 && j <= g.Nx - 1;
    const bool vyin = i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 1;
    const bool cellv = v == 0 || v == 3, xv = v == 1 || v == 4;
    int pi, pj;
    if (cellv ? !pin : (xv ? !vxin : !vyin)) {
        pi = i < 1 ? 1 : (i > g.Ny - 1 ? g.Ny - 1 : i);
        pj = j < 1 ? 1 : (j > g.Nx - 1 ? g.Nx - 1 : j);
    } else if (cellv) {
        pi = i;
        pj = j;
    } else if (xv) {
        pi = i;
        pj = (j + 1 <= g.Nx - 1) ? j + 1 : j;
    } else {
        pi = (i + 1 <= g.Ny - 1) ? i + 1 : i;
        pj = j;
    }
    return (pi - 1) / TILE + ((pj - 1) / TILE) * ntile_i;
}

// Window offset of an ELL entry: the x window index of the column minus that
// of the row.  |col - row - dj*RS| <= 11 for every assembled row (the stencils
// reach one cell); a row outside that raises HMEC_DEV_BOUNDS and points at the
// row itself, so nothing is read outside the window.
__device__ __forceinline__ int16_t window_offset(int row, int col, int RS, int* status) {
    const int delta = col - row;
    const int dj = delta > RS / 2 ? 1 : (delta < -RS / 2 ? -1 : 0);
    const int rem = delta - dj * RS;
    if (rem < -11 || rem > 11) {
        atomicOr(status, HMEC_DEV_BOUNDS);
        return 0;
    }
    return (int16_t)(dj * 6 * WSTR + rem);
}

// The smoother's copy of the matrix in the padded layout (see Level::vals):
// values in its precision and window offsets; the mixed form also takes its
// FP32 copy in the assembly's layout here (the residuals read it).
// offs is set only on the first assembly: the pattern never changes.
template <typename T>
__global__ void k_stage_prep(int N, int Ny1, int Nx1, int CS, const int32_t* __restrict__ col,
                             const double* __restrict__ val, T* vals, int16_t* offs, float* val32, int* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * HMEC_W) return;
    const int s = t / N, row = t - s * N;
    const int RS = 6 * Ny1;
    const int j = row / RS, r = row - j * RS;
    const size_t o = ((size_t)s * Nx1 + j) * CS + r;
    if (offs) offs[o] = window_offset(row, col[t], RS, status);
    vals[o] = (T)val[t];
    if (val32) val32[t] = (float)val[t];
}

// The standard window offsets of a level: the 11 offsets of each of the six
// rows of its centre cell (one thread per row type and slot).  Every row of
// an interior cell has them, since the assembly writes a row's entries
// sorted by column and the stencil reaches the same neighbours everywhere
// inside; which tiles hold only such rows is decided by k_tile_std.
__global__ void k_std_pattern(Geo g, int CS, const int16_t* __restrict__ offs, int16_t* std_off) {
    const int t = threadIdx.x;
    if (t >= 6 * HMEC_W) return;
    const int v = t / HMEC_W, sl = t - v * HMEC_W;
    const int ci = g.Ny1 / 2, cj = g.Nx1 / 2;
    std_off[t] = offs[((size_t)sl * g.Nx1 + cj) * CS + ci * 6 + v];
}

// Per tile (one block each): 1 when every row its patches can touch (cells
// [i0-1, i1) x [j0-1, j1), all six unknowns) has the standard offsets, so
// that the smoothing pass takes them from registers; 0 sends the tile's rows
// to the offsets in global memory.
__global__ void k_tile_std(Geo g, int ntile_i, int CS, const int16_t* __restrict__ offs,
                           const int16_t* __restrict__ std_off, uint8_t* std_t) {
    __shared__ int16_t so[6 * HMEC_W];
    if (threadIdx.x < 6 * HMEC_W) so[threadIdx.x] = std_off[threadIdx.x];
    __syncthreads();
    const int tile = blockIdx.x;
    const int ti = tile % ntile_i, tj = tile / ntile_i;
    const int i0 = 1 + ti * TILE, j0 = 1 + tj * TILE;
    const int i1 = min(i0 + TILE, g.Ny), j1 = min(j0 + TILE, g.Nx);
    const int RI = (i1 - i0 + 1) * 6, n = RI * (j1 - j0 + 1);
    int bad = 0;
    for (int k = threadIdx.x; k < n * HMEC_W; k += blockDim.x) {
        const int sl = k / n, rr = k - sl * n;
        const int jj = rr / RI, ii = rr - jj * RI;
        const int16_t o = offs[((size_t)sl * g.Nx1 + (j0 - 1 + jj)) * CS + (i0 - 1) * 6 + ii];
        bad |= o != so[(ii % 6) * HMEC_W + sl];
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) std_t[tile] = bad ? 0 : 1;
}

// Byte size of one tile's boundary-row pack: values [W][cap], diagonal [cap]
// (T); window offsets [W][cap], window index [cap] (int16); row [cap] (int32).
template <typename T>
__host__ __device__ __forceinline__ int pack_bytes(int cap) {
    return cap * (HMEC_W * (int)sizeof(T) + (int)sizeof(T) + HMEC_W * 2 + 2 + 4);
}

// One thread per (tile, boundary slot): the tile's boundary rows packed in
// the pack layout, zero past the tile's count (rebuilt with each assembly).
template <typename T>
__global__ void k_stage_bpack(Geo g, int ntile_i, int ntiles, int cap, const int32_t* __restrict__ tb_start,
                              const int32_t* __restrict__ tb_list, const int32_t* __restrict__ col,
                              const double* __restrict__ val, unsigned char* pack, int* status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntiles * cap) return;
    const int tile = t / cap, k = t - tile * cap;
    unsigned char* base = pack + (size_t)tile * pack_bytes<T>(cap);
    T* bval = reinterpret_cast<T*>(base);
    T* bdiag = bval + HMEC_W * cap;
    int16_t* boff = reinterpret_cast<int16_t*>(bdiag + cap);
    int16_t* blr = boff + HMEC_W * cap;
    int32_t* brow = reinterpret_cast<int32_t*>(blr + cap);
    const int kb = tb_start[tile], n = tb_start[tile + 1] - kb;
    if (k >= n) {
#pragma unroll
        for (int s = 0; s < HMEC_W; s++) {
            bval[s * cap + k] = (T)0;
            boff[s * cap + k] = 0;
        }
        bdiag[k] = (T)0;
        blr[k] = 0;
        brow[k] = 0;
        return;
    }
    const int ti = tile % ntile_i, tj = tile / ntile_i;
    const int wi0 = TILE * ti - 1, wj0 = TILE * tj - 1;  // window origin: two cells before the tile
    const int row = tb_list[kb + k], cell = row / 6;
    const int RS = 6 * g.Ny1;
    blr[k] = (int16_t)((((cell / g.Ny1) - wj0) * WSTR + ((cell % g.Ny1) - wi0)) * 6 + (row - 6 * cell));
    brow[k] = row;
    T diag = 0;
#pragma unroll
    for (int s = 0; s < HMEC_W; s++) {
        const size_t o = (size_t)s * g.N + row;
        const T v = (T)val[o];
        bval[s * cap + k] = v;
        boff[s * cap + k] = window_offset(row, col[o], RS, status);
        if (col[o] == row) diag += v;
    }
    bdiag[k] = diag;
}

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

template <int B>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(smem_u32(dst)), "l"(src), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// TMA tensor copy of a 3-D box at element coordinates (c0, c1, c2); elements
// outside the tensor arrive as zeros, and the full box counts on the barrier.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

// Prefetch of a 3-D box into L2 (no shared memory, no barrier): the next
// tile's stage streams from DRAM while this tile computes.
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap* map, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];\n" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(c0), "r"(c1), "r"(c2)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a phase of a TMA barrier: on the cap the status bit is set
// and the caller carries on (every block must still reach the grid barriers).
constexpr int MBAR_SPIN_CAP = 1 << 22;
__device__ __forceinline__ void mbar_wait(unsigned long long* bar, unsigned parity, int* status) {
    for (int it = 0; it < MBAR_SPIN_CAP; it++)
        if (mbar_try_wait(bar, parity)) return;
    atomicOr(status, HMEC_DEV_TIMEOUT);
}

template <typename T>
__device__ __forceinline__ void restrict_apply(int Nc, const int32_t* __restrict__ ridx, const T* __restrict__ rw,
                                               const T* __restrict__ rf, T* bc, int tid, int nth);

template <typename T>
struct StageArgs {
    CUtensorMap tm_val;    // smoother copy of the values: box (RSTR, TILE+1, W)
    CUtensorMap tm_pinv;   // inverses (100, Ny-1, Nx-1): box (100, TILE, TILE)
    Geo g;
    const int16_t* offs;   // window offsets in the padded layout (tiles without the standard pattern)
    const int16_t* std_off;  // the level's standard offsets [6][W]
    const uint8_t* std_t;  // per tile: 1 when its rows all have the standard offsets
    int cs;                // the padded layout's column stride
    const int32_t* col;    // ELL in the assembly's layout (residual)
    const T* val;
    const T* pinv;         // inverses (per-colour copies)
    const T* b;
    T* x;
    T* xalt;
    const int32_t* tb_start;
    const uint32_t* own_t; // per tile: window ownership bits
    const int32_t* meta_t; // per tile: per-lane colour table
    const unsigned char* bpack;  // per tile: boundary-row pack
    int ntile_i, ntiles;
    Geo gc;                // prolongation source (mode 1)
    const T* xc;
    const XferEnt *pmx, *pmy;
    int nc;                // if bc is set: the residual restricted into bc
    const int32_t* ridx;
    const T* rw;
    T* bc;
    int tb_cap;            // boundary rows one tile's stage holds
    int local;             // HMEC_MG_LOCAL_SWEEPS: a tile's sweeps back to back on one stage
    int* status;
    const int* done;       // the solve's convergence flag: set, the pass does nothing
};

// Whether the stage holds an edge tile's boundary pack, the per-lane colour
// table and the boundary rows' corrections (FP32), or the pass reads the
// pack from global memory and keeps the table and corrections in registers
// (FP64: the smaller stage leaves more of the SM's memory to L1, which the
// window loads, prolongation and restriction use; 1001x401: 53 -> 46 ms per
// step without the pack, 53.5 -> 49.8 without the table and corrections).
// The FP32 stage measured slower without them even with two blocks per SM
// (1001x401: 19.2 against 18.4 ms; 201x201: 20.1 against 12.5).
template <typename T>
__host__ __device__ constexpr bool stage_pack() {
    return sizeof(T) == 4;
}

// Shared-memory layout of the staged pass, in bytes.  Its size depends on the
// inverse mode and on the level's boundary-row capacity (FP32 with whole-tile
// inverses: about 143 KB, one block per SM; a level with more tiles than
// blocks restages a tile every time a block takes it up).
struct StageLayout {
    int xs, val, b, pv, pack, own, meta, bb, bdel, bar, total;
};

__host__ __device__ __forceinline__ int align_up(int x, int a) { return (x + a - 1) / a * a; }

// TMA destinations start on 128 bytes, the rest on 16.
template <typename T>
__host__ __device__ __forceinline__ StageLayout stage_layout(int pv_whole, int tb_cap) {
    StageLayout L;
    int o = 0;
    auto take = [&o](int& at, int bytes, int a) {
        o = align_up(o, a);
        at = o;
        o += bytes;
    };
    const int st = (int)sizeof(T);
    take(L.val, HMEC_W * ROWS_MAX * st, 128);
    take(L.pv, (pv_whole ? TILE * TILE : 2 * PV_MAX) * 100 * st, 128);
    if (stage_pack<T>()) take(L.pack, pack_bytes<T>(tb_cap), 128);
    take(L.own, OWN_BYTES, 16);
    L.meta = L.bdel = 0;
    if (stage_pack<T>()) take(L.meta, META_BYTES, 16);
    take(L.xs, WIN_MAX * st, 16);
    take(L.b, ROWS_MAX * st, 16);
    take(L.bb, tb_cap * st, 16);
    if (stage_pack<T>()) take(L.bdel, tb_cap * st, 16);
    take(L.bar, 3 * 8, 16);
    L.total = align_up(o, 16);
    return L;
}

// Bytes one tile's stage receives on its barrier (the colour table in the
// FP32 stage, the boundary pack only for a tile that has boundary rows).
template <typename T>
__host__ __device__ __forceinline__ unsigned stage_tx_bytes(bool whole, int tb_cap, bool pack) {
    return (unsigned)(HMEC_W * (TILE + 1) * RSTR * sizeof(T) + (whole ? TILE * TILE * 100 * sizeof(T) : 0) +
                      (pack ? pack_bytes<T>(tb_cap) : 0) + OWN_BYTES + (stage_pack<T>() ? META_BYTES : 0));
}

// bc = R (b - A x): each coarse row forms the residuals of its fine rows.
template <typename T>
__device__ __forceinline__ void restrict_resid(int Nc, const int32_t* __restrict__ ridx, const T* __restrict__ rw,
                                               int N, const int32_t* __restrict__ col, const T* __restrict__ val,
                                               const T* __restrict__ b, const T* __restrict__ x, T* bc, int tid,
                                               int nth) {
    for (int t = tid; t < Nc; t += nth) {
        T s = 0;
#pragma unroll
        for (int e = 0; e < HMEC_RW; e++) {
            const size_t o = (size_t)e * Nc + t;
            const T w = rw[o];
            if (w == (T)0) continue;
            const int k = ridx[o];
            T r = b[k];
#pragma unroll
            for (int sl = 0; sl < HMEC_W; sl++) {
                const size_t q = (size_t)sl * N + k;
                r -= val[q] * x[col[q]];
            }
            s += w * r;
        }
        bc[t] = s;
    }
}

// Patches of colour c = (ri, rj) in the tile [i0, i1) x [j0, j1): the first
// row/column of the class and the counts.
__host__ __device__ __forceinline__ void colour_grid(int c, int i0, int j0, int i1, int j1, int& fi, int& fj, int& ni,
                                            int& nj) {
    const int ri = c / 3, rj = c % 3;
    fi = i0 + ((ri - i0 % 3) + 3) % 3;
    fj = j0 + ((rj - j0 % 3) + 3) % 3;
    ni = fi < i1 ? (i1 - 1 - fi) / 3 + 1 : 0;
    nj = fj < j1 ? (j1 - 1 - fj) / 3 + 1 : 0;
}

// One thread: the inverses of colour c's patches into buffer bb of pv.
template <typename T>
__device__ __forceinline__ void issue_pinv(const StageArgs<T>& t, T* pv, unsigned long long* bar, int c, int bb,
                                           int i0, int j0, int i1, int j1) {
    int fi, fj, ni, nj;
    colour_grid(c, i0, j0, i1, j1, fi, fj, ni, nj);
    const int npc = ni * nj;
    constexpr unsigned PBYTES = 100 * sizeof(T);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    mbar_expect_tx(&bar[bb], npc * PBYTES);
    T* buf = pv + bb * PV_MAX * 100;
    for (int p = 0; p < npc; p++) {
        const int i = fi + 3 * (p % ni), j = fj + 3 * (p / ni);
        bulk_g2s(buf + p * 100, t.pinv + ((size_t)(j - 1) * (t.g.Ny - 1) + (i - 1)) * 100, PBYTES, &bar[bb]);
    }
}

// Per-lane colour table entry: valid << 30 | patch in tile << 22 | staged
// row << 11 | window index, for the patch row this lane forms in colour c of
// a tile (host-built per tile; the kernel loads it when it stages the tile).
__host__ __device__ __forceinline__ int lane_meta(int c, int lanetid, int i0, int j0, int i1, int j1) {
    const int q = (lanetid & 31) & 15, slot = lanetid >> 4;
    const int qv = q < 2 ? 3 * q : (q < 6 ? 1 + (q - 2) / 2 : (q < PB ? 4 + (q - 6) / 2 : 0));
    const int qdi = (q == 4 || q == 8) ? 1 : 0, qdj = (q == 2 || q == 6) ? 1 : 0;
    int fi, fj, ni, nj;
    colour_grid(c, i0, j0, i1, j1, fi, fj, ni, nj);
    if (!(slot < ni * nj && q < PB)) return 0;
    const int i = fi + 3 * (slot % ni), j = fj + 3 * (slot / ni);
    const int ci = i - qdi, cj = j - qdj;
    const int lrow = ((cj - (j0 - 2)) * WSTR + (ci - (i0 - 2))) * 6 + qv;
    const int rl = (cj - j0 + 1) * RSTR + (ci - i0 + 1) * 6 + qv;
    const int lp = (i - i0) + (j - j0) * TILE;
    return (1 << 30) | (lp << 22) | (rl << 11) | lrow;
}

// The TMA barriers of a smoothing block and their phase counters, kept across
// the passes of one launch.
struct StageBars {
    unsigned long long* bar;  // [0], [1]: per-colour inverses (streamed mode); [2]: a tile's stage
    unsigned use0, use1, use2;
};

__device__ __forceinline__ void stage_bars_init(unsigned long long* bar) {
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init(&bar[2], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
}

// One smoothing pass of one level (nsweeps sweeps, then the optional
// restriction), run by every block of the launch.  t lives in kernel
// parameter space or in global memory (its tensor maps are read from where
// it lives).  Lo: the launch's shared-memory layout, sized for at least this
// level's boundary-row capacity.  WHOLE: the inverse mode.  REV: odd
// sweeps visit the block's tiles in reverse (the fused V-cycle).
template <typename T, bool WHOLE, bool REV>
__device__ __forceinline__ void stage_pass(const StageArgs<T>& t, int nsweeps, int mode, unsigned char* smem_raw,
                                           const StageLayout& Lo, StageBars& sb_) {
    T* xs = reinterpret_cast<T*>(smem_raw + Lo.xs);
    T* sval = reinterpret_cast<T*>(smem_raw + Lo.val);
    T* sb = reinterpret_cast<T*>(smem_raw + Lo.b);
    uint32_t* ownb = reinterpret_cast<uint32_t*>(smem_raw + Lo.own);
    int32_t* smeta = reinterpret_cast<int32_t*>(smem_raw + Lo.meta);

    unsigned long long* bar = sb_.bar;
    T* pv = reinterpret_cast<T*>(smem_raw + Lo.pv);
    const int TBC = t.tb_cap;
    T* bbv = reinterpret_cast<T*>(smem_raw + Lo.bb);
    T* bdel = reinterpret_cast<T*>(smem_raw + Lo.bdel);
    constexpr bool whole = WHOLE;
    const Geo& g = t.g;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, q = lane & 15, slot = threadIdx.x >> 4;
    const int warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    // the barriers' phase counters in registers for the pass, written back at its end
    unsigned use0 = sb_.use0, use1 = sb_.use1, use2 = sb_.use2;
    int staged = -1, nbt = 0, tstd = 0;
    int meta[9];  // FP64 stage: this lane's colour table for the staged tile
    // the standard window offsets of this lane's patch row (its unknown type
    // is fixed by the lane), two int16 per register
    constexpr int NSO = (HMEC_W + 1) / 2;
    unsigned sop[NSO];
    {
        const int qv = q < 2 ? 3 * q : (q < 6 ? 1 + (q - 2) / 2 : (q < PB ? 4 + (q - 6) / 2 : 0));
#pragma unroll
        for (int k = 0; k < NSO; k++) {
            const unsigned lo = (uint16_t)t.std_off[qv * HMEC_W + 2 * k];
            const unsigned hi = 2 * k + 1 < HMEC_W ? (uint16_t)t.std_off[qv * HMEC_W + 2 * k + 1] : 0u;
            sop[k] = lo | (hi << 16);
        }
    }
    const size_t goff_slot = (size_t)g.Nx1 * t.cs;  // slot stride of the padded layout
    const T* src = t.x;  // sweep s > 0 reads the previous sweep's result
    T* dst = t.xalt;
    // one tile for the whole level (the coarsest levels): the window holds
    // every unknown, so the sweeps stay in shared memory and only the last
    // one is published -- no grid barrier or window reload in between
    const bool solo = t.ntiles == 1 && gridDim.x == 1;
    // local sweeps (a solo tile, or on request for every level): a tile runs
    // all the pass's sweeps on one stage, its neighbours' unknowns taken from
    // the start of the pass -- one stage, one window load and one grid
    // barrier per pass instead of per sweep
    const bool local = solo || t.local;
    const int outer = local ? 1 : nsweeps, inner = local ? nsweeps : 1;
    // post-smoothing: x += P xc as one streaming pass over the level, every
    // block at once, then a grid barrier -- formed per tile inside the window
    // loads the dependent table and coarse loads cost ~10 us per tile
    if (mode == 1) {
        prolong_add(g, t.gc, t.pmx, t.pmy, t.xc, t.x, tid, nth);
        cg::this_grid().sync();
    }
    // this block's tiles: blockIdx.x + k * gridDim.x.  With REV odd sweeps
    // visit them in reverse, so the tile a sweep ends on starts the next one
    // and stays staged; the order within a sweep changes nothing, as a
    // sweep's tiles read only the previous sweep's values
    const int ntb = (int)blockIdx.x < t.ntiles ? (t.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    for (int so = 0; so < outer; so++) {
        const bool rev = REV && (so & 1) != 0;
        for (int kt = 0; kt < ntb; kt++) {
            const int tile = (int)blockIdx.x + (rev ? ntb - 1 - kt : kt) * (int)gridDim.x;
            const int ti = tile % t.ntile_i, tj = tile / t.ntile_i;
            const int i0 = 1 + ti * TILE, j0 = 1 + tj * TILE;
            const int i1 = min(i0 + TILE, g.Ny), j1 = min(j0 + TILE, g.Nx);  // exclusive
            const int wi0 = i0 - 2, wj0 = j0 - 2;
            const bool fresh = staged != tile;
            if (fresh) {
                nbt = min(t.tb_start[tile + 1] - t.tb_start[tile], TBC);
                tstd = t.std_t[tile];
                // one thread: the tile's rows (values, one 3-D box), its
                // inverses, its window's ownership bits, its per-lane colour
                // table and, when it has boundary rows, its boundary pack
                if (threadIdx.x == 0) {
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                    mbar_expect_tx(&bar[2], stage_tx_bytes<T>(whole, TBC, stage_pack<T>() && nbt > 0));
                    tma_load_3d(sval, &t.tm_val, (i0 - 1) * 6, j0 - 1, 0, &bar[2]);
                    if (whole) tma_load_3d(pv, &t.tm_pinv, 0, i0 - 1, j0 - 1, &bar[2]);
                    bulk_g2s(ownb, t.own_t + (size_t)tile * (OWN_BYTES / 4), OWN_BYTES, &bar[2]);
                    if (stage_pack<T>()) bulk_g2s(smeta, t.meta_t + (size_t)tile * 9 * TILE_BS, META_BYTES, &bar[2]);
                    if (stage_pack<T>() && nbt > 0)
                        bulk_g2s(smem_raw + Lo.pack, t.bpack + (size_t)tile * pack_bytes<T>(TBC), pack_bytes<T>(TBC),
                                 &bar[2]);
                    // the tile this block stages next into L2: this sweep's
                    // next, or, in forward order, the next sweep's first when
                    // it is another tile (in reverse the next sweep starts on
                    // this one)
                    int nx;
                    if (REV)
                        nx = kt + 1 < ntb ? (int)blockIdx.x + (rev ? ntb - 2 - kt : kt + 1) * (int)gridDim.x : -1;
                    else
                        nx = kt + 1 < ntb ? tile + (int)gridDim.x : (so + 1 < outer ? (int)blockIdx.x : -1);
                    if (nx >= 0 && nx != tile) {
                        const int ni0 = 1 + (nx % t.ntile_i) * TILE, nj0 = 1 + (nx / t.ntile_i) * TILE;
                        tma_prefetch_3d(&t.tm_val, (ni0 - 1) * 6, nj0 - 1, 0);
                        if (whole) tma_prefetch_3d(&t.tm_pinv, 0, ni0 - 1, nj0 - 1);
                    }
                }
                // the rows' rhs: per staged column one run of RI*6 values
                const int RI = i1 - i0 + 1, RJ = j1 - j0 + 1, nch = RI * 3;
                constexpr int CH = 2 * sizeof(T);
                for (int c = warp; c < RJ; c += nwarp) {
                    const size_t g0 = ((size_t)(j0 - 1 + c) * g.Ny1 + (i0 - 1)) * 6;
                    for (int k = lane; k < nch; k += 32) cp_async<CH>(&sb[c * RSTR + 2 * k], t.b + g0 + 2 * k);
                }
                // the boundary rows' rhs, gathered by their row numbers in the pack
                const int32_t* brow = reinterpret_cast<const int32_t*>(
                    t.bpack + (size_t)tile * pack_bytes<T>(TBC) + (size_t)TBC * (HMEC_W * sizeof(T) + sizeof(T) + HMEC_W * 2 + 2));
                for (int k = threadIdx.x; k < nbt; k += blockDim.x) bbv[k] = t.b[brow[k]];
                if (!stage_pack<T>()) {
#pragma unroll
                    for (int c = 0; c < 9; c++) meta[c] = __ldg(t.meta_t + ((size_t)tile * 9 + c) * TILE_BS + threadIdx.x);
                }
                staged = tile;
            }
            for (int si = 0; si < inner; si++) {
            const int s = local ? si : so;  // the sweep
            if (!whole && threadIdx.x == 0) issue_pinv(t, pv, bar, 0, 0, i0, j0, i1, j1);
            // the x window: zero, x + P xc, or the previous sweep's values
            // (local sweeps keep the window from the previous sweep)
            if (!(local && s > 0)) {
                constexpr int WPT = (WIN_MAX + TILE_BS - 1) / TILE_BS;
                T xv[WPT];
#pragma unroll
                for (int u = 0; u < WPT; u++) {
                    const int lw = threadIdx.x + u * TILE_BS;
                    const int lc = lw / 6, v = lw - 6 * lc;
                    const int ci = wi0 + lc % WSTR, cj = wj0 + lc / WSTR;
                    xv[u] = (T)0;
                    if (lw < WIN_MAX && ci >= 0 && ci <= g.Ny && cj >= 0 && cj <= g.Nx && (s > 0 || mode == 1)) {
                        xv[u] = src[(cj * g.Ny1 + ci) * 6 + v];
                    }
                }
#pragma unroll
                for (int u = 0; u < WPT; u++) {
                    const int lw = threadIdx.x + u * TILE_BS;
                    if (lw < WIN_MAX) xs[lw] = xv[u];
                }
            }
            cp_async_wait_all();
            __syncthreads();
            if (fresh && si == 0) {
                mbar_wait(&bar[2], use2 & 1, t.status);
                use2++;
            }
#pragma unroll
            for (int c = 0; c < 9; c++) {
                const int bb = c & 1;
                if (!whole) {
                    if (bb == 0) {
                        mbar_wait(&bar[0], use0 & 1, t.status);
                        use0++;
                    } else {
                        mbar_wait(&bar[1], use1 & 1, t.status);
                        use1++;
                    }
                    // the other buffer's readers passed the previous colour's barrier
                    if (c < 8 && threadIdx.x == 0) issue_pinv(t, pv, bar, c + 1, bb ^ 1, i0, j0, i1, j1);
                }
                const int m = stage_pack<T>() ? smeta[c * TILE_BS + threadIdx.x] : meta[c];
                const bool valid = (m >> 30) & 1;
                const bool mine = ((unsigned)m >> 31) != 0u;  // the tile owns this patch row's unknown
                const int lrow = m & 2047, rl = (m >> 11) & 2047;
                T pr[PB];
                T r = 0;
                if (valid) {
                    const T* pi = whole ? pv + ((m >> 22) & 255) * 100 + q * PB : pv + (bb * PV_MAX + slot) * 100 + q * PB;
#pragma unroll
                    for (int cc = 0; cc < PB; cc++) pr[cc] = pi[cc];
                    T acc = sb[rl];
                    if (tstd) {
#pragma unroll
                        for (int sl = 0; sl < HMEC_W; sl++) {
                            const int o = (int16_t)(uint16_t)(sop[sl >> 1] >> ((sl & 1) * 16));
                            acc -= sval[sl * ROWS_MAX + rl] * xs[lrow + o];
                        }
                    } else {
                        // staged row rl is element (i0-1)*6 + ii of column j0-1+jj
                        const int jj = rl / RSTR, ii = rl - jj * RSTR;
                        const int16_t* go = t.offs + (size_t)(j0 - 1 + jj) * t.cs + (i0 - 1) * 6 + ii;
#pragma unroll
                        for (int sl = 0; sl < HMEC_W; sl++)
                            acc -= sval[sl * ROWS_MAX + rl] * xs[lrow + __ldg(go + sl * goff_slot)];
                    }
                    r = acc;
                } else {
#pragma unroll
                    for (int cc = 0; cc < PB; cc++) pr[cc] = (T)0;
                }
                T d = 0;
#pragma unroll
                for (int cc = 0; cc < PB; cc++) {
                    const T rc = __shfl_sync(0xffffffffu, r, (lane & 16) + cc);
                    d += pr[cc] * rc;
                }
                // same-class patches never read each other's unknowns, and the
                // shuffles above order this patch's reads before its writes
                if (valid && mine) xs[lrow] += d;
                __syncthreads();
            }
            // this tile's boundary rows: one Jacobi pass on the window (the
            // pack in k_stage_bpack's layout, staged or in global memory)
            const unsigned char* pack =
                stage_pack<T>() ? smem_raw + Lo.pack : t.bpack + (size_t)tile * pack_bytes<T>(TBC);
            const T* bval = reinterpret_cast<const T*>(pack);
            const T* bdiag = bval + HMEC_W * TBC;
            const int16_t* boff = reinterpret_cast<const int16_t*>(bdiag + TBC);
            const int16_t* blr = boff + HMEC_W * TBC;
            if (stage_pack<T>()) {
                for (int k = threadIdx.x; k < nbt; k += blockDim.x) {
                    const int lr = blr[k];
                    T acc = bbv[k];
#pragma unroll
                    for (int sl = 0; sl < HMEC_W; sl++) acc -= bval[sl * TBC + k] * xs[lr + boff[sl * TBC + k]];
                    bdel[k] = bdiag[k] != (T)0 ? acc / bdiag[k] : (T)0;
                }
                __syncthreads();
                for (int k = threadIdx.x; k < nbt; k += blockDim.x) xs[blr[k]] += bdel[k];
            } else {
                constexpr int BDR = (TB_MAX + TILE_BS - 1) / TILE_BS;
                T bd[BDR];
#pragma unroll
                for (int u = 0; u < BDR; u++) {
                    const int k = threadIdx.x + u * TILE_BS;
                    bd[u] = (T)0;
                    if (k < nbt) {
                        const int lr = blr[k];
                        T acc = bbv[k];
#pragma unroll
                        for (int sl = 0; sl < HMEC_W; sl++) acc -= bval[sl * TBC + k] * xs[lr + boff[sl * TBC + k]];
                        bd[u] = bdiag[k] != (T)0 ? acc / bdiag[k] : (T)0;
                    }
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < BDR; u++) {
                    const int k = threadIdx.x + u * TILE_BS;
                    if (k < nbt) xs[blr[k]] += bd[u];
                }
            }
            __syncthreads();
            // publish the owned unknowns
            if (!local || s == nsweeps - 1) {
                for (int lw = threadIdx.x; lw < WIN_MAX; lw += blockDim.x) {
                    if (!((ownb[lw >> 5] >> (lw & 31)) & 1u)) continue;
                    const int lc = lw / 6, v = lw - 6 * lc;
                    const int ci = wi0 + lc % WSTR, cj = wj0 + lc / WSTR;
                    dst[(cj * g.Ny1 + ci) * 6 + v] = xs[lw];
                }
            }
            __syncthreads();
            }
        }
        // the last sweep needs the barrier only when this launch reads the
        // result back: the residual restriction, or a copy into x
        const bool last_in_x = so == outer - 1 && dst == t.x && !t.bc;
        if (!solo && !last_in_x) cg::this_grid().sync();
        src = dst;
        dst = (dst == t.xalt) ? t.x : t.xalt;
    }
    // the last sweep's barrier made src complete
    if (src != t.x)
        for (int r = tid; r < g.N; r += nth) t.x[r] = src[r];
    if (t.bc) restrict_resid(t.nc, t.ridx, t.rw, g.N, t.col, t.val, t.b, src, t.bc, tid, nth);
    sb_.use0 = use0;
    sb_.use1 = use1;
    sb_.use2 = use2;
}

// One smoothing pass as its own cooperative launch.
template <typename T, bool WHOLE>
__global__ void __launch_bounds__(TILE_BS, 2) k_smooth_stage(const __grid_constant__ StageArgs<T> t, int nsweeps,
                                                             int mode) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // a V-cycle launched after the solve converged (the host looks at the
    // flag only now and then) does no work; no kernel of a V-cycle writes
    // the flag, so every block sees the same value
    if (*t.done) return;
    const StageLayout Lo = stage_layout<T>(WHOLE ? 1 : 0, t.tb_cap);
    StageBars sb{reinterpret_cast<unsigned long long*>(smem_raw + Lo.bar), 0, 0, 0};
    stage_bars_init(sb.bar);
    stage_pass<T, WHOLE, false>(t, nsweeps, mode, smem_raw, Lo, sb);
}

// A whole V-cycle's smoothing passes in one cooperative launch: pass p of
// the table (a kernel parameter, tensor maps included) with a grid barrier
// between passes -- the pre-smoothing passes down the levels (each
// restricting its residual into the next level's rhs), the coarsest level's
// sweeps, and the post-smoothing passes back up (each adding the coarser
// correction).  cap: the largest boundary-row capacity of the levels (the
// shared-memory layout); done: the solve's convergence flag.
template <typename T>
struct VPass {
    StageArgs<T> a;
    int nsweeps, mode;
};
constexpr int MAX_VPASS = 11;  // six levels
template <typename T>
struct VTable {
    VPass<T> p[MAX_VPASS];
    int npass, cap;
    const int* done;
};

template <typename T, bool WHOLE>
__global__ void __launch_bounds__(TILE_BS, 2) k_vcycle_stage(const __grid_constant__ VTable<T> v) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if (*v.done) return;
    const StageLayout Lo = stage_layout<T>(WHOLE ? 1 : 0, v.cap);
    StageBars sb{reinterpret_cast<unsigned long long*>(smem_raw + Lo.bar), 0, 0, 0};
    stage_bars_init(sb.bar);
    for (int p = 0; p < v.npass; p++) {
        if (p > 0) cg::this_grid().sync();
        stage_pass<T, WHOLE, true>(v.p[p].a, v.p[p].nsweeps, v.p[p].mode, smem_raw, Lo, sb);
    }
}

// ------------------------------------------------ multigrid restriction
// Whether the row of unknown v at staggered cell (i, j) is an interior
// equation (x/y-Stokes, continuity, Darcy) rather than a boundary or ghost
// row; the ranges are those of the assembly branches (:698-980).
__host__ __device__ __forceinline__ bool row_interior(const Geo& g, int i, int j, int v) {
    switch (v) {
        case 0: return i >= 1 && i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 1;         // Pt
        case 3: return i >= 2 && i <= g.Ny - 2 && j >= 1 && j <= g.Nx - 1;         // Pf
        case 1: case 4: return i >= 1 && i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 2; // vx, vxD
        default: return i >= 1 && i <= g.Ny - 2 && j >= 1 && j <= g.Nx - 1;        // vy, vyD
    }
}

// r = b - A x on one level (the untiled smoother does not produce it).
template <typename T>
__global__ void k_resid(int N, const int32_t* __restrict__ col, const T* __restrict__ val, const T* __restrict__ b,
                        const T* __restrict__ x, T* r) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    T acc = b[k];
#pragma unroll
    for (int q = 0; q < HMEC_W; q++) {
        const size_t o = (size_t)q * N + k;
        acc -= val[o] * x[col[o]];
    }
    r[k] = acc;
}

// Coarse assembly coefficients from the fine ones.
struct CoefIn {
    const double *ETA, *GGG, *RHO;                          // basic
    const double *ETAP, *GGGP, *ETAB, *POR, *GGGB;          // P
    const double *RHOX, *RHOFX, *PORX, *ETADX;              // Vx
    const double *RHOY, *RHOFY, *PORY, *ETADY;              // Vy
};
struct CoefOut {
    double *ETA, *GGG, *RHO, *ETAP, *GGGP, *ETAB, *POR, *GGGB, *RHOX, *RHOFX, *PORX, *ETADX, *RHOY, *RHOFY, *PORY, *ETADY;
};

__global__ void k_coarsen_coef(Geo gf, Geo gc, CoefIn F, CoefOut C, int flags) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int J = blockIdx.y;
    // blockIdx.z: the section (basic, P, Vx, Vy nodes), independent of one
    // another; one thread each keeps the serial fine-node loops short
    const int sec = blockIdx.z;
    if (I >= gc.Ny1) return;
    const Map1D mx = mapx(gf, gc), my = mapy(gf, gc);
    // basic nodes: hat (full) weighting of the fine nodes; G harmonically
    if (sec == 0 && I < gc.Ny && J < gc.Nx) {
        double se = 0, sg = 0, sr = 0, w = 0;
        int i0, i1, j0, j1;
        m_hat_range(my, I, i0, i1);
        m_hat_range(mx, J, j0, j1);
        for (int i = i0; i <= min(i1, gf.Ny - 1); i++)
            for (int j = j0; j <= min(j1, gf.Nx - 1); j++) {
                const double ww = m_hat(my, i, I) * m_hat(mx, j, J);
                if (ww == 0.0) continue;
                const size_t o = (size_t)j * gf.Ny + i;
                se += ww * F.ETA[o];
                sg += ww / F.GGG[o];
                sr += ww * F.RHO[o];
                w += ww;
            }
        const size_t oc = (size_t)J * gc.Ny + I;
        C.ETA[oc] = se / w;
        C.GGG[oc] = w / sg;
        C.RHO[oc] = sr / w;
    }
    const size_t oc = (size_t)J * gc.Ny1 + I;
    // P nodes: average of the fine cells whose centres lie in the coarse cell
    if (sec != 1) {
    } else if (I >= 1 && I <= gc.Ny - 1 && J >= 1 && J <= gc.Nx - 1) {
        double se = 0, sg = 0, sb = 0, sp = 0, sgb = 0, w = 0;
        int i0, i1, j0, j1;
        m_cell_range(my, I, i0, i1);
        m_cell_range(mx, J, j0, j1);
        for (int i = i0; i <= i1; i++) {
            if (m_cell(my, i) != I) continue;
            for (int j = j0; j <= j1; j++) {
                if (m_cell(mx, j) != J) continue;
                const size_t o = (size_t)j * gf.Ny1 + i;
                se += F.ETAP[o];
                sg += 1.0 / F.GGGP[o];
                sb += F.ETAB[o];
                sp += F.POR[o];
                sgb += 1.0 / F.GGGB[o];
                w += 1.0;
            }
        }
        C.ETAP[oc] = se / w;
        C.GGGP[oc] = w / sg;
        C.ETAB[oc] = sb / w;
        C.POR[oc] = sp / w;
        C.GGGB[oc] = w / sgb;
    } else {
        C.ETAP[oc] = 1;
        C.GGGP[oc] = 1;
        C.ETAB[oc] = 1;
        C.POR[oc] = 0.5;
        C.GGGB[oc] = 1;
    }
    // Vx nodes (I, J): fine rows in coarse row I, fine columns hat-weighted
    // around coarse column J (ghost columns excluded)
    if (sec == 2) {
        double a[4] = {0, 0, 0, 0}, w = 0;
        int r0, r1, q0, q1;
        m_cell_range(my, I, r0, r1);
        m_hat_range(mx, J, q0, q1);
        q1 = min(q1, gf.Nx - 1);
        for (int i = r0; i <= r1; i++) {
            if (m_cell(my, i) != I) continue;
            for (int j = q0; j <= q1; j++) {
                const double ww = m_hat(mx, j, J);
                if (ww == 0.0) continue;
                const size_t o = (size_t)j * gf.Ny1 + i;
                a[0] += ww * F.RHOX[o];
                a[1] += ww * F.RHOFX[o];
                a[2] += ww * F.PORX[o];
                a[3] += ww * F.ETADX[o];
                w += ww;
            }
        }
        if (w > 0) {
            C.RHOX[oc] = a[0] / w;
            C.RHOFX[oc] = a[1] / w;
            C.PORX[oc] = a[2] / w;
            C.ETADX[oc] = a[3] / w;
            if (flags & HMEC_MG_DARCY_HARMONIC) {
                // x-flow: rows in parallel (mean conductance), columns in series (mean resistance)
                double rs = 0, wr = 0;
                for (int j = q0; j <= q1; j++) {
                    const double ww = m_hat(mx, j, J);
                    if (ww == 0.0) continue;
                    double cs = 0;
                    int nc = 0;
                    for (int i = r0; i <= r1; i++) {
                        if (m_cell(my, i) != I) continue;
                        const double e = F.ETADX[(size_t)j * gf.Ny1 + i];
                        if (e > 0) {
                            cs += 1.0 / e;
                            nc++;
                        }
                    }
                    if (nc == 0) continue;
                    rs += ww * (nc / cs);
                    wr += ww;
                }
                if (wr > 0) C.ETADX[oc] = rs / wr;
            }
        } else {
            C.RHOX[oc] = 0;
            C.RHOFX[oc] = 0;
            C.PORX[oc] = 1;
            C.ETADX[oc] = 1;
        }
    }
    // Vy nodes (I, J): fine columns in coarse column J, fine rows hat-weighted
    // around coarse row I (ghost rows excluded)
    if (sec == 3) {
        double a[4] = {0, 0, 0, 0}, w = 0;
        int c0, c1, q0, q1;
        m_cell_range(mx, J, c0, c1);
        m_hat_range(my, I, q0, q1);
        q1 = min(q1, gf.Ny - 1);
        for (int j = c0; j <= c1; j++) {
            if (m_cell(mx, j) != J) continue;
            for (int i = q0; i <= q1; i++) {
                const double ww = m_hat(my, i, I);
                if (ww == 0.0) continue;
                const size_t o = (size_t)j * gf.Ny1 + i;
                a[0] += ww * F.RHOY[o];
                a[1] += ww * F.RHOFY[o];
                a[2] += ww * F.PORY[o];
                a[3] += ww * F.ETADY[o];
                w += ww;
            }
        }
        if (w > 0) {
            C.RHOY[oc] = a[0] / w;
            C.RHOFY[oc] = a[1] / w;
            C.PORY[oc] = a[2] / w;
            C.ETADY[oc] = a[3] / w;
            if (flags & HMEC_MG_DARCY_HARMONIC) {
                // y-flow: columns in parallel, rows in series
                double rs = 0, wr = 0;
                for (int i = q0; i <= q1; i++) {
                    const double ww = m_hat(my, i, I);
                    if (ww == 0.0) continue;
                    double cs = 0;
                    int nc = 0;
                    for (int j = c0; j <= c1; j++) {
                        if (m_cell(mx, j) != J) continue;
                        const double e = F.ETADY[(size_t)j * gf.Ny1 + i];
                        if (e > 0) {
                            cs += 1.0 / e;
                            nc++;
                        }
                    }
                    if (nc == 0) continue;
                    rs += ww * (nc / cs);
                    wr += ww;
                }
                if (wr > 0) C.ETADY[oc] = rs / wr;
            }
        } else {
            C.RHOY[oc] = 0;
            C.RHOFY[oc] = 0;
            C.PORY[oc] = 1;
            C.ETADY[oc] = 1;
        }
    }
}

// Restriction: coarse rhs = the transpose of the prolongation applied to the
// fine residual in physical units r/df, weights normalised, scaled by the
// coarse row scale.  Only interior equations are restricted, and only from
// fine interior equations; coarse boundary rows get a zero residual, so the
// coarse correction obeys the homogeneous boundary conditions, which the
// prolongation preserves.  The geometric part is a fixed table of HMEC_RW
// (fine unknown, weight) pairs per coarse unknown, slot-major (built once per
// allocation); the row-scale ratio dsc/df is folded in after each assembly.
static bool restrict_table(const Geo& gf, const Geo& gc, std::vector<int32_t>& idx, std::vector<double>& w) {
    const size_t Nc = (size_t)gc.N;
    idx.assign(HMEC_RW * Nc, 0);
    w.assign(HMEC_RW * Nc, 0.0);
    const Map1D mx = mapx(gf, gc), my = mapy(gf, gc);
    for (int J = 0; J <= gc.Nx; J++)
        for (int I = 0; I <= gc.Ny; I++)
            for (int v = 0; v < 6; v++) {
                const size_t t = ((size_t)J * gc.Ny1 + I) * 6 + v;
                if (!row_interior(gc, I, J, v)) continue;
                const bool xnode = v == 1 || v == 4, ynode = v == 2 || v == 5;
                int i0, i1, j0, j1;
                if (ynode) m_hat_range(my, I, i0, i1); else m_cell_range(my, I, i0, i1);
                if (xnode) m_hat_range(mx, J, j0, j1); else m_cell_range(mx, J, j0, j1);
                int n = 0;
                int32_t ks[HMEC_RW];
                double ws[HMEC_RW], sum = 0;
                for (int i = i0; i <= i1; i++) {
                    const double wi = ynode ? m_hat(my, i, I) : (m_cell(my, i) == I ? 1.0 : 0.0);
                    if (wi == 0.0) continue;
                    for (int j = j0; j <= j1; j++) {
                        const double wj = xnode ? m_hat(mx, j, J) : (m_cell(mx, j) == J ? 1.0 : 0.0);
                        if (wj == 0.0 || !row_interior(gf, i, j, v)) continue;
                        if (n == HMEC_RW) return false;
                        ks[n] = (int32_t)(((size_t)j * gf.Ny1 + i) * 6 + v);
                        ws[n] = wi * wj;
                        sum += ws[n];
                        n++;
                    }
                }
                for (int e = 0; e < HMEC_RW; e++) {
                    idx[e * Nc + t] = n ? ks[e < n ? e : 0] : 0;
                    w[e * Nc + t] = e < n ? ws[e] / sum : 0.0;
                }
            }
    return true;
}

// rw = rwg * dsc / df (after each assembly of the two levels)
__global__ void k_restrict_scale(int Nc, const int32_t* __restrict__ ridx, const double* __restrict__ rwg,
                                 const double* __restrict__ dsf, const double* __restrict__ dsc, double* rw,
                                 float* rw32) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Nc) return;
#pragma unroll
    for (int e = 0; e < HMEC_RW; e++) {
        const size_t o = (size_t)e * Nc + t;
        const double g = rwg[o];
        const double v = g == 0.0 ? 0.0 : g * dsc[t] / dsf[ridx[o]];
        rw[o] = v;
        if (rw32) rw32[o] = (float)v;
    }
}

template <typename T>
__device__ __forceinline__ void restrict_apply(int Nc, const int32_t* __restrict__ ridx, const T* __restrict__ rw,
                                               const T* __restrict__ rf, T* bc, int tid, int nth) {
    for (int t = tid; t < Nc; t += nth) {
        T s = 0;
#pragma unroll
        for (int e = 0; e < HMEC_RW; e++) {
            const size_t o = (size_t)e * Nc + t;
            s += rw[o] * rf[ridx[o]];
        }
        bc[t] = s;
    }
}

template <typename T>
__global__ void k_restrict(int Nc, const int32_t* __restrict__ ridx, const T* __restrict__ rw,
                           const T* __restrict__ rf, T* bc) {
    restrict_apply(Nc, ridx, rw, rf, bc, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

template <typename S, typename D>
__global__ void k_convert(size_t n, const S* __restrict__ a, D* b) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (D)a[t];
}

template <typename T>
__global__ void k_zero(size_t n, T* a) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = (T)0;
}

// ------------------------------------------------------------ FGMRES
// r = b - A x, with partial sums of |r|^2 and |b|^2
__global__ void k_true_resid(int N, const int32_t* __restrict__ col, const double* __restrict__ val,
                             const double* __restrict__ b, const double* __restrict__ x, double* r, double* partial,
                             int nblk) {
    __shared__ double s1[RED_BS], s2[RED_BS];
    double a1 = 0, a2 = 0;
    for (int row = blockIdx.x * RED_BS + threadIdx.x; row < N; row += nblk * RED_BS) {
        double acc = b[row];
#pragma unroll
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * N + row;
            acc -= val[o] * x[col[o]];
        }
        r[row] = acc;
        a1 += acc * acc;
        a2 += b[row] * b[row];
    }
    s1[threadIdx.x] = a1;
    s2[threadIdx.x] = a2;
    __syncthreads();
    for (int s = RED_BS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            s1[threadIdx.x] += s1[threadIdx.x + s];
            s2[threadIdx.x] += s2[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = s1[0];
        partial[nblk + blockIdx.x] = s2[0];
    }
}

// Start of a restart cycle: beta = ||r||, relres check, V0 = r / beta, g = beta e1.
struct Gm {
    double* H;
    double* cs;
    double* sn;
    double* g;
    double* y;
    double* dots;
    double* bnorm;
    int* done;
    int* kcur;
    DevScalars* ds;
};

// Sum of p[0..n) by one warp in a fixed order (lane-strided partial sums, then
// a shuffle-down tree); the result is lane 0's, broadcast to the warp.
__device__ __forceinline__ double warp_sum_fixed(const double* __restrict__ p, int n) {
    double a = 0;
    for (int b = threadIdx.x; b < n; b += 32) a += p[b];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    return __shfl_sync(0xffffffffu, a, 0);
}

// One warp; lane 0 does the scalar updates.
__global__ void k_cycle_begin(Gm G, const double* __restrict__ partial, int nblk, int first, double rtol, int m) {
    const double rr = warp_sum_fixed(partial, nblk);
    const double bb = warp_sum_fixed(partial + nblk, nblk);
    for (int k = 1 + threadIdx.x; k <= m; k += 32) G.g[k] = 0;
    if (threadIdx.x != 0) return;
    if (first) *G.bnorm = sqrt(bb);
    const double bn = *G.bnorm;
    const double beta = sqrt(rr);
    const double rel = bn > 0 ? beta / bn : beta;
    G.ds->krylov_relres = rel;
    G.g[0] = beta;
    *G.kcur = 0;
    *G.done = (rel <= rtol || !(beta > 0) || !isfinite(beta)) ? 1 : 0;
    G.dots[0] = beta > 0 ? 1.0 / beta : 0.0;  // scale for V0
}

// b = a * sc[0]; the preconditioner's first input is copied beside it when
// c32 (mixed form) or c64 (FP64 form, device-controlled solve) is set.
__global__ void k_scale_vec(int N, const double* __restrict__ a, const double* sc, double* b, const int* done,
                            float* c32, double* c64) {
    if (*done) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < N) {
        const double v = a[r] * sc[0];
        b[r] = v;
        if (c32) c32[r] = (float)v;
        if (c64) c64[r] = v;
    }
}

// After the two CGS passes: column j of H, Givens rotation, residual estimate.
// One warp; lane 0 applies the rotations.
__device__ __forceinline__ void arnoldi_update(const Gm& G, const double* __restrict__ h1,
                                               const double* __restrict__ partial, int nblk, int j, int m, double rtol,
                                               double* hscale) {
    const double hn = sqrt(warp_sum_fixed(partial, nblk));
    double* Hc = G.H + (size_t)j * (m + 1);  // column j, rows 0..j+1
    for (int k = threadIdx.x; k <= j; k += 32) Hc[k] = h1[k] + G.dots[k];  // first + second CGS pass
    __syncwarp();
    if (threadIdx.x != 0) return;
    Hc[j + 1] = hn;
    for (int k = 0; k < j; k++) {  // previous rotations
        const double t = G.cs[k] * Hc[k] + G.sn[k] * Hc[k + 1];
        Hc[k + 1] = -G.sn[k] * Hc[k] + G.cs[k] * Hc[k + 1];
        Hc[k] = t;
    }
    const double a = Hc[j], b = Hc[j + 1];
    const double rho = sqrt(a * a + b * b);
    const double c = rho > 0 ? a / rho : 1.0, s = rho > 0 ? b / rho : 0.0;
    G.cs[j] = c;
    G.sn[j] = s;
    Hc[j] = rho;
    Hc[j + 1] = 0;
    G.g[j + 1] = -s * G.g[j];
    G.g[j] = c * G.g[j];
    *G.kcur = j + 1;
    const double rel = fabs(G.g[j + 1]) / *G.bnorm;
    G.ds->krylov_relres = rel;
    G.ds->krylov_iters += 1;
    hscale[0] = hn > 0 ? 1.0 / hn : 0.0;
    if (rel <= rtol || !(hn > 0) || !isfinite(rel)) *G.done = 1;
}

// One Arnoldi step of FGMRES after the preconditioner, as one cooperative
// launch: z_j (FP64, from the preconditioner's output zsrc), w = A z_j,
// classical Gram-Schmidt twice against V_0..V_j, the Hessenberg column with
// its Givens rotation, and V_{j+1} = w / |w| (plus its FP32 copy, the next
// preconditioner input of the mixed form).  Every reduction is a block
// partial then one warp per coefficient in a fixed order (deterministic).
template <typename TZ>
struct ArnArgs {
    int N, j, m, nblk;
    const int32_t* col;
    const double* val;
    const TZ* zsrc;
    double* Zj;          // z_j in FP64 (may equal zsrc)
    double* V;           // (m+1) x N basis
    double* w;
    double* partial;     // (m+2) x nblk
    Gm G;
    double rtol;
    float* next32;       // if set: FP32 copy of V_{j+1}
    double* next64;      // if set: FP64 copy of V_{j+1} (the FP64 form's next preconditioner input)
    // device-controlled solve (graph): j is read from jdev (the steps taken
    // in the cycle) and z_j lands in Zbase + j N
    const int* jdev;
    double* Zbase;
};

constexpr int ARN_BS = 256;

// thread 0 of the block gets the block's sum of v (fixed order)
__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int k = 0; k < ARN_BS / 32; k++) s += sh[k];
    __syncthreads();
    return s;
}

// partial[k*nblk + block] = this block's part of V_k . w, k = 0..j: the block
// takes a contiguous range of rows and each warp whole coefficients, so no
// block barrier is needed (w stays in L1 across the warp's coefficients)
__device__ __forceinline__ void dots_partial(const double* __restrict__ V, const double* __restrict__ w, int N, int j,
                                             double* partial, int nblk) {
    const int chunk = ((N + nblk - 1) / nblk + 31) / 32 * 32;
    const int r0 = blockIdx.x * chunk, r1 = min(N, r0 + chunk);
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x >> 5; k <= j; k += ARN_BS / 32) {
        const double* v = V + (size_t)k * N;
        double a = 0;
        for (int r = r0 + lane; r < r1; r += 32) a += v[r] * w[r];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) partial[(size_t)k * nblk + blockIdx.x] = a;
    }
}

// Every block: shh[k] = sum over blocks of partial[k][.], one warp per k, in
// a fixed order (so all blocks hold identical coefficients and no grid
// barrier is needed to share them); block 0 also stores them in h.
__device__ __forceinline__ void dots_local(const double* __restrict__ partial, int nblk, int j, double* shh,
                                           double* h) {
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x >> 5; k <= j; k += ARN_BS / 32) {
        double a = 0;
        for (int b = lane; b < nblk; b += 32) a += partial[(size_t)k * nblk + b];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) {
            shh[k] = a;
            if (blockIdx.x == 0) h[k] = a;
        }
    }
    __syncthreads();
}

// w -= sum_k shh[k] V_k; normp[block] = this block's part of |w|^2
__device__ __forceinline__ void orth_update(const double* __restrict__ V, double* w, int N, int j, double* normp,
                                            int nblk, double* sh, const double* shh) {
    double a2 = 0;
    const int chunk = ((N + nblk - 1) / nblk + 31) / 32 * 32;
    const int r1 = min(N, (int)blockIdx.x * chunk + chunk);
    for (int r = blockIdx.x * chunk + threadIdx.x; r < r1; r += ARN_BS) {
        double x = w[r];
        for (int k = 0; k <= j; k++) x -= shh[k] * V[(size_t)k * N + r];
        w[r] = x;
        a2 += x * x;
    }
    if (!normp) {
        __syncthreads();
        return;
    }
    const double s = block_sum(a2, sh);
    if (threadIdx.x == 0) normp[blockIdx.x] = s;
}

// dynamic shared memory: (m + 1) doubles
template <typename TZ>
__global__ void __launch_bounds__(ARN_BS) k_arnoldi(ArnArgs<TZ> a) {
    __shared__ double sh[ARN_BS / 32];
    extern __shared__ double shh[];
    if (*a.G.done) return;  // set only by an earlier launch: uniform across the grid
    cg::grid_group grid = cg::this_grid();
    const int N = a.N, m = a.m, nblk = a.nblk;
    // the step index: a kernel argument, or (device-controlled solve) the
    // steps taken so far, read before the first grid barrier and rewritten
    // by block 0 only after the last one
    const int j = a.jdev ? *a.jdev : a.j;
    double* const Zj = a.jdev ? a.Zbase + (size_t)j * N : a.Zj;
    double* dots = a.G.dots;
    // z_j and w = A z_j (rows in the block's contiguous range, as below)
    const int chunk = ((N + nblk - 1) / nblk + 31) / 32 * 32;
    const int rend = min(N, (int)blockIdx.x * chunk + chunk);
    // (an FP32 z is widened through its bit pattern: the same FP64 values in
    // z_j and in the product, without FP64-rate conversions)
    for (int r = blockIdx.x * chunk + threadIdx.x; r < rend; r += ARN_BS) {
        if ((const void*)a.zsrc != (const void*)Zj) Zj[r] = to_f64(a.zsrc[r]);
        double acc = 0;
#pragma unroll
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * N + r;
            acc += a.val[o] * to_f64(a.zsrc[a.col[o]]);
        }
        a.w[r] = acc;
    }
    // from here on a block reads and writes only its own rows of w
    __syncthreads();
    // classical Gram-Schmidt, two passes ("twice is enough"); the second
    // pass's partials use rows m+1.. of partial, so the first pass's rows are
    // not overwritten while slower blocks still read them, and |w|^2 goes to
    // row 2m+2.  Three grid barriers: each pass's partials, then |w|.
    double* part2 = a.partial + (size_t)(m + 1) * nblk;
    double* normp = a.partial + (size_t)(2 * m + 2) * nblk;
    dots_partial(a.V, a.w, N, j, a.partial, nblk);
    grid.sync();
    dots_local(a.partial, nblk, j, shh, dots + m + 2);
    orth_update(a.V, a.w, N, j, nullptr, nblk, sh, shh);
    dots_partial(a.V, a.w, N, j, part2, nblk);
    grid.sync();
    dots_local(part2, nblk, j, shh, dots);
    orth_update(a.V, a.w, N, j, normp, nblk, sh, shh);
    grid.sync();
    if (blockIdx.x == 0 && threadIdx.x < 32)
        arnoldi_update(a.G, dots + m + 2, normp, nblk, j, m, a.rtol, dots + 2 * m + 3);
    // V_{j+1} = w / |w| (written whether or not this step converged): every
    // block forms |w| from the same partials in the same order as
    // arnoldi_update and scales the rows it updated itself, so no grid
    // barrier is needed
    __shared__ double s_sc;
    if (threadIdx.x < 32) {
        const double hn = sqrt(warp_sum_fixed(normp, nblk));
        if (threadIdx.x == 0) s_sc = hn > 0 ? 1.0 / hn : 0.0;
    }
    __syncthreads();
    const double sc = s_sc;
    double* Vn = a.V + (size_t)(j + 1) * N;
    for (int r = blockIdx.x * chunk + threadIdx.x; r < rend; r += ARN_BS) {
        const double v = a.w[r] * sc;
        Vn[r] = v;
        if (a.next32) a.next32[r] = (float)v;
        if (a.next64) a.next64[r] = v;
    }
}

// ------------------------------------------- device-controlled solve (graph)
// The decisions the host takes between launches in solver_solve, taken on
// the device so that a solve can run inside a CUDA graph: conditional WHILE
// nodes repeat the restart cycle and the Arnoldi step, and these one-thread
// kernels set their conditions.  Every loop is bounded: an inner trip either
// ends the loop or advances the step count (at most m per cycle), and a
// cycle either stops or runs at least one Arnoldi step (at most krylov_maxit
// in the solve).
__global__ void k_solve_init(Gm G, GmCtl* c, int maxit, cudaGraphConditionalHandle h_restart) {
    G.ds->krylov_iters = 0;
    c->prev = INFINITY;
    c->first = 1;
    c->maxit = maxit;
    cudaGraphSetConditional(h_restart, 1u);
}

// k_cycle_begin, then the restart decision of solver_solve: converged,
// failed (non-finite or out of iterations; HMEC_DEV_KRYLOV_NOCONV), stalled
// near the rounding floor (accepted within 100 x rtol), or another cycle.
__global__ void k_cycle_begin_g(Gm G, const double* __restrict__ partial, int nblk, double rtol, int m, GmCtl* c,
                                cudaGraphConditionalHandle h_restart, cudaGraphConditionalHandle h_inner) {
    const double rr = warp_sum_fixed(partial, nblk);
    const double bb = warp_sum_fixed(partial + nblk, nblk);
    for (int k = 1 + threadIdx.x; k <= m; k += 32) G.g[k] = 0;
    if (threadIdx.x != 0) return;
    if (c->first) *G.bnorm = sqrt(bb);
    c->first = 0;
    const double bn = *G.bnorm;
    const double beta = sqrt(rr);
    const double rel = bn > 0 ? beta / bn : beta;
    G.ds->krylov_relres = rel;
    G.ds->krylov_cycles += 1;
    G.g[0] = beta;
    *G.kcur = 0;
    G.dots[0] = beta > 0 ? 1.0 / beta : 0.0;
    const int total = G.ds->krylov_iters;
    int more = 1, conv = 0;
    if (rel <= rtol) {
        more = 0;
        conv = 1;
    } else if (!isfinite(rel) || total >= c->maxit) {
        more = 0;
    } else if (total > 0 && rel > 0.5 * c->prev && rel <= 1e-10) {
        more = 0;
        conv = rel <= 100 * rtol;
    }
    c->prev = rel;
    *G.done = more ? 0 : 1;
    if (!more && !conv) atomicOr(&G.ds->status, HMEC_DEV_KRYLOV_NOCONV);
    cudaGraphSetConditional(h_restart, more ? 1u : 0u);
    cudaGraphSetConditional(h_inner, more ? 1u : 0u);
}

__global__ void k_inner_cond(Gm G, int m, const GmCtl* c, cudaGraphConditionalHandle h_inner) {
    const int more = !*G.done && *G.kcur < m && G.ds->krylov_iters < c->maxit;
    cudaGraphSetConditional(h_inner, more ? 1u : 0u);
}

// y = H^{-1} g (upper triangular, kcur columns)
__global__ void k_lsq(Gm G, int m) {
    const int k = *G.kcur;
    for (int r = k - 1; r >= 0; r--) {
        double s = G.g[r];
        for (int c = r + 1; c < k; c++) s -= G.H[(size_t)c * (m + 1) + r] * G.y[c];
        const double d = G.H[(size_t)r * (m + 1) + r];
        G.y[r] = d != 0 ? s / d : 0.0;
    }
}

__global__ void k_xupdate(int N, const double* __restrict__ Z, const double* __restrict__ y, const int* kcur, double* x) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    const int k = *kcur;
    double acc = x[r];
    for (int c = 0; c < k; c++) acc += y[c] * Z[(size_t)c * N + r];
    x[r] = acc;
}

}  // namespace


// ===================================================================== host

static std::vector<int32_t> boundary_rows(const Geo& g) {
    std::vector<int32_t> r;
    for (int j = 0; j <= g.Nx; j++)
        for (int i = 0; i <= g.Ny; i++) {
            const int kp = (j * g.Ny1 + i) * 6;
            const bool pin = (i >= 1 && i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 1);
            const bool vxin = (i >= 1 && i <= g.Ny - 1 && j <= g.Nx - 1);
            const bool vyin = (i <= g.Ny - 1 && j >= 1 && j <= g.Nx - 1);
            if (!pin) {
                r.push_back(kp + 0);
                r.push_back(kp + 3);
            }
            if (!vxin) {
                r.push_back(kp + 1);
                r.push_back(kp + 4);
            }
            if (!vyin) {
                r.push_back(kp + 2);
                r.push_back(kp + 5);
            }
        }
    std::sort(r.begin(), r.end());
    return r;
}

// A 3-D TMA descriptor of a dense array [d2][d1][d0] (d0 fastest) with box
// (b0, b1, b2); elements outside the array load as zero.  The encoder is the
// driver's cuTensorMapEncodeTiled, reached through the runtime.
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int encode_map3(hmec_inst* ctx, CUtensorMap* map, CUtensorMapDataType dt, size_t esize, void* base,
                       uint64_t d0, uint64_t d1, uint64_t d2, uint32_t b0, uint32_t b1, uint32_t b2) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
            ctx->err = "cuTensorMapEncodeTiled is not available from the driver";
            return HMEC_ERR_CUDA;
        }
        fn = (EncodeTiledFn)p;
    }
    const cuuint64_t dims[3] = {d0, d1, d2};
    const cuuint64_t strides[2] = {d0 * esize, d0 * d1 * esize};
    const cuuint32_t box[3] = {b0, b1, b2};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = fn(map, dt, 3, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        ctx->err = "cuTensorMapEncodeTiled rejected a smoother descriptor";
        return HMEC_ERR_CUDA;
    }
    return HMEC_OK;
}

static int alloc_level(hmec_inst* ctx, Level& L, bool mixed, bool coarse) {
    const Geo& g = L.g;
    const size_t N = (size_t)g.N;
    L.npatch = (g.Ny - 1) * (g.Nx - 1);
    L.pmx = L.pmy = nullptr;
    L.ridx = nullptr;
    L.rwg = L.rw = nullptr;
    L.rw32 = nullptr;
    HMEC_CUDA(ctx, cudaMalloc(&L.col, sizeof(int32_t) * HMEC_W * N));
    HMEC_CUDA(ctx, cudaMalloc(&L.val, sizeof(double) * HMEC_W * N));
    HMEC_CUDA(ctx, cudaMalloc(&L.dscale, sizeof(double) * N));
    std::vector<int32_t> br = boundary_rows(g);
    L.nbnd = (int)br.size();
    HMEC_CUDA(ctx, cudaMalloc(&L.bnd_rows, sizeof(int32_t) * std::max<size_t>(br.size(), 1)));
    HMEC_CUDA(ctx, cudaMemcpy(L.bnd_rows, br.data(), sizeof(int32_t) * br.size(), cudaMemcpyHostToDevice));
    L.pinv = nullptr;
    L.pinv32 = nullptr;
    L.val32 = nullptr;
    L.fx = L.fb = L.fr = nullptr;
    L.dx_ = L.db = L.dr = L.pb = nullptr;
    HMEC_CUDA(ctx, cudaMalloc(&L.db, sizeof(double) * N));  // fine: scaled rhs; coarse: FP64 rhs
    L.dx2 = nullptr;
    L.fx2 = nullptr;
    if (mixed) {
        HMEC_CUDA(ctx, cudaMalloc(&L.val32, sizeof(float) * HMEC_W * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.pinv32, sizeof(float) * 100 * (size_t)L.npatch));
        HMEC_CUDA(ctx, cudaMalloc(&L.fx, sizeof(float) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.fx2, sizeof(float) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.fb, sizeof(float) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.fr, sizeof(float) * std::max(N, (size_t)L.nbnd)));
    } else {
        HMEC_CUDA(ctx, cudaMalloc(&L.pinv, sizeof(double) * 100 * (size_t)L.npatch));
        HMEC_CUDA(ctx, cudaMalloc(&L.dx_, sizeof(double) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.dx2, sizeof(double) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.dr, sizeof(double) * std::max(N, (size_t)L.nbnd)));
        // the fine level's fixed preconditioner input (device-controlled solve)
        if (!coarse) HMEC_CUDA(ctx, cudaMalloc(&L.pb, sizeof(double) * N));
    }
    {
        // tile ownership of every unknown (the tiled smoothing pass)
        L.tsz = TILE;
        L.ntile_i = (g.Ny - 1 + TILE - 1) / TILE;
        const int ntile_j = (g.Nx - 1 + TILE - 1) / TILE;
        L.ntiles = L.ntile_i * ntile_j;
        std::vector<int32_t> owner(N);
        std::vector<char> isb(N, 0);
        for (int32_t r : br) isb[r] = 1;
        for (int j = 0; j <= g.Nx; j++)
            for (int i = 0; i <= g.Ny; i++)
                for (int v = 0; v < 6; v++) owner[(j * g.Ny1 + i) * 6 + v] = unknown_tile(g, L.ntile_i, i, j, v);
        // each tile's boundary rows, listed tile by tile
        std::vector<int32_t> bs(L.ntiles + 1, 0);
        for (size_t u = 0; u < N; u++)
            if (isb[u]) bs[owner[u] + 1]++;
        int tbm = 0;
        for (int k = 0; k < L.ntiles; k++) tbm = std::max(tbm, (int)bs[k + 1]);
        if (tbm > TB_MAX) {
            ctx->err = "a smoothing tile has more boundary rows than its shared-memory stage holds";
            return HMEC_ERR_ARG;
        }
        L.tb_cap = std::max(16, (tbm + 15) / 16 * 16);
        for (int k = 0; k < L.ntiles; k++) bs[k + 1] += bs[k];
        std::vector<int32_t> bl(std::max<size_t>(br.size(), 1)), bc(bs.begin(), bs.end() - 1);
        for (size_t u = 0; u < N; u++)
            if (isb[u]) bl[bc[owner[u]]++] = (int32_t)u;
        HMEC_CUDA(ctx, cudaMalloc(&L.tbnd_start, sizeof(int32_t) * bs.size()));
        HMEC_CUDA(ctx, cudaMalloc(&L.tbnd_list, sizeof(int32_t) * bl.size()));
        HMEC_CUDA(ctx, cudaMemcpy(L.tbnd_start, bs.data(), sizeof(int32_t) * bs.size(), cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(L.tbnd_list, bl.data(), sizeof(int32_t) * bl.size(), cudaMemcpyHostToDevice));
        // per tile: its window's ownership bits, and the per-lane colour
        // table with bit 31 set where the tile owns the unknown of the lane's
        // patch row
        std::vector<uint32_t> ownt((size_t)L.ntiles * (OWN_BYTES / 4), 0u);
        std::vector<int32_t> meta((size_t)L.ntiles * 9 * TILE_BS, 0);
        for (int tile = 0; tile < L.ntiles; tile++) {
            const int ti = tile % L.ntile_i, tj = tile / L.ntile_i;
            const int i0 = 1 + ti * TILE, j0 = 1 + tj * TILE;
            const int i1 = std::min(i0 + TILE, g.Ny), j1 = std::min(j0 + TILE, g.Nx);
            for (int lw = 0; lw < WIN_MAX; lw++) {
                const int lc = lw / 6, v = lw - 6 * lc;
                const int ci = i0 - 2 + lc % WSTR, cj = j0 - 2 + lc / WSTR;
                if (ci >= 0 && ci <= g.Ny && cj >= 0 && cj <= g.Nx && owner[(cj * g.Ny1 + ci) * 6 + v] == tile)
                    ownt[(size_t)tile * (OWN_BYTES / 4) + (lw >> 5)] |= 1u << (lw & 31);
            }
            for (int c = 0; c < 9; c++)
                for (int tt = 0; tt < TILE_BS; tt++) {
                    int m = lane_meta(c, tt, i0, j0, i1, j1);
                    if ((m >> 30) & 1) {
                        const int lw = m & 2047, lc = lw / 6, v = lw - 6 * lc;
                        const int ci = i0 - 2 + lc % WSTR, cj = j0 - 2 + lc / WSTR;
                        if (ci >= 0 && ci <= g.Ny && cj >= 0 && cj <= g.Nx &&
                            owner[(cj * g.Ny1 + ci) * 6 + v] == tile)
                            m = (int)((unsigned)m | 0x80000000u);
                    }
                    meta[((size_t)tile * 9 + c) * TILE_BS + tt] = m;
                }
        }
        HMEC_CUDA(ctx, cudaMalloc(&L.own_t, sizeof(uint32_t) * ownt.size()));
        HMEC_CUDA(ctx, cudaMemcpy(L.own_t, ownt.data(), sizeof(uint32_t) * ownt.size(), cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMalloc(&L.meta_t, sizeof(int32_t) * meta.size()));
        HMEC_CUDA(ctx, cudaMemcpy(L.meta_t, meta.data(), sizeof(int32_t) * meta.size(), cudaMemcpyHostToDevice));
        // the smoother's padded matrix copy, the boundary packs, and their TMA maps
        const size_t st = mixed ? sizeof(float) : sizeof(double);
        L.CS = align_up(6 * g.Ny1, 8);
        const size_t ns = (size_t)HMEC_W * g.Nx1 * L.CS;
        HMEC_CUDA(ctx, cudaMalloc(&L.vals, st * ns));
        HMEC_CUDA(ctx, cudaMalloc(&L.offs, sizeof(int16_t) * ns));
        HMEC_CUDA(ctx, cudaMemset(L.vals, 0, st * ns));
        HMEC_CUDA(ctx, cudaMemset(L.offs, 0, sizeof(int16_t) * ns));
        HMEC_CUDA(ctx, cudaMalloc(&L.std_off, sizeof(int16_t) * 6 * HMEC_W));
        HMEC_CUDA(ctx, cudaMalloc(&L.std_t, (size_t)L.ntiles));
        HMEC_CUDA(ctx, cudaMemset(L.std_off, 0, sizeof(int16_t) * 6 * HMEC_W));
        HMEC_CUDA(ctx, cudaMemset(L.std_t, 0, (size_t)L.ntiles));
        L.pack_bytes = mixed ? pack_bytes<float>(L.tb_cap) : pack_bytes<double>(L.tb_cap);
        HMEC_CUDA(ctx, cudaMalloc(&L.bpack, (size_t)L.ntiles * L.pack_bytes));
        const CUtensorMapDataType dt = mixed ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
        int rc = encode_map3(ctx, &L.tm_val, dt, st, L.vals, L.CS, g.Nx1, HMEC_W, RSTR, TILE + 1, HMEC_W);
        if (!rc)
            rc = encode_map3(ctx, &L.tm_pinv, dt, st, mixed ? (void*)L.pinv32 : (void*)L.pinv, 100, g.Ny - 1, g.Nx - 1,
                             100, TILE, TILE);
        if (rc) return rc;
    }
    if (coarse) {
        const size_t nb = (size_t)g.Nx * g.Ny, ns = (size_t)g.Nx1 * g.Ny1;
        auto mk = [&](size_t n) -> double* {
            double* p = nullptr;
            if (cudaMalloc(&p, sizeof(double) * n) != cudaSuccess) return nullptr;
            cudaMemset(p, 0, sizeof(double) * n);
            L.owned.push_back(p);
            return p;
        };
        AsmFields& a = L.af;
        memset(&a, 0, sizeof(a));
        a.ETA = mk(nb);
        a.GGG = mk(nb);
        a.RHO = mk(nb);
        a.ETAP = mk(ns);
        a.GGGP = mk(ns);
        a.ETAB = mk(ns);
        a.POR = mk(ns);
        a.GGGB = mk(ns);
        a.RHOX = mk(ns);
        a.RHOFX = mk(ns);
        a.PORX = mk(ns);
        a.ETADX = mk(ns);
        a.RHOY = mk(ns);
        a.RHOFY = mk(ns);
        a.PORY = mk(ns);
        a.ETADY = mk(ns);
        for (double* p : L.owned)
            if (!p) {
                ctx->err = "cudaMalloc failed for a coarse level";
                return HMEC_ERR_NOMEM;
            }
    }
    return HMEC_OK;
}

int solver_alloc(hmec_inst* ctx) {
    Solver& sv = ctx->sv;
    const hmec_params& p = ctx->p;
    const bool mixed = p.form == HMEC_FORM_MIXED;
    sv.m = std::max(2, p.krylov_restart);
    sv.N = ctx->g.N;
    {
        // Arnoldi blocks: the tuned count, else two per SM
        int nsm = 0;
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
        sv.nblk = p.krylov_blocks > 0 ? std::min(p.krylov_blocks, 65536) : 2 * std::max(1, nsm);
    }
    // levels: ceil-halve the cell counts while the coarse grid keeps >= 4 cells per side
    Level L0;
    L0.g = ctx->g;
    sv.lv.push_back(L0);
    int nx = ctx->g.Nx, ny = ctx->g.Ny;
    double xs = p.xsize, ys = p.ysize;
    while ((int)sv.lv.size() < std::max(1, p.mg_levels)) {
        const int cx = (nx - 1 + 1) / 2, cy = (ny - 1 + 1) / 2;
        if (cx < 4 || cy < 4) break;
        nx = cx + 1;
        ny = cy + 1;
        Level L;
        geo_make(L.g, nx, ny, xs, ys);
        sv.lv.push_back(L);
    }
    for (size_t l = 0; l < sv.lv.size(); l++) {
        int rc = alloc_level(ctx, sv.lv[l], mixed, l > 0);
        if (rc) return rc;
    }
    // grid transfer tables between consecutive levels
    for (size_t l = 0; l + 1 < sv.lv.size(); l++) {
        Level& F = sv.lv[l];
        Level& C = sv.lv[l + 1];
        const std::vector<XferEnt> tx = xfer_table(mapx(F.g, C.g)), ty = xfer_table(mapy(F.g, C.g));
        HMEC_CUDA(ctx, cudaMalloc(&F.pmx, sizeof(XferEnt) * tx.size()));
        HMEC_CUDA(ctx, cudaMalloc(&F.pmy, sizeof(XferEnt) * ty.size()));
        HMEC_CUDA(ctx, cudaMemcpy(F.pmx, tx.data(), sizeof(XferEnt) * tx.size(), cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(F.pmy, ty.data(), sizeof(XferEnt) * ty.size(), cudaMemcpyHostToDevice));
        std::vector<int32_t> ri;
        std::vector<double> rg;
        if (!restrict_table(F.g, C.g, ri, rg)) {
            ctx->err = "restriction stencil wider than HMEC_RW entries";
            return HMEC_ERR_ARG;
        }
        const size_t n = ri.size();
        HMEC_CUDA(ctx, cudaMalloc(&C.ridx, sizeof(int32_t) * n));
        HMEC_CUDA(ctx, cudaMalloc(&C.rwg, sizeof(double) * n));
        HMEC_CUDA(ctx, cudaMalloc(&C.rw, sizeof(double) * n));
        if (mixed) HMEC_CUDA(ctx, cudaMalloc(&C.rw32, sizeof(float) * n));
        HMEC_CUDA(ctx, cudaMemcpy(C.ridx, ri.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(C.rwg, rg.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
    }
    // fine-level assembly reads the model fields
    AsmFields& a = sv.lv[0].af;
    double* const* f = ctx->f;
    a.ETA = f[HMEC_F_ETA];
    a.GGG = f[HMEC_F_GGG];
    a.RHO = f[HMEC_F_RHO];
    a.SXY0 = f[HMEC_F_SXY0];
    a.ETAP = f[HMEC_F_ETAP];
    a.GGGP = f[HMEC_F_GGGP];
    a.ETAB = f[HMEC_F_ETAB];
    a.POR = f[HMEC_F_POR];
    a.GGGB = f[HMEC_F_GGGB];
    a.SXX0 = f[HMEC_F_SXX0];
    a.SYY0 = f[HMEC_F_SYY0];
    a.RHOX = f[HMEC_F_RHOX];
    a.RHOFX = f[HMEC_F_RHOFX];
    a.PORX = f[HMEC_F_PORX];
    a.ETADX = f[HMEC_F_ETADX];
    a.VX0 = f[HMEC_F_VX0];
    a.VXF0 = f[HMEC_F_VXF0];
    a.RHOY = f[HMEC_F_RHOY];
    a.RHOFY = f[HMEC_F_RHOFY];
    a.PORY = f[HMEC_F_PORY];
    a.ETADY = f[HMEC_F_ETADY];
    a.VY0 = f[HMEC_F_VY0];
    a.VYF0 = f[HMEC_F_VYF0];
    a.PT0 = f[HMEC_F_PT0];
    a.PF0 = f[HMEC_F_PF0];
    a.DILP = f[HMEC_F_DILP];
    const size_t N = (size_t)sv.N, m = (size_t)sv.m;
    HMEC_CUDA(ctx, cudaMalloc(&sv.V, sizeof(double) * (m + 1) * N));
    HMEC_CUDA(ctx, cudaMalloc(&sv.Z, sizeof(double) * m * N));
    HMEC_CUDA(ctx, cudaMalloc(&sv.w, sizeof(double) * N));
    HMEC_CUDA(ctx, cudaMalloc(&sv.H, sizeof(double) * (m + 1) * m));
    HMEC_CUDA(ctx, cudaMalloc(&sv.cs, sizeof(double) * (m + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.sn, sizeof(double) * (m + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.gvec, sizeof(double) * (m + 2)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.yvec, sizeof(double) * (m + 1)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.partial, sizeof(double) * (2 * m + 3) * (size_t)sv.nblk));
    HMEC_CUDA(ctx, cudaMalloc(&sv.dots, sizeof(double) * (2 * m + 4)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.bnorm, sizeof(double) * 2));
    HMEC_CUDA(ctx, cudaMalloc(&sv.done, sizeof(int) * 2));
    HMEC_CUDA(ctx, cudaMalloc(&sv.kcur, sizeof(int) * 2));
    HMEC_CUDA(ctx, cudaMemset(sv.done, 0, sizeof(int) * 2));
    HMEC_CUDA(ctx, cudaMalloc(&sv.gctl, sizeof(GmCtl)));
    HMEC_CUDA(ctx, cudaMemset(sv.gctl, 0, sizeof(GmCtl)));
    const size_t nl = sv.lv.size();
    sv.aux.assign(nl, nullptr);
    sv.ev_coef.assign(nl, nullptr);
    sv.ev_asm.assign(nl, nullptr);
    sv.ev_done.assign(nl, nullptr);
    for (size_t l = 0; l < nl; l++) {
        HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&sv.aux[l], cudaStreamNonBlocking));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&sv.ev_coef[l], cudaEventDisableTiming));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&sv.ev_asm[l], cudaEventDisableTiming));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&sv.ev_done[l], cudaEventDisableTiming));
    }
    HMEC_CUDA(ctx, cudaEventCreateWithFlags(&sv.ev_fork, cudaEventDisableTiming));
    return HMEC_OK;
}

void solver_free(hmec_inst* ctx) {
    Solver& sv = ctx->sv;
    for (Level& L : sv.lv) {
        cudaFree(L.col);
        cudaFree(L.val);
        cudaFree(L.val32);
        cudaFree(L.dscale);
        cudaFree(L.bnd_rows);
        cudaFree(L.pinv);
        cudaFree(L.pinv32);
        cudaFree(L.dx_);
        cudaFree(L.pb);
        cudaFree(L.db);
        cudaFree(L.dr);
        cudaFree(L.fx);
        cudaFree(L.fb);
        cudaFree(L.fr);
        cudaFree(L.dx2);
        cudaFree(L.fx2);
        cudaFree(L.tbnd_start);
        cudaFree(L.tbnd_list);
        cudaFree(L.vals);
        cudaFree(L.offs);
        cudaFree(L.std_off);
        cudaFree(L.std_t);
        cudaFree(L.own_t);
        cudaFree(L.meta_t);
        cudaFree(L.bpack);
        cudaFree(L.pmx);
        cudaFree(L.pmy);
        cudaFree(L.ridx);
        cudaFree(L.rwg);
        cudaFree(L.rw);
        cudaFree(L.rw32);
        for (double* p : L.owned) cudaFree(p);
    }
    sv.lv.clear();
    for (cudaStream_t s : sv.aux)
        if (s) cudaStreamDestroy(s);
    for (auto* evs : {&sv.ev_coef, &sv.ev_asm, &sv.ev_done})
        for (cudaEvent_t e : *evs)
            if (e) cudaEventDestroy(e);
    if (sv.ev_fork) cudaEventDestroy(sv.ev_fork);
    sv.aux.clear();
    sv.ev_coef.clear();
    sv.ev_asm.clear();
    sv.ev_done.clear();
    sv.ev_fork = nullptr;
    if (ctx->p.form == HMEC_FORM_MIXED)
        delete static_cast<VTable<float>*>(sv.vpass);
    else
        delete static_cast<VTable<double>*>(sv.vpass);
    sv.vpass = nullptr;
    sv.vpass_state = 0;
    cudaFree(sv.V);
    cudaFree(sv.Z);
    cudaFree(sv.w);
    cudaFree(sv.H);
    cudaFree(sv.cs);
    cudaFree(sv.sn);
    cudaFree(sv.gvec);
    cudaFree(sv.yvec);
    cudaFree(sv.partial);
    cudaFree(sv.dots);
    cudaFree(sv.bnorm);
    cudaFree(sv.done);
    cudaFree(sv.kcur);
    cudaFree(sv.gctl);
}

// Rebuilds every level after a fine assembly.  The work is a graph, not a
// chain: the coarse coefficients form a chain on the main stream (level l
// needs level l-1's), each level's assembly, inverses, smoother copy and
// boundary pack run on its own stream once its coefficients exist, and the
// restriction scaling of level l also waits for level l-1's row scale.  The
// small coarse levels' kernels thus overlap instead of queueing.
int solver_setup(hmec_inst* ctx) {
    Solver& sv = ctx->sv;
    const bool mixed = ctx->p.form == HMEC_FORM_MIXED;
    int* status = &ctx->ds->status;
    const cudaStream_t main = ctx->stream;
    HMEC_CUDA(ctx, cudaEventRecord(sv.ev_fork, main));
    for (size_t l = 1; l < sv.lv.size(); l++) {
        Level& L = sv.lv[l];
        Level& F = sv.lv[l - 1];
        CoefIn ci{F.af.ETA, F.af.GGG, F.af.RHO, F.af.ETAP, F.af.GGGP, F.af.ETAB, F.af.POR, F.af.GGGB,
                  F.af.RHOX, F.af.RHOFX, F.af.PORX, F.af.ETADX, F.af.RHOY, F.af.RHOFY, F.af.PORY, F.af.ETADY};
        AsmFields& a = L.af;
        CoefOut co{(double*)a.ETA, (double*)a.GGG, (double*)a.RHO, (double*)a.ETAP, (double*)a.GGGP,
                   (double*)a.ETAB, (double*)a.POR, (double*)a.GGGB, (double*)a.RHOX, (double*)a.RHOFX,
                   (double*)a.PORX, (double*)a.ETADX, (double*)a.RHOY, (double*)a.RHOFY, (double*)a.PORY,
                   (double*)a.ETADY};
        const dim3 cg4(nblocks(L.g.Ny1, ctx->bs_st), L.g.Nx1, 4);  // z: basic, P, Vx, Vy sections
        HMEC_LAUNCH(ctx, k_coarsen_coef, cg4, ctx->bs_st, 0, F.g, L.g, ci, co, ctx->p.mg_flags);
        HMEC_CUDA(ctx, cudaEventRecord(sv.ev_coef[l], main));
    }
    for (size_t l = 0; l < sv.lv.size(); l++) {
        Level& L = sv.lv[l];
        StreamScope scope(ctx, sv.aux[l]);
        HMEC_CUDA(ctx, cudaStreamWaitEvent(sv.aux[l], l == 0 ? sv.ev_fork : sv.ev_coef[l], 0));
        if (l > 0) launch_assemble(ctx, L.g, L.af, L.col, L.val, L.dscale, nullptr, nullptr, nullptr);
        HMEC_CUDA(ctx, cudaEventRecord(sv.ev_asm[l], sv.aux[l]));
        if (mixed)
            HMEC_LAUNCH(ctx, k_vanka_setup<float>, nblocks((long long)L.npatch * 16, VS_BS), VS_BS, 0, L.g, L.col,
                        L.val, L.pinv32, status);
        else
            HMEC_LAUNCH(ctx, k_vanka_setup<double>, nblocks((long long)L.npatch * 16, VS_BS), VS_BS, 0, L.g, L.col,
                        L.val, L.pinv, status);
        const size_t n = (size_t)HMEC_W * L.g.N;
        const size_t nb = (size_t)L.ntiles * L.tb_cap;
        // the window offsets follow the pattern, which never changes: formed
        // on the first assembly (a setup captured into a graph forms them on
        // every replay)
        int16_t* offs = L.offs_ready ? nullptr : L.offs;
        if (mixed) {
            HMEC_LAUNCH(ctx, k_stage_prep<float>, nblocks(n, 256), 256, 0, L.g.N, L.g.Ny1, L.g.Nx1, L.CS, L.col,
                        L.val, (float*)L.vals, offs, L.val32, status);
            HMEC_LAUNCH(ctx, k_stage_bpack<float>, nblocks(nb, 128), 128, 0, L.g, L.ntile_i, L.ntiles, L.tb_cap,
                        L.tbnd_start, L.tbnd_list, L.col, L.val, L.bpack, status);
        } else {
            HMEC_LAUNCH(ctx, k_stage_prep<double>, nblocks(n, 256), 256, 0, L.g.N, L.g.Ny1, L.g.Nx1, L.CS, L.col,
                        L.val, (double*)L.vals, offs, nullptr, status);
            HMEC_LAUNCH(ctx, k_stage_bpack<double>, nblocks(nb, 128), 128, 0, L.g, L.ntile_i, L.ntiles, L.tb_cap,
                        L.tbnd_start, L.tbnd_list, L.col, L.val, L.bpack, status);
        }
        if (offs) {
            HMEC_LAUNCH(ctx, k_std_pattern, 1, 6 * HMEC_W, 0, L.g, L.CS, L.offs, L.std_off);
            HMEC_LAUNCH(ctx, k_tile_std, L.ntiles, 256, 0, L.g, L.ntile_i, L.CS, L.offs, L.std_off, L.std_t);
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            HMEC_CUDA(ctx, cudaStreamIsCapturing(sv.aux[l], &cs));
            if (cs == cudaStreamCaptureStatusNone) L.offs_ready = true;
        }
        if (l > 0) {
            HMEC_CUDA(ctx, cudaStreamWaitEvent(sv.aux[l], sv.ev_asm[l - 1], 0));
            HMEC_LAUNCH(ctx, k_restrict_scale, nblocks(L.g.N, 256), 256, 0, L.g.N, L.ridx, L.rwg,
                        sv.lv[l - 1].dscale, L.dscale, L.rw, L.rw32);
        }
        HMEC_CUDA(ctx, cudaEventRecord(sv.ev_done[l], sv.aux[l]));
    }
    for (size_t l = 0; l < sv.lv.size(); l++) HMEC_CUDA(ctx, cudaStreamWaitEvent(main, sv.ev_done[l], 0));
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}

template <typename T>
struct LvPtr;
template <>
struct LvPtr<double> {
    static double* x(Level& L) { return L.dx_; }
    static double* b(Level& L) { return L.db; }
    static double* r(Level& L) { return L.dr; }
    static const double* val(Level& L) { return L.val; }
    static const double* pinv(Level& L) { return L.pinv; }
    static const double* rw(Level& L) { return L.rw; }
};
template <>
struct LvPtr<float> {
    static float* x(Level& L) { return L.fx; }
    static float* b(Level& L) { return L.fb; }
    static float* r(Level& L) { return L.fr; }
    static const float* val(Level& L) { return L.val32; }
    static const float* pinv(Level& L) { return L.pinv32; }
    static const float* rw(Level& L) { return L.rw32; }
};

// Levels with at most this many patches are smoothed by one block (a block
// barrier is cheaper than a grid barrier, but one block leaves the GPU idle:
// measured slower than a small cooperative grid for every level size here).
constexpr int SINGLE_BLOCK_PATCHES = 0;
// Levels whose x, b and boundary deltas fit in this much shared memory are
// smoothed by k_smooth_smem (one block, everything but the matrix on chip).
constexpr size_t SMEM_LIMIT = 200 * 1024;

template <typename T>
static int max_coop_blocks(hmec_inst* ctx) {
    static int cached[2] = {0, 0};
    int& c = cached[sizeof(T) == 8 ? 0 : 1];
    if (c == 0) {
        int per_sm = 0, nsm = 0;
        HMEC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth<T, true>, SM_BS, 0));
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
        c = std::max(1, per_sm * nsm);
    }
    return c;
}

// Launch configuration of the staged pass on one level: whole-tile inverses
// when they fit in shared memory (FP32), else per-colour inverses (FP64); the
// grid is the co-resident block count or the tile count, whichever is smaller.
template <typename T>
static int stage_config(hmec_inst* ctx, Level& L) {
    if (L.st_whole >= 0) return HMEC_OK;
    int nsm = 0, optin = 0;
    HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
    HMEC_CUDA(ctx, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
    int blocks[2], smem[2];
    for (int w = 0; w < 2; w++) {
        const void* kern = w ? (const void*)k_smooth_stage<T, true> : (const void*)k_smooth_stage<T, false>;
        HMEC_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
        smem[w] = stage_layout<T>(w, L.tb_cap).total;
        int per_sm = 0;
        if (smem[w] <= optin)
            HMEC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TILE_BS, (size_t)smem[w]));
        blocks[w] = per_sm * nsm;
    }
    if (blocks[0] < 1 && blocks[1] < 1) {
        ctx->err = "the staged smoothing pass does not fit in shared memory";
        return HMEC_ERR_ARG;
    }
    // whole-tile inverses whenever they fit: a block that waits for each
    // colour's inverses is slower even with twice the blocks resident (FP32,
    // 1001x401: 31.0 against 18.9 ms per step; 201x201: 21.4 against 12.4)
    int w = blocks[1] > 0 ? 1 : 0;
    if (ctx->p.smooth_inverses == 2 && blocks[0] > 0) w = 0;
    L.st_whole = w;
    L.st_grid = std::min(L.ntiles, blocks[w]);
    if (ctx->p.smooth_blocks > 0) {
        L.st_grid = std::min(L.st_grid, ctx->p.smooth_blocks);
    } else if (ctx->p.mg_flags & HMEC_MG_PASS_LAUNCHES) {
        // models that share the GPU (ensembles) take at most a quarter of it
        // per pass unless told otherwise, so that four members' passes run
        // side by side instead of each large level holding every SM in turn
        // (64 uneven members: 125 member-steps/s at a quarter, 118 at half,
        // 106 at an eighth, 102 at all)
        L.st_grid = std::min(L.st_grid, std::max(1, nsm / 4));
    }
    L.st_smem = smem[w];
    return HMEC_OK;
}

template <typename T>
static T* x_alt(Level& L);
template <>
double* x_alt<double>(Level& L) {
    return L.dx2;
}
template <>
float* x_alt<float>(Level& L) {
    return L.fx2;
}

// The staged pass's arguments for level l (its stage_config done); *ab gets
// the pass's algorithmic bytes: per sweep the level's matrix (values and
// int16 window offsets), every inverse, the unknowns read and written and the
// rhs; the prolonged correction; the fused residual (one pass over the
// matrix, x and b) and restriction.
// Compulsory bytes of smoothing sweeps on a level of N unknowns (N/6 cells):
// per cell and sweep the 42 coefficients of its six rows and three vectors
// (unknowns read and written, right-hand side) of six values, in the
// smoother's precision; the residual and restriction that end a
// pre-smoothing pass count as one more sweep.
template <typename T>
static double sweep_bytes_compulsory(double N, double sweeps) {
    return sweeps * (N / 6.0) * (42.0 + 18.0) * sizeof(T);
}

template <typename T>
static StageArgs<T> stage_args(hmec_inst* ctx, size_t l, const T* b, T* x, int nsweeps, int mode, bool restrict_next,
                               double* ab, double* ab_alg) {
    Solver& sv = ctx->sv;
    Level& L = sv.lv[l];
    StageArgs<T> t;
    t.tm_val = L.tm_val;
    t.tm_pinv = L.tm_pinv;
    t.g = L.g;
    t.offs = L.offs;
    t.std_off = L.std_off;
    t.std_t = L.std_t;
    t.cs = L.CS;
    t.col = L.col;
    t.val = LvPtr<T>::val(L);
    t.pinv = LvPtr<T>::pinv(L);
    t.b = b;
    t.x = x;
    t.xalt = x_alt<T>(L);
    t.tb_start = L.tbnd_start;
    t.own_t = L.own_t;
    t.meta_t = L.meta_t;
    t.bpack = L.bpack;
    t.ntile_i = L.ntile_i;
    t.ntiles = L.ntiles;
    t.gc = (mode == 1) ? sv.lv[l + 1].g : L.g;
    t.xc = (mode == 1) ? LvPtr<T>::x(sv.lv[l + 1]) : nullptr;
    t.pmx = L.pmx;
    t.pmy = L.pmy;
    t.nc = 0;
    t.ridx = nullptr;
    t.rw = nullptr;
    t.bc = nullptr;
    t.tb_cap = L.tb_cap;
    t.local = (ctx->p.mg_flags & HMEC_MG_LOCAL_SWEEPS) ? 1 : 0;
    t.status = &ctx->ds->status;
    t.done = sv.done;
    const double st = sizeof(T), N = L.g.N;
    *ab = nsweeps * (N * HMEC_W * st + (double)L.npatch * 100.0 * st + 3.0 * N * st) +
          (mode ? N * st * 1.5 : 0.0);
    *ab_alg = sweep_bytes_compulsory<T>(N, nsweeps + (restrict_next ? 1 : 0));
    if (restrict_next) {
        Level& C = sv.lv[l + 1];
        t.nc = C.g.N;
        t.ridx = C.ridx;
        t.rw = LvPtr<T>::rw(C);
        t.bc = LvPtr<T>::b(C);
        *ab += N * HMEC_W * (st + 4) + 2.0 * N * st + (double)C.g.N * (HMEC_RW * (st + 4) + st);
    }
    return t;
}

// One smoothing pass on level l (x = 0 or x += P xc first, then nsweeps
// sweeps).  restrict_next (tiled pass): also restrict the residual into the
// next coarser level's rhs in the same launch.
template <typename T>
static int smooth(hmec_inst* ctx, size_t l, const T* b, T* x, int nsweeps, int mode, bool restrict_next = false) {
    Solver& sv = ctx->sv;
    Level& L = sv.lv[l];
    SmoothArgs<T> a;
    a.g = L.g;
    a.col = L.col;
    a.val = LvPtr<T>::val(L);
    a.pinv = LvPtr<T>::pinv(L);
    a.b = b;
    a.x = x;
    a.tmp = LvPtr<T>::r(L);
    a.bnd = L.bnd_rows;
    a.nbnd = L.nbnd;
    a.gc = (mode == 1) ? sv.lv[l + 1].g : L.g;
    a.xc = (mode == 1) ? LvPtr<T>::x(sv.lv[l + 1]) : nullptr;
    a.pmx = L.pmx;
    a.pmy = L.pmy;
    // algorithmic bytes: per sweep every patch's 10 ELL rows, inverse, rhs and
    // unknowns, and the boundary rows; plus the zero fill or the prolongation
    const double st = sizeof(T);
    const double bpp = 10.0 * HMEC_W * (st + 4) + 100.0 * st + 30.0 * st;
    const double bnd = (double)L.nbnd * (HMEC_W * (st + 4) + 4.0 * st);
    const double bytes = nsweeps * ((double)L.npatch * bpp + bnd) + (double)L.g.N * st * (mode ? 2.5 : 1.0);
    const double alg = sweep_bytes_compulsory<T>(L.g.N, nsweeps);
    if (L.npatch <= SINGLE_BLOCK_PATCHES) {
        HMEC_LAUNCH_B(ctx, bytes, alg, (k_smooth<T, false>), 1, SM_BS, 0, a, nsweeps, mode);
        return HMEC_OK;
    }
    if (!(ctx->p.mg_flags & HMEC_MG_UNTILED)) {
        int rc = stage_config<T>(ctx, L);
        if (rc) return rc;
        double ab = 0, ab_alg = 0;
        StageArgs<T> t = stage_args<T>(ctx, l, b, x, nsweeps, mode, restrict_next, &ab, &ab_alg);
        void* args[] = {&t, &nsweeps, &mode};
        // live timing by name prefix: "k_smooth" is every level, "k_smooth<l>" one
        static const char* const lname[8] = {"k_smooth0", "k_smooth1", "k_smooth2", "k_smooth3",
                                             "k_smooth4", "k_smooth5", "k_smooth6", "k_smooth7"};
        const bool prof = hmec_prof_begin(ctx, lname[l < 8 ? l : 7], ab, ab_alg);
        const void* kern = L.st_whole ? (const void*)k_smooth_stage<T, true> : (const void*)k_smooth_stage<T, false>;
        HMEC_CUDA(ctx, cudaLaunchCooperativeKernel(kern, dim3(L.st_grid), dim3(TILE_BS), args,
                                                   (size_t)L.st_smem, ctx->stream));
        ctx->launches++;
        if (prof) hmec_prof_end(ctx);
        return HMEC_OK;
    }
    const size_t smem = (2 * (size_t)L.g.N + (size_t)L.nbnd) * sizeof(T);
    if (smem <= SMEM_LIMIT) {
        static bool attr_set[2] = {false, false};
        if (!attr_set[sizeof(T) == 8 ? 0 : 1]) {
            HMEC_CUDA(ctx, cudaFuncSetAttribute(k_smooth_smem<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)SMEM_LIMIT));
            attr_set[sizeof(T) == 8 ? 0 : 1] = true;
        }
        HMEC_LAUNCH_B(ctx, bytes, alg, k_smooth_smem<T>, 1, SMEM_BS, smem, a, nsweeps, mode);
        return HMEC_OK;
    }
    // size the grid to one colour phase (the zero/prolongation and boundary
    // phases are grid-stride loops); fewer blocks make the grid barrier cheaper
    const long long work = std::max<long long>((long long)L.npatch * 16 / 9 + SM_BS, 2LL * SM_BS);
    const int grid = (int)std::min<long long>(max_coop_blocks<T>(ctx), std::max<long long>(1, (work + SM_BS - 1) / SM_BS));
    void* args[] = {&a, &nsweeps, &mode};
    const bool prof = hmec_prof_begin(ctx, "k_smooth", bytes, alg);
    HMEC_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_smooth<T, true>, dim3(grid), dim3(SM_BS), args, 0, ctx->stream));
    ctx->launches++;
    if (prof) hmec_prof_end(ctx);
    return HMEC_OK;
}

// A whole V-cycle for A x = b on the fine level as one k_vcycle_stage
// launch.  *used is false when it does not apply -- untiled smoothing, one
// level, levels in different inverse modes, or a grid that cannot be
// co-resident -- and the caller launches level by level.  The pass table is
// built once; only the fine level's b and x (the FP64 form's Krylov vectors)
// are set per call, in the parameter copy the launch takes.
template <typename T>
static int vcycle_fused(hmec_inst* ctx, const T* b0, T* x0, bool* used) {
    Solver& sv = ctx->sv;
    const hmec_params& p = ctx->p;
    *used = false;
    const size_t nl = sv.lv.size();
    if (sv.vpass_state < 0) return HMEC_OK;
    if (sv.vpass_state == 0) {
        sv.vpass_state = -1;
        if (nl < 2 || (p.mg_flags & (HMEC_MG_UNTILED | HMEC_MG_PASS_LAUNCHES))) return HMEC_OK;
        int whole = -1, grid = 0, cap = 0;
        for (size_t l = 0; l < nl; l++) {
            int rc = stage_config<T>(ctx, sv.lv[l]);
            if (rc) return rc;
            if (whole >= 0 && sv.lv[l].st_whole != whole) return HMEC_OK;
            whole = sv.lv[l].st_whole;
            grid = std::max(grid, sv.lv[l].st_grid);
            cap = std::max(cap, sv.lv[l].tb_cap);
        }
        const int smem = stage_layout<T>(whole, cap).total;
        const void* kern = whole ? (const void*)k_vcycle_stage<T, true> : (const void*)k_vcycle_stage<T, false>;
        int optin = 0, nsm = 0, per_sm = 0;
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
        if (smem > optin) return HMEC_OK;
        // the device maximum, not this model's size: the attribute belongs to
        // the kernel, and concurrent models (ensembles) launch it with
        // different layouts
        HMEC_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
        HMEC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TILE_BS, (size_t)smem));
        if (grid < 1 || grid > per_sm * nsm) return HMEC_OK;
        // pre-smoothing down the levels, the coarsest level, post-smoothing up
        std::vector<VPass<T>> ps;
        double bytes = 0, ab = 0, alg = 0, ab_alg = 0;
        for (size_t l = 0; l + 1 < nl; l++) {
            Level& L = sv.lv[l];
            ps.push_back(
                {stage_args<T>(ctx, l, LvPtr<T>::b(L), LvPtr<T>::x(L), p.mg_pre, 0, true, &ab, &ab_alg), p.mg_pre, 0});
            bytes += ab;
            alg += ab_alg;
        }
        {
            Level& L = sv.lv[nl - 1];
            const int ns = std::max(1, p.mg_coarse_sweeps);
            ps.push_back({stage_args<T>(ctx, nl - 1, LvPtr<T>::b(L), LvPtr<T>::x(L), ns, 0, false, &ab, &ab_alg), ns, 0});
            bytes += ab;
            alg += ab_alg;
        }
        for (size_t l = nl - 1; l-- > 0;) {
            Level& L = sv.lv[l];
            ps.push_back(
                {stage_args<T>(ctx, l, LvPtr<T>::b(L), LvPtr<T>::x(L), p.mg_post, 1, false, &ab, &ab_alg), p.mg_post, 1});
            bytes += ab;
            alg += ab_alg;
        }
        if ((int)ps.size() > MAX_VPASS) return HMEC_OK;
        VTable<T>* tab = new (std::nothrow) VTable<T>();
        if (!tab) return HMEC_OK;
        for (size_t k = 0; k < ps.size(); k++) tab->p[k] = ps[k];
        tab->npass = (int)ps.size();
        tab->cap = cap;
        tab->done = sv.done;
        sv.vpass = tab;
        sv.vpass_n = (int)ps.size();
        sv.vpass_grid = grid;
        sv.vpass_smem = smem;
        sv.vpass_whole = whole;
        sv.vpass_cap = cap;
        sv.vpass_bytes = bytes;
        sv.vpass_bytes_alg = alg;
        sv.vpass_state = 1;
    }
    VTable<T>* tab = static_cast<VTable<T>*>(sv.vpass);
    tab->p[0].a.b = b0;  // the fine level's pre- and post-smoothing passes
    tab->p[0].a.x = x0;
    tab->p[sv.vpass_n - 1].a.b = b0;
    tab->p[sv.vpass_n - 1].a.x = x0;
    void* args[] = {tab};
    const void* kern =
        sv.vpass_whole ? (const void*)k_vcycle_stage<T, true> : (const void*)k_vcycle_stage<T, false>;
    const bool prof = hmec_prof_begin(ctx, "k_smooth_vcycle", sv.vpass_bytes, sv.vpass_bytes_alg);
    HMEC_CUDA(ctx, cudaLaunchCooperativeKernel(kern, dim3(sv.vpass_grid), dim3(TILE_BS), args, (size_t)sv.vpass_smem,
                                               ctx->stream));
    ctx->launches++;
    if (prof) hmec_prof_end(ctx);
    *used = true;
    return HMEC_OK;
}

// V-cycle on level l for A x = b, x = 0 on entry (b, x default to the level's buffers).
template <typename T>
static int vcycle(hmec_inst* ctx, size_t l, const T* b_in = nullptr, T* x_in = nullptr) {
    // one launch per V-cycle for the FP32 smoother; the FP64 form (streamed
    // inverses) measured faster with a launch per pass (33.3 vs 32.7 ms per
    // 201x201 step), so it keeps those
    if (l == 0 && std::is_same<T, float>::value) {
        Level& F = ctx->sv.lv[0];
        bool used = false;
        const int rc = vcycle_fused<T>(ctx, b_in ? b_in : LvPtr<T>::b(F), x_in ? x_in : LvPtr<T>::x(F), &used);
        if (rc || used) return rc;
    }
    Solver& sv = ctx->sv;
    Level& L = sv.lv[l];
    const hmec_params& p = ctx->p;
    const T* b = b_in ? b_in : LvPtr<T>::b(L);
    T* x = x_in ? x_in : LvPtr<T>::x(L);
    if (!b || !x) {
        ctx->err = "vcycle: a level vector is missing";
        return HMEC_ERR_STATE;
    }
    int rc;
    if (l + 1 == sv.lv.size()) {
        const int ns = (sv.lv.size() == 1) ? std::max(1, p.mg_pre + p.mg_post) : std::max(1, p.mg_coarse_sweeps);
        return smooth<T>(ctx, l, b, x, ns, 0);
    }
    Level& C = sv.lv[l + 1];
    if (!(p.mg_flags & HMEC_MG_UNTILED)) {
        // the pre-smoothing pass also forms the residual and restricts it
        if ((rc = smooth<T>(ctx, l, b, x, p.mg_pre, 0, true))) return rc;
    } else {
        if ((rc = smooth<T>(ctx, l, b, x, p.mg_pre, 0))) return rc;
        HMEC_LAUNCH(ctx, k_resid<T>, nblocks(L.g.N, 256), 256, 0, L.g.N, L.col, LvPtr<T>::val(L), b, x,
                    LvPtr<T>::r(L));
        HMEC_LAUNCH(ctx, k_restrict<T>, nblocks(C.g.N, 256), 256, 0, C.g.N, C.ridx, LvPtr<T>::rw(C),
                    (const T*)LvPtr<T>::r(L), LvPtr<T>::b(C));
    }
    if ((rc = vcycle<T>(ctx, l + 1))) return rc;
    return smooth<T>(ctx, l, b, x, p.mg_post, 1);
}

// z = M^{-1} v on the fine level (v, z FP64 vectors of the scaled system)
// (mixed form: z is left in FP32 in the fine level's x; input_ready: its
// FP32 input is already in the fine level's b)
static int precondition(hmec_inst* ctx, const double* v, double* z, bool input_ready) {
    Solver& sv = ctx->sv;
    Level& L = sv.lv[0];
    const size_t N = (size_t)L.g.N;
    if (ctx->p.form == HMEC_FORM_MIXED) {
        if (!input_ready) HMEC_LAUNCH(ctx, (k_convert<double, float>), nblocks(N, 256), 256, 0, N, v, L.fb);
        return vcycle<float>(ctx, 0);
    }
    return vcycle<double>(ctx, 0, v, z);
}

// One cooperative Arnoldi step (k_arnoldi) after the preconditioner.
// devj: the step index and z_j's slot come from the device (graph mode; j
// is then only the estimate used for the byte accounting).
template <typename TZ>
static int arnoldi(hmec_inst* ctx, const TZ* zsrc, double* Zj, int j, const Gm& G, double rtol, bool devj = false) {
    Solver& sv = ctx->sv;
    Level& L0 = sv.lv[0];
    static int cached = 0;
    if (!cached) {
        int per_sm = 0, nsm = 0;
        HMEC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_arnoldi<TZ>, ARN_BS,
                                                                     sizeof(double) * 129));
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
        cached = std::max(1, per_sm * nsm);
    }
    ArnArgs<TZ> a;
    a.N = sv.N;
    a.j = j;
    a.m = sv.m;
    a.nblk = std::min(sv.nblk, cached);
    a.col = L0.col;
    a.val = L0.val;
    a.zsrc = zsrc;
    a.Zj = Zj;
    a.V = sv.V;
    a.w = sv.w;
    a.partial = sv.partial;
    a.G = G;
    a.rtol = rtol;
    a.next32 = ctx->p.form == HMEC_FORM_MIXED ? L0.fb : nullptr;
    a.next64 = (devj && ctx->p.form != HMEC_FORM_MIXED) ? L0.pb : nullptr;
    a.jdev = devj ? sv.kcur : nullptr;
    a.Zbase = sv.Z;
    void* args[] = {&a};
    // algorithmic bytes: SpMV (FP64 values, int32 columns, z gathered, w and
    // z_j written) and two CGS passes (each a dot and an update over j+1
    // basis vectors), V_{j+1} written
    const double N = sv.N, nb = j + 1;
    const double bytes = N * (HMEC_W * 12.0 + sizeof(TZ) + 16.0) + 2.0 * N * 8.0 * (3.0 * nb + 2.0) + N * 12.0;
    // compulsory: the FP64 operator, 42 coefficients and two vectors per
    // cell (432 B), and the orthogonalisation against j+1 basis vectors,
    // (2j+2) vectors of six FP64 values per cell
    const double alg = (N / 6.0) * (432.0 + (2.0 * nb) * 48.0);
    const bool prof = hmec_prof_begin(ctx, "k_arnoldi", bytes, alg);
    HMEC_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_arnoldi<TZ>, dim3(a.nblk), dim3(ARN_BS), args,
                                               sizeof(double) * (sv.m + 1), ctx->stream));
    ctx->launches++;
    if (prof) hmec_prof_end(ctx);
    return HMEC_OK;
}

int solver_solve(hmec_inst* ctx, int* iters_out, double* relres_out) {
    Solver& sv = ctx->sv;
    Level& L0 = sv.lv[0];
    const int N = sv.N, m = sv.m, nblk = sv.nblk;
    const double rtol = ctx->p.krylov_rtol;
    const int maxit = std::max(1, ctx->p.krylov_maxit);
    const bool mixed = ctx->p.form == HMEC_FORM_MIXED;
    double* x = ctx->S;
    const double* b = L0.db;
    Gm G{sv.H, sv.cs, sv.sn, sv.gvec, sv.yvec, sv.dots, sv.bnorm, sv.done, sv.kcur, ctx->ds};
    HMEC_CUDA(ctx, cudaMemsetAsync(&ctx->ds->krylov_iters, 0, sizeof(int), ctx->stream));
    int total = 0;
    bool first = true;
    bool converged = false;
    const int check_every = 8;
    double* r = sv.w;
    double prev = INFINITY;
    while (true) {
        // true residual at every restart: the only convergence decision
        HMEC_LAUNCH(ctx, k_true_resid, nblk, RED_BS, 0, N, L0.col, L0.val, b, x, r, sv.partial, nblk);
        HMEC_LAUNCH(ctx, k_cycle_begin, 1, 32, 0, G, sv.partial, nblk, first ? 1 : 0, rtol, m);
        HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->hs, ctx->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
        HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        first = false;
        total = ctx->hs->krylov_iters;
        const double rel = ctx->hs->krylov_relres;
        if (rel <= rtol) {
            converged = true;
            break;
        }
        if (!std::isfinite(rel) || total >= maxit) break;
        if (total > 0 && rel > 0.5 * prev && rel <= 1e-10) {
            // a whole restart cycle gained less than a factor 2 near the FP64
            // rounding floor of the residual; accept it when within 100x the
            // tolerance (far above the floor a slow cycle just continues)
            converged = rel <= 100 * rtol;
            break;
        }
        prev = rel;
        HMEC_LAUNCH(ctx, k_scale_vec, nblocks(N, 256), 256, 0, N, r, sv.dots, sv.V, sv.done, nullptr, nullptr);
        // The host looks at the convergence flag only now and then (a look
        // drains the stream); steps queued after convergence return at once
        // but still cost their launches.  So the next look is placed where the
        // residual estimate's observed rate says the tolerance will be met:
        // the first after a few steps, then after the predicted number of
        // steps (1 to check_every).
        int next_check = std::min(4, check_every);
        double rel_last = rel;
        int j_last = 0;
        for (int j = 0; j < m && total + j < maxit; j++) {
            double* Vj = sv.V + (size_t)j * N;
            double* Zj = sv.Z + (size_t)j * N;
            if (j > 0 && j == next_check) {
                HMEC_CUDA(ctx, cudaMemcpyAsync(&ctx->hs->pad0, sv.done, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
                HMEC_CUDA(ctx, cudaMemcpyAsync(&ctx->hs->krylov_relres, &ctx->ds->krylov_relres, sizeof(double),
                                               cudaMemcpyDeviceToHost, ctx->stream));
                HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                if (ctx->hs->pad0) break;
                const double est = ctx->hs->krylov_relres;
                int step = check_every;
                if (std::isfinite(est) && est > 0 && est < rel_last) {
                    const double rate = std::pow(est / rel_last, 1.0 / (j - j_last));
                    const double need = std::ceil(std::log(rtol / est) / std::log(rate));
                    step = (int)std::max(1.0, std::min((double)check_every, need));
                }
                next_check = j + step;
                rel_last = est;
                j_last = j;
            }
            // the previous Arnoldi step already wrote the mixed form's FP32 input
            int prc = precondition(ctx, Vj, Zj, j > 0);
            if (prc) return prc;
            if (mixed)
                prc = arnoldi<float>(ctx, L0.fx, Zj, j, G, rtol);
            else
                prc = arnoldi<double>(ctx, Zj, Zj, j, G, rtol);
            if (prc) return prc;
        }
        HMEC_LAUNCH(ctx, k_lsq, 1, 1, 0, G, m);
        HMEC_LAUNCH(ctx, k_xupdate, nblocks(N, 256), 256, 0, N, sv.Z, sv.yvec, sv.kcur, x);
    }
    if (iters_out) *iters_out = total;
    if (relres_out) *relres_out = ctx->hs->krylov_relres;
    if (!converged) {
        HMEC_CUDA(ctx, cudaMemcpyAsync(&ctx->hs->pad0, &ctx->ds->status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return HMEC_ERR_KRYLOV_NOCONV;
    }
    return HMEC_OK;
}

// The solve of solver_solve for the graph of a timestep: the same kernels
// and the same decisions, taken on the device.  The restart cycle and the
// Arnoldi step are the bodies of two nested conditional WHILE nodes; the
// preconditioner reads fixed buffers (the mixed form's FP32 input fb and
// output fx; the FP64 form's pb and dx_, which the Arnoldi step fills and
// copies into z_j), so nothing in the graph depends on the step index.
int solver_capture_solve(hmec_inst* ctx, cudaStream_t s_restart, cudaStream_t s_inner, int64_t* n_restart,
                         int64_t* n_inner) {
    Solver& sv = ctx->sv;
    Level& L0 = sv.lv[0];
    const int N = sv.N, m = sv.m, nblk = sv.nblk;
    const double rtol = ctx->p.krylov_rtol;
    const int maxit = std::max(1, ctx->p.krylov_maxit);
    const bool mixed = ctx->p.form == HMEC_FORM_MIXED;
    Gm G{sv.H, sv.cs, sv.sn, sv.gvec, sv.yvec, sv.dots, sv.bnorm, sv.done, sv.kcur, ctx->ds};
    // the fixed buffers the captured preconditioner reads and writes
    if (mixed ? (!L0.fb || !L0.fx) : (!L0.pb || !L0.dx_)) {
        ctx->err = "solver_capture_solve: a preconditioner buffer is missing";
        return HMEC_ERR_STATE;
    }
    cudaGraphConditionalHandle hr = 0, hi = 0;
    int rc = graph_handle(ctx, ctx->stream, &hr);
    if (rc) return rc;
    HMEC_LAUNCH(ctx, k_solve_init, 1, 1, 0, G, sv.gctl, maxit, hr);
    if ((rc = graph_while_begin(ctx, ctx->stream, hr, s_restart))) return rc;
    const int64_t l0 = ctx->launches;
    {
        StreamScope scope(ctx, s_restart);
        HMEC_LAUNCH(ctx, k_true_resid, nblk, RED_BS, 0, N, L0.col, L0.val, L0.db, ctx->S, sv.w, sv.partial, nblk);
        if ((rc = graph_handle(ctx, s_restart, &hi))) return rc;
        HMEC_LAUNCH(ctx, k_cycle_begin_g, 1, 32, 0, G, sv.partial, nblk, rtol, m, sv.gctl, hr, hi);
        HMEC_LAUNCH(ctx, k_scale_vec, nblocks(N, 256), 256, 0, N, sv.w, sv.dots, sv.V, sv.done, mixed ? L0.fb : nullptr,
                    mixed ? nullptr : L0.pb);
        if ((rc = graph_while_begin(ctx, s_restart, hi, s_inner))) return rc;
        const int64_t l1 = ctx->launches;
        {
            StreamScope scope2(ctx, s_inner);
            if (mixed) {
                if ((rc = vcycle<float>(ctx, 0))) return rc;
                if ((rc = arnoldi<float>(ctx, L0.fx, nullptr, m / 2, G, rtol, true))) return rc;
            } else {
                if ((rc = vcycle<double>(ctx, 0, L0.pb, L0.dx_))) return rc;
                if ((rc = arnoldi<double>(ctx, L0.dx_, nullptr, m / 2, G, rtol, true))) return rc;
            }
            HMEC_LAUNCH(ctx, k_inner_cond, 1, 1, 0, G, m, sv.gctl, hi);
        }
        *n_inner = ctx->launches - l1;
        if ((rc = graph_while_end(ctx, s_inner))) return rc;
        HMEC_LAUNCH(ctx, k_lsq, 1, 1, 0, G, m);
        HMEC_LAUNCH(ctx, k_xupdate, nblocks(N, 256), 256, 0, N, sv.Z, sv.yvec, sv.kcur, ctx->S);
    }
    *n_restart = ctx->launches - l0 - *n_inner;
    if ((rc = graph_while_end(ctx, s_restart))) return rc;
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}
