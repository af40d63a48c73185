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
// Gauss-Jordan with partial pivoting on the 10x10 patch block of D A;
// inverses stored patch-major, pinv[p*100 + r*10 + c].
__global__ void k_vanka_setup(Geo g, const int32_t* __restrict__ col, const double* __restrict__ val,
                              double* pinv, float* pinv32, int* status) {
    const int pi = blockIdx.x * blockDim.x + threadIdx.x;
    const int np = (g.Ny - 1) * (g.Nx - 1);
    if (pi >= np) return;
    const int i = 1 + pi % (g.Ny - 1), j = 1 + pi / (g.Ny - 1);
    int u[PB];
    for (int q = 0; q < PB; q++) u[q] = patch_unknown(i, j, g.Ny1, q);
    double a[PB][PB], b[PB][PB];
    for (int r = 0; r < PB; r++)
        for (int c = 0; c < PB; c++) {
            a[r][c] = 0;
            b[r][c] = (r == c) ? 1.0 : 0.0;
        }
    for (int r = 0; r < PB; r++) {
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * g.N + u[r];
            const int cc = col[o];
            const double v = val[o];
            for (int c = 0; c < PB; c++)
                if (u[c] == cc) a[r][c] += v;
        }
    }
    bool singular = false;
    for (int c = 0; c < PB; c++) {
        int pr = c;
        double best = fabs(a[c][c]);
        for (int r = c + 1; r < PB; r++)
            if (fabs(a[r][c]) > best) {
                best = fabs(a[r][c]);
                pr = r;
            }
        if (!(best > 0)) {
            singular = true;
            break;
        }
        if (pr != c)
            for (int k = 0; k < PB; k++) {
                double t = a[c][k];
                a[c][k] = a[pr][k];
                a[pr][k] = t;
                t = b[c][k];
                b[c][k] = b[pr][k];
                b[pr][k] = t;
            }
        const double inv = 1.0 / a[c][c];
        for (int k = 0; k < PB; k++) {
            a[c][k] *= inv;
            b[c][k] *= inv;
        }
        for (int r = 0; r < PB; r++) {
            if (r == c) continue;
            const double f = a[r][c];
            if (f != 0)
                for (int k = 0; k < PB; k++) {
                    a[r][k] -= f * a[c][k];
                    b[r][k] -= f * b[c][k];
                }
        }
    }
    if (singular) {
        atomicOr(status, HMEC_DEV_NAN);
        for (int r = 0; r < PB; r++)
            for (int c = 0; c < PB; c++) b[r][c] = 0;
    }
    for (int r = 0; r < PB; r++)
        for (int c = 0; c < PB; c++) {
            const size_t o = (size_t)pi * 100 + r * PB + c;
            if (pinv) pinv[o] = b[r][c];
            if (pinv32) pinv32[o] = (float)b[r][c];
        }
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
};

__device__ __forceinline__ int m_cell(const Map1D& m, int k) {
    if (k <= 0) return 0;
    if (k >= m.nf + 1) return m.nc + 1;
    return (int)(((long long)(2 * k - 1) * m.nc) / (2LL * m.nf)) + 1;
}

// hat weight of coarse node K at fine node j
__device__ __forceinline__ double m_hat(const Map1D& m, int j, int K) {
    long long d = (long long)j * m.nc - (long long)K * m.nf;
    if (d < 0) d = -d;
    return d >= m.nf ? 0.0 : 1.0 - (double)d / (double)m.nf;
}

// fine nodes that can have a nonzero hat weight for coarse node K
__device__ __forceinline__ void m_hat_range(const Map1D& m, int K, int& j0, int& j1) {
    j0 = max(0, (int)(((long long)(K - 1) * m.nf) / m.nc));
    j1 = min(m.nf + 1, (int)(((long long)(K + 1) * m.nf + m.nc - 1) / m.nc));
}

// fine cells that can map to coarse cell K (filter with m_cell(k) == K)
__device__ __forceinline__ void m_cell_range(const Map1D& m, int K, int& k0, int& k1) {
    if (K <= 0) {
        k0 = k1 = 0;
    } else if (K >= m.nc + 1) {
        k0 = k1 = m.nf + 1;
    } else {
        k0 = max(1, (int)(((long long)(K - 1) * m.nf) / m.nc));
        k1 = min(m.nf, (int)(((long long)K * m.nf) / m.nc) + 1);
    }
}

__device__ __forceinline__ Map1D mapx(const Geo& gf, const Geo& gc) { return Map1D{gf.Nx - 1, gc.Nx - 1}; }
__device__ __forceinline__ Map1D mapy(const Geo& gf, const Geo& gc) { return Map1D{gf.Ny - 1, gc.Ny - 1}; }

// x_f += P x_c: cell-centred unknowns piecewise constant, face unknowns linear
// along the face normal and constant across it (ghost rows map to ghost rows,
// which keeps the homogeneous boundary relations of the coarse correction).
template <typename T>
__device__ __forceinline__ void prolong_add(const Geo& gf, const Geo& gc, const T* __restrict__ xc, T* xf, int tid,
                                            int nth) {
    const Map1D mx = mapx(gf, gc), my = mapy(gf, gc);
    const int ncell = gf.Ny1 * gf.Nx1;
    for (int t = tid; t < ncell; t += nth) {
        const int i = t % gf.Ny1, j = t / gf.Ny1;
        const int kf = kp_of(i, j, gf.Ny1);
        auto xcv = [&](int I, int J, int v) -> T {
            if (I < 0 || I > gc.Ny || J < 0 || J > gc.Nx) return (T)0;
            return xc[kp_of(I, J, gc.Ny1) + v];
        };
        const int Ic = m_cell(my, i), Jc = m_cell(mx, j);
        if (i >= 1 && i <= gf.Ny - 1 && j >= 1 && j <= gf.Nx - 1) {
            xf[kf + 0] += xcv(Ic, Jc, 0);
            xf[kf + 3] += xcv(Ic, Jc, 3);
        }
        {  // x faces: linear in x between coarse nodes J0, J0+1
            const int J0 = (int)(((long long)j * mx.nc) / mx.nf);
            const T w1 = (T)m_hat(mx, j, J0 + 1), w0 = (T)m_hat(mx, j, J0);
            xf[kf + 1] += w0 * xcv(Ic, J0, 1) + w1 * xcv(Ic, J0 + 1, 1);
            xf[kf + 4] += w0 * xcv(Ic, J0, 4) + w1 * xcv(Ic, J0 + 1, 4);
        }
        {  // y faces: linear in y between coarse nodes I0, I0+1
            const int I0 = (int)(((long long)i * my.nc) / my.nf);
            const T w1 = (T)m_hat(my, i, I0 + 1), w0 = (T)m_hat(my, i, I0);
            xf[kf + 2] += w0 * xcv(I0, Jc, 2) + w1 * xcv(I0 + 1, Jc, 2);
            xf[kf + 5] += w0 * xcv(I0, Jc, 5) + w1 * xcv(I0 + 1, Jc, 5);
        }
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
        prolong_add(a.g, a.gc, a.xc, a.x, tid, nth);
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
        prolong_add(a.g, a.gc, a.xc, xs, tid, nth);
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

template <typename T>
struct TileArgs {
    SmoothArgs<T> a;
    T* xalt;
    const int32_t *owner, *own_start, *own_list, *tb_start, *tb_list;
    int ntile_i, ntiles;
    T* r_out;  // if set, r = b - A x is written after the last sweep
};

// The tile's window of unknowns is staged in shared memory.  Window = the
// cells the tile's patch rows and boundary rows can read (the tile's patches
// extended by two cells up/left and one down/right), at most (TILE+3)^2
// cells.  Per sweep: load the window from P, run the 9 colour classes and the
// boundary rows (one Jacobi pass) on shared memory (unknowns the tile does not
// own stay at their P values), write the owned unknowns to Q.  A matrix
// column maps to its window slot from its offset to the row: delta = col -
// row = dj*6*Ny1 + (di*6 + dv) with |di*6 + dv| < 12, so dj follows from two
// comparisons and the window offset is dj*6*WI + (delta - dj*6*Ny1).
constexpr int WIN_MAX = (TILE + 3) * (TILE + 3) * 6;

template <typename T>
__global__ void __launch_bounds__(TILE_BS) k_smooth_win(TileArgs<T> t, int nsweeps, int mode) {
    __shared__ T xs[WIN_MAX];
    __shared__ unsigned char own[WIN_MAX];
    const SmoothArgs<T>& a = t.a;
    const Geo& g = a.g;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int RS = 6 * g.Ny1;
    T* P = a.x;
    T* Q = t.xalt;
    if (mode == 0) {
        for (int r = tid; r < g.N; r += nth) P[r] = (T)0;
    } else {
        prolong_add(g, a.gc, a.xc, P, tid, nth);
    }
    cg::this_grid().sync();
    const int lane = threadIdx.x & 31, q = lane & 15, slot = threadIdx.x >> 4;
    for (int s = 0; s < nsweeps; s++) {
        for (int tile = blockIdx.x; tile < t.ntiles; tile += gridDim.x) {
            const int ti = tile % t.ntile_i, tj = tile / t.ntile_i;
            const int i0 = 1 + ti * TILE, j0 = 1 + tj * TILE;
            const int i1 = min(i0 + TILE, g.Ny), j1 = min(j0 + TILE, g.Nx);  // exclusive
            const int wi0 = max(i0 - 2, 0), wj0 = max(j0 - 2, 0);
            const int WI = min(i1, g.Ny) - wi0 + 1, WJ = min(j1, g.Nx) - wj0 + 1;
            const int W = WI * WJ * 6, SJ = 6 * WI;
            // stage the window
            for (int lw = threadIdx.x; lw < W; lw += blockDim.x) {
                const int lc = lw / 6, v = lw - 6 * lc;
                const int cj = wj0 + lc / WI, ci = wi0 + lc % WI;
                const int gw = (cj * g.Ny1 + ci) * 6 + v;
                xs[lw] = P[gw];
                own[lw] = (t.owner[gw] == tile) ? 1 : 0;
            }
            __syncthreads();
            for (int c = 0; c < 9; c++) {
                const int ri = c / 3, rj = c % 3;
                const int fi = i0 + ((ri - i0 % 3) + 3) % 3, fj = j0 + ((rj - j0 % 3) + 3) % 3;
                const int ni = fi < i1 ? (i1 - 1 - fi) / 3 + 1 : 0;
                const int nj = fj < j1 ? (j1 - 1 - fj) / 3 + 1 : 0;
                const bool valid = slot < ni * nj;
                int i = i0, j = j0;
                if (valid) {
                    i = fi + 3 * (slot % ni);
                    j = fj + 3 * (slot / ni);
                }
                T pr[PB];
                {
                    const T* Pi = a.pinv + (size_t)((j - 1) * (g.Ny - 1) + (i - 1)) * 100 + (q < PB ? q : 0) * PB;
#pragma unroll
                    for (int cc = 0; cc < PB; cc++) pr[cc] = (valid && q < PB) ? Pi[cc] : (T)0;
                }
                T r = 0;
                int lrow = 0;
                if (valid && q < PB) {
                    const int row = patch_unknown(i, j, g.Ny1, q);
                    // cell of unknown q: (i, j), left (i, j-1) or top (i-1, j)
                    const int ci = (q == 4 || q == 8) ? i - 1 : i;
                    const int cj = (q == 2 || q == 6) ? j - 1 : j;
                    lrow = ((cj - wj0) * WI + (ci - wi0)) * 6 + (row - 6 * (row / 6));
                    T acc = a.b[row];
#pragma unroll
                    for (int sl = 0; sl < HMEC_W; sl++) {
                        const size_t o = (size_t)sl * g.N + row;
                        const int delta = a.col[o] - row;
                        const int dj = delta > RS / 2 ? 1 : (delta < -RS / 2 ? -1 : 0);
                        acc -= a.val[o] * xs[lrow + dj * SJ + (delta - dj * RS)];
                    }
                    r = acc;
                }
                T d = 0;
#pragma unroll
                for (int cc = 0; cc < PB; cc++) {
                    const T rc = __shfl_sync(0xffffffffu, r, (lane & 16) + cc);
                    d += pr[cc] * rc;
                }
                // same-class patches never read each other's unknowns, and the
                // shuffles above order this patch's reads before its writes
                if (valid && q < PB && own[lrow]) xs[lrow] += d;
                __syncthreads();
            }
            // this tile's boundary rows: one Jacobi pass on the window
            const int kb = t.tb_start[tile], ke = t.tb_start[tile + 1];
            for (int k = kb + threadIdx.x; k < ke; k += blockDim.x) {
                const int row = t.tb_list[k];
                const int cell = row / 6;
                const int lr = (((cell / g.Ny1) - wj0) * WI + ((cell % g.Ny1) - wi0)) * 6 + (row - 6 * cell);
                T acc = a.b[row], diag = 0;
#pragma unroll
                for (int sl = 0; sl < HMEC_W; sl++) {
                    const size_t o = (size_t)sl * g.N + row;
                    const int cl = a.col[o];
                    const int delta = cl - row;
                    const int dj = delta > RS / 2 ? 1 : (delta < -RS / 2 ? -1 : 0);
                    const T v = a.val[o];
                    acc -= v * xs[lr + dj * SJ + (delta - dj * RS)];
                    if (cl == row) diag += v;
                }
                a.tmp[k] = diag != 0 ? acc / diag : (T)0;
            }
            __syncthreads();
            for (int k = kb + threadIdx.x; k < ke; k += blockDim.x) {
                const int row = t.tb_list[k];
                const int cell = row / 6;
                const int lr = (((cell / g.Ny1) - wj0) * WI + ((cell % g.Ny1) - wi0)) * 6 + (row - 6 * cell);
                xs[lr] += a.tmp[k];
            }
            __syncthreads();
            // publish the owned unknowns
            for (int lw = threadIdx.x; lw < W; lw += blockDim.x) {
                if (!own[lw]) continue;
                const int lc = lw / 6, v = lw - 6 * lc;
                const int cj = wj0 + lc / WI, ci = wi0 + lc % WI;
                Q[(cj * g.Ny1 + ci) * 6 + v] = xs[lw];
            }
            __syncthreads();
        }
        cg::this_grid().sync();
        T* sw = P;
        P = Q;
        Q = sw;
    }
    if (P != a.x)
        for (int r = tid; r < g.N; r += nth) a.x[r] = P[r];
    if (t.r_out) {  // residual for the restriction, fused to save a launch
        cg::this_grid().sync();
        for (int row = tid; row < g.N; row += nth) {
            T acc = a.b[row];
#pragma unroll
            for (int sl = 0; sl < HMEC_W; sl++) {
                const size_t o = (size_t)sl * g.N + row;
                acc -= a.val[o] * a.x[a.col[o]];
            }
            t.r_out[row] = acc;
        }
    }
}

// ------------------------------------------------ multigrid restriction
// Whether the row of unknown v at staggered cell (i, j) is an interior
// equation (x/y-Stokes, continuity, Darcy) rather than a boundary or ghost
// row; the ranges are those of the assembly branches (:698-980).
__device__ __forceinline__ bool row_interior(const Geo& g, int i, int j, int v) {
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
    if (I >= gc.Ny1) return;
    const Map1D mx = mapx(gf, gc), my = mapy(gf, gc);
    // basic nodes: hat (full) weighting of the fine nodes; G harmonically
    if (I < gc.Ny && J < gc.Nx) {
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
    if (I >= 1 && I <= gc.Ny - 1 && J >= 1 && J <= gc.Nx - 1) {
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
    {
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
    {
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

// Coarse rhs = restricted fine residual, in physical units r/df, scaled by the
// coarse row scale (the transpose of the prolongation, weights normalised).
// Only interior equations are restricted, and only from fine interior
// equations; coarse boundary rows get a zero residual, so the coarse
// correction obeys the homogeneous boundary conditions, which the
// prolongation preserves.
template <typename T>
__global__ void k_restrict_r(Geo gf, Geo gc, const T* __restrict__ rf, const double* __restrict__ dsf,
                             const double* __restrict__ dsc, T* bc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= gc.Ny1 * gc.Nx1 * 6) return;
    const int v = t % 6, cell = t / 6, I = cell % gc.Ny1, J = cell / gc.Ny1;
    double s = 0, w = 0;
    if (row_interior(gc, I, J, v)) {
        const Map1D mx = mapx(gf, gc), my = mapy(gf, gc);
        const bool xnode = v == 1 || v == 4, ynode = v == 2 || v == 5;
        int i0, i1, j0, j1;
        if (ynode) m_hat_range(my, I, i0, i1); else m_cell_range(my, I, i0, i1);
        if (xnode) m_hat_range(mx, J, j0, j1); else m_cell_range(mx, J, j0, j1);
        for (int i = i0; i <= i1; i++) {
            const double wi = ynode ? m_hat(my, i, I) : (m_cell(my, i) == I ? 1.0 : 0.0);
            if (wi == 0.0) continue;
            for (int j = j0; j <= j1; j++) {
                const double wj = xnode ? m_hat(mx, j, J) : (m_cell(mx, j) == J ? 1.0 : 0.0);
                if (wj == 0.0 || !row_interior(gf, i, j, v)) continue;
                const int k = kp_of(i, j, gf.Ny1) + v;
                s += wi * wj * ((double)rf[k] / dsf[k]);
                w += wi * wj;
            }
        }
    }
    bc[t] = (T)(w > 0 ? (s / w) * dsc[t] : 0.0);
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
// partial[k * nblk + blk] = sum over the block's rows of V_k . w   (k = blockIdx.y)
__global__ void k_dots(int N, const double* __restrict__ V, const double* __restrict__ w, double* partial, int nblk,
                       const int* done) {
    if (*done) return;
    __shared__ double sh[RED_BS];
    const int k = blockIdx.y;
    const double* v = V + (size_t)k * N;
    double acc = 0;
    for (int r = blockIdx.x * RED_BS + threadIdx.x; r < N; r += nblk * RED_BS) acc += v[r] * w[r];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = RED_BS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)k * nblk + blockIdx.x] = sh[0];
}

// dots[k] = sum_b partial[k][b], one warp per k, fixed order.
__global__ void k_dots_final(const double* __restrict__ partial, int nblk, int nk, double* dots, const int* done) {
    if (*done) return;
    const int k = blockIdx.x;
    if (k >= nk) return;
    double acc = 0;
    for (int b = threadIdx.x; b < nblk; b += 32) acc += partial[(size_t)k * nblk + b];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) dots[k] = acc;
}

// w -= sum_k h_k V_k; partial sums of |w|^2 into partial[0..nblk)
__global__ void k_orth_update(int N, const double* __restrict__ V, int nk, const double* __restrict__ h, double* w,
                              double* partial, int nblk, const int* done) {
    if (*done) return;
    __shared__ double sh[RED_BS];
    double acc2 = 0;
    for (int r = blockIdx.x * RED_BS + threadIdx.x; r < N; r += nblk * RED_BS) {
        double x = w[r];
        for (int k = 0; k < nk; k++) x -= h[k] * V[(size_t)k * N + r];
        w[r] = x;
        acc2 += x * x;
    }
    sh[threadIdx.x] = acc2;
    __syncthreads();
    for (int s = RED_BS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// w = A z (scaled rows)
__global__ void k_spmv(int N, const int32_t* __restrict__ col, const double* __restrict__ val,
                       const double* __restrict__ z, double* w, const int* done) {
    if (*done) return;
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= N) return;
    double acc = 0;
#pragma unroll
    for (int s = 0; s < HMEC_W; s++) {
        const size_t o = (size_t)s * N + row;
        acc += val[o] * z[col[o]];
    }
    w[row] = acc;
}

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

__global__ void k_cycle_begin(Gm G, const double* __restrict__ partial, int nblk, int first, double rtol, int m) {
    double rr = 0, bb = 0;
    for (int b = 0; b < nblk; b++) {
        rr += partial[b];
        bb += partial[nblk + b];
    }
    if (first) *G.bnorm = sqrt(bb);
    const double bn = *G.bnorm;
    const double beta = sqrt(rr);
    const double rel = bn > 0 ? beta / bn : beta;
    G.ds->krylov_relres = rel;
    G.g[0] = beta;
    for (int k = 1; k <= m; k++) G.g[k] = 0;
    *G.kcur = 0;
    *G.done = (rel <= rtol || !(beta > 0) || !isfinite(beta)) ? 1 : 0;
    G.dots[0] = beta > 0 ? 1.0 / beta : 0.0;  // scale for V0
}

__global__ void k_scale_vec(int N, const double* __restrict__ a, const double* sc, double* b, const int* done) {
    if (*done) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < N) b[r] = a[r] * sc[0];
}

// After the two CGS passes: column j of H, Givens rotation, residual estimate.
__global__ void k_arnoldi_step(Gm G, const double* __restrict__ h1, const double* __restrict__ partial, int nblk,
                               int j, int m, double rtol, double* hscale) {
    if (*G.done) return;
    double ww = 0;
    for (int b = 0; b < nblk; b++) ww += partial[b];
    const double hn = sqrt(ww);
    double* Hc = G.H + (size_t)j * (m + 1);  // column j, rows 0..j+1
    for (int k = 0; k <= j; k++) Hc[k] = h1[k] + G.dots[k];  // first + second CGS pass
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

static void make_geo(Geo& g, int Nx, int Ny, double xsize, double ysize) {
    g.Nx = Nx;
    g.Ny = Ny;
    g.Nx1 = Nx + 1;
    g.Ny1 = Ny + 1;
    g.N = g.Nx1 * g.Ny1 * 6;
    g.line_fault = (int)((Ny - 1) / 2.);
    g.dx = xsize / (Nx - 1);
    g.dy = ysize / (Ny - 1);
    g.dx2 = g.dx * g.dx;
    g.dy2 = g.dy * g.dy;
    g.dx_dy = g.dx * g.dy;
    g.lower_block = ysize / 2. + g.dy;
    g.upper_block = ysize / 2. - g.dy;
    g.dy_faultw = g.dy / g.dx;
}

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

static int alloc_level(hmec_ctx* ctx, Level& L, bool mixed, bool coarse) {
    const Geo& g = L.g;
    const size_t N = (size_t)g.N;
    L.npatch = (g.Ny - 1) * (g.Nx - 1);
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
    }
    {
        // tile ownership of every unknown (the tiled smoothing pass)
        L.tsz = TILE;
        L.ntile_i = (g.Ny - 1 + TILE - 1) / TILE;
        const int ntile_j = (g.Nx - 1 + TILE - 1) / TILE;
        L.ntiles = L.ntile_i * ntile_j;
        auto tile_of = [&](int pi, int pj) { return (pi - 1) / TILE + ((pj - 1) / TILE) * L.ntile_i; };
        std::vector<int32_t> owner(N);
        std::vector<char> isb(N, 0);
        for (int32_t r : br) isb[r] = 1;
        for (int j = 0; j <= g.Nx; j++)
            for (int i = 0; i <= g.Ny; i++)
                for (int v = 0; v < 6; v++) {
                    const int u = (j * g.Ny1 + i) * 6 + v;
                    int pi, pj;
                    if (isb[u]) {  // boundary row: the adjacent patch
                        pi = std::min(std::max(i, 1), g.Ny - 1);
                        pj = std::min(std::max(j, 1), g.Nx - 1);
                    } else if (v == 0 || v == 3) {
                        pi = i;
                        pj = j;
                    } else if (v == 1 || v == 4) {  // x face: the patch on its right
                        pi = i;
                        pj = (j + 1 <= g.Nx - 1) ? j + 1 : j;
                    } else {  // y face: the patch below
                        pi = (i + 1 <= g.Ny - 1) ? i + 1 : i;
                        pj = j;
                    }
                    owner[u] = tile_of(pi, pj);
                }
        std::vector<int32_t> os(L.ntiles + 1, 0), bs(L.ntiles + 1, 0);
        for (size_t u = 0; u < N; u++) {
            os[owner[u] + 1]++;
            if (isb[u]) bs[owner[u] + 1]++;
        }
        for (int k = 0; k < L.ntiles; k++) {
            os[k + 1] += os[k];
            bs[k + 1] += bs[k];
        }
        std::vector<int32_t> ol(N), bl(std::max<size_t>(br.size(), 1)), oc(os.begin(), os.end() - 1),
            bc(bs.begin(), bs.end() - 1);
        for (size_t u = 0; u < N; u++) {
            ol[oc[owner[u]]++] = (int32_t)u;
            if (isb[u]) bl[bc[owner[u]]++] = (int32_t)u;
        }
        HMEC_CUDA(ctx, cudaMalloc(&L.owner, sizeof(int32_t) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.own_start, sizeof(int32_t) * os.size()));
        HMEC_CUDA(ctx, cudaMalloc(&L.own_list, sizeof(int32_t) * N));
        HMEC_CUDA(ctx, cudaMalloc(&L.tbnd_start, sizeof(int32_t) * bs.size()));
        HMEC_CUDA(ctx, cudaMalloc(&L.tbnd_list, sizeof(int32_t) * bl.size()));
        HMEC_CUDA(ctx, cudaMemcpy(L.owner, owner.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(L.own_start, os.data(), sizeof(int32_t) * os.size(), cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(L.own_list, ol.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(L.tbnd_start, bs.data(), sizeof(int32_t) * bs.size(), cudaMemcpyHostToDevice));
        HMEC_CUDA(ctx, cudaMemcpy(L.tbnd_list, bl.data(), sizeof(int32_t) * bl.size(), cudaMemcpyHostToDevice));
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

int solver_alloc(hmec_ctx* ctx) {
    Solver& sv = ctx->sv;
    const hmec_params& p = ctx->p;
    const bool mixed = p.form == HMEC_FORM_MIXED;
    sv.m = std::max(2, p.krylov_restart);
    sv.N = ctx->g.N;
    sv.nblk = 152 * 2;
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
        make_geo(L.g, nx, ny, xs, ys);
        sv.lv.push_back(L);
    }
    for (size_t l = 0; l < sv.lv.size(); l++) {
        int rc = alloc_level(ctx, sv.lv[l], mixed, l > 0);
        if (rc) return rc;
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
    HMEC_CUDA(ctx, cudaMalloc(&sv.partial, sizeof(double) * (m + 2) * (size_t)sv.nblk));
    HMEC_CUDA(ctx, cudaMalloc(&sv.dots, sizeof(double) * (2 * m + 4)));
    HMEC_CUDA(ctx, cudaMalloc(&sv.bnorm, sizeof(double) * 2));
    HMEC_CUDA(ctx, cudaMalloc(&sv.done, sizeof(int) * 2));
    HMEC_CUDA(ctx, cudaMalloc(&sv.kcur, sizeof(int) * 2));
    HMEC_CUDA(ctx, cudaMemset(sv.done, 0, sizeof(int) * 2));
    return HMEC_OK;
}

void solver_free(hmec_ctx* ctx) {
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
        cudaFree(L.db);
        cudaFree(L.dr);
        cudaFree(L.fx);
        cudaFree(L.fb);
        cudaFree(L.fr);
        cudaFree(L.dx2);
        cudaFree(L.fx2);
        cudaFree(L.owner);
        cudaFree(L.own_start);
        cudaFree(L.own_list);
        cudaFree(L.tbnd_start);
        cudaFree(L.tbnd_list);
        for (double* p : L.owned) cudaFree(p);
    }
    sv.lv.clear();
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
}

static inline dim3 sgrid(const Geo& g) { return dim3(nblocks(g.Ny1, 64), g.Nx1); }

int solver_setup(hmec_ctx* ctx) {
    Solver& sv = ctx->sv;
    const bool mixed = ctx->p.form == HMEC_FORM_MIXED;
    int* status = &ctx->ds->status;
    for (size_t l = 0; l < sv.lv.size(); l++) {
        Level& L = sv.lv[l];
        if (l > 0) {
            Level& F = sv.lv[l - 1];
            CoefIn ci{F.af.ETA, F.af.GGG, F.af.RHO, F.af.ETAP, F.af.GGGP, F.af.ETAB, F.af.POR, F.af.GGGB,
                      F.af.RHOX, F.af.RHOFX, F.af.PORX, F.af.ETADX, F.af.RHOY, F.af.RHOFY, F.af.PORY, F.af.ETADY};
            AsmFields& a = L.af;
            CoefOut co{(double*)a.ETA, (double*)a.GGG, (double*)a.RHO, (double*)a.ETAP, (double*)a.GGGP,
                       (double*)a.ETAB, (double*)a.POR, (double*)a.GGGB, (double*)a.RHOX, (double*)a.RHOFX,
                       (double*)a.PORX, (double*)a.ETADX, (double*)a.RHOY, (double*)a.RHOFY, (double*)a.PORY,
                       (double*)a.ETADY};
            HMEC_LAUNCH(ctx, k_coarsen_coef, sgrid(L.g), 64, 0, F.g, L.g, ci, co, ctx->p.mg_flags);
            launch_assemble(ctx, L.g, L.af, L.col, L.val, L.dscale, nullptr, nullptr, nullptr);
        }
        HMEC_LAUNCH(ctx, k_vanka_setup, nblocks(L.npatch, 64), 64, 0, L.g, L.col, L.val, L.pinv, L.pinv32, status);
        if (mixed) {
            const size_t n = (size_t)HMEC_W * L.g.N;
            HMEC_LAUNCH(ctx, (k_convert<double, float>), nblocks(n, 256), 256, 0, n, L.val, L.val32);
        }
    }
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
};
template <>
struct LvPtr<float> {
    static float* x(Level& L) { return L.fx; }
    static float* b(Level& L) { return L.fb; }
    static float* r(Level& L) { return L.fr; }
    static const float* val(Level& L) { return L.val32; }
    static const float* pinv(Level& L) { return L.pinv32; }
};

// Levels with at most this many patches are smoothed by one block (a block
// barrier is cheaper than a grid barrier, but one block leaves the GPU idle:
// measured slower than a small cooperative grid for every level size here).
constexpr int SINGLE_BLOCK_PATCHES = 0;
// Levels whose x, b and boundary deltas fit in this much shared memory are
// smoothed by k_smooth_smem (one block, everything but the matrix on chip).
constexpr size_t SMEM_LIMIT = 200 * 1024;

template <typename T>
static int max_coop_blocks(hmec_ctx* ctx) {
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

template <typename T>
static int max_tiled_blocks(hmec_ctx* ctx) {
    static int cached[2] = {0, 0};
    int& c = cached[sizeof(T) == 8 ? 0 : 1];
    if (c == 0) {
        int per_sm = 0, nsm = 0;
        HMEC_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_smooth_win<T>, TILE_BS, 0));
        HMEC_CUDA(ctx, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
        c = std::max(1, per_sm * nsm);
    }
    return c;
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

// One smoothing pass on level l (x = 0 or x += P xc first, then nsweeps sweeps).
template <typename T>
static int smooth(hmec_ctx* ctx, size_t l, const T* b, T* x, int nsweeps, int mode, T* r_out = nullptr) {
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
    // algorithmic bytes: per sweep every patch's 10 ELL rows, inverse, rhs and
    // unknowns, and the boundary rows; plus the zero fill or the prolongation
    const double st = sizeof(T);
    const double bpp = 10.0 * HMEC_W * (st + 4) + 100.0 * st + 30.0 * st;
    const double bnd = (double)L.nbnd * (HMEC_W * (st + 4) + 4.0 * st);
    const double bytes = nsweeps * ((double)L.npatch * bpp + bnd) + (double)L.g.N * st * (mode ? 2.5 : 1.0);
    if (L.npatch <= SINGLE_BLOCK_PATCHES) {
        HMEC_LAUNCH_B(ctx, bytes, (k_smooth<T, false>), 1, SM_BS, 0, a, nsweeps, mode);
        return HMEC_OK;
    }
    if (!(ctx->p.mg_flags & HMEC_MG_UNTILED)) {
        TileArgs<T> t;
        t.a = a;
        t.xalt = x_alt<T>(L);
        t.owner = L.owner;
        t.own_start = L.own_start;
        t.own_list = L.own_list;
        t.tb_start = L.tbnd_start;
        t.tb_list = L.tbnd_list;
        t.ntile_i = L.ntile_i;
        t.ntiles = L.ntiles;
        t.r_out = r_out;
        // the owner tests add one int per matrix entry read and the second buffer
        const double tb = nsweeps * ((double)L.npatch * (10.0 * HMEC_W * 4 + 10.0 * HMEC_W * st) +
                                     (double)L.g.N * (2 * st + 8)) + bytes;
        const int grid = std::min(L.ntiles, max_tiled_blocks<T>(ctx));
        void* args[] = {&t, &nsweeps, &mode};
        const bool prof = hmec_prof_begin(ctx, "k_smooth", tb);
        HMEC_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_smooth_win<T>, dim3(grid), dim3(TILE_BS), args, 0,
                                                   ctx->stream));
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
        HMEC_LAUNCH_B(ctx, bytes, k_smooth_smem<T>, 1, SMEM_BS, smem, a, nsweeps, mode);
        return HMEC_OK;
    }
    // size the grid to one colour phase (the zero/prolongation and boundary
    // phases are grid-stride loops); fewer blocks make the grid barrier cheaper
    const long long work = std::max<long long>((long long)L.npatch * 16 / 9 + SM_BS, 2LL * SM_BS);
    const int grid = (int)std::min<long long>(max_coop_blocks<T>(ctx), std::max<long long>(1, (work + SM_BS - 1) / SM_BS));
    void* args[] = {&a, &nsweeps, &mode};
    const bool prof = hmec_prof_begin(ctx, "k_smooth", bytes);
    HMEC_CUDA(ctx, cudaLaunchCooperativeKernel((void*)k_smooth<T, true>, dim3(grid), dim3(SM_BS), args, 0, ctx->stream));
    ctx->launches++;
    if (prof) hmec_prof_end(ctx);
    return HMEC_OK;
}

// V-cycle on level l for A x = b, x = 0 on entry (b, x default to the level's buffers).
template <typename T>
static int vcycle(hmec_ctx* ctx, size_t l, const T* b_in = nullptr, T* x_in = nullptr) {
    Solver& sv = ctx->sv;
    Level& L = sv.lv[l];
    const hmec_params& p = ctx->p;
    const T* b = b_in ? b_in : LvPtr<T>::b(L);
    T* x = x_in ? x_in : LvPtr<T>::x(L);
    int rc;
    if (l + 1 == sv.lv.size()) {
        const int ns = (sv.lv.size() == 1) ? std::max(1, p.mg_pre + p.mg_post) : std::max(1, p.mg_coarse_sweeps);
        return smooth<T>(ctx, l, b, x, ns, 0);
    }
    Level& C = sv.lv[l + 1];
    if (!(p.mg_flags & HMEC_MG_UNTILED)) {
        // the pre-smoothing pass leaves the residual in the level's r buffer
        if ((rc = smooth<T>(ctx, l, b, x, p.mg_pre, 0, LvPtr<T>::r(L)))) return rc;
    } else {
        if ((rc = smooth<T>(ctx, l, b, x, p.mg_pre, 0))) return rc;
        HMEC_LAUNCH(ctx, k_resid<T>, nblocks(L.g.N, 256), 256, 0, L.g.N, L.col, LvPtr<T>::val(L), b, x,
                    LvPtr<T>::r(L));
    }
    const long long nc = (long long)C.g.N;
    HMEC_LAUNCH(ctx, k_restrict_r<T>, nblocks(nc, 128), 128, 0, L.g, C.g, LvPtr<T>::r(L), L.dscale, C.dscale,
                LvPtr<T>::b(C));
    if ((rc = vcycle<T>(ctx, l + 1))) return rc;
    return smooth<T>(ctx, l, b, x, p.mg_post, 1);
}

// z = M^{-1} v on the fine level (v, z FP64 vectors of the scaled system)
static int precondition(hmec_ctx* ctx, const double* v, double* z) {
    Solver& sv = ctx->sv;
    Level& L = sv.lv[0];
    const size_t N = (size_t)L.g.N;
    if (ctx->p.form == HMEC_FORM_MIXED) {
        HMEC_LAUNCH(ctx, (k_convert<double, float>), nblocks(N, 256), 256, 0, N, v, L.fb);
        int rc = vcycle<float>(ctx, 0);
        if (rc) return rc;
        HMEC_LAUNCH(ctx, (k_convert<float, double>), nblocks(N, 256), 256, 0, N, L.fx, z);
        return HMEC_OK;
    }
    return vcycle<double>(ctx, 0, v, z);
}

int solver_solve(hmec_ctx* ctx, int* iters_out, double* relres_out) {
    Solver& sv = ctx->sv;
    Level& L0 = sv.lv[0];
    const int N = sv.N, m = sv.m, nblk = sv.nblk;
    const double rtol = ctx->p.krylov_rtol;
    const int maxit = std::max(1, ctx->p.krylov_maxit);
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
        HMEC_LAUNCH(ctx, k_cycle_begin, 1, 1, 0, G, sv.partial, nblk, first ? 1 : 0, rtol, m);
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
        HMEC_LAUNCH(ctx, k_scale_vec, nblocks(N, 256), 256, 0, N, r, sv.dots, sv.V, sv.done);
        for (int j = 0; j < m && total + j < maxit; j++) {
            double* Vj = sv.V + (size_t)j * N;
            double* Zj = sv.Z + (size_t)j * N;
            // preconditioner (skipped cheaply when converged: its kernels are not predicated,
            // so check the flag before launching a whole V-cycle)
            if (j > 0 && (j % check_every) == 0) {
                int hd = 0;
                HMEC_CUDA(ctx, cudaMemcpyAsync(&ctx->hs->pad0, sv.done, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
                HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                hd = ctx->hs->pad0;
                if (hd) break;
            }
            int prc = precondition(ctx, Vj, Zj);
            if (prc) return prc;
            HMEC_LAUNCH_B(ctx, (double)N * (HMEC_W * 12.0 + 16.0), k_spmv, nblocks(N, 256), 256, 0, N, L0.col, L0.val,
                          Zj, sv.w, sv.done);
            // CGS pass 1
            HMEC_LAUNCH(ctx, k_dots, dim3(nblk, j + 1), RED_BS, 0, N, sv.V, sv.w, sv.partial, nblk, sv.done);
            HMEC_LAUNCH(ctx, k_dots_final, j + 1, 32, 0, sv.partial, nblk, j + 1, sv.dots + m + 2, sv.done);
            HMEC_LAUNCH(ctx, k_orth_update, nblk, RED_BS, 0, N, sv.V, j + 1, sv.dots + m + 2, sv.w, sv.partial, nblk, sv.done);
            // CGS pass 2
            HMEC_LAUNCH(ctx, k_dots, dim3(nblk, j + 1), RED_BS, 0, N, sv.V, sv.w, sv.partial, nblk, sv.done);
            HMEC_LAUNCH(ctx, k_dots_final, j + 1, 32, 0, sv.partial, nblk, j + 1, sv.dots, sv.done);
            HMEC_LAUNCH(ctx, k_orth_update, nblk, RED_BS, 0, N, sv.V, j + 1, sv.dots, sv.w, sv.partial, nblk, sv.done);
            HMEC_LAUNCH(ctx, k_arnoldi_step, 1, 1, 0, G, sv.dots + m + 2, sv.partial, nblk, j, m, rtol, sv.dots + 2 * m + 3);
            HMEC_LAUNCH(ctx, k_scale_vec, nblocks(N, 256), 256, 0, N, sv.w, sv.dots + 2 * m + 3, sv.V + (size_t)(j + 1) * N, sv.done);
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
