// k_p2g_static.cu -- markers -> nodes for callers that cannot allocate
// device memory.
//
// Some hosts may not call cudaMalloc at all: a solver embedded in another
// application that owns the device allocator (and forbids allocations behind
// its back), or a real-time loop that must never block on the allocator.
// This file
// gives them one entry point, hmec_markers_to_nodes_noalloc(), which computes
// exactly what hmec_markers_to_nodes() computes (sections a1-a4 of
// cpp/h_mec_rsf_v9.cpp:376-583: the half-cell counting sort and the
// deterministic node gathers) from marker and node arrays the caller already
// holds on the device.  Its only scratch memory -- the sort permutation and
// the per-half-cell counts and offsets -- is one file-scope __device__ array
// of fixed size, so the library allocates nothing for it, here or anywhere.
//
// Limits: at most HMEC_NOALLOC_MAX_MARKERS markers and
// HMEC_NOALLOC_MAX_HALF_CELLS half cells (4 (Nx-1)(Ny-1)); the array takes
// about 6 MiB on every device that loads the library, until the process
// exits.  All calls share it, so two calls that overlap on the GPU (other
// streams, other host threads) race and corrupt each other: serialise them.
#include <cstdio>
#include <mutex>

#include "hmec_internal.cuh"

#define HMEC_NOALLOC_MAX_MARKERS (1 << 20)
#define HMEC_NOALLOC_MAX_HALF_CELLS (1 << 18)

namespace {

constexpr int SCAN_CHUNK = 2048;
constexpr int MAX_PARTS = (HMEC_NOALLOC_MAX_HALF_CELLS + 1 + SCAN_CHUNK - 1) / SCAN_CHUNK + 1;
// layout: [perm: MAX_MARKERS][count: MAX_HALF+1][start: MAX_HALF+2][scan partials: MAX_PARTS]
constexpr size_t OFF_COUNT = HMEC_NOALLOC_MAX_MARKERS;
constexpr size_t OFF_START = OFF_COUNT + HMEC_NOALLOC_MAX_HALF_CELLS + 1;
constexpr size_t OFF_PART = OFF_START + HMEC_NOALLOC_MAX_HALF_CELLS + 2;
constexpr size_t SCRATCH_INTS = OFF_PART + MAX_PARTS;

}  // namespace

static __device__ __align__(256) int32_t g_p2g_scratch[SCRATCH_INTS];

namespace {

// Eigen LinSpaced(n, low, high), element i, in the host's IEEE operations.
__device__ __forceinline__ double linsp(int n, double low, double high, int i) {
    if (i == n - 1) return high;
    const double step = __ddiv_rn(__dsub_rn(high, low), (double)(n - 1));
    return __dadd_rn(low, __dmul_rn((double)i, step));
}

struct Mk {
    const double *xm, *ym, *t_marker, *rhom, *etasm, *etam, *cohescm, *cohestm, *frictcm, *dilatcm, *fricttm,
        *porm, *kkkm, *gm, *rhofm, *etafm;
};

struct Cells {
    int ib, jb, iP, jP;
};

__device__ __forceinline__ Cells cells_of(double xm, double ym, const Geo& g) {
    Cells c;
    const float rdx = rcp_f32(g.dx), rdy = rcp_f32(g.dy);
    c.jb = check_bounds(fix_quot(xm, g.dx, rdx, false), g.Nx);
    c.ib = check_bounds(fix_quot(ym, g.dy, rdy, false), g.Ny);
    c.jP = check_bounds(fix_quot(xm, g.dx, rdx, true), g.Nx);
    c.iP = check_bounds(fix_quot(ym, g.dy, rdy, true), g.Ny);
    return c;
}

__device__ __forceinline__ int half_key(const Cells& c, const Geo& g) {
    const int di = min(max(c.iP - c.ib, 0), 1), dj = min(max(c.jP - c.jb, 0), 1);
    return (2 * c.jb + dj) * (2 * (g.Ny - 1)) + 2 * c.ib + di;
}

// Marker properties of :389-423.
struct Props {
    double rho, kkk, ttt, invg, eta0, coht, frit, cohc, fric, dilc, etap, por, etab0, invetad, rhof;
};

__device__ __forceinline__ double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ Props props_of(const Mk& mk, int m, const hmec_params& p) {
    Props q;
    const double por = mk.porm[m];
    const double kkkmm = clampd(mk.kkkm[m] * pow(por / p.POR0, 3.0), p.kkkmin, p.kkkmax);
    const double tm = mk.t_marker[m];
    double etamm0;
    if (tm != 0) {
        q.cohc = mk.cohescm[m] * (1 - por);
        q.coht = mk.cohestm[m] * (1 - por);
        q.dilc = mk.dilatcm[m];
        etamm0 = mk.etasm[m] * exp(-p.alpha * por);
        q.rho = mk.rhom[m] * (1 - por) + mk.rhofm[m] * por;
    } else {
        q.cohc = mk.cohescm[m];
        q.coht = mk.cohestm[m];
        q.dilc = 0;
        etamm0 = mk.etasm[m];
        q.rho = mk.rhom[m];
    }
    q.fric = mk.frictcm[m];
    q.frit = mk.fricttm[m];
    q.eta0 = clampd(etamm0, p.etamin, p.etamax);
    q.etap = clampd(mk.etam[m], p.etamin, p.etamax);
    q.etab0 = mk.etasm[m];
    q.kkk = kkkmm;
    q.ttt = tm;
    q.invg = 1. / mk.gm[m];
    q.por = por;
    q.invetad = 1. / (mk.etafm[m] / kkkmm);
    q.rhof = mk.rhofm[m];
    return q;
}

__global__ void k_nz_zero(int32_t* a, int n) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = 0;
}

__global__ void k_nz_count(Mk mk, int64_t n, Geo g, int32_t* count) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int k = -1;
    if (m < n) k = half_key(cells_of(mk.xm[m], mk.ym[m], g), g);
    const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
    if (k >= 0) {
        const unsigned peers = __match_any_sync(active, k);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&count[k], __popc(peers));
    }
}

// Exclusive scan in chunks of SCAN_CHUNK, then chunk offsets (one block), then add.
__global__ void k_nz_scan1(const int32_t* in, int n, int32_t* out, int32_t* part) {
    __shared__ int32_t sh[SCAN_CHUNK];
    const int base = blockIdx.x * SCAN_CHUNK, t = threadIdx.x;
    for (int k = t; k < SCAN_CHUNK; k += blockDim.x) sh[k] = (base + k < n) ? in[base + k] : 0;
    __syncthreads();
    if (t == 0) {  // chunks are short; a serial scan keeps this variant simple
        int32_t acc = 0;
        for (int k = 0; k < SCAN_CHUNK; k++) {
            const int32_t v = sh[k];
            sh[k] = acc;
            acc += v;
        }
        part[blockIdx.x] = acc;
    }
    __syncthreads();
    for (int k = t; k < SCAN_CHUNK; k += blockDim.x)
        if (base + k < n) out[base + k] = sh[k];
}

__global__ void k_nz_scan2(int32_t* part, int nparts) {
    if (threadIdx.x != 0) return;
    int32_t acc = 0;
    for (int k = 0; k < nparts; k++) {
        const int32_t v = part[k];
        part[k] = acc;
        acc += v;
    }
}

__global__ void k_nz_scan3(int32_t* out, int n, const int32_t* part, int32_t* cursor) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const int32_t v = out[t] + part[t / SCAN_CHUNK];
        out[t] = v;
        cursor[t] = v;
    }
}

__global__ void k_nz_scatter(Mk mk, int64_t n, Geo g, int32_t* cursor, int32_t* perm) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int k = -1;
    if (m < n) k = half_key(cells_of(mk.xm[m], mk.ym[m], g), g);
    const unsigned active = __ballot_sync(0xffffffffu, k >= 0);
    if (k >= 0) {
        const unsigned peers = __match_any_sync(active, k);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&cursor[k], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        perm[base + __popc(peers & ((1u << lane) - 1u))] = (int32_t)m;
    }
}

__global__ void k_nz_segsort(const int32_t* start, int nseg, int32_t* perm) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const int b = start[s], e = start[s + 1];
    for (int a = b + 1; a < e; a++) {
        const int v = perm[a];
        int q = a;
        while (q > b && perm[q - 1] > v) {
            perm[q] = perm[q - 1];
            q--;
        }
        perm[q] = v;
    }
}

struct Out {
    double *RHO, *KKK, *TTT, *GGG, *ETA0, *COHT, *FRIT, *COHC, *FRIC, *DILC;
    double *ETAP, *POR, *ETAB0, *ETAP0, *GGGP;
    double *RHOX, *ETADX, *RHOFX, *PORX, *RHOY, *ETADY, *RHOFY, *PORY;
};

// grid: 0 basic, 1 P, 2 Vx, 3 Vy.  One thread per node; the same half-cell
// runs, visiting order and weights as the context path.
template <int GRID>
__global__ void k_nz_gather(Mk mk, hmec_params p, Geo g, const int32_t* __restrict__ start,
                            const int32_t* __restrict__ perm, Out o) {
    constexpr bool ROWP = (GRID == 1 || GRID == 2), COLP = (GRID == 1 || GRID == 3);
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    const int nrow = (GRID == 0 || GRID == 3) ? g.Ny : g.Ny1;
    const int ncol = (GRID == 0 || GRID == 2) ? g.Nx : g.Nx1;
    if (i >= nrow || j >= ncol) return;
    const int HR = 2 * (g.Ny - 1), HC = 2 * (g.Nx - 1);
    const int r0 = ROWP ? 2 * i - 3 : 2 * i - 2, c0 = COLP ? 2 * j - 3 : 2 * j - 2;
    const int rlo = r0 < 0 ? 0 : r0, rhi = (r0 + 3) > HR - 1 ? HR - 1 : r0 + 3;
    double wt = 0, a[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (rlo <= rhi) {
        for (int hc = (c0 < 0 ? 0 : c0); hc <= c0 + 3 && hc < HC; hc++) {
            const int cj = COLP ? (hc + 1) >> 1 : hc >> 1;
            const int b = start[hc * HR + rlo], e = start[hc * HR + rhi + 1];
            const int split_hr = ROWP ? 2 * i - 1 : 2 * i;
            const int bsplit = (split_hr <= rlo) ? b : (split_hr > rhi ? e : start[hc * HR + split_hr]);
            for (int k = b; k < e; k++) {
                const int m = perm[k];
                const double xmm = mk.xm[m], ymm = mk.ym[m];
                const Cells c = cells_of(xmm, ymm, g);
                double xn, yn;
                if (GRID == 0) {
                    xn = linsp(g.Nx, 0, p.xsize, c.jb);
                    yn = linsp(g.Ny, 0, p.ysize, c.ib);
                } else if (GRID == 1) {
                    xn = linsp(g.Nx1, 0 - g.dx / 2., p.xsize + g.dx / 2., c.jP);
                    yn = linsp(g.Ny1, 0 - g.dy / 2., p.ysize + g.dy / 2., c.iP);
                } else if (GRID == 2) {
                    xn = linsp(g.Nx1, 0, p.xsize + g.dx, c.jb);
                    yn = linsp(g.Ny1, 0 - g.dy / 2., p.ysize + g.dy / 2., c.iP);
                } else {
                    xn = linsp(g.Nx1, 0 - g.dx / 2., p.xsize + g.dx / 2., c.jP);
                    yn = linsp(g.Ny1, 0, p.ysize + g.dy, c.ib);
                }
                const double dxm = (xmm - xn) / g.dx, dym = (ymm - yn) / g.dy;
                const double fx = (cj == j) ? (1 - dxm) : dxm;
                const double fy = (k >= bsplit) ? (1 - dym) : dym;
                const double w = fx * fy;
                const Props q = props_of(mk, m, p);
                wt += w;
                if (GRID == 0) {
                    a[0] += q.rho * w;
                    a[1] += q.kkk * w;
                    a[2] += q.ttt * w;
                    a[3] += q.invg * w;
                    a[4] += q.eta0 * w;
                    a[5] += q.coht * w;
                    a[6] += q.frit * w;
                    a[7] += q.cohc * w;
                    a[8] += q.fric * w;
                    a[9] += q.dilc * w;
                } else if (GRID == 1) {
                    a[0] += q.etap * w;
                    a[1] += q.por * w;
                    a[2] += q.etab0 * w;
                    a[3] += q.eta0 * w;
                    a[4] += q.invg * w;
                } else {
                    a[0] += q.rho * w;
                    a[1] += q.invetad * w;
                    a[2] += q.rhof * w;
                    a[3] += q.por * w;
                }
            }
        }
    }
    if (!(wt > 0)) return;  // nodes without markers keep their values (:536 etc.)
    const size_t oo = (size_t)j * nrow + i;
    if (GRID == 0) {
        o.RHO[oo] = a[0] / wt;
        o.KKK[oo] = a[1] / wt;
        o.TTT[oo] = a[2] / wt;
        o.GGG[oo] = 1. / (a[3] / wt);
        o.ETA0[oo] = a[4] / wt;
        o.COHT[oo] = a[5] / wt;
        o.FRIT[oo] = a[6] / wt;
        o.COHC[oo] = a[7] / wt;
        o.FRIC[oo] = a[8] / wt;
        o.DILC[oo] = a[9] / wt;
    } else if (GRID == 1) {
        const double por = a[1] / wt;
        o.ETAP[oo] = a[0] / wt;
        o.POR[oo] = por;
        o.ETAB0[oo] = a[2] / wt / por;
        o.ETAP0[oo] = a[3] / wt;
        o.GGGP[oo] = 1. / (a[4] / wt);
    } else {
        const size_t os = (size_t)j * g.Ny1 + i;  // Vx/Vy fields are stored staggered-sized
        double* R = GRID == 2 ? o.RHOX : o.RHOY;
        double* E = GRID == 2 ? o.ETADX : o.ETADY;
        double* F = GRID == 2 ? o.RHOFX : o.RHOFY;
        double* P = GRID == 2 ? o.PORX : o.PORY;
        R[os] = a[0] / wt;
        E[os] = 1. / (a[1] / wt);
        F[os] = a[2] / wt;
        P[os] = a[3] / wt;
    }
}

std::mutex g_setup_mutex;
int32_t* g_scratch_addr[256];  // device address of g_p2g_scratch, per device ordinal

int noalloc_fail(int code, const char* msg) {
    fprintf(stderr, "hmec_markers_to_nodes_noalloc: %s\n", msg);
    return code;
}

}  // namespace

extern "C" int32_t hmec_markers_to_nodes_noalloc(const hmec_params* p, const double* const* markers,
                                                 int64_t n, double* const* fields, void* stream) {
    if (!p || !markers || !fields) return noalloc_fail(HMEC_ERR_ARG, "null argument");
    for (int k = 0; k < HMEC_M_COUNT; k++)
        if (!markers[k]) return noalloc_fail(HMEC_ERR_ARG, "null marker array");
    const int outs[] = {HMEC_F_RHO, HMEC_F_KKK, HMEC_F_TTT, HMEC_F_GGG, HMEC_F_ETA0, HMEC_F_COHT, HMEC_F_FRIT,
                        HMEC_F_COHC, HMEC_F_FRIC, HMEC_F_DILC, HMEC_F_ETAP, HMEC_F_POR, HMEC_F_ETAB0, HMEC_F_ETAP0,
                        HMEC_F_GGGP, HMEC_F_RHOX, HMEC_F_ETADX, HMEC_F_RHOFX, HMEC_F_PORX, HMEC_F_RHOY,
                        HMEC_F_ETADY, HMEC_F_RHOFY, HMEC_F_PORY};
    for (int f : outs)
        if (!fields[f]) return noalloc_fail(HMEC_ERR_ARG, "null output field");
    if (p->Nx < 5 || p->Ny < 5 || !(p->xsize > 0) || !(p->ysize > 0))
        return noalloc_fail(HMEC_ERR_ARG, "grid parameters out of range (Nx, Ny >= 5, sizes > 0)");
    if (n < 1 || n > HMEC_NOALLOC_MAX_MARKERS)
        return noalloc_fail(HMEC_ERR_ARG, "marker count outside [1, HMEC_NOALLOC_MAX_MARKERS = 1048576]");
    const long long nh = 4LL * (p->Nx - 1) * (p->Ny - 1);
    if (nh > HMEC_NOALLOC_MAX_HALF_CELLS)
        return noalloc_fail(HMEC_ERR_ARG, "grid too large: 4*(Nx-1)*(Ny-1) exceeds HMEC_NOALLOC_MAX_HALF_CELLS = 262144");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256)
        return noalloc_fail(HMEC_ERR_CUDA, "cudaGetDevice failed");
    int32_t* scratch = nullptr;
    {
        // Set-up, once per device, with that device current: the host name of
        // g_p2g_scratch is only a stand-in, the kernels need its device address.
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            int32_t* ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_p2g_scratch);
            if (e != cudaSuccess || !ptr) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e));
            g_scratch_addr[dev] = ptr;
        }
        scratch = g_scratch_addr[dev];
    }
    int32_t* perm = scratch;
    int32_t* count = scratch + OFF_COUNT;
    int32_t* start = scratch + OFF_START;
    int32_t* part = scratch + OFF_PART;
    Geo g;
    g.Nx = p->Nx;
    g.Ny = p->Ny;
    g.Nx1 = p->Nx + 1;
    g.Ny1 = p->Ny + 1;
    g.N = g.Nx1 * g.Ny1 * 6;
    g.line_fault = (int)((p->Ny - 1) / 2.);
    g.dx = p->xsize / (p->Nx - 1);
    g.dy = p->ysize / (p->Ny - 1);
    g.dx2 = g.dx * g.dx;
    g.dy2 = g.dy * g.dy;
    g.dx_dy = g.dx * g.dy;
    g.lower_block = p->ysize / 2. + g.dy;
    g.upper_block = p->ysize / 2. - g.dy;
    g.dy_faultw = g.dy / g.dx;
    geo_reciprocals(g);
    Mk mk{markers[HMEC_M_xm], markers[HMEC_M_ym], markers[HMEC_M_t_marker], markers[HMEC_M_rhom],
          markers[HMEC_M_etasm], markers[HMEC_M_etam], markers[HMEC_M_cohescm], markers[HMEC_M_cohestm],
          markers[HMEC_M_frictcm], markers[HMEC_M_dilatcm], markers[HMEC_M_fricttm], markers[HMEC_M_porm],
          markers[HMEC_M_kkkm], markers[HMEC_M_gm], markers[HMEC_M_rhofm], markers[HMEC_M_etafm]};
    Out o{fields[HMEC_F_RHO], fields[HMEC_F_KKK], fields[HMEC_F_TTT], fields[HMEC_F_GGG], fields[HMEC_F_ETA0],
          fields[HMEC_F_COHT], fields[HMEC_F_FRIT], fields[HMEC_F_COHC], fields[HMEC_F_FRIC], fields[HMEC_F_DILC],
          fields[HMEC_F_ETAP], fields[HMEC_F_POR], fields[HMEC_F_ETAB0], fields[HMEC_F_ETAP0], fields[HMEC_F_GGGP],
          fields[HMEC_F_RHOX], fields[HMEC_F_ETADX], fields[HMEC_F_RHOFX], fields[HMEC_F_PORX],
          fields[HMEC_F_RHOY], fields[HMEC_F_ETADY], fields[HMEC_F_RHOFY], fields[HMEC_F_PORY]};
    cudaStream_t s = (cudaStream_t)stream;
    const int ns = (int)nh + 1;
    const int nparts = (ns + SCAN_CHUNK - 1) / SCAN_CHUNK;
    // the array keeps the last call's contents: the histogram must start at zero
    k_nz_zero<<<nblocks(ns, 256), 256, 0, s>>>(count, ns);
    k_nz_count<<<nblocks(n, 256), 256, 0, s>>>(mk, n, g, count);
    k_nz_scan1<<<nparts, 256, 0, s>>>(count, ns, start, part);
    k_nz_scan2<<<1, 32, 0, s>>>(part, nparts);
    k_nz_scan3<<<nblocks(ns, 256), 256, 0, s>>>(start, ns, part, count);  // count becomes the scatter cursor
    k_nz_scatter<<<nblocks(n, 256), 256, 0, s>>>(mk, n, g, count, perm);
    k_nz_segsort<<<nblocks(nh, 128), 128, 0, s>>>(start, (int)nh, perm);
    const dim3 bb(64);
    k_nz_gather<0><<<dim3(nblocks(g.Ny, 64), g.Nx), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<1><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<2><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<3><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e));
    return HMEC_OK;
}
