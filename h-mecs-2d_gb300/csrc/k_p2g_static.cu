// k_p2g_static.cu -- markers -> nodes for callers that cannot allocate
// device memory.
//
// Some hosts may not call cudaMalloc at all: a solver embedded in another
// application that owns the device allocator (and forbids allocations behind
// its back), or a real-time loop that must never block on the allocator.
// This file gives them one entry point, hmec_markers_to_nodes_noalloc(),
// which computes what hmec_markers_to_nodes() computes (sections a1-a4 of
// cpp/h_mec_rsf_v9.cpp:376-583) from marker and node arrays the caller
// already holds on the device.  It sorts the markers with the same
// deterministic half-cell sort (hmec_sort.cuh) and gathers each node's sums
// from its half cells with the reference's weights; its summation order
// differs from the context path's (per node here, per cell corner there), so
// the two agree to about 1e-13 relative, not bit for bit.  Its only scratch
// memory -- marker keys, the permutation, the per-half-cell counts, offsets
// and cursors, and the radix sort's buffers -- is one file-scope __device__
// array of fixed size, so nothing is allocated for it, here or anywhere.
//
// Limits: at most HMEC_NOALLOC_MAX_MARKERS markers and
// HMEC_NOALLOC_MAX_HALF_CELLS half cells (4 (Nx-1)(Ny-1)); the array takes
// about 25 MiB of device memory.  The driver reserves it when it loads the
// library's device code on a device -- under lazy module loading (the
// default) that is the first call on that device -- and keeps it until the
// process exits.  All calls share it, so two calls that overlap on the GPU
// (other streams, other host threads) race and corrupt each other:
// serialise them.
#include <cstdio>
#include <mutex>

#include "hmec_internal.cuh"
#include "hmec_mprop.cuh"
#include "hmec_sort.cuh"

#define HMEC_NOALLOC_MAX_MARKERS (1 << 20)
#define HMEC_NOALLOC_MAX_HALF_CELLS (1 << 18)

namespace {

constexpr int64_t MAXN = HMEC_NOALLOC_MAX_MARKERS;
constexpr int64_t MAXH = HMEC_NOALLOC_MAX_HALF_CELLS;
constexpr int64_t MAX_PARTS = (MAXH + 1 + 2047) / 2048 + 1;
constexpr int64_t MAX_TILES = (MAXN + hsort::RS_BS - 1) / hsort::RS_BS;  // also bounds the radix grid
// layout (int32): key [MAXN] | perm [MAXN] | count [MAXH+1] | start [MAXH+2] |
// fill [MAXH+1] | scan partials [MAX_PARTS] | long flag [16] | radix scratch
constexpr size_t OFF_PERM = MAXN;
constexpr size_t OFF_COUNT = OFF_PERM + MAXN;
constexpr size_t OFF_START = OFF_COUNT + MAXH + 1;
constexpr size_t OFF_FILL = OFF_START + MAXH + 2;
constexpr size_t OFF_PART = OFF_FILL + MAXH + 1;
constexpr size_t OFF_FLAG = OFF_PART + MAX_PARTS;
constexpr size_t OFF_RADIX = (OFF_FLAG + 16 + 63) / 64 * 64;
constexpr size_t SCRATCH_INTS = OFF_RADIX + 3 * MAXN + hsort::RS_BINS * MAX_TILES + MAX_TILES + 16;

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

// Marker properties of :389-423 (the FP64 values of hmec_mprop.cuh, as the
// context path forms them, plus the two reciprocals in FP64).
struct Props {
    double rho, kkk, ttt, invg, eta0, coht, frit, cohc, fric, dilc, etap, por, etab0, invetad, rhof;
};

__device__ __forceinline__ Props props_of(const Mk& mk, int m, const hmec_params& p, double ipor0) {
    const MarkerProps mp = marker_props(mk, m, p, ipor0);
    Props q;
    q.rho = mp.rho;
    q.kkk = mp.kkk;
    q.ttt = mp.tm;
    q.invg = 1. / mk.gm[m];
    q.eta0 = mp.eta0;
    q.coht = mp.coht;
    q.frit = mp.frit;
    q.cohc = mp.cohc;
    q.fric = mp.fric;
    q.dilc = mp.dilc;
    q.etap = mp.eta;
    q.por = mp.por;
    q.etab0 = mp.etas;
    q.invetad = 1. / (mk.etafm[m] / mp.kkk);
    q.rhof = mk.rhofm[m];
    return q;
}

struct Out {
    double *RHO, *KKK, *TTT, *GGG, *ETA0, *COHT, *FRIT, *COHC, *FRIC, *DILC;
    double *ETAP, *POR, *ETAB0, *ETAP0, *GGGP;
    double *RHOX, *ETADX, *RHOFX, *PORX, *RHOY, *ETADY, *RHOFY, *PORY;
};

// grid: 0 basic, 1 P, 2 Vx, 3 Vy.  One thread per node sums over the
// markers of the half cells around it (in the sorted order) with the
// reference's bilinear weights, in FP64; the context path sums per cell
// corner in double-float and then adds four cells, so the results agree to
// about 1e-13 relative.
template <int GRID>
__global__ void k_nz_gather(Mk mk, hmec_params p, Geo g, const int32_t* __restrict__ start,
                            const int32_t* __restrict__ perm, Out o) {
    constexpr bool ROWP = (GRID == 1 || GRID == 2), COLP = (GRID == 1 || GRID == 3);
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    const int nrow = (GRID == 0 || GRID == 3) ? g.Ny : g.Ny1;
    const int ncol = (GRID == 0 || GRID == 2) ? g.Nx : g.Nx1;
    if (i >= nrow || j >= ncol) return;
    const int HR = 2 * (g.Ny - 1), HC = 2 * (g.Nx - 1);
    const double ipor0 = 1.0 / p.POR0;
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
                const MarkerCells c = marker_cells(xmm, ymm, g);
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
                const Props q = props_of(mk, m, p, ipor0);
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

// The device address of g_p2g_scratch for the current device.  The host
// name of the array is only a stand-in, so the address is looked up with the
// device current, once per device and CUDA context: a context that was torn
// down and created again (cudaDeviceReset) gets a new ID, and the address is
// looked up again.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

struct ScratchAddr {
    unsigned long long ctx_id;
    int32_t* ptr;
};
std::mutex g_setup_mutex;
ScratchAddr g_scratch_addr[256];

bool current_ctx_id(unsigned long long* id) {
    static PfnCtxGetCurrent get_cur = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!get_cur || !get_id) {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa = cudaDriverEntryPointSymbolNotFound, qb = qa;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
            qa != cudaDriverEntryPointSuccess || qb != cudaDriverEntryPointSuccess || !a || !b)
            return false;
        get_cur = (PfnCtxGetCurrent)a;
        get_id = (PfnCtxGetId)b;
    }
    CUcontext c = nullptr;
    if (get_cur(&c) != CUDA_SUCCESS || !c) return false;
    return get_id(c, id) == CUDA_SUCCESS;
}

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
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        unsigned long long id = 0;
        const bool have_id = current_ctx_id(&id);
        ScratchAddr& sa = g_scratch_addr[dev];
        if (!sa.ptr || !have_id || sa.ctx_id != id) {
            int32_t* ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_p2g_scratch);
            if (e != cudaSuccess || !ptr) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e));
            unsigned long long id2 = 0;
            sa.ptr = ptr;
            sa.ctx_id = current_ctx_id(&id2) ? id2 : 0;  // the lookup made the context current
        }
        scratch = sa.ptr;
    }
    Geo g;
    geo_make(g, p->Nx, p->Ny, p->xsize, p->ysize);
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
    hsort::SortBufs sb{scratch, scratch + OFF_COUNT, scratch + OFF_START, scratch + OFF_FILL, scratch + OFF_PART,
                       scratch + OFF_PERM, scratch + OFF_FLAG, scratch + OFF_RADIX};
    const int32_t* start = sb.start;
    const int32_t* perm = sb.perm;
    // the array keeps the last call's contents: the histogram starts at zero
    cudaError_t e0 = cudaMemsetAsync(sb.count, 0, sizeof(int32_t) * ((size_t)nh + 1), s);
    if (e0 != cudaSuccess) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e0));
    hsort::k_keys<<<nblocks(n, 256), 256, 0, s>>>(mk.xm, mk.ym, n, g, sb.key, sb.count, nullptr);
    e0 = hsort::sort_by_half_cell(s, sb, n, (int)nh, nullptr);
    if (e0 != cudaSuccess) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e0));
    const dim3 bb(64);
    k_nz_gather<0><<<dim3(nblocks(g.Ny, 64), g.Nx), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<1><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<2><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    k_nz_gather<3><<<dim3(nblocks(g.Ny1, 64), g.Nx1), bb, 0, s>>>(mk, *p, g, start, perm, o);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(HMEC_ERR_CUDA, cudaGetErrorString(e));
    return HMEC_OK;
}
