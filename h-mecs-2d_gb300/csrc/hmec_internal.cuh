// hmec_internal.cuh -- device-side data layout and helpers shared by the
// translation units of libhmec_gpu.so (GB300, sm_103a).
//
// HBM layout: every node field is its own FP64 column-major array with the
// reference's shape (basic Ny x Nx, staggered (Ny+1) x (Nx+1)), so uploads
// and downloads are plain copies of Eigen storage.  Kernels map the row index
// i to threadIdx.x, which makes a warp read 32 consecutive doubles of one
// grid column.  Scalars of the global-iteration control live in one
// DevScalars block in device memory and are only touched by single-thread
// control kernels, so the whole loop runs without host round trips.
#pragma once

#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's driver entry point)
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hmec.h"
#include "hmec_bits.cuh"

#define HMEC_W 11  // ELL width: the longest assembled row (x/y-Stokes) has 11 entries

// Status bits raised by device code (device word -> host status).
enum {
    HMEC_DEV_BOUNDS = 1,
    HMEC_DEV_NAN = 2,
    HMEC_DEV_RSF_NOCONV = 4,
    HMEC_DEV_KRYLOV_NOCONV = 8,
    HMEC_DEV_TIMEOUT = 16,
};

// One fine index of a 1D grid transfer: the coarse cell holding the fine
// cell centre, and the coarse nodes node0, node0+1 with their hat weights at
// the fine node.
struct XferEnt {
    int cell, node0;
    double w0, w1;
};
#define HMEC_RW 8  // restriction entries per coarse unknown (2 cells x 4 nodes at most)

// Grid geometry of one level (the fine level is the model grid).
struct Geo {
    int Nx, Ny, Nx1, Ny1, N, line_fault;
    double dx, dy, dx2, dy2, dx_dy, lower_block, upper_block, dy_faultw;
    // 1/dx, 1/dy, 1/dx^2, 1/dy^2, 1/(dx dy), 1/(2 dx), 1/(2 dy): the kernels
    // multiply where the reference divides by these grid constants (FP64
    // division costs ~8 FMAs); results move by at most an ulp or two
    double idx, idy, idx2, idy2, idx_dy, i2dx, i2dy;
};

// Fills the reciprocal grid constants of g (after dx, dy, dx2, dy2, dx_dy).
inline void geo_reciprocals(Geo& g) {
    g.idx = 1.0 / g.dx;
    g.idy = 1.0 / g.dy;
    g.idx2 = 1.0 / g.dx2;
    g.idy2 = 1.0 / g.dy2;
    g.idx_dy = 1.0 / g.dx_dy;
    g.i2dx = 1.0 / (2. * g.dx);
    g.i2dy = 1.0 / (2. * g.dy);
}

// Control scalars of one model instance (device resident).
struct DevScalars {
    double timesum, dt, dt00, dtx, dty, dtlapusta, Vmax, maxvxy, maxvxy0;
    double ptscale, pfscale;
    double guess_ratio;  // previous pressure scale / current one, applied to the warm start
    double dsylsq, dsylsq_prev;
    double maxvxsmod, minvxsmod, maxvysmod, minvysmod;
    double krylov_relres, krylov_maxrel;
    int yndtdecrease, timestep, ynlast, iterstep;
    int ynpl, stop, loop_done, status;
    int krylov_iters, krylov_total, iters_in_step, pad0;
    int krylov_cycles, pad1;  // restart cycles of the step's solves
};

// Device state of a solve whose restart and Arnoldi loops run on the device
// (graph mode): the previous cycle's residual, the first-cycle flag, the cap.
struct GmCtl {
    double prev;
    int first, maxit;
};

// Pointers to the node fields read by the assembly of one level.
struct AsmFields {
    const double *ETA, *GGG, *RHO, *SXY0;                            // basic
    const double *ETAP, *GGGP, *ETAB, *POR, *GGGB, *SXX0, *SYY0;     // P
    const double *RHOX, *RHOFX, *PORX, *ETADX, *VX0, *VXF0;          // Vx
    const double *RHOY, *RHOFY, *PORY, *ETADY, *VY0, *VYF0;          // Vy
    const double *PT0, *PF0, *DILP;                                  // P (rhs)
};

// One multigrid level of the preconditioner.
struct Level {
    Geo g;
    int npatch;            // interior P cells: (Ny-1)*(Nx-1)
    int nbnd;              // rows not covered by any Vanka patch
    int32_t* col;          // ELL columns, slot-major [HMEC_W][N]
    double* val;           // row-scaled matrix values (FP64), slot-major
    float* val32;          // FP32 copy (mixed form)
    double* dscale;        // row scale (power of two) applied to the matrix
    int32_t* bnd_rows;     // rows outside every patch
    double* pinv;          // Vanka patch inverses, [100][npatch] (FP64 form)
    float* pinv32;         // same in FP32 (mixed form)
    // work vectors (FP64 form uses d*, mixed form uses f*); db of level 0 is
    // the scaled system rhs, pb the preconditioner input of the FP64 form
    double *dx_, *db, *dr, *pb;
    float *fx, *fb, *fr;
    // tiled smoother: tiles of tsz x tsz patches, one block each; every
    // unknown has one owning tile; tbnd_start/tbnd_list list each tile's
    // boundary rows
    int tsz, ntile_i, ntiles;
    int32_t *tbnd_start, *tbnd_list;
    int tb_cap = 16;       // most boundary rows of one tile (rounded up to 16)
    // staged smoothing launch of this level: inverse mode, grid, shared memory
    int st_whole = -1, st_grid = 0, st_smem = 0;
    double* dx2;
    float* fx2;
    // staged smoothing pass.  The smoother's copy of the matrix in a padded
    // layout, [slot][column j][CS] with CS = 6*Ny1 rounded up to 8, so that a
    // tile's rows form one 3-D box for a TMA tensor copy: values in the
    // smoother's precision (vals) and every column as an int16 offset in the
    // tile's window of unknowns (offs), rebuilt with each assembly
    int CS = 0;
    void* vals = nullptr;
    int16_t* offs = nullptr;
    // the standard offsets of an interior cell's six rows [6][W], and per
    // tile whether all its rows have them (set once: the pattern is fixed)
    int16_t* std_off = nullptr;
    uint8_t* std_t = nullptr;
    bool offs_ready = false;
    // per tile: its window's ownership bits and the per-lane colour table
    // with the ownership of each lane's unknown (fixed by the geometry), and
    // its boundary rows packed (rebuilt with each assembly; the smoothing
    // pass reads them from global memory)
    uint32_t* own_t = nullptr;
    int32_t* meta_t = nullptr;
    unsigned char* bpack = nullptr;
    int pack_bytes = 0;
    // TMA descriptors of vals and the patch inverses
    CUtensorMap tm_val, tm_pinv;
    // prolongation from the next coarser level: per fine x index (Nx+1) and
    // y index (Ny+1) the coarse cell and the two coarse nodes' hat weights
    XferEnt *pmx, *pmy;
    // restriction from the next finer level into this one: per coarse unknown
    // HMEC_RW (fine unknown, weight) pairs, slot-major; rwg holds the
    // geometric weights, rw / rw32 those times the row-scale ratio
    int32_t* ridx;
    double *rwg, *rw;
    float* rw32;
    // coarse-level coefficient fields (owned for l > 0)
    std::vector<double*> owned;
    AsmFields af;
};

struct Solver {
    int m;                 // restart length
    int N;
    double* V;             // (m+1) x N Krylov basis
    double* Z;             // m x N preconditioned directions
    double* w;
    double* H;             // (m+1) x m Hessenberg (device)
    double* cs; double* sn; double* gvec; double* yvec;
    double* partial;       // block partial sums [(2m+3) x nblk]: both CGS passes and |w|^2
    double* dots;          // (m+1) reduced dot products
    double* bnorm;         // ||D b||
    int* done;             // convergence flag of the current solve
    int* kcur;             // Arnoldi steps taken in the current cycle
    GmCtl* gctl = nullptr; // device-controlled solve state (graph mode)
    int nblk;
    std::vector<Level> lv;
    // setup of the levels as a dependency graph: level l's assembly and its
    // smoother data on aux[l]; coef[l]: level l's coarse coefficients are
    // ready (main stream), asm[l]: its matrix and row scale are, done[l]: all
    // of its setup is
    std::vector<cudaStream_t> aux;
    std::vector<cudaEvent_t> ev_coef, ev_asm, ev_done;
    cudaEvent_t ev_fork = nullptr;
    // the mixed form's V-cycle as one launch: its pass table (the kernel
    // parameter, built once: it holds only the levels' fixed buffers), launch
    // shape and algorithmic bytes; state 0 unbuilt, 1 in use, -1 per-level
    // launches instead
    void* vpass = nullptr;
    int vpass_state = 0, vpass_n = 0, vpass_grid = 0, vpass_smem = 0, vpass_whole = 0, vpass_cap = 0;
    double vpass_bytes = 0, vpass_bytes_alg = 0;
};

// Live timing of one kernel family (bench.py roofline): CUDA events around
// each launch whose name starts with `name`, on the context stream.
struct ProfState {
    std::string name;
    std::vector<cudaEvent_t> pool;
    std::vector<cudaEvent_t> pending;  // start/stop pairs
    int64_t launches = 0;
    // bytes: what the launches move by this implementation's own account;
    // bytes_alg: the compulsory bytes of the work they do (the per-cell
    // figures of the hot-path byte model: matrix coefficients, unknowns and
    // right-hand sides, nothing this implementation adds)
    double ms = 0, bytes = 0, bytes_alg = 0;
};

// The timestep as a CUDA graph: the global-iteration loop, the FGMRES restart
// loop and the Arnoldi loop are conditional WHILE nodes whose conditions the
// device sets, so one graph launch runs a whole timestep without the host.
// n_*: kernel launches per execution of each part (the launch count of a
// step follows from the loop trip counts the device reports).
struct GraphCtl {
    int gi;  // global iterations run by the graph in this step (a guard on the loop)
    int cap;
};
struct GraphState {
    int state = 0;  // 0 not built yet, 1 ready, -1 off (host-driven steps)
    int warm = 0;   // a host-driven step ran (lazy set-up done) before the capture
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t body[3] = {nullptr, nullptr, nullptr};
    GraphCtl* ctl = nullptr;
    int64_t n_top = 0, n_global = 0, n_restart = 0, n_inner = 0;
    std::string why;  // why the graph is off
};

struct hmec_inst {
    hmec_params p;
    int dev;
    cudaStream_t stream;
    Geo g;
    int64_t marknum;
    double* crd[8];          // x, y, xvx, yvx, xvy, yvy, xp, yp (Eigen LinSpaced)
    double* mk[HMEC_M_COUNT];
    double* f[HMEC_F_COUNT];
    // marker sort scratch
    int32_t* mkey;           // half-cell key per marker
    int32_t* perm;           // marker ids sorted by key
    int32_t* hc_count;       // markers per half-cell
    int32_t* hc_start;       // exclusive scan of hc_count (+ total)
    int32_t* hc_fill;        // scatter cursors
    int32_t* scan_part;      // scan block partials
    int* sort_long;          // set when a half cell holds more markers than the per-segment sort takes
    int32_t* mord;           // caller index of each stored marker (markers are stored in half-cell order)
    size_t stage_off = 0;    // floats of mprop before the marker transfers' staging
    cudaStream_t gs4[4] = {nullptr, nullptr, nullptr, nullptr};  // the four grids' gathers
    cudaEvent_t ev_g_fork = nullptr, ev_g_done[4] = {nullptr, nullptr, nullptr, nullptr};
    // hmec_stream_markers: the page-locked host marker arrays every timestep
    // copies in after its markers->nodes section, on a stream of its own
    const double* src_mk[HMEC_M_COUNT] = {};
    bool src_set = false;
    cudaStream_t up_stream = nullptr;
    cudaEvent_t ev_up_fork = nullptr, ev_up_done = nullptr;
    float* mprop;            // sorted per-marker gather records of the four grids (double-float)
    double* cellsum;         // per-cell corner sums of the four grids (k_cell_sums)
    int nhalf;               // number of half-cells
    // global system
    double* R;               // unscaled right-hand side
    double* S;               // solution (kept as the next initial guess)
    double* red;             // reduction partials
    unsigned* ticket;        // arrival counters of the one-launch reductions (zero between launches)
    DevScalars* ds;          // device scalars
    DevScalars* hs;          // pinned host mirror
    Solver sv;
    int64_t launches;
    ProfState prof;
    int in_step;             // between timestep_begin and timestep_end
    std::string err;
    GraphState gr;
    double* rowbuf = nullptr;  // row staging: 3 slots of 64 rows of Nx+1 (2 async, 1 sync)
    // hmec_download_rows_async: the copies' stream, the gather's event, each
    // slot's copy-done event and the ticket it last carried
    cudaStream_t rows_stream = nullptr;
    cudaEvent_t rows_ready = nullptr;
    cudaEvent_t rows_done[2] = {nullptr, nullptr};
    int64_t rows_ticket[2] = {0, 0};
    int64_t rows_last = 0;
    int bs_st = 64, bs_so = 256;  // threads per block: node-stencil kernels, marker kernels
};

// The ABI's context: n model instances -- one for a single model, the
// members of an ensemble otherwise -- each with its own grid, buffers and
// stream on the device current at hmec_create.  An ensemble step is one CUDA
// graph launch: every member's timestep (hmec_graph.cu) captured side by side
// into one graph, each with its own loops, dt and convergence decisions.
struct hmec_ctx {
    std::vector<hmec_inst*> inst;
    int dev = 0;
    std::string err;
    int gstate = 0;  // ensemble graph: 0 not built, 1 ready, -1 off (member graphs or host-driven steps)
    cudaStream_t origin = nullptr;
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev_join;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::string why;
};

// ------------------------------------------------------------------ helpers
#define DMIN(a, b) ((b) < (a) ? (b) : (a))
#define DMAX(a, b) ((a) < (b) ? (b) : (a))

__host__ __device__ __forceinline__ int fix_trunc(double t) { return t < 0. ? (int)ceil(t) : (int)floor(t); }
__host__ __device__ __forceinline__ int check_bounds(int k, int bound) {
    return k < 0 ? 0 : (k > bound - 2 ? bound - 2 : k);
}
__host__ __device__ __forceinline__ double divplus(double x, double y) { return x / (x + y); }

// fix(fl(x / d)) or fix(fl(fl(x + d/2) / d)) -- the reference's cell index of
// a marker coordinate, IEEE operations -- decided in FP32 wherever that is
// provably the same answer (FP64 arithmetic is the scarce resource here).
// x is truncated to a 24-bit mantissa through its bit pattern (relative
// error < 2^-23), rdf = 1/d in FP32 (< 2^-23), so q = x * rdf (+ 0.5) is
// within 3e-7 (|q| + 0.5) of the exact quotient.  If q is farther than
// 6e-7 (|q| + 1) from every integer, the FP64 quotient cannot round across
// one and trunc(q) is the index; otherwise (and for x outside the FP32
// range) the FP64 operations decide.
__device__ __forceinline__ int fix_quot(double x, double d, float rdf, bool half) {
    const int hi = __double2hiint(x);
    const unsigned lo = (unsigned)__double2loint(x);
    const int e = ((hi >> 20) & 0x7FF) - 896;  // biased FP32 exponent
    if (e > 0 && e < 255) {
        const float xf =
            __int_as_float((hi & (int)0x80000000) | (e << 23) | ((hi & 0xFFFFF) << 3) | (int)(lo >> 29));
        const float q = fmaf(xf, rdf, half ? 0.5f : 0.0f);
        const float aq = fabsf(q);
        if (aq < 8.0e6f) {
            const float t = truncf(q);
            const float fr = fabsf(q - t);
            const float m = 6.0e-7f * (aq + 1.0f);
            if (fr > m && fr < 1.0f - m) return (int)t;
        }
    }
    const double xx = half ? __dadd_rn(x, d / 2.) : x;
    return fix_trunc(__ddiv_rn(xx, d));
}
__device__ __forceinline__ float rcp_f32(double d) { return __frcp_rn(__double2float_rn(d)); }

__device__ __forceinline__ double to_f64(float f) { return f2d_bits(f); }
__device__ __forceinline__ double to_f64(double d) { return d; }

// A marker's basic cell (ib, jb) and pressure cell (iP, jP): the indices of
// cpp/h_mec_rsf_v9.cpp:432-433 and :468-469 (fix + check_bounds, IEEE
// quotients; the Vx/Vy cells reuse them), decided in FP32 away from cell edges.
struct MarkerCells {
    int ib, jb, iP, jP;
};
__device__ __forceinline__ MarkerCells marker_cells(double xm, double ym, const Geo& g) {
    MarkerCells c;
    const float rdx = rcp_f32(g.dx), rdy = rcp_f32(g.dy);
    c.jb = check_bounds(fix_quot(xm, g.dx, rdx, false), g.Nx);
    c.ib = check_bounds(fix_quot(ym, g.dy, rdy, false), g.Ny);
    c.jP = check_bounds(fix_quot(xm, g.dx, rdx, true), g.Nx);
    c.iP = check_bounds(fix_quot(ym, g.dy, rdy, true), g.Ny);
    return c;
}

// The geometry of an Nx x Ny basic grid over xsize x ysize, as
// cpp/constants.hpp derives it (dx, dy, line_fault :43, the block limits
// :76-77, faultwidth = dx :66), plus the reciprocal constants.
inline void geo_make(Geo& g, int Nx, int Ny, double xsize, double ysize) {
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
    geo_reciprocals(g);
}

static inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// One-launch two-level reduction: every block stores its partial (thread 0),
// then calls this; the last block to arrive gets true, sees every partial
// (read them with __ldcg) and has already reset the counter for the next
// launch.  Min / max / counts are order-independent, so the result equals a
// second kernel's.
__device__ __forceinline__ bool arrive_last(unsigned* ticket) {
    __shared__ unsigned s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    if (threadIdx.x == 0) *ticket = 0;
    return true;
}

// Launch bookkeeping: every kernel launch of the library goes through this.
#define HMEC_LAUNCH(ctx, kern, grid, block, smem, ...)                          \
    do {                                                                          \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);            \
        (ctx)->launches++;                                                        \
    } while (0)

int hmec_cuda_fail(hmec_inst* ctx, cudaError_t e, const char* what);
bool hmec_prof_begin(hmec_inst* ctx, const char* kname, double bytes, double bytes_alg);
void hmec_prof_end(hmec_inst* ctx);

// The library's launch helpers use ctx->stream; inside a scope they go to s.
struct StreamScope {
    hmec_inst* ctx;
    cudaStream_t saved;
    StreamScope(hmec_inst* c, cudaStream_t s) : ctx(c), saved(c->stream) { c->stream = s; }
    ~StreamScope() { ctx->stream = saved; }
};

// Launch with byte accounting for the live roofline (bytes moved by this
// implementation, compulsory bytes of the work).
#define HMEC_LAUNCH_B(ctx, nbytes, nalg, kern, grid, block, smem, ...)         \
    do {                                                                          \
        const bool _prof = hmec_prof_begin((ctx), #kern, (nbytes), (nalg));       \
        kern<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);            \
        (ctx)->launches++;                                                        \
        if (_prof) hmec_prof_end(ctx);                                            \
    } while (0)
#define HMEC_CUDA(ctx, call)                                                     \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) return hmec_cuda_fail((ctx), _e, #call);          \
    } while (0)

// Sections (implemented in the k_*.cu units); all return an hmec status.
int p2g_alloc(hmec_inst* ctx);
void p2g_free(hmec_inst* ctx);
int p2g_run(hmec_inst* ctx);
// Marker arrays in and out of the library's storage order (see k_p2g.cu).
int p2g_store_markers(hmec_inst* ctx, const double* const* fields);
// The marker stream of a timestep (hmec_stream_markers): issue forks the copy
// of the registered host arrays (and their sort into half-cell order) from
// the current stream after the markers->nodes section; join makes the
// current stream wait for it.  Both do nothing without registered arrays.
int markers_stream_issue(hmec_inst* ctx);
int markers_stream_join(hmec_inst* ctx);
int p2g_load_markers(hmec_inst* ctx, double* const* fields);
int iter_prepare(hmec_inst* ctx);
int iter_assemble(hmec_inst* ctx);
int iter_finish(hmec_inst* ctx);
int step_begin(hmec_inst* ctx);
int step_end(hmec_inst* ctx);
int advect_run(hmec_inst* ctx);
int solver_alloc(hmec_inst* ctx);
void solver_free(hmec_inst* ctx);
int solver_setup(hmec_inst* ctx);            // build coarse levels + Vanka inverses for the current matrix
int solver_solve(hmec_inst* ctx, int* iters, double* relres);  // solve A S = R in place (S = guess)
// Graph capture helpers (hmec_graph.cu): a conditional handle of the graph
// being captured on s; a WHILE node on handle h appended to that capture,
// whose body is captured on stream bs until graph_while_end(bs).
int graph_handle(hmec_inst* ctx, cudaStream_t s, cudaGraphConditionalHandle* h);
int graph_while_begin(hmec_inst* ctx, cudaStream_t s, cudaGraphConditionalHandle h, cudaStream_t bs);
int graph_while_end(hmec_inst* ctx, cudaStream_t bs);
// The solve with its decisions on the device, captured on ctx->stream (its
// restart loop's body on s_restart, the Arnoldi loop's on s_inner);
// *n_restart / *n_inner: kernel launches per trip of each loop.
int solver_capture_solve(hmec_inst* ctx, cudaStream_t s_restart, cudaStream_t s_inner, int64_t* n_restart,
                         int64_t* n_inner);
// One timestep as a graph launch (built on first use); *used is false when
// the graph is off for this context and the caller runs the host-driven step.
int graph_timestep(hmec_inst* ctx, hmec_step_report* rep, bool* used);
void graph_free(hmec_inst* ctx);
// The tuning table's entry for p's grid and form applied to p (hmec_tune.cu);
// 1 when one was applied.
int hmec_tune_apply(hmec_params* p);
// One timestep of every member of an ensemble as one graph launch (built on
// first use, once every member has run a host-driven step); *used false:
// the caller steps the members one by one.
int ensemble_graph_step(hmec_ctx* E, hmec_step_report* reps, bool* used);
void ensemble_graph_free(hmec_ctx* E);
// The report of a member's graph step from its device scalars (hs).
int graph_report(hmec_inst* ctx, hmec_step_report* rep);
// Assembly of one level into (col, val, dscale, rhs); rhs may be null.
void launch_assemble(hmec_inst* ctx, const Geo& g, const AsmFields& af, int32_t* col, double* val, double* dscale,
                     double* rhs_scaled, double* rhs_raw, const double* sc_dev);
