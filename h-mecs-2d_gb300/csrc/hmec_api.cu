// hmec_api.cu -- the extern "C" boundary of libhmec_gpu.so (include/hmec.h).
//
// Lifecycle, host<->device transfers of Eigen column-major storage, and the
// section entry points that a host loop mirroring cpp/h_mec_rsf_v9.cpp:main
// calls in place of the inline sections.  No exception crosses the ABI;
// every function returns an hmec status and records a message on the
// context.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "hmec_internal.cuh"

int hmec_cuda_fail(hmec_inst* ctx, cudaError_t e, const char* what) {
    if (ctx) {
        char buf[512];
        snprintf(buf, sizeof(buf), "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
        ctx->err = buf;
    }
    return HMEC_ERR_CUDA;
}

bool hmec_prof_begin(hmec_inst* ctx, const char* kname, double bytes, double bytes_alg) {
    ProfState& P = ctx->prof;
    while (*kname == '(' || *kname == ' ') kname++;  // template launches are parenthesised
    if (P.name.empty() || strncmp(kname, P.name.c_str(), P.name.size()) != 0) return false;
    for (int k = 0; k < 2; k++) {
        cudaEvent_t e;
        if (P.pool.empty()) {
            if (cudaEventCreate(&e) != cudaSuccess) return false;
        } else {
            e = P.pool.back();
            P.pool.pop_back();
        }
        P.pending.push_back(e);
    }
    cudaEventRecord(P.pending[P.pending.size() - 2], ctx->stream);
    P.launches++;
    P.bytes += bytes;
    P.bytes_alg += bytes_alg;
    return true;
}

void hmec_prof_end(hmec_inst* ctx) { cudaEventRecord(ctx->prof.pending.back(), ctx->stream); }

static void prof_drain(hmec_inst* ctx) {
    ProfState& P = ctx->prof;
    if (P.pending.empty()) return;
    cudaStreamSynchronize(ctx->stream);
    for (size_t k = 0; k + 1 < P.pending.size(); k += 2) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, P.pending[k], P.pending[k + 1]) == cudaSuccess) P.ms += ms;
        P.pool.push_back(P.pending[k]);
        P.pool.push_back(P.pending[k + 1]);
    }
    P.pending.clear();
}

static int fail(hmec_inst* ctx, int code, const char* msg) {
    if (ctx) ctx->err = msg;
    return code;
}

// Eigen 3.3 LinSpaced(n, low, high) for |high| >= |low| (every grid here).
static void linspaced(std::vector<double>& out, int n, double low, double high) {
    out.resize(n);
    const double step = (n == 1) ? 0. : (high - low) / (double)(n - 1);
    for (int i = 0; i < n; i++) out[i] = (i == n - 1) ? high : low + (double)i * step;
}

// Row `row` of nf fields into consecutive slots of out (a field's row has
// cols[k] entries; the column-major field has rows[k] rows).
struct RowGather {
    const double* f[64];
    int rows[64], cols[64], off[64];
};
__global__ void k_gather_rows(RowGather g, int nf, int row, double* out) {
    const int k = blockIdx.y;
    if (k >= nf) return;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < g.cols[k]; j += gridDim.x * blockDim.x)
        out[g.off[k] + j] = g.f[k][(size_t)j * g.rows[k] + row];
}

// Map device status bits to the ABI status.
static int status_from_bits(int bits) {
    if (bits & HMEC_DEV_BOUNDS) return HMEC_ERR_BOUNDS;
    if (bits & HMEC_DEV_NAN) return HMEC_ERR_NAN;
    if (bits & HMEC_DEV_RSF_NOCONV) return HMEC_ERR_RSF_NOCONV;
    if (bits & HMEC_DEV_KRYLOV_NOCONV) return HMEC_ERR_KRYLOV_NOCONV;
    if (bits & HMEC_DEV_TIMEOUT) return HMEC_ERR_TIMEOUT;
    return HMEC_OK;
}

static int pull_scalars(hmec_inst* ctx) {
    HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->hs, ctx->ds, sizeof(DevScalars), cudaMemcpyDeviceToHost, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->prof.pending.size() > 4096) prof_drain(ctx);
    return HMEC_OK;
}

extern "C" {

int32_t hmec_abi_version(void) { return HMEC_ABI_VERSION; }

void hmec_params_default(hmec_params* p) {
    if (!p) return;
    // cpp/constants.hpp:13-146
    memset(p, 0, sizeof(*p));
    p->Nx = 401;
    p->Ny = 51;
    p->xsize = 40000.;
    p->ysize = 10000.;
    p->mx = 4;
    p->my = 4;
    p->TS_1 = 2e3;
    p->TS_2 = 4e3;
    p->TS_3 = 34e3;
    p->TS_4 = 38e3;
    p->dtelastic0 = 5e8;
    p->dtmin = 1e-4;
    p->inertia = 1.;
    p->arsfm[0] = .025;
    p->arsfm[1] = .006;
    p->brsfm[0] = .001;
    p->brsfm[1] = .015;
    p->lrsfm[0] = .020;
    p->lrsfm[1] = .0085;
    p->omm[0] = 10;
    p->omm[1] = -10;
    p->V0 = 1.e-9;
    p->alpha = 29;
    p->POR0 = .01;
    p->cohes = 0.;
    p->friction = .6;
    p->dilatation = 0.;
    p->tensile = 1.;
    p->shearmod = 3.e10;
    p->BETAFLUID = 1.e-8;
    p->BETASOLID = 2.e-11;
    p->gx = 0.;
    p->gy = 0.;
    p->PCONF = 1.e7;
    p->PTFDIFF = 3.e7;
    p->etamin = 1e-3;
    p->etamax = 1e50;
    p->kkkmin = 1e-22;
    p->kkkmax = 1e-12;
    p->stpmax = 2e-4;
    p->stpmax1 = 6e-5;
    p->bcupper = -1e-9;
    p->bclower = 1e-9;
    p->bcvyflower = 0;
    p->niterglobal = 10000;
    p->ynlastmax = 499;
    p->dtstep = 5;
    p->vratiomax = 0.001;
    p->dtkoef = 1.1;
    p->dtkoefup = 1.2;
    p->dtkoefv = 1.001;
    p->errmin = 1e2;
    p->etawt = 0.0;
    p->syieldmin = 1e-3;
    p->tyield = 1;
    p->num_timesteps = 100000;
    // library extensions
    p->form = HMEC_FORM_FP64;
    p->krylov_rtol = 1e-15;
    p->krylov_restart = 40;
    p->krylov_maxit = 2000;
    p->mg_levels = 5;
    p->mg_pre = 2;
    p->mg_post = 2;
    p->mg_coarse_sweeps = 8;
    p->rsf_maxit = 10000;
    p->advect_markers = 0;
    p->rk4_as_written = 0;
    p->quirk_accumulate_sums = 0;
    p->bounds_check = 0;
    p->mg_flags = 1; /* HMEC_MG_DARCY_HARMONIC */
    p->graph = 1;
    p->autotune = 1;
    p->invariants_every = 1;
}

#define HMEC_X_NAME(name, grid) #name,
#define HMEC_X_GRID(name, grid) grid,
static const char* const kFieldNames[] = {HMEC_FIELD_LIST(HMEC_X_NAME)};
static const int kFieldGrid[] = {HMEC_FIELD_LIST(HMEC_X_GRID)};
#undef HMEC_X_NAME
#undef HMEC_X_GRID
#define HMEC_X_NAME1(name) #name,
static const char* const kMarkerNames[] = {HMEC_MARKER_LIST(HMEC_X_NAME1)};
static const char* const kScalarNames[] = {HMEC_SCALAR_LIST(HMEC_X_NAME1)};
#undef HMEC_X_NAME1

const char* hmec_field_name(int32_t f) { return (f >= 0 && f < HMEC_F_COUNT) ? kFieldNames[f] : nullptr; }
int32_t hmec_field_grid(int32_t f) { return (f >= 0 && f < HMEC_F_COUNT) ? kFieldGrid[f] : -1; }
const char* hmec_marker_name(int32_t f) { return (f >= 0 && f < HMEC_M_COUNT) ? kMarkerNames[f] : nullptr; }
const char* hmec_scalar_name(int32_t s) { return (s >= 0 && s < HMEC_S_COUNT) ? kScalarNames[s] : nullptr; }

int64_t hmec_marknum(const hmec_params* p) {
    if (!p) return -1;
    return (int64_t)(p->Nx - 1) * p->mx * (int64_t)(p->Ny - 1) * p->my;
}

}  // extern "C"

static const char* inst_last_error(const hmec_inst* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

static int64_t inst_kernel_launches(const hmec_inst* ctx) { return ctx ? ctx->launches : -1; }

static int32_t inst_graph_status(hmec_inst* ctx) {
    if (!ctx) return -1;
    if (!ctx->p.graph) return -1;
    if (ctx->gr.state < 0) {
        ctx->err = ctx->gr.why.empty() ? "graph capture failed" : ctx->gr.why;
        return -1;
    }
    return ctx->gr.state == 1 ? 1 : 0;
}

static void inst_destroy(hmec_inst* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->dev);
    cudaStreamSynchronize(ctx->stream);
    for (cudaEvent_t e : ctx->prof.pool) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->prof.pending) cudaEventDestroy(e);
    graph_free(ctx);
    solver_free(ctx);
    p2g_free(ctx);
    for (int k = 0; k < 8; k++) cudaFree(ctx->crd[k]);
    for (int k = 0; k < HMEC_M_COUNT; k++) cudaFree(ctx->mk[k]);
    for (int k = 0; k < HMEC_F_COUNT; k++) cudaFree(ctx->f[k]);
    cudaFree(ctx->R);
    cudaFree(ctx->S);
    cudaFree(ctx->red);
    cudaFree(ctx->ticket);
    cudaFree(ctx->ds);
    if (ctx->rows_stream) {
        cudaStreamSynchronize(ctx->rows_stream);
        cudaStreamDestroy(ctx->rows_stream);
        cudaEventDestroy(ctx->rows_ready);
        for (auto e : ctx->rows_done) cudaEventDestroy(e);
    }
    cudaFree(ctx->rowbuf);
    cudaFreeHost(ctx->hs);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

// Parameter checks made before any device work; the reason, or NULL.
static const char* params_problem(const hmec_params& p) {
    if (p.Nx < 5 || p.Ny < 5 || p.mx < 1 || p.my < 1 || !(p.xsize > 0) || !(p.ysize > 0))
        return "grid parameters out of range (Nx, Ny >= 5; mx, my >= 1; sizes > 0)";
    if (p.krylov_restart < 2 || p.krylov_restart > 200) return "krylov_restart must be in [2, 200]";
    if (p.form != HMEC_FORM_FP64 && p.form != HMEC_FORM_MIXED) return "unknown solver form";
    if (p.invariants_every < 0) return "invariants_every must be >= 0";
    if (p.smooth_inverses < 0 || p.smooth_inverses > 2) return "smooth_inverses must be 0, 1 or 2";
    return nullptr;
}

// A block size from a tuned value: a multiple of 32 in [32, 1024], or dflt.
static int block_size(int v, int dflt) {
    if (v <= 0) return dflt;
    v = (v + 31) / 32 * 32;
    return v < 32 ? 32 : (v > 1024 ? 1024 : v);
}

static int create_inner(hmec_inst* ctx) {
    const hmec_params& p = ctx->p;
    if (const char* why = params_problem(p)) return fail(ctx, HMEC_ERR_ARG, why);
    ctx->bs_st = block_size(p.bs_stencil, 64);
    ctx->bs_so = block_size(p.bs_sort, 256);
    HMEC_CUDA(ctx, cudaGetDevice(&ctx->dev));
    HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    Geo& g = ctx->g;
    geo_make(g, p.Nx, p.Ny, p.xsize, p.ysize);
    ctx->marknum = hmec_marknum(&p);
    // coordinates, constants.hpp:57-64
    std::vector<double> c[8];
    const double dx = g.dx, dy = g.dy;
    linspaced(c[0], p.Nx, 0, p.xsize);
    linspaced(c[1], p.Ny, 0, p.ysize);
    linspaced(c[2], p.Nx + 1, 0, p.xsize + dx);
    linspaced(c[3], p.Ny + 1, 0 - dy / 2., p.ysize + dy / 2.);
    linspaced(c[4], p.Nx + 1, 0 - dx / 2., p.xsize + dx / 2.);
    linspaced(c[5], p.Ny + 1, 0, p.ysize + dy);
    linspaced(c[6], p.Nx + 1, 0 - dx / 2., p.xsize + dx / 2.);
    linspaced(c[7], p.Ny + 1, 0 - dy / 2., p.ysize + dy / 2.);
    for (int k = 0; k < 8; k++) {
        HMEC_CUDA(ctx, cudaMalloc(&ctx->crd[k], sizeof(double) * c[k].size()));
        HMEC_CUDA(ctx, cudaMemcpy(ctx->crd[k], c[k].data(), sizeof(double) * c[k].size(), cudaMemcpyHostToDevice));
    }
    const size_t nb = (size_t)g.Nx * g.Ny, ns = (size_t)g.Nx1 * g.Ny1;
    for (int k = 0; k < HMEC_F_COUNT; k++) {
        const size_t n = hmec_field_grid(k) ? ns : nb;
        HMEC_CUDA(ctx, cudaMalloc(&ctx->f[k], sizeof(double) * n));
        HMEC_CUDA(ctx, cudaMemset(ctx->f[k], 0, sizeof(double) * n));
    }
    for (int k = 0; k < HMEC_M_COUNT; k++) {
        HMEC_CUDA(ctx, cudaMalloc(&ctx->mk[k], sizeof(double) * (size_t)ctx->marknum));
        HMEC_CUDA(ctx, cudaMemset(ctx->mk[k], 0, sizeof(double) * (size_t)ctx->marknum));
    }
    HMEC_CUDA(ctx, cudaMalloc(&ctx->R, sizeof(double) * (size_t)g.N));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->S, sizeof(double) * (size_t)g.N));
    HMEC_CUDA(ctx, cudaMemset(ctx->S, 0, sizeof(double) * (size_t)g.N));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->red, sizeof(double) * (4096 + 3 * (size_t)g.Nx + 64)));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->ticket, sizeof(unsigned) * 8));
    HMEC_CUDA(ctx, cudaMemset(ctx->ticket, 0, sizeof(unsigned) * 8));
    HMEC_CUDA(ctx, cudaMalloc(&ctx->ds, sizeof(DevScalars)));
    HMEC_CUDA(ctx, cudaMallocHost(&ctx->hs, sizeof(DevScalars)));
    DevScalars s;
    memset(&s, 0, sizeof(s));
    s.dt = p.dtelastic0;  // h_mec_rsf_v9.cpp:101-103
    s.yndtdecrease = 1;
    s.timestep = 1;
    HMEC_CUDA(ctx, cudaMemcpy(ctx->ds, &s, sizeof(s), cudaMemcpyHostToDevice));
    *ctx->hs = s;
    int rc = p2g_alloc(ctx);
    if (rc) return rc;
    rc = solver_alloc(ctx);
    if (rc) return rc;
    HMEC_CUDA(ctx, cudaDeviceSynchronize());
    return HMEC_OK;
}

static hmec_inst* inst_create(const hmec_params* p, int32_t* status) {
    if (!p) {
        if (status) *status = HMEC_ERR_ARG;
        return nullptr;
    }
    hmec_inst* ctx = new (std::nothrow) hmec_inst();
    if (!ctx) {
        if (status) *status = HMEC_ERR_NOMEM;
        return nullptr;
    }
    ctx->p = *p;
    ctx->launches = 0;
    ctx->in_step = 0;
    int rc = create_inner(ctx);
    if (rc != HMEC_OK) {
        fprintf(stderr, "inst_create: %s\n", ctx->err.c_str());
        if (status) *status = rc;
        if (ctx->stream) inst_destroy(ctx);
        else delete ctx;
        return nullptr;
    }
    if (status) *status = HMEC_OK;
    return ctx;
}

static int32_t inst_upload_markers(hmec_inst* ctx, const double* const* fields, int64_t n) {
    if (!ctx || !fields) return fail(ctx, HMEC_ERR_ARG, "null argument");
    if (n != ctx->marknum) return fail(ctx, HMEC_ERR_ARG, "marker count differs from (Nx-1)*mx*(Ny-1)*my");
    for (int k = 0; k < HMEC_M_COUNT; k++)
        if (!fields[k]) return fail(ctx, HMEC_ERR_ARG, "null marker array");
    int rc = p2g_store_markers(ctx, fields);
    if (rc) return rc;
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

// Registers (fields set) or drops (fields NULL) the host marker arrays that
// every timestep copies in after its markers->nodes section.  They must be
// page-locked, since the copies run asynchronously and inside the timestep's
// graph (whose capture the registration invalidates).
static int32_t inst_stream_markers(hmec_inst* ctx, const double* const* fields, int64_t n) {
    if (!ctx) return HMEC_ERR_ARG;
    if (fields) {
        if (n != ctx->marknum) return fail(ctx, HMEC_ERR_ARG, "marker count differs from (Nx-1)*mx*(Ny-1)*my");
        if (ctx->p.advect_markers)
            return fail(ctx, HMEC_ERR_STATE, "marker streaming replaces the markers the advection moves");
        for (int k = 0; k < HMEC_M_COUNT; k++) {
            if (!fields[k]) return fail(ctx, HMEC_ERR_ARG, "null marker array");
            // the first and the last element in page-locked memory (the
            // copies run while the caller's thread goes on)
            for (const double* q : {fields[k], fields[k] + (n - 1)}) {
                cudaPointerAttributes at;
                if (cudaPointerGetAttributes(&at, q) != cudaSuccess || at.type != cudaMemoryTypeHost) {
                    cudaGetLastError();
                    return fail(ctx, HMEC_ERR_ARG, "streamed marker arrays must be page-locked (hmec_host_alloc)");
                }
            }
        }
        for (int k = 0; k < HMEC_M_COUNT; k++) ctx->src_mk[k] = fields[k];
    }
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->src_set = fields != nullptr;
    graph_free(ctx);  // the captured copies name the arrays: capture again
    return HMEC_OK;
}

static int32_t inst_download_markers(hmec_inst* ctx, double* const* fields, int64_t n) {
    if (!ctx || !fields) return fail(ctx, HMEC_ERR_ARG, "null argument");
    if (n != ctx->marknum) return fail(ctx, HMEC_ERR_ARG, "marker count differs from (Nx-1)*mx*(Ny-1)*my");
    int rc = p2g_load_markers(ctx, fields);
    if (rc) return rc;
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

static int field_dims_ok(hmec_inst* ctx, int32_t f, int32_t rows, int32_t cols) {
    if (f < 0 || f >= HMEC_F_COUNT) return 0;
    const int g = hmec_field_grid(f);
    return rows == ctx->g.Ny + g && cols == ctx->g.Nx + g;
}

static int32_t inst_upload_field(hmec_inst* ctx, int32_t f, const double* a, int32_t rows, int32_t cols) {
    if (!ctx || !a) return fail(ctx, HMEC_ERR_ARG, "null argument");
    if (!field_dims_ok(ctx, f, rows, cols)) return fail(ctx, HMEC_ERR_ARG, "unknown field or wrong dimensions");
    HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->f[f], a, sizeof(double) * (size_t)rows * cols, cudaMemcpyHostToDevice, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

// Several fields in one call: the copies queued back to back, one wait.
static int32_t inst_move_fields(hmec_inst* ctx, int32_t nf, const int32_t* ids, double* const* ptrs, bool up) {
    if (!ctx || (nf > 0 && (!ids || !ptrs))) return fail(ctx, HMEC_ERR_ARG, "null argument");
    for (int k = 0; k < nf; k++)
        if (ids[k] < 0 || ids[k] >= HMEC_F_COUNT || !ptrs[k]) return fail(ctx, HMEC_ERR_ARG, "unknown field or null array");
    for (int k = 0; k < nf; k++) {
        const int gr = hmec_field_grid(ids[k]);
        const size_t bytes = sizeof(double) * (size_t)(ctx->g.Ny + gr) * (ctx->g.Nx + gr);
        if (up)
            HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->f[ids[k]], ptrs[k], bytes, cudaMemcpyHostToDevice, ctx->stream));
        else
            HMEC_CUDA(ctx, cudaMemcpyAsync(ptrs[k], ctx->f[ids[k]], bytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

static int32_t inst_download_field(hmec_inst* ctx, int32_t f, double* a, int32_t rows, int32_t cols) {
    if (!ctx || !a) return fail(ctx, HMEC_ERR_ARG, "null argument");
    if (!field_dims_ok(ctx, f, rows, cols)) return fail(ctx, HMEC_ERR_ARG, "unknown field or wrong dimensions");
    HMEC_CUDA(ctx, cudaMemcpyAsync(a, ctx->f[f], sizeof(double) * (size_t)rows * cols, cudaMemcpyDeviceToHost, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

// The gather of hmec_download_rows: checks the fields and the row, fills g,
// and returns the doubles the rows take (0 on an argument error).
static int rows_gather(hmec_inst* ctx, int32_t row, int32_t nf, const int32_t* fields, RowGather* g) {
    if (nf < 1 || nf > 64) return fail(ctx, HMEC_ERR_ARG, "nfields must be in [1, 64]"), 0;
    int total = 0;
    for (int k = 0; k < nf; k++) {
        const int f = fields[k];
        if (f < 0 || f >= HMEC_F_COUNT) return fail(ctx, HMEC_ERR_ARG, "unknown field"), 0;
        const int gr = hmec_field_grid(f);
        g->f[k] = ctx->f[f];
        g->rows[k] = ctx->g.Ny + gr;
        g->cols[k] = ctx->g.Nx + gr;
        g->off[k] = total;
        total += g->cols[k];
        if (row < 0 || row >= g->rows[k]) return fail(ctx, HMEC_ERR_ARG, "row outside the field"), 0;
    }
    return total;
}

static int rows_slots(hmec_inst* ctx) {
    if (!ctx->rowbuf) HMEC_CUDA(ctx, cudaMalloc(&ctx->rowbuf, sizeof(double) * 3 * 64 * (size_t)(ctx->g.Nx + 1)));
    return HMEC_OK;
}

static int32_t inst_download_rows(hmec_inst* ctx, int32_t row, int32_t nf, const int32_t* fields, double* out) {
    if (!ctx || !fields || !out) return fail(ctx, HMEC_ERR_ARG, "null argument");
    RowGather g;
    const int total = rows_gather(ctx, row, nf, fields, &g);
    if (!total) return HMEC_ERR_ARG;
    if (int rc = rows_slots(ctx)) return rc;
    // slot 2: slots 0 and 1 belong to the asynchronous copies
    double* buf = ctx->rowbuf + (size_t)2 * 64 * (size_t)(ctx->g.Nx + 1);
    HMEC_LAUNCH(ctx, k_gather_rows, dim3(nblocks(ctx->g.Nx + 1, 128), nf), 128, 0, g, nf, row, buf);
    HMEC_CUDA(ctx, cudaMemcpyAsync(out, buf, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

// The rows are gathered on the instance's stream into one of two device
// slots; the host waits for the gather only (a few microseconds), so that
// the next step may write the fields, and the copy to `out` runs on the
// rows stream, overlapped with that step.  A slot is gathered into again only
// after its previous copy is done (a wait queued on the instance's stream).
static int32_t inst_download_rows_async(hmec_inst* ctx, int32_t row, int32_t nf, const int32_t* fields, double* out,
                                        int64_t* ticket) {
    if (!ctx || !fields || !out || !ticket) return fail(ctx, HMEC_ERR_ARG, "null argument");
    RowGather g;
    const int total = rows_gather(ctx, row, nf, fields, &g);
    if (!total) return HMEC_ERR_ARG;
    if (int rc = rows_slots(ctx)) return rc;
    if (!ctx->rows_stream) {
        HMEC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->rows_stream, cudaStreamNonBlocking));
        HMEC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->rows_ready, cudaEventDisableTiming));
        for (auto& e : ctx->rows_done) HMEC_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const int slot = (int)(ctx->rows_last & 1);
    double* buf = ctx->rowbuf + (size_t)slot * 64 * (size_t)(ctx->g.Nx + 1);
    HMEC_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->rows_done[slot], 0));
    HMEC_LAUNCH(ctx, k_gather_rows, dim3(nblocks(ctx->g.Nx + 1, 128), nf), 128, 0, g, nf, row, buf);
    HMEC_CUDA(ctx, cudaEventRecord(ctx->rows_ready, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamWaitEvent(ctx->rows_stream, ctx->rows_ready, 0));
    HMEC_CUDA(ctx, cudaMemcpyAsync(out, buf, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost,
                                   ctx->rows_stream));
    HMEC_CUDA(ctx, cudaEventRecord(ctx->rows_done[slot], ctx->rows_stream));
    HMEC_CUDA(ctx, cudaEventSynchronize(ctx->rows_ready));
    ctx->rows_ticket[slot] = ++ctx->rows_last;
    *ticket = ctx->rows_last;
    return HMEC_OK;
}

// Waits for the copy of `ticket`: its slot's last copy is that one or a
// later one, which the stream order puts after it.
static int32_t inst_rows_wait(hmec_inst* ctx, int64_t ticket) {
    if (!ctx) return HMEC_ERR_ARG;
    if (ticket < 1 || ticket > ctx->rows_last) return fail(ctx, HMEC_ERR_ARG, "unknown rows ticket");
    HMEC_CUDA(ctx, cudaEventSynchronize(ctx->rows_done[(ticket - 1) & 1]));
    return HMEC_OK;
}

// Scalars: the host mirror is refreshed from the device, edited, pushed back.
static int32_t inst_set_scalar(hmec_inst* ctx, int32_t id, double v) {
    if (!ctx) return HMEC_ERR_ARG;
    if (id < 0 || id >= HMEC_S_COUNT) return fail(ctx, HMEC_ERR_ARG, "unknown scalar id");
    int rc = pull_scalars(ctx);
    if (rc) return rc;
    DevScalars& s = *ctx->hs;
    switch (id) {
        case HMEC_S_timesum: s.timesum = v; break;
        case HMEC_S_dt: s.dt = v; break;
        case HMEC_S_dt00: s.dt00 = v; break;
        case HMEC_S_dtx: s.dtx = v; break;
        case HMEC_S_dty: s.dty = v; break;
        case HMEC_S_dtlapusta: s.dtlapusta = v; break;
        case HMEC_S_Vmax: s.Vmax = v; break;
        case HMEC_S_maxvxy: s.maxvxy = v; break;
        case HMEC_S_yndtdecrease: s.yndtdecrease = (int)v; break;
        case HMEC_S_timestep: s.timestep = (int)v; break;
        case HMEC_S_ynlast: s.ynlast = (int)v; break;
        case HMEC_S_iterstep: s.iterstep = (int)v; break;
        case HMEC_S_maxvxsmod: s.maxvxsmod = v; break;
        case HMEC_S_minvxsmod: s.minvxsmod = v; break;
        case HMEC_S_maxvysmod: s.maxvysmod = v; break;
        case HMEC_S_minvysmod: s.minvysmod = v; break;
    }
    HMEC_CUDA(ctx, cudaMemcpyAsync(ctx->ds, ctx->hs, sizeof(DevScalars), cudaMemcpyHostToDevice, ctx->stream));
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

static int32_t inst_get_scalar(hmec_inst* ctx, int32_t id, double* v) {
    if (!ctx || !v) return fail(ctx, HMEC_ERR_ARG, "null argument");
    if (id < 0 || id >= HMEC_S_COUNT) return fail(ctx, HMEC_ERR_ARG, "unknown scalar id");
    int rc = pull_scalars(ctx);
    if (rc) return rc;
    const DevScalars& s = *ctx->hs;
    switch (id) {
        case HMEC_S_timesum: *v = s.timesum; break;
        case HMEC_S_dt: *v = s.dt; break;
        case HMEC_S_dt00: *v = s.dt00; break;
        case HMEC_S_dtx: *v = s.dtx; break;
        case HMEC_S_dty: *v = s.dty; break;
        case HMEC_S_dtlapusta: *v = s.dtlapusta; break;
        case HMEC_S_Vmax: *v = s.Vmax; break;
        case HMEC_S_maxvxy: *v = s.maxvxy; break;
        case HMEC_S_yndtdecrease: *v = s.yndtdecrease; break;
        case HMEC_S_timestep: *v = s.timestep; break;
        case HMEC_S_ynlast: *v = s.ynlast; break;
        case HMEC_S_iterstep: *v = s.iterstep; break;
        case HMEC_S_maxvxsmod: *v = s.maxvxsmod; break;
        case HMEC_S_minvxsmod: *v = s.minvxsmod; break;
        case HMEC_S_maxvysmod: *v = s.maxvysmod; break;
        case HMEC_S_minvysmod: *v = s.minvysmod; break;
    }
    return HMEC_OK;
}

static void* inst_stream(hmec_inst* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

static int32_t inst_profile_kernel(hmec_inst* ctx, const char* name) {
    if (!ctx) return HMEC_ERR_ARG;
    prof_drain(ctx);
    ctx->prof.name = name ? name : "";
    ctx->prof.launches = 0;
    ctx->prof.ms = 0;
    ctx->prof.bytes = 0;
    ctx->prof.bytes_alg = 0;
    return HMEC_OK;
}

static int32_t inst_profile_read(hmec_inst* ctx, int64_t* launches, double* total_ms, double* bytes_compulsory,
                          double* bytes_moved) {
    if (!ctx) return HMEC_ERR_ARG;
    prof_drain(ctx);
    if (launches) *launches = ctx->prof.launches;
    if (total_ms) *total_ms = ctx->prof.ms;
    if (bytes_compulsory) *bytes_compulsory = ctx->prof.bytes_alg;
    if (bytes_moved) *bytes_moved = ctx->prof.bytes;
    return HMEC_OK;
}

static int32_t inst_synchronize(hmec_inst* ctx) {
    if (!ctx) return HMEC_ERR_ARG;
    HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HMEC_OK;
}

static int32_t inst_markers_to_nodes(hmec_inst* ctx) {
    if (!ctx) return HMEC_ERR_ARG;
    // a new timestep starts here: clear the device status word of the last one
    HMEC_CUDA(ctx, cudaMemsetAsync(&ctx->ds->status, 0, sizeof(int), ctx->stream));
    int rc = p2g_run(ctx);
    if (rc) return rc;
    return HMEC_OK;
}

static int32_t inst_timestep_begin(hmec_inst* ctx) {
    if (!ctx) return HMEC_ERR_ARG;
    int rc = step_begin(ctx);
    if (rc) return rc;
    ctx->in_step = 1;
    return HMEC_OK;
}

static int iteration(hmec_inst* ctx, hmec_iter_report* rep, int* krylov_rc) {
    int rc = iter_prepare(ctx);
    if (rc) return rc;
    rc = iter_assemble(ctx);
    if (rc) return rc;
    rc = solver_setup(ctx);
    if (rc) return rc;
    int its = 0;
    double rel = 0;
    *krylov_rc = solver_solve(ctx, &its, &rel);
    if (*krylov_rc != HMEC_OK && *krylov_rc != HMEC_ERR_KRYLOV_NOCONV) return *krylov_rc;
    rc = iter_finish(ctx);
    if (rc) return rc;
    rc = pull_scalars(ctx);
    if (rc) return rc;
    const DevScalars& s = *ctx->hs;
    if (rep) {
        rep->iterstep = s.stop ? s.iterstep : s.iterstep - 1;
        rep->stop = s.stop;
        rep->ynpl = s.ynpl;
        rep->krylov_iters = its;
        rep->dt = s.dt;
        rep->DSYLSQ = s.dsylsq;
        rep->ptscale = s.ptscale;
        rep->pfscale = s.pfscale;
        rep->Vmax = s.Vmax;
        rep->krylov_relres = rel;
    }
    return HMEC_OK;
}

static int32_t inst_global_iteration(hmec_inst* ctx, hmec_iter_report* rep) {
    if (!ctx) return HMEC_ERR_ARG;
    if (!ctx->in_step) return fail(ctx, HMEC_ERR_STATE, "inst_global_iteration before inst_timestep_begin");
    int krc = HMEC_OK;
    int rc = iteration(ctx, rep, &krc);
    if (rc) return rc;
    const int bits = ctx->hs->status;
    if (bits) return fail(ctx, status_from_bits(bits), "device status raised in the global iteration");
    if (krc) return fail(ctx, krc, "FGMRES did not reach krylov_rtol within krylov_maxit");
    return HMEC_OK;
}

static int32_t inst_timestep_end(hmec_inst* ctx) {
    if (!ctx) return HMEC_ERR_ARG;
    int rc = step_end(ctx);
    if (rc) return rc;
    ctx->in_step = 0;
    rc = pull_scalars(ctx);
    if (rc) return rc;
    return HMEC_OK;
}

static int32_t inst_advect_markers(hmec_inst* ctx) {
    if (!ctx) return HMEC_ERR_ARG;
    return advect_run(ctx);
}

static int32_t inst_timestep(hmec_inst* ctx, hmec_step_report* rep) {
    if (!ctx) return HMEC_ERR_ARG;
    bool by_graph = false;
    int rc = graph_timestep(ctx, rep, &by_graph);
    if (by_graph) return rc;
    if (rc) return rc;
    rc = inst_markers_to_nodes(ctx);
    if (rc) return rc;
    rc = markers_stream_issue(ctx);
    if (rc) return rc;
    rc = inst_timestep_begin(ctx);
    if (rc) return rc;
    int first_bad = HMEC_OK;
    int ktot = 0;
    double kmax = 0;
    for (;;) {
        hmec_iter_report ir;
        int krc = HMEC_OK;
        rc = iteration(ctx, &ir, &krc);
        if (rc) return rc;
        ktot += ir.krylov_iters;
        kmax = std::fmax(kmax, ir.krylov_relres);
        if (krc && !first_bad) first_bad = krc;
        if (ctx->hs->loop_done) break;
        if (ctx->hs->status & HMEC_DEV_NAN) {  // a non-finite solution cannot recover
            first_bad = HMEC_ERR_NAN;
            break;
        }
    }
    const int iters = ctx->hs->iters_in_step;
    const int ynlast = ctx->hs->ynlast;
    const int timestep = ctx->hs->timestep;
    rc = inst_timestep_end(ctx);
    if (rc) return rc;
    if (ctx->p.advect_markers) {
        rc = advect_run(ctx);
        if (rc) return rc;
        rc = pull_scalars(ctx);
        if (rc) return rc;
    }
    if (ctx->src_set) {
        rc = markers_stream_join(ctx);
        if (rc) return rc;
        HMEC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    const int bits = ctx->hs->status;
    if (bits && !first_bad) first_bad = status_from_bits(bits);
    if (rep) {
        rep->timestep = timestep;
        rep->global_iters = iters;
        rep->ynlast = ynlast + 1;
        rep->krylov_iters = ktot;
        rep->status = first_bad;
        rep->timesum = ctx->hs->timesum;
        rep->dt = ctx->hs->dt;
        rep->Vmax = ctx->hs->Vmax;
        rep->max_krylov_relres = kmax;
    }
    ctx->gr.warm = 1;  // the lazy set-up is done: later steps may run as a graph
    if (first_bad) return fail(ctx, first_bad, "timestep finished with a non-OK status (see report)");
    return HMEC_OK;
}

static int32_t inst_assemble_csr(hmec_inst* ctx, int64_t* indptr, int32_t* indices, double* data, double* rhs, int64_t* nnz,
                          double* ptscale, double* pfscale) {
    if (!ctx || !nnz) return fail(ctx, HMEC_ERR_ARG, "null argument");
    int rc = iter_prepare(ctx);
    if (rc) return rc;
    rc = iter_assemble(ctx);
    if (rc) return rc;
    const Level& L = ctx->sv.lv[0];
    const size_t N = (size_t)ctx->g.N;
    std::vector<int32_t> col(HMEC_W * N);
    std::vector<double> val(HMEC_W * N), ds(N);
    HMEC_CUDA(ctx, cudaMemcpyAsync(col.data(), L.col, sizeof(int32_t) * col.size(), cudaMemcpyDeviceToHost, ctx->stream));
    HMEC_CUDA(ctx, cudaMemcpyAsync(val.data(), L.val, sizeof(double) * val.size(), cudaMemcpyDeviceToHost, ctx->stream));
    HMEC_CUDA(ctx, cudaMemcpyAsync(ds.data(), L.dscale, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    if (rhs) HMEC_CUDA(ctx, cudaMemcpyAsync(rhs, ctx->R, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    rc = pull_scalars(ctx);
    if (rc) return rc;
    if (ptscale) *ptscale = ctx->hs->ptscale;
    if (pfscale) *pfscale = ctx->hs->pfscale;
    // ELL -> CSR: drop the padding slots (column == row with value 0 after the real entries)
    int64_t k = 0;
    for (size_t r = 0; r < N; r++) {
        if (indptr) indptr[r] = k;
        for (int s = 0; s < HMEC_W; s++) {
            const size_t o = (size_t)s * N + r;
            const bool pad = (s > 0 && col[o] == (int32_t)r && val[o] == 0.0 && col[o - N] >= (int32_t)r);
            if (pad) continue;
            if (indptr) {
                indices[k] = col[o];
                data[k] = val[o] / ds[r];  // power-of-two scale: exact
            }
            k++;
        }
    }
    if (indptr) indptr[N] = k;
    *nnz = k;
    return HMEC_OK;
}

static int32_t inst_solve_system(hmec_inst* ctx, const double* rhs, double* x, int32_t* iters, double* relres) {
    if (!ctx || !rhs || !x) return fail(ctx, HMEC_ERR_ARG, "null argument");
    const size_t N = (size_t)ctx->g.N;
    Level& L = ctx->sv.lv[0];
    std::vector<double> ds(N), bs(N);
    HMEC_CUDA(ctx, cudaMemcpy(ds.data(), L.dscale, sizeof(double) * N, cudaMemcpyDeviceToHost));
    for (size_t r = 0; r < N; r++) bs[r] = rhs[r] * ds[r];
    HMEC_CUDA(ctx, cudaMemcpy(L.db, bs.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    HMEC_CUDA(ctx, cudaMemcpy(ctx->S, x, sizeof(double) * N, cudaMemcpyHostToDevice));
    int rc = solver_setup(ctx);
    if (rc) return rc;
    int its = 0;
    double rel = 0;
    int krc = solver_solve(ctx, &its, &rel);
    HMEC_CUDA(ctx, cudaMemcpy(x, ctx->S, sizeof(double) * N, cudaMemcpyDeviceToHost));
    if (iters) *iters = its;
    if (relres) *relres = rel;
    if (krc) return fail(ctx, krc, "FGMRES did not reach krylov_rtol within krylov_maxit");
    return HMEC_OK;
}



// ===================================================================== ABI
// The context holds n instances; every data and section entry point names
// the instance it acts on.  A failure's message is kept on the instance and
// copied to the context, where hmec_last_error() reads it.

static hmec_inst* inst_of(hmec_ctx* E, int32_t i) {
    if (!E) return nullptr;
    if (i < 0 || i >= (int32_t)E->inst.size()) {
        E->err = "instance index out of range";
        return nullptr;
    }
    return E->inst[i];
}

static int32_t relay(hmec_ctx* E, hmec_inst* m, int32_t rc) {
    if (rc != HMEC_OK) E->err = m->err;
    return rc;
}

#define HMEC_INST(E, i)                                   \
    hmec_inst* m_ = inst_of((E), (i));                    \
    if (!m_) return HMEC_ERR_ARG

extern "C" {

hmec_ctx* hmec_create(const hmec_params* p, int32_t n_instances, const hmec_grid* grids, int32_t* status) {
    if (!p || n_instances < 1) {
        if (status) *status = HMEC_ERR_ARG;
        return nullptr;
    }
    hmec_ctx* E = new (std::nothrow) hmec_ctx();
    if (!E) {
        if (status) *status = HMEC_ERR_NOMEM;
        return nullptr;
    }
    std::vector<hmec_params> qs(n_instances, *p);
    for (int32_t k = 0; k < n_instances; k++) {
        hmec_params& q = qs[k];
        if (grids) {
            q.Nx = grids[k].Nx;
            q.Ny = grids[k].Ny;
            q.xsize = grids[k].xsize;
            q.ysize = grids[k].ysize;
            q.mx = grids[k].mx;
            q.my = grids[k].my;
        }
        // members of an ensemble share the GPU: one launch per smoothing
        // pass on a share of the SMs (HMEC_MG_PASS_LAUNCHES)
        if (n_instances > 1) q.mg_flags |= HMEC_MG_PASS_LAUNCHES;
        if (q.autotune) {
            // the table's smoothing grid is a single model's; ensemble members
            // keep theirs (the quarter of the SMs per pass, or the caller's)
            const int32_t sb = q.smooth_blocks;
            hmec_tune_apply(&q);
            if (n_instances > 1) q.smooth_blocks = sb;
        }
        if (const char* why = params_problem(q)) {
            fprintf(stderr, "hmec_create: instance %d: %s\n", (int)k, why);
            delete E;
            if (status) *status = HMEC_ERR_ARG;
            return nullptr;
        }
    }
    cudaGetDevice(&E->dev);
    for (int32_t k = 0; k < n_instances; k++) {
        int32_t st = HMEC_OK;
        hmec_inst* m = inst_create(&qs[k], &st);
        if (!m) {
            for (hmec_inst* x : E->inst) inst_destroy(x);
            delete E;
            if (status) *status = st;
            return nullptr;
        }
        E->inst.push_back(m);
    }
    if (status) *status = HMEC_OK;
    return E;
}

void hmec_destroy(hmec_ctx* E) {
    if (!E) return;
    cudaSetDevice(E->dev);
    if (E->origin) cudaStreamSynchronize(E->origin);
    ensemble_graph_free(E);
    for (hmec_inst* m : E->inst) inst_destroy(m);
    delete E;
}

int32_t hmec_instances(const hmec_ctx* E) { return E ? (int32_t)E->inst.size() : 0; }

const char* hmec_last_error(const hmec_ctx* E) { return E ? E->err.c_str() : "null context"; }

int64_t hmec_kernel_launches(const hmec_ctx* E) {
    if (!E) return -1;
    int64_t t = 0;
    for (hmec_inst* m : E->inst) t += inst_kernel_launches(m);
    return t;
}

int32_t hmec_graph_status(hmec_ctx* E) {
    if (!E) return -1;
    if (E->inst.size() > 1) {
        if (E->gstate < 0) {
            E->err = E->why.empty() ? "ensemble graph capture failed" : E->why;
            return -1;
        }
        if (!E->inst[0]->p.graph) return -1;
        return E->gstate == 1 ? 1 : 0;
    }
    const int32_t r = inst_graph_status(E->inst[0]);
    if (r < 0) E->err = E->inst[0]->err;
    return r;
}

int32_t hmec_upload_markers(hmec_ctx* E, int32_t i, const double* const* fields, int64_t n) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_upload_markers(m_, fields, n));
}
int32_t hmec_download_markers(hmec_ctx* E, int32_t i, double* const* fields, int64_t n) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_download_markers(m_, fields, n));
}
int32_t hmec_upload_field(hmec_ctx* E, int32_t i, int32_t f, const double* a, int32_t rows, int32_t cols) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_upload_field(m_, f, a, rows, cols));
}
int32_t hmec_download_field(hmec_ctx* E, int32_t i, int32_t f, double* a, int32_t rows, int32_t cols) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_download_field(m_, f, a, rows, cols));
}
int32_t hmec_download_rows(hmec_ctx* E, int32_t i, int32_t row, int32_t nf, const int32_t* fields, double* out) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_download_rows(m_, row, nf, fields, out));
}
int32_t hmec_upload_fields(hmec_ctx* E, int32_t i, int32_t nfields, const int32_t* ids, const double* const* arrays) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_move_fields(m_, nfields, ids, const_cast<double* const*>(arrays), true));
}
int32_t hmec_download_fields(hmec_ctx* E, int32_t i, int32_t nfields, const int32_t* ids, double* const* arrays) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_move_fields(m_, nfields, ids, arrays, false));
}
int32_t hmec_stream_markers(hmec_ctx* E, int32_t i, const double* const* fields, int64_t n) {
    HMEC_INST(E, i);
    if (E->exec) {  // an ensemble graph holds the members' captures: build it again
        ensemble_graph_free(E);
        if (E->gstate > 0) E->gstate = 0;
    }
    return relay(E, m_, inst_stream_markers(m_, fields, n));
}
int32_t hmec_download_rows_async(hmec_ctx* E, int32_t i, int32_t row, int32_t nf, const int32_t* fields, double* out,
                                 int64_t* ticket) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_download_rows_async(m_, row, nf, fields, out, ticket));
}
int32_t hmec_rows_wait(hmec_ctx* E, int32_t i, int64_t ticket) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_rows_wait(m_, ticket));
}
void* hmec_host_alloc(size_t bytes) {
    void* p = nullptr;
    return cudaMallocHost(&p, bytes ? bytes : 1) == cudaSuccess ? p : nullptr;
}
void hmec_host_free(void* p) {
    if (p) cudaFreeHost(p);
}
int32_t hmec_set_scalar(hmec_ctx* E, int32_t i, int32_t id, double v) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_set_scalar(m_, id, v));
}
int32_t hmec_get_scalar(hmec_ctx* E, int32_t i, int32_t id, double* v) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_get_scalar(m_, id, v));
}
void* hmec_stream(hmec_ctx* E, int32_t i) {
    hmec_inst* m = inst_of(E, i);
    return m ? inst_stream(m) : nullptr;
}
int32_t hmec_profile_kernel(hmec_ctx* E, int32_t i, const char* name) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_profile_kernel(m_, name));
}
int32_t hmec_profile_read(hmec_ctx* E, int32_t i, int64_t* launches, double* total_ms, double* bytes_compulsory,
                          double* bytes_moved) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_profile_read(m_, launches, total_ms, bytes_compulsory, bytes_moved));
}
int32_t hmec_synchronize(hmec_ctx* E) {
    if (!E) return HMEC_ERR_ARG;
    if (E->origin) cudaStreamSynchronize(E->origin);
    for (hmec_inst* m : E->inst) {
        const int32_t rc = inst_synchronize(m);
        if (rc) return relay(E, m, rc);
    }
    return HMEC_OK;
}
int32_t hmec_markers_to_nodes(hmec_ctx* E, int32_t i) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_markers_to_nodes(m_));
}
int32_t hmec_timestep_begin(hmec_ctx* E, int32_t i) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_timestep_begin(m_));
}
int32_t hmec_global_iteration(hmec_ctx* E, int32_t i, hmec_iter_report* rep) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_global_iteration(m_, rep));
}
int32_t hmec_timestep_end(hmec_ctx* E, int32_t i) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_timestep_end(m_));
}
int32_t hmec_advect_markers(hmec_ctx* E, int32_t i) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_advect_markers(m_));
}

int32_t hmec_timestep(hmec_ctx* E, hmec_step_report* reports) {
    if (!E) return HMEC_ERR_ARG;
    if (E->inst.size() == 1) return relay(E, E->inst[0], inst_timestep(E->inst[0], reports));
    bool used = false;
    const int32_t rc = ensemble_graph_step(E, reports, &used);
    if (used) return rc;
    // members one by one (the first step of each, or graphs off)
    int32_t first_bad = HMEC_OK;
    for (size_t k = 0; k < E->inst.size(); k++) {
        const int32_t r = inst_timestep(E->inst[k], reports ? &reports[k] : nullptr);
        if (r && !first_bad) {
            first_bad = r;
            E->err = E->inst[k]->err;
        }
    }
    return first_bad;
}

int32_t hmec_assemble_csr(hmec_ctx* E, int32_t i, int64_t* indptr, int32_t* indices, double* data, double* rhs,
                          int64_t* nnz, double* ptscale, double* pfscale) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_assemble_csr(m_, indptr, indices, data, rhs, nnz, ptscale, pfscale));
}
int32_t hmec_solve_system(hmec_ctx* E, int32_t i, const double* rhs, double* x, int32_t* iters, double* relres) {
    HMEC_INST(E, i);
    return relay(E, m_, inst_solve_system(m_, rhs, x, iters, relres));
}

}  // extern "C"
