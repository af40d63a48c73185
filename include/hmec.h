/*
 * hmec.h -- C ABI of libhmec_gpu.so, the GB300 (sm_103a) implementation of the
 * per-timestep hot path of H-MEC (hydro-mechanical earthquake cycles, 2D).
 *
 * The reference program (cpp/h_mec_rsf_v9.cpp) has no functions on its hot
 * path: every section is inline in main() and its state lives in globals.
 * This header therefore defines the boundary section by section.  Each entry
 * point below names the reference lines it replaces; a host loop that mirrors
 * main() calls them in the same order (see driver/hmec_run.cpp).
 *
 * Conventions
 *   - Node fields are Eigen column-major double arrays: element (i, j) of a
 *     field with `rows` rows lives at [j * rows + i].  Basic-grid fields are
 *     Ny x Nx, staggered fields are (Ny+1) x (Nx+1), exactly as the reference
 *     declares them (cpp/h_mec_rsf_v9.cpp:54-89).  The pointer of an Eigen
 *     MatrixXd (`M.data()`) can be passed directly.
 *   - Host buffers are copied; the library never keeps a host pointer.
 *   - Every entry point returns an int status (HMEC_OK == 0, negative on
 *     error); no C++ exception crosses the ABI.  hmec_last_error() gives the
 *     message of the last failure on a context.
 *   - A context holds n model instances (n = 1: one model; n > 1: the
 *     members of an ensemble, each with its own grid).  Every data and
 *     section entry point names the instance `inst` it acts on; an instance
 *     holds the reference's global state of one model.
 *   - One host thread per context.  The context owns all device memory and
 *     one CUDA stream per instance on the device current at hmec_create().
 */
#ifndef HMEC_H
#define HMEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HMEC_ABI_VERSION 2

/* ------------------------------------------------------------------ status */
enum hmec_status {
    HMEC_OK = 0,
    HMEC_ERR_ARG = -1,           /* bad argument (null pointer, wrong size, unknown id) */
    HMEC_ERR_CUDA = -2,          /* a CUDA runtime call failed */
    HMEC_ERR_BOUNDS = -3,        /* a device-side index check failed */
    HMEC_ERR_NAN = -4,           /* a non-finite value in the solution */
    HMEC_ERR_RSF_NOCONV = -5,    /* the fault-stress bisection hit its iteration cap */
    HMEC_ERR_KRYLOV_NOCONV = -6, /* FGMRES did not reach its tolerance within its cap */
    HMEC_ERR_NOMEM = -7,         /* device allocation failed */
    HMEC_ERR_STATE = -8,         /* call out of order (e.g. iteration before timestep_begin) */
    HMEC_ERR_TIMEOUT = -9        /* a device-side wait hit its iteration cap */
};

/* ------------------------------------------------------------ solver forms */
enum hmec_form {
    HMEC_FORM_FP64 = 0,  /* FP64 FGMRES, FP64 multigrid preconditioner */
    HMEC_FORM_MIXED = 1  /* FP64 FGMRES, FP32 multigrid preconditioner  */
};

/*
 * Runtime parameters.  hmec_params_default() fills the values of
 * cpp/constants.hpp:13-146 (the reference compiles them in); derived
 * quantities (dx, line_fault, block limits, ...) are computed from these by
 * the library exactly as constants.hpp computes them.
 */
typedef struct hmec_params {
    /* grid, constants.hpp:23-26 */
    int32_t Nx, Ny;
    double xsize, ysize;
    /* markers per basic cell in x and y, constants.hpp:81-82 (4, 4) */
    int32_t mx, my;
    /* RSF transition abscissae, constants.hpp:29-33 */
    double TS_1, TS_2, TS_3, TS_4;
    /* time stepping, constants.hpp:71-74 */
    double dtelastic0, dtmin, inertia;
    /* RSF, constants.hpp:93-98: [0] block, [1] fault */
    double arsfm[2], brsfm[2], lrsfm[2], omm[2];
    double V0;
    double alpha;
    /* porosity / rheology, constants.hpp:101-111 */
    double POR0, cohes, friction, dilatation, tensile, shearmod, BETAFLUID, BETASOLID;
    /* body force / pressures, constants.hpp:115-118 */
    double gx, gy, PCONF, PTFDIFF;
    /* limits, constants.hpp:122-127 */
    double etamin, etamax, kkkmin, kkkmax, stpmax, stpmax1;
    /* boundary conditions, constants.hpp:130-132 */
    double bcupper, bclower, bcvyflower;
    /* iteration / timestep control, constants.hpp:135-146 */
    int32_t niterglobal, ynlastmax, dtstep;
    double vratiomax, dtkoef, dtkoefup, dtkoefv, errmin, etawt, syieldmin, tyield;
    int32_t num_timesteps;

    /* ---- extensions of this library (no counterpart in constants.hpp) ---- */
    int32_t form;             /* enum hmec_form */
    double krylov_rtol;       /* FGMRES tolerance on the row-equilibrated residual (1e-15);
                                 a restart cycle that gains less than 2x ends the solve,
                                 accepted when within 100x of it (FP64 rounding floor) */
    int32_t krylov_restart;   /* FGMRES restart length m */
    int32_t krylov_maxit;     /* total FGMRES iteration cap per solve */
    int32_t mg_levels;        /* max multigrid levels (1 = Vanka smoother only) */
    int32_t mg_pre, mg_post;  /* Vanka sweeps before / after the coarse correction */
    int32_t mg_coarse_sweeps; /* Vanka sweeps on the coarsest level */
    int32_t rsf_maxit;        /* cap of the fault-stress bisection (reference: none) */
    int32_t advect_markers;   /* 1: run marker advection (reference: loop never runs) */
    int32_t rk4_as_written;   /* 1: reproduce the shifted RK stages of the reference */
    int32_t quirk_accumulate_sums; /* oracle only: marker sums accumulate across steps */
    int32_t bounds_check;     /* 1: device index checks set HMEC_ERR_BOUNDS */
    int32_t mg_flags;         /* multigrid coarsening options, HMEC_MG_* bits */
    int32_t graph;            /* 1: hmec_timestep runs a whole step as one CUDA graph launch, its
                                 loops (global iterations, FGMRES restarts, Arnoldi steps) as
                                 conditional nodes decided on the device; 0: host-driven launches */
    /* launch shapes (0: the library's default) and the tuning table */
    int32_t bs_stencil;       /* threads per block of the node-stencil kernels (64) */
    int32_t bs_sort;          /* threads per block of the marker key, scatter and property kernels (256) */
    int32_t krylov_blocks;    /* blocks of the cooperative Arnoldi step (two per SM) */
    int32_t smooth_blocks;    /* most blocks of one smoothing launch (every co-resident block) */
    int32_t autotune;         /* 1: at hmec_create, take mg_levels, mg_pre, mg_post,
                                 mg_coarse_sweeps and the launch shapes above from the tuning
                                 table entry of this form nearest this grid (the table of
                                 hmec/tune.py: $HMEC_TUNE_TABLE, else tune_table.json beside the
                                 library's package), when there is one within 4x in cells */
    int32_t invariants_every; /* k > 1: the output-only fields of a17 (EII, EIIVP, SII, DIS,
                                 pt_ave, pf_ave, VIS_COMP, EL_DECOM) over the whole grid only on
                                 steps whose number is a multiple of k, on the other steps only
                                 their fault-line row (what the per-step EVO_*.txt series print);
                                 0 or 1: every step, as the reference (1) */
    int32_t smooth_inverses;  /* the staged smoothing pass's Vanka inverses: 1 a whole tile's
                                 staged with its rows, 2 one colour's at a time, double
                                 buffered (more blocks per SM), 0 the library's choice (1 when
                                 it fits in shared memory: FP32; else 2: FP64) */
} hmec_params;

/* mg_flags bits */
enum hmec_mg_flags {
    /* Darcy resistance eta_f/k of a coarse face: conductances averaged across
     * the flow direction (parallel paths), resistances along it (series);
     * otherwise plain arithmetic averages. */
    HMEC_MG_DARCY_HARMONIC = 1,
    /* Smooth each level with one grid-wide barrier per Vanka colour class
     * (a true multiplicative sweep over the whole level) instead of the
     * default tiled sweep (multiplicative inside 12x12-patch tiles, the
     * neighbours' unknowns taken from the start of the sweep). */
    HMEC_MG_UNTILED = 2,
    /* For models that share the GPU concurrently (ensembles): one
     * cooperative launch per smoothing pass instead of one per V-cycle (the
     * fused V-cycle holds its fine level's grid through the small coarse
     * levels too), and at most a quarter of the SMs per pass, so that
     * several models' passes run side by side. */
    HMEC_MG_PASS_LAUNCHES = 4,
    /* Local sweeps: a tile runs all the sweeps of a smoothing pass back to
     * back on one stage, its neighbours' unknowns taken from the start of the
     * pass (multiplicative inside a tile for every sweep, additive across
     * tile borders for the pass): one stage, one window load and one grid
     * barrier per pass instead of per sweep. */
    HMEC_MG_LOCAL_SWEEPS = 8
};

/* ------------------------------------------------------------- node fields */
/* X(name, grid): grid 0 = basic (Ny x Nx), 1 = staggered (Ny+1 x Nx+1).
 * Names are the reference's (cpp/h_mec_rsf_v9.cpp:55-112).                 */
#define HMEC_FIELD_LIST(X) \
    X(OM0, 0) X(OM, 0) X(OM5, 0) X(ARSF, 0) X(BRSF, 0) X(LRSF, 0) \
    X(RHO, 0) X(ETA, 0) X(ETA0, 0) X(ETA1, 0) X(ETA5, 0) X(ETA00, 0) X(ETA50, 0) \
    X(IETAPLB, 0) X(SXY, 0) X(SXY0, 0) X(YNY0, 0) X(YNY, 0) X(KKK, 0) X(GGG, 0) \
    X(COHC, 0) X(COHT, 0) X(FRIC, 0) X(FRIT, 0) X(DILC, 0) X(TTT, 0) X(EIIB, 0) \
    X(VSLIPB, 0) X(SIIB, 0) X(ESP, 0) X(EXY, 0) X(DSY, 0) X(SigmaY, 0) X(SII_fault, 0) \
    X(pt, 1) X(vxs, 1) X(vys, 1) X(pf, 1) X(vxD, 1) X(vyD, 1) \
    X(ETAB, 1) X(ETAB0, 1) X(ETAP, 1) X(ETAP0, 1) X(POR, 1) X(GGGP, 1) X(GGGB, 1) \
    X(PTF0, 1) X(PT0, 1) X(PF0, 1) X(SXX, 1) X(SXX0, 1) X(SYY, 1) X(SYY0, 1) \
    X(EXX, 1) X(EYY, 1) X(DILP, 1) \
    X(RHOX, 1) X(RHOFX, 1) X(ETADX, 1) X(PORX, 1) X(VX0, 1) X(VXF0, 1) \
    X(RHOY, 1) X(RHOFY, 1) X(ETADY, 1) X(PORY, 1) X(VY0, 1) X(VYF0, 1) \
    X(EII, 1) X(EIIVP, 1) X(SII, 1) X(DIS, 1) X(pt_ave, 1) X(pf_ave, 1) \
    X(VIS_COMP, 1) X(EL_DECOM, 1)

#define HMEC_X_ENUM(name, grid) HMEC_F_##name,
enum hmec_field { HMEC_FIELD_LIST(HMEC_X_ENUM) HMEC_F_COUNT };
#undef HMEC_X_ENUM

/* ----------------------------------------------------------- marker arrays */
/* The 19 per-marker arrays of cpp/constants.hpp:153-173 (VecXd, length marknum). */
#define HMEC_MARKER_LIST(X) \
    X(xm) X(ym) X(t_marker) X(rhom) X(etasm) X(etam) X(cohescm) X(cohestm) \
    X(frictcm) X(dilatcm) X(fricttm) X(porm) X(kkkm) X(sxxm) X(syym) X(sxym) \
    X(gm) X(rhofm) X(etafm)

#define HMEC_X_MENUM(name) HMEC_M_##name,
enum hmec_marker_field { HMEC_MARKER_LIST(HMEC_X_MENUM) HMEC_M_COUNT };
#undef HMEC_X_MENUM

/* ----------------------------------------------------------------- scalars */
/* Scalars of cpp/h_mec_rsf_v9.cpp:99-105 and the 9 restart values of :1862,
 * all exchanged as double.                                                  */
#define HMEC_SCALAR_LIST(X) \
    X(timesum) X(dt) X(dt00) X(dtx) X(dty) X(dtlapusta) X(Vmax) X(maxvxy) \
    X(yndtdecrease) X(timestep) X(ynlast) X(iterstep) \
    X(maxvxsmod) X(minvxsmod) X(maxvysmod) X(minvysmod)

#define HMEC_X_SENUM(name) HMEC_S_##name,
enum hmec_scalar { HMEC_SCALAR_LIST(HMEC_X_SENUM) HMEC_S_COUNT };
#undef HMEC_X_SENUM

/* ----------------------------------------------------------------- reports */
typedef struct hmec_iter_report {
    int32_t iterstep;      /* index of the global iteration just run */
    int32_t stop;          /* 1 if the exit test of :1436 passed */
    int32_t ynpl;          /* yielding fault nodes (:1277-1298) */
    int32_t krylov_iters;  /* FGMRES iterations of this solve */
    double dt;             /* dt after the adaptive-step logic of :1418-1427 */
    double DSYLSQ;         /* :1311-1314 */
    double ptscale, pfscale;
    double Vmax;
    double krylov_relres;  /* final row-equilibrated relative residual */
} hmec_iter_report;

typedef struct hmec_step_report {
    int32_t timestep;        /* the step just completed */
    int32_t global_iters;    /* iterstep + 1, as printed at :1736 */
    int32_t ynlast;          /* ynlast + 1, as printed at :1737 */
    int32_t krylov_iters;    /* FGMRES iterations summed over the step */
    int32_t status;          /* first non-OK status seen in the step */
    double timesum, dt, Vmax;
    double max_krylov_relres;
} hmec_step_report;

typedef struct hmec_ctx hmec_ctx;

/* ---------------------------------------------------------------- metadata */
int32_t hmec_abi_version(void);
/* Fill *p with the values of cpp/constants.hpp and the library defaults. */
void hmec_params_default(hmec_params* p);
const char* hmec_field_name(int32_t field);   /* NULL for an unknown id */
int32_t hmec_field_grid(int32_t field);        /* 0 basic, 1 staggered, -1 unknown */
const char* hmec_marker_name(int32_t field);
const char* hmec_scalar_name(int32_t id);
/* Marker count of the lattice: (Nx-1)*mx * (Ny-1)*my (constants.hpp:81-85). */
int64_t hmec_marknum(const hmec_params* p);
/* What hmec_create does with p->autotune set, without creating anything:
 * overwrite p's cycle shape and launch shapes with the tuning table's entry
 * for p's form nearest p's grid.  1 if an entry was applied, 0 if none (no
 * table, or none within 4x in cells).  No counterpart in the reference.     */
int32_t hmec_tune_params(hmec_params* p);

/* --------------------------------------------------------------- lifecycle */
/* The grid of one instance: the fields of hmec_params it overrides. */
typedef struct hmec_grid {
    int32_t Nx, Ny;
    double xsize, ysize;
    int32_t mx, my;
} hmec_grid;

/* Replaces the global declarations of cpp/h_mec_rsf_v9.cpp:54-112 and
 * constants.hpp:153-173, once per instance: allocates every node field,
 * marker array and solver buffer of n_instances models on the current
 * device.  grids[k] (NULL: p's grid for all) gives instance k its grid; the
 * other parameters are shared (per-instance friction, permeability and the
 * like are node fields and marker arrays, uploaded per instance).  An
 * ensemble (n_instances > 1) advances all its members with one
 * hmec_timestep() call, each member with its own adaptive dt, iteration
 * counts and convergence decisions.  Fields start at zero.  *status
 * receives the error code when NULL is returned.                            */
hmec_ctx* hmec_create(const hmec_params* p, int32_t n_instances, const hmec_grid* grids, int32_t* status);
void hmec_destroy(hmec_ctx* ctx);
int32_t hmec_instances(const hmec_ctx* ctx);
const char* hmec_last_error(const hmec_ctx* ctx);

/* ------------------------------------------------------------ data motion */
/* Marker arrays of instance inst: fields[k] points to the array of marker
 * field k (enum hmec_marker_field order), each of length n == hmec_marknum()
 * of the instance's grid.  Replaces the initialisation of :188-209 (and the
 * HDF5 reads of :245-251).                                                 */
int32_t hmec_upload_markers(hmec_ctx* ctx, int32_t inst, const double* const* fields, int64_t n);
int32_t hmec_download_markers(hmec_ctx* ctx, int32_t inst, double* const* fields, int64_t n);
/* One node field; rows/cols must match the field's grid. */
int32_t hmec_upload_field(hmec_ctx* ctx, int32_t inst, int32_t field, const double* colmajor, int32_t rows,
                          int32_t cols);
int32_t hmec_download_field(hmec_ctx* ctx, int32_t inst, int32_t field, double* colmajor, int32_t rows,
                            int32_t cols);
/* Row `row` of each of nfields node fields, gathered on the device and
 * copied back in one transfer: out receives the rows one after another, each
 * as long as its field's row (Nx basic, Nx+1 staggered).  The per-step
 * EVO_*.txt series print such rows of the fault line (:1751-1805); this
 * replaces downloading the whole fields.                                    */
int32_t hmec_download_rows(hmec_ctx* ctx, int32_t inst, int32_t row, int32_t nfields, const int32_t* fields,
                           double* out);
/* Several whole fields in one call (arrays[k] of field ids[k], each of its
 * field's shape as in hmec_upload_field): the copies are queued back to back
 * and waited for once -- a host that moves its state every step (the
 * reference's globals) saves a wait per field.                              */
int32_t hmec_upload_fields(hmec_ctx* ctx, int32_t inst, int32_t nfields, const int32_t* ids,
                           const double* const* arrays);
int32_t hmec_download_fields(hmec_ctx* ctx, int32_t inst, int32_t nfields, const int32_t* ids,
                             double* const* arrays);
/* hmec_download_rows without waiting for the copy: the rows are gathered
 * after the work queued so far (the host waits for that gather only) and
 * copied to `out` on a stream of their own, overlapped with the next
 * hmec_timestep.  *ticket names the copy; `out` must stay valid and unread
 * until hmec_rows_wait(ticket) returns.  With page-locked `out`
 * (hmec_host_alloc) the copy is asynchronous; with pageable memory this call
 * returns after the copy.  Two copies per instance can be in flight; a third
 * gather waits (on the device) for the oldest.  The reference writes the
 * fault rows synchronously every step (:1751-1805).                          */
int32_t hmec_download_rows_async(hmec_ctx* ctx, int32_t inst, int32_t row, int32_t nfields,
                                 const int32_t* fields, double* out, int64_t* ticket);
int32_t hmec_rows_wait(hmec_ctx* ctx, int32_t inst, int64_t ticket);
/* Marker streaming: registers the host's marker arrays (page-locked, e.g.
 * from hmec_host_alloc; fields[HMEC_M_COUNT], each n doubles long inside
 * its page-locked allocation, the layout of hmec_upload_markers) that every
 * later timestep copies into the device, in the caller's order, right after
 * its markers->nodes section, on a stream of its own, overlapped with the
 * rest of the step (the next step's sort orders them, as every step does).
 * So step k+1 uses what the arrays held while step k ran (the reference's
 * P2G reads its host marker arrays every step, :384-528).  The arrays must
 * stay valid and must not be written while a timestep runs.  fields = NULL
 * stops the streaming.  Refused with advect_markers (the device then moves
 * the markers itself).  The first step after a change runs host-driven and
 * the second captures the step's graph again.                               */
int32_t hmec_stream_markers(hmec_ctx* ctx, int32_t inst, const double* const* fields, int64_t n);
/* Page-locked host memory for hmec_download_rows_async (NULL on failure). */
void* hmec_host_alloc(size_t bytes);
void hmec_host_free(void* ptr);
int32_t hmec_set_scalar(hmec_ctx* ctx, int32_t inst, int32_t id, double value);
int32_t hmec_get_scalar(hmec_ctx* ctx, int32_t inst, int32_t id, double* value);

/* ---------------------------------------------------------------- sections */
/* a1-a4: marker properties, counting sort by cell, deterministic node
 * reductions and normalisation.  Replaces :376-583.                         */
int32_t hmec_markers_to_nodes(hmec_ctx* ctx, int32_t inst);
/* a5: viscosity reset, dt growth, iteration counters.  Replaces :585-608.   */
int32_t hmec_timestep_begin(hmec_ctx* ctx, int32_t inst);
/* a6-a15: one global (plastic) iteration -- viscosity limits, assembly,
 * FGMRES solve, reload, stress, fault RSF, error and adaptive dt, exit test
 * and viscosity update.  Replaces one pass of the loop body :611-1456.
 * report may be NULL.                                                        */
int32_t hmec_global_iteration(hmec_ctx* ctx, int32_t inst, hmec_iter_report* report);
/* a16-a19: dt recheck, post-step stress and invariants, state rollover.
 * Replaces :1463-1559 and :1658-1726 (advection excluded).                  */
int32_t hmec_timestep_end(hmec_ctx* ctx, int32_t inst);
/* a18, a20: node-to-marker velocity/spin gather, RK4 advection, stress
 * rotation, periodic recycling.  Replaces the (never executed) loop
 * :1561-1656.                                                               */
int32_t hmec_advect_markers(hmec_ctx* ctx, int32_t inst);
/* a1-a20 in order: one whole timestep of every instance, loop control on
 * the device.  Replaces the body of `for (; timestep <= num_timesteps; ...)`
 * up to the output section (:377-1726).  reports: NULL or an array of
 * hmec_instances() reports (one per instance).  With graph = 1 every step
 * after the first is one CUDA graph launch -- for an ensemble, one launch
 * for all members.  Returns the first non-OK status of any instance.        */
int32_t hmec_timestep(hmec_ctx* ctx, hmec_step_report* reports);

/* --------------------------------------------------------- testing hooks */
/* Assemble the global system of the current state (after the iteration
 * preparation of :611-677) and return it as CSR with duplicates summed, the
 * form Eigen's setFromTriplets produces at :1046-1049.  With indptr == NULL
 * only *nnz is returned.  rhs receives R (length N).                        */
int32_t hmec_assemble_csr(hmec_ctx* ctx, int32_t inst, int64_t* indptr, int32_t* indices, double* data,
                          double* rhs, int64_t* nnz, double* ptscale, double* pfscale);
/* Solve the system assembled by the last hmec_assemble_csr / iteration with
 * the configured solver for the given right-hand side; x holds the initial
 * guess on entry and the solution on return.                                 */
int32_t hmec_solve_system(hmec_ctx* ctx, int32_t inst, const double* rhs, double* x, int32_t* iters,
                          double* relres);
/* The CUDA stream (cudaStream_t) instance inst launches on, for timing with
 * CUDA events (no counterpart in the reference). */
void* hmec_stream(hmec_ctx* ctx, int32_t inst);
/* Time every launch of the kernel family whose name starts with `name`
 * (NULL: stop) with CUDA events on the context stream, and accumulate the
 * bytes those launches move; read and reset with hmec_profile_read():
 * *bytes_compulsory is the compulsory traffic of the work done (per cell:
 * the 42 matrix coefficients and the vectors a sweep or a Krylov step must
 * touch), *bytes_moved what this implementation moves by its own account
 * (stored patch inverses, column offsets, padding included).  Used by the
 * benchmark's live roofline (no counterpart in the reference).             */
int32_t hmec_profile_kernel(hmec_ctx* ctx, int32_t inst, const char* name);
int32_t hmec_profile_read(hmec_ctx* ctx, int32_t inst, int64_t* launches, double* total_ms,
                          double* bytes_compulsory, double* bytes_moved);
/* Markers -> nodes without allocating device memory.  No counterpart in the
 * reference: it serves hosts that may not call cudaMalloc (an application
 * that owns the device allocator, a real-time loop that must not block on
 * the allocator).  Computes the same
 * 23 node fields as hmec_markers_to_nodes() from arrays the caller already
 * holds on the current device: markers[k] is the device array of marker
 * field k (enum hmec_marker_field), fields[f] the column-major device array
 * of node field f (entries of fields that are not outputs may be NULL).
 * Scratch memory is one fixed array compiled into the library, about 25 MiB
 * of device memory; hence the limits: at most HMEC_NOALLOC_MAX_MARKERS =
 * 1048576 markers and 4*(Nx-1)*(Ny-1) <= HMEC_NOALLOC_MAX_HALF_CELLS =
 * 262144, larger inputs return HMEC_ERR_ARG.  The driver reserves the array
 * when it loads the library's device code on a device and keeps it until the
 * process exits; under lazy module loading (the CUDA default) that happens
 * in the first call on the device, which can then fail if the host's own
 * allocator has already taken the device's memory -- make one call early, or
 * set CUDA_MODULE_LOADING=EAGER.  Kernels go to `stream` (a cudaStream_t;
 * NULL = legacy default stream).  The first call on a device (and the first
 * after a device reset) looks up the array's device address, so make it
 * before any stream capture.  All calls share the array, which keeps the
 * last call's contents: calls that overlap on the GPU race, serialise them. */
int32_t hmec_markers_to_nodes_noalloc(const hmec_params* p, const double* const* markers, int64_t n,
                                      double* const* fields, void* stream);
/* The library's marker cell index on n host coordinates x[k] (copied to the
 * current device and back): out[k] = fix(fl(x/d)) (half = 0) or
 * fix(fl(fl(x + d/2) / d)) (half != 0), IEEE operations as in
 * cpp/h_mec_rsf_v9.cpp:432-433 and :468-469, before the clamp to the grid.
 * The kernels decide most indices in FP32 and fall back to FP64 division
 * near cell edges; this entry exposes that rule so it can be checked
 * bit-exactly (no counterpart in the reference).                           */
int32_t hmec_cell_index(const double* x, int64_t n, double d, int32_t half, int32_t* out);
/* How hmec_timestep runs on this context (no counterpart in the reference):
 * 1 = each step is one CUDA graph launch (for an ensemble: one launch for all
 * members), 0 = host-driven launches so far (the first step, or while a
 * kernel is profiled), -1 = host-driven for good (graph = 0, or the capture
 * failed; hmec_last_error() then gives why).                                */
int32_t hmec_graph_status(hmec_ctx* ctx);
/* Device-kernel launches of all instances since hmec_create (kernels run by
 * a graph launch included). */
int64_t hmec_kernel_launches(const hmec_ctx* ctx);
/* Synchronise every instance's stream. */
int32_t hmec_synchronize(hmec_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* HMEC_H */
