// checkpoint.hpp -- checkpoint and restart files of the host loop, in the
// reference's layout (cpp/h_mec_rsf_v9.cpp:211-282 read, :1807-1870 write).
//
// One file per saved step, `nname + timestep + ".h5"`: group /Matrix with 24
// basic-grid (Ny x Nx) and 30 staggered (Ny1 x Nx1) node fields, group /Vector
// with six per-timestep histories (num_timesteps) and five marker arrays
// (marknum), group /Value with nine scalars; matrices in C order (row i of
// the dataset is grid row i, cpp/hdf5.cpp:46-51).  The names, their order,
// the shapes and the byte order are the file format, so they are the
// reference's.  With H5Cpp.h present the file is HDF5; otherwise (as here) a
// stub container with the same groups, names, shapes and C-order FP64 bytes,
// the layout h-mecs-2d_gb300/hmec/checkpoint.py reads and writes too:
//
//   "HMECH5S1", u32 count, per dataset: u16 + group, u16 + name, u8 rank,
//   rank x u64 dims, then the values as f64 (little endian)
//
// The reference copies each dataset through a stack array (cpp/hdf5.cpp:46,
// :74, :107, :138), which overflows for large grids or marker counts; these
// buffers are on the heap.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hmec.h"

namespace ckpt {

// /Matrix (:1826-1841), /Vector (:1844-1857), /Value (:1860-1863)
static const char* const MATRIX_BASIC[24] = {"SIIB", "OM0", "OM", "ARSF", "BRSF", "LRSF", "RHO", "ETA0",
                                             "ETA1", "ETA5", "ETA00", "IETAPLB", "SXY0", "YNY0", "KKK", "GGG",
                                             "COHC", "COHT", "FRIC", "FRIT", "DILC", "TTT", "EIIB", "VSLIPB"};
static const char* const MATRIX_STAGGERED[30] = {
    "pt", "vxs", "vys", "pf", "vxD", "vyD", "ETAB", "ETAB0", "ETAP", "ETAP0", "POR", "GGGP", "GGGB", "PTF0", "PT0",
    "PF0", "SXX0", "SYY0", "RHOX", "RHOFX", "ETADX", "PORX", "VX0", "VXF0", "RHOY", "RHOFY", "ETADY", "PORY", "VY0",
    "VYF0"};
static const char* const HISTORY[6] = {"timesumcur", "dtcur", "maxvxsmod", "minvxsmod", "maxvysmod", "minvysmod"};
static const char* const MARKERS[5] = {"xm", "ym", "sxxm", "syym", "sxym"};
static const char* const VALUES[9] = {"timesum", "dt00", "dtx", "dty", "dtlapusta", "Vmax", "maxvxy", "dt",
                                      "yndtdecrease"};

struct Dataset {
    std::string group, name;
    std::vector<uint64_t> dims;
    std::vector<double> v;  // C order
};

inline int field_id(const char* name) {
    for (int f = 0; f < HMEC_F_COUNT; f++)
        if (!strcmp(hmec_field_name(f), name)) return f;
    return -1;
}
inline int marker_id(const char* name) {
    for (int k = 0; k < HMEC_M_COUNT; k++)
        if (!strcmp(hmec_marker_name(k), name)) return k;
    return -1;
}
inline int scalar_id(const char* name) {
    for (int s = 0; s < HMEC_S_COUNT; s++)
        if (!strcmp(hmec_scalar_name(s), name)) return s;
    return -1;
}

// The six histories the host loop keeps (:1658-1696), one entry per step.
struct History {
    std::vector<std::vector<double>> v;
    explicit History(int num_timesteps) : v(6, std::vector<double>((size_t)num_timesteps, 0.0)) {}
    // after step `timestep` (1-based) has run: index timestep - 1
    void record(hmec_ctx* ctx, int timestep, int32_t inst = 0) {
        const size_t t = (size_t)(timestep - 1);
        if (t >= v[0].size()) return;
        const char* src[6] = {"timesum", "dt", "maxvxsmod", "minvxsmod", "maxvysmod", "minvysmod"};
        for (int k = 0; k < 6; k++) hmec_get_scalar(ctx, inst, scalar_id(src[k]), &v[k][t]);
    }
};

// The checkpoint of the context's state after a step, in write order.
inline int collect(hmec_ctx* ctx, const hmec_params& p, const History& h, std::vector<Dataset>& out,
                   int32_t inst = 0) {
    const int Ny = p.Ny, Nx = p.Nx, Ny1 = Ny + 1, Nx1 = Nx + 1;
    std::vector<double> colmajor;
    auto matrix = [&](const char* name, int rows, int cols) {
        Dataset d{"Matrix", name, {(uint64_t)rows, (uint64_t)cols}, std::vector<double>((size_t)rows * cols)};
        colmajor.resize((size_t)rows * cols);
        const int rc = hmec_download_field(ctx, inst, field_id(name), colmajor.data(), rows, cols);
        for (int i = 0; i < rows; i++)  // data(i, j) -> out[i][j]
            for (int j = 0; j < cols; j++) d.v[(size_t)i * cols + j] = colmajor[(size_t)j * rows + i];
        out.push_back(std::move(d));
        return rc;
    };
    for (const char* n : MATRIX_BASIC)
        if (int rc = matrix(n, Ny, Nx)) return rc;
    for (const char* n : MATRIX_STAGGERED)
        if (int rc = matrix(n, Ny1, Nx1)) return rc;
    for (int k = 0; k < 6; k++) out.push_back({"Vector", HISTORY[k], {(uint64_t)h.v[k].size()}, h.v[k]});
    const int64_t n = hmec_marknum(&p);
    std::vector<std::vector<double>> mk(HMEC_M_COUNT, std::vector<double>((size_t)n));
    std::vector<double*> mp(HMEC_M_COUNT);
    for (int k = 0; k < HMEC_M_COUNT; k++) mp[k] = mk[k].data();
    if (int rc = hmec_download_markers(ctx, inst, mp.data(), n)) return rc;
    for (const char* m : MARKERS) out.push_back({"Vector", m, {(uint64_t)n}, mk[marker_id(m)]});
    Dataset vals{"Value", "values", {9}, std::vector<double>(9)};
    for (int k = 0; k < 9; k++) hmec_get_scalar(ctx, inst, scalar_id(VALUES[k]), &vals.v[k]);
    out.push_back(std::move(vals));
    return HMEC_OK;
}

// ------------------------------------------------------------ stub container
inline bool write_stub(const std::string& path, const std::vector<Dataset>& ds) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    bool ok = fwrite("HMECH5S1", 1, 8, f) == 8;
    const uint32_t count = (uint32_t)ds.size();
    ok = ok && fwrite(&count, 4, 1, f) == 1;
    for (const Dataset& d : ds) {
        for (const std::string* s : {&d.group, &d.name}) {
            const uint16_t len = (uint16_t)s->size();
            ok = ok && fwrite(&len, 2, 1, f) == 1 && fwrite(s->data(), 1, len, f) == len;
        }
        const uint8_t rank = (uint8_t)d.dims.size();
        ok = ok && fwrite(&rank, 1, 1, f) == 1 && fwrite(d.dims.data(), 8, rank, f) == rank;
        ok = ok && fwrite(d.v.data(), 8, d.v.size(), f) == d.v.size();
    }
    return fclose(f) == 0 && ok;
}

inline bool read_stub(const std::string& path, std::vector<Dataset>& ds) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    char magic[8];
    uint32_t count = 0;
    bool ok = fread(magic, 1, 8, f) == 8 && !memcmp(magic, "HMECH5S1", 8) && fread(&count, 4, 1, f) == 1;
    for (uint32_t c = 0; ok && c < count; c++) {
        Dataset d;
        for (std::string* s : {&d.group, &d.name}) {
            uint16_t len = 0;
            ok = ok && fread(&len, 2, 1, f) == 1;
            s->resize(len);
            ok = ok && fread(&(*s)[0], 1, len, f) == len;
        }
        uint8_t rank = 0;
        ok = ok && fread(&rank, 1, 1, f) == 1;
        d.dims.resize(rank);
        ok = ok && fread(d.dims.data(), 8, rank, f) == rank;
        uint64_t n = 1;
        for (uint64_t x : d.dims) n *= x;
        d.v.resize(n);
        ok = ok && fread(d.v.data(), 8, n, f) == n;
        ds.push_back(std::move(d));
    }
    fclose(f);
    return ok;
}

inline const Dataset* find(const std::vector<Dataset>& ds, const char* group, const char* name) {
    for (const Dataset& d : ds)
        if (d.group == group && d.name == name) return &d;
    return nullptr;
}

// Restart as :211-282: every dataset into the context (the markers' other
// arrays keep what the context holds -- the reference rebuilds them from its
// lattice first), the histories into h, and the step counter past `timestep`.
inline int restore(hmec_ctx* ctx, const hmec_params& p, const std::vector<Dataset>& ds, int timestep, History& h,
                   int32_t inst = 0) {
    const int Ny = p.Ny, Nx = p.Nx;
    std::vector<double> colmajor;
    auto matrix = [&](const char* name, int rows, int cols) {
        const Dataset* d = find(ds, "Matrix", name);
        if (!d || d->dims.size() != 2 || d->dims[0] != (uint64_t)rows || d->dims[1] != (uint64_t)cols)
            return (int)HMEC_ERR_ARG;
        colmajor.resize((size_t)rows * cols);
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) colmajor[(size_t)j * rows + i] = d->v[(size_t)i * cols + j];
        return (int)hmec_upload_field(ctx, inst, field_id(name), colmajor.data(), rows, cols);
    };
    for (const char* n : MATRIX_BASIC)
        if (int rc = matrix(n, Ny, Nx)) return rc;
    for (const char* n : MATRIX_STAGGERED)
        if (int rc = matrix(n, Ny + 1, Nx + 1)) return rc;
    const int64_t n = hmec_marknum(&p);
    std::vector<std::vector<double>> mk(HMEC_M_COUNT, std::vector<double>((size_t)n));
    std::vector<double*> mp(HMEC_M_COUNT);
    for (int k = 0; k < HMEC_M_COUNT; k++) mp[k] = mk[k].data();
    if (int rc = hmec_download_markers(ctx, inst, mp.data(), n)) return rc;
    for (const char* m : MARKERS) {
        const Dataset* d = find(ds, "Vector", m);
        if (!d || d->v.size() != (size_t)n) return HMEC_ERR_ARG;
        mk[marker_id(m)] = d->v;
        mp[marker_id(m)] = mk[marker_id(m)].data();
    }
    std::vector<const double*> cmp(mp.begin(), mp.end());
    if (int rc = hmec_upload_markers(ctx, inst, cmp.data(), n)) return rc;
    const Dataset* vals = find(ds, "Value", "values");
    if (!vals || vals->v.size() != 9) return HMEC_ERR_ARG;
    for (int k = 0; k < 9; k++) hmec_set_scalar(ctx, inst, scalar_id(VALUES[k]), vals->v[k]);
    hmec_set_scalar(ctx, inst, scalar_id("timestep"), (double)(timestep + 1));
    for (int k = 0; k < 6; k++)
        if (const Dataset* d = find(ds, "Vector", HISTORY[k])) h.v[k] = d->v;
    return HMEC_OK;
}

// The layout as JSON (one line), for checking against the reference's lists.
inline void print_layout(FILE* out) {
    auto list = [&](const char* key, const char* const* v, int n, bool last) {
        fprintf(out, "\"%s\": [", key);
        for (int k = 0; k < n; k++) fprintf(out, "%s\"%s\"", k ? ", " : "", v[k]);
        fprintf(out, "]%s", last ? "" : ", ");
    };
    fprintf(out, "{");
    list("matrix_basic", MATRIX_BASIC, 24, false);
    list("matrix_staggered", MATRIX_STAGGERED, 30, false);
    list("history", HISTORY, 6, false);
    list("markers", MARKERS, 5, false);
    list("values", VALUES, 9, true);
    fprintf(out, "}\n");
}

}  // namespace ckpt
