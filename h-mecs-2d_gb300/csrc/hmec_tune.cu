// hmec_tune.cu -- the tuning table read at hmec_create.
//
// hmec/tune.py times a few timesteps of a model per candidate cycle shape
// (multigrid levels, pre/post/coarse sweeps) and launch shape (block sizes of
// the stencil and marker kernels, block counts of the Arnoldi step and of the
// smoothing launches) on the GPU and writes the fastest per grid and form to
// a JSON table:
//   {"version": 1, "entries": [{"Nx": 201, "Ny": 201, "form": 1,
//     "mg_levels": 5, "mg_pre": 2, "mg_post": 2, "mg_coarse_sweeps": 8,
//     "bs_stencil": 64, "bs_sort": 256, "krylov_blocks": 304,
//     "smooth_blocks": 0, "smooth_inverses": 0, "ms_per_step": 12.1}, ...]}
// With hmec_params.autotune set, hmec_create takes the entry of the same form
// whose grid is nearest in cells (within 4x) and applies its fields.  The
// table is $HMEC_TUNE_TABLE, else tune_table.json in the package directory
// above the library (hmec/_build/libhmec_gpu.so -> hmec/tune_table.json).
#include <dlfcn.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "hmec_internal.cuh"

namespace {

// A reader for the subset of JSON the table uses: objects, arrays, numbers,
// strings, true/false/null.  Objects' numeric members are kept (every object,
// at any depth, is listed); everything else is skipped.
struct Reader {
    const char* s;
    const char* e;
    bool ok = true;
    void ws() {
        while (s < e && (*s == ' ' || *s == '\n' || *s == '\r' || *s == '\t')) s++;
    }
    bool eat(char c) {
        ws();
        if (s < e && *s == c) {
            s++;
            return true;
        }
        return false;
    }
    std::string str() {
        std::string out;
        if (!eat('"')) {
            ok = false;
            return out;
        }
        while (s < e && *s != '"') {
            if (*s == '\\' && s + 1 < e) s++;
            out.push_back(*s++);
        }
        if (s < e) s++;
        return out;
    }
    double num() {
        ws();
        char* end = nullptr;
        const double v = strtod(s, &end);
        if (end == s) ok = false;
        s = end;
        return v;
    }
    void value(std::vector<std::map<std::string, double>>* objs, double* v, bool* has_num, int depth) {
        ws();
        if (!ok || s >= e || depth > 16) {
            ok = false;
            return;
        }
        if (*s == '{') {
            s++;
            std::map<std::string, double> m;
            if (!eat('}')) {
                do {
                    const std::string k = str();
                    if (!eat(':')) {
                        ok = false;
                        return;
                    }
                    double x = 0;
                    bool hn = false;
                    value(objs, &x, &hn, depth + 1);
                    if (!ok) return;
                    if (hn) m[k] = x;
                } while (eat(','));
                if (!eat('}')) {
                    ok = false;
                    return;
                }
            }
            objs->push_back(m);
        } else if (*s == '[') {
            s++;
            if (!eat(']')) {
                do {
                    double x = 0;
                    bool hn = false;
                    value(objs, &x, &hn, depth + 1);
                    if (!ok) return;
                } while (eat(','));
                if (!eat(']')) ok = false;
            }
        } else if (*s == '"') {
            str();
        } else if (e - s >= 4 && (!strncmp(s, "true", 4) || !strncmp(s, "null", 4))) {
            s += 4;
        } else if (e - s >= 5 && !strncmp(s, "false", 5)) {
            s += 5;
        } else {
            *v = num();
            *has_num = ok;
        }
    }
};

std::string table_path() {
    const char* env = getenv("HMEC_TUNE_TABLE");
    if (env && *env) return env;
    Dl_info info;
    if (dladdr((const void*)&hmec_tune_apply, &info) && info.dli_fname) {
        std::string so = info.dli_fname;
        const size_t k = so.rfind('/');
        const std::string dir = k == std::string::npos ? "." : so.substr(0, k);
        return dir + "/../tune_table.json";
    }
    return "";
}

}  // namespace

// Applies the nearest entry of the tuning table to p (see above); returns 1
// when an entry was applied, 0 otherwise (no table, no entry near enough).
int hmec_tune_apply(hmec_params* p) {
    const std::string path = table_path();
    if (path.empty()) return 0;
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return 0;
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    fclose(f);
    Reader r{text.data(), text.data() + text.size()};
    std::vector<std::map<std::string, double>> objs;
    double v = 0;
    bool hn = false;
    r.value(&objs, &v, &hn, 0);
    if (!r.ok) return 0;
    const double cells = (double)(p->Nx + 1) * (p->Ny + 1);
    const std::map<std::string, double>* best = nullptr;
    double best_d = 1e300;
    for (const auto& m : objs) {
        auto nx = m.find("Nx"), ny = m.find("Ny"), fm = m.find("form");
        if (nx == m.end() || ny == m.end() || fm == m.end()) continue;
        if ((int)fm->second != p->form) continue;
        const double c = (nx->second + 1) * (ny->second + 1);
        if (!(c > 0)) continue;
        const double d = std::fabs(std::log(c / cells));
        if (d < best_d) {
            best_d = d;
            best = &m;
        }
    }
    if (!best || best_d > std::log(4.0)) return 0;
    auto get = [&](const char* k, int32_t* dst, int lo, int hi) {
        auto it = best->find(k);
        if (it == best->end()) return;
        const int x = (int)it->second;
        if (x >= lo && x <= hi) *dst = x;
    };
    get("mg_levels", &p->mg_levels, 1, 8);
    get("mg_pre", &p->mg_pre, 1, 8);
    get("mg_post", &p->mg_post, 1, 8);
    get("mg_coarse_sweeps", &p->mg_coarse_sweeps, 1, 64);
    get("bs_stencil", &p->bs_stencil, 0, 1024);
    get("bs_sort", &p->bs_sort, 0, 1024);
    get("krylov_blocks", &p->krylov_blocks, 0, 1 << 16);
    get("smooth_blocks", &p->smooth_blocks, 0, 1 << 16);
    get("smooth_inverses", &p->smooth_inverses, 0, 2);
    {
        // the tuned multigrid options (local sweeps); the others stay
        int32_t f = -1;
        get("mg_flags", &f, 0, 15);
        if (f >= 0) p->mg_flags = (p->mg_flags & ~HMEC_MG_LOCAL_SWEEPS) | (f & HMEC_MG_LOCAL_SWEEPS);
    }
    return 1;
}

extern "C" int32_t hmec_tune_params(hmec_params* p) { return p ? hmec_tune_apply(p) : 0; }
