// hmec_run.cpp -- host loop mirroring main() of cpp/h_mec_rsf_v9.cpp, with the
// hot path delegated to libhmec_gpu.so through include/hmec.h.
//
// What stays on the host, as in the reference: the initial marker lattice and
// node fields (:188-209, :283-338), the per-step stdout report (:1732-1737),
// the EVO_*.txt time series of the fault row (:1751-1805) and the checkpoint
// files every `savestep` steps with restart from one (:211-282,
// :1807-1870; checkpoint.hpp).  Everything in between (:377-1726) is one
// hmec_timestep() call per step.
//
//   hmec_run [steps] [Nx Ny xsize ysize] [--mixed] [--outdir DIR]
//            [--savestep N] [--restart T] [--print-layout]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "checkpoint.hpp"
#include "hmec.h"

namespace {

struct Grid {
    int rows, cols;
    std::vector<double> a;
    Grid(int r, int c, double v = 0) : rows(r), cols(c), a((size_t)r * c, v) {}
    double& operator()(int i, int j) { return a[(size_t)j * rows + i]; }
};

std::vector<double> linspaced(int n, double low, double high) {  // Eigen LinSpaced
    std::vector<double> v(n);
    const double step = (n == 1) ? 0. : (high - low) / (double)(n - 1);
    for (int i = 0; i < n; i++) v[i] = (i == n - 1) ? high : low + (double)i * step;
    return v;
}

// A double as an ostream with the default flags and precision 6 prints it
// (the %g conversion).
std::string fmt_g(double v) {
    char b[64];
    snprintf(b, sizeof(b), "%g", v);
    return b;
}

// A vector the way Eigen's operator<< prints a matrix with its default
// IOFormat (the output the reference's EVO and fault files hold): every
// coefficient right-aligned to the width of the widest one, coefficients
// separated by one space (a row vector) or one per line (a column vector).
std::string eigen_text(const double* v, int n, bool column) {
    std::vector<std::string> t(n);
    size_t w = 0;
    for (int k = 0; k < n; k++) {
        t[k] = fmt_g(v[k]);
        if (t[k].size() > w) w = t[k].size();
    }
    std::string out;
    for (int k = 0; k < n; k++) {
        if (k) out += column ? "\n" : " ";
        out.append(w - t[k].size(), ' ');
        out += t[k];
    }
    return out;
}

// One line of an EVO_*.txt series (:1751-1799): time, dt, the fault row.
void append_row(const std::string& path, double timesum, double dt, const double* row, int n) {
    FILE* f = fopen(path.c_str(), "a");
    if (!f) return;
    const std::string line = fmt_g(timesum) + "    " + fmt_g(dt) + "    " + eigen_text(row, n, false) + "\n";
    fwrite(line.data(), 1, line.size(), f);
    fclose(f);
}

int check(hmec_ctx* ctx, int rc, const char* what) {
    if (rc != HMEC_OK) fprintf(stderr, "%s failed (%d): %s\n", what, rc, hmec_last_error(ctx));
    return rc;
}

}  // namespace

int main(int argc, char** argv) {
    hmec_params p;
    hmec_params_default(&p);  // cpp/constants.hpp
    int steps = 10;
    int savestep = 500;  // constants.hpp:15
    int restart = 0;     // the saved step to restart from (the reference reads it from file.txt, :180-186)
    std::string outdir = ".";
    std::vector<const char*> pos;
    for (int k = 1; k < argc; k++) {
        if (!strcmp(argv[k], "--mixed")) p.form = HMEC_FORM_MIXED;
        else if (!strcmp(argv[k], "--outdir") && k + 1 < argc) outdir = argv[++k];
        else if (!strcmp(argv[k], "--savestep") && k + 1 < argc) savestep = atoi(argv[++k]);
        else if (!strcmp(argv[k], "--restart") && k + 1 < argc) restart = atoi(argv[++k]);
        else if (!strcmp(argv[k], "--print-layout")) {
            ckpt::print_layout(stdout);
            return 0;
        } else pos.push_back(argv[k]);
    }
    if (pos.size() >= 1) steps = atoi(pos[0]);
    if (pos.size() >= 5) {
        p.Nx = atoi(pos[1]);
        p.Ny = atoi(pos[2]);
        p.xsize = atof(pos[3]);
        p.ysize = atof(pos[4]);
    }
    const int Nx = p.Nx, Ny = p.Ny, Nx1 = Nx + 1, Ny1 = Ny + 1;
    const double dx = p.xsize / (Nx - 1), dy = p.ysize / (Ny - 1);
    const double upper_block = p.ysize / 2. - dy, lower_block = p.ysize / 2. + dy;
    const int line_fault = (int)((Ny - 1) / 2.);

    // markers, :188-209 (rand() % 1 == 0: no jitter)
    const int64_t nxm = (int64_t)(Nx - 1) * p.mx, nym = (int64_t)(Ny - 1) * p.my;
    const int64_t marknum = nxm * nym;
    const double dxms = p.xsize / (double)nxm, dyms = p.ysize / (double)nym;
    std::vector<std::vector<double>> mk(HMEC_M_COUNT, std::vector<double>((size_t)marknum, 0.0));
    for (int64_t m = 0; m < marknum; m++) {
        double& xm = mk[HMEC_M_xm][m];
        double& ym = mk[HMEC_M_ym][m];
        xm = 0 + (double)(m / nym) * dxms;
        ym = 0 + (double)(m % nym) * dyms;
        mk[HMEC_M_t_marker][m] = 1;
        mk[HMEC_M_rhom][m] = 2800;
        mk[HMEC_M_etasm][m] = 1e21;
        mk[HMEC_M_cohescm][m] = p.cohes;
        mk[HMEC_M_cohestm][m] = p.cohes;
        mk[HMEC_M_frictcm][m] = .5;
        mk[HMEC_M_dilatcm][m] = p.dilatation;
        mk[HMEC_M_fricttm][m] = p.tensile;
        mk[HMEC_M_kkkm][m] = 2e-16;
        mk[HMEC_M_gm][m] = p.shearmod;
        mk[HMEC_M_rhofm][m] = 1000;
        mk[HMEC_M_etafm][m] = 1e-3;
        mk[HMEC_M_porm][m] = .01 * (1 + .0 * (0 - .5));
        mk[HMEC_M_etam][m] = mk[HMEC_M_etasm][m] * exp(-p.alpha * mk[HMEC_M_porm][m]);
        if (ym < upper_block || ym > lower_block) {
            mk[HMEC_M_t_marker][m] = -1;
            mk[HMEC_M_etam][m] = 1e23;
            mk[HMEC_M_etasm][m] = 1e23;
            mk[HMEC_M_rhom][m] = 2800;
            mk[HMEC_M_kkkm][m] = 2e-16;
            mk[HMEC_M_cohescm][m] = p.cohes * 1e3;
            mk[HMEC_M_cohestm][m] = p.cohes * 1e3;
            mk[HMEC_M_frictcm][m] = .8;
            mk[HMEC_M_dilatcm][m] = p.dilatation;
            mk[HMEC_M_fricttm][m] = p.tensile;
        }
    }
    // node fields of a fresh start, :283-338
    Grid OM0(Ny, Nx, p.omm[0]), ARSF(Ny, Nx, p.arsfm[1]), BRSF(Ny, Nx, p.brsfm[1]), LRSF(Ny, Nx, p.lrsfm[0]);
    const std::vector<double> x = linspaced(Nx, 0, p.xsize), y = linspaced(Ny, 0, p.ysize);
    for (int i = 0; i < Ny; i++) {
        if (!(y[i] > upper_block && y[i] < lower_block)) continue;
        for (int j = 0; j < Nx; j++) {
            OM0(i, j) = p.omm[1];
            const double xj = x[j];
            if (xj < p.TS_1) {
                BRSF(i, j) = p.brsfm[0];
                ARSF(i, j) = p.arsfm[0];
            }
            if (xj >= p.TS_1 && xj < p.TS_2) {
                const double t = (xj - p.TS_1) / (p.TS_2 - p.TS_1);
                BRSF(i, j) = p.brsfm[0] - (p.brsfm[0] - p.brsfm[1]) * t;
                ARSF(i, j) = p.arsfm[0] - (p.arsfm[0] - p.arsfm[1]) * t;
                LRSF(i, j) = p.lrsfm[0] - (p.lrsfm[0] - p.lrsfm[1]) * t;
            }
            if (xj >= p.TS_2 && xj <= p.TS_3) LRSF(i, j) = p.lrsfm[1];
            if (xj > p.TS_3 && xj <= p.TS_4) {
                const double t = (xj - p.TS_3) / (p.TS_4 - p.TS_3);
                BRSF(i, j) = p.brsfm[1] - (p.brsfm[1] - p.brsfm[0]) * t;
                ARSF(i, j) = p.arsfm[1] - (p.arsfm[1] - p.arsfm[0]) * t;
                LRSF(i, j) = p.lrsfm[1] - (p.lrsfm[1] - p.lrsfm[0]) * t;
            }
            if (xj > p.TS_4) {
                BRSF(i, j) = p.brsfm[0];
                ARSF(i, j) = p.arsfm[0];
            }
        }
    }
    Grid PT0(Ny1, Nx1, p.PCONF + p.PTFDIFF), PF0(Ny1, Nx1, p.PCONF);

    int32_t st = 0;
    hmec_ctx* ctx = hmec_create(&p, 1, nullptr, &st);
    if (!ctx) {
        fprintf(stderr, "hmec_create failed (%d)\n", st);
        return 1;
    }
    std::vector<const double*> mptr(HMEC_M_COUNT);
    for (int k = 0; k < HMEC_M_COUNT; k++) mptr[k] = mk[k].data();
    if (check(ctx, hmec_upload_markers(ctx, 0, mptr.data(), marknum), "upload_markers")) return 1;
    struct {
        int id;
        Grid* g;
    } init[] = {{HMEC_F_OM0, &OM0}, {HMEC_F_OM, &OM0}, {HMEC_F_ARSF, &ARSF}, {HMEC_F_BRSF, &BRSF},
                {HMEC_F_LRSF, &LRSF}, {HMEC_F_PT0, &PT0}, {HMEC_F_PF0, &PF0}};
    for (auto& f : init)
        if (check(ctx, hmec_upload_field(ctx, 0, f.id, f.g->a.data(), f.g->rows, f.g->cols), "upload_field")) return 1;

    const std::string d = outdir + "/";
    ckpt::History history(p.num_timesteps);
    if (restart > 0) {  // :211-282
        const std::string name = d + "h_mec_" + std::to_string(restart) + ".h5.stub";
        std::vector<ckpt::Dataset> ds;
        if (!ckpt::read_stub(name, ds)) {
            fprintf(stderr, "cannot read checkpoint %s\n", name.c_str());
            return 1;
        }
        if (check(ctx, ckpt::restore(ctx, p, ds, restart, history), "restore")) return 1;
        // EVO_*.txt keep the lines of the steps up to the saved one (:268-281;
        // the reference lists "EVO_VxD.txt" but writes "EVO_vxD.txt", so its
        // Darcy series is not trimmed on a case-sensitive file system)
        for (const char* evo : {"EVO_Vslip.txt", "EVO_viscosity.txt", "EVO_press_flu.txt", "EVO_press_eff.txt",
                                "EVO_SigmaY.txt", "EVO_Sii.txt", "EVO_Theta.txt", "EVO_Visc_comp.txt",
                                "EVO_Elast_comp.txt", "EVO_vxD.txt", "EVO_data.txt"}) {
            const std::string path = d + evo;
            FILE* f = fopen(path.c_str(), "r");
            if (!f) continue;
            std::string keep;
            int lines = 0;
            for (int c; lines < restart && (c = fgetc(f)) != EOF;) {
                keep.push_back((char)c);
                if (c == '\n') lines++;
            }
            fclose(f);
            f = fopen(path.c_str(), "w");
            if (f) {
                fwrite(keep.data(), 1, keep.size(), f);
                fclose(f);
            }
        }
    }

    // the fault-row series of :1751-1799, in one row gather per step
    const int evo_ids[] = {HMEC_F_VSLIPB, HMEC_F_ETA, HMEC_F_pf, HMEC_F_pt, HMEC_F_SigmaY, HMEC_F_SII_fault,
                           HMEC_F_OM, HMEC_F_VIS_COMP, HMEC_F_EL_DECOM, HMEC_F_vxD};
    const int nevo = (int)(sizeof(evo_ids) / sizeof(evo_ids[0]));
    std::vector<int> evo_off(nevo + 1, 0);
    for (int k = 0; k < nevo; k++) evo_off[k + 1] = evo_off[k] + (hmec_field_grid(evo_ids[k]) ? Nx1 : Nx);
    // The rows of a step are gathered right after it and copied to
    // page-locked memory while the next step runs
    // (hmec_download_rows_async); that step's EVO lines are written once the
    // next step has returned, so the files keep the reference's line order.
    struct Pending {
        hmec_step_report r;
        int64_t ticket = 0;
        double* buf = nullptr;
        bool live = false;
    } pend[2];
    std::vector<double> fallback[2];
    for (int k = 0; k < 2; k++) {
        pend[k].buf = (double*)hmec_host_alloc(sizeof(double) * (size_t)evo_off[nevo]);
        if (!pend[k].buf) {
            fallback[k].resize(evo_off[nevo]);
            pend[k].buf = fallback[k].data();
        }
    }
    std::vector<double> peff(Nx1);
    auto write_evo = [&](Pending& q) {
        if (!q.live) return 0;
        q.live = false;
        if (check(ctx, hmec_rows_wait(ctx, 0, q.ticket), "rows_wait")) return 1;
        const hmec_step_report& r = q.r;
        const double* row = q.buf;
        for (int j = 0; j < Nx1; j++) peff[j] = row[evo_off[3] + j] - row[evo_off[2] + j];  // pt - pf
        append_row(d + "EVO_Vslip.txt", r.timesum, r.dt, row + evo_off[0], Nx);
        append_row(d + "EVO_viscosity.txt", r.timesum, r.dt, row + evo_off[1], Nx);
        append_row(d + "EVO_press_flu.txt", r.timesum, r.dt, row + evo_off[2], Nx1);
        append_row(d + "EVO_press_eff.txt", r.timesum, r.dt, peff.data(), Nx1);
        append_row(d + "EVO_SigmaY.txt", r.timesum, r.dt, row + evo_off[4], Nx);
        append_row(d + "EVO_Sii.txt", r.timesum, r.dt, row + evo_off[5], Nx);
        append_row(d + "EVO_Theta.txt", r.timesum, r.dt, row + evo_off[6], Nx);
        append_row(d + "EVO_Visc_comp.txt", r.timesum, r.dt, row + evo_off[7], Nx1);
        append_row(d + "EVO_Elast_comp.txt", r.timesum, r.dt, row + evo_off[8], Nx1);
        append_row(d + "EVO_vxD.txt", r.timesum, r.dt, row + evo_off[9], Nx1);
        FILE* f = fopen((d + "EVO_data.txt").c_str(), "a");
        if (f) {
            fprintf(f, "%20g%20g%20g%20d%20d\n", r.timesum, r.dt, r.Vmax, r.ynlast, r.global_iters);
            fclose(f);
        }
        return 0;
    };
    int failed = 0;
    for (int s = 0; s < steps && !failed; s++) {
        hmec_step_report r;
        if (check(ctx, hmec_timestep(ctx, &r), "hmec_timestep")) break;
        history.record(ctx, r.timestep);
        // :1732-1737
        printf("====================================\n");
        printf("total time:        %g sec\n", r.timesum);
        printf("time step:         %g sec\n", r.dt);
        printf("Vslip max:         %g\n", r.Vmax);
        printf("iter - iterations:   %d\n", r.global_iters);
        printf("global - iterations: %d\n", r.ynlast);
        if (r.timestep == 1) {  // :1739-1749
            FILE* fx = fopen((d + "x_fault.txt").c_str(), "w");
            if (fx) {
                const std::string t = eigen_text(x.data(), Nx, true) + "\n";
                fwrite(t.data(), 1, t.size(), fx);
                fclose(fx);
            }
            const int rsf_ids[] = {HMEC_F_ARSF, HMEC_F_BRSF, HMEC_F_LRSF};
            std::vector<double> rr(3 * (size_t)Nx);
            if (!check(ctx, hmec_download_rows(ctx, 0, line_fault, 3, rsf_ids, rr.data()), "download_rows")) {
                FILE* fr = fopen((d + "rsf_fault.txt").c_str(), "a");
                if (fr) {
                    const std::string t = eigen_text(rr.data(), Nx, false) + "\n\n" +
                                          eigen_text(rr.data() + Nx, Nx, false) + "\n\n" +
                                          eigen_text(rr.data() + 2 * Nx, Nx, false) + "\n";
                    fwrite(t.data(), 1, t.size(), fr);
                    fclose(fr);
                }
            }
        }
        // the previous step's lines (its copy ran during this step)
        if (write_evo(pend[(s + 1) & 1])) break;
        Pending& q = pend[s & 1];
        q.r = r;
        if (check(ctx, hmec_download_rows_async(ctx, 0, line_fault, nevo, evo_ids, q.buf, &q.ticket),
                  "download_rows_async"))
            break;
        q.live = true;
        if (savestep > 0 && r.timestep % savestep == 0) {  // :1807-1870
            if (write_evo(q)) break;  // the EVO files hold every step up to the saved one
            FILE* ft = fopen((d + "file.txt").c_str(), "w");
            if (ft) {
                fprintf(ft, "%d\n", r.timestep);
                fclose(ft);
            }
            std::vector<ckpt::Dataset> ds;
            const std::string name = d + "h_mec_" + std::to_string(r.timestep) + ".h5.stub";
            if (check(ctx, ckpt::collect(ctx, p, history, ds), "checkpoint") || !ckpt::write_stub(name, ds)) {
                fprintf(stderr, "cannot write checkpoint %s\n", name.c_str());
                break;
            }
        }
    }
    for (auto& q : pend) failed |= write_evo(q);
    for (int k = 0; k < 2; k++)
        if (fallback[k].empty()) hmec_host_free(pend[k].buf);
    hmec_destroy(ctx);
    return failed ? 1 : 0;
}
