// k_advect.cu -- node -> marker gather and marker advection (sections a18,
// a20; the loop of cpp/h_mec_rsf_v9.cpp:1561-1656, which never runs in the
// reference because its bound is 0).  One thread per marker: four RK stages,
// each a bilinear gather of vx (Vx nodes), vy (Vy nodes) and the spin ESP
// (basic nodes) from L2-resident node fields, then the Jaumann rotation of
// the marker stress by spin * dt and periodic recycling in x.
// rk4_as_written = 1 reproduces the reference's stage shift (:1622-1630:
// stage 3 is evaluated at the point of stage 2); 0 is classic RK4.
#include "hmec_internal.cuh"

namespace {

__device__ __forceinline__ double bilin(const double* __restrict__ F, int rows, int i, int j, double dxm, double dym) {
    const double* c0 = F + (size_t)j * rows + i;
    const double* c1 = c0 + rows;
    return c0[0] * (1 - dxm) * (1 - dym) + c0[1] * (1 - dxm) * dym + c1[0] * dxm * (1 - dym) + c1[1] * dxm * dym;
}

struct AdvIn {
    const double *vxs, *vys, *ESP;
    const double *x, *y, *xvx, *yvx, *xvy, *yvy;
};

__global__ void k_advect(Geo g, const DevScalars* ds, hmec_params p, AdvIn in, int64_t n, double* xm, double* ym,
                         double* sxxm, double* syym, double* sxym) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const double dt = ds->dt, dx = g.dx, dy = g.dy;
    const double xold = xm[m], yold = ym[m];
    double xc = xold, yc = yold;
    double vxm[4], vym[4], spm0 = 0;
    for (int rk = 0; rk < 4; rk++) {
        int j = check_bounds(fix_trunc(__ddiv_rn(xc, dx)), g.Nx);
        int i = check_bounds(fix_trunc(__ddiv_rn(__dadd_rn(yc, dy / 2.), dy)), g.Ny);
        vxm[rk] = bilin(in.vxs, g.Ny1, i, j, (xc - in.xvx[j]) / dx, (yc - in.yvx[i]) / dy);
        j = check_bounds(fix_trunc(__ddiv_rn(__dadd_rn(xc, dx / 2.), dx)), g.Nx);
        i = check_bounds(fix_trunc(__ddiv_rn(yc, dy)), g.Ny);
        vym[rk] = bilin(in.vys, g.Ny1, i, j, (xc - in.xvy[j]) / dx, (yc - in.yvy[i]) / dy);
        if (rk == 0) {
            j = check_bounds(fix_trunc(__ddiv_rn(xc, dx)), g.Nx);
            i = check_bounds(fix_trunc(__ddiv_rn(yc, dy)), g.Ny);
            spm0 = bilin(in.ESP, g.Ny, i, j, (xc - in.x[j]) / dx, (yc - in.y[i]) / dy);
        }
        if (rk < 2) {
            xc = xold + vxm[rk] * dt / 2.;
            yc = yold + vym[rk] * dt / 2.;
        } else if (rk == (p.rk4_as_written ? 3 : 2)) {
            xc = xold + vxm[rk] * dt;
            yc = yold + vym[rk] * dt;
        }
    }
    const double dspeff = spm0 * dt;  // :1636-1643 (only stage 0's spin is used)
    const double o_xx = sxxm[m], o_yy = syym[m], o_xy = sxym[m];
    double s2, c2, s1, c1;
    sincos(2 * dspeff, &s2, &c2);
    sincos(dspeff, &s1, &c1);
    sxym[m] = .5 * (o_xx - o_yy) * s2 + o_xy * c2;
    sxxm[m] = o_xx * (c1 * c1) + o_yy * (s1 * s1) - o_xy * s2;
    syym[m] = o_xx * (s1 * s1) + o_yy * (c1 * c1) + o_xy * s2;
    double xn = xold + (vxm[0] + 2 * vxm[1] + 2 * vxm[2] + vxm[3]) / 6. * dt;  // :1646-1647
    const double yn = yold + (vym[0] + 2 * vym[1] + 2 * vym[2] + vym[3]) / 6. * dt;
    if (xn < 0) xn = xn + p.xsize;  // :1650-1655
    if (xn > p.xsize) xn = xn - p.xsize;
    xm[m] = xn;
    ym[m] = yn;
}

}  // namespace

int advect_run(hmec_inst* ctx) {
    const Geo& g = ctx->g;
    double* const* f = ctx->f;
    AdvIn in{f[HMEC_F_vxs], f[HMEC_F_vys], f[HMEC_F_ESP], ctx->crd[0], ctx->crd[1], ctx->crd[2], ctx->crd[3],
             ctx->crd[4], ctx->crd[5]};
    HMEC_LAUNCH(ctx, k_advect, nblocks(ctx->marknum, 256), 256, 0, g, ctx->ds, ctx->p, in, ctx->marknum,
                ctx->mk[HMEC_M_xm], ctx->mk[HMEC_M_ym], ctx->mk[HMEC_M_sxxm], ctx->mk[HMEC_M_syym], ctx->mk[HMEC_M_sxym]);
    HMEC_CUDA(ctx, cudaGetLastError());
    return HMEC_OK;
}
