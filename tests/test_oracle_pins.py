"""Pins of the CPU oracle (no GPU).

The reference ships no tests, fixtures or golden vectors and cannot be
built here, so the oracle is pinned by known answers derived by hand from the
equations of cpp/h_mec_rsf_v9.cpp, by a manufactured simple-shear solution,
by an independent vectorised restatement of single sections, and by the
behaviour of the quirks it reproduces.
"""
import math

import numpy as np
import pytest

import oracle as O
from hmec import synth
import pairs


def fresh(preset="tiny", **extra):
    return pairs.oracle_for(preset, **extra)


def test_linspaced_coordinates():
    o, _, _ = fresh()
    p = o.params
    dx = p.xsize / (p.Nx - 1)
    dy = p.ysize / (p.Ny - 1)
    x = o.coords(0)
    assert x[0] == 0.0 and x[-1] == p.xsize
    step = p.xsize / (p.Nx - 1)
    assert np.array_equal(x[:-1], np.arange(p.Nx - 1) * step)
    yp = o.coords(7)
    assert yp[0] == -dy / 2 and yp[-1] == p.ysize + dy / 2
    assert np.allclose(np.diff(yp), dy, rtol=1e-12)
    xvx = o.coords(2)
    assert xvx[-1] == p.xsize + dx
    assert np.array_equal(o.coords(4), o.coords(6))  # xvy == xp
    assert np.array_equal(o.coords(3), o.coords(7))  # yvx == yp


def test_marker_lattice_and_materials():
    p = O.default_params()  # constants.hpp: 401 x 51, 4 x 4 markers per cell
    mk = synth.reference_markers(p)
    assert mk["xm"].shape == (320000,)
    nym = 50 * 4
    dxms, dyms = 40000.0 / 1600, 10000.0 / 200
    m = 12345
    assert mk["xm"][m] == (m // nym) * dxms and mk["ym"][m] == (m % nym) * dyms
    blk = (mk["ym"] < 4800) | (mk["ym"] > 5200)
    assert np.all(mk["etasm"][blk] == 1e23) and np.all(mk["etasm"][~blk] == 1e21)
    assert np.all(mk["frictcm"][blk] == 0.8) and np.all(mk["frictcm"][~blk] == 0.5)
    assert np.allclose(mk["etam"][~blk], 1e21 * math.exp(-0.29), rtol=1e-15)
    assert np.all(mk["porm"] == 0.01)


def test_p2g_uniform_material_reproduces_marker_properties():
    o, mk, _ = fresh()
    n = mk["xm"].shape[0]
    uni = dict(mk)
    for k, v in dict(t_marker=1.0, rhom=2700.0, etasm=2e22, etam=3e21, cohescm=5e6, cohestm=4e6, frictcm=0.7,
                     dilatcm=0.1, fricttm=0.9, porm=0.02, kkkm=3e-18, gm=2.5e10, rhofm=1100.0, etafm=2e-3).items():
        uni[k] = np.full(n, v)
    o.set_markers(uni)
    o.markers_to_nodes()
    por = 0.02
    kk = min(max(3e-18 * (por / 0.01) ** 3, 1e-22), 1e-12)
    exp_vals = dict(RHO=2700 * (1 - por) + 1100 * por, KKK=kk, TTT=1.0, GGG=2.5e10, ETA0=2e22 * math.exp(-29 * por),
                    COHT=4e6 * (1 - por), FRIT=0.9, COHC=5e6 * (1 - por), FRIC=0.7, DILC=0.1,
                    ETAP=3e21, POR=por, ETAB0=2e22 / por, ETAP0=2e22 * math.exp(-29 * por), GGGP=2.5e10,
                    RHOX=2700 * (1 - por) + 1100 * por, ETADX=2e-3 / kk, RHOFX=1100.0, PORX=por,
                    RHOY=2700 * (1 - por) + 1100 * por, ETADY=2e-3 / kk, RHOFY=1100.0, PORY=por)
    Ny, Nx = o.Ny, o.Nx
    for f, v in exp_vals.items():
        a = o.field(f)
        if a.shape == (Ny, Nx):
            sub = a
        elif f in ("RHOX", "ETADX", "RHOFX", "PORX"):
            sub = a[:Ny, :Nx]  # Vx nodes that receive markers
        elif f in ("RHOY", "ETADY", "RHOFY", "PORY"):
            sub = a[:Ny, :Nx]
        else:
            sub = a[:Ny, :Nx]
        assert np.allclose(sub, v, rtol=2e-14, atol=0), f


def test_p2g_clamped_edge_weights_are_extrapolated():
    # check_bounds clamps the P cell to Nx-2, so markers beyond the last
    # interior P node get a weight outside [0, 1] (:468-474); the normalised
    # field is still exact for a uniform property.
    o, mk, _ = fresh()
    o.markers_to_nodes()
    wt_rows = o.field("POR")[1:o.Ny, 1:o.Nx]
    assert np.allclose(wt_rows, 0.01, rtol=1e-14)
    assert np.all(o.field("POR")[o.Ny, :] == 0)  # P ghost row never gets markers


def test_assembly_known_entries_and_duplicates():
    o, _, _ = fresh()
    o.markers_to_nodes()
    o.timestep_begin()
    o.iter_prepare()
    A, R = o.assemble()
    A = A.tocsr()
    p = o.params
    Nx, Ny = p.Nx, p.Ny
    Ny1 = Ny + 1
    pfscale, ptscale = o.scales()

    def kp(i, j):
        return (j * Ny1 + i) * 6

    # Q7: vxD at (0, 0) gets the upper-symmetry and left no-penetration rows -> diag 2
    assert A[kp(0, 0) + 4, kp(0, 0) + 4] == 2.0
    assert A[kp(0, 0) + 4, kp(1, 0) + 4] == -1.0
    # Q7: vy at (Ny, 0): ghost diag 1 + free slip diag 1 -> 2, off-diagonal +1
    assert A[kp(Ny, 0) + 2, kp(Ny, 0) + 2] == 2.0
    assert A[kp(Ny, 0) + 2, kp(Ny, 1) + 2] == 1.0
    # prescribed shear velocity rows (:707-717)
    assert R[kp(0, 3) + 1] == 2 * p.bcupper and R[kp(Ny, 3) + 1] == 2 * p.bclower
    # real fluid-pressure BC rows (:955-957)
    for i in (1, Ny - 1):
        k = kp(i, 4)
        assert A[k + 3, k + 3] == pfscale and A[k + 3, k] == -ptscale and R[k + 3] == -p.PTFDIFF
    # interior x-Stokes row, recomputed from the oracle's node fields (:740-767)
    i, j = 3, 5
    dx = p.xsize / (Nx - 1)
    dy = p.ysize / (Ny - 1)
    dt = o.scalar("dt")
    ETA, GGG = o.field("ETA"), o.field("GGG")
    ETAP, GGGP, RHOX = o.field("ETAP"), o.field("GGGP"), o.field("RHOX")

    def num(eta, g):
        return eta * (dt * g / (dt * g + eta))

    exy1, exy2 = num(ETA[i - 1, j], GGG[i - 1, j]), num(ETA[i, j], GGG[i, j])
    exx1, exx2 = num(ETAP[i, j], GGGP[i, j]), num(ETAP[i, j + 1], GGGP[i, j + 1])
    kx = kp(i, j) + 1
    diag = -(exx1 + exx2) / dx ** 2 - (exy1 + exy2) / dy ** 2 - RHOX[i, j] / dt
    assert A[kx, kx] == pytest.approx(diag, rel=1e-14)
    assert A[kx, kx - 6 * Ny1] == pytest.approx(exx1 / dx ** 2, rel=1e-14)
    assert A[kx, kx + 6] == pytest.approx(exy2 / dy ** 2, rel=1e-14)
    assert A[kx, kp(i, j)] == pytest.approx(ptscale / dx, rel=1e-15)
    assert A[kx, kp(i, j + 1)] == pytest.approx(-ptscale / dx, rel=1e-15)
    assert A[kx].nnz == 11
    # every row carries its diagonal
    assert np.all(A.diagonal() != 0)


def test_first_solve_is_simple_shear():
    # From rest, the x-velocity between the prescribed boundary velocities
    # (bcupper at the top, bclower at the bottom) is linear in y.
    o, _, _ = fresh()
    o.markers_to_nodes()
    o.timestep_begin()
    o.iter_prepare()
    A, R = o.assemble()
    x = O.direct_solve(A, R)
    p = o.params
    Ny1 = p.Ny + 1
    vx = x.reshape(-1, 6)[:, 1].reshape((Ny1, p.Nx + 1), order="F")
    yvx = o.coords(3)
    expect = p.bcupper + (p.bclower - p.bcupper) * yvx / p.ysize
    inner = vx[:, 2:p.Nx - 2]
    assert np.allclose(inner, expect[:, None], rtol=0, atol=2e-3 * abs(p.bclower))


def test_direct_solve_reaches_machine_precision():
    o, _, _ = fresh()
    for _ in range(3):
        o.timestep()
    o.markers_to_nodes()
    o.timestep_begin()
    o.iter_prepare()
    A, R = o.assemble()
    x = O.direct_solve(A, R)
    Dr, _ = O.equilibrate(A)
    rel = np.linalg.norm(Dr @ (R - A @ x)) / np.linalg.norm(Dr @ R)
    assert rel < 1e-14


def rsf_numpy(o, i, dt, timestep):
    """Independent vectorised restatement of the fault update :1169-1305 for row i."""
    p = o.params
    f = {k: o.field(k) for k in ("ARSF", "BRSF", "LRSF", "FRIC", "ETA0", "SXX", "SYY", "SXY", "GGG", "ETA", "OM",
                                 "OM0", "pt", "pf")}
    Nx = p.Nx
    dx = p.xsize / (Nx - 1)
    j = np.arange(Nx)
    blk = lambda a: a[i, j] + a[i + 1, j] + a[i, j + 1] + a[i + 1, j + 1]
    a, b, L, fr, e0 = f["ARSF"][i], f["BRSF"][i], f["LRSF"][i], f["FRIC"][i], f["ETA0"][i]
    sxx, syy, sxy = blk(f["SXX"]), blk(f["SYY"]), f["SXY"][i]
    siib = np.sqrt(sxy ** 2 + (sxx ** 2 + syy ** 2 + (sxx + syy) ** 2) / 32)
    G, eta = f["GGG"][i], f["ETA"][i]
    siiel = siib / (eta / (G * dt + eta))
    prt = (blk(f["pt"]) - blk(f["pf"])) / 4
    prB = np.maximum(prt, 1e3)
    eom = np.exp(-(b * f["OM"][i] + fr) / a)

    def resid(s):
        V = 2 * p.V0 * np.sinh(np.maximum(s, 0) / a / prB) * eom
        etavp = 1 / (1 / e0 + 1 / (s / 2 / (V / dx / 2)))
        return siiel * etavp / (G * dt + etavp) - s, V

    s1 = siib.copy()
    V1 = p.V0 * np.sinh(np.maximum(s1, 0) / a / prB) * eom / dx
    etavp = 1 / (1 / e0 + 1 / (s1 / 2 / V1))
    s2 = siiel * etavp / (G * dt + etavp)
    d1 = s2 - s1
    d2, V = resid(s2)
    for jj in range(Nx):  # bisection per node, same rule as :1221-1243
        if (d1[jj] >= 0 and d2[jj] <= 0) or (d1[jj] <= 0 and d2[jj] >= 0):
            lo, hi, ds = s1[jj], s2[jj], 1e9
            while abs(ds) > 1e-3:
                mid = (lo + hi) / 2
                V0s = 2 * p.V0 * math.sinh(max(mid, 0) / a[jj] / prB[jj]) * eom[jj]
                ev = 1 / (1 / e0[jj] + 1 / (mid / 2 / (V0s / dx / 2)))
                ds = siiel[jj] * ev / (G[jj] * dt + ev) - mid
                V[jj] = V0s
                if (ds >= 0 and d1[jj] >= 0) or (ds <= 0 and d1[jj] <= 0):
                    lo = mid
                else:
                    hi = mid
    x = V * dt / L
    om5 = np.where(x > 1e-6, np.log(p.V0 / V + (np.exp(f["OM0"][i]) - p.V0 / V) * np.exp(-x)),
                   np.log(np.exp(f["OM0"][i]) * (1 - x) + p.V0 * dt / L))
    syield = np.maximum(p.syieldmin, prt * a * np.arcsinh(V / 2 / p.V0 * np.exp((b * om5 + fr) / a)))
    return V, om5, syield


def test_rsf_update_matches_independent_restatement():
    o, _, _ = fresh()
    for _ in range(3):
        o.timestep()
    o.markers_to_nodes()
    o.timestep_begin()
    o.iter_prepare()
    A, R = o.assemble()
    S = O.direct_solve(A, R)
    dt = o.scalar("dt")
    before = o.snapshot()  # ETA, OM, OM0 as the fault update sees them
    o.iter_finish(S)
    i = int((o.params.Ny - 1) / 2)
    V_o, om5_o, sy_o = o.field("VSLIPB")[i].copy(), o.field("OM5")[i].copy(), o.field("SigmaY")[i].copy()
    o2, _, _ = fresh()
    o2.load_state(before)
    for k in ("SXX", "SYY", "SXY", "pt", "pf"):  # final stresses/pressures of the iteration
        o2.set_field(k, o.field(k))
    V, om5, sy = rsf_numpy(o2, i, dt, o.scalar("timestep"))
    assert np.all(V_o > 0)
    assert np.allclose(V, V_o, rtol=1e-12)
    assert np.allclose(om5, om5_o, rtol=1e-12, atol=1e-14)
    assert np.allclose(sy, sy_o, rtol=1e-12)


def test_aging_law_fixed_point():
    # With OM0 = ln(V0/V) and constant V the aging law (:1245-1249) keeps the state.
    V0, V, dt, L = 1e-6, 1e-9, 1e7, 0.02
    om0 = math.log(V0 / V)
    x = V * dt / L
    om5 = math.log(V0 / V + (math.exp(om0) - V0 / V) * math.exp(-x))
    assert om5 == pytest.approx(om0, rel=1e-14)


def test_quirk_q1_accumulated_sums_give_same_ratios():
    a, _, _ = fresh(quirk_accumulate_sums=1)
    b, _, _ = fresh(quirk_accumulate_sums=0)
    for _ in range(4):
        a.timestep()
        b.timestep()
    for f in pairs.P2G_FIELDS:
        x, y = a.field(f), b.field(f)
        den = np.max(np.abs(y)) or 1.0
        assert np.max(np.abs(x - y)) / den < 1e-13, f


def test_quirk_q2_ghost_stress_rows_stay_zero():
    o, _, _ = fresh()
    for _ in range(4):
        o.timestep()
    for f in ("SXX", "SYY"):
        a = o.field(f)
        assert np.all(a[0, :] == 0) and np.all(a[-1, :] == 0) and np.all(a[:, 0] == 0) and np.all(a[:, -1] == 0)
        assert np.any(a[1:-1, 1:-1] != 0)


def test_reference_check_values():
    # nucleation size and cohesive zone printed by the reference (:363-370)
    p = O.default_params()
    hstar = math.pi / 2 * p.shearmod * p.lrsfm[1] * p.brsfm[1] / (p.brsfm[1] - p.arsfm[1]) ** 2 / p.PTFDIFF
    coh = 9.0 / 32 * math.pi * p.shearmod * p.lrsfm[1] / p.brsfm[1] / p.PTFDIFF
    assert hstar / 1e3 == pytest.approx(2.47255, rel=1e-5)
    assert coh == pytest.approx(500.71, rel=1e-4)
    assert (((p.TS_4 + p.TS_3) / 2) - ((p.TS_2 + p.TS_1) / 2)) / 1e3 == 33.0


def test_timestep_sequence_starts_like_the_reference_control_logic():
    o, _, _ = fresh()
    it1 = o.timestep()
    # step 1: no fault update (timestep == tyield), dt cut from 5e8 by the
    # displacement criteria, then capped by dtlapusta = 1e7 at the end (:1472)
    assert it1 >= 1
    assert o.scalar("dt") <= 1e7
    assert o.scalar("timestep") == 2
    it2 = o.timestep()
    assert o.scalar("timestep") == 3 and it2 >= 1


P2G_FIELDS = ("RHO", "KKK", "TTT", "GGG", "ETA0", "COHT", "FRIT", "COHC", "FRIC", "DILC", "ETAP", "POR", "ETAB0",
              "ETAP0", "GGGP", "RHOX", "ETADX", "RHOFX", "PORX", "RHOY", "ETADY", "RHOFY", "PORY")


@pytest.mark.parametrize("threads", [2, 3, 8])
def test_threaded_marker_loop_matches_the_serial_one(threads):
    # the CPU baseline's marker loop on several threads: per-thread sums
    # added in thread order -- deterministic, and equal to the serial loop
    # up to the order of the additions
    o, _, _ = fresh("c1")
    o.markers_to_nodes()
    ref = {f: o.field(f).copy() for f in P2G_FIELDS}
    o.set_threads(threads)
    o.markers_to_nodes()
    one = {f: o.field(f).copy() for f in P2G_FIELDS}
    o.markers_to_nodes()
    for f in P2G_FIELDS:
        assert np.array_equal(one[f], o.field(f)), f  # same thread count, same bits
        scale = np.max(np.abs(ref[f]))
        assert np.max(np.abs(one[f] - ref[f])) <= 1e-13 * scale, f
    o.set_threads(1)
    o.markers_to_nodes()
    for f in P2G_FIELDS:
        assert np.array_equal(o.field(f), ref[f]), f  # back to the serial loop


def test_threaded_marker_loop_keeps_accumulated_sums():
    # quirk Q1 (sums kept across steps): the threads add to what the sums
    # already hold, as the serial loop does
    o1, _, _ = fresh("c0", quirk_accumulate_sums=1)
    o2, _, _ = fresh("c0", quirk_accumulate_sums=1)
    o2.set_threads(4)
    for _ in range(2):
        o1.markers_to_nodes()
        o2.markers_to_nodes()
    for f in P2G_FIELDS:
        a, b = o1.field(f), o2.field(f)
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(a)), f
