"""Initial states for the H-MEC hot path (section a21).

``reference_state`` restates the reference's own initialisation:
cpp/h_mec_rsf_v9.cpp:188-209 (marker lattice and block/fault material) and
:283-338 (RSF parameters on nodes, state variable, PT0/PF0), with the values
of cpp/constants.hpp.  ``config_state`` builds the seeded synthetic models of
the benchmark configurations on the same skeleton (jittered markers,
per-marker permeability, viscosity fields, RSF patch, overpressure).

The generator is host input synthesis: identical arrays are fed to the GPU
library and to the CPU oracle, so both start from the same bytes.
"""
from __future__ import annotations

import math

import numpy as np

# --------------------------------------------------------------- presets

#: Extra parameter overrides per named preset (applied on top of
#: hmec_params_default(), which holds cpp/constants.hpp).
PRESETS = {
    # cpp/constants.hpp as shipped: 401 x 51 nodes, 40 km x 10 km
    "ref": {},
    # the reference material model on a small grid (fast tests); transition
    # abscissae scaled with the domain
    "tiny": dict(Nx=21, Ny=11, xsize=4000.0, ysize=2000.0, TS_1=200.0, TS_2=400.0, TS_3=3400.0, TS_4=3800.0),
    "small": dict(Nx=41, Ny=21, xsize=8000.0, ysize=4000.0, TS_1=400.0, TS_2=800.0, TS_3=6800.0, TS_4=7600.0),
    # benchmark configuration 0: 10 km x 10 km, 51 x 51, 4 x 4 markers per cell
    "c0": dict(Nx=51, Ny=51, xsize=10000.0, ysize=10000.0, mx=4, my=4,
               TS_1=2500.0, TS_2=3000.0, TS_3=7000.0, TS_4=7500.0,
               arsfm=(0.017, 0.011), brsfm=(0.017, 0.017), lrsfm=(0.02, 0.02),
               V0=1e-6, PCONF=7e7, PTFDIFF=3e7),
    # configuration 1: same material model, 201 x 201, 5 x 5 markers per cell
    "c1": dict(Nx=201, Ny=201, xsize=10000.0, ysize=10000.0, mx=5, my=5,
               TS_1=2500.0, TS_2=3000.0, TS_3=7000.0, TS_4=7500.0,
               arsfm=(0.017, 0.011), brsfm=(0.017, 0.017), lrsfm=(0.02, 0.02),
               V0=1e-6, PCONF=7e7, PTFDIFF=3e7),
    # configuration 2: 40 km x 16 km, 1001 x 401, 6 x 6 markers per cell
    "c2": dict(Nx=1001, Ny=401, xsize=40000.0, ysize=16000.0, mx=6, my=6,
               TS_1=17500.0, TS_2=18000.0, TS_3=22000.0, TS_4=22500.0,
               arsfm=(0.017, 0.011), brsfm=(0.017, 0.017), lrsfm=(0.02, 0.02),
               V0=1e-6, PCONF=7e7, PTFDIFF=3e7),
}

#: Material description of each synthetic configuration.
MATERIALS = {
    "c0": dict(host_eta=1e23, host_eta_sigma_dec=0.0, host_por=0.01, host_k=(1e-20, 1e-20), host_fric=0.6,
               fault_eta=1e21, fault_por=0.05, fault_k=(1e-17, 1e-15), fault_fric=0.6,
               v_init=1e-9, overpressure=0.10, jitter=True),
    "c1": dict(host_eta=1e23, host_eta_sigma_dec=0.0, host_por=0.01, host_k=(1e-20, 1e-20), host_fric=0.6,
               fault_eta=1e21, fault_por=0.05, fault_k=(1e-17, 1e-15), fault_fric=0.6,
               v_init=1e-9, overpressure=0.10, jitter=True),
    "c2": dict(host_eta=1e22, host_eta_sigma_dec=1.0, host_por=0.01, host_k=(1e-21, 1e-14), host_fric=0.6,
               fault_eta=1e19, fault_por=0.05, fault_k=(1e-21, 1e-14), fault_fric=0.6,
               v_init=1e-9, overpressure=0.10, jitter=True),
}

SEEDS = {"c0": 1000, "c1": 1001, "c2": 1002}

MARKER_NAMES = ["xm", "ym", "t_marker", "rhom", "etasm", "etam", "cohescm", "cohestm", "frictcm", "dilatcm",
                "fricttm", "porm", "kkkm", "sxxm", "syym", "sxym", "gm", "rhofm", "etafm"]


def linspaced(n: int, low: float, high: float) -> np.ndarray:
    """Eigen 3.3 LinSpaced for |high| >= |low|: low + i*step, last point == high."""
    step = (high - low) / float(n - 1) if n > 1 else 0.0
    out = low + np.arange(n, dtype=np.float64) * step
    out[-1] = high
    return out


def derived(p) -> dict:
    """Quantities cpp/constants.hpp derives from the grid constants."""
    dx = p.xsize / (p.Nx - 1)
    dy = p.ysize / (p.Ny - 1)
    return dict(dx=dx, dy=dy, line_fault=int((p.Ny - 1) / 2.0),
                lower_block=p.ysize / 2.0 + dy, upper_block=p.ysize / 2.0 - dy,
                Nx_markers=(p.Nx - 1) * p.mx, Ny_markers=(p.Ny - 1) * p.my)


def _marker_lattice(p, rng=None):
    """:188-191 -- regular lattice; rand()%1 is always 0, so no jitter unless rng is given."""
    d = derived(p)
    nxm, nym = d["Nx_markers"], d["Ny_markers"]
    dxms = p.xsize / float(nxm)
    dyms = p.ysize / float(nym)
    m = np.arange(nxm * nym, dtype=np.int64)
    col = (m // nym).astype(np.float64)
    row = (m % nym).astype(np.float64)
    if rng is None:
        ux = np.zeros(m.shape)
        uy = np.zeros(m.shape)
    else:
        ux = rng.random(m.shape[0])
        uy = rng.random(m.shape[0])
    xm = 0.0 + col * dxms + ux * dxms
    ym = 0.0 + row * dyms + uy * dyms
    return xm, ym


def reference_markers(p) -> dict:
    """Marker arrays of :188-209 with the defaults of constants.hpp:153-173."""
    d = derived(p)
    xm, ym = _marker_lattice(p)
    n = xm.shape[0]
    mk = {k: np.zeros(n) for k in MARKER_NAMES}
    mk["xm"], mk["ym"] = xm, ym
    mk["t_marker"][:] = 1
    mk["rhom"][:] = 2800
    mk["etasm"][:] = 1e21
    mk["cohescm"][:] = p.cohes
    mk["cohestm"][:] = p.cohes
    mk["frictcm"][:] = 0.5
    mk["dilatcm"][:] = p.dilatation
    mk["fricttm"][:] = p.tensile
    mk["kkkm"][:] = 2e-16
    mk["gm"][:] = p.shearmod
    mk["rhofm"][:] = 1000
    mk["etafm"][:] = 1e-3
    mk["porm"][:] = 0.01 * (1 + 0.0 * (0 - 0.5))
    mk["etam"] = mk["etasm"] * np.exp(-p.alpha * mk["porm"])
    blk = (ym < d["upper_block"]) | (ym > d["lower_block"])
    mk["t_marker"][blk] = -1
    mk["etam"][blk] = 1e23
    mk["etasm"][blk] = 1e23
    mk["rhom"][blk] = 2800
    mk["kkkm"][blk] = 2e-16
    mk["cohescm"][blk] = p.cohes * 1e3
    mk["cohestm"][blk] = p.cohes * 1e3
    mk["frictcm"][blk] = 0.8
    mk["dilatcm"][blk] = p.dilatation
    mk["fricttm"][blk] = p.tensile
    return mk


def reference_nodes(p) -> dict:
    """Node fields of the fresh start :283-338 (all other fields are zero)."""
    d = derived(p)
    Nx, Ny = p.Nx, p.Ny
    x = linspaced(Nx, 0.0, p.xsize)
    y = linspaced(Ny, 0.0, p.ysize)
    OM0 = np.full((Ny, Nx), float(p.omm[0]), order="F")
    ARSF = np.full((Ny, Nx), float(p.arsfm[1]), order="F")
    BRSF = np.full((Ny, Nx), float(p.brsfm[1]), order="F")
    LRSF = np.full((Ny, Nx), float(p.lrsfm[0]), order="F")
    a0, a1 = p.arsfm[0], p.arsfm[1]
    b0, b1 = p.brsfm[0], p.brsfm[1]
    l0, l1 = p.lrsfm[0], p.lrsfm[1]
    for i in range(Ny):
        if y[i] > d["upper_block"] and y[i] < d["lower_block"]:
            for j in range(Nx):
                OM0[i, j] = p.omm[1]
                xj = x[j]
                if xj < p.TS_1:
                    BRSF[i, j] = b0
                    ARSF[i, j] = a0
                if xj >= p.TS_1 and xj < p.TS_2:
                    t = (xj - p.TS_1) / (p.TS_2 - p.TS_1)
                    BRSF[i, j] = b0 - (b0 - b1) * t
                    ARSF[i, j] = a0 - (a0 - a1) * t
                    LRSF[i, j] = l0 - (l0 - l1) * t
                if xj >= p.TS_2 and xj <= p.TS_3:
                    LRSF[i, j] = l1
                if xj > p.TS_3 and xj <= p.TS_4:
                    t = (xj - p.TS_3) / (p.TS_4 - p.TS_3)
                    BRSF[i, j] = b1 - (b1 - b0) * t
                    ARSF[i, j] = a1 - (a1 - a0) * t
                    LRSF[i, j] = l1 - (l1 - l0) * t
                if xj > p.TS_4:
                    BRSF[i, j] = b0
                    ARSF[i, j] = a0
    fields = dict(OM0=OM0, OM=OM0.copy(), ARSF=ARSF, BRSF=BRSF, LRSF=LRSF,
                  PT0=np.full((Ny + 1, Nx + 1), p.PCONF + p.PTFDIFF, order="F"),
                  PF0=np.full((Ny + 1, Nx + 1), p.PCONF, order="F"))
    return fields


def reference_state(p):
    """(markers, node fields) of a fresh reference run (file.txt == 0)."""
    return reference_markers(p), reference_nodes(p)


def config_state(p, name: str, seed: int | None = None, mat: dict | None = None):
    """Seeded synthetic model of benchmark configuration ``name`` (or material ``mat``) on params ``p``."""
    mat = MATERIALS[name] if mat is None else mat
    seed = SEEDS[name] if seed is None else seed
    rng = np.random.default_rng(seed)
    d = derived(p)
    xm, ym = _marker_lattice(p, rng if mat["jitter"] else None)
    n = xm.shape[0]
    mk = {k: np.zeros(n) for k in MARKER_NAMES}
    mk["xm"], mk["ym"] = xm, ym
    fault = ~((ym < d["upper_block"]) | (ym > d["lower_block"]))
    blk = ~fault
    mk["t_marker"][:] = np.where(fault, 1.0, -1.0)
    mk["rhom"][:] = 2800
    mk["gm"][:] = p.shearmod
    mk["rhofm"][:] = 1000
    mk["etafm"][:] = 1e-3
    mk["fricttm"][:] = p.tensile
    mk["dilatcm"][:] = p.dilatation
    mk["cohescm"][:] = p.cohes
    mk["cohestm"][:] = p.cohes
    mk["porm"][:] = np.where(fault, mat["fault_por"], mat["host_por"])
    mk["frictcm"][:] = np.where(fault, mat["fault_fric"], mat["host_fric"])

    def loguniform(lo, hi, size):
        if lo == hi:
            return np.full(size, lo)
        return np.exp(math.log(lo) + rng.random(size) * (math.log(hi) - math.log(lo)))

    kk = np.empty(n)
    kk[fault] = loguniform(*mat["fault_k"], int(fault.sum()))
    kk[blk] = loguniform(*mat["host_k"], int(blk.sum()))
    mk["kkkm"][:] = kk
    eta_host = np.full(int(blk.sum()), mat["host_eta"])
    if mat["host_eta_sigma_dec"] > 0:
        eta_host = mat["host_eta"] * 10.0 ** (mat["host_eta_sigma_dec"] * rng.standard_normal(eta_host.shape[0]))
    mk["etasm"][blk] = eta_host
    mk["etasm"][fault] = mat["fault_eta"]
    # :194 for fault markers; :199 (etam = etasm) for block markers
    mk["etam"][:] = np.where(fault, mk["etasm"] * np.exp(-p.alpha * mk["porm"]), mk["etasm"])
    nodes = reference_nodes(p)
    # initial slip rate v_init on the fault rows: steady state of the aging
    # law, OM0 = ln(V0 / V)
    om_fault = math.log(p.V0 / mat["v_init"])
    y = linspaced(p.Ny, 0.0, p.ysize)
    frows = (y > d["upper_block"]) & (y < d["lower_block"])
    nodes["OM0"][frows, :] = om_fault
    nodes["OM"] = nodes["OM0"].copy()
    # pore pressure: PCONF everywhere, plus the overpressure on the fault rows
    yp = linspaced(p.Ny + 1, -d["dy"] / 2.0, p.ysize + d["dy"] / 2.0)
    prow = (yp > d["upper_block"]) & (yp < d["lower_block"])
    nodes["PF0"][prow, :] = p.PCONF * (1.0 + mat["overpressure"])
    # a cycle-phase offset: a uniform shear pre-stress (the stress the
    # previous step leaves, SXY0) -- above the fault's steady-state strength
    # the first step starts a rupture (dt of milliseconds), below it the
    # instance stays interseismic
    if mat.get("prestress", 0.0) > 0.0:
        nodes["SXY0"] = np.full((p.Ny, p.Nx), float(mat["prestress"]))
    return mk, nodes


def make_state(p, preset: str, seed: int | None = None):
    if preset in MATERIALS:
        return config_state(p, preset, seed)
    return reference_state(p)


def ensemble_members(n: int = 64, seed: int = 1003, side=(51, 301), mpc: int = 4):
    """Parameter overrides of the instances of an ensemble (configuration 3).

    Each instance: per-side node counts uniform in ``side`` (uneven grids),
    ``mpc`` x ``mpc`` markers per cell, the configuration-0 material model on a
    10 km x 10 km domain, and per-instance rate-and-state a in [0.008, 0.016]
    and b in [0.012, 0.020] on the velocity-weakening patch, L in
    [0.005, 0.05] m, and a fault permeability log-uniform in [1e-18, 1e-14] m^2.
    Returns a list of (overrides, material) pairs for ``instance_state``.
    """
    rng = np.random.default_rng(seed)
    out = []
    base = dict(PRESETS["c0"])
    for k in range(n):
        nx = int(rng.integers(side[0], side[1] + 1))
        ny = int(rng.integers(side[0], side[1] + 1))
        a = float(rng.uniform(0.008, 0.016))
        b = float(rng.uniform(0.012, 0.020))
        L = float(rng.uniform(0.005, 0.05))
        kf = float(np.exp(np.log(1e-18) + rng.random() * (np.log(1e-14) - np.log(1e-18))))
        over = dict(base, Nx=nx, Ny=ny, mx=mpc, my=mpc, arsfm=(0.017, a), brsfm=(b, b), lrsfm=(L, L))
        mat = dict(MATERIALS["c0"], fault_k=(kf, kf))
        out.append((over, mat, seed * 1000 + k))
    return out


#: configuration 4: cycle phases of the instances (fraction, uniform shear
#: pre-stress in Pa): interseismic from rest, late interseismic, and in
#: rupture from the first step (16 MPa exceeds the fault's steady-state
#: strength of about 15.9 MPa at 1e-9 m/s under 24.6 MPa effective pressure)
C4_PHASES = ((0.6, 0.0), (0.2, 14e6), (0.2, 16e6))


def ensemble_members_c4(n: int = 256, seed: int = 1004):
    """The instances of configuration 4: per-side node counts uniform in
    101..401 (x) and 101..201 (y), 4 x 4 markers per cell, friction and
    fault permeability drawn as in configuration 3, and a seeded cycle phase
    per instance (C4_PHASES) so that some instances rupture while others
    load interseismically."""
    rng = np.random.default_rng(seed)
    out = []
    base = dict(PRESETS["c0"])
    cum = np.cumsum([f for f, _ in C4_PHASES])
    for k in range(n):
        nx = int(rng.integers(101, 402))
        ny = int(rng.integers(101, 202))
        a = float(rng.uniform(0.008, 0.016))
        b = float(rng.uniform(0.012, 0.020))
        L = float(rng.uniform(0.005, 0.05))
        kf = float(np.exp(np.log(1e-18) + rng.random() * (np.log(1e-14) - np.log(1e-18))))
        phase = C4_PHASES[int(np.searchsorted(cum, rng.random() * cum[-1], side="right"))][1]
        over = dict(base, Nx=nx, Ny=ny, mx=4, my=4, arsfm=(0.017, a), brsfm=(b, b), lrsfm=(L, L))
        mat = dict(MATERIALS["c0"], fault_k=(kf, kf), prestress=phase)
        out.append((over, mat, seed * 1000 + k))
    return out


def instance_state(p, mat: dict, seed: int):
    """Initial state of one ensemble instance (configuration-0 skeleton, member material)."""
    return config_state(p, "c0", seed, mat=mat)
