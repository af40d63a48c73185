"""Helpers that set up the CPU oracle and the GPU library on identical inputs."""
from __future__ import annotations

import numpy as np

import oracle as O
from hmec import synth

# Solver settings shared by the parity tests: FGMRES to 1e-15 on the
# row-equilibrated residual.
SOLVER = dict(krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000)

# Fields compared after a section / step (velocity, pressure, stress, slip rate, state).
STEP_FIELDS = ["pt", "vxs", "vys", "pf", "vxD", "vyD", "SXX", "SYY", "SXY", "VSLIPB", "OM", "OM0", "ETA",
               "ETA00", "SigmaY", "PT0", "PF0", "VX0", "VY0", "VXF0", "VYF0", "SXX0", "SYY0", "SXY0", "ESP",
               "EXY", "EXX", "EYY", "EII", "SII", "DIS", "VIS_COMP", "EL_DECOM"]

P2G_FIELDS = ["RHO", "KKK", "TTT", "GGG", "ETA0", "COHT", "FRIT", "COHC", "FRIC", "DILC",
              "RHOY", "ETADY", "RHOFY", "PORY", "RHOX", "ETADX", "RHOFX", "PORX",
              "ETAP", "POR", "ETAB0", "ETAP0", "GGGP"]


def overrides(preset: str, **extra) -> dict:
    over = dict(synth.PRESETS[preset])
    over.update(SOLVER)
    over.update(extra)
    return over


def oracle_for(preset: str, **extra):
    p = O.default_params(**overrides(preset, **extra))
    o = O.Oracle(p)
    mk, nodes = synth.make_state(p, preset)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    return o, mk, nodes


def model_for(preset: str, mk=None, nodes=None, **extra):
    import hmec

    p = hmec.default_params(**overrides(preset, **extra))
    m = hmec.Model(p)
    if mk is None:
        mk, nodes = synth.make_state(p, preset)
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    return m


def field_errors(m, o, names):
    out = {}
    for f in names:
        a = m.field(f)
        b = o.field(f)
        den = float(np.max(np.abs(b)))
        out[f] = float(np.max(np.abs(a - b))) / den if den > 0 else float(np.max(np.abs(a - b)))
    return out


# Error groups: a vector field is compared as a whole (its components relative
# to the largest component), so a component that is zero by symmetry (vys in
# simple shear) is not held against its own round-off.
GROUPS = {
    "velocity": ["vxs", "vys"],
    "darcy": ["vxD", "vyD"],
    "pt": ["pt"],
    "pf": ["pf"],
    "stress": ["SXX", "SYY", "SXY"],
    "slip_rate": ["VSLIPB"],
    "state": ["OM"],
}


# The output-only invariants (cpp/h_mec_rsf_v9.cpp:1523-1557) and the state
# rolled over to the next step (:1658-1726), compared like the solution.
# EL_DECOM is a difference quotient of pressure changes over a step and
# VXF0/VYF0 carry the Darcy velocity; they are held to the Darcy tolerance.
GROUPS_ALL = dict(GROUPS)
GROUPS_ALL.update({
    "invariants": ["EII", "EIIVP", "SII", "DIS", "VIS_COMP"],
    "rollover": ["PT0", "PF0", "PTF0", "SXX0", "SYY0", "SXY0", "VX0", "VY0"],
    "fluid_rollover": ["VXF0", "VYF0"],
    "el_decom": ["EL_DECOM"],
})
#: groups held to the Darcy tolerance instead of the solution's
LOOSE_GROUPS = ("darcy", "fluid_rollover", "el_decom")


def group_errors(m, o, groups=GROUPS):
    out = {}
    for g, names in groups.items():
        num = 0.0
        den = 0.0
        for f in names:
            a, b = m.field(f), o.field(f)
            num = max(num, float(np.max(np.abs(a - b))))
            den = max(den, float(np.max(np.abs(b))))
        out[g] = num / den if den > 0 else num
    return out


def solution_errors(xg, x):
    """Grouped relative errors of a solution vector S (6 unknowns per cell)."""
    S, G = x.reshape(-1, 6), xg.reshape(-1, 6)
    idx = {"pt": [0], "velocity": [1, 2], "pf": [3], "darcy": [4, 5]}
    out = {}
    for g, cols in idx.items():
        num = max(float(np.max(np.abs(G[:, c] - S[:, c]))) for c in cols)
        den = max(float(np.max(np.abs(S[:, c]))) for c in cols)
        out[g] = num / den if den > 0 else num
    return out


class OracleView:
    """Gives an oracle the field() accessor of a Model (for group_errors)."""

    def __init__(self, o):
        self.o = o

    def field(self, name):
        return self.o.field(name)


def bisection_resolution(o):
    """Relative slip-rate resolution of the reference's fault-stress bisection.

    The bisection of cpp/h_mec_rsf_v9.cpp:1224 stops at |dS| <= 1e-3 Pa and
    V ~ sinh(S / (a prB)), so V is determined to about 1e-3 / (a prB).
    """
    p = o.params
    i = int((p.Ny - 1) / 2.0)
    j = np.arange(p.Nx)
    pt, pf = o.field("pt"), o.field("pf")
    blk = lambda f: f[i, j] + f[i + 1, j] + f[i, j + 1] + f[i + 1, j + 1]
    prb = np.maximum((blk(pt) - blk(pf)) / 4.0, 1e3)
    a = o.field("ARSF")[i]
    return float(1e-3 / np.min(a * prb))
