"""The synthetic configurations' generators (CPU): the ensemble members of
configurations 3 and 4 and the cycle-phase offsets of configuration 4."""
import numpy as np

import hmec
from hmec import synth


def test_config4_instances_ranges_and_phases():
    members = synth.ensemble_members_c4(256)
    assert len(members) == 256
    nx = np.array([o["Nx"] for o, _, _ in members])
    ny = np.array([o["Ny"] for o, _, _ in members])
    assert nx.min() >= 101 and nx.max() <= 401 and ny.min() >= 101 and ny.max() <= 201
    assert all(o["mx"] == 4 and o["my"] == 4 for o, _, _ in members)
    a = np.array([o["arsfm"][1] for o, _, _ in members])
    b = np.array([o["brsfm"][1] for o, _, _ in members])
    L = np.array([o["lrsfm"][1] for o, _, _ in members])
    kf = np.array([m["fault_k"][0] for _, m, _ in members])
    assert a.min() >= 0.008 and a.max() <= 0.016 and b.min() >= 0.012 and b.max() <= 0.020
    assert L.min() >= 0.005 and L.max() <= 0.05 and kf.min() >= 1e-18 and kf.max() <= 1e-14
    phases = np.array([m["prestress"] for _, m, _ in members])
    for frac, tau in synth.C4_PHASES:
        share = float(np.mean(phases == tau))
        assert abs(share - frac) < 0.1, (tau, share)
    # seeded: the same list every time
    assert synth.ensemble_members_c4(256)[17] == members[17]


def test_prestress_offset_sets_the_previous_stress():
    over, mat, seed = [m for m in synth.ensemble_members_c4(64) if m[1]["prestress"] > 0][0]
    p = hmec.default_params(**dict(over, Nx=31, Ny=21))
    mk, nodes = synth.instance_state(p, mat, seed)
    assert nodes["SXY0"].shape == (p.Ny, p.Nx) and np.all(nodes["SXY0"] == mat["prestress"])
    mk0, nodes0 = synth.instance_state(p, dict(mat, prestress=0.0), seed)
    assert "SXY0" not in nodes0
    assert np.array_equal(mk["xm"], mk0["xm"])
