"""Ensemble members advanced concurrently equal the same members run alone."""
import numpy as np
import pytest

import hmec
from hmec import synth
from hmec.ensemble import Ensemble

pytestmark = pytest.mark.gpu

FIELDS = ("pt", "vxs", "vys", "pf", "SXX", "SXY", "VSLIPB", "OM0", "ETA00")


def test_concurrent_members_bit_identical_to_solo_runs():
    # uneven sizes: the members' smoothing launches have different shared-
    # memory layouts while they run concurrently
    members = synth.ensemble_members(6, seed=77, side=(21, 121))
    common = dict(krylov_rtol=1e-15, form=hmec.FORM_MIXED)
    ens = Ensemble(members, **common)
    reps = ens.step(3)
    assert all(r["rc"] == 0 for rs in reps for r in rs)
    got = [{f: m.field(f) for f in FIELDS} for m in ens.models]
    ens.close()
    for k, (over, mat, seed) in enumerate(members):
        p = hmec.default_params(**dict(over, **common))
        m = hmec.Model(p)
        mk, nodes = synth.instance_state(p, mat, seed)
        m.upload_markers(mk)
        for key, v in nodes.items():
            m.upload_field(key, v)
        for _ in range(3):
            m.timestep()
        for f in FIELDS:
            assert np.array_equal(m.field(f), got[k][f]), (k, f)
        m.close()
