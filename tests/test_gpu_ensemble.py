"""An ensemble in one library context equals its members run alone.

The members are instances of one context (hmec_create with n_instances > 1),
each with its own grid; hmec_timestep advances all of them, after the first
step as one CUDA graph launch in which every member's loops (global
iterations, FGMRES restarts, Arnoldi steps) and adaptive dt are decided on
the device for that member alone.  Members never exchange data, so each one's
fields are bit-identical to the same member in a context of its own.
"""
import numpy as np
import pytest

import hmec
from hmec import synth
from hmec.ensemble import Ensemble, Sequential

pytestmark = pytest.mark.gpu

FIELDS = ("pt", "vxs", "vys", "pf", "SXX", "SXY", "VSLIPB", "OM0", "ETA00", "SII")


@pytest.mark.parametrize("form", [hmec.FORM_MIXED, hmec.FORM_FP64])
def test_packed_members_bit_identical_to_solo_runs(form):
    # uneven sizes: the members' smoothing launches have different shared-
    # memory layouts while they run concurrently
    members = synth.ensemble_members(6, seed=77, side=(21, 121))
    common = dict(krylov_rtol=1e-15, form=form)
    ens = Ensemble(members, **common)
    assert len(ens) == 6 and ens.graph_status == 0
    l0 = ens.launches
    reps = ens.step(4)
    assert ens.graph_status == 1, "the ensemble steps did not run as one graph"
    assert all(r["rc"] == 0 for rs in reps for r in rs), reps
    assert ens.launches > l0
    got = [{f: m.field(f) for f in FIELDS} for m in ens.members]
    dts = [m.scalar("dt") for m in ens.members]
    ens.close()
    solo = Sequential(members, **common)
    solo_reps = solo.step(4)
    for k, m in enumerate(solo.models):
        for f in FIELDS:
            assert np.array_equal(m.field(f), got[k][f]), (k, f)
        assert m.scalar("dt") == dts[k]
        assert [r["global_iters"] for r in solo_reps[k]] == [r["global_iters"] for r in reps[k]]
        assert [r["krylov_iters"] for r in solo_reps[k]] == [r["krylov_iters"] for r in reps[k]]
    solo.close()


def test_member_data_entry_points_address_their_instance():
    members = synth.ensemble_members(3, seed=5, side=(21, 41))
    ens = Ensemble(members, krylov_rtol=1e-15)
    shapes = [m.shape("pt") for m in ens.members]
    assert len(set(shapes)) > 1  # uneven grids
    for k, m in enumerate(ens.members):
        m.set_scalar("timesum", 100.0 + k)
    for k, m in enumerate(ens.members):
        assert m.scalar("timesum") == 100.0 + k
        assert m.field("pt").shape == shapes[k]
    ens.close()
