"""The timestep as one CUDA graph launch.

With hmec_params.graph = 1 (the default) every timestep after the first runs
as one graph launch: the global-iteration loop, the FGMRES restart loop and
the Arnoldi loop are conditional nodes whose conditions the device sets
(cpp/h_mec_rsf_v9.cpp:610-1457, the reference's loop with a direct solve per
iteration).  The graph launches the same kernels in the same order as the
host-driven step, so the two give bit-identical fields, reports and dt.
"""
import numpy as np
import pytest

import hmec
import pairs

pytestmark = pytest.mark.gpu

FIELDS = ["pt", "vxs", "vys", "pf", "vxD", "vyD", "SXX", "SXY", "VSLIPB", "OM", "ETA", "SII", "EL_DECOM", "PT0"]


def _pair(preset, form, **extra):
    o, mk, nodes = pairs.oracle_for(preset)
    a = pairs.model_for(preset, mk, nodes, form=form, graph=1, **extra)
    b = pairs.model_for(preset, mk, nodes, form=form, graph=0, **extra)
    return a, b


@pytest.mark.parametrize("form", [hmec.FORM_MIXED, hmec.FORM_FP64])
@pytest.mark.parametrize("preset", ["tiny", "c0"])
def test_graph_steps_equal_host_driven_steps(preset, form):
    a, b = _pair(preset, form)
    assert a.graph_status == 0 and b.graph_status == -1
    for step in range(5):
        ra, rb = a.timestep(), b.timestep()
        if step >= 1:
            assert a.graph_status == 1, a.graph_error()
        for k in ("timestep", "global_iters", "ynlast", "krylov_iters", "status"):
            assert ra[k] == rb[k], (step, k, ra, rb)
        assert ra["dt"] == rb["dt"] and ra["timesum"] == rb["timesum"] and ra["Vmax"] == rb["Vmax"], (ra, rb)
        assert ra["max_krylov_relres"] == rb["max_krylov_relres"], (ra, rb)
        for f in FIELDS:
            assert np.array_equal(a.field(f), b.field(f)), (step, f)
    # the launch count of a graph step follows from its loop trip counts
    la, lb = a.launches, b.launches
    a.timestep()
    b.timestep()
    da, db = a.launches - la, b.launches - lb
    assert da > 0 and db > 0
    # host-driven steps launch Arnoldi steps past convergence (the host looks
    # at the flag only now and then); graph steps run the restart body's tail
    # (least squares, update) in the converged cycle too
    assert abs(da - db) <= 0.35 * db, (da, db)
    a.close()
    b.close()


def test_graph_rupture_phase_and_advection():
    """A rupture-phase step (many global iterations, dt of milliseconds) and
    marker advection inside the graph."""
    o, mk, nodes = pairs.oracle_for("c0")
    for _ in range(3):
        o.timestep()
    snap = o.snapshot()
    snap["SXY0"] = np.full_like(snap["SXY0"], 16e6)
    for adv in (0, 1):
        a = pairs.model_for("c0", mk, nodes, graph=1, advect_markers=adv)
        b = pairs.model_for("c0", mk, nodes, graph=0, advect_markers=adv)
        for m in (a, b):
            m.timestep()  # the host-driven first step of a (lazy set-up)
            m.load_state(snap)
        for step in range(3):
            ra, rb = a.timestep(check=False), b.timestep(check=False)
            assert a.graph_status == 1
            assert ra["status"] == rb["status"] and ra["rc"] == rb["rc"], (ra, rb)
            assert ra["global_iters"] == rb["global_iters"] and ra["dt"] == rb["dt"], (ra, rb)
            assert ra["krylov_iters"] == rb["krylov_iters"], (ra, rb)
            for f in FIELDS:
                assert np.array_equal(a.field(f), b.field(f)), (adv, step, f)
        if adv:
            ma, mb = a.download_markers(), b.download_markers()
            for k in ("xm", "ym", "sxym"):
                assert np.array_equal(ma[k], mb[k]), k
        a.close()
        b.close()


def test_graph_reports_statuses_like_the_host_path():
    """A solve that runs out of iterations and a fault-stress bisection that
    hits its cap are reported by the graph as by the host-driven step."""
    o, mk, nodes = pairs.oracle_for("tiny")
    for extra, code in ((dict(krylov_maxit=1, krylov_restart=2), -6), (dict(rsf_maxit=1), -5)):
        for _ in range(1):
            a = pairs.model_for("tiny", mk, nodes, graph=1, **extra)
            b = pairs.model_for("tiny", mk, nodes, graph=0, **extra)
            for s in range(4):
                ra, rb = a.timestep(check=False), b.timestep(check=False)
                if s >= 1:
                    assert a.graph_status == 1
                assert ra["global_iters"] == rb["global_iters"], (extra, s, ra, rb)
            assert code in (ra["rc"], ra["status"]) and code in (rb["rc"], rb["status"]), (extra, ra, rb)
            a.close()
            b.close()
