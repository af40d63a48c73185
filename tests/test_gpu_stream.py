"""Marker streaming (hmec_stream_markers): every timestep copies the host's
page-locked marker arrays into the device after its markers->nodes section,
overlapped with the rest of the step, so step k+1 uses what the arrays held
while step k ran.  The streamed run equals, bit for bit, a run that uploads
the same marker sets before each step (graph-launched and host-driven
steps), including markers whose positions move (a new half-cell order)."""
import numpy as np
import pytest

import hmec
from hmec import synth

pytestmark = pytest.mark.gpu

FIELDS = ["vxs", "vys", "pt", "pf", "SXY", "SXX", "ETA", "RHO", "VSLIPB", "OM"]


def _model(p, mk, nodes):
    m = hmec.Model(p)
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    return m


def _sets(p, mk, n=3):
    rng = np.random.default_rng(7)
    dx, dy = p.xsize / (p.Nx - 1) / p.mx, p.ysize / (p.Ny - 1) / p.my
    out = []
    for k in range(n):
        s = {f: v.copy() for f, v in mk.items()}
        s["rhom"] = mk["rhom"] * (1.0 + 0.01 * k)
        s["xm"] = np.clip(mk["xm"] + rng.uniform(-0.3, 0.3, mk["xm"].shape) * dx, 0.0, p.xsize * (1 - 1e-12))
        s["ym"] = np.clip(mk["ym"] + rng.uniform(-0.3, 0.3, mk["ym"].shape) * dy, 0.0, p.ysize * (1 - 1e-12))
        out.append(s)
    return out


@pytest.mark.parametrize("graph", [1, 0])
def test_streamed_markers_equal_uploads_before_each_step(graph):
    p = hmec.default_params(**dict(synth.PRESETS["tiny"], graph=graph))
    mk, nodes = synth.make_state(p, "tiny")
    sets = _sets(p, mk)
    a = _model(p, sets[0], nodes)
    b = _model(p, sets[0], nodes)
    host = {f: hmec.HostArray(len(mk["xm"])) for f in hmec.MARKERS}
    try:
        for f in hmec.MARKERS:
            host[f].a[...] = sets[1][f]
        a.stream_markers({f: host[f].a for f in hmec.MARKERS})
        for step in range(4):
            ra = a.timestep()
            rb = b.timestep()
            assert ra["global_iters"] == rb["global_iters"] and ra["dt"] == rb["dt"], (step, ra, rb)
            for f in FIELDS:
                assert np.array_equal(a.field(f), b.field(f)), (step, f)
            # what a streamed during this step, b uploads now
            nxt = sets[min(step + 1, 2)]
            b.upload_markers(nxt)
            if step + 2 <= 2:
                for f in hmec.MARKERS:
                    host[f].a[...] = sets[step + 2][f]
        got, want = a.download_markers(), b.download_markers()
        for f in hmec.MARKERS:
            assert np.array_equal(got[f], want[f]), f
        if graph:
            assert a.graph_status == 1
        a.stream_markers(None)
        a.timestep()
    finally:
        a.close()
        b.close()
        for h in host.values():
            h.close()


def test_stream_markers_refusals():
    p = hmec.default_params(**synth.PRESETS["tiny"])
    mk, nodes = synth.make_state(p, "tiny")
    m = _model(p, mk, nodes)
    try:
        with pytest.raises(hmec.HmecError):
            m.stream_markers({f: np.ascontiguousarray(mk[f]) for f in hmec.MARKERS})  # pageable
    finally:
        m.close()
    p2 = hmec.default_params(**dict(synth.PRESETS["tiny"], advect_markers=1))
    m2 = _model(p2, mk, nodes)
    host = {f: hmec.HostArray(len(mk["xm"])) for f in hmec.MARKERS}
    try:
        with pytest.raises(hmec.HmecError):
            m2.stream_markers({f: host[f].a for f in hmec.MARKERS})
    finally:
        m2.close()
        for h in host.values():
            h.close()


def test_batched_field_transfers_equal_single_ones():
    import ctypes as C

    p = hmec.default_params(**synth.PRESETS["tiny"])
    mk, nodes = synth.make_state(p, "tiny")
    m = _model(p, mk, nodes)
    try:
        m.timestep()
        names = ["vxs", "pt", "SXY", "ETA", "VSLIPB", "OM0"]
        ids = (C.c_int32 * len(names))(*[hmec.FIELDS.index(n) for n in names])
        bufs = [np.zeros(m.shape(n), order="F") for n in names]
        ptrs = (C.POINTER(C.c_double) * len(names))(*[b.ctypes.data_as(C.POINTER(C.c_double)) for b in bufs])
        m._check(m.L.hmec_download_fields(m.h, 0, len(names), ids, ptrs), "download_fields")
        for n, b in zip(names, bufs):
            assert np.array_equal(b, m.field(n)), n
        rng = np.random.default_rng(3)
        for b in bufs:
            b[...] = rng.standard_normal(b.shape)
        m._check(m.L.hmec_upload_fields(m.h, 0, len(names), ids, ptrs), "upload_fields")
        for n, b in zip(names, bufs):
            assert np.array_equal(m.field(n), b), n
        bad = (C.c_int32 * 1)(10_000)
        assert m.L.hmec_download_fields(m.h, 0, 1, bad, ptrs) == -1  # HMEC_ERR_ARG
    finally:
        m.close()
