"""The allocation-free markers -> nodes entry point.

hmec_markers_to_nodes_noalloc() is for hosts that may not call cudaMalloc
(an application that owns the device allocator, code under CUDA-graph
capture, a real-time loop that must not block on the allocator).  It keeps
its scratch in a fixed array compiled into the library and must produce the
node fields of the context path, hmec_markers_to_nodes(), on the same
markers.  This file is collected last so a failure here never hides another
test; it passes alone in a fresh process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import hmec
import pairs
from hmec import synth
from pairs import P2G_FIELDS

pytestmark = pytest.mark.gpu

MAX_MARKERS = 1 << 20


def _setup(preset):
    import torch

    p = hmec.default_params(**pairs.overrides(preset))
    mk, nodes = synth.make_state(p, preset)
    # device inputs and outputs are the caller's (allocated here by torch)
    dev_mk = [torch.from_numpy(np.ascontiguousarray(mk[k])).cuda() for k in hmec.MARKERS]
    shapes = {}
    for f in hmec.FIELDS:
        g = hmec.load().hmec_field_grid(hmec.FIELDS.index(f))
        shapes[f] = (p.Ny + g, p.Nx + g)
    dev_out = {f: torch.zeros(shapes[f][0] * shapes[f][1], dtype=torch.float64, device="cuda") for f in P2G_FIELDS}
    mk_ptrs = (C.POINTER(C.c_double) * len(dev_mk))(*[C.cast(t.data_ptr(), C.POINTER(C.c_double)) for t in dev_mk])
    f_ptrs = (C.POINTER(C.c_double) * len(hmec.FIELDS))()
    for f, t in dev_out.items():
        f_ptrs[hmec.FIELDS.index(f)] = C.cast(t.data_ptr(), C.POINTER(C.c_double))
    return p, mk, nodes, dev_mk, dev_out, shapes, mk_ptrs, f_ptrs


def test_noalloc_matches_context_path_on_two_calls():
    import torch

    p, mk, nodes, dev_mk, dev_out, shapes, mk_ptrs, f_ptrs = _setup("c0")
    m = hmec.Model(p)
    m.upload_markers(mk)
    m.markers_to_nodes()
    ref = {f: m.field(f) for f in P2G_FIELDS}
    m.close()
    lib = hmec.load()
    n = len(mk["xm"])
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):  # the shared scratch keeps the first call's contents
        rc = lib.hmec_markers_to_nodes_noalloc(C.byref(p), mk_ptrs, n, f_ptrs, stream)
        assert rc == 0, call
        torch.cuda.synchronize()
        for f in P2G_FIELDS:
            got = dev_out[f].cpu().numpy().reshape(shapes[f], order="F")
            den = float(np.max(np.abs(ref[f]))) or 1.0
            assert float(np.max(np.abs(got - ref[f]))) / den < 1e-13, (call, f)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    p, mk, nodes, dev_mk, dev_out, shapes, mk_ptrs, f_ptrs = _setup("tiny")
    lib = hmec.load()
    # too many markers: rejected before any device access
    assert lib.hmec_markers_to_nodes_noalloc(C.byref(p), mk_ptrs, MAX_MARKERS + 1, f_ptrs, None) == -1
    # too many half cells: 4 * (Nx-1) * (Ny-1) > 262144
    big = hmec.default_params(Nx=1001, Ny=401, xsize=40000.0, ysize=16000.0)
    assert lib.hmec_markers_to_nodes_noalloc(C.byref(big), mk_ptrs, 10, f_ptrs, None) == -1
