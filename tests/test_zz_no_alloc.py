"""The allocation-free markers -> nodes entry point.

hmec_markers_to_nodes_noalloc() is for hosts that may not call cudaMalloc
(an application that owns the device allocator and forbids allocations
behind its back, a real-time loop that must not block on the allocator).  It
keeps its scratch in a fixed array compiled into the library and must
produce the node fields of the context path, hmec_markers_to_nodes(), on the
same markers, to the 1e-13 of the marker->node parity tests (the two sum in
different orders).  Configuration 1 (1,000,000 markers, 160,000 half cells)
sits just inside both of its limits; the clustered case sends long half-cell
segments through the radix sort.  This file is collected last so a failure
here never hides another test; it passes alone in a fresh process and after
the rest of the suite.
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


def _setup(preset, mk=None):
    import torch

    p = hmec.default_params(**pairs.overrides(preset))
    if mk is None:
        mk, nodes = synth.make_state(p, preset)
    else:
        nodes = None
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


def _clustered(preset):
    """The preset's markers with 40 % moved into one cell and 5 % onto the far
    corner of the domain (clamped into the last cell)."""
    p = hmec.default_params(**pairs.overrides(preset))
    mk, _ = synth.make_state(p, preset)
    dx, dy = p.xsize / (p.Nx - 1), p.ysize / (p.Ny - 1)
    rng = np.random.default_rng(7)
    n = len(mk["xm"])
    pick = rng.permutation(n)
    a, b = pick[: int(0.4 * n)], pick[int(0.4 * n): int(0.45 * n)]
    mk = {k: v.copy() for k, v in mk.items()}
    mk["xm"][a] = 3 * dx + rng.uniform(0.1, 0.9, a.size) * dx
    mk["ym"][a] = 2 * dy + rng.uniform(0.1, 0.9, a.size) * dy
    mk["xm"][b] = p.xsize
    mk["ym"][b] = p.ysize
    return mk


@pytest.mark.parametrize("case", ["c0", "c1", "ref-clustered"])
def test_noalloc_matches_context_path_on_two_calls(case):
    import torch

    preset = case.split("-")[0]
    mk0 = _clustered(preset) if case.endswith("clustered") else None
    p, mk, nodes, dev_mk, dev_out, shapes, mk_ptrs, f_ptrs = _setup(preset, mk0)
    # 1e-13, or for cells with very many markers the accumulation error of
    # their sums: the context path adds in double-float (48-bit
    # significands), this one in FP64 (markers in the fullest cell x 2^-45)
    dx, dy = p.xsize / (p.Nx - 1), p.ysize / (p.Ny - 1)
    cj = np.clip(np.trunc(mk["xm"] / dx).astype(np.int64), 0, p.Nx - 2)
    ci = np.clip(np.trunc(mk["ym"] / dy).astype(np.int64), 0, p.Ny - 2)
    tol = max(1e-13, int(np.bincount(cj * (p.Ny - 1) + ci).max()) * 2.0 ** -45)
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
            assert float(np.max(np.abs(got - ref[f]))) / den < tol, (call, f, tol)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    p, mk, nodes, dev_mk, dev_out, shapes, mk_ptrs, f_ptrs = _setup("tiny")
    lib = hmec.load()
    # too many markers: rejected before any device access
    assert lib.hmec_markers_to_nodes_noalloc(C.byref(p), mk_ptrs, MAX_MARKERS + 1, f_ptrs, None) == -1
    # too many half cells: 4 * (Nx-1) * (Ny-1) > 262144
    big = hmec.default_params(Nx=1001, Ny=401, xsize=40000.0, ysize=16000.0)
    assert lib.hmec_markers_to_nodes_noalloc(C.byref(big), mk_ptrs, 10, f_ptrs, None) == -1
