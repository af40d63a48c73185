"""The half-cell counting sort on markers that cluster.

Markers normally spread a few per half cell, and each segment of the sorted
order is put in marker-index order by one thread.  When many markers share a
half cell (they cluster, or coordinates outside the domain are clamped into
an edge cell by check_bounds, cpp/h_mec_rsf_v9.cpp:144-151), the long
segments are left to the stable radix sort instead.  Both must give the
oracle's node fields and be bit-identical across runs.  The tolerance is the
1e-13 of the marker->node parity tests (the summation order differs from the
reference's serial marker loop), widened for cells that hold very many
markers to the accumulation error of their sums: the GPU adds in
double-float (48-bit significands), the oracle in FP64, so the difference
grows like the number of markers in the fullest cell times 2^-45.
"""
import numpy as np
import pytest

import pairs
from pairs import P2G_FIELDS

pytestmark = pytest.mark.gpu


def tolerance(mk, p):
    """max(1e-13, (markers in the fullest cell) x 2^-45)."""
    dx, dy = p.xsize / (p.Nx - 1), p.ysize / (p.Ny - 1)
    j = np.clip(np.trunc(mk["xm"] / dx).astype(np.int64), 0, p.Nx - 2)
    i = np.clip(np.trunc(mk["ym"] / dy).astype(np.int64), 0, p.Ny - 2)
    nmax = int(np.bincount(j * (p.Ny - 1) + i).max())
    return max(1e-13, nmax * 2.0 ** -45)


def clustered(preset, frac=0.4, seed=11):
    """The preset's markers with a fraction moved into one cell and some onto
    the far corner of the domain, whose cell index fix(xsize/dx) = Nx-1 is
    clamped into the last cell by check_bounds."""
    o, mk, nodes = pairs.oracle_for(preset)
    p = o.params
    dx, dy = p.xsize / (p.Nx - 1), p.ysize / (p.Ny - 1)
    rng = np.random.default_rng(seed)
    n = len(mk["xm"])
    pick = rng.permutation(n)
    a, b = pick[: int(frac * n)], pick[int(frac * n): int((frac + 0.05) * n)]
    mk = {k: v.copy() for k, v in mk.items()}
    cx, cy = 3 * dx, 2 * dy
    mk["xm"][a] = cx + rng.uniform(0.1, 0.9, a.size) * dx
    mk["ym"][a] = cy + rng.uniform(0.1, 0.9, a.size) * dy
    mk["xm"][b] = p.xsize
    mk["ym"][b] = p.ysize
    o.set_markers(mk)
    return o, mk, nodes


@pytest.mark.parametrize("preset", ["tiny", "ref"])
def test_clustered_markers_match_oracle_and_repeat(preset):
    o, mk, nodes = clustered(preset)
    m = pairs.model_for(preset, mk, nodes)
    o.markers_to_nodes()
    m.markers_to_nodes()
    first = {f: m.field(f) for f in P2G_FIELDS}
    e = pairs.field_errors(m, o, P2G_FIELDS)
    assert max(e.values()) < tolerance(mk, o.params), (e, tolerance(mk, o.params))
    m.markers_to_nodes()
    for f in P2G_FIELDS:
        assert np.array_equal(first[f], m.field(f)), f


def test_clustered_and_spread_markers_in_one_model():
    """Upload spread markers, then clustered ones, then spread ones again:
    each P2G equals a fresh model's (the long-segment flag is cleared every
    step).  Nodes without markers keep their values (:536 etc.), so the
    outputs are cleared before each P2G, as in a fresh model."""
    o0, mk0, nodes = pairs.oracle_for("tiny")
    _, mk1, _ = clustered("tiny")
    m = pairs.model_for("tiny", mk0, nodes)
    ref0 = pairs.model_for("tiny", mk0, nodes)
    ref1 = pairs.model_for("tiny", mk1, nodes)
    ref0.markers_to_nodes()
    ref1.markers_to_nodes()
    for mk, ref in ((mk0, ref0), (mk1, ref1), (mk0, ref0)):
        m.upload_markers(mk)
        for f in P2G_FIELDS:
            m.upload_field(f, np.zeros(m.shape(f)))
        m.markers_to_nodes()
        for f in P2G_FIELDS:
            assert np.array_equal(m.field(f), ref.field(f)), f


def test_markers_stored_in_half_cell_order_round_trip():
    """The library stores markers in half-cell order; downloads return the
    caller's order, bit for bit, also after clustering and re-uploads."""
    o, mk, nodes = pairs.oracle_for("c0")
    _, mk1, _ = clustered("c0")
    m = pairs.model_for("c0", mk, nodes)
    for arrays in (mk, mk1, mk):
        m.upload_markers(arrays)
        got = m.download_markers()
        for k, v in arrays.items():
            assert np.array_equal(got[k], v), k
    m.markers_to_nodes()
    o.set_markers(mk)
    o.markers_to_nodes()
    e = pairs.field_errors(m, o, P2G_FIELDS)
    assert max(e.values()) < 1e-13, e
