"""Checkpoint files: the reference's layout, the stub container, EVO trimming.

The layout (dataset names and order, groups, file stem) is checked against
tests/golden/checkpoint_layout.json, extracted from the reference's save
block by tests/golden/make_checkpoint_layout.py.  No GPU: the container is
exercised with synthetic arrays; the restart itself is in
test_gpu_checkpoint.py.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "h-mecs-2d_gb300"))

from hmec import checkpoint as ck  # noqa: E402

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "checkpoint_layout.json")))


def test_layout_matches_the_reference():
    assert list(ck.MATRIX_BASIC) == GOLD["matrix_basic"]
    assert list(ck.MATRIX_STAGGERED) == GOLD["matrix_staggered"]
    assert list(ck.HISTORY) == GOLD["history"]
    assert list(ck.MARKERS) == GOLD["markers"]
    assert list(ck.VALUES) == GOLD["values"]
    assert GOLD["groups"][:3] == ["Matrix", "Vector", "Value"]
    assert ck.file_name(500, GOLD["nname"], stub=False) == "h_mec_500.h5"


def test_driver_layout_matches_the_reference():
    from hmec import build as B

    try:
        exe = B.build_driver()
    except Exception as e:  # no library or compiler in this environment
        pytest.skip("driver not built: %s" % e)
    out = subprocess.run([exe, "--print-layout"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    got = json.loads(out.stdout)
    for k in ("matrix_basic", "matrix_staggered", "history", "markers", "values"):
        assert got[k] == GOLD[k], k


def test_stub_container_round_trip_in_c_order(tmp_path):
    rng = np.random.default_rng(3)
    Ny, Nx = 7, 5
    items = [("Matrix", n, rng.standard_normal((Ny, Nx))) for n in ck.MATRIX_BASIC]
    items += [("Matrix", n, rng.standard_normal((Ny + 1, Nx + 1))) for n in ck.MATRIX_STAGGERED]
    items += [("Vector", n, rng.standard_normal(11)) for n in ck.HISTORY]
    items += [("Vector", n, rng.standard_normal(13)) for n in ck.MARKERS]
    items.append(("Value", "values", rng.standard_normal(9)))
    p = str(tmp_path / ck.file_name(3, stub=True))
    ck.write_stub(p, items)
    back = ck.read(p)
    assert list(back) == [(g, n) for g, n, _ in items]  # write order kept
    for g, n, a in items:
        assert back[(g, n)].shape == a.shape and np.array_equal(back[(g, n)], a), (g, n)
    # the first matrix's bytes are its rows one after another (C order)
    raw = open(p, "rb").read()
    head = 8 + 4 + 2 + len(b"Matrix") + 2 + len(ck.MATRIX_BASIC[0]) + 1 + 16
    first = np.frombuffer(raw[head:head + 8 * Ny * Nx], dtype="<f8")
    assert np.array_equal(first, items[0][2].ravel(order="C"))


CXX_PROBE = r"""
#include <cstdio>
#include "checkpoint.hpp"
int main(int argc, char** argv) {
    std::vector<ckpt::Dataset> ds;
    if (argc > 2) {  // read the container argv[1], print every dataset's sum
        if (!ckpt::read_stub(argv[1], ds)) return 2;
        for (const auto& d : ds) {
            double s = 0;
            for (size_t k = 0; k < d.v.size(); k++) s += d.v[k] * (double)(k + 1);
            std::printf("%s %s %zu %.17g\n", d.group.c_str(), d.name.c_str(), d.dims.size(), s);
        }
        return 0;
    }
    // write: a 3 x 2 matrix 0..5 (C order) and a vector of 4
    ds.push_back({"Matrix", "SIIB", {3, 2}, {0, 1, 2, 3, 4, 5}});
    ds.push_back({"Vector", "xm", {4}, {1.5, -2.5, 3.25, 1e-300}});
    return ckpt::write_stub(argv[1], ds) ? 0 : 1;
}
"""


def _probe(tmp_path):
    import shutil

    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "probe.cpp"
    src.write_text(CXX_PROBE)
    exe = tmp_path / "probe"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "h-mecs-2d_gb300", "driver"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def test_cpp_and_python_containers_agree(tmp_path):
    exe = _probe(tmp_path)
    # C++ writes, Python reads
    p = str(tmp_path / "cpp.h5.stub")
    assert subprocess.run([exe, p]).returncode == 0
    d = ck.read(p)
    assert list(d) == [("Matrix", "SIIB"), ("Vector", "xm")]
    assert np.array_equal(d[("Matrix", "SIIB")], np.arange(6.0).reshape(3, 2))
    assert np.array_equal(d[("Vector", "xm")], [1.5, -2.5, 3.25, 1e-300])
    # Python writes, C++ reads
    rng = np.random.default_rng(9)
    items = [("Matrix", "OM0", rng.standard_normal((5, 4))), ("Value", "values", rng.standard_normal(9))]
    q = str(tmp_path / "py.h5.stub")
    ck.write_stub(q, items)
    out = subprocess.run([exe, q, "read"], capture_output=True, text=True)
    assert out.returncode == 0
    lines = out.stdout.split("\n")
    for (g, n, a), line in zip(items, lines):
        group, name, rank, s = line.split()
        flat = np.ascontiguousarray(a).ravel(order="C")
        want = float(np.sum(flat * np.arange(1, flat.size + 1)))
        assert (group, name, int(rank)) == (g, n, a.ndim)
        assert float(s) == pytest.approx(want, rel=1e-12)


def test_stub_rejects_other_files(tmp_path):
    p = tmp_path / "x.h5.stub"
    p.write_bytes(b"not a checkpoint")
    with pytest.raises(ValueError):
        ck.read_stub(str(p))


def test_trim_evo_keeps_the_saved_steps(tmp_path):
    for name in ("EVO_Vslip.txt", "EVO_vxD.txt", "EVO_data.txt"):
        (tmp_path / name).write_text("".join("line %d\n" % k for k in range(1, 9)))
    ck.trim_evo(str(tmp_path), 5)
    for name in ("EVO_Vslip.txt", "EVO_vxD.txt", "EVO_data.txt"):
        assert (tmp_path / name).read_text() == "".join("line %d\n" % k for k in range(1, 6))
