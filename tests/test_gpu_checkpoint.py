"""Restart from a checkpoint continues the run (cpp/h_mec_rsf_v9.cpp:211-282).

A model checkpointed after step 3 and restored into a fresh model must reach
the state of the uninterrupted run after step 5, within the whole-step
tolerance of the parity tests (the restored solve starts from a zero Krylov
guess, so the two runs differ by the solver tolerance, not bit for bit).
The same holds for the C++ host loop's --savestep / --restart.
"""
import os
import subprocess

import numpy as np
import pytest

import pairs
from hmec import checkpoint as ck

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_DARCY = 1e-6


class _Fields:
    def __init__(self, d):
        self.d = d

    def field(self, f):
        return self.d[f]


def test_python_checkpoint_restart_continues_the_run(tmp_path):
    m = pairs.model_for("tiny")
    h = ck.History(64)
    for _ in range(3):
        r = m.timestep()
        h.record(m, r["timestep"])
    assert r["timestep"] == 3
    path = str(tmp_path / ck.file_name(3, stub=True))
    ck.save(m, path, h)
    for _ in range(2):
        m.timestep()
    ref = {f: m.field(f) for f in pairs.STEP_FIELDS}
    ref_time = m.scalar("timesum")
    m.close()

    m2 = pairs.model_for("tiny")
    h2 = ck.History(64)
    ck.load(m2, path, 3, h2)
    for k in ck.HISTORY:
        assert np.array_equal(h2.v[k], h.v[k]), k
    for _ in range(2):
        r2 = m2.timestep()
    assert r2["timestep"] == 5
    err = pairs.group_errors(m2, _Fields(ref))
    strict = {k: v for k, v in err.items() if k != "darcy"}
    assert max(strict.values()) < TOL, err
    assert err["darcy"] < TOL_DARCY, err
    assert m2.scalar("timesum") == pytest.approx(ref_time, rel=1e-12)
    m2.close()


def test_driver_savestep_and_restart(tmp_path):
    from hmec import build as B

    exe = B.build_driver()
    full, rest = tmp_path / "full", tmp_path / "rest"
    full.mkdir()
    rest.mkdir()
    args = ["51", "51", "10000", "10000", "--mixed"]
    r = subprocess.run([exe, "5"] + args + ["--outdir", str(full), "--savestep", "3"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert (full / "h_mec_3.h5.stub").exists() and (full / "file.txt").read_text().strip() == "3"
    r = subprocess.run([exe, "3"] + args + ["--outdir", str(rest), "--savestep", "3"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    # a later step's lines in the output directory, then the restart drops them
    with open(rest / "EVO_data.txt", "a") as f:
        f.write("stale line of an interrupted run\n")
    r = subprocess.run([exe, "2"] + args + ["--outdir", str(rest), "--restart", "3"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    a = np.loadtxt(full / "EVO_data.txt")
    b = np.loadtxt(rest / "EVO_data.txt")
    assert a.shape == b.shape == (5, 5)
    assert np.array_equal(a[:3], b[:3])
    # steps 4 and 5: time, dt, Vmax and iteration counts, as printed (six
    # significant digits, so a last-digit rounding step is allowed)
    np.testing.assert_allclose(b[3:], a[3:], rtol=1e-5, atol=1e-300)
    vs_a, vs_b = np.loadtxt(full / "EVO_Vslip.txt"), np.loadtxt(rest / "EVO_Vslip.txt")
    assert vs_a.shape == vs_b.shape
    np.testing.assert_allclose(vs_b[3:], vs_a[3:], rtol=1e-5, atol=1e-30)
    assert os.path.getsize(rest / "h_mec_3.h5.stub") == os.path.getsize(full / "h_mec_3.h5.stub")
