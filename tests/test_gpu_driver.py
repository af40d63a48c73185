"""The C++ host loop (driver/hmec_run.cpp) drives the library like main() does."""
import os
import subprocess

import numpy as np
import pytest

import hmec
from hmec import build as B
from hmec import synth

pytestmark = pytest.mark.gpu


def test_driver_writes_reference_outputs(tmp_path):
    exe = B.build_driver()
    steps, Nx, Ny, xs, ys = 4, 21, 11, 4000.0, 2000.0
    out = subprocess.run([exe, str(steps), str(Nx), str(Ny), str(xs), str(ys), "--outdir", str(tmp_path)],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.count("total time:") == steps
    data = open(os.path.join(tmp_path, "EVO_data.txt")).read().split("\n")
    assert len([l for l in data if l.strip()]) == steps
    vslip = [l.split() for l in open(os.path.join(tmp_path, "EVO_Vslip.txt")) if l.strip()]
    assert len(vslip) == steps and len(vslip[-1]) == 2 + Nx
    # the same model through the Python binding
    p = hmec.default_params(Nx=Nx, Ny=Ny, xsize=xs, ysize=ys)
    m = hmec.Model(p)
    mk, nodes = synth.reference_state(p)
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    for _ in range(steps):
        r = m.timestep()
    row = m.field("VSLIPB")[int((Ny - 1) / 2.0)]
    got = np.array([float(v) for v in vslip[-1][2:]])
    assert np.allclose(got, row, rtol=1e-5, atol=0)
    assert float(vslip[-1][0]) == pytest.approx(r["timesum"], rel=1e-5)
