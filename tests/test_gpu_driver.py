"""The C++ host loop (driver/hmec_run.cpp) drives the library like main() does.

Its output files follow the reference's (cpp/h_mec_rsf_v9.cpp:1739-1805):
EVO_*.txt lines of time, dt and the fault row as Eigen prints a row vector
(each coefficient right-aligned to the widest one's %g text, one space
apart), EVO_data.txt in setw(20) columns, x_fault.txt (the node abscissae,
one per line) and rsf_fault.txt (the a, b, L rows) at step 1.  The printed
values are checked against the CPU oracle run on the same model.
"""
import os
import subprocess

import numpy as np
import pytest

import hmec
import oracle as O
from hmec import build as B
from hmec import synth

pytestmark = pytest.mark.gpu


def eigen_row(v, column=False):
    t = ["%g" % x for x in v]
    w = max(len(s) for s in t)
    return ("\n" if column else " ").join(s.rjust(w) for s in t)


def test_driver_writes_reference_outputs(tmp_path):
    exe = B.build_driver()
    steps, Nx, Ny, xs, ys = 4, 21, 11, 4000.0, 2000.0
    out = subprocess.run([exe, str(steps), str(Nx), str(Ny), str(xs), str(ys), "--outdir", str(tmp_path)],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert out.stdout.count("total time:") == steps
    data = open(os.path.join(tmp_path, "EVO_data.txt")).read().split("\n")
    assert len([l for l in data if l.strip()]) == steps
    assert all(len(l) == 100 for l in data if l.strip())  # five setw(20) columns
    # the same model on the oracle
    po = O.default_params(Nx=Nx, Ny=Ny, xsize=xs, ysize=ys)
    o = O.Oracle(po)
    mk, nodes = synth.reference_state(po)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    lf = int((Ny - 1) / 2.0)
    series = {"EVO_Vslip.txt": "VSLIPB", "EVO_viscosity.txt": "ETA", "EVO_press_flu.txt": "pf",
              "EVO_SigmaY.txt": "SigmaY", "EVO_Theta.txt": "OM", "EVO_Visc_comp.txt": "VIS_COMP"}
    lines = {f: [l.rstrip("\n") for l in open(os.path.join(tmp_path, f)) if l.strip()] for f in series}
    for s in range(steps):
        o.timestep()
        for f, name in series.items():
            line = lines[f][s]
            head, row = line.split("    ", 2)[:2], line.split("    ", 2)[2]
            ref = o.field(name)[lf]
            got = np.array([float(v) for v in row.split()])
            assert got.shape == ref.shape, (f, s)
            # %g keeps six significant digits: half a unit of the sixth is
            # up to 5e-6 relative
            assert np.allclose(got, ref, rtol=1e-5, atol=1e-300), (f, s, got, ref)
            assert float(head[0]) == pytest.approx(o.scalar("timesum"), rel=1e-5), (f, s)
            # the Eigen layout of the printed values
            assert row == eigen_row(got), (f, s, row)
    # step 1 files
    x = [float(v) for v in open(os.path.join(tmp_path, "x_fault.txt")).read().split()]
    assert np.allclose(x, synth.linspaced(Nx, 0, xs), rtol=1e-5)
    xt = open(os.path.join(tmp_path, "x_fault.txt")).read()
    assert xt == eigen_row(np.array(x), column=True) + "\n"
    rsf = open(os.path.join(tmp_path, "rsf_fault.txt")).read().split("\n\n")
    assert len(rsf) == 3
    for part, name in zip(rsf, ("ARSF", "BRSF", "LRSF")):
        got = np.array([float(v) for v in part.split()])
        assert np.allclose(got, o.field(name)[lf], rtol=1e-5), name


def test_download_rows_equals_field_rows():
    p = hmec.default_params(**synth.PRESETS["tiny"])
    m = hmec.Model(p)
    mk, nodes = synth.make_state(p, "tiny")
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    m.timestep()
    names = ["VSLIPB", "pf", "ETA", "vxD", "SigmaY"]
    for row in (0, 5, p.Ny - 1):
        got = m.rows(row, names)
        for n in names:
            assert np.array_equal(got[n], m.field(n)[row]), (row, n)
    with pytest.raises(hmec.HmecError):
        m.rows(p.Ny + 5, names)
    m.close()


def _tiny_model(**extra):
    p = hmec.default_params(**dict(synth.PRESETS["tiny"], **extra))
    m = hmec.Model(p)
    mk, nodes = synth.make_state(p, "tiny")
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    return m, p


def test_download_rows_async_overlaps_the_next_step():
    """The copy of a step's rows started before the next step returns that
    step's rows (bit for bit), into page-locked and into pageable memory."""
    m, p = _tiny_model()
    names = ["VSLIPB", "pf", "ETA", "vxD", "SigmaY", "VIS_COMP"]
    lf = int((p.Ny - 1) / 2.0)
    n = sum(m.shape(k)[1] for k in names)
    pinned = [hmec.HostArray(n), hmec.HostArray(n)]
    try:
        want, tickets = [], []
        for s in range(4):
            m.timestep()
            want.append(m.rows(lf, names))
            buf = pinned[s & 1].a if s != 2 else np.empty(n)  # step 3's copy goes to pageable memory
            tickets.append((m.rows_async(lf, names, buf), buf, s))
            if s >= 1:
                t, b, k = tickets[s - 1]
                m.rows_wait(t)
                got = np.concatenate([want[k][x] for x in names])
                assert np.array_equal(b, got), k
        t, b, k = tickets[-1]
        m.rows_wait(t)
        assert np.array_equal(b, np.concatenate([want[k][x] for x in names]))
        with pytest.raises(hmec.HmecError):
            m.rows_wait(tickets[-1][0] + 1)
        with pytest.raises(hmec.HmecError):
            m.rows_async(p.Ny + 5, names, pinned[0].a)
    finally:
        m.close()
        for h in pinned:
            h.close()


def test_invariants_every_skips_output_fields_between_output_steps():
    """invariants_every = 3: steps 1 and 2 write the output-only invariants on
    the fault line only, step 3 everywhere; every state field (and the fault
    row the EVO series print) equals the every-step run bit for bit."""
    inv = ["EII", "EIIVP", "SII", "DIS", "pt_ave", "pf_ave", "VIS_COMP", "EL_DECOM"]
    a, p = _tiny_model(invariants_every=1)
    b, _ = _tiny_model(invariants_every=3)
    lf = int((p.Ny - 1) / 2.0)
    try:
        for s in (1, 2, 3):
            a.timestep()
            b.timestep()
            for f in ["vxs", "vys", "pt", "pf", "SXX", "SYY", "SXY", "SXX0", "SYY0", "EXX", "EYY", "OM", "ETA"]:
                assert np.array_equal(a.field(f), b.field(f)), (s, f)
            for f in inv:
                fa, fb = a.field(f), b.field(f)
                assert np.array_equal(fa[lf], fb[lf]), (s, f)
                if s == 3:
                    assert np.array_equal(fa, fb), (s, f)
                else:
                    rest = np.delete(np.arange(fa.shape[0]), [0, lf])
                    assert not np.array_equal(fa[rest], fb[rest]), (s, f)
    finally:
        a.close()
        b.close()
