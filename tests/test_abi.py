"""The C ABI library loads without a GPU and exports what include/hmec.h declares."""
import ctypes as C
import os
import re

import pytest

import hmec
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "hmec.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hmec_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    assert header_functions() == sorted(hmec.EXPORTS)


def test_library_exports_every_declared_symbol():
    lib = hmec.load()
    missing = [f for f in header_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_params_struct_layout_matches_oracle_mirror():
    assert C.sizeof(hmec.Params) == C.sizeof(O.HmecParams)
    assert [f for f, _ in hmec.Params._fields_] == [f for f, _ in O.HmecParams._fields_]
    for (n1, t1), (n2, t2) in zip(hmec.Params._fields_, O.HmecParams._fields_):
        assert getattr(hmec.Params, n1).offset == getattr(O.HmecParams, n2).offset
        assert C.sizeof(t1) == C.sizeof(t2)


def test_default_params_agree_with_oracle_constants():
    a = hmec.default_params()
    b = O.default_params()
    for name, _ in hmec.Params._fields_:
        va, vb = getattr(a, name), getattr(b, name)
        if isinstance(va, C.Array):
            assert list(va) == list(vb), name
        else:
            assert va == vb, name
    # a few values of cpp/constants.hpp
    assert (a.Nx, a.Ny, a.xsize, a.ysize) == (401, 51, 40000.0, 10000.0)
    assert (a.dtelastic0, a.dtmin, a.V0, a.PTFDIFF) == (5e8, 1e-4, 1e-9, 3e7)
    assert (a.niterglobal, a.ynlastmax, a.dtstep) == (10000, 499, 5)


def test_field_tables():
    lib = hmec.load()
    for k, name in enumerate(hmec.FIELDS):
        assert lib.hmec_field_name(k).decode() == name
        assert lib.hmec_field_grid(k) == (1 if k >= hmec.FIELDS.index("pt") else 0)
    assert lib.hmec_field_name(len(hmec.FIELDS)) is None
    assert lib.hmec_field_grid(-1) == -1
    for k, name in enumerate(hmec.MARKERS):
        assert lib.hmec_marker_name(k).decode() == name
    for k, name in enumerate(hmec.SCALARS):
        assert lib.hmec_scalar_name(k).decode() == name
    assert len(hmec.MARKERS) == 19


def test_marknum_formula():
    p = hmec.default_params()
    assert hmec.load().hmec_marknum(C.byref(p)) == (401 - 1) * 4 * (51 - 1) * 4 == 320000
    p = hmec.default_params(Nx=51, Ny=51)
    assert hmec.load().hmec_marknum(C.byref(p)) == 40000


def test_create_rejects_bad_params_without_touching_a_device():
    # argument validation happens before any CUDA call
    p = hmec.default_params(Nx=2)
    st = C.c_int32(0)
    h = hmec.load().hmec_create(C.byref(p), 1, None, C.byref(st))
    assert not h and st.value == -1
    # an ensemble needs at least one instance
    q = hmec.default_params()
    st = C.c_int32(0)
    h = hmec.load().hmec_create(C.byref(q), 0, None, C.byref(st))
    assert not h and st.value == -1
    # a member's grid is checked like the shared one
    grids = (hmec.Grid * 2)(hmec.Grid(51, 51, 1e4, 1e4, 4, 4), hmec.Grid(3, 51, 1e4, 1e4, 4, 4))
    st = C.c_int32(0)
    h = hmec.load().hmec_create(C.byref(q), 2, grids, C.byref(st))
    assert not h and st.value == -1


def test_no_cpu_fallback_in_product():
    # the product package never imports the oracle
    pkg = os.path.join(ROOT, "h-mecs-2d_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "hmec_oracle" not in text, f


def test_tuning_table_entry_nearest_in_cells(tmp_path, monkeypatch):
    """hmec_tune_params applies the table entry of the same form nearest the
    grid in cells (what hmec_create does with autotune set)."""
    import json

    table = {"version": 1, "entries": [
        {"Nx": 201, "Ny": 201, "form": 1, "mg_levels": 4, "mg_pre": 1, "mg_post": 1, "mg_coarse_sweeps": 6,
         "bs_stencil": 128, "bs_sort": 512, "krylov_blocks": 456, "smooth_blocks": 152, "ms_per_step": 1.0},
        {"Nx": 201, "Ny": 201, "form": 0, "mg_levels": 6, "mg_pre": 2, "mg_post": 2, "mg_coarse_sweeps": 4,
         "bs_stencil": 64, "bs_sort": 256, "krylov_blocks": 304, "smooth_blocks": 0},
        {"Nx": 1001, "Ny": 401, "form": 1, "mg_levels": 3, "mg_pre": 2, "mg_post": 2, "mg_coarse_sweeps": 8,
         "bs_stencil": 256, "bs_sort": 128, "krylov_blocks": 608, "smooth_blocks": 0, "note": "text is skipped"}]}
    path = tmp_path / "table.json"
    path.write_text(json.dumps(table))
    monkeypatch.setenv("HMEC_TUNE_TABLE", str(path))
    lib = hmec.load()
    p = hmec.default_params(Nx=181, Ny=221, form=hmec.FORM_MIXED)
    assert lib.hmec_tune_params(C.byref(p)) == 1
    assert (p.mg_levels, p.mg_pre, p.mg_post, p.mg_coarse_sweeps) == (4, 1, 1, 6)
    assert (p.bs_stencil, p.bs_sort, p.krylov_blocks, p.smooth_blocks) == (128, 512, 456, 152)
    p = hmec.default_params(Nx=201, Ny=201, form=hmec.FORM_FP64)
    assert lib.hmec_tune_params(C.byref(p)) == 1 and p.mg_levels == 6
    p = hmec.default_params(Nx=901, Ny=451, form=hmec.FORM_MIXED)
    assert lib.hmec_tune_params(C.byref(p)) == 1 and p.mg_levels == 3 and p.bs_stencil == 256
    # nothing within 4x in cells: unchanged
    p = hmec.default_params(Nx=41, Ny=41, form=hmec.FORM_MIXED)
    assert lib.hmec_tune_params(C.byref(p)) == 0 and p.mg_levels == 5
    # no table
    monkeypatch.setenv("HMEC_TUNE_TABLE", str(tmp_path / "missing.json"))
    p = hmec.default_params(Nx=201, Ny=201, form=hmec.FORM_MIXED)
    assert lib.hmec_tune_params(C.byref(p)) == 0 and p.mg_levels == 5
