"""hmec -- Python host binding of libhmec_gpu.so (GB300 H-MEC hot path).

A thin ctypes layer over the C ABI of include/hmec.h.  ``Model`` mirrors the
sections of the reference's main() (cpp/h_mec_rsf_v9.cpp:376-1726) one to one:
markers_to_nodes, timestep_begin, global_iteration, timestep_end,
advect_markers, or the whole ``timestep``.  There is no CPU fallback: if the
CUDA library is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from . import build as _build
from . import synth  # noqa: F401  (initial states)

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(os.path.dirname(_HERE))
HEADER = os.path.join(_ROOT, "include", "hmec.h")

HMEC_OK = 0
STATUS = {0: "HMEC_OK", -1: "HMEC_ERR_ARG", -2: "HMEC_ERR_CUDA", -3: "HMEC_ERR_BOUNDS", -4: "HMEC_ERR_NAN",
          -5: "HMEC_ERR_RSF_NOCONV", -6: "HMEC_ERR_KRYLOV_NOCONV", -7: "HMEC_ERR_NOMEM", -8: "HMEC_ERR_STATE",
          -9: "HMEC_ERR_TIMEOUT"}
FORM_FP64, FORM_MIXED = 0, 1
# hmec_params.mg_flags bits (include/hmec.h, enum hmec_mg_flags)
MG_DARCY_HARMONIC, MG_UNTILED, MG_PASS_LAUNCHES, MG_LOCAL_SWEEPS = 1, 2, 4, 8


class HmecError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


class Params(C.Structure):
    """ctypes mirror of ``hmec_params``."""

    _fields_ = [
        ("Nx", C.c_int32), ("Ny", C.c_int32), ("xsize", C.c_double), ("ysize", C.c_double),
        ("mx", C.c_int32), ("my", C.c_int32),
        ("TS_1", C.c_double), ("TS_2", C.c_double), ("TS_3", C.c_double), ("TS_4", C.c_double),
        ("dtelastic0", C.c_double), ("dtmin", C.c_double), ("inertia", C.c_double),
        ("arsfm", C.c_double * 2), ("brsfm", C.c_double * 2), ("lrsfm", C.c_double * 2), ("omm", C.c_double * 2),
        ("V0", C.c_double), ("alpha", C.c_double),
        ("POR0", C.c_double), ("cohes", C.c_double), ("friction", C.c_double), ("dilatation", C.c_double),
        ("tensile", C.c_double), ("shearmod", C.c_double), ("BETAFLUID", C.c_double), ("BETASOLID", C.c_double),
        ("gx", C.c_double), ("gy", C.c_double), ("PCONF", C.c_double), ("PTFDIFF", C.c_double),
        ("etamin", C.c_double), ("etamax", C.c_double), ("kkkmin", C.c_double), ("kkkmax", C.c_double),
        ("stpmax", C.c_double), ("stpmax1", C.c_double),
        ("bcupper", C.c_double), ("bclower", C.c_double), ("bcvyflower", C.c_double),
        ("niterglobal", C.c_int32), ("ynlastmax", C.c_int32), ("dtstep", C.c_int32),
        ("vratiomax", C.c_double), ("dtkoef", C.c_double), ("dtkoefup", C.c_double), ("dtkoefv", C.c_double),
        ("errmin", C.c_double), ("etawt", C.c_double), ("syieldmin", C.c_double), ("tyield", C.c_double),
        ("num_timesteps", C.c_int32),
        ("form", C.c_int32), ("krylov_rtol", C.c_double), ("krylov_restart", C.c_int32),
        ("krylov_maxit", C.c_int32), ("mg_levels", C.c_int32), ("mg_pre", C.c_int32), ("mg_post", C.c_int32),
        ("mg_coarse_sweeps", C.c_int32), ("rsf_maxit", C.c_int32), ("advect_markers", C.c_int32),
        ("rk4_as_written", C.c_int32), ("quirk_accumulate_sums", C.c_int32), ("bounds_check", C.c_int32),
        ("mg_flags", C.c_int32), ("graph", C.c_int32),
        ("bs_stencil", C.c_int32), ("bs_sort", C.c_int32), ("krylov_blocks", C.c_int32),
        ("smooth_blocks", C.c_int32), ("autotune", C.c_int32), ("invariants_every", C.c_int32),
        ("smooth_inverses", C.c_int32),
    ]


class IterReport(C.Structure):
    _fields_ = [("iterstep", C.c_int32), ("stop", C.c_int32), ("ynpl", C.c_int32), ("krylov_iters", C.c_int32),
                ("dt", C.c_double), ("DSYLSQ", C.c_double), ("ptscale", C.c_double), ("pfscale", C.c_double),
                ("Vmax", C.c_double), ("krylov_relres", C.c_double)]


class Grid(C.Structure):
    """ctypes mirror of ``hmec_grid`` (an instance's grid)."""

    _fields_ = [("Nx", C.c_int32), ("Ny", C.c_int32), ("xsize", C.c_double), ("ysize", C.c_double),
                ("mx", C.c_int32), ("my", C.c_int32)]


class StepReport(C.Structure):
    _fields_ = [("timestep", C.c_int32), ("global_iters", C.c_int32), ("ynlast", C.c_int32),
                ("krylov_iters", C.c_int32), ("status", C.c_int32), ("timesum", C.c_double), ("dt", C.c_double),
                ("Vmax", C.c_double), ("max_krylov_relres", C.c_double)]


def _xlist(macro: str):
    text = open(HEADER).read()
    start = text.index("#define %s(X)" % macro)
    body = []
    for line in text[start:].splitlines()[1:]:
        body.append(line)
        if not line.rstrip().endswith("\\"):
            break
    return re.findall(r"X\((\w+)", " ".join(body))


FIELDS = _xlist("HMEC_FIELD_LIST")
MARKERS = _xlist("HMEC_MARKER_LIST")
SCALARS = _xlist("HMEC_SCALAR_LIST")

#: every entry point include/hmec.h declares
EXPORTS = ["hmec_abi_version", "hmec_params_default", "hmec_field_name", "hmec_field_grid", "hmec_marker_name",
           "hmec_scalar_name", "hmec_marknum", "hmec_create", "hmec_destroy", "hmec_instances", "hmec_last_error",
           "hmec_upload_markers", "hmec_download_markers", "hmec_upload_field", "hmec_download_field",
           "hmec_download_rows", "hmec_download_rows_async", "hmec_rows_wait", "hmec_host_alloc", "hmec_host_free",
           "hmec_stream_markers", "hmec_upload_fields", "hmec_download_fields",
           "hmec_set_scalar", "hmec_get_scalar", "hmec_markers_to_nodes", "hmec_timestep_begin",
           "hmec_global_iteration", "hmec_timestep_end", "hmec_advect_markers", "hmec_timestep",
           "hmec_assemble_csr", "hmec_solve_system", "hmec_kernel_launches", "hmec_synchronize", "hmec_stream",
           "hmec_profile_kernel", "hmec_profile_read", "hmec_markers_to_nodes_noalloc", "hmec_cell_index",
           "hmec_graph_status", "hmec_tune_params"]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libhmec_gpu.so (building it first if needed); raises if impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libhmec_gpu.so is not built (%s)" % path)
        _build.build()
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    L.hmec_abi_version.restype = C.c_int32
    L.hmec_params_default.argtypes = [P(Params)]
    L.hmec_params_default.restype = None
    L.hmec_field_name.argtypes = [C.c_int32]
    L.hmec_field_name.restype = C.c_char_p
    L.hmec_field_grid.argtypes = [C.c_int32]
    L.hmec_field_grid.restype = C.c_int32
    L.hmec_marker_name.argtypes = [C.c_int32]
    L.hmec_marker_name.restype = C.c_char_p
    L.hmec_scalar_name.argtypes = [C.c_int32]
    L.hmec_scalar_name.restype = C.c_char_p
    L.hmec_marknum.argtypes = [P(Params)]
    L.hmec_marknum.restype = C.c_int64
    L.hmec_create.argtypes = [P(Params), C.c_int32, P(Grid), P(C.c_int32)]
    L.hmec_create.restype = vp
    L.hmec_destroy.argtypes = [vp]
    L.hmec_destroy.restype = None
    L.hmec_instances.argtypes = [vp]
    L.hmec_instances.restype = C.c_int32
    L.hmec_last_error.argtypes = [vp]
    L.hmec_last_error.restype = C.c_char_p
    i32 = C.c_int32
    L.hmec_upload_markers.argtypes = [vp, i32, P(P(C.c_double)), C.c_int64]
    L.hmec_download_markers.argtypes = [vp, i32, P(P(C.c_double)), C.c_int64]
    L.hmec_upload_field.argtypes = [vp, i32, i32, P(C.c_double), i32, i32]
    L.hmec_download_field.argtypes = [vp, i32, i32, P(C.c_double), i32, i32]
    L.hmec_download_rows.argtypes = [vp, i32, i32, i32, P(i32), P(C.c_double)]
    L.hmec_download_rows_async.argtypes = [vp, i32, i32, i32, P(i32), P(C.c_double), P(C.c_int64)]
    L.hmec_rows_wait.argtypes = [vp, i32, C.c_int64]
    L.hmec_stream_markers.argtypes = [vp, i32, P(P(C.c_double)), C.c_int64]
    L.hmec_upload_fields.argtypes = [vp, i32, i32, P(i32), P(P(C.c_double))]
    L.hmec_download_fields.argtypes = [vp, i32, i32, P(i32), P(P(C.c_double))]
    L.hmec_host_alloc.argtypes = [C.c_size_t]
    L.hmec_host_alloc.restype = vp
    L.hmec_host_free.argtypes = [vp]
    L.hmec_host_free.restype = None
    L.hmec_set_scalar.argtypes = [vp, i32, i32, C.c_double]
    L.hmec_get_scalar.argtypes = [vp, i32, i32, P(C.c_double)]
    for fn in ("hmec_markers_to_nodes", "hmec_timestep_begin", "hmec_timestep_end", "hmec_advect_markers"):
        getattr(L, fn).argtypes = [vp, i32]
        getattr(L, fn).restype = i32
    L.hmec_synchronize.argtypes = [vp]
    L.hmec_synchronize.restype = i32
    L.hmec_global_iteration.argtypes = [vp, i32, P(IterReport)]
    L.hmec_timestep.argtypes = [vp, P(StepReport)]
    L.hmec_assemble_csr.argtypes = [vp, i32, P(C.c_int64), P(i32), P(C.c_double), P(C.c_double), P(C.c_int64),
                                    P(C.c_double), P(C.c_double)]
    L.hmec_solve_system.argtypes = [vp, i32, P(C.c_double), P(C.c_double), P(i32), P(C.c_double)]
    L.hmec_kernel_launches.argtypes = [vp]
    L.hmec_kernel_launches.restype = C.c_int64
    L.hmec_graph_status.argtypes = [vp]
    L.hmec_graph_status.restype = i32
    L.hmec_stream.argtypes = [vp, i32]
    L.hmec_stream.restype = vp
    L.hmec_profile_kernel.argtypes = [vp, i32, C.c_char_p]
    L.hmec_profile_read.argtypes = [vp, i32, P(C.c_int64), P(C.c_double), P(C.c_double), P(C.c_double)]
    L.hmec_markers_to_nodes_noalloc.argtypes = [P(Params), P(P(C.c_double)), C.c_int64, P(P(C.c_double)), vp]
    L.hmec_markers_to_nodes_noalloc.restype = i32
    L.hmec_cell_index.argtypes = [P(C.c_double), C.c_int64, C.c_double, i32, P(i32)]
    L.hmec_cell_index.restype = i32
    L.hmec_tune_params.argtypes = [P(Params)]
    L.hmec_tune_params.restype = i32
    _lib = L
    return L


def default_params(**over) -> Params:
    p = Params()
    load().hmec_params_default(C.byref(p))
    for k, v in over.items():
        cur = getattr(p, k)
        if isinstance(cur, C.Array):
            for i, x in enumerate(v):
                cur[i] = x
        else:
            setattr(p, k, v)
    return p


def cell_index(x, d: float, half: bool = False):
    """The library's marker cell index (hmec_cell_index) of coordinates x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(x.shape, dtype=np.int32)
    rc = load().hmec_cell_index(_dptr(x), x.size, float(d), 1 if half else 0,
                                out.ctypes.data_as(C.POINTER(C.c_int32)))
    if rc != 0:
        raise HmecError(rc, "hmec_cell_index failed")
    return out


class HostArray:
    """A float64 array in page-locked host memory (hmec_host_alloc), freed
    with close(); `a` is the numpy view."""

    def __init__(self, n: int):
        self.L = load()
        self.ptr = self.L.hmec_host_alloc(8 * max(1, int(n)))
        if not self.ptr:
            raise HmecError(-7, "hmec_host_alloc failed")
        self.a = np.ctypeslib.as_array((C.c_double * max(1, int(n))).from_address(self.ptr))[:n]

    def close(self):
        if self.ptr:
            self.a = None
            self.L.hmec_host_free(self.ptr)
            self.ptr = None


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Instance:
    """Instance `inst` of a library context: one model's data and sections
    (the instance dimension of include/hmec.h)."""

    def __init__(self, owner, inst: int, params: Params):
        self.owner = owner
        self.L = owner.L
        self.inst = inst
        self.params = params
        self.Nx, self.Ny = params.Nx, params.Ny
        self.N = (self.Nx + 1) * (self.Ny + 1) * 6
        self.marknum = self.L.hmec_marknum(C.byref(params))

    @property
    def h(self):
        return self.owner.h

    def _check(self, rc, what):
        if rc != HMEC_OK:
            msg = self.L.hmec_last_error(self.h)
            raise HmecError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    # ------------------------------------------------------------ data
    def shape(self, name):
        g = self.L.hmec_field_grid(FIELDS.index(name))
        return (self.Ny + g, self.Nx + g)

    def upload_markers(self, arrays: dict):
        bufs = [np.ascontiguousarray(arrays[k], dtype=np.float64) for k in MARKERS]
        for b in bufs:
            if b.shape != (self.marknum,):
                raise ValueError("marker arrays must have length %d" % self.marknum)
        ptrs = (C.POINTER(C.c_double) * len(bufs))(*[_dptr(b) for b in bufs])
        self._check(self.L.hmec_upload_markers(self.h, self.inst, ptrs, self.marknum), "upload_markers")

    def stream_markers(self, arrays):
        """hmec_stream_markers: every later timestep copies these page-locked
        float64 arrays (dict by marker name, e.g. HostArray views) into the
        device after its markers->nodes section; None stops it.  The arrays
        are kept referenced while registered."""
        if arrays is None:
            self._check(self.L.hmec_stream_markers(self.h, self.inst, None, self.marknum), "stream_markers")
            self._streamed = None
            return
        bufs = [arrays[k] for k in MARKERS]
        for b in bufs:
            if b.dtype != np.float64 or not b.flags.c_contiguous or b.shape != (self.marknum,):
                raise ValueError("streamed marker arrays must be contiguous float64 of length %d" % self.marknum)
        ptrs = (C.POINTER(C.c_double) * len(bufs))(*[_dptr(b) for b in bufs])
        self._check(self.L.hmec_stream_markers(self.h, self.inst, ptrs, self.marknum), "stream_markers")
        self._streamed = bufs

    def download_markers(self) -> dict:
        bufs = [np.empty(self.marknum) for _ in MARKERS]
        ptrs = (C.POINTER(C.c_double) * len(bufs))(*[_dptr(b) for b in bufs])
        self._check(self.L.hmec_download_markers(self.h, self.inst, ptrs, self.marknum), "download_markers")
        return dict(zip(MARKERS, bufs))

    def upload_field(self, name, arr):
        r, c = self.shape(name)
        a = np.asfortranarray(np.asarray(arr, dtype=np.float64).reshape(r, c))
        buf = a.ravel(order="F")
        self._check(self.L.hmec_upload_field(self.h, self.inst, FIELDS.index(name), _dptr(buf), r, c), "upload_field")

    def field(self, name) -> np.ndarray:
        r, c = self.shape(name)
        buf = np.empty(r * c)
        self._check(self.L.hmec_download_field(self.h, self.inst, FIELDS.index(name), _dptr(buf), r, c), "download_field")
        return buf.reshape((r, c), order="F")

    def rows(self, row, names) -> dict:
        """Row `row` of each named field, in one device gather and transfer."""
        ids = (C.c_int32 * len(names))(*[FIELDS.index(n) for n in names])
        lens = [self.shape(n)[1] for n in names]
        buf = np.empty(sum(lens))
        self._check(self.L.hmec_download_rows(self.h, self.inst, row, len(names), ids, _dptr(buf)), "download_rows")
        out, o = {}, 0
        for n, k in zip(names, lens):
            out[n] = buf[o:o + k].copy()
            o += k
        return out

    def rows_async(self, row, names, out) -> int:
        """Starts the gather and copy of hmec_download_rows_async into `out`
        (a float64 array of the rows' total length, best page-locked: see
        host_array); returns the ticket to pass to rows_wait."""
        ids = (C.c_int32 * len(names))(*[FIELDS.index(n) for n in names])
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size < sum(self.shape(n)[1] for n in names):
            raise ValueError("out must be a contiguous float64 array of the rows' total length")
        t = C.c_int64(0)
        self._check(self.L.hmec_download_rows_async(self.h, self.inst, row, len(names), ids, _dptr(out), C.byref(t)),
                    "download_rows_async")
        return t.value

    def rows_wait(self, ticket):
        self._check(self.L.hmec_rows_wait(self.h, self.inst, ticket), "rows_wait")

    def set_scalar(self, name, v):
        self._check(self.L.hmec_set_scalar(self.h, self.inst, SCALARS.index(name), float(v)), "set_scalar")

    def scalar(self, name) -> float:
        v = C.c_double()
        self._check(self.L.hmec_get_scalar(self.h, self.inst, SCALARS.index(name), C.byref(v)), "get_scalar")
        return v.value

    def load_state(self, snap: dict):
        for f in FIELDS:
            if f in snap:
                self.upload_field(f, snap[f])
        for s in SCALARS:
            if "scalar_" + s in snap:
                self.set_scalar(s, snap["scalar_" + s])

    def snapshot(self) -> dict:
        out = {f: self.field(f) for f in FIELDS}
        out.update({"scalar_" + s: self.scalar(s) for s in SCALARS})
        return out

    # -------------------------------------------------------- sections
    def markers_to_nodes(self):
        self._check(self.L.hmec_markers_to_nodes(self.h, self.inst), "markers_to_nodes")

    def timestep_begin(self):
        self._check(self.L.hmec_timestep_begin(self.h, self.inst), "timestep_begin")

    def global_iteration(self) -> dict:
        rep = IterReport()
        self._check(self.L.hmec_global_iteration(self.h, self.inst, C.byref(rep)), "global_iteration")
        return {k: getattr(rep, k) for k, _ in IterReport._fields_}

    def timestep_end(self):
        self._check(self.L.hmec_timestep_end(self.h, self.inst), "timestep_end")

    def advect_markers(self):
        self._check(self.L.hmec_advect_markers(self.h, self.inst), "advect_markers")

    @property
    def stream_ptr(self) -> int:
        """cudaStream_t of the context (for CUDA-event timing)."""
        return self.L.hmec_stream(self.h, self.inst) or 0

    def profile_kernel(self, name):
        self._check(self.L.hmec_profile_kernel(self.h, self.inst, name.encode() if name else None), "profile_kernel")

    def profile_read(self):
        """(launches, total ms, compulsory bytes, bytes moved) of the profiled kernel family."""
        n, ms, b, bm = C.c_int64(), C.c_double(), C.c_double(), C.c_double()
        self._check(self.L.hmec_profile_read(self.h, self.inst, C.byref(n), C.byref(ms), C.byref(b), C.byref(bm)),
                    "profile_read")
        return n.value, ms.value, b.value, bm.value

    # ---------------------------------------------------------- hooks
    def assemble_csr(self):
        import scipy.sparse as sp

        nnz = C.c_int64()
        self._check(self.L.hmec_assemble_csr(self.h, self.inst, None, None, None, None, C.byref(nnz), None, None), "assemble_csr")
        n = self.N
        indptr = np.zeros(n + 1, dtype=np.int64)
        indices = np.zeros(nnz.value, dtype=np.int32)
        data = np.zeros(nnz.value)
        rhs = np.zeros(n)
        pt, pf = C.c_double(), C.c_double()
        self._check(self.L.hmec_assemble_csr(self.h, self.inst, indptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                             indices.ctypes.data_as(C.POINTER(C.c_int32)), _dptr(data), _dptr(rhs),
                                             C.byref(nnz), C.byref(pt), C.byref(pf)), "assemble_csr")
        return sp.csr_matrix((data, indices, indptr), shape=(n, n)), rhs, pt.value, pf.value

    def solve_system(self, rhs, x0=None):
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        its, rel = C.c_int32(), C.c_double()
        rc = self.L.hmec_solve_system(self.h, self.inst, _dptr(b), _dptr(x), C.byref(its), C.byref(rel))
        return x, its.value, rel.value, rc


class Model(Instance):
    """One model on the current CUDA device: a library context with one
    instance (instance 0)."""

    def __init__(self, params: Params):
        self.L = load()
        st = C.c_int32(0)
        self._h = self.L.hmec_create(C.byref(params), 1, None, C.byref(st))
        if not self._h:
            raise HmecError(st.value, "hmec_create failed")
        Instance.__init__(self, self, 0, params)

    @property
    def h(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self.L.hmec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def timestep(self, check=True) -> dict:
        rep = StepReport()
        rc = self.L.hmec_timestep(self.h, C.byref(rep))
        if check:
            self._check(rc, "timestep")
        d = {k: getattr(rep, k) for k, _ in StepReport._fields_}
        d["rc"] = rc
        return d

    def synchronize(self):
        self._check(self.L.hmec_synchronize(self.h), "synchronize")

    @property
    def launches(self) -> int:
        return self.L.hmec_kernel_launches(self.h)

    @property
    def graph_status(self) -> int:
        """1: timesteps run as one CUDA graph launch; 0: not yet; -1: host-driven."""
        return self.L.hmec_graph_status(self.h)

    def graph_error(self) -> str:
        """Why the graph is off (after graph_status returned -1)."""
        msg = self.L.hmec_last_error(self.h)
        return msg.decode() if msg else ""

