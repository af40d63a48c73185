"""CPU oracle driver for the H-MEC hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the oracle the GPU results are
compared with.  It is never the thing measured or shipped.

Wraps ``libhmec_oracle.so`` (the C restatement of cpp/h_mec_rsf_v9.cpp in
hmec_oracle.c).  The reference solves every global iteration with MKL Pardiso
(cpp/h_mec_rsf_v9.cpp:1046-1052); neither MKL nor Eigen is installable here,
so the direct solve is SciPy's SuperLU (COLAMD ordering) on the same summed
CSR, followed by iterative refinement in FP64 until the residual stops
improving.  That is the oracle's stand-in for Pardiso.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "libhmec_oracle.so")


class HmecParams(C.Structure):
    """ctypes mirror of ``hmec_params`` (include/hmec.h)."""

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


def _names(macro: str):
    """Read an X-macro list of include/hmec.h (keeps one source of truth for ids)."""
    import re

    text = open(os.path.join(ROOT, "include", "hmec.h")).read()
    start = text.index("#define %s(X)" % macro)
    body = []
    for line in text[start:].splitlines()[1:]:
        body.append(line)
        if not line.rstrip().endswith("\\"):
            break
    return re.findall(r"X\((\w+)", " ".join(body))


FIELDS = _names("HMEC_FIELD_LIST")
MARKERS = _names("HMEC_MARKER_LIST")
SCALARS = _names("HMEC_SCALAR_LIST")


def build(force: bool = False) -> str:
    """Compile the oracle (plain C, no FMA contraction) into oracle/_build."""
    src = os.path.join(HERE, "hmec_oracle.c")
    hdrs = [os.path.join(HERE, "hmec_oracle.h"), os.path.join(ROOT, "include", "hmec.h")]
    if not force and os.path.exists(LIB_PATH):
        newest = max(os.path.getmtime(p) for p in [src] + hdrs)
        if os.path.getmtime(LIB_PATH) >= newest:
            return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".%d.tmp" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-D_DEFAULT_SOURCE", "-pthread", "-o", tmp, src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None
SOLVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                       C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double))


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.hmo_params_default.argtypes = [P(HmecParams)]
        L.hmo_create.argtypes = [P(HmecParams)]
        L.hmo_create.restype = C.c_void_p
        L.hmo_destroy.argtypes = [C.c_void_p]
        L.hmo_marknum.argtypes = [C.c_void_p]
        L.hmo_marknum.restype = C.c_int64
        L.hmo_unknowns.argtypes = [C.c_void_p]
        L.hmo_field.argtypes = [C.c_void_p, C.c_int32]
        L.hmo_field.restype = P(C.c_double)
        L.hmo_marker.argtypes = [C.c_void_p, C.c_int32]
        L.hmo_marker.restype = P(C.c_double)
        L.hmo_get_scalar.argtypes = [C.c_void_p, C.c_int32]
        L.hmo_get_scalar.restype = C.c_double
        L.hmo_set_scalar.argtypes = [C.c_void_p, C.c_int32, C.c_double]
        L.hmo_coords.argtypes = [C.c_void_p, C.c_int32]
        L.hmo_coords.restype = P(C.c_double)
        for fn in ("hmo_markers_to_nodes", "hmo_timestep_begin", "hmo_iter_prepare", "hmo_timestep_end",
                   "hmo_advect_markers"):
            getattr(L, fn).argtypes = [C.c_void_p]
            getattr(L, fn).restype = None
        L.hmo_set_threads.argtypes = [C.c_void_p, C.c_int32]
        L.hmo_set_threads.restype = None
        L.hmo_assemble.argtypes = [C.c_void_p]
        L.hmo_assemble.restype = C.c_int64
        L.hmo_csr.argtypes = [C.c_void_p, P(P(C.c_int64)), P(P(C.c_int32)), P(P(C.c_double)), P(P(C.c_double))]
        L.hmo_iter_finish.argtypes = [C.c_void_p, P(C.c_double)]
        L.hmo_global_iteration.argtypes = [C.c_void_p, SOLVE_FN, C.c_void_p]
        L.hmo_timestep.argtypes = [C.c_void_p, SOLVE_FN, C.c_void_p]
        L.hmo_last_ynpl.argtypes = [C.c_void_p]
        L.hmo_last_dsylsq.argtypes = [C.c_void_p]
        L.hmo_last_dsylsq.restype = C.c_double
        L.hmo_rsf_noconv.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def default_params(**over) -> HmecParams:
    p = HmecParams()
    lib().hmo_params_default(C.byref(p))
    for k, v in over.items():
        cur = getattr(p, k)
        if isinstance(cur, C.Array):
            for i, x in enumerate(v):
                cur[i] = x
        else:
            setattr(p, k, v)
    return p


def equilibrate(A):
    """Row then column max-norm scaling: (Dr, Dc) with Dr A Dc of unit row/column maxima.

    The assembled rows span some thirty orders of magnitude (Darcy rows carry
    eta_f/k ~ 1e17, continuity rows 1/dx ~ 1e-2); Pardiso scales nonsymmetric
    systems by default before pivoting, and SuperLU needs the same treatment
    to pivot sensibly.
    """
    import scipy.sparse as sp

    A = sp.csr_matrix(A)
    rn = abs(A).max(axis=1).toarray().ravel()
    rn[rn == 0] = 1.0
    Dr = sp.diags(1.0 / rn)
    As = Dr @ A
    cn = abs(As).max(axis=0).toarray().ravel()
    cn[cn == 0] = 1.0
    Dc = sp.diags(1.0 / cn)
    return Dr, Dc


def direct_solve(A, b, refine: int = 4, ordering: str = "COLAMD", pivot_thresh: float = 1.0):
    """Equilibrated SuperLU solve with FP64 iterative refinement (the Pardiso stand-in)."""
    import scipy.sparse.linalg as spla

    Dr, Dc = equilibrate(A)
    As = (Dr @ A @ Dc).tocsc()
    lu = spla.splu(As, permc_spec=ordering, diag_pivot_thresh=pivot_thresh)

    def solve(r):
        return Dc @ lu.solve(Dr @ r)

    x = solve(b)
    best = np.linalg.norm(Dr @ (b - A @ x))
    for _ in range(refine):
        x2 = x + solve(b - A @ x)
        n2 = np.linalg.norm(Dr @ (b - A @ x2))
        if not n2 < best:
            break
        x, best = x2, n2
    return x


class Oracle:
    """One reference model instance on the CPU."""

    #: SuperLU column ordering and partial-pivoting threshold of the direct
    #: solve (a second ordering or threshold gives the oracle's own round-off
    #: floor: the same system solved with other pivots)
    ordering = "COLAMD"
    pivot_thresh = 1.0

    def __init__(self, params: HmecParams):
        self.L = lib()
        self.params = params
        self.h = self.L.hmo_create(C.byref(params))
        if not self.h:
            raise MemoryError("hmo_create failed")
        self.Nx, self.Ny = params.Nx, params.Ny
        self.N = self.L.hmo_unknowns(self.h)
        self.marknum = self.L.hmo_marknum(self.h)
        self.solve_calls = 0
        self.last_solution = None
        self._cb = SOLVE_FN(self._solve)

    def __del__(self):
        try:
            if self.h:
                self.L.hmo_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ------------------------------------------------------------- data
    def shape(self, name):
        grid = 1 if FIELDS.index(name) >= FIELDS.index("pt") else 0
        return (self.Ny + grid, self.Nx + grid)

    def field(self, name) -> np.ndarray:
        """Live view (rows, cols) in Fortran order of an oracle field."""
        r, c = self.shape(name)
        ptr = self.L.hmo_field(self.h, FIELDS.index(name))
        return np.ctypeslib.as_array(ptr, shape=(r * c,)).reshape((r, c), order="F")

    def set_field(self, name, arr):
        self.field(name)[...] = np.asarray(arr, dtype=np.float64)

    def marker(self, name) -> np.ndarray:
        ptr = self.L.hmo_marker(self.h, MARKERS.index(name))
        return np.ctypeslib.as_array(ptr, shape=(self.marknum,))

    def set_markers(self, arrays: dict):
        for k, v in arrays.items():
            self.marker(k)[...] = v

    def scalar(self, name) -> float:
        return self.L.hmo_get_scalar(self.h, SCALARS.index(name))

    def set_scalar(self, name, v):
        self.L.hmo_set_scalar(self.h, SCALARS.index(name), float(v))

    def coords(self, which: int):
        n = [self.Nx, self.Ny, self.Nx + 1, self.Ny + 1, self.Nx + 1, self.Ny + 1, self.Nx + 1, self.Ny + 1][which]
        return np.ctypeslib.as_array(self.L.hmo_coords(self.h, which), shape=(n,)).copy()

    def snapshot(self) -> dict:
        out = {f: self.field(f).copy() for f in FIELDS}
        out.update({"scalar_" + s: self.scalar(s) for s in SCALARS})
        return out

    def load_state(self, snap: dict):
        for f in FIELDS:
            if f in snap:
                self.set_field(f, snap[f])
        for s in SCALARS:
            if "scalar_" + s in snap:
                self.set_scalar(s, snap["scalar_" + s])

    # --------------------------------------------------------- sections
    def set_threads(self, n: int):
        """Threads of the marker loop (1, the default: the serial loop)."""
        self.L.hmo_set_threads(self.h, int(n))

    def markers_to_nodes(self):
        self.L.hmo_markers_to_nodes(self.h)

    def timestep_begin(self):
        self.L.hmo_timestep_begin(self.h)

    def iter_prepare(self):
        self.L.hmo_iter_prepare(self.h)

    def assemble(self):
        """(CSR matrix, R) of the current state (after iter_prepare)."""
        import scipy.sparse as sp

        nnz = self.L.hmo_assemble(self.h)
        ip, ix, dv, rv = (C.POINTER(C.c_int64)(), C.POINTER(C.c_int32)(), C.POINTER(C.c_double)(),
                          C.POINTER(C.c_double)())
        self.L.hmo_csr(self.h, C.byref(ip), C.byref(ix), C.byref(dv), C.byref(rv))
        n = self.N
        indptr = np.ctypeslib.as_array(ip, shape=(n + 1,)).copy()
        indices = np.ctypeslib.as_array(ix, shape=(max(nnz, 1),))[:nnz].copy()
        data = np.ctypeslib.as_array(dv, shape=(max(nnz, 1),))[:nnz].copy()
        R = np.ctypeslib.as_array(rv, shape=(n,)).copy()
        return sp.csr_matrix((data, indices, indptr), shape=(n, n)), R

    def scales(self):
        """(ptscale, pfscale) of the last preparation (recomputed from ETADX)."""
        dt = self.scalar("dt")
        mn = self.field("ETADX")[1:self.Ny, 0:self.Nx].min()
        dx = self.params.xsize / (self.Nx - 1)
        pf = mn * dx * 1e17 / (dt * dt) if dt > 2e5 else mn * dx
        return pf, pf

    def iter_finish(self, S) -> int:
        S = np.ascontiguousarray(S, dtype=np.float64)
        return self.L.hmo_iter_finish(self.h, S.ctypes.data_as(C.POINTER(C.c_double)))

    def _solve(self, user, n, indptr, indices, data, rhs, x):
        try:
            import scipy.sparse as sp

            ip = np.ctypeslib.as_array(indptr, shape=(n + 1,))
            nnz = int(ip[-1])
            A = sp.csr_matrix((np.ctypeslib.as_array(data, shape=(nnz,)).copy(),
                               np.ctypeslib.as_array(indices, shape=(nnz,)).copy(), ip.copy()), shape=(n, n))
            b = np.ctypeslib.as_array(rhs, shape=(n,)).copy()
            sol = direct_solve(A, b, ordering=self.ordering, pivot_thresh=self.pivot_thresh)
            np.ctypeslib.as_array(x, shape=(n,))[...] = sol
            self.solve_calls += 1
            self.last_solution = sol
            return 0
        except Exception as e:  # pragma: no cover - reported to the C side
            print("oracle solve failed:", e, file=sys.stderr)
            return 1

    def global_iteration(self) -> int:
        rc = self.L.hmo_global_iteration(self.h, self._cb, None)
        if rc < 0:
            raise RuntimeError("oracle solve failed")
        return rc

    def timestep_end(self):
        self.L.hmo_timestep_end(self.h)

    def advect_markers(self):
        self.L.hmo_advect_markers(self.h)

    def timestep(self) -> int:
        rc = self.L.hmo_timestep(self.h, self._cb, None)
        if rc < 0:
            raise RuntimeError("oracle solve failed")
        return rc

    @property
    def last_ynpl(self):
        return self.L.hmo_last_ynpl(self.h)

    @property
    def last_dsylsq(self):
        return self.L.hmo_last_dsylsq(self.h)

    @property
    def rsf_noconv(self):
        return self.L.hmo_rsf_noconv(self.h)
