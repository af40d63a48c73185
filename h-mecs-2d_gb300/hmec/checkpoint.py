"""Checkpoint and restart files in the reference's layout.

The reference saves every `savestep` timesteps to `nname + timestep + ".h5"`
(cpp/h_mec_rsf_v9.cpp:1807-1870) and restarts from such a file
(:211-282): group /Matrix with 24 basic-grid (Ny x Nx) and 30 staggered
(Ny1 x Nx1) node fields, group /Vector with six per-timestep histories
(length num_timesteps) and five marker arrays (length marknum), group /Value
with nine scalars.  Matrices are stored in C order (row i of the dataset is
row i of the grid, cpp/hdf5.cpp:46-51).  The dataset names, their order, the
shapes and the byte order below are the format, so they are the reference's.

HDF5 is written with h5py when it is importable.  Without it (as in this
environment) a stub container keeps the same groups, names, shapes and
C-order FP64 bytes in one file:

    b"HMECH5S1", u32 count, then per dataset: u16 + group bytes, u16 + name
    bytes, u8 rank, rank x u64 dims, dims product x f64 (little endian)

The reference's readers and writers copy every dataset through a stack
array (cpp/hdf5.cpp:46, :74, :107, :138), which overflows for large grids or
marker counts; here all buffers are on the heap.
"""
from __future__ import annotations

import os
import struct

import numpy as np

# /Matrix, basic nodes (Ny x Nx), :1826-1831
MATRIX_BASIC = ("SIIB", "OM0", "OM", "ARSF", "BRSF", "LRSF", "RHO", "ETA0", "ETA1", "ETA5", "ETA00", "IETAPLB",
                "SXY0", "YNY0", "KKK", "GGG", "COHC", "COHT", "FRIC", "FRIT", "DILC", "TTT", "EIIB", "VSLIPB")
# /Matrix, staggered nodes (Ny1 x Nx1), :1834-1841
MATRIX_STAGGERED = ("pt", "vxs", "vys", "pf", "vxD", "vyD", "ETAB", "ETAB0", "ETAP", "ETAP0", "POR", "GGGP",
                    "GGGB", "PTF0", "PT0", "PF0", "SXX0", "SYY0", "RHOX", "RHOFX", "ETADX", "PORX", "VX0", "VXF0",
                    "RHOY", "RHOFY", "ETADY", "PORY", "VY0", "VYF0")
# /Vector, per-timestep histories (num_timesteps), :1844-1849
HISTORY = ("timesumcur", "dtcur", "maxvxsmod", "minvxsmod", "maxvysmod", "minvysmod")
# /Vector, marker arrays (marknum), :1852-1857
MARKERS = ("xm", "ym", "sxxm", "syym", "sxym")
# /Value/values, :1860-1863
VALUES = ("timesum", "dt00", "dtx", "dty", "dtlapusta", "Vmax", "maxvxy", "dt", "yndtdecrease")

MAGIC = b"HMECH5S1"


def file_name(timestep: int, nname: str = "h_mec_", stub: bool | None = None) -> str:
    """`nname + timestep + ".h5"` (:1814); the stub container adds ".stub"."""
    if stub is None:
        stub = not _have_h5py()
    return "%s%d.h5%s" % (nname, timestep, ".stub" if stub else "")


def _have_h5py() -> bool:
    try:
        import h5py  # noqa: F401
    except ImportError:
        return False
    return True


class History:
    """The six per-timestep histories the host loop keeps (:1658-1696)."""

    def __init__(self, num_timesteps: int):
        self.v = {k: np.zeros(num_timesteps) for k in HISTORY}

    def record(self, model, timestep: int):
        """After timestep `timestep` (1-based) has run: index timestep - 1."""
        t = timestep - 1
        self.v["timesumcur"][t] = model.scalar("timesum")
        self.v["dtcur"][t] = model.scalar("dt")
        for k in ("maxvxsmod", "minvxsmod", "maxvysmod", "minvysmod"):
            self.v[k][t] = model.scalar(k)


def datasets(model, history: History):
    """(group, name, array) in the reference's write order; matrices as
    (rows, cols) arrays (written in C order)."""
    out = [("Matrix", n, model.field(n)) for n in MATRIX_BASIC + MATRIX_STAGGERED]
    out += [("Vector", n, history.v[n]) for n in HISTORY]
    mk = model.download_markers()
    out += [("Vector", n, mk[n]) for n in MARKERS]
    out.append(("Value", "values", np.array([model.scalar(n) for n in VALUES], dtype=np.float64)))
    return out


# ---------------------------------------------------------------- containers
def write_stub(path: str, items):
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<I", len(items)))
        for group, name, a in items:
            a = np.ascontiguousarray(a, dtype="<f8")
            for s in (group, name):
                b = s.encode()
                f.write(struct.pack("<H", len(b)))
                f.write(b)
            f.write(struct.pack("<B", a.ndim))
            f.write(struct.pack("<%dQ" % a.ndim, *a.shape))
            f.write(a.tobytes(order="C"))


def read_stub(path: str) -> dict:
    """{(group, name): array} of a stub container."""
    out = {}
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError("%s: not a checkpoint stub container" % path)
        (count,) = struct.unpack("<I", f.read(4))
        for _ in range(count):
            names = []
            for _ in range(2):
                (n,) = struct.unpack("<H", f.read(2))
                names.append(f.read(n).decode())
            (rank,) = struct.unpack("<B", f.read(1))
            shape = struct.unpack("<%dQ" % rank, f.read(8 * rank))
            count_el = int(np.prod(shape)) if rank else 1
            a = np.frombuffer(f.read(8 * count_el), dtype="<f8").reshape(shape)
            out[tuple(names)] = a.astype(np.float64)
    return out


def write_h5(path: str, items):
    import h5py

    with h5py.File(path, "w") as f:
        for group in ("Matrix", "Vector", "Value"):
            f.create_group("/" + group)
        for group, name, a in items:
            f.create_dataset("/%s/%s" % (group, name), data=np.ascontiguousarray(a, dtype=np.float64))


def read_h5(path: str) -> dict:
    import h5py

    out = {}
    with h5py.File(path, "r") as f:
        for group in ("Matrix", "Vector", "Value"):
            for name, d in f[group].items():
                out[(group, name)] = np.array(d, dtype=np.float64)
    return out


def read(path: str) -> dict:
    with open(path, "rb") as f:
        head = f.read(8)
    return read_stub(path) if head == MAGIC else read_h5(path)


# ---------------------------------------------------------------- save / load
def save(model, path: str, history: History):
    """Write the checkpoint of the model's current state (after a timestep)."""
    items = datasets(model, history)
    if path.endswith(".stub") or not _have_h5py():
        write_stub(path, items)
    else:
        write_h5(path, items)


def load(model, path: str, timestep: int, history: History | None = None):
    """Restart as :211-282 does: every dataset into the model (the markers'
    other arrays keep the values the model already holds, as the reference
    rebuilds them from its lattice first), then the step counter past the
    saved step."""
    d = read(path)
    for n in MATRIX_BASIC + MATRIX_STAGGERED:
        model.upload_field(n, d[("Matrix", n)])
    mk = model.download_markers()
    for n in MARKERS:
        mk[n] = d[("Vector", n)]
    model.upload_markers(mk)
    vals = d[("Value", "values")]
    for n, v in zip(VALUES, vals):
        model.set_scalar(n, float(v))
    model.set_scalar("timestep", float(timestep + 1))
    if history is not None:
        for n in HISTORY:
            history.v[n][:] = d[("Vector", n)]
    return d


def trim_evo(outdir: str, timestep: int):
    """The reference's restart drops EVO_*.txt lines written after the saved
    step (:268-281): every file keeps its first `timestep` lines.  Its list
    names "EVO_VxD.txt" while the series is written to "EVO_vxD.txt"
    (:1798), so on a case-sensitive file system its Darcy-velocity series is
    never trimmed; here the file that is written is."""
    for name in ("EVO_Vslip.txt", "EVO_viscosity.txt", "EVO_press_flu.txt", "EVO_press_eff.txt", "EVO_SigmaY.txt",
                 "EVO_Sii.txt", "EVO_Theta.txt", "EVO_Visc_comp.txt", "EVO_Elast_comp.txt", "EVO_vxD.txt",
                 "EVO_data.txt"):
        p = os.path.join(outdir, name)
        if not os.path.exists(p):
            continue
        with open(p) as f:
            lines = f.readlines()
        with open(p, "w") as f:
            f.writelines(lines[:timestep])
