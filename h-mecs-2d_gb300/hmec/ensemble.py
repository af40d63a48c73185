"""Ensembles of independent H-MEC models on one GPU.

``Ensemble`` holds all members in ONE library context (hmec_create with
n_instances > 1): each member is an instance with its own grid, buffers and
stream, and ``step()`` advances every member with one ``hmec_timestep``
call -- after the first step, one CUDA graph launch for all members, each
with its own adaptive dt, global iterations and solver convergence decided on
the device.  Members never exchange data, so their results are bit-identical
to running each member alone.

``Sequential`` runs the same members one after another, each in a context of
its own with the settings of a model run alone (the plain-FP64 baseline the
ensemble is compared with).
"""
from __future__ import annotations

import ctypes as C

from . import (Grid, HmecError, Instance, Model, StepReport, default_params, load, synth)


def _member_params(over, common):
    return default_params(**dict(over, **common))


class Ensemble:
    def __init__(self, members, **common):
        """members: (overrides, material, seed) triples, e.g. synth.ensemble_members().
        common: parameter overrides for every member (solver settings, form).
        The shared parameters are the first member's; each member's grid
        (Nx, Ny, xsize, ysize, mx, my) is its own."""
        self.L = load()
        n = len(members)
        params = [_member_params(o, common) for o, _, _ in members]
        grids = (Grid * n)()
        for k, p in enumerate(params):
            grids[k] = Grid(p.Nx, p.Ny, p.xsize, p.ysize, p.mx, p.my)
        st = C.c_int32(0)
        self._h = self.L.hmec_create(C.byref(params[0]), n, grids, C.byref(st))
        if not self._h:
            raise HmecError(st.value, "hmec_create failed")
        self.members = [Instance(self, k, params[k]) for k in range(n)]
        for (over, mat, seed), m in zip(members, self.members):
            mk, nodes = synth.instance_state(m.params, mat, seed)
            m.upload_markers(mk)
            for k, v in nodes.items():
                m.upload_field(k, v)

    @property
    def h(self):
        return self._h

    def __len__(self):
        return len(self.members)

    @property
    def models(self):
        return self.members

    def step(self, nsteps: int = 1):
        """Advance every member by nsteps timesteps; returns per member the list of its reports."""
        n = len(self.members)
        out = [[] for _ in range(n)]
        reps = (StepReport * n)()
        for _ in range(nsteps):
            self.L.hmec_timestep(self._h, reps)
            for k in range(n):
                d = {f: getattr(reps[k], f) for f, _ in StepReport._fields_}
                d["rc"] = d["status"]  # the member's own first non-OK status of the step
                out[k].append(d)
        return out

    @property
    def launches(self) -> int:
        return self.L.hmec_kernel_launches(self._h)

    @property
    def graph_status(self) -> int:
        return self.L.hmec_graph_status(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self.L.hmec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Sequential:
    """The same members, each in its own context, stepped one after another."""

    def __init__(self, members, **common):
        self.models = []
        for over, mat, seed in members:
            m = Model(_member_params(over, common))
            mk, nodes = synth.instance_state(m.params, mat, seed)
            m.upload_markers(mk)
            for k, v in nodes.items():
                m.upload_field(k, v)
            self.models.append(m)

    def __len__(self):
        return len(self.models)

    def step(self, nsteps: int = 1):
        return [[m.timestep(check=False) for _ in range(nsteps)] for m in self.models]

    @property
    def launches(self) -> int:
        return sum(m.launches for m in self.models)

    def close(self):
        for m in self.models:
            m.close()
