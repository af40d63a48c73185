"""Ensembles of independent H-MEC models on one GPU.

Each member is its own library context (own device buffers and CUDA stream)
and members advance concurrently: one host thread per member drives
hmec_timestep(), and because ctypes releases the interpreter lock during the
call, the members' kernels overlap on the GPU.  Members never exchange data,
so results are bit-identical to running each member alone.
"""
from __future__ import annotations

import concurrent.futures as cf

from . import MG_PASS_LAUNCHES, Model, default_params, synth


class Ensemble:
    def __init__(self, members, concurrent: bool = True, **common):
        """members: (overrides, material, seed) triples, e.g. synth.ensemble_members().

        concurrent: the members will run side by side (step()); they then
        smooth with one launch per multigrid pass and at most a quarter of
        the GPU per pass (HMEC_MG_PASS_LAUNCHES), so that different members'
        passes share the GPU.  With concurrent=False every member keeps the
        settings of a model run alone (for step_sequential())."""
        self.models = []
        for over, mat, seed in members:
            p = default_params(**dict(over, **common))
            if concurrent:
                p.mg_flags |= MG_PASS_LAUNCHES
            m = Model(p)
            mk, nodes = synth.instance_state(p, mat, seed)
            m.upload_markers(mk)
            for k, v in nodes.items():
                m.upload_field(k, v)
            self.models.append(m)
        self.pool = cf.ThreadPoolExecutor(max_workers=max(1, len(self.models)))

    def __len__(self):
        return len(self.models)

    def step(self, nsteps: int = 1):
        """Advance every member by nsteps timesteps; returns the per-member reports."""

        def run(m):
            return [m.timestep(check=False) for _ in range(nsteps)]

        return list(self.pool.map(run, self.models))

    def step_sequential(self, nsteps: int = 1):
        return [[m.timestep(check=False) for _ in range(nsteps)] for m in self.models]

    def close(self):
        self.pool.shutdown()
        for m in self.models:
            m.close()
