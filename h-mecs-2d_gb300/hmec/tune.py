"""Autotuner of the solver's cycle shape and the kernels' launch shapes.

For a grid and solver form it times a few timesteps (CUDA events on the
library stream, graph mode, after warm-up steps) of a model per candidate,
and keeps the fastest:

  - the multigrid cycle: levels, pre/post sweeps, coarse sweeps;
  - the node-stencil kernels' block size (assembly, stress, prep, gathers);
  - the marker kernels' block size (keys, scatter, marker properties);
  - the blocks of the cooperative Arnoldi step;
  - the most blocks of one smoothing launch;
  - whether the smoothing pass stages a whole tile's Vanka inverses or one
    colour's at a time;
  - whether a tile runs a pass's sweeps back to back on one stage (local
    sweeps, mg_flags bit 8).

The search is coordinate-wise: the cycle shapes first, then each launch
parameter in turn with the others at their best so far.  A candidate whose
steps take other global-iteration counts than the default's is rejected (the
solve reaches the same FP64 tolerance whatever the preconditioner, so the
step's decisions must not change).  Models are built on a seed other than
the benchmark's.  The winners go to a JSON table (tune_table.json beside this
file) that the library reads at hmec_create (hmec_params.autotune): the
entry of the same form whose grid is nearest in cells.

    python -m hmec.tune [--grids c1 c2 m51 m101 ...] [--forms 1 0]
                        [--steps 5] [--warmup 3] [--out PATH]
"""
from __future__ import annotations

import argparse
import json
import os
import time

from . import FORM_FP64, FORM_MIXED, Model, default_params, synth

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tune_table.json")

CYCLES = [(5, 2, 2, 8), (4, 2, 2, 8), (6, 2, 2, 4), (5, 1, 1, 8), (4, 1, 1, 8), (5, 1, 2, 8), (3, 2, 2, 8),
          (6, 1, 1, 4)]
LAUNCH = [("bs_stencil", [64, 128, 256]), ("bs_sort", [128, 256, 512]),
          ("krylov_blocks", [152, 304, 456, 608]), ("smooth_blocks", [0, 152]), ("smooth_inverses", [1, 2]),
          ("mg_flags", [1 | 8])]
SOLVER = dict(krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000)
DEFAULT = dict(mg_levels=5, mg_pre=2, mg_post=2, mg_coarse_sweeps=8, bs_stencil=64, bs_sort=256, krylov_blocks=0,
               smooth_blocks=0, smooth_inverses=0, mg_flags=1)


def grid_case(name: str, seed_shift: int = 17):
    """(parameter overrides, markers, node fields) of a named grid class, on a
    seed other than the benchmark's: presets c0-c2, or an ensemble member
    'm<side>' / 'm<Nx>x<Ny>' (configuration-0 material on that grid)."""
    if name in synth.PRESETS:
        over = dict(synth.PRESETS[name], **SOLVER)
        p = default_params(**over)
        mk, nodes = synth.make_state(p, name, seed=synth.SEEDS.get(name, 1000) + seed_shift)
        return over, mk, nodes
    dims = name[1:].split("x")
    nx, ny = int(dims[0]), int(dims[-1])
    over = dict(synth.PRESETS["c0"], Nx=nx, Ny=ny, **SOLVER)
    p = default_params(**over)
    mk, nodes = synth.instance_state(p, dict(synth.MATERIALS["c0"]), 4242 + nx * 7 + ny)
    return over, mk, nodes


def time_candidate(over, mk, nodes, form, cand, steps, warmup):
    """ms per timestep and per-step global-iteration counts of one candidate."""
    import torch

    p = default_params(**dict(over, form=form, autotune=0, **cand))
    m = Model(p)
    try:
        m.upload_markers(mk)
        for k, v in nodes.items():
            m.upload_field(k, v)
        for _ in range(warmup):
            m.timestep()
        s = torch.cuda.ExternalStream(m.stream_ptr)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        reps = [m.timestep() for _ in range(steps)]
        b.record(s)
        b.synchronize()
        return a.elapsed_time(b) / steps, [r["global_iters"] for r in reps]
    finally:
        m.close()


def tune(name: str, form: int, steps: int = 5, warmup: int = 3, log=print):
    over, mk, nodes = grid_case(name)
    base = dict(DEFAULT)
    base_ms, base_gi = time_candidate(over, mk, nodes, form, base, steps, warmup)
    best, best_ms = dict(base), base_ms
    tried = [dict(base, ms=base_ms)]

    def consider(cand):
        nonlocal best, best_ms
        ms, gi = time_candidate(over, mk, nodes, form, cand, steps, warmup)
        ok = gi == base_gi
        tried.append(dict(cand, ms=ms, same_iterations=ok))
        log("  %s form %d %s: %.3f ms%s" % (name, form, {k: cand[k] for k in cand if cand[k] != base[k]}, ms,
                                            "" if ok else " (other global iterations: rejected)"))
        if ok and ms < best_ms:
            best, best_ms = dict(cand), ms

    for lv, pre, post, cs in CYCLES[1:]:
        consider(dict(best, mg_levels=lv, mg_pre=pre, mg_post=post, mg_coarse_sweeps=cs))
    for key, values in LAUNCH:
        for v in values:
            if v != best[key]:
                consider(dict(best, **{key: v}))
    entry = dict(Nx=over["Nx"], Ny=over["Ny"], form=form, **best, ms_per_step=best_ms, default_ms_per_step=base_ms,
                 case=name, candidates=len(tried))
    return entry, tried


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grids", nargs="+", default=["c2", "c1", "m51", "m101", "m201x101", "m301", "m401x201"])
    ap.add_argument("--forms", nargs="+", type=int, default=[FORM_MIXED, FORM_FP64])
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--out", default=TABLE)
    a = ap.parse_args()
    t0 = time.time()
    entries = []
    for g in a.grids:
        for f in a.forms:
            e, _ = tune(g, f, a.steps, a.warmup)
            print("%s form %d: %.3f -> %.3f ms/step %s" % (g, f, e["default_ms_per_step"], e["ms_per_step"],
                                                          {k: e[k] for k in DEFAULT}), flush=True)
            entries.append(e)
            # written after every entry, so a cut-short run keeps what it found
            import torch

            table = {"version": 1, "device": torch.cuda.get_device_name(0), "seconds": time.time() - t0,
                     "how": "coordinate search, %d timed steps after %d warm-up steps per candidate (CUDA events, "
                            "graph mode); candidates that change the global-iteration counts are rejected"
                            % (a.steps, a.warmup),
                     "entries": entries}
            with open(a.out, "w") as fh:
                json.dump(table, fh, indent=1)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
