#!/usr/bin/env python
"""Simulated timesteps/s of the H-MEC per-timestep hot path on GB300.

A step is one timestep of the reference loop (markers -> nodes, global
iterations with assembly + solve + stress + fault update + adaptive dt, end of
step), run through the C ABI of libhmec_gpu.so on synthetic configuration 1
(201 x 201 nodes, 5 x 5 markers per cell, 1.0 M markers).  `value` is the
mixed form (FP32 multigrid-preconditioned FP64 FGMRES) with inputs resident in
HBM; the plain FP64 form is measured the same way beside it; `e2e` re-runs the
mixed form with the model state copied from pinned host buffers every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference (the oracle: the
reference itself needs Eigen, HDF5 and MKL Pardiso, none of which exist here)
on the host cores, on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "h-mecs-2d_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "timesteps/s on 1 GB300: mixed-prec batched vs plain FP64, at ≤1e-8 rel err"
CONFIG = "c1"
WORKLOAD = "config 1: 201x201 nodes, 10x10 km, 5x5 markers/cell (1,000,000 markers), seeded synthetic fault model"
DOMINANT = "k_smooth"
# DRAM bytes (read + write) per launch of the fused V-cycle kernel (one launch
# = one config-1 V-cycle), from one ncu capture of the kernel (profiles/)
SMOOTH_TRAFFIC_BYTES = 94.97e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=CONFIG)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- several ranks
# One process per GPU.  A single model does not shard (replicas only); the
# members of an ensemble shard by rank with no collective on the data path.
# The only collectives are the barriers and the max over ranks of the timed
# interval.
def rank_max(x, world):
    """Max of x over all ranks (NCCL tensors on the GPU, CPU tensors on gloo)."""
    if world == 1:
        return x
    import torch

    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def rank_barrier(world):
    if world > 1:
        import torch

        torch.distributed.barrier()


def shard(items, rank, world):
    """This rank's share of independent work items (round robin)."""
    return list(items)[rank::world]


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units all ranks processed per second of the slowest rank."""
    return units_per_rank * world / seconds_max


# -------------------------------------------------------------------- GPU arm
def make_model(form, cfg, device_index):
    import hmec
    from hmec import synth

    over = dict(synth.PRESETS[cfg], form=form, krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000)
    p = hmec.default_params(**over)
    m = hmec.Model(p)
    mk, nodes = synth.make_state(p, cfg)
    m.upload_markers(mk)
    for k, v in nodes.items():
        m.upload_field(k, v)
    return m, mk, nodes, p


def timed_steps(m, steps, flush, per_step=None):
    """Per-step CUDA-event durations (ms) on the library stream; L2 flushed between steps."""
    import torch

    s = torch.cuda.ExternalStream(m.stream_ptr)
    total = 0.0
    reps = []
    for _ in range(steps):
        flush()
        torch.cuda.synchronize()
        if per_step:
            per_step("before")
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        if per_step:
            per_step("upload")
        reps.append(m.timestep())
        if per_step:
            per_step("download")
        b.record(s)
        b.synchronize()
        total += a.elapsed_time(b)
    return total, reps


def run_gpu(args, rank, world, device_index):
    import numpy as np
    import torch

    import hmec
    from hmec import synth

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.fill_(1.0)

    def barrier():
        rank_barrier(world)

    def max_over_ranks(x):
        return rank_max(x, world)

    out = {}
    # ---- mixed form (value), with the live roofline of the dominant kernel
    m, mk, nodes, p = make_model(hmec.FORM_MIXED, args.config, device_index)
    for _ in range(args.warmup):
        m.timestep()
    m.profile_kernel(DOMINANT)
    barrier()
    torch.cuda.synchronize()
    l0 = m.launches
    with ClockSampler(device_index) as clk:
        ms, reps = timed_steps(m, args.steps, flush)
    launches = m.launches - l0
    nprof, prof_ms, prof_bytes = m.profile_read()
    m.profile_kernel(None)
    ms = max_over_ranks(ms)
    barrier()
    gi = sum(r["global_iters"] for r in reps)
    kr = sum(r["krylov_iters"] for r in reps)
    out["mixed"] = dict(ms=ms, reps=reps, launches=launches, gi=gi, kr=kr, clocks=clk.summary(),
                        prof=(nprof, prof_ms, prof_bytes))
    mixed_state = ("vxs", "vys", "pt", "pf", "VSLIPB")  # the fields the accuracy check compares

    # ---- e2e: model state through pinned host buffers every step
    if not args.no_e2e:
        pin = {}
        for k, v in mk.items():
            t = torch.empty(v.shape, dtype=torch.float64, pin_memory=True)
            t.numpy()[...] = v
            pin[k] = t.numpy()
        # The host keeps the model state between steps, as the reference's globals
        # do; each step uploads it with the markers and downloads the new state
        # plus the fault outputs (pinned, column-major buffers).
        state_names = ["pt", "vxs", "vys", "pf", "vxD", "vyD", "SXX0", "SYY0", "SXY0", "PT0", "PF0", "VX0", "VY0",
                       "VXF0", "VYF0", "OM0", "ETA00", "YNY0"]
        out_names = ["SXX", "SYY", "SXY", "VSLIPB", "OM", "SigmaY"]
        import ctypes as C

        def pinned(f):
            r, c = m.shape(f)
            flat = torch.empty(r * c, dtype=torch.float64, pin_memory=True).numpy()
            return flat, r, c

        host_state = {f: pinned(f) for f in state_names}
        host_out = {f: pinned(f) for f in out_names}
        for f, (flat, r, c) in host_state.items():
            flat[...] = m.field(f).ravel(order="F")
        h2d = sum(v.nbytes for v in pin.values()) + sum(v[0].nbytes for v in host_state.values())
        d2h = sum(v[0].nbytes for v in host_out.values()) + sum(v[0].nbytes for v in host_state.values())

        def ptr(flat):
            return flat.ctypes.data_as(C.POINTER(C.c_double))

        def hook(phase):
            if phase == "upload":
                m.upload_markers(pin)
                for f, (flat, r, c) in host_state.items():
                    m.L.hmec_upload_field(m.h, hmec.FIELDS.index(f), ptr(flat), r, c)
            elif phase == "download":
                for f, (flat, r, c) in list(host_out.items()) + list(host_state.items()):
                    m.L.hmec_download_field(m.h, hmec.FIELDS.index(f), ptr(flat), r, c)

        barrier()
        e2e_ms, e2e_reps = timed_steps(m, args.steps, flush, per_step=hook)
        e2e_ms = max_over_ranks(e2e_ms)
        out["e2e"] = dict(ms=e2e_ms, h2d=h2d, d2h=d2h)
    m.close()

    # ---- plain FP64 form, same steps
    if not args.no_fp64:
        m2, _, _, _ = make_model(hmec.FORM_FP64, args.config, device_index)
        for _ in range(args.warmup):
            m2.timestep()
        barrier()
        ms2, reps2 = timed_steps(m2, args.steps, flush)
        ms2 = max_over_ranks(ms2)
        # accuracy of the mixed form: one timestep from the same state in both
        # forms (after many steps the adaptive dt sequences of the two runs
        # part ways on discrete decisions, and their states are then at
        # different times)
        snap = m2.snapshot()
        m2.timestep()
        fp64_next = {f: m2.field(f) for f in mixed_state}
        dt64 = m2.scalar("dt")
        m2.close()
        m3, _, _, _ = make_model(hmec.FORM_MIXED, args.config, device_index)
        m3.load_state(snap)
        m3.timestep()
        err = {}
        got = {f: m3.field(f) for f in fp64_next}
        for f, b in fp64_next.items():
            den = float(np.max(np.abs(b))) or 1.0
            err[f] = float(np.max(np.abs(got[f] - b))) / den
        # the velocity field as one quantity (as the parity tests group it):
        # vys alone is small in this simple-shear setup
        den = max(float(np.max(np.abs(fp64_next[f]))) for f in ("vxs", "vys")) or 1.0
        err["velocity"] = max(float(np.max(np.abs(got[f] - fp64_next[f]))) for f in ("vxs", "vys")) / den
        dt_equal = m3.scalar("dt") == dt64
        m3.close()
        out["fp64"] = dict(ms=ms2, gi=sum(r["global_iters"] for r in reps2), kr=sum(r["krylov_iters"] for r in reps2),
                           err=err, dt_equal=dt_equal)
    return out, peaks


# ------------------------------------------------------------------ CPU arm
def cpu_sample(cfg, budget_s=30.0, max_steps=2):
    """Time the CPU oracle (restatement of the reference) on the first steps of cfg."""
    import oracle as O
    from hmec import synth

    over = dict(synth.PRESETS[cfg])
    p = O.default_params(**over)
    o = O.Oracle(p)
    mk, nodes = synth.make_state(p, cfg)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    t0 = time.perf_counter()
    steps = 0
    gi = 0
    while steps < max_steps:
        gi += o.timestep()
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return dict(value=steps / el, steps=steps, seconds=el, global_iters=gi)


def run_ensemble(args, rank=0, world=1, device_index=0, nmembers=64):
    """Configuration 3: 64 uneven members advanced concurrently (mixed form)
    against the same members run one after another in the plain FP64 form.
    Many streams are in flight, so this mode times with a device-wide
    synchronize on both sides of the timed region.  Under torchrun the
    members shard by rank (64 per rank, weak scaling)."""
    import torch

    import hmec
    from hmec import synth
    from hmec.ensemble import Ensemble

    torch.cuda.set_device(device_index)
    # every rank advances 64 distinct members: rank r takes members r, r+world, ... of 64*world
    members = shard(synth.ensemble_members(nmembers * world), rank, world)
    common = dict(krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000)
    out = {}
    for form, label in ((hmec.FORM_MIXED, "mixed"), (hmec.FORM_FP64, "fp64")):
        # the FP64 baseline runs one member at a time, each with the settings
        # of a model run alone
        ens = Ensemble(members, concurrent=(form == hmec.FORM_MIXED), form=form, **common)
        (ens.step if form == hmec.FORM_MIXED else ens.step_sequential)(args.warmup)
        torch.cuda.synchronize()
        rank_barrier(world)
        l0 = sum(m.launches for m in ens.models)
        t0 = time.perf_counter()
        reps = (ens.step if form == hmec.FORM_MIXED else ens.step_sequential)(args.steps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        rank_barrier(world)
        out[label] = dict(s=rank_max(el, world), launches=sum(m.launches for m in ens.models) - l0,
                          bad=sum(1 for rs in reps for r in rs if r["rc"] != 0),
                          gi=sum(r["global_iters"] for rs in reps for r in rs))
        ens.close()
    if rank != 0:
        return 0
    K = args.steps
    mx, fp = out["mixed"], out["fp64"]
    value = whole_job_rate(len(members) * K, world, mx["s"])
    line = {
        "metric": METRIC, "value": value, "unit": "member-timesteps/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": 1e3 * mx["s"] / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
        "config": {"workload": "config 3: %d members per GPU, per-side nodes 51-301, 4x4 markers/cell, "
                               "seeded a/b/L/k" % len(members),
                   "form": "mixed, members concurrent (one context and stream each)",
                   "timing": "device-wide synchronize around the timed region (many streams)",
                   "parallelism": "members sharded by rank" if world > 1 else "single",
                   "failed_member_steps": mx["bad"]},
        "gpu_launches": mx["launches"],
        "fp64_sequential": {"value": whole_job_rate(len(members) * K, world, fp["s"]),
                            "ms_per_step": 1e3 * fp["s"] / K, "failed_member_steps": fp["bad"]},
        "speedup_batched_mixed_vs_sequential_fp64": fp["s"] / mx["s"],
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.config == "c3" and args.impl == "ours":
        import torch

        if world > 1:
            torch.cuda.set_device(local)
            torch.distributed.init_process_group("nccl")
        rc = run_ensemble(args, rank, world, local if world > 1 else 0)
        if world > 1:
            torch.distributed.destroy_process_group()
        return rc

    if args.impl == "reference":
        if rank != 0:
            return 0
        steps = max(1, min(args.steps, 2))
        r = cpu_sample(args.config, budget_s=90.0, max_steps=steps)
        line = {
            "metric": METRIC, "value": r["value"], "unit": "timesteps/s", "n_gpus": args.gpus, "steps": r["steps"],
            "warmup": 0, "ms_per_step": 1e3 * r["seconds"] / r["steps"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "form": "CPU oracle: C restatement + SciPy SuperLU direct solve",
                       "global_iters": r["global_iters"], "steps_requested": args.steps},
            "cpu_baseline": {"value": r["value"], "unit": "timesteps/s", "cores": 1, "kind": "port",
                             "sample": "first %d timesteps of %s from the initial state (%.1f s)" %
                                       (r["steps"], args.config, r["seconds"])},
            "e2e": {"value": r["value"], "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    import torch

    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    out, peaks = run_gpu(args, rank, world, local if world > 1 else 0)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0
    mx = out["mixed"]
    K = args.steps
    value = whole_job_rate(K, world, mx["ms"] / 1e3)
    nprof, prof_ms, prof_bytes = mx["prof"]
    achieved = (prof_bytes / nprof) / (prof_ms / nprof / 1e3) / 1e9 if nprof and prof_ms > 0 else None
    peak = peaks.get("hbm_gbs")
    roof = {"kernel": "k_vcycle_stage<float> (mixed-form V-cycle: every level's Vanka smoothing pass in one "
                      "cooperative launch)", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if (achieved and peak) else None, "traffic": SMOOTH_TRAFFIC_BYTES,
            "traffic_note": "bytes per launch (one V-cycle): DRAM read+write from one ncu capture of this kernel",
            "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak else "fallback 6800",
            "launches_timed": nprof, "avg_launch_us": (1e3 * prof_ms / nprof) if nprof else None,
            "share_of_step_time": prof_ms / mx["ms"] if mx["ms"] else None}
    if not peak:
        roof["peak"] = 6800.0
        roof["frac"] = achieved / 6800.0 if achieved else None
    line = {
        "metric": METRIC, "value": value, "unit": "timesteps/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": mx["ms"] / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64/f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "mixed: FP64 FGMRES(40), FP32 Vanka multigrid preconditioner",
                   "krylov_rtol": 1e-15, "l2": "inputs larger than L2 (1M markers x 19 FP64 arrays = 152 MB); "
                   "256 MB buffer written between timed steps", "parallelism": "replicas" if world > 1 else "single",
                   "global_iters_per_step": mx["gi"] / K, "krylov_iters_per_step": mx["kr"] / K,
                   "global_iterations_per_s": world * mx["gi"] / (mx["ms"] / 1e3)},
        "gpu_launches": mx["launches"],
        "roofline": roof,
        "clocks": mx["clocks"],
    }
    if "fp64" in out:
        f = out["fp64"]
        line["fp64_form"] = {"value": world * K / (f["ms"] / 1e3), "ms_per_step": f["ms"] / K,
                             "global_iters_per_step": f["gi"] / K, "krylov_iters_per_step": f["kr"] / K,
                             "mixed_vs_fp64_max_rel_err": f["err"], "same_dt": f["dt_equal"],
                             "err_note": "one timestep from the same state in both forms, max |mixed - fp64| / "
                                         "max |fp64| per field; 'velocity' over vxs and vys together"}
        line["speedup_mixed_vs_fp64"] = value / line["fp64_form"]["value"]
    if "e2e" in out:
        e = out["e2e"]
        line["e2e"] = {"value": world * K / (e["ms"] / 1e3), "unit": "timesteps/s", "h2d_bytes_per_step": e["h2d"],
                       "d2h_bytes_per_step": e["d2h"]}
    if not args.no_cpu_baseline and world == 1:
        r = cpu_sample(args.config, budget_s=25.0, max_steps=2)
        line["cpu_baseline"] = {"value": r["value"], "unit": "timesteps/s", "cores": 1, "kind": "port",
                                "sample": "first %d timesteps of %s from the initial state, %.1f s" %
                                          (r["steps"], args.config, r["seconds"])}
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
