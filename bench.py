#!/usr/bin/env python
"""Simulated timesteps/s of the H-MEC per-timestep hot path on GB300.

A step is one timestep of the reference loop (markers -> nodes, global
iterations with assembly + solve + stress + fault update + adaptive dt, end of
step), run through the C ABI of libhmec_gpu.so on a seeded synthetic model.
The headline line is configuration 2 (1001 x 401 nodes, 40 x 16 km, 6 x 6
markers per cell, 14.4 M markers), where the 5x target is stated: `value` is
the mixed form (FP32 multigrid-preconditioned FP64 FGMRES) with inputs
resident in HBM, `fp64_form` the plain FP64 form on the same steps, `e2e` the
mixed form with the model state copied from pinned host buffers every step.
The same line carries configuration 1 (201 x 201, 1.0 M markers; its
accuracy is measured against the FP64 CPU oracle) and configuration 3 (the
64-member ensemble) as extra blocks.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config c2|c1|c3|c4] [--no-extra] [--no-cpu-baseline]

--impl reference times the CPU restatement of the reference (the oracle: the
reference itself needs Eigen, HDF5 and MKL Pardiso, none of which exist here)
on the host cores, on a bounded sample of the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "h-mecs-2d_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "timesteps/s on 1 GB300: mixed-prec batched vs plain FP64, at ≤1e-8 rel err"
TARGET_REL_ERR = 1e-8

# Per configuration: the workload, and the DRAM bytes (read + write) of one
# launch of the dominant kernel (one V-cycle of the mixed form) from an ncu
# capture of that configuration (profiles/); None where none was taken.
CONFIGS = {
    "c1": dict(workload="config 1: 201x201 nodes, 10x10 km, 5x5 markers/cell (1,000,000 markers), "
                        "seeded synthetic fault model",
               vcycle_dram_bytes=84.04e6, dram_source="profiles/k_vcycle_stage_c1.md"),
    "c2": dict(workload="config 2: 1001x401 nodes, 40x16 km, 6x6 markers/cell (14,400,000 markers), "
                        "log-normal host viscosity (1e22 Pa s, sigma 1 decade), 1e19 Pa s fault band, "
                        "log-uniform permeability 1e-21..1e-14 m^2",
               vcycle_dram_bytes=1.859e9, dram_source="profiles/k_vcycle_stage_c2.md"),
}
DOMINANT = "k_smooth"  # library profiling prefix: the smoothing passes (the fused V-cycle in the mixed form)
FIELDS_ACC = ("vxs", "vys", "pt", "pf", "VSLIPB")
GROUPS_ACC = {"velocity": ("vxs", "vys")}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4"])
    ap.add_argument("--no-extra", action="store_true", help="headline configuration only")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-window", action="store_true",
                    help="for ncu --profile-from-start off: --warmup steps of --config's model in --form, then "
                         "--steps steps between cudaProfilerStart and cudaProfilerStop; no JSON line")
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"], help="the form --profile-window runs")
    ap.add_argument("--markers-per-side", type=int, default=0,
                    help="--profile-window only: markers per cell side instead of the configuration's (a smaller "
                         "capture for the solver's kernels, which do not depend on the marker count)")
    return ap.parse_args()


def profile_window(args):
    """The model of --config (c1, c2) in --form: warm-up steps, then the
    profiled steps bracketed by cudaProfilerStart/Stop.  The steps run
    host-driven: ncu does not profile the kernel nodes of a graph with
    conditional nodes, and the host-driven step launches the same kernels."""
    import torch

    import hmec

    torch.cuda.set_device(0)
    form = hmec.FORM_MIXED if args.form == "mixed" else hmec.FORM_FP64
    extra = dict(mx=args.markers_per_side, my=args.markers_per_side) if args.markers_per_side > 0 else {}
    m, _, _, p = make_model(form, args.config, graph=0, **extra)
    # statuses are not checked: a capture with fewer markers per cell is a
    # different model, which may not converge; the kernels are the same
    for _ in range(args.warmup):
        m.timestep(check=False)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    reps = [m.timestep(check=False) for _ in range(args.steps)]
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print("profiled %d steps of %s (%s): global iterations %s, Krylov iterations %s"
          % (args.steps, args.config, args.form, [r["global_iters"] for r in reps], [r["krylov_iters"] for r in reps]))
    m.close()
    return 0


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


def balanced_split(costs, world):
    """Indices of the work items of each rank, balancing the summed cost:
    longest-processing-time greedy (items by decreasing cost, each to the
    least-loaded rank; ties to the lower index), deterministic."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def member_cost(over):
    """Expected work of an ensemble member: its cells (the iteration counts
    of uneven members are alike, so cells carry the difference)."""
    return float((over["Nx"] + 1) * (over["Ny"] + 1))


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units all ranks processed per second of the slowest rank."""
    return units_per_rank * world / seconds_max


# ------------------------------------------------------------------ helpers
def vcycle_levels(p):
    """Cells (staggered nodes) of each multigrid level, as the library builds them."""
    nx, ny = p.Nx, p.Ny
    out = [(nx + 1) * (ny + 1)]
    while len(out) < max(1, p.mg_levels):
        cx, cy = nx // 2, ny // 2
        if cx < 4 or cy < 4:
            break
        nx, ny = cx + 1, cy + 1
        out.append((nx + 1) * (ny + 1))
    return out


def vcycle_bytes_compulsory(p, value_bytes=4):
    """Compulsory bytes of one V-cycle: per level and sweep, every cell's 42
    coefficients and three six-value vectors (unknowns read and written,
    rhs), (pre + post + 1 residual/restriction) sweeps on each level and
    the coarse sweeps on the coarsest."""
    lv = vcycle_levels(p)
    per = 60.0 * value_bytes
    tot = sum((p.mg_pre + p.mg_post + 1) * per * c for c in lv[:-1])
    return tot + max(1, p.mg_coarse_sweeps) * per * lv[-1]


def rel_errors(got, ref):
    import numpy as np

    out = {}
    for f in ref:
        den = float(np.max(np.abs(ref[f]))) or 1.0
        out[f] = float(np.max(np.abs(got[f] - ref[f]))) / den
    for g, names in GROUPS_ACC.items():
        if all(n in ref for n in names):
            den = max(float(np.max(np.abs(ref[n]))) for n in names) or 1.0
            out[g] = max(float(np.max(np.abs(got[n] - ref[n]))) for n in names) / den
    return out


def against_target(err):
    """The errors the accuracy target is checked on: velocity as one vector field (vys
    alone is near zero in simple shear), pt, pf and the slip rate."""
    keys = ("velocity", "pt", "pf", "VSLIPB")
    worst = max(err[k] for k in keys if k in err)
    return {"checked_on": list(keys), "max": worst, "target": TARGET_REL_ERR, "met": worst <= TARGET_REL_ERR}


# -------------------------------------------------------------------- GPU arm
def make_model(form, cfg, mk=None, nodes=None, **extra):
    import hmec
    from hmec import synth

    over = dict(synth.PRESETS[cfg], form=form, krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000, **extra)
    p = hmec.default_params(**over)
    m = hmec.Model(p)
    if mk is None:
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


def roofline(prof, ms_total, p, peaks, cfg, kernel):
    """The dominant kernel's live roofline from the library's CUDA-event timing."""
    nprof, prof_ms, b_alg, b_moved = prof
    peak = peaks.get("hbm_gbs")
    src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    if not peak:
        peak, src = 6800.0, "fallback 6800"
    per_launch_alg = b_alg / nprof if nprof else None
    achieved = (b_alg / nprof) / (prof_ms / nprof / 1e3) / 1e9 if nprof and prof_ms > 0 else None
    traffic = CONFIGS.get(cfg, {}).get("vcycle_dram_bytes")
    out = {"kernel": kernel, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
           "frac": achieved / peak if achieved else None, "peak_source": src,
           "bytes_per_launch_compulsory": per_launch_alg,
           "bytes_per_launch_moved": (b_moved / nprof) if nprof else None,
           "achieved_moved_gbs": (b_moved / nprof) / (prof_ms / nprof / 1e3) / 1e9 if nprof and prof_ms > 0 else None,
           "compulsory_bytes_model": "per cell and sweep 42 coefficients + 3 x 6 values (FP32: 240 B), "
                                     "(pre + post + 1) sweeps per level, coarse sweeps on the coarsest "
                                     "(V-cycle formula of %.1f MB at this grid)" % (vcycle_bytes_compulsory(p) / 1e6),
           "traffic": traffic,
           "traffic_note": ("DRAM read+write per launch from ncu (%s)" % CONFIGS[cfg]["dram_source"]) if traffic
           else "not captured for this configuration",
           "waste_ratio": (traffic / per_launch_alg) if (traffic and per_launch_alg) else None,
           "launches_timed": nprof, "avg_launch_us": (1e3 * prof_ms / nprof) if nprof else None,
           "share_of_step_time": prof_ms / ms_total if ms_total else None,
           "timing_note": "CUDA events around every launch of the kernel, in a pass of host-driven steps after the "
                          "timed (graph) steps; share = kernel time / step time of that pass"}
    return out


def run_gpu(args, cfg, world, device_index, peaks, with_fp64=True, with_e2e=True, with_acc=True):
    import numpy as np
    import torch

    import hmec

    flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.fill_(1.0)

    out = {}
    m, mk, nodes, p = make_model(hmec.FORM_MIXED, cfg)
    for _ in range(args.warmup):
        m.timestep()
    # the state the timed steps start from: the end-to-end pass restarts
    # from it, so that it times the same steps (same dt, same iterations)
    snap = m.snapshot() if with_e2e else None
    rank_barrier(world)
    torch.cuda.synchronize()
    l0 = m.launches
    with ClockSampler(device_index) as clk:
        ms, reps = timed_steps(m, args.steps, flush)
    launches = m.launches - l0
    graph = m.graph_status
    ms = rank_max(ms, world)
    rank_barrier(world)
    # the dominant kernel's launches timed one by one (CUDA events around each
    # launch need host-driven steps, so this is a separate pass of as many steps)
    m.profile_kernel(DOMINANT)
    pms, _ = timed_steps(m, args.steps, flush)
    prof = m.profile_read()
    m.profile_kernel(None)
    out["mixed"] = dict(ms=ms, reps=reps, launches=launches, gi=sum(r["global_iters"] for r in reps),
                        kr=sum(r["krylov_iters"] for r in reps), clocks=clk.summary(), prof=prof, prof_ms=pms, p=p,
                        graph=graph)

    if with_e2e:
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
        h2d = sum(v.nbytes for v in pin.values()) + sum(v[0].nbytes for v in host_state.values())
        d2h = sum(v[0].nbytes for v in host_out.values()) + sum(v[0].nbytes for v in host_state.values())

        def ptr(flat):
            return flat.ctypes.data_as(C.POINTER(C.c_double))

        up_ids = (C.c_int32 * len(host_state))(*[hmec.FIELDS.index(f) for f in host_state])
        up_ptrs = (C.POINTER(C.c_double) * len(host_state))(*[ptr(v[0]) for v in host_state.values()])
        down = list(host_out.items()) + list(host_state.items())
        down_ids = (C.c_int32 * len(down))(*[hmec.FIELDS.index(f) for f, _ in down])
        down_ptrs = (C.POINTER(C.c_double) * len(down))(*[ptr(v[0]) for _, v in down])

        def hook(phase):
            if phase == "upload":
                m._check(m.L.hmec_upload_fields(m.h, 0, len(host_state), up_ids, up_ptrs), "upload_fields")
            elif phase == "download":
                m._check(m.L.hmec_download_fields(m.h, 0, len(down), down_ids, down_ptrs), "download_fields")

        # the markers: every timestep copies the pinned host arrays in after
        # its markers->nodes section, overlapped with the rest of the step
        # (hmec_stream_markers; the next step uses them), so each timed step
        # still moves every marker array host -> device
        m.stream_markers(pin)
        # after registering, the first step runs host-driven and the second
        # captures the step graph again: both before the timed steps
        m.timestep()
        m.timestep()
        m.load_state(snap)
        for f, (flat, r, c) in host_state.items():
            flat[...] = m.field(f).ravel(order="F")
        rank_barrier(world)
        e2e_ms, e2e_reps = timed_steps(m, args.steps, flush, per_step=hook)
        m.stream_markers(None)
        out["e2e"] = dict(ms=rank_max(e2e_ms, world), h2d=h2d, d2h=d2h,
                          gi=sum(r["global_iters"] for r in e2e_reps), kr=sum(r["krylov_iters"] for r in e2e_reps))
    m.close()

    if with_fp64:
        m2, _, _, _ = make_model(hmec.FORM_FP64, cfg, mk, nodes)
        for _ in range(args.warmup):
            m2.timestep()
        rank_barrier(world)
        ms2, reps2 = timed_steps(m2, args.steps, flush)
        ms2 = rank_max(ms2, world)
        f = dict(ms=ms2, gi=sum(r["global_iters"] for r in reps2), kr=sum(r["krylov_iters"] for r in reps2))
        if with_acc:
            # accuracy of the mixed form against the FP64 form: one timestep
            # from the same state in both (after many steps the two runs' dt
            # sequences part ways on discrete decisions)
            snap = m2.snapshot()
            m2.timestep()
            ref = {k: m2.field(k) for k in FIELDS_ACC}
            dt64 = m2.scalar("dt")
            m3, _, _, _ = make_model(hmec.FORM_MIXED, cfg, mk, nodes)
            m3.load_state(snap)
            m3.timestep()
            f["err"] = rel_errors({k: m3.field(k) for k in FIELDS_ACC}, ref)
            f["same_dt"] = m3.scalar("dt") == dt64
            m3.close()
        m2.close()
        out["fp64"] = f
    return out


# ------------------------------------------------------------------ CPU arm
def host_threads():
    """Host cores this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        return max(1, os.cpu_count() or 1)


def oracle_steps(cfg, nsteps, budget_s, threads=1):
    """The CPU oracle (restatement of the reference) on the first steps of cfg
    from the initial state; returns its timing and the fields of FIELDS_ACC.
    threads: the marker loop's threads (the reference's OpenMP loop); the
    rest runs on one thread, as the reference's does."""
    import oracle as O
    from hmec import synth

    p = O.default_params(**synth.PRESETS[cfg])
    o = O.Oracle(p)
    o.set_threads(threads)
    mk, nodes = synth.make_state(p, cfg)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    t0 = time.perf_counter()
    steps = gi = 0
    while steps < nsteps:
        gi += o.timestep()
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return dict(value=steps / el, steps=steps, seconds=el, global_iters=gi,
                fields={k: o.field(k).copy() for k in FIELDS_ACC}, mk=mk, nodes=nodes)


def oracle_sample_no_solve(cfg, global_iters_per_step, threads=1):
    """A bounded CPU sample of one timestep of a configuration too large for a
    direct solve per global iteration (config 2: one SuperLU solve of its
    2.4 M unknowns takes minutes): the oracle's markers -> nodes (the marker
    loop on `threads` threads, as the reference's OpenMP loop), step begin,
    and per global iteration the preparation and assembly, timed; the direct
    solves and the sections after them are left out, so the rate is an upper
    bound of the oracle's timesteps/s.  The marker loop is also timed on one
    thread (p2g_1_s)."""
    import oracle as O
    from hmec import synth

    p = O.default_params(**synth.PRESETS[cfg])
    o = O.Oracle(p)
    mk, nodes = synth.make_state(p, cfg)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    t0 = time.perf_counter()
    o.markers_to_nodes()
    t1 = time.perf_counter()
    o.set_threads(threads)
    t2 = time.perf_counter()
    o.markers_to_nodes()
    o.timestep_begin()
    t3 = time.perf_counter()
    o.iter_prepare()
    o.assemble()
    t4 = time.perf_counter()
    per_step = (t3 - t2) + global_iters_per_step * (t4 - t3)
    return dict(value=1.0 / per_step, seconds=t4 - t0, p2g_s=t3 - t2, p2g_1_s=t1 - t0, assemble_s=t4 - t3,
                threads=threads)


def cpu_block(cfg, gi_per_step):
    nt = host_threads()
    if cfg == "c2":
        r = oracle_sample_no_solve(cfg, gi_per_step, nt)
        return {"value": r["value"], "unit": "timesteps/s", "cores": nt, "kind": "port", "upper_bound": True,
                "marker_loop_s": {"threads": nt, "all_threads": r["p2g_s"], "one_thread": r["p2g_1_s"]},
                "sample": "config 2, first timestep: oracle markers->nodes + step begin (%.2f s, the marker loop on "
                          "%d threads as the reference's OpenMP loop; %.2f s on one) and one global iteration's "
                          "preparation + assembly (%.2f s, one thread) x %.1f global iterations per step; the "
                          "direct solves (SuperLU, single thread, minutes each at 2.4 M unknowns) and the "
                          "sections after them are not run, so this is an upper bound"
                          % (r["p2g_s"], nt, r["p2g_1_s"], r["assemble_s"], gi_per_step)}
    r = oracle_steps(cfg, 3, 40.0, nt)
    return {"value": r["value"], "unit": "timesteps/s", "cores": nt, "kind": "port",
            "sample": "first %d timesteps of %s from the initial state, %.1f s (oracle: C restatement, the marker "
                      "loop on %d threads as the reference's OpenMP loop, the rest and the SciPy SuperLU direct "
                      "solve on one thread)" % (r["steps"], cfg, r["seconds"], nt)}


# ------------------------------------------------------------------ ensembles
def member_oracle_error(over, mat, seed, fields_after_step1):
    """One member's first timestep on the FP64 oracle from the member's
    initial state, against the ensemble's result for that member."""
    import oracle as O
    from hmec import synth

    o = O.Oracle(O.default_params(**dict(over, krylov_rtol=1e-15)))
    mk, nodes = synth.instance_state(o.params, mat, seed)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    gi = o.timestep()
    err = rel_errors(fields_after_step1, {k: o.field(k) for k in FIELDS_ACC})
    return dict(err, **against_target(err), Nx=over["Nx"], Ny=over["Ny"], prestress_pa=mat.get("prestress", 0.0),
                oracle_global_iters=gi, oracle_dt=o.scalar("dt"))


def run_c4(args, device_index=0):
    """Configuration 4: 256 instances (101..401 x 101..201 nodes) at seeded
    cycle phases in one context, one graph launch per ensemble step; the
    aggregate member-timesteps/s, the instances' dt spread, and the errors of
    sampled instances' first step against the FP64 oracle."""
    import numpy as np
    import torch

    import hmec
    from hmec import synth
    from hmec.ensemble import Ensemble

    torch.cuda.set_device(device_index)
    members = synth.ensemble_members_c4(256)
    common = dict(krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000, form=hmec.FORM_MIXED)
    t0 = time.perf_counter()
    ens = Ensemble(members, **common)
    t_create = time.perf_counter() - t0
    # sampled instances: the smallest of each cycle phase
    sample = {}
    for k, (o, mat, sd) in enumerate(members):
        ph = mat.get("prestress", 0.0)
        if ph not in sample or o["Nx"] * o["Ny"] < members[sample[ph]][0]["Nx"] * members[sample[ph]][0]["Ny"]:
            sample[ph] = k
    first = ens.step(1)
    after1 = {k: {f: ens.members[k].field(f) for f in FIELDS_ACC} for k in sample.values()}
    ens.step(max(0, args.warmup - 1))
    torch.cuda.synchronize()
    l0 = ens.launches
    with ClockSampler(device_index) as clk:
        t0 = time.perf_counter()
        reps = ens.step(args.steps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
    launches = ens.launches - l0
    dts = np.array([ens.members[k].scalar("dt") for k in range(len(members))])
    graph = ens.graph_status
    gi = sum(r["global_iters"] for rs in reps for r in rs)
    bad = sum(1 for rs in reps for r in rs if r["rc"] != 0)
    ens.close()
    errs = [member_oracle_error(*members[k], after1[k]) for k in sample.values()]
    K = args.steps
    return {"value": len(members) * K / el, "unit": "member-timesteps/s", "ms_per_step": 1e3 * el / K, "steps": K,
            "workload": "config 4: 256 instances, nodes 101-401 x 101-201, 4x4 markers/cell (%.0f M markers, "
                        "%.1f M cells), seeded a/b/L/k and cycle phases (%s)"
                        % (sum((o["Nx"] - 1) * (o["Ny"] - 1) * 16 for o, _, _ in members) / 1e6,
                           sum((o["Nx"] + 1) * (o["Ny"] + 1) for o, _, _ in members) / 1e6,
                           ", ".join("%d%% at %g MPa pre-stress" % (100 * f, t / 1e6) for f, t in synth.C4_PHASES)),
            "form": "mixed, all instances in one context: one CUDA graph launch per ensemble step",
            "step_as_one_graph_launch": graph == 1, "create_seconds": t_create,
            "global_iters_per_member_step": gi / (len(members) * K), "failed_member_steps": bad,
            "dt_after_timed_steps": {"min": float(dts.min()), "median": float(np.median(dts)),
                                     "max": float(dts.max())},
            "first_step_global_iters": {"min": min(r[0]["global_iters"] for r in first),
                                        "max": max(r[0]["global_iters"] for r in first)},
            "gpu_launches": launches, "clocks": clk.summary(),
            "sampled_instances_vs_oracle": errs,
            "sampled_note": "first timestep of the smallest instance of each cycle phase, ensemble result "
                            "against the FP64 oracle from the same initial state"}


def run_ensemble(args, rank=0, world=1, device_index=0, nmembers=64):
    """Configuration 3: 64 uneven members in one context, one graph launch per
    ensemble step (mixed form), against the same members run one after
    another in the plain FP64 form, each in a context of its own.  Many
    streams are in flight, so this mode times with a device-wide synchronize
    on both sides of the timed region.  Under torchrun the members shard by
    rank with balanced cells (64 per rank, weak scaling)."""
    import torch

    import hmec
    from hmec import synth
    from hmec.ensemble import Ensemble, Sequential

    torch.cuda.set_device(device_index)
    allm = synth.ensemble_members(nmembers * world)
    parts = balanced_split([member_cost(o) for o, _, _ in allm], world)
    members = [allm[i] for i in parts[rank]]
    common = dict(krylov_rtol=1e-15, krylov_restart=40, krylov_maxit=4000)
    out = {}
    for form, label in ((hmec.FORM_MIXED, "mixed"), (hmec.FORM_FP64, "fp64")):
        # mixed: all members in one context, one graph launch per ensemble
        # step; the FP64 baseline runs one member at a time, each in a
        # context of its own with the settings of a model run alone
        ens = (Ensemble if form == hmec.FORM_MIXED else Sequential)(members, form=form, **common)
        ens.step(args.warmup)
        torch.cuda.synchronize()
        rank_barrier(world)
        l0 = ens.launches
        with ClockSampler(device_index) as clk:
            t0 = time.perf_counter()
            reps = ens.step(args.steps)
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
        rank_barrier(world)
        launches = ens.launches - l0
        prof = None
        graph = None
        if form == hmec.FORM_MIXED:
            graph = ens.graph_status
            # one profiled step for the smoothing kernel's roofline (host-driven)
            for m in ens.members:
                m.profile_kernel(DOMINANT)
            ens.step(1)
            tot = [0, 0.0, 0.0, 0.0]
            for m in ens.members:
                for i, v in enumerate(m.profile_read()):
                    tot[i] += v
                m.profile_kernel(None)
            prof = tuple(tot)
        out[label] = dict(s=rank_max(el, world), launches=launches,
                          bad=sum(1 for rs in reps for r in rs if r["rc"] != 0),
                          gi=sum(r["global_iters"] for rs in reps for r in rs), clocks=clk.summary(), prof=prof,
                          graph=graph)
        ens.close()
    return out, members


def ensemble_block(args, out, members, world, peaks):
    K = args.steps
    mx, fp = out["mixed"], out["fp64"]
    nprof, prof_ms, b_alg, b_moved = mx["prof"]
    peak = peaks.get("hbm_gbs") or 6800.0
    ach = (b_alg / nprof) / (prof_ms / nprof / 1e3) / 1e9 if nprof and prof_ms > 0 else None
    return {
        "value": whole_job_rate(len(members) * K, world, mx["s"]), "unit": "member-timesteps/s",
        "workload": "config 3: %d members per GPU, per-side nodes 51-301, 4x4 markers/cell, seeded a/b/L/k"
                    % len(members),
        "form": "mixed, all members in one context: one CUDA graph launch per ensemble step (each member's "
                "global-iteration, restart and Arnoldi loops as conditional nodes, one launch per smoothing pass "
                "on at most a quarter of the SMs)",
        "step_as_one_graph_launch": mx["graph"] == 1,
        "timing": "device-wide synchronize around the timed region (many streams)",
        "ms_per_step": 1e3 * mx["s"] / K, "steps": K, "failed_member_steps": mx["bad"],
        "gpu_launches": mx["launches"], "clocks": mx["clocks"],
        "roofline": {"kernel": "k_smooth_stage<float> (one smoothing pass per launch, all members)", "bound": "hbm",
                     "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak if ach else None,
                     "launches_timed": nprof, "avg_launch_us": 1e3 * prof_ms / nprof if nprof else None,
                     "note": "compulsory bytes per launch over its CUDA-event duration, timed in one host-driven "
                             "step of every member after the timed steps"},
        "fp64_sequential": {"value": whole_job_rate(len(members) * K, world, fp["s"]),
                            "ms_per_step": 1e3 * fp["s"] / K, "failed_member_steps": fp["bad"]},
        "speedup_mixed_vs_fp64": fp["s"] / mx["s"],
    }


# ------------------------------------------------------------------ lines
def model_block(args, cfg, world, res, peaks):
    mx = res["mixed"]
    K = args.steps
    p = mx["p"]
    blk = {
        "value": whole_job_rate(K, world, mx["ms"] / 1e3), "unit": "timesteps/s", "ms_per_step": mx["ms"] / K,
        "workload": CONFIGS[cfg]["workload"],
        "form": "mixed: FP64 FGMRES(40), FP32 Vanka multigrid preconditioner",
        "global_iters_per_step": mx["gi"] / K, "krylov_iters_per_step": mx["kr"] / K,
        "global_iterations_per_s": world * mx["gi"] / (mx["ms"] / 1e3), "gpu_launches": mx["launches"],
        "step_as_one_graph_launch": mx["graph"] == 1,
        "roofline": roofline(mx["prof"], mx["prof_ms"], p, peaks, cfg,
                             "k_vcycle_stage<float> (mixed-form V-cycle: every level's Vanka smoothing pass in "
                             "one cooperative launch)"),
        "clocks": mx["clocks"],
    }
    if "fp64" in res:
        f = res["fp64"]
        blk["fp64_form"] = {"value": world * K / (f["ms"] / 1e3), "ms_per_step": f["ms"] / K,
                            "global_iters_per_step": f["gi"] / K, "krylov_iters_per_step": f["kr"] / K}
        if "err" in f:
            blk["mixed_vs_fp64_form_rel_err"] = dict(f["err"], same_dt=f["same_dt"], **against_target(f["err"]))
            blk["mixed_vs_fp64_form_rel_err"]["note"] = ("one timestep from the same state in both forms, "
                                                         "max |mixed - fp64| / max |fp64| per field; 'velocity' "
                                                         "over vxs and vys together")
        blk["speedup_mixed_vs_fp64"] = blk["value"] / blk["fp64_form"]["value"]
    if "e2e" in res:
        e = res["e2e"]
        blk["e2e"] = {"value": world * K / (e["ms"] / 1e3), "unit": "timesteps/s", "h2d_bytes_per_step": e["h2d"],
                      "d2h_bytes_per_step": e["d2h"], "global_iters_per_step": e["gi"] / K,
                      "krylov_iters_per_step": e["kr"] / K,
                      "how": "through the C ABI with host buffers: per step the model state uploaded from and the "
                             "new state and outputs downloaded to pinned host arrays (CUDA events around each "
                             "step's calls), and every marker array copied in from pinned host memory by the "
                             "library's marker stream (hmec_stream_markers) overlapped with the step's solve; "
                             "the same steps as the device-timed ones (restarted from their initial state)"}
    return blk


def accuracy_vs_oracle(cfg, nsteps=3):
    """Mixed and plain FP64 forms against the FP64 CPU oracle (its direct
    solve stands in for Pardiso): step `nsteps` (the fault active) replayed
    on the GPU from the oracle's state after nsteps - 1 steps -- the per-step
    error the target is stated on -- and, for reference, after nsteps
    free-running steps from the same initial state.  Also the oracle's timing."""
    import hmec
    import oracle as O
    from hmec import synth

    p = O.default_params(**synth.PRESETS[cfg])
    o = O.Oracle(p)
    mk, nodes = synth.make_state(p, cfg)
    o.set_markers(mk)
    for k, v in nodes.items():
        o.set_field(k, v)
    t0 = time.perf_counter()
    for _ in range(nsteps - 1):
        o.timestep()
    snap = o.snapshot()
    o.timestep()
    el = time.perf_counter() - t0
    ref = {k: o.field(k).copy() for k in FIELDS_ACC}
    out = {"replayed_step": nsteps, "oracle_seconds": el,
           "note": "replay: both sides start step %d from the oracle's state; free running: %d steps from the "
                   "initial state (round-off amplified by the plastic iterations near yield)" % (nsteps, nsteps)}
    for form, label in ((hmec.FORM_MIXED, "mixed"), (hmec.FORM_FP64, "fp64_form")):
        m, _, _, _ = make_model(form, cfg, mk, nodes)
        m.load_state(snap)
        m.timestep()
        err = rel_errors({k: m.field(k) for k in FIELDS_ACC}, ref)
        m.close()
        m, _, _, _ = make_model(form, cfg, mk, nodes)
        for _ in range(nsteps):
            m.timestep()
        free = rel_errors({k: m.field(k) for k in FIELDS_ACC}, ref)
        m.close()
        out[label] = dict(err, **against_target(err))
        out[label]["free_running"] = free
    # the oracle's own floor: the replayed step solved again with another
    # partial-pivoting threshold (the same system, other rounding)
    o2 = O.Oracle(p)
    o2.pivot_thresh = 0.1
    o2.set_markers(mk)
    o2.load_state(snap)
    o2.timestep()
    fl = rel_errors({k: o2.field(k) for k in FIELDS_ACC}, ref)
    out["oracle_floor"] = dict(fl, **against_target(fl))
    out["oracle_floor"]["note"] = ("the oracle against itself: step %d re-solved with partial-pivoting threshold "
                                   "0.1 instead of 1.0; near yield the plastic iterations amplify last-bit "
                                   "differences of the solve by up to ~1e7" % nsteps)
    cpu = {"value": nsteps / el, "unit": "timesteps/s", "cores": 1, "kind": "port",
           "sample": "first %d timesteps of %s from the initial state, %.1f s (oracle: C restatement + SciPy "
                     "SuperLU direct solve, one thread)" % (nsteps, cfg, el)}
    return out, cpu


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        cfg = "c1" if args.config == "c3" else args.config
        nt = host_threads()
        if cfg == "c2":
            r = oracle_sample_no_solve(cfg, 2.0, nt)
            val, steps = r["value"], 1
            sample = ("config 2, first timestep: markers->nodes (the marker loop on %d threads, as the reference's "
                      "OpenMP loop) + step begin and one global iteration's preparation + assembly (one thread) x 2 "
                      "global iterations per step; direct solves not run (upper bound)" % nt)
        else:
            r = oracle_steps(cfg, max(1, min(args.steps, 2)), 90.0, nt)
            val, steps = r["value"], r["steps"]
            sample = ("first %d timesteps of %s from the initial state (the marker loop on %d threads, the rest "
                      "and the direct solve on one, as the reference's)" % (steps, cfg, nt))
        line = {
            "metric": METRIC, "value": val, "unit": "timesteps/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": 0, "ms_per_step": 1e3 / val, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": CONFIGS[cfg]["workload"],
                       "form": "CPU oracle: C restatement + SciPy SuperLU direct solve", "steps_requested": args.steps},
            "cpu_baseline": {"value": val, "unit": "timesteps/s", "cores": nt, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "timesteps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return 0

    if args.profile_window:
        return profile_window(args)

    import torch

    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = local if world > 1 else 0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass

    if args.config == "c4":
        blk = run_c4(args, dev)
        line = {"metric": METRIC, "value": blk["value"], "unit": blk["unit"], "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": blk["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
                "config": {k: blk[k] for k in ("workload", "form", "global_iters_per_member_step",
                                                "failed_member_steps", "dt_after_timed_steps",
                                                "first_step_global_iters", "create_seconds")},
                "gpu_launches": blk["gpu_launches"], "clocks": blk["clocks"],
                "step_as_one_graph_launch": blk["step_as_one_graph_launch"],
                "sampled_instances_vs_oracle": blk["sampled_instances_vs_oracle"],
                "sampled_note": blk["sampled_note"]}
        print(json.dumps(line))
        return 0

    if args.config == "c3":
        out, members = run_ensemble(args, rank, world, dev)
        if rank == 0:
            blk = ensemble_block(args, out, members, world, peaks)
            line = {"metric": METRIC, "value": blk["value"], "unit": blk["unit"], "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": blk["ms_per_step"], "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
                    "config": {"workload": blk["workload"], "form": blk["form"], "timing": blk["timing"],
                               "parallelism": "members sharded by rank (balanced cells)" if world > 1 else "single"},
                    "gpu_launches": blk["gpu_launches"], "roofline": blk["roofline"], "clocks": blk["clocks"],
                    "fp64_sequential": blk["fp64_sequential"],
                    "speedup_mixed_vs_fp64": blk["speedup_mixed_vs_fp64"]}
            print(json.dumps(line))
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    cfg = args.config
    res = run_gpu(args, cfg, world, dev, peaks, with_fp64=not args.no_fp64, with_e2e=not args.no_e2e)
    extra = {}
    if not args.no_extra and world == 1:
        other = "c1" if cfg == "c2" else "c2"
        r2 = run_gpu(args, other, world, dev, peaks, with_e2e=False)
        extra["config%s" % other[1]] = model_block(args, other, world, r2, peaks)
        eo, emem = run_ensemble(args, rank, world, dev)
        extra["config3"] = ensemble_block(args, eo, emem, world, peaks)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0
    blk = model_block(args, cfg, world, res, peaks)
    K = args.steps
    line = {
        "metric": METRIC, "value": blk["value"], "unit": "timesteps/s", "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": blk["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64/f32", "data": "synthetic",
        "config": {"workload": blk["workload"], "form": blk["form"], "krylov_rtol": 1e-15,
                   "l2": "inputs larger than L2 (marker arrays alone: 19 FP64 arrays x markers); 256 MB buffer "
                         "written between timed steps", "parallelism": "replicas" if world > 1 else "single",
                   "global_iters_per_step": blk["global_iters_per_step"],
                   "krylov_iters_per_step": blk["krylov_iters_per_step"],
                   "global_iterations_per_s": blk["global_iterations_per_s"]},
        "gpu_launches": blk["gpu_launches"],
        "roofline": blk["roofline"],
        "clocks": blk["clocks"],
    }
    for k in ("fp64_form", "mixed_vs_fp64_form_rel_err", "speedup_mixed_vs_fp64", "e2e"):
        if k in blk:
            line[k] = blk[k]
    if not args.no_cpu_baseline and world == 1:
        if cfg == "c1":
            acc, cpu = accuracy_vs_oracle("c1")
            line["mixed_vs_oracle_rel_err"] = acc
            line["cpu_baseline"] = cpu
        else:
            line["cpu_baseline"] = cpu_block(cfg, blk["global_iters_per_step"])
            if "config1" in extra:
                acc, cpu = accuracy_vs_oracle("c1")
                extra["config1"]["mixed_vs_oracle_rel_err"] = acc
                extra["config1"]["cpu_baseline"] = cpu
    line.update(extra)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
