"""Benchmark: 3D travel-time grids/s of the level-set fast-sweeping solver on GB300.

Workload (the reference's plain 3D configuration): a 256 x 256 x 128 grid, h = 50 m,
8 horizontal layers with velocities uniform in [3000, 7000] m/s increasing with depth,
times (1 + p) for a Gaussian random field p (correlation length 1 km, +-5 %), nodal
velocities -> cell slowness; FP32 sweeps with FP64 corner initialisation; factored radius
3; refinement iterations until the largest decrease of an iteration is below 1e-5 s
(at most 10).  A step solves FIELDS independent fields (one seeded source each) in one
batched launch schedule.  The data are synthetic (seeded), generated by
eikonalxx_gb300/synthetic.py.

Prints one JSON line (rank 0).  ``value`` is device-timed throughput with the model
resident in HBM; ``e2e`` times the public API call a user makes (nodal velocities from
pinned host memory in, travel-time fields to pinned host memory out) every step.
``--impl reference`` times the reference's CPU sweep code (oracle/_ref when it was built
here, else the project's bit-identical CPU port) on the host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D travel-time grids/s at max err <=1e-4 s vs FP64; batched+learned vs plain"
NX, NY, NZ, H = 256, 256, 128, 50.0
MODEL_SEED, SOURCE_SEED = 20240601, 7
N_SWEEPS_MAX, TOL, RADIUS = 10, 1e-5, 3
SURFACE = [False]  # sources on the top surface (station tables by reciprocity)
SLAB = [False]     # layered + GRF model with a dipping high-velocity slab (full-scale workload)
PAIR = [False]  # pair_fields option of the GPU arm (set from the command line)
# FP32 sweeps whose factored (near-source) updates run in FP64: the analytic factor
# T0 = distance x source slowness, its gradient and tau in double (eikx_options.near_fp64)
NEAR64 = [True]
KERNEL = [0]    # sweep_kernel option of the GPU arm: 0 default, 1 node-step, 2 chunk-step
# the plain workload as a stream: this many fields in flight (eikx_options.max_in_flight),
# a converged field's slot taking the next source; 0 = all the step's sources as one batch
IN_FLIGHT = [0]
L2_BYTES = 129 * 2 ** 20
BYTES_PER_NODE_SWEEP = 12          # FP32: read T, read slowness, write T


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return world, rank


def host_available_bytes():
    """Host memory this process may still pin: MemAvailable, capped by the cgroup limit."""
    avail = 0
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    avail = int(line.split()[1]) * 1024
        with open("/sys/fs/cgroup/memory.max") as f:
            lim = f.read().strip()
        if lim.isdigit():
            avail = min(avail, int(lim))
    except OSError:
        pass
    return avail


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic():
    """DRAM bytes per sweep launch from the committed ncu summary, or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "sweep3d_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


def refinement_roofline(solve, opts, opts_init, bytes_per_update):
    """Roofline of the refinement sweeps of one solve.  `solve(options)` runs the solve and
    returns its statistics.  Time: the CUDA-event time of all sweep launches minus that of
    the initialisation pass alone (a second solve with no refinement iteration).  Work: the
    node updates the refinement sweeps performed, from the solve's statistics -- fields
    that converged are skipped by the later launches, so the count is not fields x
    launches."""
    st0 = solve(opts_init)
    st = solve(opts)
    refine_ms = st["sweep_ms"] - st0["sweep_ms"]
    launches = st["sweeps_launched"] - st0["sweeps_launched"]
    updates = st["refine_node_updates"]
    algorithmic = bytes_per_update * updates
    return {"achieved": algorithmic / (refine_ms / 1e3) / 1e9, "algorithmic_bytes": algorithmic,
            "node_updates": updates, "refine_ms": refine_ms, "refine_launches": launches,
            "launch_ms": refine_ms / max(1, launches)}


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.samples = []
        self._stop = threading.Event()
        self._proc = None
        self.device_index = device_index

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for s in self.samples for n, v in zip(names, s[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(fields):
    from eikonalxx_gb300 import synthetic
    v = (synthetic.slab_model(NX, NY, NZ, H, MODEL_SEED) if SLAB[0] else
         synthetic.layered_grf_model(NX, NY, NZ, H, MODEL_SEED))
    src = synthetic.uniform_sources(fields, NX, NY, NZ, H, SOURCE_SEED, surface=SURFACE[0])
    return v, src


def workload_config(fields, world):
    """The `config` of the 3D workloads' lines (the GPU arm and the reference arm alike)."""
    return {"workload": (f"full scale, {NX}x{NY}x{NZ} h={H:g} m layered+GRF with an 8000 m/s slab dipping 30 "
                         f"degrees, {fields} sources on the top surface per step per GPU" if SLAB[0] else
                         f"station tables, {NX}x{NY}x{NZ} h={H:g} m layered+GRF, {fields} sources on the "
                         f"top surface per step per GPU, one persistent launch per sweep" if SURFACE[0] else
                         (f"plain 3D solve, {NX}x{NY}x{NZ} h={H:g} m layered+GRF, a stream of {fields} "
                          f"independent sources per step per GPU, {IN_FLIGHT[0]} in flight" if 0 < IN_FLIGHT[0] < fields
                          else f"plain 3D solve, {NX}x{NY}x{NZ} h={H:g} m layered+GRF, "
                               f"{fields} independent sources per step per GPU")),
            "grid": [NX, NY, NZ], "h_m": H, "fields_per_step": fields,
            "precision": ("fp32 sweeps; fp64 source init and factored (near-source) branch" if NEAR64[0] else
                          "fp32 sweeps, fp64 source init"),
            "factored_radius": RADIUS, "tolerance_s": TOL, "max_iterations": N_SWEEPS_MAX,
            "in_flight": IN_FLIGHT[0] if 0 < IN_FLIGHT[0] < fields else fields,
            "l2": "flushed (write of 2x L2) between timed steps; per-step fields exceed L2",
            "parallelism": f"replicas x{world} (sources sharded, no collective)"}


FP64_TOL, FP64_MAX_ITERATIONS, ACCURACY_FIELDS = 1e-9, 40, 8


def fp64_sweeps_arm(ctx, src, opt, ex, pick, judge, max_fields, dev):
    """The precision that meets the bound where FP32 may not: FP64 sweeps at the workload's
    own tolerance and iteration cap.  grids/s over up to `max_fields` of the workload's
    sources (device-timed, device output), and the error of its fields `pick` against the
    converged FP64 solves `judge`."""
    import torch
    n = min(len(src), max_fields)
    o = ex.Options(n_sweeps=opt.n_sweeps, tolerance=opt.tolerance, factored_radius=opt.factored_radius)
    out = torch.empty((n, NZ, NY, NX), dtype=torch.float64, device=f"cuda:{dev}")
    ms = []
    for i in range(3):
        ctx.solve3d(src[:n], o, ex.F64, out=out)
        if i:
            ms.append(ctx.stats()["device_ms"])
    del out
    t = ctx.solve3d(src[pick], o, ex.F64)
    err = max(float(np.abs(a - b).max()) for a, b in zip(t, judge))
    return {"grids_s": n / (float(np.mean(ms)) / 1e3), "fields_timed": n, "max_err_vs_fp64_converged_s": err,
            "meets_1e-4": bool(err <= 1e-4), "tolerance_s": opt.tolerance}


def fp64_accuracy(ctx, src, opt, ex, n_fields=ACCURACY_FIELDS, seed=3, fp64_arm_fields=0, dev=0):
    """Max and RMS error of the FP32 fields of `n_fields` seeded sources of `src` (solved
    with the timed options `opt`) against FP64 solves of the same sources run to
    convergence (tolerance 1e-9 s, at most 40 iterations), over all their nodes.  With
    fp64_arm_fields > 0 it adds the FP64-sweeps arm (fp64_sweeps_arm) over that many fields."""
    pick = np.sort(np.random.default_rng(seed).choice(len(src), min(n_fields, len(src)), replace=False))
    t32 = ctx.solve3d(src[pick], opt, ex.F32)
    o64 = ex.Options(n_sweeps=FP64_MAX_ITERATIONS, tolerance=FP64_TOL, factored_radius=opt.factored_radius)
    t64 = ctx.solve3d(src[pick], o64, ex.F64)
    st = ctx.stats()
    mx, sq, n = 0.0, 0.0, 0
    per = []
    for a, b in zip(t32, t64):
        d = np.abs(a.astype(np.float64) - b)
        per.append(float(d.max()))
        mx = max(mx, per[-1])
        sq += float(np.sum(d * d))
        n += d.size
    acc = {"max_err_vs_fp64_s": mx, "rms_err_vs_fp64_s": float(np.sqrt(sq / n)), "meets_1e-4": bool(mx <= 1e-4),
           "fields_checked": [int(i) for i in pick], "max_err_per_field_s": per,
           "fp64_tolerance_s": FP64_TOL, "fp64_iterations_max": st["iterations_max"],
           "fp64_converged": bool(st["iterations_max"] < FP64_MAX_ITERATIONS)}
    if fp64_arm_fields > 0:
        acc["fp64_sweeps"] = fp64_sweeps_arm(ctx, src, opt, ex, pick, t64, fp64_arm_fields, dev)
    return acc


def run_gpu(args):
    import torch
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import sharding

    world, rank = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    fields = args.fields
    v, src_all = make_workload(fields * world)
    src = src_all[sharding.shard(fields * world, world, rank)]   # weak scaling: each rank its own fields
    n_nodes = NX * NY * NZ

    ctx = ex.Context(dev)
    ctx.set_grid3d(NX, NY, NZ, H, H, H)
    v_host = torch.from_numpy(v.ravel()).pin_memory()
    ctx.set_nodal_velocity3d(v_host)
    stream = 0 < IN_FLIGHT[0] < fields
    slots = IN_FLIGHT[0] if stream else fields          # fields per sweep launch
    opt = ex.Options(n_sweeps=N_SWEEPS_MAX, tolerance=TOL, factored_radius=RADIUS, pair_fields=PAIR[0],
                     sweep_kernel=KERNEL[0], near_fp64=NEAR64[0], max_in_flight=slots if stream else 0)
    out_dev = torch.empty((fields, NZ, NY, NX), dtype=torch.float32, device=f"cuda:{dev}")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")

    # autotuning (outside the timed region): kernel variant, warp-block shape, grid size
    tuning = None
    if not args.no_autotune and KERNEL[0] == 0 and not PAIR[0]:
        # a stream launches its slots' fields: tuned on that many sources
        tuning = ctx.autotune3d(src[:slots], ex.F32)

    def step_device():
        ctx.solve3d(src, opt, ex.F32, out=out_dev)
        return ctx.stats()

    # accuracy (not timed): a seeded sample of the step's fields, solved with the timed
    # options, against FP64 solves of the same sources run to convergence (GPU FP64 is
    # bit-identical to the FP64 oracle in the tests)
    acc = {}
    if rank == 0 and not args.skip_accuracy:
        # the FP64-sweeps arm where the FP32 fields may miss the bound: the station tables and
        # the full-scale slab model (at most 32 fields of the latter: FP64 fields of 67 M nodes)
        acc = fp64_accuracy(ctx, src, opt, ex, fp64_arm_fields=(32 if SLAB[0] else fields) if SURFACE[0] else 0,
                            dev=dev)
        if not SLAB[0]:
            # against closed forms on the same grid: constant velocity, and a linear gradient
            # from the top to the bottom of the grid (nodal model, one source)
            for name, (vt, vb) in {"constant_velocity_5000": (5000.0, 5000.0),
                                   "linear_gradient_3000_7000": (3000.0, 7000.0)}.items():
                vz = vt + (vb - vt) * np.arange(NZ) / (NZ - 1)
                vm = np.ascontiguousarray(np.broadcast_to(vz[:, None, None], (NZ, NY, NX)), dtype=np.float32)
                ctx.set_nodal_velocity3d(vm)
                ta = ctx.analytic3d(src[0], vt, vb)
                e32 = np.abs(ctx.solve3d(src[:1], opt, ex.F32)[0].astype(np.float64) - ta)
                o64 = ex.Options(n_sweeps=FP64_MAX_ITERATIONS, tolerance=FP64_TOL, factored_radius=RADIUS)
                e64 = np.abs(ctx.solve3d(src[:1], o64, ex.F64)[0] - ta)
                acc[name] = {"fp32_max_s": float(e32.max()), "fp32_rms_s": float(np.sqrt(np.mean(e32 ** 2))),
                             "fp64_max_s": float(e64.max()), "fp64_rms_s": float(np.sqrt(np.mean(e64 ** 2)))}
            ctx.set_nodal_velocity3d(v_host)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    sharding.barrier()
    per_step_ms, iters, launches, wall = [], [], 0, []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)             # evict L2 between timed steps (outside the timing)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = step_device()
            wall.append((time.perf_counter() - t0) * 1e3)
            per_step_ms.append(st["device_ms"])
            iters.append((st["iterations_min"], st["iterations_max"]))
            launches += st["kernel_launches"]
    torch.cuda.synchronize()
    sharding.barrier()
    ms = sharding.max_over_ranks(float(np.mean(per_step_ms)), device=f"cuda:{dev}")
    value = fields * world / (ms / 1e3)

    # end to end through the public API with host buffers every step, right after the
    # device-timed steps (the same GPU state), its clocks sampled as well.  Consecutive steps
    # write alternate pinned output buffers, as a pipeline whose consumer reads one step's
    # fields while the next step runs would (one buffer when host memory is short).  On the
    # GB300 hosts the device-to-host rate differed from one 34 GB pinned buffer to the next
    # (85 to 193 GB/s), and a slow buffer slowed further with each step that rewrote it; the
    # per-step times are in the e2e record.
    out_bytes = 4 * fields * n_nodes
    local_ranks = int(os.environ.get("LOCAL_WORLD_SIZE", "1"))
    n_out = 2 if 2 * out_bytes * local_ranks < 0.6 * host_available_bytes() else 1
    out_hosts = [torch.empty((fields, NZ, NY, NX), dtype=torch.float32).pin_memory() for _ in range(n_out)]
    e2e_ms = []
    with ClockSampler(dev) as clk_e2e:
        for i in range(max(1, args.warmup) + args.steps):
            t0 = time.perf_counter()
            ctx.set_nodal_velocity3d(v_host)
            ctx.solve3d(src, opt, ex.F32, out=out_hosts[i % n_out])
            if i >= max(1, args.warmup):
                e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = fields * world / (float(np.mean(e2e_ms)) / 1e3)

    # roofline of the sweep kernel: per-launch durations from CUDA events around each sweep
    def prof_solve(o):
        ctx.solve3d(src, o, ex.F32, out=out_dev)
        return ctx.stats()
    popts = dict(tolerance=TOL, factored_radius=RADIUS, profile_sweeps=True, pair_fields=PAIR[0], near_fp64=NEAR64[0],
                 sweep_kernel=KERNEL[0], max_in_flight=slots if stream else 0)
    if stream:
        # a stream runs the new fields' initialisation sweeps inside the same launches as the
        # others' refinement sweeps, so the time of all sweep launches is credited with both:
        # the refinement updates performed plus one grid of updates per field for its
        # initialisation pass (its 8 octants cover the grid once)
        pst = prof_solve(ex.Options(n_sweeps=N_SWEEPS_MAX, **popts))
        upd = pst["refine_node_updates"] + fields * n_nodes
        rl = {"achieved": BYTES_PER_NODE_SWEEP * upd / (pst["sweep_ms"] / 1e3) / 1e9,
              "algorithmic_bytes": BYTES_PER_NODE_SWEEP * upd, "node_updates": upd, "refine_ms": pst["sweep_ms"],
              "refine_launches": pst["sweeps_launched"], "launch_ms": pst["sweep_ms"] / max(1, pst["sweeps_launched"])}
    else:
        rl = refinement_roofline(prof_solve, ex.Options(n_sweeps=N_SWEEPS_MAX, **popts),
                                 ex.Options(n_sweeps=0, **popts), BYTES_PER_NODE_SWEEP)
    achieved = rl["achieved"]
    peak, peak_kind = _peaks()
    tr = _traffic()
    shapes = {1: "8x4", 2: "4x8", 3: "16x2"}
    if NEAR64[0]:
        # the FP64 factor runs the chunk-step kernel's table instances, never the pair or
        # node-step kernels
        kernel_name = f"sweep3ChunkNear64Kernel<float,uniform,{shapes.get(tuning['block_shape'] if tuning else 1, '8x4')}>"
    elif tuning:
        kernel_name = ("sweep3PairKernel" if tuning["pair_fields"] else "sweep3Kernel<float,uniform>"
                       if tuning["sweep_kernel"] == 1 else
                       f"sweep3ChunkKernel<float,uniform,{shapes[tuning['block_shape']]}>")
    else:
        kernel_name = ("sweep3PairKernel" if PAIR[0] and fields >= 2 else
                       "sweep3Kernel<float,uniform>" if KERNEL[0] == 1 else "sweep3ChunkKernel<float,uniform,8x4>")
    traffic, traffic_src = None, None
    if tr and tr.get("kernel") == kernel_name.replace(",8x4", ""):
        # DRAM bytes of one full sweep from the committed ncu capture, scaled by the
        # fields per launch (traffic grows in proportion to the fields swept)
        traffic = tr["dram_bytes_per_launch"] * slots / tr["fields"]
        traffic_src = f"profiles/sweep3d_traffic.json ({tr['fields']} fields, scaled to {slots} per launch)"

    # the configuration's own form, one source per solve: bound by one field's wavefront
    # latency rather than by throughput (device-resident, CUDA events, not the headline)
    single = None
    if rank == 0 and not SURFACE[0] and not SLAB[0]:
        one = torch.empty((1, NZ, NY, NX), dtype=torch.float32, device=f"cuda:{dev}")
        for _ in range(3):
            ctx.solve3d(src[:1], opt, ex.F32, out=one)
        t1 = []
        for _ in range(5):
            flush.fill_(1.0)
            ctx.solve3d(src[:1], opt, ex.F32, out=one)
            t1.append(ctx.stats()["device_ms"])
        single = {"grids_s": 1e3 / float(np.mean(t1)), "ms_per_solve": float(np.mean(t1)),
                  "iterations": ctx.stats()["iterations_max"]}


    if rank != 0:
        return
    # the metric's own comparison: the learned warm start against the plain cold start
    # (its training budget is bounded so that the default run ends within minutes)
    learned = None
    if not args.skip_learned and not SURFACE[0] and not SLAB[0]:
        learned = learned_record(args.learn_models, args.learn_steps_default, accuracy=not args.skip_accuracy)
        learned.pop("_conv")
    line = {
        "metric": METRIC, "value": value, "unit": "grids/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered+GRF model, seeded sources)",
        "config": workload_config(fields, world),
        "roofline": {"bound": "hbm", "kernel": kernel_name, "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": rl["algorithmic_bytes"], "node_updates": rl["node_updates"],
                     "refine_ms": rl["refine_ms"], "launch_ms": rl["launch_ms"],
                     "note": ("all sweep launches of the stream, credited with the refinement updates plus one grid "
                              "per field for its initialisation pass; 12 B per node update (read T, read slowness, "
                              "write T)" if stream else
                              "refinement sweeps only; 12 B per node update (read T, read slowness, write T)"),
                     "traffic": traffic, "traffic_source": traffic_src,
                     # the bytes a field's update cannot avoid: read T and write T (the slowness
                     # is one copy shared by all fields through L2)
                     "compulsory_bytes_per_update": 8, "frac_compulsory": achieved * 8 / 12 / peak},
        "e2e": {"value": e2e, "unit": "grids/s", "h2d_bytes_per_step": int(v.nbytes + 24 * fields),
                "d2h_bytes_per_step": int(4 * n_nodes * fields), "ms_per_step": float(np.mean(e2e_ms)),
                "host_out_buffers": n_out, "step_ms": [round(t, 1) for t in e2e_ms], "clocks": clk_e2e.summary()},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "iterations": {"max_over_fields": int(max(i[1] for i in iters)),
                       "min_over_fields": int(min(i[0] for i in iters))},
        "single_source": single,
        "wall_ms_per_step": float(np.mean(wall)), "accuracy": acc, "tuning": tuning,
        "learned": learned,
        "cpu_baseline": cpu_baseline(args.cpu_seconds, 1) if not args.skip_cpu else None,
    }
    print(json.dumps(line), flush=True)


def run_models(args):
    """Many models of uneven size in one schedule: `fields` layered+GRF models with nx, ny
    uniform in [64, 256], nz in [32, 128], h = 100 m, one seeded source each."""
    import torch
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import sharding, synthetic

    world, rank = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.cuda.current_device()
    n = args.fields
    everything = synthetic.uneven_models(n * world, MODEL_SEED + 1)
    # models of uneven size: split by estimated cost (nodes x sweeps), not by count
    costs = [sharding.field_cost(*m["grid"][:3], sweeps=8 * (1 + N_SWEEPS_MAX)) for m in everything]
    mine = [everything[i] for i in sharding.shard_by_cost(costs, world, rank)]
    nodes = sum(m["grid"][0] * m["grid"][1] * m["grid"][2] for m in mine)
    ctx = ex.Context(dev)
    dev_models = [{"grid": m["grid"], "model": torch.from_numpy(m["v"]).to(f"cuda:{dev}"), "nodal": True,
                   "sources": [m["source"]],
                   "out": torch.empty((1,) + m["v"].shape, dtype=torch.float32, device=f"cuda:{dev}")} for m in mine]
    host_models = [{"grid": m["grid"], "model": torch.from_numpy(m["v"]).pin_memory(), "nodal": True,
                    "sources": [m["source"]],
                    "out": torch.empty((1,) + m["v"].shape, dtype=torch.float32).pin_memory()} for m in mine]
    opt = ex.Options(n_sweeps=N_SWEEPS_MAX, tolerance=TOL, factored_radius=RADIUS, near_fp64=NEAR64[0])
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")

    acc = {}
    if rank == 0 and not args.skip_accuracy:
        t32 = ctx.solve3d_batch(dev_models, opt, ex.F32)
        t32 = [t.cpu().numpy().astype(np.float64) for t in t32]
        o64 = ex.Options(n_sweeps=FP64_MAX_ITERATIONS, tolerance=FP64_TOL, factored_radius=RADIUS)
        t64 = ctx.solve3d_batch([dict(m, out=None) for m in dev_models], o64, ex.F64)
        it64 = ctx.stats()["iterations_max"]
        per = [float(np.abs(a - b).max()) for a, b in zip(t32, t64)]
        d = np.concatenate([np.abs(a - b).ravel() for a, b in zip(t32, t64)])
        acc = {"max_err_vs_fp64_s": float(d.max()), "rms_err_vs_fp64_s": float(np.sqrt(np.mean(d ** 2))),
               "meets_1e-4": bool(d.max() <= 1e-4), "models_over_1e-4": int(sum(e > 1e-4 for e in per)),
               "fp64_iterations_max": it64, "fp64_converged": bool(it64 < FP64_MAX_ITERATIONS)}
        # the precision that meets the bound: FP64 sweeps at the workload's tolerance and cap
        o_arm = ex.Options(n_sweeps=N_SWEEPS_MAX, tolerance=TOL, factored_radius=RADIUS)
        m64 = [dict(m, out=torch.empty((1,) + tuple(m["out"].shape[1:]), dtype=torch.float64, device=f"cuda:{dev}"))
               for m in dev_models]
        ms64 = []
        for i in range(3):
            ctx.solve3d_batch(m64, o_arm, ex.F64)
            if i:
                ms64.append(ctx.stats()["device_ms"])
        e64 = max(float(np.abs(m["out"][0].cpu().numpy() - b).max()) for m, b in zip(m64, t64))
        del m64
        acc["fp64_sweeps"] = {"grids_s": n / (float(np.mean(ms64)) / 1e3), "fields_timed": n,
                              "max_err_vs_fp64_converged_s": e64, "meets_1e-4": bool(e64 <= 1e-4),
                              "tolerance_s": TOL}

    for _ in range(args.warmup):
        ctx.solve3d_batch(dev_models, opt, ex.F32)
    torch.cuda.synchronize()
    sharding.barrier()
    per_step, iters, launches = [], [], 0
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ctx.solve3d_batch(dev_models, opt, ex.F32)
            st = ctx.stats()
            per_step.append(st["device_ms"])
            iters.append((st["iterations_min"], st["iterations_max"]))
            launches += st["kernel_launches"]
    torch.cuda.synchronize()
    sharding.barrier()
    ms = sharding.max_over_ranks(float(np.mean(per_step)), device=f"cuda:{dev}")
    value = n * world / (ms / 1e3)

    def prof_solve(o):
        ctx.solve3d_batch(dev_models, o, ex.F32)
        return ctx.stats()
    rl = refinement_roofline(prof_solve,
                             ex.Options(n_sweeps=N_SWEEPS_MAX, tolerance=TOL, factored_radius=RADIUS, profile_sweeps=True,
                                        near_fp64=NEAR64[0]),
                             ex.Options(n_sweeps=0, tolerance=TOL, factored_radius=RADIUS, profile_sweeps=True),
                             BYTES_PER_NODE_SWEEP)
    achieved = rl["achieved"]
    peak, peak_kind = _peaks()

    e2e_ms = []
    for i in range(max(1, args.warmup) + args.steps):
        t0 = time.perf_counter()
        ctx.solve3d_batch(host_models, opt, ex.F32)
        if i >= max(1, args.warmup):
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = n * world / (float(np.mean(e2e_ms)) / 1e3)
    if rank != 0:
        return
    grids = [m["grid"][:3] for m in mine]
    line = {
        "metric": METRIC, "value": value, "unit": "grids/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered+GRF models, seeded sources)",
        "config": {"workload": f"{n} models of uneven size (nx, ny in [64, 256], nz in [32, 128], h=100 m) "
                               f"per step per GPU, one source each, one schedule",
                   "nodes_per_step": nodes, "grids_min": min(grids), "grids_max": max(grids),
                   "precision": ("fp32 sweeps; fp64 source init and factored (near-source) branch" if NEAR64[0]
                                 else "fp32 sweeps, fp64 source init"), "factored_radius": RADIUS, "tolerance_s": TOL,
                   "max_iterations": N_SWEEPS_MAX, "l2": "flushed (write of 2x L2) between timed steps",
                   "parallelism": f"replicas x{world} (models split by estimated cost, no collective)"},
        "roofline": {"bound": "hbm", "kernel": ("sweep3ChunkNear64Kernel<float,uniform,batch>" if NEAR64[0] else
                                                "sweep3ChunkKernel<float,uniform,batch>"), "achieved": achieved,
                     "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes": rl["algorithmic_bytes"], "node_updates": rl["node_updates"],
                     "refine_ms": rl["refine_ms"], "launch_ms": rl["launch_ms"], "traffic": None,
                     "note": "refinement sweeps only; 12 B per node update",
                     "compulsory_bytes_per_update": 8, "frac_compulsory": achieved * 8 / 12 / peak},
        "e2e": {"value": e2e, "unit": "grids/s", "h2d_bytes_per_step": int(sum(m["v"].nbytes for m in mine)),
                "d2h_bytes_per_step": int(4 * nodes), "ms_per_step": float(np.mean(e2e_ms))},
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "iterations": {"max_over_fields": int(max(i[1] for i in iters)),
                       "min_over_fields": int(min(i[0] for i in iters))}, "accuracy": acc,
    }
    print(json.dumps(line), flush=True)


def run_2d(args):
    """The reference's plain 2D configuration: FP64, 501 x 251 nodes, dx = dz = 10 m,
    v(z) = 3000 m/s + 0.5 s^-1 z, source at (2500 m, 500 m), factored radius 3, 2 sweep
    iterations, tolerance 1e-8 s.  Errors against the analytic linear-gradient times and
    the CPU oracle (the reference's 2D fast sweeping restated, bit-identical to it)."""
    import torch
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import synthetic
    from oracle import Oracle

    nx, nz, h = 501, 251, 10.0
    src = (2500.0, 500.0)
    v = synthetic.linear_gradient_2d(nx, nz, h, 3000.0, 0.5)
    dev = torch.cuda.current_device()
    ctx = ex.Context(dev)
    ctx.set_grid2d(nx, nz, h, h)
    ctx.set_nodal_velocity2d(v)
    opt = ex.Options(n_sweeps=2, tolerance=1e-8, factored_radius=3, sweep_kernel=KERNEL[0])
    fields = args.fields
    srcs = [src] * fields
    out_dev = torch.empty((fields, nz, nx), dtype=torch.float64, device=f"cuda:{dev}")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    t = ctx.solve2d([src], opt, ex.F64)[0]
    ta = ctx.analytic2d(src, 3000.0, 3000.0 + 0.5 * (nz - 1) * h)
    orc = Oracle()
    s_cells = orc.nodal_to_cell2d(v.ravel(), nx, nz, 0)
    cell = (min(nx - 2, int(src[0] / h)), min(nz - 2, int(src[1] / h)))
    t0 = time.perf_counter()
    t_or = orc.solve2d(s_cells, (nx, nz, h, h), cell, src, n_sweeps=2, radius=3, tol=1e-8)
    cpu_s = time.perf_counter() - t0
    e = np.abs(t - ta)
    acc = {"max_err_vs_analytic_s": float(e.max()), "rms_err_vs_analytic_s": float(np.sqrt(np.mean(e ** 2))),
           "max_abs_diff_vs_oracle_s": float(np.abs(t - t_or).max()),
           "bit_identical_to_oracle": bool(np.array_equal(t.view(np.uint64), t_or.view(np.uint64)))}

    for _ in range(args.warmup):
        ctx.solve2d(srcs, opt, ex.F64, out=out_dev)
    torch.cuda.synchronize()
    per, launches, iters = [], 0, []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            ctx.solve2d(srcs, opt, ex.F64, out=out_dev)
            st = ctx.stats()
            per.append(st["device_ms"])
            launches += st["kernel_launches"]
            iters.append((st["iterations_min"], st["iterations_max"]))
    ms = float(np.mean(per))
    def prof_solve(o):
        ctx.solve2d(srcs, o, ex.F64, out=out_dev)
        return ctx.stats()
    popts = dict(tolerance=1e-8, factored_radius=3, profile_sweeps=True, sweep_kernel=KERNEL[0])
    rl = refinement_roofline(prof_solve, ex.Options(n_sweeps=2, **popts), ex.Options(n_sweeps=0, **popts), 24)
    peak, peak_kind = _peaks()
    e2e_ms = []
    out_host = torch.empty((fields, nz, nx), dtype=torch.float64).pin_memory()
    v_host = torch.from_numpy(v).pin_memory()
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        ctx.set_nodal_velocity2d(v_host)
        ctx.solve2d(srcs, opt, ex.F64, out=out_host)
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    line = {
        "metric": "2D travel-time grids/s (FP64) at the reference's plain 2D configuration", "value": fields / (ms / 1e3),
        "unit": "grids/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic linear-gradient model)",
        "config": {"workload": f"plain 2D solve, {nx}x{nz} h={h:g} m, v(z)=3000+0.5z m/s, source (2500, 500) m, "
                               f"{fields} field(s) per step", "factored_radius": 3, "n_sweeps": 2, "tolerance_s": 1e-8,
                   "l2": "flushed (write of 2x L2) between timed steps"},
        "roofline": {"bound": "hbm", "kernel": ("sweep2BlockKernel<double,uniform>" if KERNEL[0] == 2 and nz <= 512
                                                else "sweep2Kernel<double,uniform>"),
                     "achieved": rl["achieved"], "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": rl["achieved"] / peak, "algorithmic_bytes": rl["algorithmic_bytes"],
                     "node_updates": rl["node_updates"], "refine_ms": rl["refine_ms"], "launch_ms": rl["launch_ms"],
                     "traffic": None, "note": "one field of 126 k nodes: latency-bound wavefront (751 levels)"},
        "e2e": {"value": fields / (float(np.mean(e2e_ms)) / 1e3), "unit": "grids/s", "h2d_bytes_per_step": int(v.nbytes),
                "d2h_bytes_per_step": int(8 * nx * nz * fields), "ms_per_step": float(np.mean(e2e_ms))},
        "gpu_launches": int(launches), "clocks": clk.summary(), "iterations": {"max_over_fields": int(max(i[1] for i in iters)),
                                                                       "min_over_fields": int(min(i[0] for i in iters))},
        "accuracy": acc,
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "grids/s", "cores": 1, "kind": "port",
                         "sample": "one full FP64 solve of the configuration by the CPU oracle"},
    }
    print(json.dumps(line), flush=True)


def run_warmstart_study(args):
    """Does a warm start save sweeps on this discretization?  Cold-start solves of the
    plain workload, then warm starts (eikx_solve3d_warm) from the best predictions any
    predictor could make: the cold-start result itself (exactly and inflated), and its
    factor tau = T / T0 sampled every F nodes and upsampled, inflated.  Reports refinement
    iterations, device time and the deviation from the cold-start fields, for factored
    radius 3 (the reference default) and 0."""
    import torch
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import synthetic
    from scipy.ndimage import zoom

    v, src = make_workload(args.fields)
    ctx = ex.Context(torch.cuda.current_device())
    ctx.set_grid3d(NX, NY, NZ, H, H, H)
    ctx.set_nodal_velocity3d(v.ravel())
    cells = np.empty((NZ - 1) * (NY - 1) * (NX - 1), np.float64)
    _check = ex._check
    _check(ctx._lib.eikx_get_slowness3d(ctx._h, cells.ctypes.data, ex.F64))
    cells = cells.reshape(NZ - 1, NY - 1, NX - 1)
    z, y, x = np.meshgrid(np.arange(NZ) * H, np.arange(NY) * H, np.arange(NX) * H, indexing="ij", sparse=True)
    T0 = []
    for p in src:
        c = [min(n - 2, int(q / H)) for q, n in zip(p, (NX, NY, NZ))]
        T0.append(np.sqrt((x - p[0]) ** 2 + (y - p[1]) ** 2 + (z - p[2]) ** 2) * cells[c[2], c[1], c[0]])
    T0 = np.stack(T0)
    rows = []
    for radius in (RADIUS, 0):
        opt = ex.Options(n_sweeps=20, tolerance=TOL, factored_radius=radius)
        cold = ctx.solve3d(src, opt, ex.F32)
        cst = ctx.stats()
        rows.append({"radius": radius, "start": "cold", "iterations": cst["iterations_max"],
                     "device_ms": cst["device_ms"]})
        tau = np.where(T0 > 0, cold / np.maximum(T0, 1e-12), 1.0)
        starts = {"cold result x1.0": cold, "cold result x1.001": cold * 1.001}
        for F in (2, 4):
            tc = tau[:, ::F, ::F, ::F]
            up = np.stack([zoom(t, (NZ / t.shape[0], NY / t.shape[1], NX / t.shape[2]), order=1) for t in tc])
            starts[f"tau every {F} nodes, x1.01"] = T0 * up * 1.01
        for name, init in starts.items():
            out = ctx.solve3d_warm(src, np.ascontiguousarray(init, dtype=np.float32), opt, ex.F32,
                                   gate_tol=1e9 if name.startswith("cold") else 1e-6)
            st = ctx.stats()
            d = out.astype(np.float64) - cold
            rows.append({"radius": radius, "start": name, "iterations": st["iterations_max"],
                         "device_ms": st["device_ms"], "reset_nodes": st["reset_nodes"],
                         "max_below_cold_s": float(-d.min()), "max_above_cold_s": float(d.max()),
                         "nodes_off_by_more_than_1e-4": int((np.abs(d) > 1e-4).sum())})
    print(json.dumps({"study": "warm start on the plain workload", "fields": args.fields,
                      "grid": [NX, NY, NZ], "rows": rows}), flush=True)


LEARN_GRID = (128, 128, 64, 50.0)
PREDICT_LAUNCHES = 22   # features, 14 convolutions, 3 poolings, 3 up-and-concats, the head


def learned_record(train_models, learn_steps, warmup=1, accuracy=True, per_model=8, test_models=4):
    """The learned warm start against the plain cold start on 128x128x64 nodes, h = 50 m.

    Training data: `train_models` random smooth models (Gaussian random fields, 1500-8000
    m/s, correlation length 0.5-3 km) with `per_model` seeded sources each, solved cold by
    the library; the network is trained on them by its own kernels (Adam, batch 8,
    `learn_steps` steps).  Evaluation on `test_models` held-out models: cold-start solves
    against warm starts from the network's prediction (prediction time included), with the
    one-sided residual gate (prediction x 1.02), the two-sided gate (prediction x 1.0 and
    x 1.02), and from T0 alone (the untrained network, x 1.02).  Errors are against FP64
    solves of the same sources run to convergence."""
    import torch
    import eikonalxx_gb300 as ex
    from eikonalxx_gb300 import warmstart as ws

    nx, ny, nz, h = LEARN_GRID
    grid = (nx, ny, nz, h, h, h)
    dev = torch.cuda.current_device()
    batch = 8
    ctx = ex.Context(dev)
    opt = ex.Options(n_sweeps=20, tolerance=TOL, factored_radius=RADIUS, near_fp64=NEAR64[0])
    t = time.perf_counter()
    data = ws.generate_fields(ctx, grid, train_models + test_models, per_model, seed=MODEL_SEED + 4, options=opt)
    gen_s = time.perf_counter() - t
    n_train = train_models * per_model
    train_idx = np.arange(n_train)
    test_idx = np.arange(n_train, n_train + test_models * per_model)
    net = ws.WarmNet(grid, batch=batch, seed=MODEL_SEED)
    p0 = net.get_params()
    net.set_params(np.zeros_like(p0))
    base_loss = ws.evaluate_loss(net, data, test_idx)
    net.set_params(p0)
    t = time.perf_counter()
    losses = ws.train(net, data, steps=learn_steps, lr=1e-3, seed=MODEL_SEED + 5, fields=train_idx)
    train_s = time.perf_counter() - t
    test_loss = ws.evaluate_loss(net, data, test_idx)
    p_trained = net.get_params()
    prof = net.profile_step(ws.samples_of(data, train_idx[:batch]), 0.0)   # lr 0: parameters unchanged
    net.set_params(p_trained)

    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    variants = {"network x1.02, one-sided gate": (p_trained, 1.02, 0),
                "network x1.0, two-sided gate": (p_trained, 1.0, 1),
                "network x1.02, two-sided gate": (p_trained, 1.02, 1),
                "T0 x1.02 (untrained), one-sided gate": (np.zeros_like(p_trained), 1.02, 0)}
    rows = {"cold": []}
    rows.update({k: [] for k in variants})
    dev_cold = torch.empty((per_model, nz, ny, nx), dtype=torch.float32, device=f"cuda:{dev}")
    dev_warm = torch.empty_like(dev_cold)
    init = torch.empty_like(dev_cold)
    launches = 0
    o64 = ex.Options(n_sweeps=FP64_MAX_ITERATIONS, tolerance=FP64_TOL, factored_radius=RADIUS)
    fp64_iters = 0
    for k in range(test_models):
        idx = test_idx[k * per_model:(k + 1) * per_model]
        m = int(data["model"][idx[0]])
        ctx.set_grid3d(nx, ny, nz, h, h, h)
        ctx.set_nodal_velocity3d(data["velocity"][m])
        src = data["sources"][idx]
        t64 = None
        if accuracy:
            t64 = ctx.solve3d(src, o64, ex.F64)
            fp64_iters = max(fp64_iters, ctx.stats()["iterations_max"])
        for _ in range(warmup):
            ctx.solve3d(src, opt, ex.F32, out=dev_cold)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ctx.solve3d(src, opt, ex.F32, out=dev_cold)
        st = ctx.stats()
        launches += st["kernel_launches"]
        cold = dev_cold.cpu().numpy().astype(np.float64)
        row = {"ms": st["device_ms"], "iterations": st["iterations_max"]}
        if t64 is not None:
            row["max_err_fp64_s"] = float(np.max(np.abs(cold - t64)))
        rows["cold"].append(row)
        for name, (params, inflate, gate) in variants.items():
            net.set_params(params)
            wopt = ex.Options(n_sweeps=20, tolerance=TOL, factored_radius=RADIUS, warm_gate=gate,
                              near_fp64=NEAR64[0])
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t = time.perf_counter()
            net.predict(ws.samples_of(data, idx, with_target=False), inflate=inflate, out=init)
            torch.cuda.synchronize()
            pred_ms = (time.perf_counter() - t) * 1e3
            ctx.solve3d_warm(src, init, wopt, ex.F32, gate_tol=1e-6, out=dev_warm)
            st = ctx.stats()
            launches += st["kernel_launches"] + PREDICT_LAUNCHES
            warm = dev_warm.cpu().numpy().astype(np.float64)
            d = warm - cold
            row = {"ms": st["device_ms"] + pred_ms, "predict_ms": pred_ms, "iterations": st["iterations_max"],
                   "reset_nodes": st["reset_nodes"], "max_dev_s": float(np.max(np.abs(d))),
                   "rms_dev_s": float(np.sqrt(np.mean(d * d)))}
            if t64 is not None:
                row["max_err_fp64_s"] = float(np.max(np.abs(warm - t64)))
            rows[name].append(row)
    net.set_params(p_trained)
    fields = test_models * per_model

    def rate(r):
        return fields / (sum(x["ms"] for x in r) / 1e3)

    def summary(r):
        out = {"grids_per_s": rate(r), "ms_per_field": sum(x["ms"] for x in r) / fields,
               "iterations_max": max(x["iterations"] for x in r)}
        if "max_err_fp64_s" in r[0]:
            out["max_err_vs_fp64_s"] = max(x["max_err_fp64_s"] for x in r)
            out["meets_1e-4"] = bool(out["max_err_vs_fp64_s"] <= 1e-4)
        if "max_dev_s" in r[0]:
            out.update({"max_dev_from_cold_s": max(x["max_dev_s"] for x in r),
                        "rms_dev_from_cold_s": float(np.sqrt(np.mean([x["rms_dev_s"] ** 2 for x in r]))),
                        "predict_ms_per_field": sum(x["predict_ms"] for x in r) / fields,
                        "reset_nodes": int(sum(x["reset_nodes"] for x in r))})
        return out

    cold_rate = rate(rows["cold"])
    var = {k: dict(summary(rows[k]), speedup_vs_cold=rate(rows[k]) / cold_rate) for k in variants}
    ok = [v["speedup_vs_cold"] for v in var.values() if v.get("meets_1e-4")]
    conv_ms = sum(prof["ms"][k] for k in ("forward_conv", "input_grad_conv", "weight_grad"))
    conv_fl = sum(prof["flops"].values())
    return {
        "workload": f"learned warm start, {nx}x{ny}x{nz} h={h:g} m: {train_models} training models x {per_model} "
                    f"sources ({n_train} solver-generated fields), {learn_steps} Adam steps of batch {batch}; "
                    f"{test_models} held-out models x {per_model} sources, warm starts vs cold starts",
        "cold": summary(rows["cold"]), "variants": var,
        "learned_vs_plain": var["network x1.02, one-sided gate"]["speedup_vs_cold"],
        "best_speedup_meeting_1e-4": max(ok) if ok else None,
        "fp64_iterations_max": fp64_iters if accuracy else None,
        "test_loss": test_loss, "tau_1_loss": base_loss,
        "train_loss_first_last": [float(np.mean(losses[:20])), float(np.mean(losses[-20:]))],
        "generate_s": gen_s, "train_s": train_s, "train_steps_per_s": learn_steps / train_s,
        "conv_tflops": conv_fl / (conv_ms / 1e3) / 1e12, "step_profile": prof, "gpu_launches": int(launches),
        "_conv": (conv_fl, conv_ms),
    }


def run_learned(args):
    """The learned workload's own line: value = the cold-start grids/s of the held-out
    fields (the path that meets the error bound); the learned variants under "learned";
    the roofline is the network's convolutions (tensor-bound) over one training step."""
    import torch

    dev = torch.cuda.current_device()
    with ClockSampler(dev) as clk:
        rec = learned_record(args.fields, args.learn_steps, warmup=args.warmup, accuracy=not args.skip_accuracy)
    conv_fl, conv_ms = rec.pop("_conv")
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            tpeak, tkind = float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        tpeak, tkind = 1900.0, "fallback"
    achieved = conv_fl / (conv_ms / 1e3) / 1e12
    cold_rate = rec["cold"]["grids_per_s"]
    nx, ny, nz, h = LEARN_GRID
    line = {
        "metric": METRIC, "value": cold_rate, "unit": "grids/s", "n_gpus": 1, "steps": 1,
        "warmup": args.warmup, "ms_per_step": rec["cold"]["ms_per_field"] * 32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 sweeps, bf16 network",
        "data": "synthetic (seeded random smooth models, seeded sources; fields solved by the library)",
        "config": {"workload": rec["workload"], "precision": "fp32 sweeps, fp64 init; network bf16 with fp32 "
                                                            "accumulation", "factored_radius": RADIUS,
                   "tolerance_s": TOL, "gate_tol_s": 1e-6, "l2": "flushed (write of 2x L2) before each timed solve"},
        "learned": rec,
        "roofline": {"bound": "tensor", "kernel": "convTcKernel + convKernel + wgradKernel (BF16, FP32 accumulate)",
                     "achieved": achieved, "peak": tpeak, "peak_kind": tkind, "unit": "TFLOP/s",
                     "frac": achieved / tpeak, "traffic": None,
                     "note": "one training step of batch 8; algorithmic FLOPs 2 x nodes x 27 x in x out per "
                             "convolution, forward, input-gradient and weight-gradient passes"},
        "gpu_launches": rec["gpu_launches"], "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def profile_learned_case(batch=4):
    """One training step of the learned warm start's network on 128x128x64 nodes (for ncu
    captures): synthetic samples, no solver; about 3 GB on the device at batch 4."""
    import torch
    from eikonalxx_gb300 import warmstart as ws

    nx, ny, nz, h = LEARN_GRID
    net = ws.WarmNet((nx, ny, nz, h, h, h), batch=batch, seed=MODEL_SEED)
    rng = np.random.default_rng(MODEL_SEED)
    z, y, x = np.meshgrid(np.arange(nz) * h, np.arange(ny) * h, np.arange(nx) * h, indexing="ij")
    samples = []
    for _ in range(batch):
        v = rng.uniform(2000, 6000)
        src = rng.uniform(0, 1, 3) * np.array([(nx - 1) * h, (ny - 1) * h, (nz - 1) * h])
        d = np.sqrt((x - src[0]) ** 2 + (y - src[1]) ** 2 + (z - src[2]) ** 2)
        vel = torch.full((nx * ny * nz,), v, dtype=torch.float32, device="cuda")
        tt = torch.from_numpy((d / v * (1 + 0.05 * np.sin(x / 700.0))).astype(np.float32).ravel()).cuda()
        samples.append((vel, tt, tuple(src)))
    net.train_step(samples, 1e-4)
    torch.cuda.synchronize()


def profile_case(fields, fp64=False):
    """The workload's grid and model, `fields` sources, one refinement iteration, without
    the CUDA graph: 8 source-limited sweeps then 8 full sweeps (launches 9-16).  With
    --in-flight below `fields`: the stream of those sources to the bench's tolerance.  fp64:
    FP64 sweeps (the reference's own precision) instead of FP32 with the FP64 factor."""
    import torch
    import eikonalxx_gb300 as ex
    v, src = make_workload(fields)
    ctx = ex.Context(torch.cuda.current_device())
    ctx.set_grid3d(NX, NY, NZ, H, H, H)
    ctx.set_nodal_velocity3d(v.ravel())
    stream = 0 < IN_FLIGHT[0] < fields
    # a stream: the bench's tolerance, so that slots refill; else one refinement iteration
    opt = ex.Options(n_sweeps=N_SWEEPS_MAX if stream else 1, tolerance=TOL if stream else -1, factored_radius=RADIUS,
                     profile_sweeps=True, pair_fields=PAIR[0], sweep_kernel=KERNEL[0],
                     near_fp64=NEAR64[0] and not fp64, max_in_flight=IN_FLIGHT[0] if stream else 0)
    out = torch.empty((fields, NZ, NY, NX), dtype=torch.float64 if fp64 else torch.float32, device="cuda")
    ctx.solve3d(src, opt, ex.F64 if fp64 else ex.F32, out=out)
    st = ctx.stats()
    print(json.dumps({"profile_case": True, "fields": fields, "sweep_ms_mean": st["sweep_ms"] / st["sweeps_launched"],
                      "device_ms": st["device_ms"]}))


class CpuColdSolves:
    """Real cold-start FP32 solves of the workload on host threads, for the CPU baselines.

    Each thread solves the workload's seeded sources one after another with the oracle
    (the project's CPU restatement, pinned bit for bit to the reference's sweep code):
    FP64 corner initialisation, the 8 source-limited initialisation sweeps, then
    refinement sweeps until the convergence rule (tolerance 1e-5 s, at most
    N_SWEEPS_MAX iterations), exactly as the GPU solves them.  A step advances every
    thread by `per_step` sweeps of its solves (a thread whose field converges starts the
    next source within the step).  Work is credited per field as the fraction of that
    field's sweeps run inside the timed steps; fields left unfinished are run to their end
    untimed, so every credit divides by a field's real sweep count."""

    def __init__(self, threads, per_step=8):
        from oracle import ColdSolve3, Oracle
        self._cls = ColdSolve3
        self.orc = Oracle()
        self.threads = max(1, threads)
        self.per_step = per_step
        v, src = make_workload(64 * self.threads)
        self.src = src
        self.slow = self.orc.nodal_to_cell3d(v.ravel(), NX, NY, NZ, 0)   # FP32, as the GPU forms it
        self.orc.lib.oracle_set_near_fp64(int(NEAR64[0]))                 # the GPU arm's precision
        self.next_src = list(range(self.threads))    # thread t takes sources t, t + T, t + 2T, ...
        self.cur = [self._start(t) for t in range(self.threads)]
        self.timed = {}          # source index -> sweeps run inside timed steps
        self.total = {}          # source index -> sweeps its solve took
        self.step_s = []

    def _start(self, t):
        i = self.next_src[t]
        self.next_src[t] += self.threads
        return i, self._cls(self.orc, self.slow, (NX, NY, NZ, H, H, H), self.src[i % len(self.src)],
                            N_SWEEPS_MAX, RADIUS, TOL)

    def _advance(self, t, timed):
        left = self.per_step
        while left > 0:
            i, cs = self.cur[t]
            before = cs.sweeps
            done = cs.advance(left)
            ran = cs.sweeps - before
            left -= ran
            if timed:
                self.timed[i] = self.timed.get(i, 0) + ran
            if done:
                self.total[i] = cs.sweeps
                self.cur[t] = self._start(t)

    def step(self, timed):
        t0 = time.perf_counter()
        th = [threading.Thread(target=self._advance, args=(t, timed)) for t in range(self.threads)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        dt = time.perf_counter() - t0
        if timed:
            self.step_s.append(dt)
        return dt

    def finish(self):
        """Run the fields the timed steps left unfinished to their end (untimed) and
        return (grids credited, timed seconds, mean sweeps per completed grid, grids)."""
        def run(t):
            i, cs = self.cur[t]
            if i in self.timed:
                while not cs.advance(64):
                    pass
                self.total[i] = cs.sweeps
        th = [threading.Thread(target=run, args=(t,)) for t in range(self.threads)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        credit = sum(n / self.total[i] for i, n in self.timed.items())
        spg = float(np.mean([self.total[i] for i in self.timed]))
        return credit, float(sum(self.step_s)), spg, len(self.timed)


def cpu_baseline(seconds, threads=1):
    """The GPU arm's CPU baseline: one host thread solving the workload's fields for about
    `seconds` (steps of 8 sweeps), credited per field."""
    arm = CpuColdSolves(threads)
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        arm.step(True)
    credit, secs, spg, n = arm.finish()
    return {"value": credit / secs, "unit": "grids/s", "cores": threads, "kind": "port",
            "sample": f"{secs:.1f} s of real cold-start FP32 solves of the workload on {threads} host thread(s): "
                      f"{n} field(s), {sum(arm.timed.values())} sweeps timed, credited per field as the fraction of "
                      f"its sweeps run ({spg:.1f} sweeps per grid on average, convergence rule as on the GPU)",
            "sweeps_per_grid": spg, "fields": n}


def run_reference(args):
    world, rank = _dist()
    if rank != 0:
        return
    threads = args.cpu_threads or (os.cpu_count() or 1)
    arm = CpuColdSolves(threads)
    for _ in range(args.warmup):
        arm.step(False)
    for _ in range(args.steps):
        arm.step(True)
    credit, secs, spg, n = arm.finish()
    value = credit / secs
    line = {
        "metric": METRIC, "value": value, "unit": "grids/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered+GRF model, seeded sources)", "impl": "reference",
        "config": workload_config(args.fields, world),
        "cpu_baseline": {"value": value, "unit": "grids/s", "cores": threads, "kind": "port",
                         "sample": f"each step: every one of {threads} host threads advances its real cold-start FP32 "
                                   f"solve of the workload by {arm.per_step} sweeps (the oracle, bit-identical to the "
                                   f"reference's sweep code); {n} fields, {sum(arm.timed.values())} sweeps timed, "
                                   f"credited per field as the fraction of its sweeps run",
                         "sweeps_per_grid": spg, "fields": n},
        "e2e": {"value": value, "unit": "grids/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "stations", "models", "full", "2d", "warmstart", "learned"],
                    help="plain: 256x256x128 h=50 m, independent sources; stations: 200x200x100 h=100 m, "
                         "sources on the top surface; models: uneven models, one source each; full: "
                         "512x512x256 h=25 m with a dipping slab, surface sources; 2d: 501x251 FP64; "
                         "learned: the learned warm start, 128x128x64 h=50 m (training included)")
    ap.add_argument("--fields", type=int, default=None,
                    help="sources (plain: 64, stations: 64, full: 256) or models (models: 32) per step per GPU")
    ap.add_argument("--learn-steps", type=int, default=2000, help="learned: training steps")
    ap.add_argument("--learn-models", type=int, default=256,
                    help="plain: training models of the learned sub-record (8 fields each)")
    ap.add_argument("--learn-steps-default", type=int, default=1500,
                    help="plain: training steps of the learned sub-record")
    ap.add_argument("--skip-learned", action="store_true", help="plain: leave out the learned sub-record")
    ap.add_argument("--in-flight", type=int, default=None,
                    help="plain: fields in flight of the step's stream of sources (0 = one batch of all of them)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--sweep-kernel", type=int, default=0, choices=[0, 1, 2],
                    help="3D sweep kernel: 0 default (chunk-step), 1 node-step, 2 chunk-step")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip eikx_autotune3d before timing (default chunk-step 8x4 configuration)")
    ap.add_argument("--fp32-near", action="store_true",
                    help="3D: factored (near-source) updates in FP32 too, instead of FP64")
    ap.add_argument("--pair-fields", action="store_true",
                    help="sweep two fields per lane (the paired FP32 kernel) instead of one")
    ap.add_argument("--profile-case", action="store_true",
                    help="one solve of the workload (1 refinement iteration) for ncu captures")
    ap.add_argument("--profile-fp64", action="store_true",
                    help="with --profile-case: FP64 sweeps instead of FP32")
    args = ap.parse_args()
    global NX, NY, NZ, H
    if args.workload == "stations":
        NX, NY, NZ, H = 200, 200, 100, 100.0
        SURFACE[0] = True
    global N_SWEEPS_MAX
    if args.workload == "full":
        NX, NY, NZ, H = 512, 512, 256, 25.0
        SURFACE[0] = True
        SLAB[0] = True
        N_SWEEPS_MAX = 20      # the slab model converges more slowly than 10 iterations
    if args.in_flight is None:
        # plain: a stream of sources with 256 fields in flight.  A sweep launch costs a fixed
        # wavefront fill and drain (about 0.33 ms) plus about 0.047 ms per field, so more
        # fields per launch amortise it; and a stream refills the slots of fields that
        # converged, so no launch runs with a few slow fields only (64, 128, 256 slots:
        # 429, 457, 482 grids/s on the bench model)
        args.in_flight = 256 if args.workload == "plain" and not args.profile_case else 0
    if args.fields is None:
        # plain: 4 sources per slot of the stream; 64 as one batch without one
        # learned: 2,500 training models x 8 sources = the configuration's 20,000 fields
        args.fields = {"stations": 64, "full": 256, "2d": 1, "warmstart": 8, "models": 32,
                       "learned": 2500}.get(args.workload, 64)
        if args.workload == "plain" and args.in_flight > 0:
            args.fields = 4 * args.in_flight
    IN_FLIGHT[0] = args.in_flight
    PAIR[0] = args.pair_fields
    NEAR64[0] = not args.fp32_near
    KERNEL[0] = args.sweep_kernel
    if args.profile_case:
        if args.workload == "learned":
            profile_learned_case()
        else:
            profile_case(args.fields, fp64=args.profile_fp64)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "models":
        run_models(args)
    elif args.workload == "2d":
        run_2d(args)
    elif args.workload == "warmstart":
        run_warmstart_study(args)
    elif args.workload == "learned":
        run_learned(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
