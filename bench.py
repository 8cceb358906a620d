"""Benchmark of the WCSPH time step: particle-steps/s on one GB300.

Workload (default): the 2D natural-convection cavity, 256 x 256 = 65,536
ThermalLiquidParticle + 3,108 wall particles, WendlandC2, FluidCompulsiveThermostatic-
WallSolve, density re-initialisation every 30 steps.  A "step" is one eachStep! of
that scene.  Under torchrun each rank steps its own replica of the scene (the scene
does not shard; replicas are independent), so `value` is the sum over ranks.

  python bench.py [--gpus N --steps K --warmup W --precision fp64|fp32c --impl ours|reference]

Timing: W untimed warm-up steps, then K steps, each bracketed by CUDA events on the
handle's stream with an L2 flush (a 512 MB write) before every step outside the
events (the scene's state, ~9 MB, would otherwise sit in the 129 MB L2).  The step
numbers of the timed window are chosen so that it ends on a density re-initialisation
step: it holds ceil(K / 30) of them (every 30th step, as a long run does, or more for
K < 30), so the timed steps carry their share of the Shepard work.  `e2e` times the
C-ABI path a Julia caller uses: upload from host arrays, 100 steps (one output
interval), download of the full state to host arrays; for both forms.
`--impl reference` times the CPU restatement of the reference's algorithm (half pair
list with atomic scatter, OpenMP over all host cores) on the same scene.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s"
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
LANES_LIST = 16  # SPH_LANES_LIST: momentum lanes codes >= 15 read the neighbour list
# Counters of one launch of each gather on the default workload (n=256, FP32-compensated)
# from ncu --set full --clock-control none (cold L2, as the bench's flushed steps), per
# launch shape captured (continuity lanes, momentum lanes, block; the third entry of a
# shape is unused): DRAM bytes read + written, issue-active fraction and FP64-pipe
# fraction.
NCU_256 = {
    ("-1,18,128", "continuity"): {"traffic": 3.99616e6, "issue_active": 0.400, "fp64_pipe": 0.145},
    ("-1,18,128", "momentum"): {"traffic": 15.517184e6, "issue_active": 0.410, "fp64_pipe": 0.304},
    ("-1,18,64", "continuity"): {"traffic": 3.996416e6, "issue_active": 0.411, "fp64_pipe": 0.142},
    ("-1,18,64", "momentum"): {"traffic": 15.513856e6, "issue_active": 0.419, "fp64_pipe": 0.300},
}


def timed_window(steps, warmup, interval):
    """(first warm-up step, first timed step): the timed window [s0, s0 + steps) ends on a
    density re-initialisation step and holds ceil(steps / interval) of them."""
    if interval <= 0:
        return 1, 1 + warmup
    end = interval * -(-steps // interval)
    while end - steps + 1 - warmup < 1:
        end += interval
    s0 = end - steps + 1
    return s0 - warmup, s0


def reinit_count(s0, steps, interval):
    return sum(1 for s in range(s0, s0 + steps) if interval > 0 and s % interval == 0)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 3,000 one-step graphs (each after an L2 flush) take about half a second: long
    # enough for several clock samples at 100 ms inside the timed region
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "fp32c"], default="fp32c")
    ap.add_argument("--fp64-steps", type=int, default=30, help="steps of the plain FP64 form reported beside")
    ap.add_argument("--n", type=int, default=256, help="cavity resolution (n x n fluid particles)")
    ap.add_argument("--cpu-sample-steps", type=int, default=0, help="CPU baseline steps (0: auto, ~15 s)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 512-scene batched workload")
    ap.add_argument("--no-served", action="store_true", help="skip the served Poisson stream")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 0 and 2 (dam breaks) beside the headline")
    ap.add_argument("--batched-steps", type=int, default=20)
    ap.add_argument("--served-requests", type=int, default=24, help="requests per served stream (per rate)")
    ap.add_argument("--served-rate", type=float, default=100.0)
    ap.add_argument("--launch-shape", default="",
                    help="FP32 launch shape 'lanes,lanes,lanes,block' instead of the autotuner's pick")
    ap.add_argument("--only-steps", action="store_true",
                    help="upload, warm up and run the timed steps only (the command profiled with ncu)")
    ap.add_argument("--profile-scene", default="", choices=["", "dam_break_3d", "dam_break_2d"],
                    help="with --only-steps: step this scene instead of the cavity (profiling at other sizes)")
    ap.add_argument("--dx", type=float, default=0.01, help="particle spacing of --profile-scene")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(n):
    from ethersph_gb300 import scenes
    return scenes.natural_convection_2d(n=n)


def config_of(scene, args, world):
    return {
        "workload": f"natural_convection_2d n={args.n}: {scene.n_fluid} ThermalLiquidParticle + {scene.n_wall} "
                    "walls, WendlandC2, FluidCompulsiveThermostaticWallSolve, reinit every 30",
        "fluid_particles": scene.n_fluid,
        "wall_particles": scene.n_wall,
        "form": args.precision,
        "replicas": world,
        "l2": "flushed before every timed step (512 MB write)",
        "parallelism": f"replicas x{world}",
    }


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------- CPU baseline
def time_cpu(scene, steps, threads):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    fluid, walls = oracle.scene_arrays(scene)
    prm = scene.params()
    t0 = time.perf_counter()
    oracle.run(prm, fluid, walls, 1, steps, mode=oracle.SCATTER, threads=threads)
    return time.perf_counter() - t0


def time_cpu_window(scene, steps, warmup, threads):
    """The oracle (scatter mode, the reference's half pair list) over our arm's timed
    window: `warmup` steps untimed, then `steps` steps timed in one run."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    fluid, walls = oracle.scene_arrays(scene)
    prm = scene.params()
    first, s0 = timed_window(steps, warmup, scene.td.density_reinitialized_interval_)
    if warmup:
        fluid = oracle.run(prm, fluid, walls, first, warmup, mode=oracle.SCATTER, threads=threads)
    t0 = time.perf_counter()
    oracle.run(prm, fluid, walls, s0, steps, mode=oracle.SCATTER, threads=threads)
    return time.perf_counter() - t0, s0


def cpu_baseline(scene, args):
    threads = cpu_threads()
    steps = args.cpu_sample_steps
    if steps <= 0:
        probe = time_cpu(scene, 2, threads)
        steps = int(max(3, min(300, 15.0 / max(probe / 2, 1e-3))))
    secs = time_cpu(scene, steps, threads)
    return {
        "value": scene.n_fluid * steps / secs,
        "unit": METRIC,
        "cores": threads,
        "kind": "port",
        "sample": f"{steps} steps of the same scene (steps 1..{steps}), {secs:.2f} s, C++ restatement of "
                  "EtherSPHCPU.jl eachStep! (half pair list + atomic scatter, OpenMP)",
    }


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()  # the first sample marks a running sampler
            while not self.samples and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
            self.samples.clear()  # keep only samples taken during the timed region
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, nm in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# ---------------------------------------------------------------- our arm
def algorithmic_bytes(scene, precision, stage, list_entries=0.0):
    """Bytes one launch of the continuity (K4) or momentum (K5) gather must move on the 2D
    thermal cavity: each per-particle SoA element the kernel reads or writes, once
    (neighbour re-reads count zero; the neighbour list, when the launch shape uses it, is
    a per-particle array of `list_entries` 4-byte entries on average plus a 4-byte count,
    written once by K4 and read once by K5).  The numerator of roofline.achieved."""
    nf, nw = scene.n_fluid, scene.n_wall
    assert scene.fluid.x_vec_.shape[1] == 2 and scene.fluid.thermal
    lst = 4 + 4 * list_entries if list_entries else 0
    if stage == "continuity":
        if precision == "fp64":
            fluid = (16 + 16 + 8 + 8 + 4) + 4 * 8    # x v m rho scene | rhoc p c P
        else:
            fluid = (16 + 16 + 4 + 4 + 8 + 8) + (5 * 8 + 16) + lst  # fa fb cell scene rho m | rhoc p c P vol fb
        return nf * fluid
    writes = 16 + 16 + 8 + 8 + 4 + 4  # x' v' (double2) T' rho' key slot
    if precision == "fp64":
        fluid = (16 + 16 + 8 * 8 + 4) + writes  # x v | rhoc P m gap c T kappa cp | scene
        wall = 16 + 16 + 16 + 8 + 8 + 8 + 4     # x n v gap T kappa kind
    else:
        fluid = (16 + 16 + 16 + 8 + 4 + 4 + 16 + 16 + 8 + 8) + writes + lst  # fa fb fc c cell scene | x v T rhoc
        wall = 16 + 16 + 16                                                 # float4 shadows fa fb fc
    return nf * fluid + nw * wall


def scan_launches(cells):
    """Kernels of a step's cell scan (sph_sort.cu launch_scan): one block up to 16,384
    cells; up to 262,144 cells one down-sweep (the momentum epilogue sums the 1,024-cell
    tiles); above, tile sums, top and down-sweep."""
    return 1 if cells <= 64 * 4096 else 3


def grid_cells(scene, precision):
    """Cells of the scene's grid, as the library builds it."""
    from ethersph_gb300 import batch
    return batch.grid_cells(scene, 0, precision)


def time_form(pkg, _abi, scene, precision, steps, warmup, tune=False, shape=None, stages=True):
    """Plain device timing of one form on one scene: CUDA events around each step on the
    handle's stream, L2 flushed before every step, a timed window that ends on a density
    re-initialisation step.  Returns (ms per step, stage times, launch shape, window)."""
    import torch
    prm = scene.params(precision=precision)
    with pkg.Simulation(prm, scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        sim.upload_fluid(scene.fluid)
        if shape:
            sim.set_launch_shape(*shape)
        elif tune and precision == _abi.PRECISION_FP32_COMPENSATED:
            shape = sim.autotune(2)
        lib, h = sim.lib, sim.h
        stream = torch.cuda.ExternalStream(sim.stream())
        flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        interval = scene.td.density_reinitialized_interval_
        step, s0 = timed_window(steps, warmup, interval)
        for _ in range(warmup):
            _abi.check(lib, h, lib.sph_step(h, step, 1))
            step += 1
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for k in range(steps):
                flush.zero_()
                ev[k][0].record(stream)
                _abi.check(lib, h, lib.sph_step_async(h, step, 1))
                ev[k][1].record(stream)
                step += 1
        _abi.check(lib, h, lib.sph_synchronize(h))
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        st = sim.time_stages(5) if stages else None
    window = {"steps": [s0, s0 + steps - 1], "reinit_steps": reinit_count(s0, steps, interval)}
    return ms, st, shape, window


def time_e2e(pkg, scene, precision, shape, steps=100, iters=3):
    """End to end through the C ABI with host arrays, as a Julia caller runs it: upload
    the fluid, `steps` steps, download the state into the caller's arrays (allocated
    before the timed region; the reference updates its particle vectors in place)."""
    import torch
    f = scene.fluid
    names = [("x", "x_vec_"), ("v", "v_vec_"), ("rho", "rho_"), ("p", "p_"), ("c", "c_"), ("mass", "mass_"),
             ("gap", "gap_")] + ([("t", "t_"), ("kappa", "kappa_"), ("cp", "cp_")]
                                 if getattr(f, "thermal", False) else [])
    h2d = sum(getattr(f, a).nbytes for _, a in names)
    out = {k: np.zeros_like(getattr(f, a)) for k, a in names}
    with pkg.Simulation(scene.params(precision=precision), scene.n_fluid, scene.n_wall) as sim:
        for w in scene.walls:
            sim.upload_walls(w)
        if shape:
            sim.set_launch_shape(*shape)
        # one untimed iteration: the step graphs of both buffer parities, the neighbour list
        # and the download scratch exist before the timed region
        sim.upload_fluid(f)
        sim.step(1, steps)
        sim.download(scene.n_fluid, out=out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = {}
        for _ in range(iters):
            sim.upload_fluid(f)
            sim.step(1, steps)
            r = sim.download(scene.n_fluid, out=out)
        secs = time.perf_counter() - t0
    d2h = sum(a.nbytes for a in r.values())
    return {"value": scene.n_fluid * steps * iters / secs, "unit": METRIC, "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": d2h / steps,
            "what": f"upload + {steps} steps (re-initialisations at 30, 60, 90) + download per iteration, "
                    f"{iters} iterations"}


def run_configs(pkg, _abi, args):
    """Configs 0 and 2 of the benchmark list beside the headline: the 2D dry dam break
    (5,000 fluid) and the 3D dam break at dx = 0.005 (3,456,000 fluid + 1,678,380 walls),
    both forms, the FP32-compensated one at its autotuned launch shape."""
    from ethersph_gb300 import scenes
    res = {}
    cases = (("config0_dam_break_2d", lambda: scenes.dam_break_2d(dx=0.02), 200, 20),
             ("config2_dam_break_3d", lambda: scenes.dam_break_3d(dx=0.005), 20, 3))
    for key, make, steps32, steps64 in cases:
        scene = make()
        ms32, st32, shape, win32 = time_form(pkg, _abi, scene, _abi.PRECISION_FP32_COMPENSATED, steps32, 3,
                                             tune=True, stages=False)
        ms64, _, _, win64 = time_form(pkg, _abi, scene, _abi.PRECISION_FP64, steps64, 1, stages=False)
        res[key] = {"fluid_particles": scene.n_fluid, "wall_particles": scene.n_wall,
                    "fp32c": {"ms_per_step": ms32, "value": scene.n_fluid / (ms32 / 1e3), "launch_shape": shape,
                              "window": win32},
                    "fp64": {"ms_per_step": ms64, "value": scene.n_fluid / (ms64 / 1e3), "window": win64},
                    "fp32c_over_fp64": ms64 / ms32}
    return res


def run_ours(args, rank, world, local):
    import torch
    import ethersph_gb300 as pkg
    from ethersph_gb300 import _abi

    torch.cuda.set_device(local)
    scene = workload(args.n)
    if args.only_steps and args.profile_scene:
        from ethersph_gb300 import scenes
        scene = getattr(scenes, args.profile_scene)(dx=args.dx)
    prec = _abi.PRECISION_FP64 if args.precision == "fp64" else _abi.PRECISION_FP32_COMPENSATED
    prm = scene.params(precision=prec)
    sim = pkg.Simulation(prm, scene.n_fluid, scene.n_wall)
    for w in scene.walls:
        sim.upload_walls(w)
    sim.upload_fluid(scene.fluid)
    if args.launch_shape:
        launch_shape = tuple(int(v) for v in args.launch_shape.split(","))
        sim.set_launch_shape(*launch_shape)
        chosen_by = "--launch-shape"
    else:
        launch_shape = sim.autotune(3)  # lanes per particle x block size, picked on this scene
        chosen_by = "sph_autotune"
    lib, h = sim.lib, sim.h
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    interval = scene.td.density_reinitialized_interval_
    step, s0 = timed_window(args.steps, args.warmup, interval)
    for _ in range(args.warmup):
        _abi.check(lib, h, lib.sph_step(h, step, 1))
        step += 1
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                ev[k][0].record(stream)
                _abi.check(lib, h, lib.sph_step_async(h, step, 1))
                ev[k][1].record(stream)
                step += 1
        _abi.check(lib, h, lib.sph_synchronize(h))
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    reinit_steps = reinit_count(s0, args.steps, interval)
    if args.only_steps:
        sim.close()
        if rank == 0:
            print(json.dumps({"only_steps": True, "ms_per_step": ms / args.steps, "form": args.precision}))
        return None
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = scene.n_fluid * args.steps * world / (ms_max / 1e3)
    clocks = clk.summary()

    # per-stage times (CUDA events on the handle's stream), roofline of the two gathers
    stages = sim.time_stages(20)
    # what a persistent step kernel could remove: warm steps as the library runs them (CUDA
    # graphs of 10-step bundles, programmatic launches) against the sum of the warm
    # per-stage kernel times of one step (continuity, momentum, scan, hash-free placement)
    warm_steps = 300
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        _abi.check(lib, h, lib.sph_step_async(h, step, 30))
        step += 30
        e0.record(stream)
        _abi.check(lib, h, lib.sph_step_async(h, step, warm_steps))
        e1.record(stream)
        step += warm_steps
    _abi.check(lib, h, lib.sph_synchronize(h))
    warm_ms = e0.elapsed_time(e1) / warm_steps
    kernels_ms = (stages["continuity"] + stages["momentum"] + stages["scan"] + stages["sort"] +
                  (stages["reinit"] - stages["momentum"]) / interval)
    launch_overhead = {"warm_step_ms": warm_ms, "sum_of_stage_kernels_ms": kernels_ms,
                       "overhead_ms": warm_ms - kernels_ms, "overhead_frac": (warm_ms - kernels_ms) / warm_ms,
                       "what": f"{warm_steps} steps in 10-step graph bundles without L2 flush, against the warm "
                               "per-stage times (sph_time_stages) of one step, Shepard amortised"}
    peaks = json.loads(MEASURED_PEAKS.read_text()) if MEASURED_PEAKS.exists() else {}
    hbm = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or FALLBACK_HBM_GBS
    pairs_ff, pairs_fw = sim.count_pairs()
    sim.close()
    uses_list = args.precision == "fp32c" and launch_shape[1] >= LANES_LIST - 1
    entries = 2.0 * pairs_ff / scene.n_fluid if uses_list else 0.0
    shape_key = f"{launch_shape[0]},{launch_shape[1]},{launch_shape[3]}"

    def roofline(stage, label):
        b = algorithmic_bytes(scene, args.precision, stage, entries)
        achieved = b / (stages[stage] / 1e3) / 1e9
        ncu = NCU_256.get((shape_key, stage)) if (args.n == 256 and args.precision == "fp32c") else None
        return {
            "bound": "hbm",
            "kernel": label,
            "achieved": achieved,
            "peak": hbm,
            "unit": "GB/s",
            "frac": achieved / hbm,
            "peak_source": f"{peak_src} hbm_gbs (burst copy)",
            "algorithmic_bytes_per_launch": b,
            "neighbour_list_bytes_per_launch": (4 + 4 * entries) * scene.n_fluid if uses_list else 0,
            "launch_ms": stages[stage],
            "traffic": ncu["traffic"] if ncu else None,
            "traffic_source": (f"ncu --set full of this launch at n=256 and this launch shape ({shape_key}): "
                               "dram__bytes_read.sum + dram__bytes_write.sum" if ncu else
                               f"no capture at this launch shape ({shape_key})"),
            "issue_frac": ncu["issue_active"] if ncu else None,
            "fp64_pipe_frac": ncu["fp64_pipe"] if ncu else None,
            "limiter": ("FP64 ALU (FP64 at 1/64 of the FP32 rate on GB300)" if args.precision == "fp64" else
                        "issue/latency: dependent neighbour loads and pair arithmetic on 13-23 warps per SM; "
                        "DRAM reads at or below the algorithmic bytes"),
        }

    roof = {"continuity": roofline("continuity", "continuity + EOS (K4)"),
            "momentum": roofline("momentum", "momentum + integrate, the fused pair kernel (K5)")}
    dominant = max(roof, key=lambda k: stages[k])

    e2e = time_e2e(pkg, scene, prec, launch_shape if prec == _abi.PRECISION_FP32_COMPENSATED else None,
                   iters=10 if prec == _abi.PRECISION_FP32_COMPENSATED else 3)
    et = torch.tensor([e2e["value"]], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(et, op=torch.distributed.ReduceOp.MIN)
    e2e["value"] = float(et.item()) * world

    other = None
    if args.precision == "fp32c" and args.fp64_steps > 0:
        ms64, st64, _, win64 = time_form(pkg, _abi, scene, _abi.PRECISION_FP64, args.fp64_steps, 3)
        e64 = time_e2e(pkg, scene, _abi.PRECISION_FP64, None)
        e64["value"] *= world
        v64 = scene.n_fluid * world / (ms64 / 1e3)
        other = {"form": "plain fp64 (equal to the CPU restatement to FP64 rounding)", "ms_per_step": ms64,
                 "value": v64, "window": win64, "stages_ms": st64, "e2e": e64,
                 "speedup_of_fp32c": value / v64, "e2e_speedup_of_fp32c": e2e["value"] / e64["value"]}
    configs = run_configs(pkg, _abi, args) if not args.no_configs else None
    if rank != 0:
        return None
    out = {
        "metric": METRIC,
        "value": value,
        "unit": METRIC,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32",
        "data": "synthetic (seeded scene generator)",
        "config": config_of(scene, args, world),
        "timed_window": {"steps": [s0, s0 + args.steps - 1], "reinit_steps": reinit_steps},
        "pair_interactions_per_s": pairs_ff * args.steps * world / (ms_max / 1e3),
        "pairs": {"fluid_fluid_unique": pairs_ff, "fluid_wall": pairs_fw},
        "stages_ms": stages,
        "launch_overhead": launch_overhead,
        "roofline": roof[dominant],
        "roofline_other_gather": roof["continuity" if dominant == "momentum" else "momentum"],
        "e2e": e2e,
        "plain_fp64": other,
        "configs": configs,
        "launch_shape": {"continuity_lanes": launch_shape[0], "momentum_lanes": launch_shape[1],
                         "block": launch_shape[3], "chosen_by": chosen_by},
        # per step: continuity, momentum (with the Shepard sums on re-initialisation steps),
        # scan (1 kernel up to 262,144 cells, else 3), fill, placement
        "gpu_launches": args.steps * (4 + scan_launches(grid_cells(scene, prec))),
        "clocks": clocks,
    }
    return out


def time_batch_steps(bt, steps, warmup):
    """CUDA-event time of `steps` steps of a batch (its state is larger than L2)."""
    import torch
    stream = torch.cuda.ExternalStream(bt.stream())
    for _ in range(warmup):
        bt.step(1)
    bt.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    bt.step(steps)
    e1.record(stream)
    bt.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_batched(args, rank=0, world=1):
    """512 seeded 2D dam breaks (dx 0.01, 450-67,500 fluid particles each) stepped in one
    set of launches: FP32-compensated with an autotuned launch shape, and plain FP64.
    Every scene starts at the step number that puts a density re-initialisation step at
    the end of the timed window.  Under torchrun every rank steps its share of the scenes
    (k % world == rank); the slowest rank's time and all ranks' particles give the
    whole-job rate."""
    import ethersph_gb300  # noqa: F401
    from ethersph_gb300 import batch, distributed, scenes
    every = scenes.batched_dam_breaks(512, seed=0)
    sc = distributed.shard(every, rank, world)
    nf = sum(s.n_fluid for s in sc)
    nw = sum(s.n_wall for s in sc)
    nc = sum(batch.footprint(s, 1)[1] for s in sc)          # FP32 form
    nc64 = sum(batch.footprint(s, 0)[1] for s in sc)        # FP64 form
    nf_all = sum(s.n_fluid for s in every)
    res = {"workload": f"512 batched 2D dam breaks, {nf_all} fluid + {sum(s.n_wall for s in every)} wall "
                       "particles, CubicSpline, FluidWallSolve, per-scene c0 and dt", "fluid_particles": nf_all,
           "l2": "state larger than L2 (no flush)", "ranks": world}
    interval = every[0].td.density_reinitialized_interval_
    for prec, steps in ((1, args.batched_steps), (0, 2)):
        warm = 2
        first, s0 = timed_window(steps, warm, interval)
        cells = (nc if prec == 1 else nc64) + 1024
        with batch.Batch(sc[0].params(precision=prec), nf + 1024, cells, nw + 1024, 512) as bt:
            for s in sc:
                bt.add_scene(s, first, 1000)
            shape = bt.autotune(2) if prec == 1 else None
            ms = time_batch_steps(bt, steps, warm)
            ms_all, _, rate = distributed.aggregate(ms, nf, device="cuda")
            key = "fp32c" if prec == 1 else "fp64"
            res[key] = {"ms_per_step": ms_all, "particle_steps_per_s": rate, "steps": steps,
                        "window": {"steps": [s0, s0 + steps - 1], "reinit_steps": reinit_count(s0, steps, interval)}}
            if shape:
                res[key]["launch_shape"] = shape
                res[key]["stages_ms"] = bt.time_stages(3)
    res["fp32c_over_fp64"] = res["fp32c"]["particle_steps_per_s"] / res["fp64"]["particle_steps_per_s"]
    return res


SERVED_RATES = (10.0, 30.0, 100.0, 300.0, 1000.0)


def run_served(args, rank=0, world=1):
    """A Poisson stream of mixed scene requests (2D dam breaks, periodic 2D Poiseuille,
    3D dam breaks) served by continuous batching, in the FP32-compensated form with the
    full step budgets U{500..5000}, at every arrival rate of SERVED_RATES (latency p50/p99
    and particle-steps/s per rate); and FP32-compensated against plain FP64 on the same
    shorter stream with the same 150 GB admission budget."""
    import ethersph_gb300  # noqa: F401
    from ethersph_gb300 import distributed, scenes, serve
    budget = 150e9
    out = {"budget_bytes": budget}

    def serve_stream(prec, count, steps, seed, rate):
        reqs = distributed.shard(scenes.poisson_stream(rate=rate, count=count, seed=seed, steps=steps), rank, world)
        srv = serve.Server(budget_bytes=budget, precision=prec)  # FP32c: the fixed list shape
        try:
            rep = srv.run(reqs)
        finally:
            srv.close()
        s = serve.summarize_ranks(rep, world)
        s.update(rate_per_s=rate, steps_per_request=list(steps), stream_seed=seed)
        return s

    out["fp32c_rate_sweep"] = [serve_stream(1, args.served_requests, (500, 5000), 1, r) for r in SERVED_RATES]
    short = 12  # the same 12 requests in both forms
    out["fp32c_short"] = serve_stream(1, short, (200, 800), 2, args.served_rate)
    out["fp64_short"] = serve_stream(0, short, (200, 800), 2, args.served_rate)
    out["fp32c_over_fp64_same_stream"] = (out["fp32c_short"]["particle_steps_per_s"] /
                                          out["fp64_short"]["particle_steps_per_s"])
    out["workload"] = ("Poisson arrivals, 1/3 each 2D dam break (batched distribution), periodic 2D Poiseuille "
                       "(H=1mm, Re~U[0.01,1], dx=H/U{20..80}), 3D dam break (dx~U[0.01,0.02]); "
                       "150 GB device admission budget for both forms")
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        if rank == 0:
            scene = workload(args.n)
            threads = cpu_threads()
            secs, s0 = time_cpu_window(scene, args.steps, args.warmup, threads)
            val = scene.n_fluid * args.steps / secs
            line = {"metric": METRIC, "value": val, "unit": METRIC, "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
                    "config": config_of(scene, args, 1), "impl": "reference",
                    "cpu_baseline": {"value": val, "unit": METRIC, "cores": threads, "kind": "port",
                                     "sample": f"steps {s0}..{s0 + args.steps - 1} of the same scene after "
                                               f"{args.warmup} warm-up steps (the timed window of our arm), one "
                                               "run; C++ restatement of EtherSPHCPU.jl eachStep! (Julia absent)"},
                    "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line))
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    out = run_ours(args, rank, world, local)
    batched = run_batched(args, rank, world) if not (args.no_batched or args.only_steps) else None
    served = run_served(args, rank, world) if not (args.no_served or args.only_steps) else None
    if rank == 0 and out is not None:
        if batched:
            out["batched"] = batched
        if served:
            out["served"] = served
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(workload(args.n), args)
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
