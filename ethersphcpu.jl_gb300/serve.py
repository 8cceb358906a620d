"""Serving loop: scene requests arrive over time, stay resident on the device, are
admitted by device-memory footprint, stepped together, retired when done.

This is continuous batching, not a queue: requests that arrive while others run are
added to the running batch as soon as particle slots, a contiguous run of cells and of
wall slots and a scene slot are free (sph_batch_free), every bundle of steps advances
every resident scene in the same kernel launches, and finished scenes are downloaded and
retired between bundles, which frees their memory for the queue.  2D and 3D scenes use
two batch handles (the kernels are specialised by dimension); each has its own CUDA
stream, so their bundles overlap on the GPU.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .batch import Batch, bytes_per, footprint


@dataclass
class Completed:
    request: object
    t_admit: float
    t_done: float
    n_fluid: int
    result: dict = field(repr=False, default=None)

    @property
    def latency(self) -> float:
        return self.t_done - self.request.t_arrival


@dataclass
class Report:
    completed: list
    wall_s: float
    particle_steps: int

    def summary(self) -> dict:
        lat = np.array([c.latency for c in self.completed]) if self.completed else np.zeros(1)
        return {
            "requests": len(self.completed),
            "wall_s": self.wall_s,
            "particle_steps": self.particle_steps,
            "particle_steps_per_s": self.particle_steps / self.wall_s if self.wall_s > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99)),
            "latency_mean_s": float(lat.mean()),
        }


def summarize_ranks(report: Report, world: int = 1) -> dict:
    """Report.summary() over every rank of a sharded stream: the slowest rank's wall
    time, all ranks' particle-steps, and percentiles over all ranks' latencies.  Every
    rank must call it (it gathers); with one rank it is the local summary."""
    if world <= 1:
        return report.summary()
    import torch.distributed as dist
    mine = (report.wall_s, report.particle_steps, [c.latency for c in report.completed])
    every = [None] * world
    dist.all_gather_object(every, mine)
    wall = max(w for w, _, _ in every)
    steps = sum(p for _, p, _ in every)
    lat = np.array([x for _, _, ls in every for x in ls]) if any(ls for _, _, ls in every) else np.zeros(1)
    return {
        "requests": sum(len(ls) for _, _, ls in every),
        "wall_s": wall,
        "particle_steps": steps,
        "particle_steps_per_s": steps / wall if wall > 0 else 0.0,
        "latency_p50_s": float(np.percentile(lat, 50)),
        "latency_p99_s": float(np.percentile(lat, 99)),
        "latency_mean_s": float(lat.mean()),
        "ranks": world,
    }


# Launch shape of the FP32-compensated form in a served batch: continuity on one pipelined
# lane recording the neighbour list, momentum reading it on two lanes, 128-thread blocks.
# Fixed (not re-tuned as the mix changes): a served result equals the same scene run alone
# at this shape, and on GB300 the fixed list shape served the bench's 48-request stream
# faster (500 M particle-steps/s, p50 6.0 s) than re-tuning whenever the live particles
# doubled (458 M/s, p50 6.7 s: the tuning launches cost more than they won).
DEFAULT_LAUNCH_SHAPE = (-1, _abi.LANES_LIST + 2, -1, 128)


class Server:
    def __init__(self, budget_bytes: float = 150e9, precision: int = _abi.PRECISION_FP32_COMPENSATED,
                 share_3d: float = 0.4, bundle: int = 10, scene_capacity: int = 4096, keep_results: bool = False,
                 launch_shape=None, autotune: bool = False, lib=None):
        from . import scenes
        self.bundle = bundle
        self.precision = precision
        self.keep_results = keep_results
        # re-tune a batch's launch shape (sph_autotune) whenever its live particles have
        # doubled since the last tuning; off by default, because the FP32 form's results
        # depend on the shape and a served result should equal the same scene run alone
        self.autotune = autotune and launch_shape is None and precision == _abi.PRECISION_FP32_COMPENSATED
        if launch_shape is None and not self.autotune and precision == _abi.PRECISION_FP32_COMPENSATED:
            launch_shape = DEFAULT_LAUNCH_SHAPE
        proto2 = scenes.dam_break_2d(dx=0.05).params(precision=precision)
        proto3 = scenes.dam_break_3d(dx=0.05, tank=(0.4, 0.2, 0.4), column=(0.1, 0.1, 0.2)).params(precision=precision)
        # cells of r_cut/3 (the library's default grid): a dam-break tank takes about 6.75 cells
        # per fluid particle in 2D and in 3D
        self.batches = {
            2: Batch.for_budget(proto2, int(budget_bytes * (1.0 - share_3d)), scene_capacity,
                                cells_per_particle=6.75, walls_per_particle=0.6, lib=lib),
            3: Batch.for_budget(proto3, int(budget_bytes * share_3d), scene_capacity,
                                cells_per_particle=6.75, walls_per_particle=3.0, lib=lib),
        }
        if launch_shape is not None:
            for b in self.batches.values():
                b.set_launch_shape(*launch_shape)

    def close(self):
        for b in self.batches.values():
            b.close()

    def run(self, requests, time_limit: float | None = None) -> Report:
        pending = collections.deque(sorted(requests, key=lambda r: r.t_arrival))
        queues = {2: collections.deque(), 3: collections.deque()}
        active = {}  # (dim, sid) -> [request, t_admit, steps_left, n_fluid]
        tuned_at = {2: 0, 3: 0}
        done = []
        particle_steps = 0
        t0 = time.perf_counter()
        while pending or active or any(queues.values()):
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                break
            while pending and pending[0].t_arrival <= now:
                r = pending.popleft()
                scene = r.build()
                queues[scene.kernel.dim_].append((r, scene))
            # admission: first come first served per dimension, while the footprint fits
            for dim, q in queues.items():
                b = self.batches[dim]
                while q:
                    r, scene = q[0]
                    p, c, w = footprint(scene, self.precision)
                    fr = b.free()
                    if not (p <= fr["particles"] and c <= fr["cells"] and w <= fr["walls"] and fr["scenes"] >= 1):
                        if not any(d == dim for d, _sid in active):  # an empty batch cannot hold it
                            raise ValueError(f"request {r.kind} (seed {r.seed}) needs {p} particles, {c} cells and "
                                             f"{w} walls: more than the {dim}D batch holds ({fr})")
                        break
                    q.popleft()
                    sid = b.add_scene(scene, first_step=1, nsteps=r.nsteps)
                    active[(dim, sid)] = [r, time.perf_counter() - t0, r.nsteps, scene.n_fluid]
            if not active:
                if pending:
                    time.sleep(max(0.0, min(0.01, pending[0].t_arrival - (time.perf_counter() - t0))))
                continue
            if self.autotune:
                for dim, b in self.batches.items():
                    live = sum(rec[3] for (d, _sid), rec in active.items() if d == dim)
                    if live >= 20_000 and live >= 2 * tuned_at[dim]:
                        b.autotune(2)
                        tuned_at[dim] = live
            # one bundle of steps for every resident scene (both batches, overlapping)
            running = {dim for (dim, _sid) in active}
            for dim in running:
                self.batches[dim].step(self.bundle)
            for dim in running:
                self.batches[dim].synchronize()
            t_now = time.perf_counter() - t0
            for key in list(active):
                rec = active[key]
                steps = min(self.bundle, rec[2])
                particle_steps += steps * rec[3]
                rec[2] -= steps
                if rec[2] <= 0:
                    dim, sid = key
                    b = self.batches[dim]
                    result = b.download(sid) if self.keep_results else None
                    n_end = b.info(sid)["n_fluid"] if not self.keep_results else len(result["rho"])
                    b.retire(sid)
                    done.append(Completed(rec[0], rec[1], t_now, n_end, result))
                    del active[key]
        return Report(done, time.perf_counter() - t0, particle_steps)
