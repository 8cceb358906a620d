"""The serving loop's host logic on the CPU, with a stand-in for the device batches:
admission by footprint (particles, cells, walls, scene slots), continuous batching (new
requests join while others run), retirement when a scene's step budget is done, the
particle-step accounting and the latency percentiles.  The batches record what the loop
asks of them; no GPU is involved."""
import numpy as np
import pytest

from ethersph_gb300 import _abi, scenes, serve
from ethersph_gb300.batch import footprint


class FakeBatch:
    """Capacity bookkeeping of a device batch (sph_batch_free / add / retire), stepping
    by counting steps per resident scene."""

    instances = []

    def __init__(self, particles, cells, walls, slots):
        self.cap = {"particles": particles, "cells": cells, "walls": walls, "scenes": slots}
        self.used = {k: 0 for k in self.cap}
        self.live = {}
        self.next_id = 0
        self.shape = None
        self.max_resident = 0
        self.log = []
        FakeBatch.instances.append(self)

    @classmethod
    def for_budget(cls, prototype, budget_bytes, scene_capacity=4096, cells_per_particle=2.0, walls_per_particle=1.0,
                   lib=None):
        particles = int(budget_bytes // 500)
        return cls(particles, int(particles * cells_per_particle), int(particles * walls_per_particle),
                   scene_capacity)

    def set_launch_shape(self, *shape):
        self.shape = shape

    def autotune(self, reps=3):
        return (1, 1, 1, 128)

    def free(self):
        return {k: self.cap[k] - self.used[k] for k in self.cap}

    def add_scene(self, scene, first_step=1, nsteps=None):
        p, c, w = footprint(scene, _abi.PRECISION_FP32_COMPENSATED)
        need = {"particles": p, "cells": c, "walls": w, "scenes": 1}
        for k, v in need.items():
            assert self.used[k] + v <= self.cap[k], f"admitted beyond the {k} capacity"
            self.used[k] += v
        sid = self.next_id
        self.next_id += 1
        self.live[sid] = {"need": need, "nsteps": nsteps, "done": 0, "n": scene.n_fluid}
        self.max_resident = max(self.max_resident, len(self.live))
        self.log.append(("add", sid))
        return sid

    def step(self, n):
        for rec in self.live.values():
            rec["done"] = min(rec["nsteps"], rec["done"] + n)  # frozen after its budget

    def synchronize(self):
        pass

    def info(self, sid):
        return {"n_fluid": self.live[sid]["n"]}

    def download(self, sid):
        n = self.live[sid]["n"]
        return {"rho": np.ones(n), "x": np.zeros((n, 2))}

    def retire(self, sid):
        rec = self.live.pop(sid)
        assert rec["done"] == rec["nsteps"], "retired before its step budget ran"
        for k, v in rec["need"].items():
            self.used[k] -= v
        self.log.append(("retire", sid))

    def close(self):
        pass


@pytest.fixture
def fake_batches(monkeypatch):
    FakeBatch.instances = []
    monkeypatch.setattr(serve, "Batch", FakeBatch)
    return FakeBatch


def test_every_request_served_once_with_exact_accounting(fake_batches):
    reqs = scenes.poisson_stream(rate=2000.0, count=9, seed=4, steps=(20, 75))
    srv = serve.Server(budget_bytes=2e9, bundle=10)
    rep = srv.run(reqs)
    s = rep.summary()
    assert s["requests"] == len(reqs)
    assert sorted(id(c.request) for c in rep.completed) == sorted(id(r) for r in reqs)
    # particle-steps: each scene's budget times its particles, nothing more
    assert rep.particle_steps == sum(r.nsteps * c.n_fluid for c in rep.completed for r in [c.request])
    assert all(c.t_done >= c.request.t_arrival for c in rep.completed)
    assert s["latency_p99_s"] >= s["latency_p50_s"] > 0
    # the FP32-compensated batches run at the fixed neighbour-list shape
    for b in fake_batches.instances:
        assert b.shape == serve.DEFAULT_LAUNCH_SHAPE
        assert not b.live  # everything retired


def test_admission_waits_for_memory_and_batches_continuously(fake_batches):
    # a budget that holds only a few scenes at a time: later requests wait in the queue
    # and are admitted as earlier ones retire, into the running batch
    reqs = scenes.poisson_stream(rate=5000.0, count=8, seed=7, steps=(30, 60), kinds=("dam_break_2d",))
    biggest = max(footprint(r.build(), _abi.PRECISION_FP32_COMPENSATED)[0] for r in reqs)
    budget = 500 * 2.5 * biggest / 0.6  # 2D share of the budget: room for about two scenes
    srv = serve.Server(budget_bytes=budget, bundle=10)
    rep = srv.run(reqs)
    assert rep.summary()["requests"] == len(reqs)
    b2 = fake_batches.instances[0]
    assert 1 <= b2.max_resident < len(reqs)
    # some scene was added after another retired (continuous batching, not one wave)
    first_retire = next(k for k, (op, _) in enumerate(b2.log) if op == "retire")
    assert any(op == "add" for op, _ in b2.log[first_retire:])


def test_summarize_ranks_on_one_rank_is_the_local_summary(fake_batches):
    reqs = scenes.poisson_stream(rate=1000.0, count=3, seed=2, steps=(10, 20), kinds=("poiseuille_2d",))
    rep = serve.Server(budget_bytes=1e9).run(reqs)
    assert serve.summarize_ranks(rep, 1) == rep.summary()


def test_request_larger_than_an_empty_batch_is_refused(fake_batches):
    # the loop would otherwise wait forever for room that never comes
    reqs = scenes.poisson_stream(rate=1000.0, count=2, seed=3, steps=(10, 20), kinds=("dam_break_2d",))
    srv = serve.Server(budget_bytes=2e5)
    with pytest.raises(ValueError, match="more than the 2D batch holds"):
        srv.run(reqs)
