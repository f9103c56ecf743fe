"""The serving loop's host logic (fdps_sph_gb300/serve.py) on the CPU, against a stand-in context
that records the run calls: FIFO admission within the particle budget and the run-slot limit,
a new run's first batched step taken as its prologue and not counted, each run downloaded and
removed once after its steps, the batch backfilled from the queue, and the report's counts."""
import numpy as np

from fdps_sph_gb300 import serve


class FakeContext:
    def __init__(self):
        self.runs, self.next, self.steps, self.log = {}, 1, 0, []
        self.max_resident = self.max_runs = 0

    def add_run(self, F, ids, mats):
        h = self.next
        self.next += 1
        self.runs[h] = F.shape[1]
        self.log.append(("add", h, self.steps))
        self.max_resident = max(self.max_resident, sum(self.runs.values()))
        self.max_runs = max(self.max_runs, len(self.runs))
        return h

    def step(self, k):
        self.steps += k

    def download_run(self, h):
        self.log.append(("download", h, self.steps))
        n = self.runs[h]
        return np.zeros((34, n)), np.arange(n), np.zeros(n, np.int32)

    def remove_run(self, h):
        self.log.append(("remove", h, self.steps))
        del self.runs[h]

    def close(self):
        pass


def _requests(steps):
    return [serve.Request(k, 0.0, s, 500 + k, 2000, 3000) for k, s in enumerate(steps)]


def test_admission_budget_prologue_and_backfill():
    ctx = FakeContext()
    steps = (3, 1, 4, 2, 2)
    reqs = _requests(steps)
    budget = serve.BYTES_PER_PARTICLE * 6500    # room for two runs of 2,000-3,000 particles
    srv = serve.Server(budget_bytes=budget, ctx=ctx)
    rep = srv.run(reqs)
    assert rep["completed"] == len(reqs) and rep["resident_at_end"] == 0 and rep["queued_at_end"] == 0
    assert ctx.max_resident <= 6500 and not ctx.runs
    adds = [e for e in ctx.log if e[0] == "add"]
    assert [h for _, h, _ in adds] == sorted(h for _, h, _ in adds)         # FIFO: handles in arrival order
    by_handle = {r.handle: r for r in reqs}
    for h, r in by_handle.items():
        t_add = next(t for e, hh, t in ctx.log if e == "add" and hh == h)
        t_dl = next(t for e, hh, t in ctx.log if e == "download" and hh == h)
        assert t_dl - t_add == r.steps + 1                                  # prologue + its steps
        assert [e for e, hh, _ in ctx.log if hh == h] == ["add", "download", "remove"]
    assert rep["particle_steps"] == sum(r.n * r.steps for r in reqs)
    assert rep["batched_steps"] == ctx.steps
    assert rep["time_to_completion_s"]["p50"] > 0 and rep["step_latency_s"]["p99"] is not None
    # the time inside the batched steps is part of the wall time; its throughput excludes admission
    assert 0.0 < rep["stepping_s"] <= rep["wall_s"]
    assert rep["particle_steps_per_stepping_s"] >= rep["particle_steps_per_s"]


def test_run_slots_limit_and_oversized_first_run():
    ctx = FakeContext()
    reqs = _requests((2, 2, 2))
    srv = serve.Server(budget_bytes=serve.BYTES_PER_PARTICLE * 10 ** 6, max_runs=1, ctx=ctx)
    rep = srv.run(reqs)
    assert rep["completed"] == 3 and ctx.max_runs == 1
    # a run larger than the whole budget is still admitted when nothing else is resident
    ctx2 = FakeContext()
    srv2 = serve.Server(budget_bytes=serve.BYTES_PER_PARTICLE * 100, ctx=ctx2)
    rep2 = srv2.run(_requests((1, 1)))
    assert rep2["completed"] == 2 and ctx2.max_runs == 1
