"""Batched sweeps and a serving loop over one multi-run context.

Many impacts of uneven size advance together: one context holds all resident
runs, and each pass of a step is one set of launches over all their particles
(per-run offsets; every run keeps its own octree, dt and time, and its result
does not depend on the other runs).

* ``sweep``: a fixed set of runs (the 256-impact batched sweep), all admitted
  at once when they fit, each removed when it has taken its steps.
* ``serve``: a request loop.  Requests arrive as a Poisson stream; a request
  is admitted (FIFO) when the resident particles plus its own fit the HBM
  budget and a run slot is free, its state stays on the device until it has
  taken its steps, then it is downloaded and removed and the batch is
  backfilled from the queue.  Reported: p50 / p99 per-step latency (the wall
  time of the batched step each resident run advanced in), p50 / p99
  time-to-completion (arrival to result on the host), and aggregate
  particle-steps/s.

    python -m fdps_sph_gb300.serve sweep --runs 256 --steps 100
    python -m fdps_sph_gb300.serve serve --duration 600 --rate 2
"""
import argparse
import collections
import json
import queue
import threading
import time

import numpy as np

from . import eos, ic, lib

# device bytes per resident particle, the admission unit: state and its ping-pong
# copy (0.6 KB), octree (0.4 KB), neighbour superset rows (12 B x row capacity,
# about 4 KB), exact lists (about 1.5 KB), packs; doubled for the peak while a
# row capacity grows (old and new rows are held together)
BYTES_PER_PARTICLE = 16384


def make_context(precision="mixed", device=0):
    ctx = lib.Context(precision=precision, device=device)
    for k, name in enumerate(("iron", "dunite")):
        ctx.set_material(k, eos.synthetic_table(name))
    return ctx


def hbm_budget(device=0, fraction=0.8):
    """bytes the runs may hold: a fraction of the device memory free now"""
    import torch
    free, _ = torch.cuda.mem_get_info(device)
    return int(free * fraction)


def percentiles(v):
    if not len(v):
        return {"p50": None, "p99": None}
    a = np.asarray(v, np.float64)
    return {"p50": float(np.percentile(a, 50)), "p99": float(np.percentile(a, 99))}


class Request:
    __slots__ = ("k", "t_arrive", "steps", "rng_seed", "n_lo", "n_hi", "n", "handle", "t_admit", "t_done",
                 "done", "fresh", "result", "params", "state")

    def __init__(self, k, t_arrive, steps, seed, n_lo, n_hi):
        self.k, self.t_arrive, self.steps, self.rng_seed = k, t_arrive, steps, seed
        self.n_lo, self.n_hi = n_lo, n_hi
        self.n = None
        self.handle = None
        self.t_admit = self.t_done = None
        self.done = 0
        self.fresh = True
        self.result = None
        self.params = None
        self.state = None

    def planned_n(self):
        """the request's particle count, drawn from its seed without building its state"""
        n_t, n_i, _, _, _ = ic.sweep_draw(np.random.default_rng(self.rng_seed), self.n_lo, self.n_hi)
        return n_t + n_i

    def initial_state(self):
        """the request's initial particles (the client's part: built once, kept until admission)"""
        if self.state is None:
            F, ids, mats, params = ic.sweep_impact(np.random.default_rng(self.rng_seed), self.n_lo, self.n_hi,
                                                   self.rng_seed)
            self.n, self.params = params["n"], params
            self.state = (F, ids, mats)
        return self.state


class Server:
    """Continuous batching of impact runs on one GPU (see the module docstring)."""

    # initial states built ahead of admission at most: under overload the backlog is kept as
    # arrival records and the client builds the next state once an admission frees a place
    BUILT_AHEAD = 32

    def __init__(self, precision="mixed", device=0, budget_bytes=None, max_runs=None, keep_results=False, ctx=None,
                 built_ahead=None):
        # ctx: a context of the lib.Context run interface (add_run, step, download_run, remove_run,
        # close); by default a new device context with the iron / dunite tables.  built_ahead:
        # initial states the client may hold built before admission (default BUILT_AHEAD)
        self.ctx = ctx if ctx is not None else make_context(precision, device)
        self.budget = budget_bytes if budget_bytes is not None else hbm_budget(device)
        self.max_particles = max(1, self.budget // BYTES_PER_PARTICLE)
        self.max_runs = max_runs
        self.keep_results = keep_results
        self.queue = collections.deque()
        self.active = {}
        self.resident = 0
        self.step_lat, self.ttc, self.completed = [], [], []
        self.particle_steps = 0
        self.steps_taken = 0
        self.stepping_s = 0.0   # wall time inside the batched steps (no admission, IC building or idling)
        self.admitted = 0
        self.built = threading.BoundedSemaphore(built_ahead or self.BUILT_AHEAD)

    def _fits(self, n_guess):
        if self.max_runs is not None and len(self.active) >= self.max_runs:
            return False
        return self.resident + n_guess <= self.max_particles or not self.active

    def admit(self, now):
        while self.queue and self._fits(self.queue[0].n_hi if self.queue[0].n is None else self.queue[0].n):
            r = self.queue.popleft()
            F, ids, mats = r.initial_state()
            if not self._fits(r.n):
                self.queue.appendleft(r)
                break
            r.handle = self.ctx.add_run(F, ids, mats)
            r.state = None
            r.t_admit = now
            self.admitted += 1
            self.built.release()
            self.active[r.handle] = r
            self.resident += r.n

    def step(self, now_fn):
        t0 = time.perf_counter()
        self.ctx.step(1)
        lat = time.perf_counter() - t0
        self.steps_taken += 1
        self.stepping_s += lat
        finished = []
        for h, r in self.active.items():
            if r.fresh:           # the run's prologue
                r.fresh = False
                continue
            r.done += 1
            self.step_lat.append(lat)
            self.particle_steps += r.n
            if r.done >= r.steps:
                finished.append(h)
        for h in finished:
            r = self.active.pop(h)
            out = self.ctx.download_run(h)
            self.ctx.remove_run(h)
            self.resident -= r.n
            r.t_done = now_fn()
            r.result = out if self.keep_results else None
            self.ttc.append(r.t_done - r.t_arrive)
            self.completed.append(r)

    def run(self, requests, duration=None, drain=True):
        """requests: arrival-ordered Request list (t_arrive in seconds from the start).  A client
        thread builds each request's initial state at its arrival time and hands it over, holding
        at most BUILT_AHEAD built states that wait for admission (a later arrival is built when
        an admission frees a place; its time to completion still counts from its arrival); the
        loop admits, steps and retires runs."""
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0
        arrived = queue.Queue()
        quit_ = threading.Event()
        self.window = duration
        self.requests = requests

        def client():
            for r in requests:
                while not quit_.is_set() and now() < r.t_arrive:
                    time.sleep(min(0.01, max(0.0, r.t_arrive - now())))
                if quit_.is_set() or (duration is not None and r.t_arrive > duration):
                    break
                while not quit_.is_set() and not self.built.acquire(timeout=0.05):
                    pass
                if quit_.is_set():
                    break
                r.initial_state()
                arrived.put(r)
            arrived.put(None)

        th = threading.Thread(target=client, daemon=True)
        th.start()
        client_done = False
        try:
            while True:
                while True:
                    try:
                        r = arrived.get_nowait()
                    except queue.Empty:
                        break
                    if r is None:
                        client_done = True
                    else:
                        self.queue.append(r)
                t = now()
                if duration is not None and t >= duration and not drain:
                    break
                self.admit(t)
                if not self.active:
                    if client_done and not self.queue:
                        break
                    time.sleep(0.005)
                    continue
                self.step(now)
        finally:
            quit_.set()
            th.join(timeout=5.0)
        wall = now()
        return self.report(wall)

    def report(self, wall):
        reqs = getattr(self, "requests", None) or []
        horizon = min(wall, self.window) if getattr(self, "window", None) is not None else wall
        arrived = sum(1 for r in reqs if r.t_arrive <= horizon)
        waiting = [r for r in reqs if r.t_arrive <= horizon and r.t_admit is None]
        return {
            "wall_s": wall,
            "arrived": arrived,
            "admitted": self.admitted,
            "completed": len(self.completed),
            "resident_at_end": len(self.active),
            "queued_at_end": len(waiting) if reqs else len(self.queue),
            "oldest_wait_at_end_s": max((wall - r.t_arrive for r in waiting), default=0.0),
            "batched_steps": self.steps_taken,
            "particle_steps": int(self.particle_steps),
            "particle_steps_per_s": self.particle_steps / wall if wall > 0 else 0.0,
            "stepping_s": self.stepping_s,
            "particle_steps_per_stepping_s": self.particle_steps / self.stepping_s if self.stepping_s > 0 else 0.0,
            "step_latency_s": percentiles(self.step_lat),
            "time_to_completion_s": percentiles(self.ttc),
            "max_resident_particles": int(self.max_particles),
        }

    def close(self):
        self.ctx.close()


def poisson_requests(seed, rate, duration, n_lo, n_hi, steps_lo, steps_hi):
    rng = np.random.default_rng(seed)
    out, t, k = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            return out
        out.append(Request(k, t, int(rng.integers(steps_lo, steps_hi + 1)), seed * 1_000_003 + k, n_lo, n_hi))
        k += 1


def sweep(n_runs=256, steps=100, seed=3, n_lo=5_000, n_hi=200_000, precision="mixed", device=0):
    """The batched sweep: n_runs impacts admitted at once (as far as they fit), each for `steps` steps."""
    reqs = [Request(k, 0.0, steps, seed * 100_003 + k, n_lo, n_hi) for k in range(n_runs)]
    srv = Server(precision, device, built_ahead=n_runs)
    try:
        rep = srv.run(reqs)
    finally:
        srv.close()
    rep.update({"runs": n_runs, "steps_per_run": steps,
                "particles": int(sum(r.n for r in reqs if r.n is not None))})
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    sub = ap.add_subparsers(dest="mode", required=True)
    a1 = sub.add_parser("sweep")
    a1.add_argument("--runs", type=int, default=256)
    a1.add_argument("--steps", type=int, default=100)
    a1.add_argument("--seed", type=int, default=3)
    a2 = sub.add_parser("serve")
    a2.add_argument("--duration", type=float, default=600.0, help="seconds of arrivals")
    a2.add_argument("--rate", type=float, default=2.0, help="requests per second")
    a2.add_argument("--seed", type=int, default=4)
    a2.add_argument("--n-lo", type=float, default=1e4)
    a2.add_argument("--n-hi", type=float, default=5e5)
    a2.add_argument("--steps-lo", type=int, default=200)
    a2.add_argument("--steps-hi", type=int, default=2000)
    a2.add_argument("--no-drain", action="store_true", help="stop at the end of the arrival window")
    for a in (a1, a2):
        a.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    a = ap.parse_args(argv)
    if a.mode == "sweep":
        print(json.dumps(sweep(a.runs, a.steps, a.seed, precision=a.precision)))
    else:
        reqs = poisson_requests(a.seed, a.rate, a.duration, a.n_lo, a.n_hi, a.steps_lo, a.steps_hi)
        srv = Server(a.precision)
        try:
            rep = srv.run(reqs, duration=a.duration, drain=not a.no_drain)
        finally:
            srv.close()
        rep.update({"requests": len(reqs), "rate_per_s": a.rate, "duration_s": a.duration})
        print(json.dumps(rep))


if __name__ == "__main__":
    main()
