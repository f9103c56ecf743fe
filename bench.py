#!/usr/bin/env python
"""Benchmark: SPH particle-steps/s on the 1M-particle impact (mixed
precision, with the plain FP64 path beside it), through the C ABI of
libsph_gb300.so.

Workload: two-layer iron-core / dunite-mantle bodies, 900k + 100k particles,
30 degrees at 1.2 v_esc, ANEOS-style synthetic 200 x 200 rho-u tables,
theta = 0.5.  One step = one iteration of main.cpp:125-173 (kick-drift-
predict, sort + octree, density x 4, EoS, derivative, hydro, tree gravity,
final kick, global dt).  Inputs (1M particles x 256 B of state plus lists)
are larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: the path does not shard within a run on this build (replicas
only), so N > 1 runs N independent replicas, one per rank, and reports the
aggregate.
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

import numpy as np

from fdps_sph_gb300.ic import FIELD

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic flops per pair interaction (adds, muls, compares 1; FMA 2;
# sqrt / div / rsqrt 1): density, derivative, hydro, gravity
FLOPS_PER_PAIR = {"dens": 24, "drvt": 75, "hydro": 120, "grav": 24}

# DRAM bytes (read + write) per launch per particle, from the ncu captures
# summarised in profiles/ (dram__bytes_read.sum + dram__bytes_write.sum of one
# launch divided by the particle count of that capture)
NCU_TRAFFIC = {}
_tf = os.path.join(ROOT, "profiles", "ncu_traffic_per_particle.txt")
if os.path.exists(_tf):
    for _ln in open(_tf):
        _p = _ln.split()
        if len(_p) >= 2 and not _ln.startswith("#"):
            NCU_TRAFFIC[_p[0]] = float(_p[1])


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="total particles (default: the 1M workload)")
    ap.add_argument("--cpu-n", type=int, default=0,
                    help="particles of the CPU baseline (default: the workload's own count)")
    ap.add_argument("--cpu-steps", type=int, default=5, help="timed steps of the cpu_baseline leg")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched sweep and the serving window")
    ap.add_argument("--config", default="1m", choices=["1m", "4m"], help="geometry of the workload (see workload())")
    ap.add_argument("--theta", type=float, default=0.5, help="gravity opening angle")
    ap.add_argument("--mode", type=int, default=1, choices=[1, 2],
                    help="2: every step ends with SetConstantEntropy + CalcAll (120 x 120 tables)")
    ap.add_argument("--tpi", type=int, default=0,
                    help="threads per particle of the derivative / hydro kernels instead of autotuning (1, 2, 4)")
    ap.add_argument("--batch-runs", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--serve-s", type=float, default=600.0, help="seconds of Poisson arrivals (2 per second)")
    ap.add_argument("--serve-steps", default="200,2000", help="steps per request, uniform in [lo, hi]")
    ap.add_argument("--no-4m", action="store_true", help="skip the 4M three-layer case at theta 0.5 / 0.7")
    ap.add_argument("--no-multiwalk", action="store_true",
                    help="skip the drop-in measurement through the MultiWalk dispatch / retrieve callbacks")
    ap.add_argument("--contact-steps", type=int, default=20,
                    help="mixed steps of the 1M contact state before its mixed-vs-FP64 comparison")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region: sampling is running
    (its first line read) before the region starts, and only the lines that arrive between the
    start and one interval after the end are summarised."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=20):
        self.gpu = gpu_index
        self.interval = interval_ms
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def _start(self, interval_ms):
        self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits", "-lms", str(interval_ms)],
                                     stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        deadline = time.perf_counter() + 5.0
        while not self.lines and self.proc.poll() is None and time.perf_counter() < deadline:
            time.sleep(0.005)
        return bool(self.lines)

    def __enter__(self):
        try:
            if not self._start(self.interval):   # an interval nvidia-smi refuses: its default-style one
                self.interval = 200
                self._start(self.interval)
        except Exception:
            self.proc = None
        self.t0 = time.perf_counter()
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.perf_counter(), ln.strip()))

    def __exit__(self, *a):
        self.t1 = time.perf_counter()
        if self.proc:
            time.sleep(1.5 * self.interval * 1e-3)   # the sample that closes the region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lim = (self.t1 or time.perf_counter()) + 1.5 * self.interval * 1e-3
        for t, ln in self.lines:
            if self.t0 is None or t < self.t0 or t > lim:
                continue
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "interval_ms": self.interval}


def workload(n_total, seed=2024, config="1m", mode=1):
    """1m: two-layer iron / dunite impact, 30 deg, 1.2 v_esc (the headline workload, at n_total);
    4m: three-layer iron / dunite / granite-crust impact, 45 deg, 1.0 v_esc.  Mode 2 reads the
    tables through the reference's 120-line slices, so it takes 120 x 120 tables (the size of the
    reference's own) reaching down to 1e-3 kg/m^3 instead of the 200 x 200 ones."""
    from fdps_sph_gb300 import eos, ic
    nt = int(round(n_total * 0.9))
    names = ("iron", "dunite", "granite") if config == "4m" else ("iron", "dunite")
    if mode == 2:
        materials = [eos.synthetic_table(m, 120, 120, rho_range=(1e-3, 3e4)) for m in names]
    else:
        materials = [eos.synthetic_table(m) for m in names]
    if config == "4m":
        F, ids, mats, info = ic.config_4m_impact(n_target=nt, n_impactor=n_total - nt)
    else:
        F, ids, mats, info = ic.config_1m_impact(seed=seed, n_target=nt, n_impactor=n_total - nt)
    return F, ids, mats, materials


# the headline metric (both arms print it; `batch` carries the batched sweep's p99 step latency)
METRIC = "SPH particle-steps/s at 1M (plain FP64 vs mixed, same error); batch p99 latency"


def workload_name(n, a):
    return (f"{n:,}-particle {WORKLOADS[a.config]}, theta {a.theta}" +
            (", mode 2 (constant entropy, 120 x 120 tables)" if a.mode == 2 else ""))


WORKLOADS = {"1m": "two-layer impact (90% target, 10% impactor, iron/dunite, 30 deg, 1.2 v_esc)",
             "4m": "three-layer impact (90% target, 10% impactor, iron/dunite/granite crust 5%, 45 deg, 1.0 v_esc)"}


def run_gpu(F, ids, mats, materials, precision, steps, warmup, device, theta=0.5, mode=1, dist=None):
    from fdps_sph_gb300 import lib
    ctx = lib.Context(precision=precision, device=device, theta=theta, mode=mode)
    for k, m in enumerate(materials):
        ctx.set_material(k, m)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    Fp, idp, _ = ctx.download()   # the forces of the initial state, for the mixed-vs-FP64 errors
    first = Fp[:, np.argsort(idp, kind="stable")]
    del Fp
    for _ in range(warmup):
        ctx.step(1)
    tune = None
    if precision == "mixed":   # launch shapes: tuned on this workload, or given
        if TPI:
            ctx.set_tune(TPI, TPI)
            tune = {"drvt_tpi": TPI, "hydro_tpi": TPI, "given": True}
        else:
            tune = ctx.autotune()
    # segment breakdown: event marks between the passes (launched directly, not as graphs)
    ctx.enable_timing(True)
    ctx.step_timed(steps)
    seg = ctx.timings()
    ctx.enable_timing(False)
    # the timed steps (the octree build replays as a CUDA graph); events around the steps only
    c0 = ctx.counters()["launches"]
    d0 = ctx.diagnostics()
    replica_barrier(dist)
    with ClockSampler(device) as clk:
        ms = ctx.step_timed(steps)
    d1 = ctx.diagnostics()
    c1 = ctx.counters()
    return ctx, ms, seg, c1, c1["launches"] - c0, clk.summary(), drift(d0, d1, steps), tune, first


def state_errors(a, device, materials, mixed, f64):
    """the mixed path's forces against the FP64 path's (held to the oracle by the parity tests) on
    three states of the workload, all particles, bar 1e-5:
      contact -- the bodies placed in contact and advanced a.contact_steps mixed steps, so the
                 contact region is shocked (artificial viscosity and du/dt active);
      warm    -- the state the mixed timed run reached (the prologue, the warm-up, timed and
                 end-to-end steps), bodies compressing under their own gravity;
      initial -- the prologue of the initial state (rigid bodies: du/dt is zero in both paths).
    The top-level numbers are the contact state's."""
    from fdps_sph_gb300 import accuracy, ic, lib
    res = {}
    if a.config == "1m" and a.mode == 1:
        n = a.n
        nt = int(round(n * 0.9))
        F, ids, mats, _ = ic.config_1m_contact(n_target=nt, n_impactor=n - nt)
        ctx = lib.Context(precision="mixed", device=device, theta=a.theta)
        try:
            for k, m in enumerate(materials):
                ctx.set_material(k, m)
            ctx.upload(F, ids, mats)
            ctx.prologue()
            ctx.step(a.contact_steps)
            t_c, _, _ = ctx.time()
            S, sid, smat = ctx.download()
        finally:
            ctx.close()
        e = accuracy.compare_on_state(S, sid, smat, materials, a.theta, device, t_c)
        # the hydro error split between the density (through P) and the pair arithmetic
        e["hydro_error_sources"] = accuracy.hydro_error_sources(S, sid, smat, materials, a.theta, device, t_c)
        e["state"] = (f"{n:,} particles placed in contact (centres 0.98 (R_t + R_i) apart, contact velocity of the "
                      f"30 deg / 1.2 v_esc orbit), after the prologue and {a.contact_steps} mixed steps")
        res["contact"] = e
        del S
    S, sid, smat, t_w, step_w = mixed["state"]
    e = accuracy.compare_on_state(S, sid, smat, materials, a.theta, device, t_w)
    e["state"] = (f"the state the mixed run reached after the prologue and about {step_w} steps (warm-up, "
                  f"segment-timed, timed and end-to-end steps): bodies compressing under their own gravity")
    res["warm"] = e
    mixed.pop("state")
    e = accuracy.force_errors(mixed["first"], f64["first"])
    e["activity"] = accuracy.activity(f64["first"])
    e["distribution"] = accuracy.error_distribution(mixed["first"], f64["first"])
    e["state"] = "the initial state's prologue (rigid bodies 4 R_t apart: no approaching pairs, du/dt = 0)"
    res["initial"] = e
    top = res.get("contact", res["warm"])
    out = {k: v for k, v in top.items() if k not in ("activity", "distribution")}
    out.update(res)
    out["bar"] = 1e-5
    out["note"] = ("per-quantity max over particles: density and potential relative, vectors and du/dt "
                   "relative with the RMS over particles as floor; the FP64 path is held to the oracle by the "
                   "parity tests; top-level values are the contact state's")
    return out


def config_4m(device, thetas=(0.5, 0.7), warmup=3, steps=5):
    """The 4M three-layer impact (3.6M + 0.4M iron / dunite / granite-crust bodies, 45 deg, 1.0 v_esc)
    at each opening angle: the mixed path timed (CUDA events, `steps` steps after the prologue and
    `warmup` steps), an FP64 rerun of the same steps from the same initial state, the energy and
    angular-momentum drift of both, the mixed path's force errors against FP64 on the state the
    mixed run reached, and how far the two runs' positions have moved apart (in units of h)."""
    from fdps_sph_gb300 import accuracy
    F, ids, mats, materials = workload(4_000_000, config="4m")
    n = F.shape[1]
    out = {"workload": workload_name(n, argparse.Namespace(config="4m", theta=0.5, mode=1)).rsplit(", theta", 1)[0],
           "particles": n, "steps": steps, "warmup": warmup}
    for theta in thetas:
        row = {}
        for prec in ("mixed", "fp64"):
            from fdps_sph_gb300 import lib
            ctx = lib.Context(precision=prec, device=device, theta=theta)
            try:
                for k, m in enumerate(materials):
                    ctx.set_material(k, m)
                ctx.upload(F, ids, mats)
                ctx.prologue()
                ctx.step(warmup)
                d0 = ctx.diagnostics()
                with ClockSampler(device) as clk:
                    ms = ctx.step_timed(steps)
                d1 = ctx.diagnostics()
                t_s, _, step_s = ctx.time()
                S, sid, smat = ctx.download()
            finally:
                ctx.close()
            row[prec] = {"ms_per_step": ms / steps, "value": n * steps / (ms * 1e-3), "drift": drift(d0, d1, steps),
                         "clocks": clk.summary()}
            row[prec + "_state"] = (accuracy.by_id(S, sid), np.sort(sid), smat[np.argsort(sid, kind="stable")],
                                    t_s, step_s)
            del S
        Sm, sid, smat, t_s, step_s = row.pop("mixed_state")
        Sf = row.pop("fp64_state")[0]
        e = accuracy.compare_on_state(Sm, sid, smat, materials, theta, device, t_s)
        e["state"] = f"the mixed run's state after step {step_s}"
        row["mixed_error_vs_fp64"] = e
        dx = np.linalg.norm(np.stack([Sm[FIELD[c]] - Sf[FIELD[c]] for c in "xyz"], 1), axis=1)
        row["divergence_max_dx_over_h"] = float(np.max(dx / Sf[FIELD["smth"]]))
        row["speedup_mixed_over_fp64"] = row["fp64"]["ms_per_step"] / row["mixed"]["ms_per_step"]
        out[f"theta_{theta}"] = row
        del Sm, Sf
    return out


def drift(d0, d1, steps):
    """relative change per step of the total energy and the angular momentum over the timed steps
    (sph_diagnostics: E = sum m (u + v^2/2 + pot/2), L = sum m x cross v, both in FP64)"""
    import numpy as np
    e = abs(d1[0] - d0[0]) / max(abs(d0[0]), 1e-300) / steps
    lv = float(np.linalg.norm(d1[4:7] - d0[4:7]) / max(np.linalg.norm(d0[4:7]), 1e-300)) / steps
    return {"energy_rel_per_step": e, "angmom_rel_per_step": lv}


def run_e2e(ctx, F, ids, mats, steps, warmup=2, dist=None):
    """upload (pinned host) -> one step -> download (pinned host), every step.  The upload copies
    the fields the step reads or carries (SPH_UPLOAD_STEP_INPUTS); every field the step writes
    (SPH_STEP_OUTPUT_FIELDS) goes back into the host's block as soon as the step has written it
    (sph_step_download, the copies overlapping the rest of the step); the block's other rows
    (mass, AVa, entropy, temperature; ids and materials, in upload order) the step leaves
    unchanged.
    `warmup` round trips run untimed first (the first ones capture the CUDA graphs of the new
    buffer layout)."""
    import torch
    from fdps_sph_gb300 import lib
    n = F.shape[1]
    hostF = torch.empty((F.shape[0], n), dtype=torch.float64).pin_memory().numpy()
    hid = torch.empty(n, dtype=torch.int64).pin_memory().numpy()
    hmat = torch.empty(n, dtype=torch.int32).pin_memory().numpy()
    # start from the context's current state (forces valid)
    Fc, idc, matc = ctx.download()
    hostF[:] = Fc
    hid[:] = idc
    hmat[:] = matc
    outs = lib.STEP_OUTPUT_FIELDS + (["ent", "temp"] if ctx.cfg.mode == 2 else [])
    t_now, dt, _ = ctx.time()

    def round_trip():
        nonlocal t_now, dt
        ctx.upload(hostF, hid, hmat, time=t_now, dt=dt, forces_valid=True, inputs_only=True)
        ctx.step_download(hostF, outs)   # each field to the host as soon as the step has written it
        t_now, dt, _ = ctx.time()

    for _ in range(warmup):
        round_trip()
    replica_barrier(dist)
    t0 = time.perf_counter()
    for _ in range(steps):
        round_trip()
    el = time.perf_counter() - t0
    h2d = 8 * n * len(lib.STEP_INPUT_FIELDS) + hid.nbytes + hmat.nbytes
    d2h = 8 * n * len(outs)
    return el, h2d, d2h


def cpu_sample(n_cpu, steps, fast=True, config="1m", mode=1):
    """the oracle restatement of the path (OpenMP, all host threads) on the
    workload at n_cpu particles (the GPU's own when n_cpu is its count):
    prologue untimed, `steps` timed"""
    from oracle import pyoracle as po
    F, ids, mats, materials = workload(n_cpu, config=config, mode=mode)
    ms = po.MaterialSet([m.as_material() for m in materials])
    cfg = po.make_config(ms)
    s = po.OracleSystem(F, ids, mats, fast=fast)
    s.prologue(cfg)
    t0 = time.perf_counter()
    s.step(cfg, steps)
    el = time.perf_counter() - t0
    return n_cpu * steps / el, el, po.lib(fast).or_num_threads()


def dist_init(n_gpus):
    if n_gpus <= 1 and "WORLD_SIZE" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", n_gpus))
    local = int(os.environ.get("LOCAL_RANK", rank))
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, dist


def replica_barrier(dist):
    """every replica enters its timed steps together (a no-op for one process)"""
    if dist is not None:
        dist.barrier()


def replica_max(x, dist, device=None):
    """the slowest replica's time: the job ends when the last replica does (x for one process)"""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_throughput(world, n, ms_per_step):
    """whole-job particle-steps/s: every replica advances its own n particles per step"""
    return world * n / (ms_per_step * 1e-3)


TPI = 0


def main():
    global TPI
    a = parse()
    TPI = a.tpi
    rank, world, dist = dist_init(a.gpus)
    if a.impl == "reference":
        if rank != 0:
            return
        # the reference's CPU path on this host: the oracle restatement (the reference itself
        # needs FDPS, which is not vendored, so it cannot be built here); all host threads, on the
        # GPU arm's own workload (the same particles, the same steps)
        n_cpu = a.cpu_n or a.n
        from oracle import pyoracle as po
        F, ids, mats, materials = workload(n_cpu, config=a.config, mode=a.mode)
        ms = po.MaterialSet([m.as_material() for m in materials])
        cfg = po.make_config(ms)
        s = po.OracleSystem(F, ids, mats, fast=True)
        s.prologue(cfg)
        if a.warmup:
            s.step(cfg, a.warmup)
        t0 = time.perf_counter()
        s.step(cfg, a.steps)
        el = time.perf_counter() - t0
        v = n_cpu * a.steps / el
        cores = po.lib(True).or_num_threads()
        out = {"metric": METRIC,
               "value": v, "unit": "particle-steps/s", "impl": "reference", "n_gpus": a.gpus, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": 1e3 * el / a.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded IC generator)",
               "config": {"workload": workload_name(a.n, a), "particles": a.n, "precision": "fp64",
                          "sample": (f"the workload itself ({n_cpu} particles), every step" if n_cpu == a.n else
                                     f"{n_cpu} particles of the same geometry per step (bounded CPU sample)"),
                          "parallelism": f"OpenMP x{cores} (host cores)"},
               "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                                "sample": f"{n_cpu} particles, {a.steps} steps after the prologue and "
                                          f"{a.warmup} warm-up steps"},
               "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    from fdps_sph_gb300 import lib
    import torch
    device = int(os.environ.get("LOCAL_RANK", 0))
    F, ids, mats, materials = workload(a.n, config=a.config, mode=a.mode)
    n = F.shape[1]

    results = {}
    precisions = ["mixed"] if a.no_fp64 else ["mixed", "fp64"]
    for prec in precisions:
        ctx, ms, seg, cnt, launches, clocks, dr, tune, first = run_gpu(F, ids, mats, materials, prec, a.steps,
                                                                       a.warmup, device, a.theta, a.mode,
                                                                       dist if prec == "mixed" else None)
        e2e = run_e2e(ctx, F, ids, mats, a.e2e_steps, dist=dist) if prec == "mixed" else None
        results[prec] = dict(ms=ms, seg=seg, cnt=cnt, launches=launches, clocks=clocks, e2e=e2e, drift=dr, tune=tune,
                             first=first)
        if prec == "mixed" and not a.no_fp64:   # the state the timed steps reached, for the warm comparison
            t_now, _, _ = ctx.time()
            n_steps = a.warmup + 2 * a.steps + 2 + a.e2e_steps   # warm-up, segment-timed, timed, end to end
            results[prec]["state"] = ctx.download() + (t_now, n_steps)
        ctx.close()

    results["mixed"]["ms"] = replica_max(results["mixed"]["ms"], dist, f"cuda:{device}")
    if results["mixed"]["e2e"] is not None:
        el, h2d, d2h = results["mixed"]["e2e"]
        results["mixed"]["e2e"] = (replica_max(el, dist, f"cuda:{device}"), h2d, d2h)
    if rank != 0:
        return

    peak32 = lib.probe_peak(False, device)
    peak64 = lib.probe_peak(True, device)
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        peaks = {"hbm_gbs": 6800.0}   # the profiling recipe's fallback
    mixed = results["mixed"]
    ms_step = mixed["ms"] / a.steps
    value = replica_throughput(world, n, ms_step)

    # algorithmic work of each segment of one step: flops on the FP32 pipe
    # for the pair kernels, compulsory HBM bytes for the list / tree / streaming kernels
    w = mixed["cnt"]
    seg, st = mixed["seg"], a.steps
    entries = w.get("superset_entries", 0)
    kernels = {
        "sup_walk": ("dens_list", "hbm", 12 * entries + 68 * n, 1),         # rows (idx, r2, m) + particle reads
        "density": ("dens", "fp32", FLOPS_PER_PAIR["dens"] * w["pairs_gather"], 4),
        # one pass: superset (idx, r2) read once, gather and symmetric lists written
        "filters": (None, "hbm", 8 * entries + 4 * (w["pairs_gather"] + w["pairs_sym"]), 1),
        "derivative": ("drvt", "fp32", FLOPS_PER_PAIR["drvt"] * w["pairs_gather"], 1),
        "hydro": ("hydro", "fp32", FLOPS_PER_PAIR["hydro"] * w["pairs_sym"], 1),
        "grav_groups": ("grav_list", "hbm", 16 * w["cells"], 1),            # count / parent / flag per cell
        "gravity": ("grav", "fp32", FLOPS_PER_PAIR["grav"] * w["pairs_grav"], 1),   # walk fused in
        "sort_tree": ("sort_tree", "hbm", (36 + 8 * 24 + 2 * 32 * 8) * n, 1),
    }
    filt_ms = seg["drvt_list"] + seg["hydro_list"]
    seg = dict(seg, sort_tree=seg["sort"] + seg["tree"] + seg["nbr_prep"])
    hbm = peaks.get("hbm_gbs")
    rows = {}
    for name, (sname, bound, work, launches_per_step) in kernels.items():
        seg_ms_step = filt_ms / st if name == "filters" else seg[sname] / st
        per_launch_ms = seg_ms_step / launches_per_step
        if per_launch_ms <= 0:
            continue
        if bound == "fp32":
            ach = work / (per_launch_ms * 1e-3) / 1e12
            rows[name] = {"bound": "fp32", "achieved": ach, "peak": peak32, "unit": "TFLOP/s",
                          "frac": ach / peak32, "work_per_launch": work, "ms_per_launch": per_launch_ms}
        else:
            ach = work / (per_launch_ms * 1e-3) / 1e9
            rows[name] = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                          "frac": ach / hbm if hbm else None, "work_per_launch": work, "ms_per_launch": per_launch_ms}
    dom = max(rows, key=lambda k: rows[k]["ms_per_launch"] * kernels[k][3])
    traffic = NCU_TRAFFIC.get(dom)
    seg_share = {k: round(v / max(sum(seg.values()), 1e-9), 4) for k, v in seg.items()}
    roof = dict(rows[dom])
    roof.update({"kernel": dom, "traffic": traffic * n if traffic else None,
                 "peak_source": ("MEASURED_PEAKS.json hbm_gbs (copy bandwidth)" if roof["bound"] == "hbm" else
                                 "measured FMA-chain probe (sph_probe_peak); MEASURED_PEAKS.json has no FP32 figure")})

    out = {
        "metric": METRIC,
        "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 pair sums + f64", "data": "synthetic (seeded IC generator, synthetic " + ("120x120" if a.mode == 2 else "200x200") + " rho-u tables)",
        "config": {"workload": workload_name(n, a), "particles": n,
                   "precision": "mixed",
                   "l2": "inputs larger than L2 (no flush)", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "gpu_launches": int(mixed["launches"]),
        "clocks": mixed["clocks"],
        "roofline": roof,
        "rooflines": rows,
        "segments_ms_per_step": {k: v / a.steps for k, v in mixed["seg"].items()},
        "segment_share": seg_share,
        "work": {k: v for k, v in mixed["cnt"].items() if k != "launches"},
        "peaks": {"fp32_tflops_measured": peak32, "fp64_tflops_measured": peak64, "hbm_gbs": hbm},
    }
    out["autotune"] = mixed["tune"]
    out["drift"] = {"mixed": mixed["drift"], "steps": a.steps,
                    "note": "relative change per timed step of E and |L| (FP64 diagnostics)"}
    if mixed["e2e"] is not None:
        el, h2d, d2h = mixed["e2e"]
        out["e2e"] = {"value": world * n * a.e2e_steps / el, "unit": "particle-steps/s",
                      "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": a.e2e_steps}
    if "fp64" in results:
        f = results["fp64"]
        v64 = world * n / (f["ms"] / a.steps * 1e-3)
        dom64 = max(("dens", "drvt", "hydro", "grav"), key=lambda k: f["seg"][k])
        p64 = {"dens": f["cnt"]["pairs_gather"], "drvt": f["cnt"]["pairs_gather"], "hydro": f["cnt"]["pairs_sym"],
               "grav": f["cnt"]["pairs_grav"]}[dom64]
        pl64 = f["seg"][dom64] / (a.steps * (4 if dom64 == "dens" else 1))
        ach64 = FLOPS_PER_PAIR[dom64] * p64 / (pl64 * 1e-3) / 1e12
        out["fp64"] = {"value": v64, "ms_per_step": f["ms"] / a.steps, "speedup_mixed_over_fp64": value / v64,
                       "segments_ms_per_step": {k: v / a.steps for k, v in f["seg"].items()},
                       "roofline": {"bound": "fp64", "kernel": dom64, "achieved": ach64, "peak": peak64,
                                    "unit": "TFLOP/s", "frac": ach64 / peak64 if peak64 else None},
                       "clocks": f["clocks"], "gpu_launches": int(f["launches"])}
        out["drift"]["fp64"] = f["drift"]
    # the MultiWalk boundary first, in a process that has not yet held the larger workloads (the
    # device gather of the payload form reads the callers' pageable arrays, and measured slower
    # after them)
    if not a.no_multiwalk and world == 1 and a.config == "1m" and a.mode == 1:
        out["multiwalk"] = multiwalk(a, device)
    if "fp64" in results:
        out["mixed_error_vs_fp64"] = state_errors(a, device, materials, mixed, results["fp64"])
    if not a.no_4m and world == 1 and a.config == "1m" and a.mode == 1:
        out["config_4m"] = config_4m(device)
    if not a.no_batch and world == 1:
        out.update(batch_and_serving(a, device))
    if not a.no_cpu:
        n_cpu = a.cpu_n or n
        v_cpu, el_cpu, cores = cpu_sample(n_cpu, a.cpu_steps, config=a.config, mode=a.mode)
        out["cpu_baseline"] = {"value": v_cpu, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                               "sample": f"oracle restatement (OpenMP) on the same workload ({n_cpu} particles), "
                                         f"{a.cpu_steps} steps after the prologue ({el_cpu:.1f} s on {cores} threads)"}
        for k in ("batch", "serving", "multiwalk"):
            if k in out:
                out[k]["vs_cpu_baseline"] = out[k]["value"] / v_cpu
        if "multiwalk" in out:
            out["multiwalk"]["index_form"]["vs_cpu_baseline"] = out["multiwalk"]["index_form"]["value"] / v_cpu
    print(json.dumps(out))


def multiwalk(a, device, n_walk_limit=256, n_tags=4, steps=2):
    """The drop-in boundary the way a host that keeps FDPS drives it: the functor calls of one step
    (density x 4, derivative, hydro, gravity) on the walks of every gravity group of the workload's
    prologue state, through sph_dispatch_* / sph_retrieve_* (batches of n_walk_limit walks over
    n_tags tags, class.h payloads staged by the library; the functor kernels in mixed precision for
    the line's value, in FP64 for its "fp64" entry).  The walks are built first (FDPS-style supersets, fdps_sph_gb300.walks), outside the timing."""
    from fdps_sph_gb300 import lib, walks
    F, ids, mats, materials = workload(a.n, config=a.config, mode=a.mode)
    n = F.shape[1]
    ctx = lib.Context(precision="fp64", device=device, theta=a.theta)
    try:
        for k, m in enumerate(materials):
            ctx.set_material(k, m)
        ctx.upload(F, ids, mats)
        ctx.prologue()
        t0 = time.perf_counter()
        W = walks.Walks(ctx)
        build_s = time.perf_counter() - t0
    finally:
        ctx.close()
    del F
    W.step(n_walk_limit=n_walk_limit, n_tags=n_tags)   # warm-up: the tags' streams and staging
    runs = [W.step(n_walk_limit=n_walk_limit, n_tags=n_tags) for _ in range(steps)]
    best = min(runs, key=lambda r: sum(r.values()))
    t_step = sum(best.values())
    lib.batch_precision("mixed")   # the same walks with the mixed-precision functor kernels
    try:
        W.step(n_walk_limit=n_walk_limit, n_tags=n_tags)
        runs32 = [W.step(n_walk_limit=n_walk_limit, n_tags=n_tags) for _ in range(steps)]
        # the index form: each pass's EPJ / SPJ arrays sent once, the walks as indices into them
        W.step(n_walk_limit=n_walk_limit, n_tags=n_tags, index=True)
        runs_ix = [W.step(n_walk_limit=n_walk_limit, n_tags=n_tags, index=True) for _ in range(steps)]
        lib.batch_staging("host")   # the walks copied by the host into pinned staging instead
        W.step(n_walk_limit=n_walk_limit, n_tags=n_tags)
        runs_h = [W.step(n_walk_limit=n_walk_limit, n_tags=n_tags) for _ in range(steps)]
    finally:
        lib.batch_precision("fp64")
        lib.batch_staging("auto")
    best32 = min(runs32, key=lambda r: sum(r.values()))
    t32 = sum(best32.values())
    t_h = min(sum(r.values()) for r in runs_h)
    best_ix = min(runs_ix, key=lambda r: sum(r.values()))
    t_ix = sum(best_ix.values())
    index_bytes = 4 * W.index_bytes["dens"] + sum(W.index_bytes[k] for k in ("drvt", "hydro", "grav"))
    staged = 4 * W.staged_bytes["dens"] + sum(W.staged_bytes[k] for k in ("drvt", "hydro", "grav"))
    jl = {k: int(len(W.jlist[k][0])) for k in ("dens", "hydro", "grav")}
    return {"metric": "particle-steps/s through the MultiWalk dispatch / retrieve callbacks",
            "value": n / t32, "unit": "particle-steps/s", "precision": "mixed (sph_batch_set_precision)",
            "s_per_step": t32, "s_per_pass": {k: v for k, v in best32.items()},
            "staging": "auto (sph_batch_set_staging: the GPU gathers the walks from host memory where it "
                       "can read pageable memory)",
            "host_staging": {"value": n / t_h, "s_per_step": t_h},
            "index_form": {"value": n / t_ix, "s_per_step": t_ix, "s_per_pass": {k: v for k, v in best_ix.items()},
                           "bytes_per_step": int(index_bytes),
                           "note": "the dispatch callbacks of calcForceAllAndWriteBackMultiWalkIndex "
                                   "(sph_dispatch_index_*): each pass's EPJ / SPJ arrays sent once with "
                                   "send_flag, the walks as int32 indices; mixed precision, same results"},
            "fp64": {"value": n / t_step, "s_per_step": t_step, "s_per_pass": {k: v for k, v in best.items()}},
            "groups": int(W.n_group),
            "n_walk_limit": n_walk_limit, "tags": n_tags, "staged_bytes_per_step": int(staged),
            "j_entries": {"gather": jl["dens"], "symmetric": jl["hydro"], "grav_epj": jl["grav"],
                          "grav_spj": int(len(W.spj[0]))},
            "walk_build_s": build_s,
            "config": f"{n:,}-particle workload after its prologue; i-groups = the octree's gravity groups "
                      "(<= 256 particles); gravity lists from the device tree (theta " + str(a.theta) + "), SPH "
                      "j-lists = FDPS-style group supersets; one step = the functor calls of main.cpp:136-147; "
                      "payloads staged from host memory by the library and results written back to host "
                      "memory inside the timing; the functor kernels in mixed precision (value) and in FP64 (fp64)"}


def batch_and_serving(a, device):
    """the batched sweep (256 impacts of uneven size, 100 steps each, one context) and the serving
    loop (Poisson arrivals at 2 per second, continuous batching), both mixed precision"""
    from fdps_sph_gb300 import ic, serve
    res = {}
    bt = serve.sweep(a.batch_runs, a.batch_steps, device=device)
    res["batch"] = {"metric": "aggregate particle-steps/s, batched sweep", "value": bt["particle_steps_per_s"],
                    "unit": "particle-steps/s", "runs": bt["runs"], "steps_per_run": bt["steps_per_run"],
                    "particles": bt["particles"], "batched_steps": bt["batched_steps"], "wall_s": bt["wall_s"],
                    "stepping_s": bt["stepping_s"], "value_stepping_only": bt["particle_steps_per_stepping_s"],
                    "step_latency_s": bt["step_latency_s"], "time_to_completion_s": bt["time_to_completion_s"],
                    "config": "impacts with N log-uniform 5e3-2e5, mass ratio U[0.05, 0.5], angle U[0, 75] deg, "
                              "speed U[1, 2] v_esc, iron/dunite tables; wall time includes the host IC generation"}
    # the serving configuration as specified: Poisson arrivals at 2 per second for a.serve_s seconds,
    # N log-uniform 1e4-5e5, steps uniform in [lo, hi]; the window ends the measurement
    lo, hi = (int(x) for x in a.serve_steps.split(","))
    reqs = serve.poisson_requests(4, 2.0, a.serve_s, 1e4, 5e5, lo, hi)
    srv = serve.Server("mixed", device)
    try:
        with ClockSampler(device, interval_ms=1000) as clk:
            rep = srv.run(reqs, duration=a.serve_s, drain=False)
    finally:
        srv.close()
    offered = sum(r.steps * r.planned_n() for r in reqs)
    # the plain FP64 per-run path on a request-sized impact (100k particles), alone
    F, ids, mats, _ = ic.sweep_impact(np.random.default_rng(5), 1e5, 1e5 + 1, 5)
    ctx = serve.make_context("fp64", device)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    ms = ctx.step_timed(3)
    ctx.close()
    v64 = F.shape[1] * 3 / (ms * 1e-3)
    res["serving"] = {"metric": "aggregate particle-steps/s, serving loop", "value": rep["particle_steps_per_s"],
                      "unit": "particle-steps/s", "requests_arrived": rep["arrived"], "admitted": rep["admitted"],
                      "completed": rep["completed"], "resident_at_end": rep["resident_at_end"],
                      "queued_at_end": rep["queued_at_end"], "oldest_wait_at_end_s": rep["oldest_wait_at_end_s"],
                      "window_s": a.serve_s, "steps_per_request": [lo, hi], "batched_steps": rep["batched_steps"],
                      "step_latency_s": rep["step_latency_s"], "time_to_completion_s": rep["time_to_completion_s"],
                      "max_resident_particles": rep["max_resident_particles"],
                      "stepping_s": rep["stepping_s"], "value_stepping_only": rep["particle_steps_per_stepping_s"],
                      "offered_particle_steps": int(offered),
                      "offered_particle_steps_per_s": offered / a.serve_s,
                      "fp64_per_run_value": v64, "vs_fp64_per_run": rep["particle_steps_per_s"] / v64,
                      "clocks": clk.summary(),
                      "config": f"Poisson arrivals at 2/s for {a.serve_s:g} s; N log-uniform 1e4-5e5; {lo}-{hi} "
                                "steps per request; parameters as the sweep; initial states built by a client thread "
                                "at arrival (at most 32 built ahead of admission); admission by HBM footprint, state "
                                "resident, backfill as runs finish; the window ends the measurement (runs still "
                                "resident or queued are counted, not drained); time to completion over the "
                                "completed requests"}
    return res


if __name__ == "__main__":
    main()
