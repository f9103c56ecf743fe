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
    ap.add_argument("--cpu-n", type=int, default=100_000, help="particles of the bounded CPU sample")
    ap.add_argument("--cpu-steps", type=int, default=10, help="timed steps of the bounded CPU sample")
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
    ap.add_argument("--serve-s", type=float, default=60.0, help="seconds of Poisson arrivals (2 per second)")
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
    first = Fp[:, np.argsort(idp, kind="stable")][[FIELD[k] for k in ERR_FIELDS]].copy()
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


ERR_FIELDS = ("dens", "ax", "ay", "az", "eng_dot", "gx", "gy", "gz", "pot")


def mixed_errors(mx, f64):
    """per-quantity error of the mixed path's initial forces against the FP64 path's (pinned to
    the oracle by the parity tests): density relative per particle; vectors and du/dt relative
    per particle, floored at the RMS over particles"""
    ix = {k: i for i, k in enumerate(ERR_FIELDS)}

    def vec(X, keys):
        return np.stack([X[ix[k]] for k in keys], 1)

    def vrms(A, B):
        nb = np.linalg.norm(B, axis=1)
        rms = max(float(np.sqrt(np.mean(nb * nb))), 1e-300)
        return float(np.max(np.linalg.norm(A - B, axis=1) / np.maximum(nb, rms)))

    def srms(a, b):   # du/dt is zero in both paths while the bodies move rigidly: then 0
        rms = max(float(np.sqrt(np.mean(b * b))), 1e-300)
        return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), rms)))

    return {"dens": float(np.max(np.abs(mx[0] - f64[0]) / np.abs(f64[0]))),
            "acc_hydro": vrms(vec(mx, ("ax", "ay", "az")), vec(f64, ("ax", "ay", "az"))),
            "eng_dot": srms(mx[ix["eng_dot"]], f64[ix["eng_dot"]]),
            "acc_grav": vrms(vec(mx, ("gx", "gy", "gz")), vec(f64, ("gx", "gy", "gz"))),
            "pot": float(np.max(np.abs(mx[ix["pot"]] - f64[ix["pot"]]) / np.abs(f64[ix["pot"]]))),
            "acc_total": vrms(vec(mx, ("ax", "ay", "az")) + vec(mx, ("gx", "gy", "gz")),
                              vec(f64, ("ax", "ay", "az")) + vec(f64, ("gx", "gy", "gz")))}


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


def cpu_sample(n_cpu, steps, fast=True):
    """the oracle restatement of the path (OpenMP, all host threads) on the
    same body geometry at n_cpu particles: prologue untimed, `steps` timed"""
    from oracle import pyoracle as po
    F, ids, mats, materials = workload(n_cpu, seed=77)
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
        # needs FDPS, which is not vendored, so it cannot be built here); all host threads
        n_cpu = a.cpu_n
        from oracle import pyoracle as po
        F, ids, mats, materials = workload(n_cpu, seed=77)
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
                          "sample": f"{n_cpu} particles of the same geometry per step (bounded CPU sample)",
                          "parallelism": f"OpenMP x{cores} (host cores)"},
               "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                                "sample": f"{n_cpu} particles, {a.steps} steps after {a.warmup} warm-up steps"},
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
        out["mixed_error_vs_fp64"] = dict(mixed_errors(mixed["first"], f["first"]),
                                          note="forces of the initial state (prologue), all particles; the FP64 "
                                               "path is held to the oracle by the parity tests; bar 1e-5")
    if not a.no_batch and world == 1:
        out.update(batch_and_serving(a, device))
    if not a.no_cpu:
        v_cpu, el_cpu, cores = cpu_sample(a.cpu_n, a.cpu_steps)
        out["cpu_baseline"] = {"value": v_cpu, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                               "sample": f"oracle restatement (OpenMP) on the same geometry at {a.cpu_n} particles, "
                                         f"{a.cpu_steps} steps after the prologue ({el_cpu:.1f} s on {cores} threads)"}
        for k in ("batch", "serving"):
            if k in out:
                out[k]["vs_cpu_baseline"] = out[k]["value"] / v_cpu
    print(json.dumps(out))


def batch_and_serving(a, device):
    """the batched sweep (256 impacts of uneven size, 100 steps each, one context) and a window of
    the serving loop (Poisson arrivals at 2 per second, continuous batching), both mixed precision"""
    from fdps_sph_gb300 import ic, serve
    res = {}
    bt = serve.sweep(a.batch_runs, a.batch_steps, device=device)
    res["batch"] = {"metric": "aggregate particle-steps/s, batched sweep", "value": bt["particle_steps_per_s"],
                    "unit": "particle-steps/s", "runs": bt["runs"], "steps_per_run": bt["steps_per_run"],
                    "particles": bt["particles"], "batched_steps": bt["batched_steps"], "wall_s": bt["wall_s"],
                    "step_latency_s": bt["step_latency_s"], "time_to_completion_s": bt["time_to_completion_s"],
                    "config": "impacts with N log-uniform 5e3-2e5, mass ratio U[0.05, 0.5], angle U[0, 75] deg, "
                              "speed U[1, 2] v_esc, iron/dunite tables; wall time includes the host IC generation"}
    # steps per request scaled by 1/10 (20-200) so that requests complete inside the short window;
    # `python -m fdps_sph_gb300.serve serve --duration 600` runs the unscaled stream
    reqs = serve.poisson_requests(4, 2.0, a.serve_s, 1e4, 5e5, 20, 200)
    srv = serve.Server("mixed", device)
    try:
        rep = srv.run(reqs, duration=a.serve_s, drain=False)
    finally:
        srv.close()
    # the plain FP64 per-run path on a request-sized impact (100k particles), alone
    F, ids, mats, _ = ic.sweep_impact(np.random.default_rng(5), 1e5, 1e5 + 1, 5)
    ctx = serve.make_context("fp64", device)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    ms = ctx.step_timed(3)
    ctx.close()
    v64 = F.shape[1] * 3 / (ms * 1e-3)
    res["serving"] = {"metric": "aggregate particle-steps/s, serving loop", "value": rep["particle_steps_per_s"],
                      "unit": "particle-steps/s", "requests_arrived": len(reqs), "completed": rep["completed"],
                      "resident_at_end": rep["resident_at_end"], "queued_at_end": rep["queued_at_end"],
                      "window_s": a.serve_s, "step_latency_s": rep["step_latency_s"],
                      "time_to_completion_s": rep["time_to_completion_s"],
                      "fp64_per_run_value": v64, "vs_fp64_per_run": rep["particle_steps_per_s"] / v64,
                      "config": "Poisson arrivals at 2/s; N log-uniform 1e4-5e5; 20-200 steps per request (the "
                                "serving configuration's 200-2000 scaled by 1/10 to fit the window); parameters as "
                                "the sweep; initial states built by a client thread at arrival; admission by HBM "
                                "footprint, state resident, backfill as runs finish; the window ends the "
                                "measurement (runs still resident are not drained)"}
    return res


if __name__ == "__main__":
    main()
