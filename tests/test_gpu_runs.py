"""Several runs in one context (the batched path): each run's state after
any sequence of steps is bit-identical to the same run advanced alone, in
both precisions, including runs removed and runs added between steps."""
import numpy as np
import pytest

from helpers import device_context, small_impact, tillotson_materials

pytestmark = pytest.mark.gpu


def _bodies():
    return [small_impact(n_target=nt, n_impactor=ni, seed=sd)[:3]
            for nt, ni, sd in ((1500, 150, 21), (700, 120, 22), (2400, 300, 23))]


def _alone(body, prec, steps):
    F, ids, mats = body
    ctx = device_context(tillotson_materials(), precision=prec)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    ctx.step(steps)
    out = ctx.download()
    info = ctx.time()
    ctx.close()
    return out, info


def _same(a, b):
    (Fa, ida, ma), (Fb, idb, mb) = a, b
    assert np.array_equal(ida, idb) and np.array_equal(ma, mb)
    assert np.array_equal(Fa, Fb), float(np.max(np.abs(Fa - Fb)))


@pytest.mark.parametrize("prec", [0, 1])
def test_runs_in_a_mix_equal_runs_alone(prec):
    bodies = _bodies()
    ctx = device_context(tillotson_materials(), precision=prec)
    hs = [ctx.add_run(*b) for b in bodies]
    ctx.step(1 + 4)              # the first step is every run's prologue
    for h, b in zip(hs, bodies):
        alone, (t, dt, st) = _alone(b, prec, 4)
        _same(ctx.download_run(h), alone)
        info = ctx.run_info(h)
        assert info["steps"] == 4 and info["time"] == t and info["dt"] == dt


def test_density_sums_do_not_depend_on_the_conversion_path():
    """A run holding a particle 40 times its mean mass sends the whole context's density sums
    through the FP64-pipe conversion (__float2ll_rn); the other runs, which alone take the
    FP32 / integer split, give the same bits in that mix, and so does the heavy run (each run's
    sums are rounded on its own mass scale)."""
    from fdps_sph_gb300.ic import FIELD
    bodies = _bodies()
    F, ids, mats = small_impact(n_target=900, n_impactor=100, seed=24)[:3]
    F = F.copy()
    F[FIELD["mass"], 5] *= 40.0
    runs = (bodies[0], (F, ids, mats), bodies[1])
    ctx = device_context(tillotson_materials(), precision=1)
    hs = [ctx.add_run(*b) for b in runs]
    ctx.step(1 + 3)
    for h, b in zip(hs, runs):
        _same(ctx.download_run(h), _alone(b, 1, 3)[0])
    ctx.close()


def test_run_on_another_mass_scale_equals_run_alone():
    """a run whose particles are 2^10 times heavier than the first run's: its density sums are
    rounded on its own scale (the context's FP32 masses carry the first run's), so it matches the
    run advanced alone; a run 2^65 times heavier is refused"""
    from fdps_sph_gb300 import lib
    from fdps_sph_gb300.ic import FIELD
    bodies = _bodies()
    F, ids, mats = small_impact(n_target=900, n_impactor=100, seed=25)[:3]
    F = F.copy()
    F[FIELD["mass"]] *= 1024.0
    runs = (bodies[0], (F, ids, mats))
    ctx = device_context(tillotson_materials(), precision=1)
    hs = [ctx.add_run(*b) for b in runs]
    ctx.step(1 + 3)
    for h, b in zip(hs, runs):
        _same(ctx.download_run(h), _alone(b, 1, 3)[0])
    G = F.copy()
    G[FIELD["mass"]] *= 2.0 ** 55
    with pytest.raises(lib.SphError) as ei:
        ctx.add_run(G, ids, mats)
    assert ei.value.code == -1 and "2^" in str(ei.value)
    ctx.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_runs_removed_and_added_between_steps(prec):
    bodies = _bodies()
    ctx = device_context(tillotson_materials(), precision=prec)
    h0 = ctx.add_run(*bodies[0])
    h1 = ctx.add_run(*bodies[1])
    ctx.step(1 + 2)
    ctx.remove_run(h0)           # the first run leaves, the second moves down
    h2 = ctx.add_run(*bodies[2])  # a new run joins: its next step is its prologue
    ctx.step(1 + 3)
    assert ctx.runs() == [h1, h2]
    _same(ctx.download_run(h1), _alone(bodies[1], prec, 6)[0])
    _same(ctx.download_run(h2), _alone(bodies[2], prec, 3)[0])
    # diagnostics per run add up to the context's
    tot = ctx.diagnostics()
    per = ctx.run_diagnostics(h1) + ctx.run_diagnostics(h2)
    assert np.allclose(tot, per, rtol=1e-12, atol=0.0)


def test_serving_loop_results_equal_runs_alone():
    """Continuous batching: four requests through two run slots (so the batch
    is backfilled as runs finish); every result equals its run advanced alone."""
    from fdps_sph_gb300 import ic, serve
    reqs = [serve.Request(k, 0.0, steps, 900 + k, 2000, 5000) for k, steps in enumerate((3, 5, 2, 4))]
    srv = serve.Server("mixed", budget_bytes=1 << 34, max_runs=2, keep_results=True)
    try:
        rep = srv.run(reqs)
    finally:
        srv.close()
    assert rep["completed"] == 4 and rep["resident_at_end"] == 0
    assert rep["step_latency_s"]["p99"] is not None and rep["time_to_completion_s"]["p50"] is not None
    for r in reqs:
        F, ids, mats, _ = ic.sweep_impact(np.random.default_rng(r.rng_seed), r.n_lo, r.n_hi, r.rng_seed)
        ctx = serve.make_context("mixed")
        ctx.upload(F, ids, mats)
        ctx.prologue()
        ctx.step(r.steps)
        alone = ctx.download()
        ctx.close()
        _same(r.result, alone)


@pytest.mark.parametrize("prec", [0, 1])
def test_checkpoint_resume_is_exact(prec, tmp_path):
    """steps after a checkpoint and a restore into a new context give the same
    state as stepping on without one"""
    from fdps_sph_gb300 import snapshot
    bodies = _bodies()
    ctx = device_context(tillotson_materials(), precision=prec)
    hs = [ctx.add_run(*b) for b in bodies[:2]]
    ctx.step(1 + 3)
    path = str(tmp_path / "c.ckpt")
    snapshot.write_checkpoint(path, ctx)
    ctx.step(2)
    ctx2 = device_context(tillotson_materials(), precision=prec)
    hs2 = snapshot.restore(ctx2, path)
    ctx2.step(2)
    for a, b in zip(hs, hs2):
        _same(ctx.download_run(a), ctx2.download_run(b))
        assert ctx.run_info(a)["time"] == ctx2.run_info(b)["time"]


@pytest.mark.parametrize("prec", [0, 1])
def test_step_inputs_upload_equals_full_upload(prec):
    """A host that keeps its particles uploads only the fields a step reads or carries
    (SPH_UPLOAD_STEP_INPUTS); the step's results equal those after a full upload, bit for bit."""
    from fdps_sph_gb300 import lib
    F, ids, mats = _bodies()[0]
    ctx = device_context(tillotson_materials(), precision=prec)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    ctx.step(2)
    Fh, idh, mh = ctx.download()
    t, dt, _ = ctx.time()
    ctx.close()
    out = []
    for inputs_only in (False, True):
        c = device_context(tillotson_materials(), precision=prec)
        G = Fh.copy()
        if inputs_only:   # what is not an input must not matter
            keep = [lib.FIELD[f] for f in lib.STEP_INPUT_FIELDS]
            drop = np.setdiff1d(np.arange(lib.NFIELD), keep)
            G[drop] = np.nan
        c.upload(G, idh, mh, time=t, dt=dt, forces_valid=True, inputs_only=inputs_only)
        c.step(2)
        out.append(c.download())
        c.close()
    _same(out[0], out[1])


def test_upload_checks_masses_and_materials():
    from fdps_sph_gb300 import lib
    F, ids, mats = _bodies()[1]
    ctx = device_context(tillotson_materials(), precision=1)
    G = F.copy()
    G[lib.FIELD["mass"], 17] = -1.0
    with pytest.raises(lib.SphError) as ei:
        ctx.upload(G, ids, mats)
    assert ei.value.code == -5 and "particle 17" in str(ei.value)
    G[lib.FIELD["mass"], 17] = np.inf
    with pytest.raises(lib.SphError):
        ctx.upload(G, ids, mats)
    bad = mats.copy()
    bad[40] = 9                      # a slot that was never set
    with pytest.raises(lib.SphError) as ei:
        ctx.upload(F, ids, bad)
    assert ei.value.code == -1 and "particle 40" in str(ei.value)
    ctx.upload(F, ids, mats)         # the context is usable after the refusals
    ctx.prologue()
    ctx.step(1)
    ctx.close()


def test_download_fields_copies_only_the_masked_rows():
    from fdps_sph_gb300 import lib
    F, ids, mats = _bodies()[1]
    ctx = device_context(tillotson_materials(), precision=1)
    ctx.upload(F, ids, mats)
    ctx.prologue()
    ctx.step(1)
    full, _, _ = ctx.download()
    part = np.full_like(full, -7.0)
    ctx.download_fields(part, lib.STEP_OUTPUT_FIELDS)
    for k, f in enumerate(lib.FIELDS):
        if f in lib.STEP_OUTPUT_FIELDS:
            assert np.array_equal(part[k], full[k]), f
        else:
            assert np.all(part[k] == -7.0), f
    # what the step does not write is what was uploaded
    for f in ("mass", "ava", "ent", "temp"):
        assert np.array_equal(full[lib.FIELD[f]], F[lib.FIELD[f]]), f
    ctx.close()


@pytest.mark.parametrize("prec,ext_damp,n_runs", [(1, False, 1), (0, True, 1), (1, False, 2)])
def test_step_download_equals_step_then_download(prec, ext_damp, n_runs):
    """fields streamed out during the step equal a download after it, bit for bit"""
    from fdps_sph_gb300 import lib
    bodies = _bodies()[:n_runs]
    out = []
    for streamed in (False, True):
        ctx = device_context(tillotson_materials(), precision=prec, ext_damp=int(ext_damp))
        if n_runs == 1:
            ctx.upload(*bodies[0])
            ctx.prologue()
        else:
            for b in bodies:
                ctx.add_run(*b)
            ctx.step(1)   # the runs' prologue
        ctx.step(1)
        n = ctx.n_particles()
        blk = np.full((lib.NFIELD, n), -3.0)
        if streamed:
            ctx.step_download(blk, lib.STEP_OUTPUT_FIELDS)
        else:
            ctx.step(1)
            ctx.download_fields(blk, lib.STEP_OUTPUT_FIELDS)
        out.append(blk)
        ctx.close()
    assert np.array_equal(out[0], out[1])
    assert np.all(out[1][lib.FIELD["mass"]] == -3.0)
