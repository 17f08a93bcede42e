"""The persistent multi-collision queue (ptg_collide_multi): each collision
of a batch must reproduce the single-collision entry point with the same
laser, seed and id_base, particle for particle (streams are the same), and
the batch must be deterministic under graph replay, overflow reruns and the
autotuner's launch shapes."""

import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu

# LMA kinematics amplify last-bit differences (see test_gpu_parity.LMA_TOL);
# LCFA showers agree to rounding.
TOL = {abi.FAST_FOCUSED_LASER: 1e-9, abi.FAST_PLANE_WAVE: 1e-9, abi.FOCUSED_LASER: 5e-7, abi.PLANE_WAVE: 5e-7}


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    yield e
    e.close()


def _concat(parts):
    keys = parts[0].keys()
    return {k: np.concatenate([p[k] for p in parts]) for k in keys}


def _batch(specs):
    """specs: (laser, n, energy_gev, seed).  Returns collisions, primaries."""
    colls, prims, first = [], [], 0
    for k, (laser, n, energy, seed) in enumerate(specs):
        g = beam.gamma_from_energy(energy)
        p = beam.build(n, g, sigma=0.001 * g, radius=1e-6, length=2e-6, rms_div=8e-6, laser=laser, seed=seed)
        prims.append(p)
        colls.append({"laser": laser, "seed": 100 + 7 * k, "id_base": 1000 * (k + 1), "first": first, "count": n})
        first += n
    return colls, _concat(prims)


def _compare(a, b, tol, frac_bad):
    ia = {int(s): i for i, s in enumerate(a["stream"])}
    ib = {int(s): i for i, s in enumerate(b["stream"])}
    common = set(ia) & set(ib)
    assert len(common) >= 0.97 * len(ib), (len(common), len(ib), len(ia))
    bad = 0
    for s in common:
        i, j = ia[s], ib[s]
        assert a["species"][i] == b["species"][j]
        scale = np.linalg.norm(b["u"][j])
        if np.max(np.abs(a["u"][i] - b["u"][j])) > tol * scale:
            bad += 1
    assert bad <= max(1, frac_bad * len(common)), (bad, len(common))


def _mixed_specs():
    ffl = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                         fwhm_duration=30e-15)
    fl_cp = abi.laser_desc(abi.FOCUSED_LASER, 3.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    fpw = abi.laser_desc(abi.FAST_PLANE_WAVE, 2.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=8.0)
    fl_lp = abi.laser_desc(abi.FOCUSED_LASER, 1.5, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=25e-15)
    return [(ffl, 40, 10.0, 1), (fl_cp, 30, 16.5, 2), (fpw, 30, 10.0, 3), (fl_lp, 30, 16.5, 4)]


@pytest.mark.parametrize("variant,use_graph", [(0, 0), (0, 1), (3, 0), (3, 1)])
def test_queue_matches_single_collisions(eng, variant, use_graph):
    """Four collisions of the four field models in one launch: whole
    particles per lane (variant 0) or every lane one step per pass with the
    warp sampling emissions (variant 3)."""
    # emission only: linearly polarised LMA pair creation is not built
    colls, prim = _batch(_mixed_specs())
    opts = abi.collide_options(max_generation=2, tracking_photons=0)
    eng.queue_config(variant=variant, blocks_per_sm=0, chunk=1, use_graph=use_graph)
    parts, stats, total = eng.collide_multi(colls, opts, prim)
    assert total["particle_errors"] == 0
    for k, c in enumerate(colls):
        sub = {name: v[c["first"]:c["first"] + c["count"]] for name, v in prim.items()}
        single, sst = eng.collide(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"])
        _compare(parts[k], single, TOL[c["laser"].model], 0.02)
        assert stats[k]["emissions"] == pytest.approx(sst["emissions"], rel=0.03, abs=2)
        assert stats[k]["n_primaries"] == c["count"]
    assert sum(s["n_out"] for s in stats) == total["n_out"]


def test_queue_is_deterministic_under_replay(eng):
    colls, prim = _batch(_mixed_specs())
    opts = abi.collide_options(max_generation=2, tracking_photons=0)
    eng.queue_config(variant=0, blocks_per_sm=0, chunk=2, use_graph=1)
    runs = [eng.collide_multi(colls, opts, prim)[0] for _ in range(2)]
    eng.queue_config(use_graph=0)
    runs.append(eng.collide_multi(colls, opts, prim)[0])
    for k in range(len(colls)):
        ref = runs[0][k]
        o0 = np.argsort(ref["stream"])
        for other in runs[1:]:
            o1 = np.argsort(other[k]["stream"])
            for name in ("species", "u", "r", "pol", "weight", "work", "stream"):
                assert np.array_equal(ref[name][o0], other[k][name][o1]), (k, name)


def test_queue_overflow_reruns(eng):
    """Showers larger than the initial store (4 slots per primary plus
    1024): the batch is rerun with a larger store and still matches the
    single runs."""
    ffl = abi.laser_desc(abi.FAST_FOCUSED_LASER, 20.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=2e-6,
                         fwhm_duration=30e-15)
    colls, prim = _batch([(ffl, 320, 16.5, 5), (ffl, 80, 16.5, 6)])
    opts = abi.collide_options(max_generation=-1, rate_increase=1.0)
    from ptarmigan_gb300 import engine
    fresh = engine.Engine(initial_capacity=16)
    try:
        fresh.queue_config(variant=1, chunk=1, use_graph=1)
        parts, stats, total = fresh.collide_multi(colls, opts, prim)
        assert total["n_created"] > 4 * total["n_primaries"] + 1024
        assert total["waves"] >= 2 and total["particle_errors"] == 0
        for k, c in enumerate(colls):
            sub = {name: v[c["first"]:c["first"] + c["count"]] for name, v in prim.items()}
            single, _ = fresh.collide(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"])
            _compare(parts[k], single, 1e-9, 0.02)
    finally:
        fresh.close()


@pytest.mark.parametrize("variant", [0, 3])
def test_queue_a0_scan_uneven(eng, variant):
    """A small a0 scan in one launch: 16 collisions, a0 log-spaced 0.5..20,
    LMA (circular) below a0 = 5 and LCFA above, uneven beam sizes."""
    rng = np.random.default_rng(3)
    specs = []
    for k, a0 in enumerate(np.geomspace(0.5, 20.0, 16)):
        model = abi.FOCUSED_LASER if a0 < 5.0 else abi.FAST_FOCUSED_LASER
        pol = abi.CIRCULAR if a0 < 5.0 else abi.LINEAR
        laser = abi.laser_desc(model, float(a0), 0.8e-6, pol, abi.GAUSSIAN, waist=5e-6, fwhm_duration=25e-15)
        specs.append((laser, int(rng.integers(1, 40)), 16.5, 10 + k))
    colls, prim = _batch(specs)
    opts = abi.collide_options()
    eng.queue_config(variant=variant, blocks_per_sm=0, chunk=1, use_graph=1)
    parts, stats, total = eng.collide_multi(colls, opts, prim)
    eng.queue_config(variant=0)
    assert total["particle_errors"] == 0
    for k in (0, 7, 15):
        c = colls[k]
        sub = {name: v[c["first"]:c["first"] + c["count"]] for name, v in prim.items()}
        single, sst = eng.collide(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"])
        _compare(parts[k], single, TOL[c["laser"].model], 0.03)


def test_queue_autotune_picks_a_valid_shape(eng):
    import torch
    colls, prim = _batch(_mixed_specs())
    opts = abi.collide_options(max_generation=2, tracking_photons=0)
    dev = torch.device("cuda", 0)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    best, ms = eng.queue_autotune(colls, opts, d_prim, sample_fraction=0.5)
    # a mixed batch: the single-collision variant is not a candidate
    assert best["variant"] in (0, 1, 3) and 1 <= best["chunk"] <= 64 and best["blocks_per_sm"] >= 1
    assert ms > 0.0 and math.isfinite(ms)
    assert eng.queue_config() == best
    out, offs, stats, total = eng.collide_multi_device(colls, opts, d_prim)
    assert offs[-1] == total["n_out"] and total["particle_errors"] == 0


@pytest.mark.parametrize("model", [abi.FAST_FOCUSED_LASER, abi.FOCUSED_LASER])
def test_single_collision_queue_matches_wave_path(eng, model):
    """The single-collision queue kernel (variant 2: one step per pass with
    lane refill, parameters in the launch arguments), pairs and every
    generation on, matches the wave path particle for particle; a batch of
    several collisions asked for variant 2 runs variant 0."""
    if model == abi.FAST_FOCUSED_LASER:
        laser = abi.laser_desc(model, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=3e-6, fwhm_duration=30e-15)
    else:
        laser = abi.laser_desc(model, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6, fwhm_duration=30e-15)
    colls, prim = _batch([(laser, 120, 16.5, 21)])
    opts = abi.collide_options(pol_resolved=1)
    eng.queue_config(variant=2, blocks_per_sm=0, chunk=1, use_graph=1)
    try:
        parts, stats, total = eng.collide_multi(colls, opts, prim)
        assert total["particle_errors"] == 0
        c = colls[0]
        single, sst = eng.collide(c["laser"], opts, prim, seed=c["seed"], id_base=c["id_base"])
        _compare(parts[0], single, TOL[model], 0.02)
        assert stats[0]["emissions"] == pytest.approx(sst["emissions"], rel=0.03, abs=2)
        assert stats[0]["lepton_steps"] == pytest.approx(sst["lepton_steps"], rel=0.01)
        colls_m, prim_m = _batch(_mixed_specs())
        parts_m, _, total_m = eng.collide_multi(colls_m, abi.collide_options(max_generation=2, tracking_photons=0),
                                                prim_m)
        assert total_m["particle_errors"] == 0 and len(parts_m) == len(colls_m)
    finally:
        eng.queue_config(variant=0)


def test_lp_emissions_warp_sampled_match_serial_sampler(eng):
    """Linear polarisation, LMA: the wave kernel samples emissions with the
    whole warp (lp_sample_warp), the queue kernel lane by lane
    (lp_sample); both give the same particles."""
    laser = abi.laser_desc(abi.PLANE_WAVE, 1.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=30.0)
    colls, prim = _batch([(laser, 800, 5.0, 31)])
    opts = abi.collide_options(tracking_photons=0)
    eng.queue_config(variant=2, blocks_per_sm=0, chunk=1, use_graph=0)
    try:
        parts, stats, total = eng.collide_multi(colls, opts, prim)
    finally:
        eng.queue_config(variant=0)
    c = colls[0]
    single, sst = eng.collide(c["laser"], opts, prim, seed=c["seed"], id_base=c["id_base"])
    assert total["particle_errors"] == 0 and sst["particle_errors"] == 0
    assert sst["emissions"] > 50
    _compare(parts[0], single, TOL[abi.PLANE_WAVE], 0.02)
    assert stats[0]["emissions"] == pytest.approx(sst["emissions"], rel=0.03, abs=2)
    assert stats[0]["lepton_steps"] == pytest.approx(sst["lepton_steps"], rel=0.01)


def test_graph_replay_follows_seed_and_sampler(eng):
    """A replayed graph must run with the call's own kernel arguments: the
    single-collision kernel takes the laser, seed and id base by value, and
    every variant takes the learned proposal's switch.  Each graph-replayed
    queue call must equal the wave path with the same seed and sampler, event
    count for event count."""
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    n = 3000
    prim = beam.build(n, g, sigma=0.001 * g, radius=2e-6, length=10e-6, rms_div=8e-6, laser=laser, seed=8)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    eng.mlp_init(3)
    eng.mlp_train(n_samples=200_000, batch=4096, epochs=1)
    keys = ("lepton_steps", "photon_steps", "emissions", "pair_events", "rejections", "n_out")
    for variant in (2, 0):
        eng.queue_config(variant=variant, blocks_per_sm=0, chunk=1, use_graph=1)
        for learned in (False, True, False):
            eng.mlp_use(learned)
            for seed in (31, 32):
                _, ref = eng.collide(laser, opts, prim, seed=seed, id_base=n)
                coll = [{"laser": laser, "seed": seed, "id_base": n, "first": 0, "count": n}]
                _, _, total = eng.collide_multi(coll, opts, prim)
                assert all(total[k] == ref[k] for k in keys), (variant, learned, seed, total, ref)
    eng.mlp_use(False)
    eng.queue_config(variant=0, blocks_per_sm=0, chunk=1, use_graph=1)


def test_lockstep_queue_lp_a0_scan_matches_single_collisions(eng):
    """Linearly polarised collisions (LMA below a0 = 5, LCFA above) in one
    lockstep launch (variant 3): the warp samples the LP emissions of lanes
    that belong to different collisions, and every collision reproduces its
    single-collision run."""
    specs = []
    for k, a0 in enumerate((0.8, 1.5, 3.0, 6.0, 12.0)):
        model = abi.FOCUSED_LASER if a0 < 5.0 else abi.FAST_FOCUSED_LASER
        laser = abi.laser_desc(model, a0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=5e-6, fwhm_duration=25e-15)
        specs.append((laser, 120, 16.5, 40 + k))
    colls, prim = _batch(specs)
    opts = abi.collide_options(max_generation=2, tracking_photons=0)
    eng.queue_config(variant=3, blocks_per_sm=0, chunk=1, use_graph=1)
    try:
        parts, stats, total = eng.collide_multi(colls, opts, prim)
    finally:
        eng.queue_config(variant=0)
    assert total["particle_errors"] == 0
    assert sum(s["emissions"] for s in stats[:3]) > 20
    for k, c in enumerate(colls):
        sub = {name: v[c["first"]:c["first"] + c["count"]] for name, v in prim.items()}
        single, sst = eng.collide(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"])
        _compare(parts[k], single, TOL[c["laser"].model], 0.02)
        assert stats[k]["emissions"] == pytest.approx(sst["emissions"], rel=0.03, abs=2)
