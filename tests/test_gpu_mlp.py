"""The learned proposal for the CP photon-energy sampler: tensor-core
inference and gradients against the CPU reference network
(tests/mlp_reference.py, with the device's BF16 operand rounding
emulated), training on the GPU, and what the trained network gains over
the reference's ceiling-and-rejection sampler at an unchanged
distribution."""

import numpy as np
import pytest

from mlp_reference import IN, OFF, forward, init, loss_and_grad
from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    e.load_tables()
    yield e
    e.close()


@pytest.fixture(scope="module")
def trained(eng):
    stats = eng.mlp_train(n_samples=4_000_000, batch=4096, epochs=2, lr=2e-3, tau=0.98, seed=7)
    return stats


def _ks(a, b):
    a, b = np.sort(a), np.sort(b)
    grid = np.concatenate([a, b])
    return np.max(np.abs(np.searchsorted(a, grid, side="right") / len(a) -
                         np.searchsorted(b, grid, side="right") / len(b)))


def _ks_bound(n, m):
    # two-sample KS critical value at significance 1e-3
    return 1.95 * np.sqrt((n + m) / (n * m))


def test_inference_matches_reference(eng):
    p = init(11)
    eng.mlp_params(set_to=p)
    got_p = eng.mlp_params()
    np.testing.assert_array_equal(got_p, p)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1.2, 1.2, (1003, IN)).astype(np.float32)  # not a multiple of 16 rows
    out = eng.mlp_infer(x)
    ref, _ = forward(p, x, emulate=True)
    exact, _ = forward(p, x, emulate=False)
    scale = 1.0 + np.max(np.abs(ref))
    # BF16 operands, FP32 accumulation: same rounding as the emulated
    # reference up to accumulation order and the rare flip of an
    # activation's last BF16 bit
    assert np.max(np.abs(out - ref)) <= 2e-2 * scale
    assert np.mean(np.abs(out - ref)) <= 2e-3 * scale
    assert np.max(np.abs(out - exact)) <= 6e-2 * scale


def test_gradient_matches_reference(eng):
    p = init(12)
    eng.mlp_params(set_to=p)
    rng = np.random.default_rng(2)
    n = 4096
    x = rng.uniform(-1, 1, (n, IN))
    bins = rng.integers(0, 16, n)
    o_ref, _ = forward(p, x, emulate=True)
    # targets well away from the outputs, so that no residual's sign
    # depends on rounding
    off = rng.uniform(0.1, 2.0, n) * rng.choice([-1.0, 1.0], n)
    t = o_ref[np.arange(n), bins] + off
    samples = np.column_stack([x, bins, t]).astype(np.float32)
    samples[::97, IN] = -1  # invalid rows are skipped
    samples[5::101, IN + 1] = np.nan
    tau = 0.9
    g, loss = eng.mlp_grad(samples, tau)
    loss_ref, g_ref = loss_and_grad(p, samples.astype(np.float64), tau, emulate=True)
    assert loss == pytest.approx(loss_ref, rel=2e-3)
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    assert cos > 0.9995, cos
    for name, (o, sz) in OFF.items():
        ref = g_ref[o:o + sz]
        err = np.linalg.norm(g[o:o + sz] - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err < 3e-2, (name, err)
    # the padding columns of the first layer get no gradient
    w0 = g[OFF["W0"][0]:OFF["W0"][0] + OFF["W0"][1]].reshape(64, 16)
    assert np.all(w0[:, IN:] == 0.0)


def test_training_lowers_the_loss(eng, trained):
    assert trained["steps"] == 2 * (4_000_000 // 4096)
    assert np.isfinite(trained["loss_last"])
    assert trained["loss_last"] < 0.3 * trained["loss_first"], trained


def test_learned_sampler_gain_at_unchanged_distribution(eng, trained):
    """Same (a, eta, n) per emission for both methods: the learned envelope
    needs far fewer spectrum evaluations, envelope violations (which fall
    back to the reference's sampler) are rare, and the sampled v follow the
    same distribution."""
    n = 400_000
    v0, v1, st = eng.sampler_bench(n, seed=5, margin=0.25)
    assert st["errors_plain"] == 0 and st["errors_learned"] == 0, st
    assert st["fallbacks"] <= 2e-3 * n, st
    assert st["exhausted"] <= 2e-2 * n, st
    assert st["learned_evals"] < st["plain_evals"] / 4.0, st
    assert np.all((v0 > 0) & (v0 < 1)) and np.all((v1 > 0) & (v1 < 1))
    assert _ks(v0, v1) < _ks_bound(n, n), (_ks(v0, v1), st)


def test_untrained_network_hands_over(eng):
    """A network whose envelope lies under the spectrum: the violations are
    detected and those emissions go to the reference's sampler, with no
    failed emission."""
    e2 = type(eng)()
    try:
        e2.load_tables()
        p = init(13)
        p[OFF["b3"][0]:OFF["b3"][0] + 16] = -5.0  # envelope far under the spectrum
        e2.mlp_params(set_to=p)
        n = 50_000
        v0, v1, st = e2.sampler_bench(n, seed=9, margin=0.0)
        assert st["errors_plain"] == 0 and st["errors_learned"] == 0, st
        assert st["fallbacks"] > 0.5 * n
        assert np.all((v1 > 0) & (v1 < 1))
    finally:
        e2.close()


def test_learned_collide_cp_shower_statistics(eng, trained):
    """CP focused laser, LMA emission: the learned proposal inside the
    collision kernel gives the same photon spectrum and yield as the
    reference's sampler (independent Monte Carlo, compared by KS)."""
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(16000, g, sigma=0.001 * g, radius=1e-6, length=3e-6, rms_div=8e-6, laser=laser, seed=21)
    opts = abi.collide_options(pol_resolved=1, tracking_photons=0)
    eng.mlp_use(False)
    out0, st0 = eng.collide(laser, opts, prim, seed=31)
    eng.mlp_use(True, margin=0.25)
    try:
        out1, st1 = eng.collide(laser, opts, prim, seed=31)
    finally:
        eng.mlp_use(False)
    assert st0["particle_errors"] == 0 and st1["particle_errors"] == 0
    e0 = out0["u"][out0["species"] == abi.PHOTON, 0]
    e1 = out1["u"][out1["species"] == abi.PHOTON, 0]
    assert len(e0) > 20_000
    # yields agree within Poisson noise (5 sigma)
    assert abs(len(e1) - len(e0)) < 5.0 * np.sqrt(2.0 * len(e0))
    assert _ks(e0, e1) < _ks_bound(len(e0), len(e1))
    # Stokes parameters of the photons
    s0 = out0["pol"][out0["species"] == abi.PHOTON]
    s1 = out1["pol"][out1["species"] == abi.PHOTON]
    for k in range(4):
        assert abs(s0[:, k].mean() - s1[:, k].mean()) < 5.0 * np.sqrt(
            (s0[:, k].var() + s1[:, k].var()) / len(e0)) + 1e-12


def _learned_points(m, seed):
    rng = np.random.default_rng(seed)
    a = np.exp(rng.uniform(np.log(0.1), np.log(10.0), m))
    eta = np.exp(rng.uniform(np.log(2e-3), np.log(1.0), m))
    return a, eta, np.arange(m, dtype=np.uint64) * 7919 + 11


@pytest.mark.parametrize("network", ["trained", "trained_from_8", "under", "over"])
def test_learned_warp_sampler_matches_lane_sampler(eng, trained, network):
    """The collision kernels sample CP emissions with the learned proposal
    on the whole warp (network units, the 16 trials and f(v*) spread over
    the lanes); the multi-collision queue kernel samples them on the
    emitting lane.  Both draw the same numbers and return the same samples
    bit for bit, for a trained network (used at every harmonic, or from
    harmonic 8 up with the reference's sampler below), for an envelope under
    the spectrum
    (every emission handed over to the reference's sampler) and for one far
    above it (16 rejections, then the capped continuation)."""
    e = eng
    own = None
    if not network.startswith("trained"):
        own = type(eng)()
        own.load_tables()
        p = init(13)
        p[OFF["b3"][0]:OFF["b3"][0] + 16] = -5.0 if network == "under" else 9.0
        own.mlp_params(set_to=p)
        e = own
    prev = None
    try:
        e.mlp_use(True, margin=0.25)
        # the network from harmonic 8 up, the reference's sampler below
        prev = e.mlp_min_harmonic(8 if network == "trained_from_8" else 1)
        a, eta, streams = _learned_points(4096, 3)
        out_l, st_l = e.cp_sample(a, eta, 17, streams, 5, learned=True)
        out_w, st_w = e.cp_sample(a, eta, 17, streams, 5, warp=True, learned=True)
        assert np.array_equal(st_l, st_w)
        assert np.count_nonzero(st_l == 0) >= 0.99 * len(a), np.unique(st_l, return_counts=True)
        assert np.array_equal(out_l, out_w)
        # the same distribution as the reference's sampler on other draws
        out_r, st_r = e.cp_sample(a, eta, 18, streams, 5)
        ok = (st_l == 0) & (st_r == 0)
        assert _ks(out_l[ok, 1], out_r[ok, 1]) < _ks_bound(ok.sum(), ok.sum())
    finally:
        e.mlp_use(False)
        if own is None:
            if prev is not None:
                e.mlp_min_harmonic(prev)
        else:
            own.close()
