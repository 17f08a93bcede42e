"""Primary beams generated on the device (ptg_build_beam) against the
reference's distributions (particle/dstr.rs, particle/builder.rs):
moments, correlations and shapes at 1e6 primaries, the host builder
(ptarmigan_gb300/beam.py) by two-sample KS, and the oracle's pwmci
inverse for tabulated spectra."""

import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu

N = 1_000_000


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    yield e
    e.close()


def _host(d):
    return {k: v.cpu().numpy() for k, v in d.items()}


def _ks(a, b):
    a, b = np.sort(a), np.sort(b)
    g = np.concatenate([a, b])
    return np.max(np.abs(np.searchsorted(a, g, side="right") / len(a) - np.searchsorted(b, g, side="right") / len(b)))


def _ks_crit(n, m):
    return 1.95 * math.sqrt((n + m) / (n * m))  # significance 1e-3


def _ks1(x, cdf):
    x = np.sort(x)
    f = cdf(x)
    i = np.arange(1, len(x) + 1) / len(x)
    return max(np.max(i - f), np.max(f - (i - 1.0 / len(x))))


def test_normal_beam_moments_and_correlations(eng):
    g0, sg = 32289.0, 32.3
    d = abi.beam_desc(gamma_mean=g0, gamma_sigma=sg, energy_chirp=0.4, sigma_x=2e-6, sigma_y=3e-6, sigma_z=20e-6,
                      rms_div=50e-6, initial_z=1e-4, stokes=(0.1, 0.2, 0.3), weight=2.5)
    b = _host(eng.build_beam(d, N, seed=7, first_id=100))
    u, r = b["u"], b["r"]
    gamma = u[:, 0]
    tol = 5.0 / math.sqrt(N)
    assert abs(gamma.mean() - g0) < 5 * sg / math.sqrt(N)
    assert abs(gamma.std() / sg - 1.0) < 5 * tol
    dz = r[:, 3] - 1e-4
    # rho = -energy_chirp (builder.rs:120-124)
    assert abs(np.corrcoef(gamma, dz)[0, 1] + 0.4) < 5 * tol
    assert abs(r[:, 1].std() / 2e-6 - 1.0) < 5 * tol and abs(r[:, 2].std() / 3e-6 - 1.0) < 5 * tol
    assert abs(dz.std() / 20e-6 - 1.0) < 5 * tol
    assert np.all(r[:, 0] == -1e-4)
    assert np.all(u[:, 3] < 0)  # heading towards -z, into the laser
    assert abs((u[:, 1] / -u[:, 3]).std() / 50e-6 - 1.0) < 5 * tol
    np.testing.assert_allclose(u[:, 0] ** 2 - (u[:, 1:] ** 2).sum(axis=1), 1.0, rtol=1e-6)
    assert np.all(b["species"] == abi.ELECTRON) and np.all(b["weight"] == 2.5)
    assert np.array_equal(b["id"], np.arange(100, 100 + N, dtype=np.uint64))
    assert np.array_equal(b["parent_id"], b["id"])
    assert np.all(b["pol"] == np.array([1.0, 0.1, 0.2, 0.3]))


def test_device_beam_matches_host_builder(eng):
    """Same parameters (collision angle, plane and offset included): the
    device beam and the host builder agree by KS in every coordinate."""
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    kw = dict(radius=2e-6, length=20e-6, rms_div=50e-6, collision_angle=0.3, collision_plane=0.5,
              offset=(1e-6, -2e-6, 5e-6))
    n = 200_000
    host = beam.build(n, g, sigma=0.01 * g, laser=laser, seed=3, **kw)
    z0 = beam.initial_z(laser, 20e-6)
    d = abi.beam_desc(gamma_mean=g, gamma_sigma=0.01 * g, sigma_x=2e-6, sigma_z=20e-6, rms_div=50e-6,
                      collision_angle=0.3, collision_plane=0.5, offset=(1e-6, -2e-6, 5e-6), initial_z=z0)
    dev = _host(eng.build_beam(d, n, seed=3))
    for key in ("r", "u"):
        for c in range(4):
            a, b_ = host[key][:, c], dev[key][:, c]
            if np.ptp(a) == 0.0:
                assert np.allclose(b_, a[0])
                continue
            assert _ks(a, b_) < _ks_crit(n, n), (key, c)


def test_brem_spectrum(eng):
    gmin, gmax = 2000.0, 20000.0
    d = abi.beam_desc(species=abi.PHOTON, gamma_dstr=abi.GAMMA_BREM, gamma_min=gmin, gamma_max=gmax,
                      sigma_x=1e-6, sigma_z=1e-6)
    b = _host(eng.build_beam(d, 300_000, seed=11))
    x = b["u"][:, 0] / gmax  # photons: u0 = |u| = gamma
    np.testing.assert_allclose(b["u"][:, 0] ** 2, (b["u"][:, 1:] ** 2).sum(axis=1), rtol=1e-12)
    x0 = gmin / gmax

    def F(t):
        def prim(s):
            return 4.0 / 3.0 * np.log(s) - 4.0 / 3.0 * s + 0.5 * s * s
        return (prim(t) - prim(x0)) / (prim(1.0) - prim(x0))
    assert x.min() >= x0 and x.max() <= 1.0
    assert _ks1(x, F) < 1.95 / math.sqrt(len(x))


def test_custom_spectrum_follows_the_oracle_inverse(eng, orc):
    """Tabulated spectrum (GammaDistribution::custom): NORTA transform then
    the pwmci inverse of the CDF; compared with the oracle's pwmci inverse
    applied to the same transform of independent normals."""
    vals = np.array([1.0, 3.0, 6.0, 4.0, 2.0, 1.0, 0.5])
    gmin, step = 1000.0, 500.0
    nodes = [[gmin, 0.0]]
    acc = 0.0
    for k, v in enumerate(vals):
        acc += v
        nodes.append([gmin + (k + 1) * step, acc / vals.sum()])
    cdf = np.ascontiguousarray(nodes, dtype=np.float64)
    d = abi.beam_desc(gamma_dstr=abi.GAMMA_CUSTOM, custom_cdf=cdf, sigma_x=1e-6, sigma_z=1e-6)
    n = 100_000
    b = _host(eng.build_beam(d, n, seed=5))
    g = b["u"][:, 0]
    rng = np.random.default_rng(2)
    x = rng.standard_normal(20_000) / math.sqrt(2.0)
    u1 = 0.5 * (1.0 + np.tanh(167.0 * x / 148.0 + 11.0 * x ** 3 / 109.0))
    ref = np.array([orc.pwmci_invert(cdf, f) for f in u1])
    assert g.min() >= gmin - 1e-9 and g.max() <= gmin + len(vals) * step + 1e-9
    assert _ks(g, ref) < _ks_crit(len(g), len(ref))


def test_truncated_and_uniform_transverse_shapes(eng):
    d = abi.beam_desc(gamma_mean=5000.0, radial_dstr=abi.RADIAL_TRUNC_NORMAL, sigma_x=2e-6, sigma_y=1e-6,
                      x_max=3e-6, y_max=2e-6, sigma_z=1e-6)
    b = _host(eng.build_beam(d, 200_000, seed=1))
    x, y = b["r"][:, 1], b["r"][:, 2]
    assert np.all(x * x / 9e-12 + y * y / 4e-12 <= 1.0 + 1e-12)
    assert x.std() < 2e-6 and y.std() < 1e-6
    d = abi.beam_desc(gamma_mean=5000.0, radial_dstr=abi.RADIAL_UNIFORM, r_max=4e-6, sigma_z=1e-6)
    b = _host(eng.build_beam(d, 200_000, seed=2))
    r2 = (b["r"][:, 1] ** 2 + b["r"][:, 2] ** 2) / 16e-12
    assert r2.max() <= 1.0 + 1e-12
    assert _ks1(r2, lambda t: t) < 1.95 / math.sqrt(len(r2))


def test_device_beam_feeds_the_collision_loop(eng):
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    d = abi.beam_desc(gamma_mean=g, gamma_sigma=0.01 * g, sigma_x=2e-6, sigma_z=20e-6, rms_div=50e-6,
                      initial_z=beam.initial_z(laser, 20e-6))
    prim = eng.build_beam(d, 20_000, seed=9)
    out, st = eng.collide_device(laser, abi.collide_options(max_generation=2), prim, seed=9)
    assert st["particle_errors"] == 0 and st["emissions"] > 10_000


def test_invalid_beams_are_rejected(eng):
    from ptarmigan_gb300.engine import PtgError
    with pytest.raises(PtgError):
        eng.build_beam(abi.beam_desc(gamma_mean=0.5), 10, seed=1)
    with pytest.raises(PtgError):
        eng.build_beam(abi.beam_desc(gamma_mean=100.0, energy_chirp=1.5), 10, seed=1)
    bad = np.array([[1.0, 0.0], [0.5, 1.0]])
    with pytest.raises(PtgError):
        eng.build_beam(abi.beam_desc(gamma_dstr=abi.GAMMA_CUSTOM, custom_cdf=bad), 10, seed=1)
