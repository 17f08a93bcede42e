"""GPU parity: the CUDA path, called through the C ABI, against the FP64
oracle on the same inputs.

Deterministic quantities (fields, pushes, rates, sampler outputs for given
uniforms) are compared element by element with the tolerance written in
each test.  The collision loop is compared particle by particle: the GPU and
the oracle draw from the same counter-based streams, so each secondary is
identified by its stream id on both sides.
"""

import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu

C_LIGHT = 2.997925e8
RQM_E = -1.602177e-19 / 9.109383e-31


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    e.load_tables()
    yield e
    e.close()


def _lasers():
    return [
        abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                       fwhm_duration=30e-15),
        abi.laser_desc(abi.FAST_FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                       fwhm_duration=30e-15),
        abi.laser_desc(abi.FAST_FOCUSED_LASER, 20.0, 0.8e-6, abi.LINEAR, abi.COS2, waist=5e-6, n_cycles=10.0,
                       pol_angle=0.3),
        abi.laser_desc(abi.FAST_PLANE_WAVE, 1.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=30.87),
        abi.laser_desc(abi.FAST_PLANE_WAVE, 3.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, n_cycles=8.0),
        abi.laser_desc(abi.FAST_PLANE_WAVE, 2.0, 0.8e-6, abi.LINEAR, abi.FLATTOP, n_cycles=6.0, chirp_b=1e-3),
    ]


def _positions(laser, n, seed):
    rng = np.random.default_rng(seed)
    lam = laser.wavelength
    z = rng.uniform(-8 * lam, 8 * lam, n)
    t = rng.uniform(-8 * lam, 8 * lam, n)
    x = rng.normal(0, 2e-6, n)
    y = rng.normal(0, 2e-6, n)
    return np.stack([t, x, y, z], axis=1)


@pytest.mark.parametrize("li", range(6))
def test_lcfa_fields_match_oracle(eng, orc, li):
    laser = _lasers()[li]
    r = _positions(laser, 400, li)
    E, B, a = eng.fields(laser, r)
    scale_e = np.abs(E).max()
    scale_b = np.abs(B).max()
    for i in range(len(r)):
        Eo, Bo, ao = orc.fields(laser, r[i])
        # The focused beam's diffraction corrections of order eps^2..eps^4
        # are FP32 on the device (the leading orders FP64): 1e-8 of the
        # field scale.  Plane waves are FP64 throughout.
        tol = 1e-8 if laser.model == abi.FAST_FOCUSED_LASER else 1e-12
        assert np.all(np.abs(E[i] - Eo) <= tol * scale_e), (i, E[i], Eo)
        assert np.all(np.abs(B[i] - Bo) <= tol * scale_b), (i, B[i], Bo)
        assert abs(a[i] - ao) <= tol * max(1.0, ao)


@pytest.mark.parametrize("model,pol,env", [(abi.PLANE_WAVE, abi.LINEAR, abi.COS2),
                                           (abi.FOCUSED_LASER, abi.CIRCULAR, abi.GAUSSIAN),
                                           (abi.FOCUSED_LASER, abi.LINEAR, abi.FLATTOP)])
def test_lma_a_sqd_matches_oracle(eng, orc, model, pol, env):
    laser = abi.laser_desc(model, 5.0, 0.8e-6, pol, env, waist=3e-6, n_cycles=12.0)
    r = _positions(laser, 300, 7)
    _, _, a = eng.fields(laser, r)
    for i in range(len(r)):
        ao = math.sqrt(orc.a_sqd(laser, r[i]))
        assert abs(a[i] - ao) <= 1e-13 * max(1.0, ao)


def _beam_start(laser, n, gamma, seed):
    return beam.build(n, gamma, sigma=0.01 * gamma, radius=2e-6, length=5e-6, rms_div=50e-6, laser=laser,
                      seed=seed)


@pytest.mark.parametrize("li,eqn", [(0, abi.LORENTZ), (1, abi.LORENTZ), (3, abi.LORENTZ), (4, abi.LANDAU_LIFSHITZ),
                                    (0, abi.MODIFIED_LANDAU_LIFSHITZ)])
def test_classical_trajectories_match_oracle(eng, orc, li, eqn):
    """Emission off: full crossings of the pulse, FP64 push error <= 1e-10
    relative against the oracle."""
    laser = _lasers()[li]
    dt = orc.max_timestep(laser)
    z0 = orc.initial_z(laser)
    prim = _beam_start(laser, 64, 2000.0, li)
    # enough steps to cross the whole pulse: the phase k.r grows by about
    # 2 k c dt per step for a head-on ultrarelativistic particle
    k = 2 * math.pi / laser.wavelength
    nc = laser.n_cycles
    max_phase = {abi.COS2: math.pi * nc, abi.FLATTOP: math.pi * (nc + 1), abi.GAUSSIAN: 6 * math.pi * nc}[laser.envelope]
    phase0 = min(k * (r[0] - r[3]) for r in prim["r"])
    nsteps = min(int((max_phase - phase0) / (2 * k * C_LIGHT * dt)) + 10, 40000)
    r_g, u_g, w_g = eng.push_steps(laser, prim["r"], prim["u"], RQM_E, dt, nsteps, eqn)
    r_o, u_o, w_o = orc.push_steps(laser, prim["r"], prim["u"], RQM_E, dt, nsteps, eqn)
    assert z0 > 0
    for i in range(len(r_g)):
        assert np.max(np.abs(u_g[i] - u_o[i])) <= 1e-10 * np.linalg.norm(u_o[i]), (i, u_g[i], u_o[i])
        assert np.max(np.abs(r_g[i] - r_o[i])) <= 1e-10 * np.linalg.norm(r_o[i]), (i, r_g[i], r_o[i])


@pytest.mark.parametrize("model,pol,env,eqn", [(abi.PLANE_WAVE, abi.LINEAR, abi.COS2, abi.LANDAU_LIFSHITZ),
                                               (abi.FOCUSED_LASER, abi.CIRCULAR, abi.GAUSSIAN, abi.LORENTZ),
                                               (abi.FOCUSED_LASER, abi.LINEAR, abi.GAUSSIAN, abi.LANDAU_LIFSHITZ)])
def test_lma_trajectories_match_oracle(eng, orc, model, pol, env, eqn):
    laser = abi.laser_desc(model, 5.0, 0.8e-6, pol, env, waist=3e-6, n_cycles=12.0)
    dt = orc.max_timestep(laser)
    prim = _beam_start(laser, 64, 5000.0, 3)
    nsteps = 800
    r_g, u_g, w_g = eng.push_steps(laser, prim["r"], prim["u"], RQM_E, dt, nsteps, eqn)
    r_o, u_o, w_o = orc.push_steps(laser, prim["r"], prim["u"], RQM_E, dt, nsteps, eqn)
    for i in range(len(r_g)):
        assert np.max(np.abs(u_g[i] - u_o[i])) <= 1e-10 * np.linalg.norm(u_o[i])
        assert np.max(np.abs(r_g[i] - r_o[i])) <= 1e-10 * np.linalg.norm(r_o[i])
        assert abs(w_g[i] - w_o[i]) <= 1e-9 * max(1e-3, abs(w_o[i]))


def test_lcfa_photon_rate_matches_oracle(eng, orc):
    chi = np.exp(np.linspace(math.log(1e-4), math.log(500.0), 777))
    gamma = np.full_like(chi, 1000.0)
    got = eng.lcfa_photon_rate(chi, gamma)
    for c, g in zip(chi, got):
        ref = orc.lcfa_photon_rate(c, 1000.0)
        assert abs(g - ref) <= 1e-13 * ref


def test_lcfa_pair_t_matches_oracle(eng, orc):
    chi = np.exp(np.linspace(math.log(5e-3), math.log(300.0), 555))
    tp, tq = eng.lcfa_pair_t(chi)
    for c, a, b in zip(chi, tp, tq):
        ra, rb = orc.lcfa_pair_t(c)
        assert abs(a - ra) <= 1e-13 * max(ra, 1e-300)
        assert abs(b - rb) <= 1e-13 * max(rb, 1e-300)


def test_lcfa_photon_sample_matches_oracle(eng, orc):
    rng = np.random.default_rng(5)
    n = 3000
    chi = np.exp(rng.uniform(math.log(0.005), math.log(300.0), n))
    gamma = np.exp(rng.uniform(math.log(50.0), math.log(5e4), n))
    rand3 = rng.random((n, 3))
    om, th = eng.lcfa_photon_sample(chi, gamma, rand3)
    for i in range(n):
        o, t, _ = orc.lcfa_photon_sample(chi[i], gamma[i], *rand3[i])
        assert abs(om[i] - o) <= 1e-12 * o, i
        if t is None:
            assert th[i] < 0
        else:
            assert abs(th[i] - t) <= 1e-9 * max(t, 1e-12), i


def _config1_small(n, seed=1):
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(n, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=seed)
    return laser, prim


def _match_by_stream(a, b):
    ia = {int(s): i for i, s in enumerate(a["stream"])}
    ib = {int(s): i for i, s in enumerate(b["stream"])}
    common = sorted(set(ia) & set(ib))
    return common, ia, ib


@pytest.mark.parametrize("rate_increase", [1.0, 200.0])
def test_collide_matches_oracle_particle_by_particle(eng, orc, rate_increase):
    laser, prim = _config1_small(48)
    opts = abi.collide_options(max_generation=2, rate_increase=rate_increase)
    gout, gst = eng.collide(laser, opts, prim, seed=11)
    oout, ost = orc.collide(laser, opts, prim, seed=11, threads=8)
    assert gst["lepton_steps"] + gst["photon_steps"] > 0
    assert abs(len(gout["species"]) - len(oout["species"])) <= max(2, 0.02 * len(oout["species"]))
    common, ia, ib = _match_by_stream(gout, oout)
    assert len(common) >= 0.98 * len(oout["species"])
    bad = 0
    for s in common:
        i, j = ia[s], ib[s]
        assert gout["species"][i] == oout["species"][j]
        scale = np.linalg.norm(oout["u"][j])
        if np.max(np.abs(gout["u"][i] - oout["u"][j])) > 1e-8 * scale:
            bad += 1
    # an event decision can flip where u is within rounding of the probability
    assert bad <= max(1, 0.01 * len(common))
    assert gst["emissions"] == pytest.approx(ost["emissions"], rel=0.02, abs=2)


def test_collide_is_deterministic(eng):
    laser, prim = _config1_small(64, seed=3)
    opts = abi.collide_options(max_generation=2, rate_increase=100.0)
    a, sa = eng.collide(laser, opts, prim, seed=5)
    b, sb = eng.collide(laser, opts, prim, seed=5)
    oa, ob = np.argsort(a["stream"]), np.argsort(b["stream"])
    for k in ("species", "u", "r", "pol", "weight", "work", "stream"):
        assert np.array_equal(a[k][oa], b[k][ob]), k
    assert sa["emissions"] == sb["emissions"]


def test_collide_options_filters(eng, orc):
    laser, prim = _config1_small(40, seed=4)
    opts = abi.collide_options(max_generation=2, min_energy=50.0, max_angle=0.01, discard_bg_e=1)
    gout, _ = eng.collide(laser, opts, prim, seed=2)
    oout, _ = orc.collide(laser, opts, prim, seed=2, threads=4)
    assert len(gout["species"]) == pytest.approx(len(oout["species"]), abs=2)
    e = 0.510999 * gout["u"][:, 0]
    assert np.all(e > 50.0)


# LMA emission builds the photon in the zero-momentum frame of q + n k, whose
# four-velocity comes from (q + n k)^2 ~ 1 + a^2 + 2 n eta, a difference of
# squares of size gamma^2: one ulp of the electron's momentum moves the
# photon by up to ~gamma^2 / (1 + a^2) ulp (1.5e-8 relative at gamma = 2e4,
# a = 2, measured on the oracle).  LMA showers are compared at 5e-7.
LMA_TOL = 5e-7


def _compare_showers(gout, oout, tol=1e-8, frac_bad=0.02):
    common, ia, ib = _match_by_stream(gout, oout)
    n_ref = len(oout["species"])
    assert len(common) >= 0.97 * n_ref, (len(common), n_ref, len(gout["species"]))
    bad = 0
    for s in common:
        i, j = ia[s], ib[s]
        assert gout["species"][i] == oout["species"][j]
        scale = np.linalg.norm(oout["u"][j])
        if np.max(np.abs(gout["u"][i] - oout["u"][j])) > tol * scale:
            bad += 1
    assert bad <= max(1, frac_bad * len(common)), (bad, len(common))
    return len(common)


@pytest.mark.parametrize("pol_resolved", [0, 1])
def test_lma_cp_focused_emission_matches_oracle(eng, orc, pol_resolved):
    """FocusedLaser, circular polarisation: LMA emission (CP harmonic
    sampler with the regenerated CDF) and the secondaries' pair creation."""
    if not orc.has_cp_cdf():
        pytest.skip("CP CDF table missing")
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(60, g, sigma=0.001 * g, radius=1e-6, length=2e-6, rms_div=8e-6, laser=laser, seed=5)
    opts = abi.collide_options(pol_resolved=pol_resolved, rate_increase=30.0)
    gout, gst = eng.collide(laser, opts, prim, seed=17)
    oout, ost = orc.collide(laser, opts, prim, seed=17, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["emissions"] > 40
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["emissions"] == pytest.approx(ost["emissions"], rel=0.03, abs=2)


@pytest.mark.parametrize("pol_resolved", [0, 1])
def test_lma_cp_focused_pairs_match_oracle(eng, orc, pol_resolved):
    """Photon beam on a CP focused laser: CP Breit-Wheeler probability
    (lookup and explicit harmonic summation), Stokes update and positron
    sampler."""
    if not orc.has_cp_cdf():
        pytest.skip("CP CDF table missing")
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(120, g, sigma=0.001 * g, radius=1e-6, length=2e-6, rms_div=8e-6, laser=laser, seed=9,
                      species=abi.PHOTON, stokes=(0.3, 0.0, 0.5))
    opts = abi.collide_options(pol_resolved=pol_resolved, rate_increase=100.0)
    gout, gst = eng.collide(laser, opts, prim, seed=23)
    oout, ost = orc.collide(laser, opts, prim, seed=23, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["pair_events"] >= 10
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["pair_events"] == pytest.approx(ost["pair_events"], rel=0.05, abs=2)
    # photons that did not decay: their Stokes vectors and interaction counts
    common, ia, ib = _match_by_stream(gout, oout)
    for s_ in common:
        i, j = ia[s_], ib[s_]
        if oout["species"][j] == abi.PHOTON and oout["generation"][j] == 0:
            assert np.max(np.abs(gout["pol"][i] - oout["pol"][j])) < 1e-9
            assert abs(gout["interaction_count"][i] - oout["interaction_count"][j]) <= 1e-9 * max(
                1e-12, abs(oout["interaction_count"][j]))


def test_lma_cp_plane_wave_collide_matches_oracle(eng, orc):
    if not orc.has_cp_cdf():
        pytest.skip("CP CDF table missing")
    laser = abi.laser_desc(abi.PLANE_WAVE, 2.0, 0.8e-6, abi.CIRCULAR, abi.COS2, n_cycles=8.0)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(24, g, sigma=0.001 * g, radius=0.0, length=2e-6, rms_div=0.0, laser=laser, seed=6)
    opts = abi.collide_options(rate_increase=1000.0)
    gout, gst = eng.collide(laser, opts, prim, seed=3)
    oout, ost = orc.collide(laser, opts, prim, seed=3, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    _compare_showers(gout, oout, tol=LMA_TOL)


# ---------------------------------------------- linear polarisation, LMA --
from kat_double_bessel import DB_KAT, DB_KAT_ABS, db_err  # noqa: E402


def test_double_bessel_device_kats(eng, orc):
    """Device J(n, x, y) by recurrence against the reference's known answers
    (double_bessel.rs:417-596, 1e-9) and the oracle (1e-11)."""
    pts = {}
    for n, fx, fy, t in DB_KAT:
        pts.setdefault(n, []).append((fx * n * math.sqrt(2.0), fy * 0.5 * n, t))
    for n, x, y, t in DB_KAT_ABS:
        pts.setdefault(n, []).append((x, y, t))
    for n, p in pts.items():
        x = np.array([q[0] for q in p])
        y = np.array([q[1] for q in p])
        j = eng.double_bessel(n, x, y, mode=0)
        for k, (xx, yy, t) in enumerate(p):
            assert db_err(j[k, 2], t) < 1e-9, (n, xx, yy, j[k, 2], t)
            ref = orc.double_bessel_at(n, n * math.sqrt(2.0), 0.5 * n, xx, yy)
            assert abs(j[k, 2] - ref) <= 1e-10 * abs(ref), (n, xx, yy, j[k, 2], ref)


@pytest.mark.parametrize("n", [12, 100, 700])
def test_double_bessel_device_evaluate(eng, orc, n):
    """The rate evaluation's J (saddle point where it applies) against the
    oracle over the whole (x, y) domain of order n: relative 1e-10, with an
    absolute floor of 1e-14 for the saddle-point form, whose cosine of an
    O(n) phase turns last-bit differences of the device's sin/cos into
    absolute errors near the zeros of J."""
    rng = np.random.default_rng(n)
    x = n * math.sqrt(2.0) * rng.random(200)
    y = 0.5 * n * rng.random(200)
    j = eng.double_bessel(n, x, y, mode=1)
    for k in range(200):
        ref = orc.double_bessel_evaluate(n, x[k], y[k])
        assert abs(j[k, 2] - ref) <= 1e-10 * abs(ref) + 1e-14, (x[k], y[k], j[k, 2], ref)


def test_lp_sampler_matches_oracle(eng, orc):
    """LP harmonic (CDF table), (s, theta) by rejection under the ceiling,
    and Stokes parameters: same streams, same samples."""
    a_vals = [0.3, 0.8, 1.414, 2.5, 4.0, 6.0]
    eta_vals = [2e-3, 0.03, 0.3]
    a, eta, streams = [], [], []
    for ai in a_vals:
        for ei in eta_vals:
            for k in range(24):
                a.append(ai)
                eta.append(ei)
                streams.append(1000 * len(a) + k)
    a, eta = np.array(a), np.array(eta)
    streams = np.array(streams, dtype=np.uint64)
    out, status = eng.lp_sample(a, eta, 99, streams, 7)
    mism = 0
    for i in range(len(a)):
        rc, ref = orc.lp_sample(a[i], eta[i], 99, int(streams[i]), 7)
        assert status[i] == rc
        if out[i, 0] != ref[0]:
            mism += 1
            continue
        assert abs(out[i, 1] - ref[1]) <= 1e-12 * ref[1]
        if abs(out[i, 2] - ref[2]) > 1e-12 * max(ref[2], 1.0):
            mism += 1
            continue
        assert np.max(np.abs(out[i, 4:6] - ref[4:6])) < 1e-9, (i, out[i], ref)
    assert mism <= 0.01 * len(a)


def test_lp_warp_sampler_equals_serial_sampler(eng):
    """The warp-cooperative LP sampler returns lp_sample's results bit for
    bit: same harmonic, (s, theta), Stokes parameters and status, over a
    range of a (including a > 5, where the ceiling scans 64 points) and
    eta."""
    a_vals = [0.3, 0.8, 1.414, 2.5, 4.0, 6.0, 9.0]
    eta_vals = [2e-3, 0.03, 0.3, 1.0]
    a, eta, streams = [], [], []
    for ai in a_vals:
        for ei in eta_vals:
            for k in range(40):
                a.append(ai)
                eta.append(ei)
                streams.append(7919 * len(a) + k)
    a, eta = np.array(a), np.array(eta)
    streams = np.array(streams, dtype=np.uint64)
    out_s, st_s = eng.lp_sample(a, eta, 5, streams, 3)
    out_w, st_w = eng.lp_sample(a, eta, 5, streams, 3, warp=True)
    assert np.array_equal(st_s, st_w)
    assert np.count_nonzero(st_s == 0) >= 0.95 * len(a)
    assert np.array_equal(out_s, out_w)


def test_cp_warp_sampler_equals_serial_sampler(eng, orc):
    """The warp-cooperative CP sampler returns cp_sample's results bit for
    bit (same harmonic, v, azimuth, Stokes parameters and status), and the
    serial sampler follows the oracle's restatement of
    nonlinear_compton/cp/mod.rs:181-234 on the same draws."""
    a_vals = [0.05, 0.3, 1.0, 2.5, 5.0, 12.0]
    eta_vals = [2e-3, 0.03, 0.3, 1.5]
    a, eta, streams = [], [], []
    for ai in a_vals:
        for ei in eta_vals:
            for k in range(40):
                a.append(ai)
                eta.append(ei)
                streams.append(104729 * len(a) + k)
    a, eta = np.array(a), np.array(eta)
    streams = np.array(streams, dtype=np.uint64)
    out_s, st_s = eng.cp_sample(a, eta, 9, streams, 4)
    out_w, st_w = eng.cp_sample(a, eta, 9, streams, 4, warp=True)
    assert np.array_equal(st_s, st_w)
    assert np.count_nonzero(st_s == 0) >= 0.99 * len(a)
    assert np.array_equal(out_s, out_w)
    mism = 0
    for i in range(0, len(a), 7):
        rc, ref = orc.cp_sample(a[i], eta[i], 9, int(streams[i]), 4)
        if rc != 0 or int(ref[0]) != int(out_s[i, 0]) or abs(out_s[i, 1] - ref[1]) > 1e-9 * max(abs(ref[1]), 1e-300):
            mism += 1
    assert mism <= 0.02 * (len(a) // 7 + 1), mism


def test_lma_lp_plane_wave_matches_oracle(eng, orc):
    """Linearly polarised plane wave (LMA), emission only, as in the
    plane-wave benchmark: electrons at 5 GeV, a0 = 1."""
    laser = abi.laser_desc(abi.PLANE_WAVE, 1.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=30.0)
    g = beam.gamma_from_energy(5.0)
    prim = beam.build(400, g, sigma=0.001 * g, radius=1e-6, length=10e-6, rms_div=0.0, laser=laser, seed=4)
    opts = abi.collide_options(tracking_photons=0)
    gout, gst = eng.collide(laser, opts, prim, seed=8)
    oout, ost = orc.collide(laser, opts, prim, seed=8, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["emissions"] > 20
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["emissions"] == pytest.approx(ost["emissions"], rel=0.03, abs=2)


def test_lma_lp_focused_matches_oracle(eng, orc):
    """Linearly polarised focused laser (LMA) at a0 = 3: harmonics beyond
    the saddle-point threshold."""
    laser = abi.laser_desc(abi.FOCUSED_LASER, 3.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=25e-15, pol_angle=0.3)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(40, g, sigma=0.001 * g, radius=1e-6, length=2e-6, rms_div=8e-6, laser=laser, seed=12)
    opts = abi.collide_options(tracking_photons=0)
    gout, gst = eng.collide(laser, opts, prim, seed=21)
    oout, ost = orc.collide(laser, opts, prim, seed=21, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["emissions"] > 20
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["emissions"] == pytest.approx(ost["emissions"], rel=0.03, abs=2)


def test_lma_lp_focused_pairs_match_oracle(eng, orc):
    """Photon beam on a linearly polarised focused laser (LMA): LP
    Breit-Wheeler rates (main and mid-range tables), Stokes update, harmonic
    inversion (regenerated mid-range CDF) and the (s, theta) sampler."""
    if not orc.has_lp_mid_cdf():
        pytest.skip("LP Breit-Wheeler mid-range CDF missing")
    laser = abi.laser_desc(abi.FOCUSED_LASER, 3.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15, pol_angle=0.2)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(120, g, sigma=0.001 * g, radius=1e-6, length=2e-6, rms_div=8e-6, laser=laser, seed=19,
                      species=abi.PHOTON, stokes=(0.4, -0.3, 0.2))
    opts = abi.collide_options(pol_resolved=1, rate_increase=300.0)
    gout, gst = eng.collide(laser, opts, prim, seed=29)
    oout, ost = orc.collide(laser, opts, prim, seed=29, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["pair_events"] >= 10
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["pair_events"] == pytest.approx(ost["pair_events"], rel=0.05, abs=2)


@pytest.mark.parametrize("pol", [abi.CIRCULAR, abi.LINEAR])
def test_lma_classical_matches_oracle(eng, orc, pol):
    """Classical radiation mode under the LMA (nonlinear_compton/{cp,lp}/
    classical.rs): table rates, harmonic CDFs, low-eta spectra and the
    Landau-Lifshitz push."""
    laser = abi.laser_desc(abi.PLANE_WAVE, 2.0, 0.8e-6, pol, abi.COS2, n_cycles=12.0)
    g = beam.gamma_from_energy(5.0)
    prim = beam.build(160, g, sigma=0.001 * g, radius=1e-6, length=4e-6, rms_div=0.0, laser=laser, seed=14)
    opts = abi.collide_options(classical=1, rr=1, tracking_photons=0)
    gout, gst = eng.collide(laser, opts, prim, seed=31)
    oout, ost = orc.collide(laser, opts, prim, seed=31, threads=8)
    assert ost["particle_errors"] == 0 and gst["particle_errors"] == 0
    assert ost["emissions"] > 30
    _compare_showers(gout, oout, tol=LMA_TOL)
    assert gst["emissions"] == pytest.approx(ost["emissions"], rel=0.03, abs=2)


@pytest.mark.parametrize("circular", [True, False])
def test_emission_rate_bound_covers_the_rate(eng, circular):
    """The emission step compares its draw first with an FP32 rate and
    decides in FP64 only where the draw falls within 2^-10 of it; the
    decision is the reference's only if the FP32 rate times (1 + 2^-10) is
    never below the FP64 rate.  Checked across the rate table and below its
    smallest amplitude (where the FP32 rate is an upper bound), and the
    bound is tight enough to spare the FP64 rate on most steps."""
    rng = np.random.default_rng(11 if circular else 12)
    m = 200_000
    a = np.exp(rng.uniform(np.log(1e-9), np.log(19.0), m))
    eta = np.exp(rng.uniform(np.log(1.1e-3), np.log(1.9), m))
    r32, r64, ok = eng.emission_rate_bound(a * a, eta, circular=circular)
    use = ~np.isnan(r32)
    assert use.mean() > 0.95, use.mean()
    assert np.all(ok[use])
    ratio = r32[use] / r64[use]
    assert np.all(ratio * (1.0 + 2.0 ** -10) >= 1.0), ratio.min()
    small = use & (a < 0.02)
    assert small.sum() > 1000
    assert np.all(r32[small] / r64[small] < 1.02)
    # a^2 = u.u - 1 at or below zero (rounding in the pulse's wings): both
    # rates are zero there, and the FP32 one applies
    a2 = np.concatenate([np.zeros(100), -np.exp(rng.uniform(np.log(1e-14), np.log(1e-6), 900))])
    eta = np.exp(rng.uniform(np.log(1e-4), np.log(1.9), a2.size))
    r32, r64, ok = eng.emission_rate_bound(a2, eta, circular=circular)
    assert np.all(ok) and np.all(r64 == 0.0) and np.all(r32 == 0.0)
