"""Photons that only drift and leptons outside the pulse.

An LCFA photon whose energy keeps its chi below 0.01 everywhere in the
field has T(chi) = 0 (lcfa/pair_creation/mod.rs:13-18) on every step, so
its steps in main.rs:212-264 only move it.  The device steps such a photon
by the same additions without evaluating the field, and, past 2^18 steps
(a photon moving almost with the laser), jumps to a few steps short of its
exit in closed form.  These tests put soft photons in every direction, some
of them nearly co-moving with the pulse, through the collision loop on the
GPU and in the oracle (which steps every one of them) and compare where
they leave.

Outside an LMA pulse (<a^2> < 2^-60) a lepton's step only drifts; the
plane-wave and focused LMA showers are compared with the oracle in
test_gpu_parity.py, and here a beam that starts far from the pulse is
checked particle by particle.
"""

import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    yield e
    e.close()


def _photons(directions, energies_mev, phase0, laser_k):
    n = len(directions)
    ell = np.array([e / 0.51099895 for e in energies_mev])
    d = np.array(directions, dtype=float)
    d /= np.linalg.norm(d, axis=1)[:, None]
    u = np.concatenate([ell[:, None], ell[:, None] * d], axis=1)
    rng = np.random.default_rng(4)
    x = 1e-6 * rng.standard_normal(n)
    y = 1e-6 * rng.standard_normal(n)
    # start at phase k (ct - z) = phase0 with z = 0
    r = np.stack([np.full(n, phase0 / laser_k), x, y, np.zeros(n)], axis=1)
    return {
        "species": np.full(n, abi.PHOTON, dtype=np.int32),
        "r": np.ascontiguousarray(r),
        "u": np.ascontiguousarray(u),
        "pol": np.ascontiguousarray(np.tile([1.0, 0.0, 0.0, 0.0], (n, 1))),
        "weight": np.ones(n),
        "id": np.arange(n, dtype=np.uint64),
        "parent_id": np.arange(n, dtype=np.uint64),
    }


def test_drifting_photons_leave_where_the_oracle_says(eng):
    from oracle import oracle
    oracle.build()
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    k = 2.0 * math.pi / 0.8e-6
    dirs, energies = [], []
    rng = np.random.default_rng(7)
    # soft photons in random directions (the pulse moves along +z)
    for _ in range(48):
        v = rng.standard_normal(3)
        dirs.append(v)
        energies.append(10 ** rng.uniform(-9, 0.5))
    # nearly along -z (the beam's direction) and nearly along +z, where the
    # phase advances by (1 - n_z) of its rate: 1e5 to 1e6 steps
    for eps in (1e-2, 3e-3, 1e-3):
        dirs.append([math.sqrt(2 * eps), 0.0, 1.0 - eps])
        energies.append(1e-6)
    dirs.append([0.01, 0.0, -1.0])
    energies.append(3.0)
    prim = _photons(dirs, energies, 100.0, k)
    opts = abi.collide_options(max_generation=-1)
    out, st = eng.collide(laser, opts, prim, seed=5)
    ref, rst = oracle.collide(laser, opts, prim, seed=5, threads=8)
    assert st["particle_errors"] == 0 and rst["particle_errors"] == 0
    # at least one photon went past the 2^18 steps stepped one by one
    assert st["max_steps"] > (1 << 18), st["max_steps"]
    # a nearly co-moving photon's phase k(ct - z) is a small difference of
    # large coordinates: rounding (the device's steps are the reference's
    # additions with c dt / ell^0 formed once) can move its last step across
    # the exit, so those four may each leave one step earlier or later
    assert abs(st["photon_steps"] - rst["photon_steps"]) <= 4, (st["photon_steps"], rst["photon_steps"])
    gi = {int(s): i for i, s in enumerate(out["stream"])}
    assert len(gi) == len(ref["stream"]) == len(dirs)
    dt = 0.1 / (2.0 * math.pi * 299792458.0 / 0.8e-6)
    for j, s in enumerate(ref["stream"]):
        i = gi[int(s)]
        assert np.array_equal(out["u"][i], ref["u"][j])
        n = ref["u"][j][1:] / ref["u"][j][0]
        d = out["r"][i] - ref["r"][j]
        scale = np.max(np.abs(ref["r"][j]))
        along = d[0]  # c t: one step is c dt
        assert abs(along) <= 1.01 * 299792458.0 * dt + 1e-9 * scale, (j, d)
        # both exits lie on the photon's line: x - n (ct) agrees to rounding
        assert np.max(np.abs(d[1:] - n * d[0])) <= 1e-9 * scale, (j, d)


def test_lma_beam_from_far_before_the_pulse(eng):
    """A CP LMA beam that starts far before the focused pulse (most of its
    steps field-free) matches the oracle particle by particle."""
    from oracle import oracle
    oracle.build()
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(200, g, sigma=0.001 * g, radius=1e-6, length=24e-6, rms_div=8e-6, laser=laser, seed=12)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    out, st = eng.collide(laser, opts, prim, seed=21)
    ref, rst = oracle.collide(laser, opts, prim, seed=21, threads=8)
    assert abs(st["lepton_steps"] - rst["lepton_steps"]) <= 0.01 * rst["lepton_steps"]
    gi = {int(s): i for i, s in enumerate(out["stream"])}
    common = [j for j, s in enumerate(ref["stream"]) if int(s) in gi]
    assert len(common) >= 0.97 * len(ref["stream"])
    bad = 0
    for j in common:
        i = gi[int(ref["stream"][j])]
        if np.max(np.abs(out["u"][i] - ref["u"][j])) > 5e-7 * np.linalg.norm(ref["u"][j]):
            bad += 1
    assert bad <= max(1, 0.02 * len(common))
