"""An input file run end to end on the GPU (python -m ptarmigan_gb300):
distribution files and statistics written in the reference's formats,
consistent with each other, and a0 loops named as the reference names
them."""

import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INPUT = """---
control:
  lcfa: true
  radiation_reaction: true
  pair_creation: false
  rng_seed: 7
laser:
  a0: {a0}
  wavelength: 0.8 * micro
  n_cycles: 8.0
  polarization: linear
beam:
  n: 3000
  species: electron
  charge: 3000 * e
  gamma: 5.0 * GeV / (me * c^2)
  sigma: 0.001 * 5.0 * GeV / (me * c^2)
  radius: [1.0 * micro, normally_distributed]
  length: 2.0 * micro
output:
  ident: auto
  units: hep
  photon:
    - energy:(auto;weight)
    - angle_x:angle_y:(20;energy)
  electron:
    - gamma:(log;weight)
stats:
  expression:
    - nominal_a0 a0_value
  photon:
    - total number
    - mean energy
  electron:
    - mean gamma
constants:
  a0_value: 2.0
"""


def _read_dat(path):
    lines = open(path).read().splitlines()
    rows = np.array([[float(x) for x in l.split("\t")] for l in lines[2:]])
    return lines[0].split("\t"), lines[1].split("\t"), rows


def test_input_file_end_to_end(tmp_path):
    from ptarmigan_gb300.driver import run
    src = tmp_path / "collision.yml"
    src.write_text(INPUT.format(a0="2.0"))
    files = run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    names = sorted(os.path.basename(f) for f in files)
    assert names == ["collision_electron_gamma_log.dat", "collision_photon_angle_x-angle_y_energy-weight.dat",
                     "collision_photon_energy.dat", "collision_stats.txt"]
    axes, units, rows = _read_dat(str(tmp_path / "out" / "collision_photon_energy.dat"))
    assert axes == ["energy", "hgram/density/energy"] and units == ["GeV", "1/GeV"]
    width = rows[1, 0] - rows[0, 0]
    stats = open(str(tmp_path / "out" / "collision_stats.txt")).read().splitlines()
    # electron stats first, then photons, then expressions (main.rs:1268-1285)
    assert stats[0].startswith("electron: mean gamma = ") and stats[0].endswith("[1]")
    assert stats[1].startswith("photon: total number = ")
    assert stats[2].startswith("photon: mean energy = ") and stats[2].endswith("[MeV]")
    assert stats[3] == "expr: nominal_a0 = 2.000000e0 [1]"
    total = float(stats[1].split("=")[1].split("[")[0])
    # the density integrates to the photons' total weight (every energy is finite and binned but the maximum)
    assert np.sum(rows[:, 1]) * width == pytest.approx(total, rel=0.01)
    assert total > 100


def test_a0_loop_names_each_run(tmp_path):
    from ptarmigan_gb300.driver import run
    src = tmp_path / "scan.yml"
    src.write_text(INPUT.format(a0="\n    start: 1.0\n    stop: 2.0\n    step: 1.0"))
    files = run(str(src), str(tmp_path), log=lambda *a: None)
    names = {os.path.basename(f) for f in files}
    assert "scan_a0_1.000_photon_energy.dat" in names and "scan_a0_2.000_stats.txt" in names


def test_final_state_hdf5_dump(tmp_path):
    """output:dump_all_particles: hdf5 writes <ident>_particles.h5 with
    every final-state particle: its photon count and total weight match
    the statistics written from the same run."""
    from ptarmigan_gb300 import hdf5
    from ptarmigan_gb300.driver import run
    src = tmp_path / "dump.yml"
    text = INPUT.format(a0="2.0").replace("output:\n  ident: auto\n", "output:\n  ident: auto\n  dump_all_particles: hdf5\n")
    src.write_text(text)
    files = run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    h5 = [f for f in files if f.endswith("_particles.h5")]
    assert [os.path.basename(f) for f in h5] == ["dump_particles.h5"]
    f = hdf5.read(h5[0])["members"]
    ph = f["final-state"]["members"]["photon"]["members"]
    el = f["final-state"]["members"]["electron"]["members"]
    assert el["weight"]["value"].size == 3000
    stats = open(str(tmp_path / "out" / "dump_stats.txt")).read().splitlines()
    total = float(stats[1].split("=")[1].split("[")[0])
    assert np.sum(ph["weight"]["value"]) == pytest.approx(total, rel=1e-9)
    assert ph["position"]["value"].shape == (ph["weight"]["value"].size, 4)
    assert f["config"]["members"]["input-file"]["value"] == text
    # momenta in GeV/c (units: hep): the photons are on shell
    p = ph["momentum"]["value"]
    assert np.allclose(p[:, 0] ** 2, np.sum(p[:, 1:] ** 2, axis=1), rtol=1e-9)


STAGE2 = """---
control:
  lcfa: true
  pair_creation: true
  rng_seed: 3
laser:
  a0: 5.0
  wavelength: 0.8 * micro
  n_cycles: 8.0
  polarization: linear
beam:
  species: photon
  from_hdf5:
    file: out/dump_particles.h5
    distance_bt_ips: 0.0
output:
  ident: stage2
  dump_all_particles: hdf5
"""


def test_staged_run_loads_the_dump(tmp_path):
    """beam:from_hdf5 (particle/loader.rs): the photons of one run's
    final-state file are the primaries of the next."""
    from ptarmigan_gb300 import hdf5
    from ptarmigan_gb300.driver import run
    src = tmp_path / "dump.yml"
    text = INPUT.format(a0="2.0").replace("output:\n  ident: auto\n", "output:\n  ident: auto\n  dump_all_particles: hdf5\n")
    src.write_text(text)
    run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    first = hdf5.read(str(tmp_path / "out" / "dump_particles.h5"))["members"]["final-state"]["members"]
    n_photons = first["photon"]["members"]["weight"]["value"].size
    assert n_photons > 100
    src2 = tmp_path / "stage2.yml"
    src2.write_text(STAGE2)
    files = run(str(src2), str(tmp_path / "out2"), log=lambda *a: None)
    second = hdf5.read([f for f in files if f.endswith("_particles.h5")][0])["members"]
    assert second["config"]["members"]["beam"]["members"]["imported_from_file"]["value"] is True
    fs = second["final-state"]["members"]
    # photons leave as photons or as pairs; every primary is accounted for
    n2 = fs["photon"]["members"]["id"]["value"]
    assert n2.size + fs["electron"]["members"]["id"]["value"].size > 0
    assert n2.size <= n_photons


def _auto_ratio_oracle(laser, gamma):
    """main.rs:294-319 written out with the oracle's rates."""
    from oracle import oracle
    from ptarmigan_gb300 import abi
    from ptarmigan_gb300.input import COMPTON_TIME, SPEED_OF_LIGHT
    oracle.build()
    lam = laser.wavelength
    if laser.model in (abi.FAST_PLANE_WAVE, abi.FAST_FOCUSED_LASER):
        omega_mc2 = 1.26e-6 / (0.510999 * 1.0e6 * lam)
        chi = 2.0 * gamma * laser.a0 * omega_mc2
        pair, _ = oracle.lcfa_pair_probability([gamma, 0.0, 0.0, -gamma], [1.0, 0.0, 0.0, 0.0], chi, [1.0, 0.0, 0.0], 1.0)
        return oracle.lcfa_photon_rate(chi, gamma) / pair
    kk = SPEED_OF_LIGHT * COMPTON_TIME * 2.0 * math.pi / lam
    kappa = np.array([kk, 0.0, 0.0, kk])
    ell = np.array([gamma, 0.0, 0.0, -gamma])
    u = np.array([math.sqrt(1.0 + gamma * gamma), 0.0, 0.0, -gamma])
    pol = 1 if laser.polarization == abi.CIRCULAR else 0
    a_rms = laser.a0 if pol else laser.a0 / math.sqrt(2.0)
    ku = kappa[0] * u[0] - kappa[3] * u[3]
    q = u + a_rms * a_rms * kappa / (2.0 * ku)
    dt = lam / SPEED_OF_LIGHT
    pair, _ = oracle.bw_probability(ell, [1.0, 0.0, 0.0, 0.0], kappa, a_rms, dt, pol, 0.0)
    photon = oracle.nlc_probability(kappa, q, dt, pol)
    return 1.0 if pair == 0.0 else max(photon / pair, 1.0)


@pytest.mark.parametrize("model,pol,a0,energy", [(2, 1, 5.0, 16.5), (2, 0, 2.0, 10.0), (3, 0, 10.0, 10.0),
                                                 (0, 1, 1.0, 5.0)])
def test_automatic_pair_rate_increase(model, pol, a0, energy):
    """control:increase_pair_rate_by: auto (main.rs:294-319) on the device
    against the same formula over the oracle's rates."""
    from ptarmigan_gb300 import abi, beam, engine
    laser = abi.laser_desc(model, a0, 0.8e-6, pol, abi.GAUSSIAN, waist=4e-6, n_cycles=10.0)
    gamma = beam.gamma_from_energy(energy)
    eng = engine.Engine()
    try:
        got = eng.pair_rate_increase(laser, gamma)
    finally:
        eng.close()
    want = _auto_ratio_oracle(laser, gamma)
    # the device's exponentials and logarithms in the rate interpolation
    # against the host's: agreement to a few parts in 1e9
    assert got == pytest.approx(want, rel=1e-7)
    assert got >= 1.0


AUTO = """---
control:
  lcfa: false
  pair_creation: true
  pol_resolved: true
  increase_pair_rate_by: auto
  stop_at_time: {stop}
  rng_seed: 5
laser:
  a0: 5.0
  wavelength: 0.8 * micro
  waist: 3.0 * micro
  fwhm_duration: 30.0 * femto
  polarization: circular
beam:
  n: 2000
  species: electron
  gamma: 1.0
  spectrum:
    function: exp(-((gamma - 32000.0) / 300.0)^2)
    min: 31000.0
    max: 33000.0
  radius: [1.0 * micro, normally_distributed]
  length: 5.0 * micro
output:
  ident: auto
  dump_all_particles: hdf5
"""


def test_auto_rate_stop_time_and_spectrum(tmp_path):
    """One LMA run with a tabulated beam spectrum, the automatic pair-rate
    increase and stop_at_time: auto: every final-state particle ends at the
    same time coordinate, the file records the rate increase, and the
    pairs carry the biased weight 1 / rate."""
    from ptarmigan_gb300 import hdf5
    from ptarmigan_gb300.driver import run
    src = tmp_path / "auto.yml"
    src.write_text(AUTO.format(stop="auto"))
    files = run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    assert [os.path.basename(f) for f in files] == ["auto_particles.h5"]
    f = hdf5.read(str(tmp_path / "out" / "auto_particles.h5"))["members"]
    ctl = f["config"]["members"]["control"]["members"]
    rate = ctl["increase_pair_rate_by"]["value"]
    assert rate > 1.0
    t_stop = ctl["stop_at_time"]["value"]
    fs = f["final-state"]["members"]
    for sp in ("photon", "electron", "positron"):
        x = fs[sp]["members"]["position"]["value"]
        if x.size:
            # positions in metres (auto units): c t = c t_stop for every particle
            np.testing.assert_allclose(x[:, 0], 2.997925e8 * t_stop, rtol=1e-12)
    w = fs["positron"]["members"]["weight"]["value"]
    if w.size:
        assert np.all(w <= 1.0 / rate * (1.0 + 1e-12))
    assert fs["electron"]["members"]["id"]["value"].size >= 2000


INTERMEDIATE = """---
control:
  lcfa: true
  pair_creation: true
  rng_seed: 9
laser:
  a0: 30.0
  wavelength: 0.8 * micro
  waist: 2.0 * micro
  fwhm_duration: 30.0 * femto
  polarization: linear
beam:
  n: 300
  species: electron
  gamma: 10.0 * GeV / (me * c^2)
  radius: [0.5 * micro, normally_distributed]
  length: 2.0 * micro
output:
  ident: inter
  dump_all_particles: hdf5
  dump_decayed_photons: true
  intermediate:
    - energy:(20;weight)
stats:
  intermediate:
    - total number
  photon:
    - total number
"""


def test_decayed_photons_are_written(tmp_path):
    """The photons that decay into pairs are kept (keep_decayed_photons)
    when an output asks for them: they fill the HDF5 file's
    intermediate-state group and their own distribution file, one per pair,
    and they are not in the final state."""
    from ptarmigan_gb300 import hdf5
    from ptarmigan_gb300.driver import run
    src = tmp_path / "inter.yml"
    src.write_text(INTERMEDIATE)
    files = run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    names = sorted(os.path.basename(f) for f in files)
    assert "inter_intermediate_energy.dat" in names and "inter_particles.h5" in names
    f = hdf5.read(str(tmp_path / "out" / "inter_particles.h5"))["members"]
    inter = f["intermediate-state"]["members"]["photon"]["members"]
    ids = inter["id"]["value"]
    assert ids.size > 0
    fs = f["final-state"]["members"]
    # each decayed photon made one pair: it is the parent of a positron
    pos_parent = set(int(x) for x in fs["positron"]["members"]["parent_id"]["value"])
    assert set(int(x) for x in ids) <= pos_parent
    assert not set(int(x) for x in ids) & set(int(x) for x in fs["photon"]["members"]["id"]["value"])
    axes, units, rows = _read_dat(str(tmp_path / "out" / "inter_intermediate_energy.dat"))
    width = rows[1, 0] - rows[0, 0]
    # the density integrates to the photons in the bins (the largest energy
    # can fall past the last bin edge)
    assert abs(np.sum(rows[:, 1]) * width - ids.size) <= 1.0 + 1e-6 * ids.size


def test_given_stop_time_moves_every_particle(tmp_path):
    from ptarmigan_gb300 import hdf5
    from ptarmigan_gb300.driver import run
    src = tmp_path / "given.yml"
    src.write_text(AUTO.format(stop="200.0 * femto"))
    run(str(src), str(tmp_path / "out"), log=lambda *a: None)
    f = hdf5.read(str(tmp_path / "out" / "given_particles.h5"))["members"]
    assert f["config"]["members"]["control"]["members"]["stop_at_time"]["value"] == pytest.approx(2e-13)
    x = f["final-state"]["members"]["electron"]["members"]["position"]["value"]
    np.testing.assert_allclose(x[:, 0], 2.997925e8 * 2e-13, rtol=1e-12)


def test_chirped_plane_wave_energy_flux():
    """FastPlaneWave::integrated_intensity (fast_plane_wave.rs:56-85) for a
    chirp so small that the pulse is the unchirped one: the numerical
    energy flux equals the closed form of fast_plane_wave.rs:204-236."""
    from ptarmigan_gb300 import abi, driver, engine
    eng = engine.Engine()
    try:
        for env in (abi.COS2, abi.GAUSSIAN):
            flat = abi.laser_desc(abi.PLANE_WAVE, 2.0, 0.8e-6, abi.LINEAR, env, n_cycles=10.0)
            chirped = abi.laser_desc(abi.PLANE_WAVE, 2.0, 0.8e-6, abi.LINEAR, env, n_cycles=10.0, chirp_b=1e-9)
            num = driver.chirped_energy_flux(chirped, eng)
            closed, unit = driver.laser_energy(flat)
            assert unit == "J/m^2"
            assert num == pytest.approx(closed, rel=2e-3)
    finally:
        eng.close()
