"""The final-state HDF5 file of the input driver (output:dump_all_particles:
hdf5), written from synthetic particles on the CPU and read back: the
reference's layout (main.rs:1289-1715), units, attributes and aliases; and
the laser energy against the reference's own test."""
import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi, driver, hdf5
from ptarmigan_gb300.input import Input
from ptarmigan_gb300.output import UnitSystem

INPUT = """---
control:
  lcfa: true
  rng_seed: 9
laser:
  a0: 5.0
  wavelength: 0.8 * micro
  waist: 4.0 * micro
  fwhm_duration: 30.0 * femto
  polarization: circular
beam:
  n: 100
  species: electron
  charge: 100 * e
  gamma: 2000.0
  sigma: 2.0
  radius: [1.0 * micro, normally_distributed]
  length: 2.0 * micro
  offset: [0.0, 1.0 * micro, 0.0]
output:
  dump_all_particles: hdf5
  units: hep
"""


def _particles(rng):
    m = 30
    species = np.array([abi.ELECTRON] * 10 + [abi.PHOTON] * 15 + [abi.POSITRON] * 5, dtype=np.int32)
    out = {"species": species}
    for k in ("r", "u", "r0", "u0", "pol"):
        out[k] = rng.normal(size=(m, 4))
    for k in ("weight", "payload", "parent_chi", "interaction_count", "work"):
        out[k] = rng.random(m)
    for k in ("id", "parent_id", "primary", "stream"):
        out[k] = rng.integers(0, 1 << 40, m).astype(np.uint64)
    for k in ("generation", "flags", "status"):
        out[k] = np.zeros(m, dtype=np.int32)
    return out


def test_final_state_file_layout(tmp_path):
    path = tmp_path / "run.yml"
    path.write_text(INPUT)
    inp = Input.from_file(str(path))
    laser = driver.laser_from_input(inp, 5.0)
    desc, n, species, angle, plane = driver.beam_from_input(inp, laser)
    opts = driver.options_from_input(inp, keep_decayed=False)
    out = _particles(np.random.default_rng(2))
    units = UnitSystem.named("hep")
    fname = str(tmp_path / "run_particles.h5")
    driver.write_particles_hdf5(fname, inp, str(path), laser, 5.0, desc, n, species, angle, plane, opts, out,
                                units, True, 123)
    f = hdf5.read(fname)["members"]
    assert set(f) == {"build", "config", "final-state"}
    cfg = f["config"]["members"]
    assert cfg["input-file"]["value"] == INPUT
    assert cfg["unit"]["members"]["position"]["value"] == "mm"
    assert cfg["unit"]["members"]["momentum"]["value"] == "GeV/c"
    ctl = cfg["control"]["members"]
    assert ctl["lcfa"]["value"] is True and ctl["rng_seed"]["value"] == 9
    las = cfg["laser"]["members"]
    assert las["polarization"]["value"] == "circular" and las["envelope"]["value"] == "gaussian"
    assert las["a0"]["value"] == 5.0 and las["a0"]["attrs"]["unit"] == "1"
    assert las["wavelength"]["value"] == pytest.approx(0.8e-3)  # mm
    assert las["fwhm_duration"]["value"] == pytest.approx(30e-15, rel=1e-6)
    assert "polarization_angle" not in las and "n_cycles" not in las
    bm = cfg["beam"]["members"]
    assert bm["n"]["value"] == 100 and bm["species"]["value"] == "electron"
    assert bm["charge"]["value"] == pytest.approx(-100 * 1.602177e-19, rel=1e-6)
    assert bm["offset"]["type"] == "array" and np.allclose(bm["offset"]["value"], [0.0, 1e-3, 0.0])
    assert bm["polarisation"]["addr"] == bm["polarization"]["addr"]
    assert bm["imported_from_file"]["value"] is False
    fs = f["final-state"]["members"]
    assert set(fs) == {"photon", "electron", "positron", "laser"}
    ph = fs["photon"]["members"]
    assert set(ph) == {"weight", "a0_at_creation", "xi", "parent_chi", "n_pos", "id", "parent_id", "polarization",
                       "polarisation", "position", "momentum"}
    sel = out["species"] == abi.PHOTON
    assert np.array_equal(ph["weight"]["value"], out["weight"][sel])
    assert np.allclose(ph["position"]["value"], out["r"][sel] * 1e3)
    assert np.allclose(ph["momentum"]["value"], out["u"][sel] * 0.510999e-3)
    assert ph["momentum"]["attrs"] == {"desc": "four-momentum of the photon", "unit": "GeV/c"}
    assert ph["xi"]["addr"] == ph["a0_at_creation"]["addr"]
    el = fs["electron"]["members"]
    assert set(el) == {"weight", "n_gamma", "id", "parent_id", "absorption", "position", "momentum"}
    sel = out["species"] == abi.ELECTRON
    assert np.array_equal(el["id"]["value"], out["id"][sel])
    assert np.allclose(el["absorption"]["value"], out["work"][sel] * 0.510999e-3)
    assert el["absorption"]["attrs"]["unit"] == "GeV"
    po = fs["positron"]["members"]
    assert {"position_at_creation", "a0_at_creation", "xi", "parent_chi"} <= set(po)
    lz = fs["laser"]["members"]
    assert lz["energy"]["attrs"]["unit"] == "J" and lz["energy"]["value"] > 0
    expect = float(np.sum(out["weight"] * out["work"])) * 0.510999 * 1e6 * 1.602177e-19
    assert lz["absorption"]["value"] == pytest.approx(expect, rel=1e-12)


def test_laser_energy_matches_reference_test():
    """field/fast_focused_laser.rs:292-314: a LUXE-like pulse of 1.2 J
    (relative error < 1e-3)."""
    wl, a0 = 0.8e-6, 3.0
    waist = 147.839 * math.sqrt(1.2) * wl / (a0 * math.sqrt(30.0))
    las = abi.laser_desc(abi.FAST_FOCUSED_LASER, a0, wl, abi.CIRCULAR, abi.GAUSSIAN, waist=waist,
                         fwhm_duration=30e-15)
    e, unit = driver.laser_energy(las)
    assert unit == "J" and abs(e - 1.2) / 1.2 < 1e-3
    # the plane-wave form is the same pulse per unit area, and a chirp has none
    pw = abi.laser_desc(abi.FAST_PLANE_WAVE, a0, wl, abi.LINEAR, abi.COS2, n_cycles=10.0)
    assert driver.laser_energy(pw)[1] == "J/m^2"
    chirped = abi.laser_desc(abi.PLANE_WAVE, a0, wl, abi.LINEAR, abi.COS2, n_cycles=10.0, chirp_b=1e-3)
    assert driver.laser_energy(chirped) is None


def _write_dump(tmp_path, laser_defines_z):
    path = tmp_path / "run.yml"
    path.write_text(INPUT)
    inp = Input.from_file(str(path))
    laser = driver.laser_from_input(inp, 5.0)
    desc, n, species, angle, plane = driver.beam_from_input(inp, laser)
    opts = driver.options_from_input(inp, keep_decayed=False)
    out = _particles(np.random.default_rng(3))
    out["u"][:, 0] = np.sqrt(1.0 + np.sum(out["u"][:, 1:] ** 2, axis=1)) + 1.0  # positive energies
    fname = str(tmp_path / "dump.h5")
    driver.write_particles_hdf5(fname, inp, str(path), laser, 5.0, desc, n, species, angle, plane, opts, out,
                                UnitSystem.named("hep"), laser_defines_z, 1)
    return fname, out


def test_loader_reads_the_final_state_back(tmp_path):
    """BeamLoader (particle/loader.rs:142-284) on this package's own file:
    no rotation when the file's beam axis is the collision axis, no
    timing shift without auto timing; ids are row indices."""
    fname, out = _write_dump(tmp_path, laser_defines_z=True)
    prim = driver.load_beam_hdf5(fname, abi.PHOTON, 0.0, 0.0, (0.0, 0.0, 0.0), False, 0.0, math.pi, 0.0)
    sel = out["species"] == abi.PHOTON
    assert np.allclose(prim["r"], out["r"][sel], rtol=1e-14, atol=1e-20)
    assert np.allclose(prim["u"], out["u"][sel], rtol=1e-14)
    assert np.array_equal(prim["pol"], out["pol"][sel])
    assert np.array_equal(prim["id"], np.arange(sel.sum(), dtype=np.uint64))
    # energy filter (MeV) and the offset
    e = 0.510999 * out["u"][sel][:, 0]
    es = np.sort(e)
    cut = float(0.5 * (es[7] + es[8]))  # between two energies, clear of rounding
    prim = driver.load_beam_hdf5(fname, abi.PHOTON, 0.0, 0.0, (1e-6, 0.0, 2e-6), False, cut, math.pi, 0.0)
    assert len(prim["weight"]) == int(np.sum(e > cut))
    keep = e > cut
    assert np.allclose(prim["r"][:, 1], out["r"][sel][keep][:, 1] + 1e-6)
    assert np.allclose(prim["r"][:, 3], out["r"][sel][keep][:, 3] + 2e-6)


def test_loader_rotates_a_beam_defined_axis(tmp_path):
    """A file whose beam defines +z is turned onto the collision axis -z (a
    rotation by pi about y); auto timing moves particles along their
    velocity, to a fixed light-cone coordinate t - z = -2 initial_z."""
    fname, out = _write_dump(tmp_path, laser_defines_z=False)
    sel = out["species"] == abi.ELECTRON
    prim = driver.load_beam_hdf5(fname, abi.ELECTRON, 0.0, 0.0, (0.0, 0.0, 0.0), False, 0.0, math.pi, 0.0)
    assert np.allclose(prim["u"][:, 1], -out["u"][sel][:, 1]) and np.allclose(prim["u"][:, 3], -out["u"][sel][:, 3])
    assert np.allclose(prim["u"][:, 2], out["u"][sel][:, 2])
    z0 = 5e-6
    prim = driver.load_beam_hdf5(fname, abi.ELECTRON, 0.0, 0.0, (0.0, 0.0, 0.0), True, 0.0, math.pi, z0)
    r = prim["r"]
    assert np.allclose(r[:, 0] - r[:, 3], -2.0 * z0, atol=1e-18)
