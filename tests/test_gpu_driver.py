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
