"""The input reader: the YAML subset of ptarmigan's input files, the
expression evaluator with the reference's constants and functions
(input/mod.rs:56-140), a0 loops (input/mod.rs:239-263) and the mapping of
the laser, beam and control sections (main.rs:339-811)."""

import math

import pytest

from ptarmigan_gb300 import abi
from ptarmigan_gb300.input import Input, InputError, evaluate, parse_yaml

DOC = """---
# a comment
control:
  lcfa: true          # trailing comment
  rng_seed: 3
  increase_pair_rate_by: 1.0e3
laser:
  a0:
    start: 1.0
    stop: 2.0
    step: 0.5
  wavelength: wavelength
  waist: 4.0 * micro
  fwhm_duration: 30.0 * femto
  polarization: "linear || y"
beam:
  n: 5000
  species: electron
  charge: 1.0e9 * e
  gamma: 10.0 * GeV / (me * c^2)
  sigma: 0.01 * 10.0 * GeV / (me * c^2)
  radius: [2.0 * micro, normally_distributed, 6.0 * micro]
  length: 20.0 * micro
  collision_angle: 2.0 * degree
  collision_plane: vertical
  offset: [0.0, 1.0 * micro, 0.0]
output:
  photon:
    - energy:(log;energy)
    - angle_x:angle_y
stats:
  photon:
    - mean energy
constants:
  wavelength: 0.8 * micro
"""


def test_yaml_subset():
    d = parse_yaml(DOC)
    assert d["control"]["lcfa"] == "true" and d["control"]["rng_seed"] == "3"
    assert d["laser"]["a0"] == {"start": "1.0", "stop": "2.0", "step": "0.5"}
    assert d["laser"]["polarization"] == "linear || y"
    assert d["beam"]["radius"] == ["2.0 * micro", "normally_distributed", "6.0 * micro"]
    assert d["output"]["photon"] == ["energy:(log;energy)", "angle_x:angle_y"]
    with pytest.raises(InputError):
        parse_yaml("a:\n\tb: 1\n")


def test_expressions():
    ctx = {"x": 2.0}
    assert evaluate("1 + 2 * 3", ctx) == 7.0
    assert evaluate("-x^2", ctx) == -4.0
    assert evaluate("(1 + x)^2 / 3", ctx) == 3.0
    assert evaluate("sqrt(16) + atan2(0, 1) + step(0.5, 0, 1)", ctx) == 5.0
    assert evaluate("1.5e-3 * 2", ctx) == 3.0e-3
    for bad in ("1 +", "y", "nope(1)", "2 $ 3"):
        with pytest.raises(InputError):
            evaluate(bad, ctx)


def test_sections_map_to_the_abi():
    from ptarmigan_gb300 import driver
    inp = Input(DOC)
    assert inp.loop("laser:a0") == [1.0, 1.5, 2.0]
    laser = driver.laser_from_input(inp, 1.5)
    assert laser.model == abi.FAST_FOCUSED_LASER and laser.polarization == abi.LINEAR
    assert laser.pol_angle == math.pi / 2 and laser.envelope == abi.GAUSSIAN
    assert laser.n_cycles == pytest.approx(2.997925e8 * 30e-15 / 0.8e-6)
    desc, n, species, angle, plane = driver.beam_from_input(inp, laser)
    assert n == 5000 and species == abi.ELECTRON and plane == math.pi / 2
    assert desc.radial_dstr == abi.RADIAL_TRUNC_NORMAL and desc.x_max == pytest.approx(6e-6)
    assert desc.weight == pytest.approx(2.0e5)  # |charge| / (e n) = 1e9 / 5000
    assert desc.gamma_mean == pytest.approx(10.0e3 / 0.5109989, rel=1e-5)
    opts = driver.options_from_input(inp, False)
    assert opts.rate_increase == 1.0e3 and opts.tracking_photons == 1 and opts.classical == 0


def test_beam_basis_rotation_undoes_the_collision_angle():
    """A particle moving along the beam's axis moves along +z in beam
    coordinates (Particle::to_beam_coordinate_basis)."""
    import numpy as np
    from ptarmigan_gb300.driver import to_beam_basis
    theta, phi = 0.3, 0.4
    # beam centroid direction (-cos phi sin theta, -sin theta sin phi, -cos theta)
    d = np.array([-math.cos(phi) * math.sin(theta), -math.sin(theta) * math.sin(phi), -math.cos(theta)])
    out = {k: np.zeros((1, 4)) for k in ("u", "u0", "r", "r0")}
    out["u"][0, 1:] = 100.0 * d
    to_beam_basis(out, theta, phi)
    np.testing.assert_allclose(out["u"][0, 1:] / 100.0, [0.0, 0.0, 1.0], atol=1e-12)


SPECTRUM = """---
beam:
  n: 1000
  gamma: 1.0
  spectrum:
    function: gamma * exp(-gamma / 2000.0)
    min: 1000.0
    max: 4000.0
    resolution: 30
control:
  stop_at_time: auto
"""


def test_spectrum_function_and_cdf():
    """beam:spectrum:function (main.rs:610-636) and GammaDistribution::custom
    (particle/dstr.rs:88-106): 30 values from min in steps of
    (max - min) / 30, a CDF from [min, 0] to [max, 1]."""
    import numpy as np
    from ptarmigan_gb300 import driver
    inp = Input(SPECTRUM)
    vals, g0, g1, step = driver.spectrum_from_input(inp, 1000)
    assert len(vals) == 30 and g0 == 1000.0 and g1 == 4000.0 and step == 100.0
    assert vals[0] == pytest.approx(1000.0 * math.exp(-0.5))
    cdf = driver.custom_cdf(vals, g0, step)
    assert cdf.shape == (31, 2) and cdf[0, 1] == 0.0 and cdf[-1, 1] == pytest.approx(1.0, abs=1e-15)
    assert cdf[-1, 0] == pytest.approx(4000.0)
    assert np.all(np.diff(cdf[:, 0]) > 0) and np.all(np.diff(cdf[:, 1]) >= 0)
    g = np.array([g0 + i * step for i in range(30)])
    assert driver.spectrum_mean_gamma(vals, g0, step) == pytest.approx(np.sum(g * vals) / np.sum(vals))
    assert driver.stop_mode(inp) == "auto"


def test_spectrum_file(tmp_path):
    """beam:spectrum:file, one value per line relative to the input file,
    over [min, min + n step]."""
    from ptarmigan_gb300 import driver
    (tmp_path / "spec.txt").write_text("1.0\n2.0\n3.0\n2.0\n1.0\n")
    inp = Input("beam:\n  spectrum:\n    file: spec.txt\n    min: 100.0\n    step: 50.0\n")
    vals, g0, g1, step = driver.spectrum_from_input(inp, 10, str(tmp_path / "in.yml"))
    assert vals == [1.0, 2.0, 3.0, 2.0, 1.0] and g0 == 100.0 and step == 50.0 and g1 == 300.0
    bad = Input("beam:\n  spectrum:\n    file: spec.txt\n    function: gamma\n    min: 1.0\n    max: 2.0\n")
    with pytest.raises(InputError):
        driver.spectrum_from_input(bad, 10, str(tmp_path / "in.yml"))


def test_stop_at_time_modes():
    from ptarmigan_gb300 import driver
    assert driver.stop_mode(Input("control:\n  stop_at_time: 3.0e-13\n")) == pytest.approx(3.0e-13)
    assert driver.stop_mode(Input("control:\n  dt_multiplier: 1.0\n")) is None
    opts = driver.options_from_input(Input("control:\n  stop_at_time: 2 * femto\n"), False)
    assert opts.t_stop == pytest.approx(2e-15)
    assert math.isinf(driver.options_from_input(Input("control:\n  stop_at_time: auto\n"), False).t_stop)


def test_project_to_time():
    import numpy as np
    from ptarmigan_gb300 import driver
    parts = {"r": np.array([[1.0, 0.0, 0.0, 0.0], [2.0, 1.0, 0.0, 1.0]]),
             "u": np.array([[2.0, 1.0, 1.0, 1.0], [10.0, 0.0, 6.0, 8.0]])}
    driver._project_to_time(parts, 3.0)
    np.testing.assert_allclose(parts["r"], [[3.0, 1.0, 1.0, 1.0], [3.0, 1.0, 0.6, 1.8]])
