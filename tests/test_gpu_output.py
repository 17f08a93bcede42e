"""Histograms generated on the device (ptg_histogram) against the CPU
restatement of the reference (oracle/hgram.py) on the particles of a real
shower: the same extent and bins (exactly), totals and heights to the
rounding of a different summation order, and the same plain-text files."""

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam
from ptarmigan_gb300.output import DistributionFunction, UnitSystem

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
def shower(eng):
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(6000, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=4)
    out, st = eng.collide(laser, abi.collide_options(pol_resolved=1, max_generation=2), prim, seed=4)
    assert st["particle_errors"] == 0
    return out


def _device(p):
    import torch
    dev = torch.device("cuda", 0)
    return {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in p.items()}


SPECS = [
    ("energy:(log;energy)", abi.PHOTON, "auto"),
    ("energy:(auto;weight)", abi.ELECTRON, "hep"),
    ("angle_x:angle_y:(auto;weight)", abi.PHOTON, "auto"),
    ("theta:(100;weight)", abi.PHOTON, "auto"),
    ("px:py:(30;energy)", abi.ELECTRON, "si"),
    ("energy:(log;weight;energy in 1.602177e-11, auto)", abi.PHOTON, "auto"),
    ("pol_x:(50;weight)", abi.PHOTON, "auto"),
    ("S3:(20;pol_y)", abi.PHOTON, "auto"),
    ("r_perp:(log;helicity)", abi.PHOTON, "auto"),
    ("x:y:(log;weight)", abi.ELECTRON, "hep"),
    ("n_inter:(auto;weight)", abi.PHOTON, "auto"),
    ("gamma:(1000.0;weight)", abi.ELECTRON, "auto"),
]


@pytest.mark.parametrize("spec,species,units", SPECS)
def test_device_histogram_matches_restatement(eng, shower, spec, species, units):
    from oracle import hgram
    d = DistributionFunction.load(spec)
    us = UnitSystem.named(units)
    sp = d.spec(species, us)
    info, cts = eng.histogram(_device(shower), sp)
    filt = None if d.filter is None else (d.filter[1], d.filter[2], d.filter[3])
    ref = hgram.generate(shower, species, d.funcs, [sp.scale[k] for k in range(d.dim)], sp.weight, sp.bin_spec,
                         sp.n_bins, sp.bin_size, sp.height, filt)
    rinfo, rcts = ref
    assert info["bins"] == rinfo["bins"]
    # the device's atan2, hypot, log and exp may differ from the host's in
    # the last bits: extents agree to a few ulp, and a particle lying within
    # rounding of a bin edge may land in the neighbouring bin
    np.testing.assert_allclose(info["min"], rinfo["min"], rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(info["max"], rinfo["max"], rtol=1e-15, atol=1e-300)
    np.testing.assert_allclose(info["bin_size"], rinfo["bin_size"], rtol=1e-14)
    assert info["unweighted_total"] == rinfo["unweighted_total"]
    np.testing.assert_allclose(info["total"], rinfo["total"], rtol=1e-12)
    scale = np.max(np.abs(rcts))
    differ = ~np.isclose(cts, rcts, rtol=1e-9, atol=1e-12 * scale)
    assert differ.sum() <= 4, (differ.sum(), np.nonzero(differ))
    assert abs(np.sum(cts) - np.sum(rcts)) <= 1e-3 * np.sum(np.abs(rcts))
    assert np.count_nonzero(rcts) > 0


def test_plain_text_file_matches_restatement(eng, shower, tmp_path):
    from oracle import hgram
    from ptarmigan_gb300.output import Histogram
    d = DistributionFunction.load("angle_x:angle_y:(40;energy)")
    us = UnitSystem.default()
    path = d.write(eng, _device(shower), abi.PHOTON, us, str(tmp_path / "photon"))
    assert path.endswith("photon_angle_x-angle_y_energy-weight.dat")
    sp = d.spec(abi.PHOTON, us)
    rinfo, rcts = hgram.generate(shower, abi.PHOTON, d.funcs, [1.0, 1.0], sp.weight, sp.bin_spec, sp.n_bins,
                                 sp.bin_size, sp.height)
    ref_path = Histogram(rinfo, rcts, d.names, ["rad", "rad"]).write_plain_text(str(tmp_path / "ref"))
    got, want = open(path).read().splitlines(), open(ref_path).read().splitlines()
    assert got[:2] == want[:2] and len(got) == len(want) == 2 + 40 * 40
    bad = 0
    for a, b in zip(got[2:], want[2:]):
        fa, fb = a.split("\t"), b.split("\t")
        assert all(abs(float(x) - float(y)) <= 1e-14 * abs(float(y)) + 1e-300 for x, y in zip(fa[:2], fb[:2]))
        bad += abs(float(fa[2]) - float(fb[2])) > 1e-9 * max(abs(float(fb[2])), 1e-300)
    assert bad <= 4


def test_empty_species_gives_no_histogram(eng, shower):
    d = DistributionFunction.load("energy")
    info, cts = eng.histogram(_device(shower), d.spec(abi.POSITRON, UnitSystem.default())) \
        if not np.any(shower["species"] == abi.POSITRON) else (None, None)
    if info is not None:
        assert info["empty"] and cts is None


STATS = [
    ("mean energy", abi.PHOTON), ("total energy`weight", abi.PHOTON), ("fraction energy in (1.602177e-11; auto)", abi.PHOTON),
    ("variance angle_x", abi.ELECTRON), ("variance energy`weight for theta in (auto; 1e-3)", abi.PHOTON),
    ("min gamma", abi.ELECTRON), ("max gamma", abi.ELECTRON), ("circmean angle_y", abi.PHOTON),
    ("circvar theta", abi.PHOTON), ("cstd angle_x", abi.ELECTRON), ("mean S1`weight", abi.PHOTON),
    ("mean pol_x", abi.PHOTON),
]


@pytest.mark.parametrize("spec,species", STATS)
def test_device_statistics_match_restatement(eng, shower, spec, species):
    from oracle import hgram
    from ptarmigan_gb300.output import SummaryStatistic
    st = SummaryStatistic(spec)
    got = st.evaluate(eng, _device(shower), species, "photon" if species == abi.PHOTON else "electron")
    ff = st.filter[1] if st.filter else -1
    want = hgram.summary(shower, species, st.op, st.var_func, st.weight_func, ff, st.min, st.max)
    if st.op == "circvar":
        # 1 - R with R near 1: an absolute comparison of the resultant length
        assert abs(got - want) < 1e-13, (spec, got, want)
    elif st.op == "circstd":
        # sqrt(-2 ln R): compare -2 ln R, which the rounding of R moves by ~1e-16
        assert abs(got ** 2 - want ** 2) < 2e-13, (spec, got, want)
    else:
        assert got == pytest.approx(want, rel=1e-9, abs=1e-15), (spec, got, want)
    line = str(st)
    assert line.startswith(st.name + ": " + st.op + " ") and line.endswith("[%s]" % st.unit)
