"""Distribution-output host logic: spec parsing (DistributionFunction::load,
output/mod.rs:173-255), file suffixes (:268-318), unit systems
(output/units.rs) and the plain-text format (output/hgram.rs:530-562)."""

import math

import numpy as np
import pytest

from ptarmigan_gb300 import abi
from ptarmigan_gb300.output import DistributionFunction, Histogram, UnitSystem, rust_exp


def test_rust_exponent_format():
    assert rust_exp(1234.5) == "1.234500000e3"
    assert rust_exp(1.5e-5) == "1.500000000e-5"
    assert rust_exp(0.0) == "0.000000000e0"
    assert rust_exp(-3.1e12) == "-3.100000000e12"
    assert rust_exp(float("nan")) == "NaN" and rust_exp(float("inf")) == "inf"


def test_load_specs_like_the_reference():
    d = DistributionFunction.load("angle_x:angle_y:(100;auto)")  # output/mod.rs:335-343
    assert d.dim == 2 and d.bin_spec == (abi.BINS_FIXED_NUMBER, 100, 0.0) and d.weight == "auto"
    assert d.suffix() == "_angle_x-angle_y"
    d = DistributionFunction.load("energy:(log;energy)")
    assert d.bin_spec[0] == abi.BINS_LOG and d.suffix() == "_energy_energy-weight_log"
    d = DistributionFunction.load("p-:(2.5;weight)")
    assert d.names == ["p_minus"] and d.bin_spec == (abi.BINS_FIXED_SIZE, 0, 2.5)
    d = DistributionFunction.load("theta:(auto;pol_x;energy in 1.602177e-10, auto)")
    assert d.filter[0] == "energy" and d.filter[3] == math.inf
    # 1e-10 J in the default unit (MeV), by the reciprocal of the SI scale
    assert d.filter[2] == 1.602177e-10 * (1.0 / (1.0e6 * 1.602177e-19))
    assert d.suffix() == "_theta_pol_x-weight_energy-cut"
    d = DistributionFunction.load("x")
    assert d.dim == 1 and d.bin_spec[0] == abi.BINS_AUTO and d.weight == "weight"
    for bad in ("nonsense", "energy:(auto;nonsense)", "x:y:z", "energy:(auto;weight;energy between 1, 2)"):
        with pytest.raises(ValueError):
            DistributionFunction.load(bad)


def test_unit_systems():
    hep, si = UnitSystem.hep(), UnitSystem.si()
    assert hep.energy.name == "GeV" and hep.energy.scale == 1.0e-3 and hep.length.scale == 1.0e3
    assert si.energy.name == "J" and si.momentum.name == "kg/m/s"
    assert UnitSystem.named("auto").energy.name == "MeV"
    with pytest.raises(ValueError):
        UnitSystem.named("cgs")


def test_plain_text_layout(tmp_path):
    info = {"dim": 2, "bins": [2, 3], "min": [0.0, 10.0], "max": [2.0, 13.0], "bin_size": [1.0, 1.0],
            "total": 6.0, "unweighted_total": 6.0}
    h = Histogram(info, np.arange(6, dtype=float), ["x", "y"], ["m", "m"])
    path = h.write_plain_text(str(tmp_path / "out"))
    lines = open(path).read().splitlines()
    assert lines[0] == "x\ty\thgram/density/x_y" and lines[1] == "m\tm\t1/(m.m)"
    # row-major: the first axis runs fastest
    assert lines[2] == "5.000000000e-1\t1.050000000e1\t0.000000000e0"
    assert lines[3] == "1.500000000e0\t1.050000000e1\t1.000000000e0"
    assert lines[4] == "5.000000000e-1\t1.150000000e1\t2.000000000e0"
    assert len(lines) == 8


def test_oracle_histogram_on_known_points():
    """The restatement's binning on a hand-made set: 1d counts and the
    reference's 2d row index (bin[1] * nbins[1] + bin[0])."""
    from oracle import hgram
    n = 8
    p = {"species": np.zeros(n, dtype=np.int32), "u": np.zeros((n, 4)), "r": np.zeros((n, 4)),
         "pol": np.tile([1.0, 0, 0, 0], (n, 1)), "weight": np.ones(n)}
    p["r"][:, 1] = np.arange(n)  # x = 0..7
    info, cts = hgram.generate(p, 0, [16], [1.0], 0, 2, n_bins=4, height=0)
    assert info["bins"] == [4] and info["min"] == [0.0] and info["max"] == [7.0]
    assert list(cts) == [2.0, 2.0, 2.0, 1.0]  # the maximum lands past the last bin
    assert info["total"] == 8.0


def test_fits_layout(tmp_path):
    info = {"dim": 2, "bins": [3, 2], "min": [-1.0, 0.25], "max": [2.0, 1.0], "bin_size": [1.0, 0.375],
            "total": 12.5, "unweighted_total": 7.0}
    cts = np.array([0.5, -1.0, 2.0, 3.0, 0.0, 4.5])
    h = Histogram(info, cts, ["angle_x", "angle_y"], ["rad", "rad"])
    path = h.write_fits(str(tmp_path / "h"))
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0 and len(raw) == 2 * 2880
    cards = [raw[i:i + 80].decode() for i in range(0, 2880, 80)]
    assert cards[0].startswith("SIMPLE  =                    T / file conforms to FITS standard")
    assert cards[1].startswith("BITPIX  =                  -64 /")
    assert cards[2].startswith("NAXIS   =                    2 /")
    assert cards[3].startswith("NAXIS1  =                    3 /") and cards[4].startswith("NAXIS2  =                    2 /")
    assert cards[6] == "CRPIX1  = " + "5.000000000E-1".rjust(20) + " " * 50
    assert cards[7] == "CRVAL1  = " + "-1.000000000E0".rjust(20) + " " * 50
    assert cards[9] == "CNAME1  = 'angle_x'" + " " * 61
    names = [c[:8] for c in cards]
    i = names.index("DATAMIN ")
    assert cards[i].split("=")[1].strip() == "-1.000000000E0" and cards[i + 1].split("=")[1].strip() == "4.500000000E0"
    assert "END" + " " * 77 in cards
    data = np.frombuffer(raw[2880:2880 + 48], dtype=">f8")
    assert np.array_equal(data, cts) and raw[2880 + 48:] == b"\0" * (2880 - 48)


def test_summary_statistic_display(tmp_path):
    from ptarmigan_gb300.output import SummaryStatistic, write_stats
    st = SummaryStatistic("fraction energy in (1.602177e-13; auto)")
    st.name, st.value = "electron", 0.561
    assert str(st) == "electron: fraction energy (energy [MeV] > 1.000000e0) = 5.610000e-1 [1]"
    st = SummaryStatistic("mean energy`weight for r_perp in (1e-3; 2e-3)")
    st.name, st.value = "photon", 1000.0
    assert str(st) == ("photon: mean energy (weight-weighted) (1.000000e-3 < r_perp [1] < 2.000000e-3) "
                       "= 1.000000e3 [MeV]")
    st2 = SummaryStatistic("variance x")
    st2.name, st2.value = "positron", 2.5e-12
    assert str(st2) == "positron: variance x = 2.500000e-12 [(m)^2]"
    path = write_stats(str(tmp_path / "stats.txt"), electron=[], positron=[st2], photon=[st])
    assert open(path).read().splitlines()[0].startswith("positron: variance x")
    for bad in ("median energy", "mean nonsense", "circmean energy", "mean energy in 1, 2"):
        with pytest.raises(ValueError):
            SummaryStatistic(bad)
