"""The regenerated CP harmonic CDF table (the reference tree lacks
nonlinear_compton/cp/tables/cdf.rs; ptarmigan_gb300/tables/regen.py runs its
generator, nonlinear_compton/cp/mod.rs:472-612, on the GPU).

Pinned two ways: its total rates reproduce the reference's shipped total
table (cp/tables/total.rs), and its CDF nodes match cumulative sums of the
oracle's independent partial rates."""

import math
import os

import numpy as np
import pytest

from ptarmigan_gb300.tables.extract import read_ptgt

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ptarmigan_gb300", "tables", "data")


def _load(name):
    shape, vals = read_ptgt(os.path.join(DATA, name + ".ptgt"))
    return np.array(vals).reshape(shape)


def test_regenerated_totals_match_shipped_table():
    tot = _load("nlc_cp_cdf_totals")
    shipped = np.exp(_load("nlc_cp_rate"))
    rel = np.abs(tot - shipped) / shipped
    # the shipped table holds ln(rate) to 13 significant digits
    assert rel.max() < 1e-9, rel.max()


def test_regenerated_cdf_is_monotone_and_normalised():
    cdf = _load("nlc_cp_cdf")
    assert cdf.shape == (4270, 32, 2)
    n, f = cdf[:, :, 0], cdf[:, :, 1]
    assert np.all(np.diff(n, axis=1) >= 0)
    assert np.all(np.diff(f, axis=1) >= -1e-15)
    assert np.all(np.abs(f[:, -1] - 1.0) < 1e-12)


@pytest.mark.parametrize("i,j", [(0, 0), (20, 10), (40, 30), (69, 33), (35, 45)])
def test_regenerated_cdf_nodes_match_oracle(orc, i, j):
    cdf = _load("nlc_cp_cdf")
    a = 0.02 * 10.0 ** (j / 20.0)
    eta = 1.0e-3 * 10.0 ** (i / 20.0)
    n_max = int(10.0 * (1.0 + a * (a * a)))
    rates = np.cumsum([orc.cp_partial_rate(n, a, eta) for n in range(1, n_max + 1)])
    total = rates[-1]
    node = cdf[i * 61 + j]
    for k in range(32):
        nn, ff = node[k]
        if nn == math.floor(nn) and nn <= n_max:
            assert abs(ff - rates[int(nn) - 1] / total) < 1e-9, (k, nn, ff)


def _load_table(name):
    import os
    from ptarmigan_gb300.tables.extract import read_ptgt
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    shape, vals = read_ptgt(os.path.join(here, "ptarmigan_gb300", "tables", "data", name))
    return np.array(vals).reshape(shape)


def test_lp_mid_cdf_totals_reproduce_shipped_table():
    """The regenerated LP Breit-Wheeler mid-range CDF (generated on the GPU
    by ptg_regen_bw_lp_mid_cdf) ends at the shipped totals: most nodes to
    1e-9; the rest within the adaptive quadrature's tolerance (1e-3), where
    a last-bit difference of a device transcendental flipped a refinement."""
    cdf = _load_table("bw_lp_mid_cdf.ptgt")
    tot = np.exp(_load_table("bw_lp_mid_total.ptgt").reshape(-1, 2))
    last = cdf[:, 15, 1:]
    pos = tot > 0.0
    rel = np.where(pos, np.abs(last - tot) / np.where(pos, tot, 1.0), 0.0).max(axis=1)
    assert np.all(last[~pos] == 0.0)
    assert np.all(rel < 1e-3)
    assert np.mean(rel < 1e-9) > 0.9


@pytest.mark.parametrize("i,j", [(0, 3), (37, 17), (80, 30), (120, 8), (156, 33)])
def test_lp_mid_cdf_nodes_match_oracle(orc, i, j):
    import math
    from ptarmigan_gb300.tables import small_tables as st
    cdf = _load_table("bw_lp_mid_cdf.ptgt")[i * 36 + j]
    a = math.exp(st.scalar("BW_LPM_LN_MIN_A")) * 10.0 ** (j / 20.0)
    eta = (1.0 + 0.5 * a * a) * math.exp(st.scalar("BW_LPM_LN_MAX_ETA_PRIME")) / (1.0 + i / 4.0)
    ref = orc.lp_pair_by_summation(a, eta)
    assert np.array_equal(cdf[:, 0], ref[:, 0])
    pos = ref[:, 1:] > 0.0
    rel = np.abs(cdf[:, 1:][pos] / ref[:, 1:][pos] - 1.0)
    assert np.all(rel < 1e-3)
