"""The statistics behind the equivalence tests, on the CPU: KS distance and
critical value, the chi-square of two histograms, and the pass rule, on
samples whose answer is known."""

import numpy as np

from ptarmigan_gb300 import abi, equivalence


def _particles(energies_mev, n_pos=0, seed=0):
    rng = np.random.default_rng(seed)
    n = len(energies_mev) + n_pos
    out = abi.empty_arrays(n)
    out["species"][:len(energies_mev)] = abi.PHOTON
    out["species"][len(energies_mev):] = abi.POSITRON
    e = np.asarray(energies_mev) / equivalence.ELECTRON_MASS_MEV
    th = rng.uniform(0, 1e-4, len(e))
    out["u"][:len(e)] = np.stack([e, e * np.sin(th), 0 * e, -e * np.cos(th)], axis=1)
    out["pol"][:, 0] = 1.0
    return out


def test_ks_matches_scipy():
    scipy_stats = __import__("pytest").importorskip("scipy.stats")
    rng = np.random.default_rng(1)
    a, b = rng.normal(size=3000), rng.normal(0.05, 1.0, size=2000)
    d = equivalence.ks_distance(a, b)
    ref = scipy_stats.ks_2samp(a, b)
    assert abs(d - ref.statistic) < 1e-12
    assert abs(equivalence.ks_pvalue(d, 3000, 2000) - ref.pvalue) < 0.02


def test_same_distribution_passes_and_shift_fails():
    rng = np.random.default_rng(2)
    def prim(n):
        return {"species": np.zeros(n, dtype=np.int32), "u": np.tile([2e4, 0, 0, -2e4], (n, 1))}
    a = _particles(np.exp(rng.uniform(0, 8, 20000)), seed=3)
    b = _particles(np.exp(rng.uniform(0, 8, 15000)), seed=4)
    cmp = equivalence.compare(a, prim(20000), b, prim(15000))
    assert equivalence.passes(cmp), cmp
    c = _particles(1.05 * np.exp(rng.uniform(0, 8, 15000)), seed=5)
    cmp2 = equivalence.compare(a, prim(20000), c, prim(15000))
    assert not equivalence.passes(cmp2)
    assert cmp2["chi2_p"] < 1e-3


def test_chi2_identical_histograms_is_zero():
    x = np.geomspace(1.0, 4000.0, 1000)
    c2, dof, p = equivalence.chi2_two_sample(x, x)
    assert c2 == 0.0 and dof > 0 and p == 1.0


def test_match_by_stream():
    a = abi.empty_arrays(3)
    a["stream"][:] = [5, 7, 9]
    a["u"][:] = [[1, 0, 0, 1], [2, 0, 0, 2], [3, 0, 0, 3]]
    b = abi.empty_arrays(3)
    b["stream"][:] = [9, 5, 8]
    b["u"][:] = [[3, 0, 0, 3], [1, 0, 0, 1.1], [1, 1, 1, 1]]
    m = equivalence.match(a, b, 1e-6)
    assert abs(m["matched_frac"] - 2 / 3) < 1e-12
    assert abs(m["momentum_agree_frac"] - 0.5) < 1e-12
