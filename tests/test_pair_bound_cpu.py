"""The bound that lets the device skip negligible CP Breit-Wheeler
summations (ptg_bw.cuh, bw_summation_bound), restated here, lies above the
oracle's harmonic sum (pair_creation/cp/mod.rs:385-393) everywhere in the
summation regime 0.02 <= a < 0.3 (above the reference's too-small cut)."""

import math

import numpy as np


def _limits(a, eta):
    # pair_creation/cp/mod.rs:349-361
    nm = math.ceil(2 * (1 + a * a) / eta)
    rng = 2 * (0.25 + a * a) / eta + 13 * a * (2 + a)
    test = 0.25 - (1 + a * a) / (2 * nm * eta)
    if test <= 2.220446049250313e-16:
        return int(nm) + 1, int(nm + 1 + rng)
    return int(nm), int(nm + rng)


def _harmonic_bound(a, eta):
    """The bound harmonic by harmonic: |J_m(x)| <= (x/2)^m / m! at each n."""
    n0, n1 = _limits(a, eta)
    a2 = a * a
    c = a / math.sqrt(1 + a2)
    total = 0.0
    for n in range(n0, n1 + 1):
        sn = 2 * n * eta / (1 + a2)
        if sn <= 4:
            continue
        s_min = min(0.5 * (1 - math.sqrt(1 - 4 / sn)), 0.5)
        q = (1 - s_min) / s_min + s_min / (1 - s_min)
        x = 0.5 * n * c
        bm = math.exp((n - 1) * math.log(x) - math.lgamma(n))
        b = bm * x / n
        bp = b * x / (n + 1)
        k = 0.5 * a2 * q
        total += b * b * (1 + k) + k * (bm * bm + bp * bp)
    return total


def _bound(a, eta):
    """ptg_bw.cuh bw_summation_bound: the geometric closed form."""
    n0, _ = _limits(a, eta)
    a2 = a * a
    c = a / math.sqrt(1 + a2)
    r = 0.5 * math.e * c
    rho = r * r
    K = 1 + 4 / (c * c) + 0.25 * c * c
    beta = 2 * eta / (1 + a2)
    A, B = 1 + 0.5 * a2 * K, 0.5 * a2 * K * beta
    n = float(n0)
    lead = math.exp(2 * n * math.log(r)) / (2 * math.pi * n)
    om = 1 - rho
    return lead * ((A + B * n) / om + B * rho / (om * om))


def _points(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        a = math.exp(rng.uniform(math.log(0.02), math.log(0.3)))
        eta = math.exp(rng.uniform(math.log(1e-3), math.log(2.0)))
        if math.log10(eta) < -1 - (math.log10(a) + 2) ** 2 / 4.5:
            continue  # the reference's too-small cut: no summation there
        out.append((a, eta))
    return out


def test_summation_bound_lies_above_the_sum(orc):
    for a, eta in _points(7, 60):
        f = orc.cp_pair_by_summation(a, eta)
        assert max(f[0], f[1]) <= _bound(a, eta), (a, eta, f)


def test_closed_form_bounds_the_harmonic_bound():
    """The closed form is above the harmonic-by-harmonic bound (so above the
    sum) and within a small factor of it: it skips the same negligible
    steps up to that factor."""
    ratios = []
    for a, eta in _points(11, 400):
        hb = _harmonic_bound(a, eta)
        cf = _bound(a, eta)
        assert cf >= hb, (a, eta, cf, hb)
        if hb > 0:
            ratios.append(cf / hb)
    assert max(ratios) < 10.0, max(ratios)
