"""Statistical comparison of two collision-loop outputs.

The GPU path and the reference draw from different random streams where
the learned proposal samples (and the reference's own Xoshiro256** streams
are pinned by no test), so equivalence is statistical: photon energy and
polar-angle spectra (two-sample Kolmogorov-Smirnov and a chi-square on 200
logarithmic energy bins from 1 MeV to 5 GeV), pair yield, mean photon
Stokes parameters and mean electron energy loss, each with its standard
error.  Where both sides share streams (the table sampler against the
oracle) particles are also matched one to one by stream id.

Every function takes the particle dicts of ``Engine.collide`` (numpy arrays
named as in ``abi.PARTICLE_FIELDS``).
"""

import math

import numpy as np

from . import abi

ELECTRON_MASS_MEV = 0.51099895
# the photon spectrum's bins: 200 logarithmic bins from 1 MeV to 5 GeV
LOG_BINS = np.geomspace(1.0, 5000.0, 201)


def ks_distance(a, b):
    """Two-sample Kolmogorov-Smirnov statistic."""
    a, b = np.sort(np.asarray(a, dtype=float)), np.sort(np.asarray(b, dtype=float))
    if len(a) == 0 or len(b) == 0:
        return float("nan")
    grid = np.concatenate([a, b])
    return float(np.max(np.abs(np.searchsorted(a, grid, side="right") / len(a) -
                               np.searchsorted(b, grid, side="right") / len(b))))


def ks_critical(n, m, alpha=1e-3):
    """Two-sample KS critical value at significance alpha (asymptotic)."""
    if n == 0 or m == 0:
        return float("nan")
    c = math.sqrt(-0.5 * math.log(alpha / 2.0))
    return c * math.sqrt((n + m) / (n * m))


def ks_pvalue(d, n, m):
    """Asymptotic p-value of a two-sample KS distance d (Kolmogorov's series)."""
    if n == 0 or m == 0 or not math.isfinite(d):
        return float("nan")
    en = math.sqrt(n * m / (n + m))
    lam = (en + 0.12 + 0.11 / en) * d
    if lam < 1e-3:
        return 1.0
    s = 0.0
    for j in range(1, 101):
        term = 2.0 * (-1) ** (j - 1) * math.exp(-2.0 * j * j * lam * lam)
        s += term
        if abs(term) < 1e-12:
            break
    return min(1.0, max(0.0, s))


def chi2_two_sample(a, b, edges=LOG_BINS):
    """Chi-square between the histograms of two samples of different sizes
    (bins empty in both are left out).  Returns (chi2, dof, p)."""
    ha, _ = np.histogram(a, bins=edges)
    hb, _ = np.histogram(b, bins=edges)
    na, nb = ha.sum(), hb.sum()
    if na == 0 or nb == 0:
        return float("nan"), 0, float("nan")
    keep = (ha + hb) > 0
    ka, kb = math.sqrt(nb / na), math.sqrt(na / nb)
    chi2 = float(np.sum((ka * ha[keep] - kb * hb[keep]) ** 2 / (ha[keep] + hb[keep])))
    dof = int(keep.sum()) - 1
    return chi2, dof, _chi2_sf(chi2, dof)


def _chi2_sf(x, k):
    """Survival function of the chi-square distribution (regularised upper
    incomplete gamma Q(k/2, x/2))."""
    if k <= 0:
        return float("nan")
    try:
        from scipy.special import gammaincc
        return float(gammaincc(0.5 * k, 0.5 * x))
    except ImportError:
        # Wilson-Hilferty normal approximation
        z = ((x / k) ** (1.0 / 3.0) - (1.0 - 2.0 / (9.0 * k))) / math.sqrt(2.0 / (9.0 * k))
        return 0.5 * math.erfc(z / math.sqrt(2.0))


def photon_energy_mev(out):
    ph = out["species"] == abi.PHOTON
    return out["u"][ph, 0] * ELECTRON_MASS_MEV


def photon_polar_angle(out):
    """Angle between each photon and the beam axis, -z (output/functions.rs
    polar_angle about the beam's direction of travel)."""
    ph = out["species"] == abi.PHOTON
    u = out["u"][ph]
    return np.arctan2(np.hypot(u[:, 1], u[:, 2]), -u[:, 3])


def summary(out, primaries):
    """Per-batch quantities with their standard errors."""
    n_prim = len(primaries["species"])
    ph = out["species"] == abi.PHOTON
    n_ph = int(ph.sum())
    n_pos = int((out["species"] == abi.POSITRON).sum())
    pol = out["pol"][ph]
    stokes = [float(x) for x in pol[:, 1:].mean(axis=0)] if n_ph else [float("nan")] * 3
    stokes_err = [float(x) for x in pol[:, 1:].std(axis=0) / math.sqrt(max(1, n_ph))] if n_ph else [float("nan")] * 3
    # energy lost by each primary electron that is still in the output
    prim_e = (out["species"] == abi.ELECTRON) & (out["generation"] == 0)
    idx = out["primary"][prim_e].astype(np.int64)
    loss = (primaries["u"][idx, 0] - out["u"][prim_e, 0]) * ELECTRON_MASS_MEV
    return {
        "primaries": n_prim,
        "photons_per_primary": n_ph / n_prim, "photons_per_primary_err": math.sqrt(n_ph) / n_prim,
        "pairs_per_primary": n_pos / n_prim, "pairs_per_primary_err": math.sqrt(max(n_pos, 1)) / n_prim,
        "stokes_mean": stokes, "stokes_mean_err": stokes_err,
        "electron_energy_loss_mev": float(loss.mean()) if len(loss) else float("nan"),
        "electron_energy_loss_mev_err": float(loss.std() / math.sqrt(len(loss))) if len(loss) > 1 else float("nan"),
    }


def compare(out_a, prim_a, out_b, prim_b, alpha=1e-3):
    """Statistical comparison of two outputs (a against b): KS and chi-square
    on the photon spectra, and the differences of the per-primary quantities
    in units of their combined standard error."""
    ea, eb = photon_energy_mev(out_a), photon_energy_mev(out_b)
    ta, tb = photon_polar_angle(out_a), photon_polar_angle(out_b)
    ks_e = ks_distance(ea, eb)
    ks_t = ks_distance(ta, tb)
    c2, dof, p = chi2_two_sample(ea, eb)
    sa, sb = summary(out_a, prim_a), summary(out_b, prim_b)

    def sig(key):
        va, vb = sa[key], sb[key]
        ea_, eb_ = sa[key + "_err"], sb[key + "_err"]
        if isinstance(va, list):
            return [abs(x - y) / math.hypot(u, v) if math.hypot(u, v) > 0 else 0.0
                    for x, y, u, v in zip(va, vb, ea_, eb_)]
        s = math.hypot(ea_, eb_)
        return abs(va - vb) / s if s > 0 else 0.0

    return {
        "photons": [len(ea), len(eb)],
        "ks_photon_energy": ks_e, "ks_photon_energy_critical": ks_critical(len(ea), len(eb), alpha),
        "ks_photon_energy_p": ks_pvalue(ks_e, len(ea), len(eb)),
        "ks_photon_polar_angle": ks_t, "ks_photon_polar_angle_critical": ks_critical(len(ta), len(tb), alpha),
        "ks_photon_polar_angle_p": ks_pvalue(ks_t, len(ta), len(tb)),
        "chi2_log_energy_200": c2, "chi2_dof": dof, "chi2_p": p,
        "a": sa, "b": sb,
        "sigma": {"photons_per_primary": sig("photons_per_primary"), "pairs_per_primary": sig("pairs_per_primary"),
                  "stokes_mean": sig("stokes_mean"), "electron_energy_loss_mev": sig("electron_energy_loss_mev")},
    }


def passes(cmp, alpha=1e-3, n_sigma=5.0):
    """True when every test of `compare` passes: both KS distances below
    their critical values, the chi-square p-value above alpha, and every
    per-primary quantity within n_sigma combined standard errors."""
    s = cmp["sigma"]
    checks = [
        not (cmp["ks_photon_energy"] > cmp["ks_photon_energy_critical"]),
        not (cmp["ks_photon_polar_angle"] > cmp["ks_photon_polar_angle_critical"]),
        not (cmp["chi2_p"] < alpha),
        s["photons_per_primary"] <= n_sigma, s["pairs_per_primary"] <= n_sigma,
        all(x <= n_sigma for x in s["stokes_mean"]),
        not (s["electron_energy_loss_mev"] > n_sigma),
    ]
    return all(checks)


def match(out, ref, tol):
    """One-to-one match of particles by stream id (both sides drew from the
    same streams).  Returns the fraction of `ref`'s particles found in `out`
    and, of those, the fraction whose momenta agree within `tol` relative."""
    so = np.asarray(out["stream"], dtype=np.uint64)
    sr = np.asarray(ref["stream"], dtype=np.uint64)
    order = np.argsort(so, kind="stable")
    pos = np.searchsorted(so[order], sr)
    pos = np.minimum(pos, max(len(so) - 1, 0))
    hit = (len(so) > 0) & (so[order][pos] == sr) if len(so) else np.zeros(len(sr), dtype=bool)
    i = order[pos[hit]]
    uo, ur = out["u"][i], ref["u"][hit]
    ok = np.max(np.abs(uo - ur), axis=1) <= tol * np.linalg.norm(ur, axis=1)
    found, agree = int(hit.sum()), int(ok.sum())
    n = len(sr)
    return {"oracle_particles": n, "gpu_particles": len(out["stream"]), "matched_frac": found / n if n else float("nan"),
            "momentum_agree_frac": agree / found if found else float("nan"), "tolerance": tol}
