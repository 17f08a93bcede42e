"""CPU restatement of the reference's distribution output, the checker of
the device histograms (test infrastructure only): the particle functions
of output/functions.rs:109-263, Stokes projection (geometry/
polarization.rs:159-214) and Histogram::generate_1d / generate_2d
(output/hgram.rs:150-448), over particle arrays as the C ABI returns them
(four-vectors in rows of 4)."""

import math

import numpy as np

ELECTRON_MASS_MEV = 0.510999  # constants.rs:21


def _pol_project(pol, u, axis):
    out = np.empty(len(u))
    a = np.asarray(axis, dtype=float)
    a = a / math.sqrt(float(a @ a))
    for i in range(len(u)):
        sv, n = pol[i], u[i, 1:] / math.sqrt(float(u[i, 1:] @ u[i, 1:]))
        frac = math.hypot(math.hypot(sv[1], sv[2]), sv[3]) / sv[0]
        mag = math.hypot(n[0], n[2])
        x = np.array([1.0, 0.0, 0.0]) if mag == 0.0 else np.array([n[2] / mag, 0.0, -n[0] / mag])
        y = np.cross(x, n)
        xa, ya = float(x @ a), float(y @ a)
        unpol = 0.5 * (xa * xa + ya * ya)
        if not frac > 0.0:
            out[i] = unpol
            continue
        q, uu, v = sv[1] / (frac * sv[0]), sv[2] / (frac * sv[0]), sv[3] / (frac * sv[0])
        if 1.0 + q < 1.0e-12:
            xs = uu * uu + v * v
            ex = math.sqrt(0.5 * (0.5 * xs + 0.125 * xs * xs))
        else:
            ex = math.sqrt(0.5 * (1.0 + q))
        ey = complex(1.0, 0.0) if ex == 0.0 else complex(0.5 * uu / ex, -0.5 * v / ex)
        out[i] = frac * abs(ex * xa + ey * ya) ** 2 + (1.0 - frac) * unpol
    return out


def value(p, f):
    """The function with device number f (ptg_output_func) of every particle."""
    m = ELECTRON_MASS_MEV
    u, r, pol = p["u"], p["r"], p["pol"]
    px, py, pz, p0 = m * u[:, 1], m * u[:, 2], m * u[:, 3], m * u[:, 0]
    with np.errstate(divide="ignore", invalid="ignore"):
        table = {
            0: lambda: np.arctan2(px, pz), 1: lambda: np.arctan2(py, pz),
            2: lambda: np.arctan2(np.hypot(px, py), -pz), 3: lambda: np.arctan2(np.hypot(px, py), pz),
            4: lambda: px, 5: lambda: py, 6: lambda: pz, 7: lambda: np.hypot(px, py),
            8: lambda: np.hypot(px, py) / (p0 - pz), 9: lambda: px / (p0 - pz), 10: lambda: py / (p0 - pz),
            11: lambda: p0 - pz, 12: lambda: p0 + pz, 13: lambda: u[:, 0].copy(), 14: lambda: u[:, 0] * m,
            15: lambda: np.ones(len(u)), 16: lambda: r[:, 1].copy(), 17: lambda: r[:, 2].copy(),
            18: lambda: r[:, 3].copy(), 19: lambda: np.hypot(r[:, 1], r[:, 2]), 20: lambda: p["payload"].copy(),
            21: lambda: p["parent_chi"].copy(), 22: lambda: p["interaction_count"].copy(),
            23: lambda: p["work"] * m, 24: lambda: pol[:, 1].copy(), 25: lambda: pol[:, 2].copy(),
            26: lambda: pol[:, 3].copy(), 27: lambda: _pol_project(pol, u, (1.0, 0.0, 0.0)),
            28: lambda: _pol_project(pol, u, (0.0, 1.0, 0.0)), 29: lambda: p["weight"].copy(),
            30: lambda: pol[:, 3] * p["weight"],
        }
        return table[f]()


def weight(p, w):
    """output/functions.rs:244-263 (device numbering ptg_weight_func)."""
    if w == 1:
        return p["weight"] * (p["u"][:, 0] * ELECTRON_MASS_MEV)
    if w == 2:
        return value(p, 27) * p["weight"]
    if w == 3:
        return value(p, 28) * p["weight"]
    if w == 4:
        return p["pol"][:, 3] * p["weight"]
    return p["weight"].copy()


def generate(p, species, funcs, scales, wfunc, bin_spec, n_bins=0, bin_size=0.0, height=1, filt=None):
    """generate_1d (len(funcs) == 1) or generate_2d; bin_spec 0 auto, 1 log,
    2 fixed number, 3 fixed size; height 0 count, 1 density, 2 pdf.
    Returns (info dict, counts) or None for an empty set."""
    sel = p["species"] == species
    q = {k: v[sel] for k, v in p.items()}
    n = int(sel.sum())
    if n == 0:
        return None
    dim = len(funcs)
    with np.errstate(divide="ignore", invalid="ignore"):
        vals = [value(q, f) * s for f, s in zip(funcs, scales)]
        if bin_spec == 1:
            vals = [np.log(v) for v in vals]
    w = weight(q, wfunc)
    total = float(np.sum(w))
    acc = np.ones(n, dtype=bool)
    if filt is not None:
        fv = value(q, filt[0])
        acc = (fv >= filt[1]) & (fv < filt[2])
    mn, mx = [], []
    for v in vals:  # min_max_by (hgram.rs:150-165)
        ok = np.isfinite(v) & acc
        mn.append(float(v[ok].min()) if ok.any() else np.finfo(float).max)
        mx.append(float(v[ok].max()) if ok.any() else -np.finfo(float).max)

    def nb(a, b):  # number_of_bins (hgram.rs:171-184)
        if a == b:
            return 1
        if bin_spec == 2:
            return n_bins
        if bin_spec == 3:
            return int(math.ceil((b - a) / bin_size))
        return int(math.ceil(2.0 * np.cbrt(float(n))))
    bins = [nb(a, b) for a, b in zip(mn, mx)]
    if dim == 1:
        vol = 1.0 if mn[0] == mx[0] else (bin_size if bin_spec == 3 else (mx[0] - mn[0]) / bins[0])
        sz = [vol]
        shown = [0.0 if bins[0] <= 1 else vol]
    else:
        sz, vol = [], 1.0
        for k in range(2):
            if mn[k] == mx[k]:
                sz.append(0.0)
            else:
                d = bin_size if bin_spec == 3 else (mx[k] - mn[k]) / bins[k]
                sz.append(d)
                vol *= d
        shown = sz
    ncts = bins[0] * (bins[1] if dim == 2 else 1)
    cts = np.zeros(ncts)
    fin = np.ones(n, dtype=bool)
    for v in vals:
        fin &= np.isfinite(v)
    use = fin & acc
    idx = []
    for k in range(dim):
        if dim == 2 and sz[k] == 0.0:
            idx.append(np.zeros(n, dtype=np.int64))
            continue
        with np.errstate(invalid="ignore"):
            b = np.floor((vals[k] - mn[k]) / sz[k])
        idx.append(np.where(b > 0, b, 0).astype(np.int64))  # `as usize`: negative and NaN to 0
    ww = w.copy()
    if bin_spec == 1 and height in (1, 2):
        for k in range(dim):
            if dim == 2 and sz[k] == 0.0:
                continue
            lin = np.exp(mn[k] + idx[k] * sz[k]) * np.expm1(sz[k])
            # 1d: w * bin_vol / vol_k (hgram.rs:277); 2d: w *= size / vol_k (hgram.rs:398-404)
            ww = ww * sz[k] / lin if dim == 1 else ww * (sz[k] / lin)
    fbin = idx[0] if dim == 1 else idx[1] * bins[1] + idx[0]
    use &= fbin < ncts
    np.add.at(cts, fbin[use], ww[use])
    if height == 1:
        cts = cts / vol
    elif height == 2:
        cts = cts / (vol * total)
    info = {"dim": dim, "bins": bins, "min": mn, "max": mx, "bin_size": shown, "bin_volume": vol, "total": total,
            "unweighted_total": float(n)}
    return info, cts


def summary(p, species, op, var_func, weight_func, filter_func, lo, hi):
    """SummaryStatistic::evaluate (output/stats.rs:265-483), sequentially
    over the particles of one species in array order."""
    sel = p["species"] == species
    q = {k: v[sel] for k, v in p.items()}
    v, w = value(q, var_func), value(q, weight_func)
    within = np.ones(len(v), dtype=bool) if filter_func < 0 else (lambda f: (f > lo) & (f < hi))(value(q, filter_func))
    vw = v * w
    if op == "total":
        return float(np.sum(vw[within]))
    if op == "fraction":
        return float(np.sum(vw[within]) / np.sum(vw))
    if op == "mean":
        return float(np.sum(vw[within]) / np.sum(w[within]))
    if op == "minimum":
        return float(np.min(vw[within])) if within.any() else math.inf
    if op == "maximum":
        return float(np.max(vw[within])) if within.any() else -math.inf
    if op == "variance":
        first = np.nonzero(within[:10])[0]
        m = float(np.sum(vw[first]) / np.sum(w[first]))
        d = v[within] - m
        s2, s1, c = np.sum(w[within] * d ** 2), np.sum(w[within] * d), np.sum(w[within])
        return float((s2 - s1 ** 2 / c) / c)
    xb = np.sum(w[within] * np.cos(v[within])) / np.sum(w[within])
    yb = np.sum(w[within] * np.sin(v[within])) / np.sum(w[within])
    if op == "circmean":
        return math.atan2(yb, xb)
    if op == "circvar":
        return 1.0 - math.hypot(xb, yb)
    return math.sqrt(-2.0 * math.log(math.hypot(xb, yb)))
