"""Runs a ptarmigan input file on the GPU: the flow of main.rs (339-1290)
for the keys below, with the collision loop, the beam and the
distribution and statistics output on the device.

    python -m ptarmigan_gb300 input.yml [output_dir]

Supported: control (dt_multiplier, lcfa, rng_seed, radiation_reaction,
pair_creation, pol_resolved, classical, select_multiplicity,
increase_pair_rate_by, bandwidth_correction, track_secondaries,
stop_at_time as a number), laser (a0 or an a0 loop, wavelength or omega,
waist, fwhm_duration or n_cycles, envelope, polarization including
"linear || y" and "linear @ angle", chirp_coeff), beam (n or ne, species,
charge or n_real, gamma, sigma, bremsstrahlung_source with gamma_min,
radius with its distribution and cutoff, length, collision_angle,
collision_plane, rms_divergence, energy_chirp, offset, stokes_pars),
output (ident, electron / photon / positron distributions, file_format,
units, coordinate_system, discard_background(_e), min_energy, max_angle),
stats (electron / photon / positron, and expressions), constants,
output:dump_all_particles: hdf5 (the final-state file of main.rs:1289-1715,
written by ptarmigan_gb300.hdf5) and beam:from_hdf5 (particle/loader.rs,
for files with the structures ptarmigan_gb300.hdf5 reads).
Also: beam:spectrum (a function of gamma over [min, max], or a file of
spectral values), control:increase_pair_rate_by: auto, control:
stop_at_time: auto (every final-state particle moved to the latest time any
of them reached) and a given stop time (every particle moved to it), and
the decayed intermediate photons (output:intermediate distributions,
stats:intermediate, output:dump_decayed_photons into the HDF5 file's
intermediate-state group).
"""

import math
import os

import numpy as np

from . import abi, engine as engine_mod, hdf5
from .input import COMPTON_TIME, ELECTRON_MASS, ELEMENTARY_CHARGE, SPEED_OF_LIGHT, Input, InputError
from .output import DistributionFunction, SummaryStatistic, UnitSystem, rust_exp

SPECIES = {"electron": abi.ELECTRON, "positron": abi.POSITRON, "photon": abi.PHOTON}


def laser_from_input(inp, a0):
    """main.rs:399-470 and the model choice of :1048-1068."""
    lcfa = inp.bool("control:lcfa", False)
    if inp.contains("laser:wavelength"):
        wavelength = inp.float("laser:wavelength")
    else:
        omega = inp.float("laser:omega")
        wavelength = 2.0 * math.pi * COMPTON_TIME * ELECTRON_MASS * SPEED_OF_LIGHT ** 3 / omega
    pol_s = inp.str("laser:polarization")
    if pol_s == "circular":
        pol, angle = abi.CIRCULAR, 0.0
    elif pol_s in ("linear", "linear || x"):
        pol, angle = abi.LINEAR, 0.0
    elif pol_s == "linear || y":
        pol, angle = abi.LINEAR, math.pi / 2
    elif pol_s.startswith("linear @"):
        pol, angle = abi.LINEAR, inp.evaluate(pol_s[len("linear @"):])
    else:
        raise InputError("laser polarization must be 'linear [|| x or y]' or 'circular'")
    focusing = inp.contains("laser:waist")
    waist = inp.float("laser:waist") if focusing else math.inf
    env_s = inp.str("laser:envelope", "")
    env = {"cos2": abi.COS2, "cos^2": abi.COS2, "cos_sqd": abi.COS2, "cos_squared": abi.COS2,
           "flattop": abi.FLATTOP, "flat-top": abi.FLATTOP, "gauss": abi.GAUSSIAN, "gaussian": abi.GAUSSIAN}.get(
        env_s, None if env_s else (abi.GAUSSIAN if focusing else abi.COS2))
    if env is None:
        raise InputError("laser envelope must be one of 'cos^2', 'flattop' or 'gaussian'")
    if env == abi.GAUSSIAN and inp.contains("laser:fwhm_duration"):
        n_cycles = SPEED_OF_LIGHT * inp.float("laser:fwhm_duration") / wavelength
    else:
        n_cycles = inp.float("laser:n_cycles")
        if env == abi.FLATTOP and n_cycles < 1.0:
            raise InputError("'n_cycles' must be >= 1.0 for flattop lasers")
    chirp = 0.0 if focusing else inp.float("laser:chirp_coeff", 0.0)
    model = (abi.FAST_FOCUSED_LASER if lcfa else abi.FOCUSED_LASER) if focusing else \
        (abi.FAST_PLANE_WAVE if lcfa else abi.PLANE_WAVE)
    return abi.laser_desc(model, a0, wavelength, pol, env, waist=waist, n_cycles=n_cycles, pol_angle=angle,
                          chirp_b=chirp, finite_bandwidth=inp.bool("control:bandwidth_correction", False))


def spectrum_from_input(inp, n_part, input_path=""):
    """beam:spectrum (main.rs:610-680): `function` (an expression in gamma)
    sampled at `resolution` points (default 10 + 2 n^(1/3)) from `min` in
    steps of (max - min) / resolution, or `file`, one spectral value per
    line (relative to the input file), over [min, max] or from min in steps
    of `step`.  Returns (values, min, max, step)."""
    analytical = inp.contains("beam:spectrum:function")
    numerical = inp.contains("beam:spectrum:file")
    if analytical and numerical:
        raise InputError("specify a function or a file in beam:spectrum, not both.")
    g_min = inp.float("beam:spectrum:min")
    if analytical:
        g_max = inp.float("beam:spectrum:max")
        n = inp.int("beam:spectrum:resolution") if inp.contains("beam:spectrum:resolution") else \
            int(10.0 + 2.0 * float(n_part) ** (1.0 / 3.0))
        step = (g_max - g_min) / n
        func = inp.func("beam:spectrum:function", "gamma")
        vals = [func(g_min + i * step) for i in range(n)]
        if not all(math.isfinite(v) for v in vals):
            raise InputError("beam:spectrum:function evaluated to non-numerical values in the specified domain.")
        return vals, g_min, g_max, step
    fname = inp.str("beam:spectrum:file")
    out_dir = os.path.dirname(input_path)
    fname = os.path.join(out_dir, fname) if out_dir else fname
    try:
        with open(fname) as fh:
            text = fh.read()
    except OSError:
        raise InputError('Unable to open "%s": no such file or directory.' % fname)
    try:
        vals = [float(line) for line in text.splitlines()]
    except ValueError:
        raise InputError('Unable to import "%s" as a 1D array of spectral values.' % fname)
    n = len(vals) - 1  # steps, not entries
    if inp.contains("beam:spectrum:max"):
        g_max = inp.float("beam:spectrum:max")
        step = (g_max - g_min) / n
    else:
        step = inp.float("beam:spectrum:step")
        g_max = g_min + n * step
    if not all(math.isfinite(v) for v in vals):
        raise InputError("beam:spectrum:file contains non-numerical values.")
    return vals, g_min, g_max, step


def custom_cdf(vals, g_min, step):
    """GammaDistribution::custom (particle/dstr.rs:88-106): CDF nodes
    [gamma, cumulative / total], gamma advanced by repeated addition of the
    step.  Returns the [len][2] array for the device builder."""
    total = sum(vals)
    cdf = [[g_min, 0.0]]
    g, rt = g_min, 0.0
    for v in vals:
        g += step
        rt += v
        cdf.append([g, rt / total])
    return np.ascontiguousarray(np.array(cdf, dtype=np.float64))


def spectrum_mean_gamma(vals, g_min, step):
    """GammaDistribution::gamma for a custom spectrum (dstr.rs:112-125)."""
    m0 = m1 = 0.0
    for i, f in enumerate(vals):
        g = g_min + i * step
        m0 += f
        m1 += g * f
    return m1 / m0


def beam_from_input(inp, laser, input_path=""):
    """main.rs:481-811 (rng-distributed beams); returns (desc, n, species)."""
    species = SPECIES.get(inp.str("beam:species", "electron"))
    if species is None:
        raise InputError("beam:species must be electron, positron or photon")
    n = inp.int("beam:n") if inp.contains("beam:n") else inp.int("beam:ne")
    w1 = abs(inp.float("beam:charge")) / (ELEMENTARY_CHARGE * n) if inp.contains("beam:charge") else None
    w2 = inp.float("beam:n_real") / n if inp.contains("beam:n_real") else None
    if w1 is not None and w2 is not None and w1 != w2:
        raise InputError("conflicting values of 'n_real' and 'charge'")
    weight = w1 if w1 is not None else (w2 if w2 is not None else 1.0)
    brem = species == abi.PHOTON and inp.bool("beam:bremsstrahlung_source", False)
    kw = {}
    spectrum = spectrum_from_input(inp, n, input_path) if inp.contains("beam:spectrum") else None
    cdf = None
    if spectrum is not None:
        vals, g_min, g_max, step = spectrum
        cdf = custom_cdf(vals, g_min, step)
        kw.update(gamma_dstr=abi.GAMMA_CUSTOM, custom_cdf=cdf)
        brem = False
    elif brem:
        kw.update(gamma_dstr=abi.GAMMA_BREM, gamma_min=inp.float("beam:gamma_min"), gamma_max=inp.float("beam:gamma"))
    else:
        kw.update(gamma_mean=inp.float("beam:gamma"), gamma_sigma=inp.float("beam:sigma", 0.0))
    length = inp.float("beam:length", 0.0)
    radius = inp.list("beam:radius", ["0.0"])
    r = inp.evaluate(radius[0])
    dist = radius[1] if len(radius) > 1 else "normally_distributed"
    if dist == "normally_distributed":
        if len(radius) > 2:
            r_max = inp.evaluate(radius[2])
            kw.update(radial_dstr=abi.RADIAL_TRUNC_NORMAL, sigma_x=r, x_max=r_max, y_max=r_max)
        else:
            kw.update(radial_dstr=abi.RADIAL_NORMAL, sigma_x=r)
    elif dist == "uniformly_distributed":
        kw.update(radial_dstr=abi.RADIAL_UNIFORM, r_max=r)
    else:
        raise InputError("beam radius distribution must be normally_ or uniformly_distributed")
    chirp = inp.float("beam:energy_chirp", 0.0)
    if brem:
        chirp = 0.0
    if abs(chirp) > 1.0:
        raise InputError("absolute value of energy chirp must be <= 1")
    plane_s = inp.str("beam:collision_plane", "horizontal")
    plane = {"horizontal": 0.0, "vertical": math.pi / 2}.get(plane_s)
    if plane is None:
        plane = inp.evaluate(plane_s)
    offset = inp.floats("beam:offset", [0.0, 0.0, 0.0])
    stokes = inp.floats("beam:stokes_pars", [0.0, 0.0, 0.0])
    if len(offset) != 3 or len(stokes) != 3:
        raise InputError("beam:offset and beam:stokes_pars are three-vectors")
    if math.sqrt(sum(x * x for x in stokes)) > 1.0:
        raise InputError("specified particle polarization does not satisfy S_1^2 + S_2^2 + S_3^2 <= 1")
    initial_z = engine_mod.laser_initial_z(laser) + 3.0 * length
    desc = abi.beam_desc(species=species, energy_chirp=chirp, sigma_z=length,
                         rms_div=inp.float("beam:rms_divergence", 0.0),
                         collision_angle=inp.float("beam:collision_angle", 0.0), collision_plane=plane,
                         offset=tuple(offset), initial_z=initial_z, stokes=tuple(stokes), weight=weight, **kw)
    desc.cdf_nodes = cdf  # the custom spectrum's nodes outlive the descriptor's use
    desc.spectrum_gamma = spectrum_mean_gamma(spectrum[0], spectrum[1], spectrum[3]) if spectrum else None
    return desc, n, species, inp.float("beam:collision_angle", 0.0), plane


def stop_mode(inp):
    """control:stop_at_time (main.rs:346-361): "auto" (every particle is
    moved to the latest time any reached), a time in seconds (tracking
    stops there and every particle is moved to it), or absent."""
    if not inp.contains("control:stop_at_time"):
        return None
    s = inp.str("control:stop_at_time")
    if s == "auto":
        return "auto"
    try:
        return inp.evaluate(s)
    except InputError:
        raise InputError("control:stop_at_time must be a numerical value or 'auto'.")


def rate_increase_from_input(inp, eng, laser, desc, spectrum_gamma=None):
    """control:increase_pair_rate_by (main.rs:1001-1034): a number, or
    "auto" for a beam built from its distributions (the ratio of the photon
    emission and pair creation rates at the beam's mean Lorentz factor)."""
    if not inp.contains("control:increase_pair_rate_by"):
        return 1.0
    v = inp.str("control:increase_pair_rate_by")
    if v != "auto":
        return inp.float("control:increase_pair_rate_by")
    if desc is None:
        raise InputError("automatic increase in pair creation not available when loading particles from file.")
    if spectrum_gamma is not None:
        gamma = spectrum_gamma
    elif desc.gamma_dstr == abi.GAMMA_BREM:
        gamma = desc.gamma_max
    else:
        gamma = desc.gamma_mean
    return eng.pair_rate_increase(laser, gamma)


def options_from_input(inp, keep_decayed, rate_increase=None):
    """main.rs:339-398, 862-880 and 1106-1124."""
    classical_s = inp.str("control:classical", "false")
    classical, gaunt = {"true": (True, False), "false": (False, False),
                        "gaunt_factor_corrected": (True, True)}.get(classical_s, (None, None))
    if classical is None:
        raise InputError("control:classical must be one of 'true', 'false' or 'gaunt_factor_corrected'")
    mult = inp.int("control:select_multiplicity") if inp.contains("control:select_multiplicity") else -1
    if rate_increase is None:
        if inp.str("control:increase_pair_rate_by", "") == "auto":
            raise InputError("increase_pair_rate_by: auto is evaluated for the beam (rate_increase_from_input)")
        rate_increase = inp.float("control:increase_pair_rate_by", 1.0)
    rate = rate_increase
    if rate < 1.0:
        raise InputError("increase in pair creation rate must be >= 1.0.")
    if rate > 1.0 and mult >= 0:
        raise InputError("event biasing (pair rate increase > 1) is incompatible with multiplicity selection.")
    stop = stop_mode(inp)
    if inp.contains("output:discard_background"):
        bg_e = bg_ph = inp.bool("output:discard_background")
    else:
        bg_e, bg_ph = inp.bool("output:discard_background_e", False), False
    return abi.collide_options(
        dt_multiplier=inp.float("control:dt_multiplier", 1.0), rate_increase=rate,
        t_stop=stop if isinstance(stop, float) else math.inf,
        min_energy=1.0e-6 * inp.float("output:min_energy") / ELEMENTARY_CHARGE if inp.contains("output:min_energy")
        else 0.0,
        max_angle=inp.float("output:max_angle", math.pi), multiplicity=mult, discard_bg_e=int(bg_e),
        discard_bg_ph=int(bg_ph), rr=int(inp.bool("control:radiation_reaction", True)),
        tracking_photons=int(inp.bool("control:pair_creation", not classical)),
        tracking_secondaries=int(inp.bool("control:track_secondaries", True)), keep_decayed_photons=int(keep_decayed),
        pol_resolved=int(inp.bool("control:pol_resolved", False)),
        rotate_stokes_pars=int(inp.bool("control:rotate_stokes_pars", True)), classical=int(classical),
        gaunt_factor=int(gaunt))


def _rotate(v, axis, theta):
    """ThreeVector::rotate_around (geometry/three_vector.rs:79-93) for the
    x or y axis, on rows of v."""
    s, c = math.sin(theta), math.cos(theta)
    ax = (1.0, 0.0, 0.0) if axis == "x" else (0.0, 1.0, 0.0)
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    a0, a1, a2 = ax
    return np.stack([
        (c + a0 * a0 * (1 - c)) * x + (a0 * a1 * (1 - c) - a2 * s) * y + (a0 * a2 * (1 - c) + a1 * s) * z,
        (a1 * a0 * (1 - c) + a2 * s) * x + (c + a1 * a1 * (1 - c)) * y + (a1 * a2 * (1 - c) - a0 * s) * z,
        (a2 * a0 * (1 - c) - a1 * s) * x + (a2 * a1 * (1 - c) + a0 * s) * y + (c + a2 * a2 * (1 - c)) * z], axis=1)


def to_beam_basis(out, theta, phi):
    """Particle::to_beam_coordinate_basis (particle/mod.rs:256-300) on the
    output arrays, in place."""
    cos_v = math.hypot(math.cos(theta), math.sin(theta) * math.cos(phi))
    if phi == 0.0 or theta == 0.0:
        vangle, hangle = 0.0, math.pi - theta
    else:
        vangle = math.copysign(math.acos(cos_v), math.sin(theta) * math.sin(phi))
        hangle = math.copysign(math.acos(-math.cos(theta) / cos_v), math.cos(phi) * math.sin(theta))
    for key in ("u", "u0", "r", "r0"):
        v = out[key]
        out[key][:, 1:] = _rotate(_rotate(v[:, 1:], "y", hangle), "x", -vangle)
    return out


def _project_to_time(parts, ct):
    """Moves every particle along its momentum to the time coordinate ct
    (main.rs:1151-1187): r + u (ct - r^0) / u^0."""
    r, u = parts["r"], parts["u"]
    if len(r):
        parts["r"] = r + u * ((ct - r[:, 0]) / u[:, 0])[:, None]


def run(path, output_dir="", engine=None, log=print):
    """Runs the input file; returns the list of files written."""
    inp = Input.from_file(path)
    ident = inp.str("output:ident", "")
    if ident == "auto":
        ident = os.path.splitext(os.path.basename(path))[0]
    dump = inp.str("output:dump_all_particles", "") if inp.contains("output:dump_all_particles") else None
    if dump is not None and dump != "hdf5":
        raise InputError("output:dump_all_particles: the only format is hdf5")
    dump_decayed = inp.bool("output:dump_decayed_photons", False)
    units = UnitSystem.named(inp.str("output:units", "auto"))
    fmt = inp.str("output:file_format", "plain_text")
    fmt = {"plain_text": "plain_text", "plain-text": "plain_text", "ascii": "plain_text", "fits": "fits"}.get(fmt)
    if fmt is None:
        fmt = "plain_text"
    dstrs = {sp: [DistributionFunction.load(s) for s in inp.list("output:" + sp)] for sp in SPECIES}
    inter_dstrs = [DistributionFunction.load(s) for s in inp.list("output:intermediate")]
    stats_specs = {sp: inp.list("stats:" + sp) for sp in SPECIES}
    inter_stats = inp.list("stats:intermediate")
    exprs = inp.list("stats:expression")
    # decayed photons are kept when any output wants them (main.rs:981-982)
    keep_decayed = bool(inter_dstrs) or bool(inter_stats) or dump_decayed
    stop = stop_mode(inp)
    beam_frame = inp.str("output:coordinate_system", "laser") == "beam"
    a0s = inp.loop("laser:a0")
    eng = engine or engine_mod.Engine()
    written = []
    if output_dir:
        os.makedirs(output_dir, exist_ok=True)
    try:
        eng.load_tables()
        seed = 0x8658B90036B165EB + inp.int("control:rng_seed", 0) * 0x32F55CDDAEBAE910
        seed &= (1 << 64) - 1
        for a0 in a0s:
            laser = laser_from_input(inp, a0)
            if inp.contains("beam:from_hdf5"):
                host, loaded = beam_from_hdf5_input(inp, laser, path)
                desc, n, species, angle, plane = None, len(host["species"]), loaded["species"], loaded["angle"], \
                    loaded["plane"]
            else:
                desc, n, species, angle, plane = beam_from_input(inp, laser, path)
                prim = eng.build_beam(desc, n, seed=seed)
                host = {k: v.cpu().numpy() for k, v in prim.items()}
                loaded = None
            rate = rate_increase_from_input(inp, eng, laser, desc, desc.spectrum_gamma if desc is not None else None)
            opts = options_from_input(inp, keep_decayed=keep_decayed, rate_increase=rate)
            out, st = eng.collide(laser, opts, host, seed=seed)
            log("a0 = %g: %d primaries -> %d particles (%d photons emitted, %d pairs), %.1f ms on the device"
                % (a0, n, st["n_out"], st["emissions"], st["pair_events"], st["device_ms"]))
            inter = (out["flags"] & 1) != 0
            decayed = {k: v[inter] for k, v in out.items()}
            out = {k: v[~inter] for k, v in out.items()}
            t_stop_global = None
            if stop == "auto":
                ct = float(np.max(out["r"][:, 0])) if len(out["r"]) else -math.inf
                _project_to_time(out, ct)
                t_stop_global = ct / SPEED_OF_LIGHT
            elif stop is not None:
                _project_to_time(out, stop * SPEED_OF_LIGHT)
                t_stop_global = stop
            if beam_frame:
                to_beam_basis(out, angle, plane)
                to_beam_basis(decayed, angle, plane)
            if dump is not None:
                cur0 = ident if len(a0s) == 1 else "%s%sa0_%.3f" % (ident, "_" if ident else "", a0)
                fname = os.path.join(output_dir, cur0 + ("_" if cur0 else "") + "particles.h5")
                write_particles_hdf5(fname, inp, path, laser, a0, desc, n, species, angle, plane, opts, out, units,
                                     not beam_frame, seed, loaded, decayed=decayed, dump_decayed=dump_decayed,
                                     t_stop_global=t_stop_global, engine=eng)
                written.append(fname)
            import torch
            device = "cuda:%d" % eng.device
            dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in out.items()}
            dev_i = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in decayed.items()}
            cur = ident if len(a0s) == 1 else "%s%sa0_%.3f" % (ident, "_" if ident else "", a0)
            base = os.path.join(output_dir, cur + ("_" if cur else "")) if output_dir else cur + ("_" if cur else "")
            for sp, code in SPECIES.items():
                for d in dstrs[sp]:
                    f = d.write(eng, dev, code, units, base + sp, fmt)
                    if f:
                        written.append(f)
            for d in inter_dstrs:
                f = d.write(eng, dev_i, abi.PHOTON, units, base + "intermediate", fmt)
                if f:
                    written.append(f)
            stat_objs = {}
            for sp, code in SPECIES.items():
                stat_objs[sp] = []
                for spec in stats_specs[sp]:
                    s = SummaryStatistic(spec)
                    s.evaluate(eng, dev, code, sp)
                    stat_objs[sp].append(s)
            # stats:intermediate is evaluated over the decayed photons but,
            # as in the reference (main.rs:1262-1287), not written to the
            # stats file
            for spec in inter_stats:
                SummaryStatistic(spec).evaluate(eng, dev_i, abi.PHOTON, "intermediate")
            lines = [str(s) for sp in ("electron", "positron", "photon") for s in stat_objs[sp]]
            for e in exprs:
                lines.append(_expression_line(inp, e))
            if lines:
                fname = base + "stats.txt"
                with open(fname, "w") as fh:
                    fh.write("\n".join(lines) + "\n")
                written.append(fname)
    finally:
        if engine is None:
            eng.close()
    return written


def _expression_line(inp, spec):
    """StatsExpression (output/stats.rs:518-575)."""
    words = spec.split()
    if len(words) < 2:
        raise InputError("cannot convert %r to a stats expression" % spec)
    name, formula = (words[0].split("`")[0], words[1]) if "`" in words[0] else (words[0], None)
    value = inp.evaluate(words[1])
    unit = words[2] if len(words) > 2 else "1"
    if formula is not None:
        return "expr: %s (%s) = %s [%s]" % (name, formula, rust_exp(value, 6), unit)
    return "expr: %s = %s [%s]" % (name, rust_exp(value, 6), unit)


# ------------------------------------------------------------ HDF5 dump ---
VACUUM_PERMITTIVITY = 8.854188e-12
ELECTRON_MASS_MEV = 0.510999


def laser_energy(laser):
    """(energy, unit) of the pulse: field/fast_focused_laser.rs:220-262 (J)
    and field/fast_plane_wave.rs:197-236 (J/m^2, per unit area), shared by
    the LMA models; None for a chirped plane wave, whose energy the
    reference integrates numerically."""
    if laser.model in (abi.PLANE_WAVE, abi.FAST_PLANE_WAVE) and laser.chirp_b != 0.0:
        return None
    omega = 2.0 * math.pi * SPEED_OF_LIGHT / laser.wavelength
    amplitude = ELECTRON_MASS * SPEED_OF_LIGHT * omega * laser.a0 / ELEMENTARY_CHARGE
    intensity = SPEED_OF_LIGHT * VACUUM_PERMITTIVITY * amplitude ** 2
    delta = 1.0 if laser.polarization == abi.CIRCULAR else 0.0
    nc = laser.n_cycles
    if laser.envelope == abi.COS2:
        duration = (1.0 + delta) * (1.0 + 3.0 * nc ** 2) * math.pi / (8.0 * nc) / omega
    elif laser.envelope == abi.GAUSSIAN:
        arg = -(math.pi * nc) ** 2 / math.log(2.0)
        large = 0.5 * nc * math.sqrt(math.pi ** 3 / math.log(2.0))
        px = large - math.expm1(arg) * math.sqrt(math.log(2.0) / math.pi) / (4.0 * nc)
        py = large + (1.0 + math.exp(arg)) * math.sqrt(math.log(2.0) / math.pi) / (4.0 * nc)
        duration = (px + delta * py) / omega
    else:
        duration = (1.0 + delta) * (nc - 3.0 / 16.0) * math.pi / omega
    if laser.model in (abi.FOCUSED_LASER, abi.FAST_FOCUSED_LASER):
        zr = math.pi * laser.waist ** 2 / laser.wavelength
        e = laser.waist / zr
        power = 0.5 * math.pi * intensity * laser.waist ** 2 * (1.0 + e * e / 4.0 + e ** 4 / 8.0)
        return power * duration, "J"
    return intensity * duration, "J/m^2"


_POL = [("linear", 0), ("circular", 1)]
_ENV = [("cos^2", 0), ("flattop", 1), ("gaussian", 2)]
_ENV_NAME = {abi.COS2: "cos^2", abi.FLATTOP: "flattop", abi.GAUSSIAN: "gaussian"}
_SPECIES_NAME = {abi.ELECTRON: "electron", abi.POSITRON: "positron", abi.PHOTON: "photon"}


def write_particles_hdf5(fname, inp, input_path, laser, a0, desc, n, species, angle, plane, opts, out, units,
                         laser_defines_z, seed, loaded=None, decayed=None, dump_decayed=False, t_stop_global=None,
                         engine=None):
    """The final-state file of main.rs:1289-1715: build information, the
    parsed configuration, and every final-state particle by species, in the
    output unit system, each dataset with its `unit` and `desc`
    attributes and the reference's aliases."""
    root = hdf5.Group()
    b = root.group("build")
    b.dataset("version", "ptarmigan-gb300")
    b.dataset("branch", "")
    b.dataset("commit-hash", "")
    b.dataset("features", "gb300")
    conf = root.group("config")
    conf.dataset("mpi-tasks", 1)
    with open(input_path, "r") as fh:
        conf.dataset("input-file", fh.read())
    u = conf.group("unit")
    u.dataset("position", units.length.name)
    u.dataset("momentum", units.momentum.name)
    c = conf.group("control")
    c.dataset("dt_multiplier", float(opts.dt_multiplier))
    c.dataset("radiation_reaction", bool(opts.rr))
    c.dataset("classical", bool(opts.classical))
    c.dataset("pair_creation", bool(opts.tracking_photons))
    c.dataset("pair_creation_is_pol_resolved", bool(opts.pol_resolved))
    c.dataset("lcfa", laser.model in (abi.FAST_PLANE_WAVE, abi.FAST_FOCUSED_LASER))
    c.dataset("rng_seed", inp.int("control:rng_seed", 0))
    c.dataset("increase_pair_rate_by", float(opts.rate_increase))
    c.dataset("bandwidth_correction", bool(laser.finite_bandwidth))
    if t_stop_global is not None:
        c.dataset("stop_at_time", float(t_stop_global), unit="s",
                  desc="tracking has continued until all particles have this time coordinate")
    c.dataset("select_multiplicity", int(opts.multiplicity) if opts.multiplicity >= 0 else False)
    focusing = laser.model in (abi.FOCUSED_LASER, abi.FAST_FOCUSED_LASER)
    lz = conf.group("laser")
    L = units.length
    lz.dataset("a0", float(a0), unit="1", desc="peak value of the laser normalized amplitude")
    lz.dataset("wavelength", laser.wavelength * L.scale, unit=L.name, desc="wavelength of the carrier")
    lz.dataset("polarization", hdf5.Enum(_POL, "circular" if laser.polarization == abi.CIRCULAR else "linear"),
               desc="linear/circular")
    if laser.polarization == abi.LINEAR:
        lz.dataset("polarization_angle", float(laser.pol_angle), unit="rad",
                   desc="angle between x-axis and electric field")
    lz.dataset("focusing", focusing, desc="true/false => pulse is modelled in 3d/1d")
    lz.dataset("envelope", hdf5.Enum(_ENV, _ENV_NAME[laser.envelope]),
               desc="pulse envelope of the laser vector potential")
    lz.dataset("chirp_b", float(laser.chirp_b), unit="1", desc="parameter that appears in carrier phase = phi + b phi^2")
    if focusing:
        lz.dataset("waist", laser.waist * L.scale, unit=L.name,
                   desc="radius in the focal plane at which intensity is 1/e^2 of its peak value")
    if laser.envelope == abi.GAUSSIAN:
        lz.dataset("fwhm_duration", laser.n_cycles * laser.wavelength / SPEED_OF_LIGHT, unit="s",
                   desc="full width at half maximum of the temporal intensity profile")
    else:
        lz.dataset("n_cycles", float(laser.n_cycles), unit="1",
                   desc="number of wavelengths corresponding to the total pulse duration")
    bm = conf.group("beam")
    bm.dataset("n", int(n), unit="1", desc="number of primary macroparticles")
    bm.dataset("species", _SPECIES_NAME[species])
    bm.dataset("collision_angle", float(angle), unit="rad",
               desc="polar angle between beam momentum and laser wavevector, zero if counterpropagating")
    bm.dataset("collision_plane_angle", float(plane), unit="rad",
               desc="azimuthal angle between beam momentum and laser wavevector, zero if p in E, k plane")
    if desc is None:
        # a beam loaded from file (main.rs:1446-1462)
        bm.dataset("offset", hdf5.Vector(np.asarray(loaded["offset"]) * L.scale), unit=L.name)
        bm.dataset("imported_from_file", True)
        bm.dataset("distance_bt_ips", loaded["distance"] * L.scale, unit=L.name,
                   desc="distance between particle beam source and focal spot")
        bm.dataset("min_energy", loaded["min_energy"] * units.energy.scale, unit=units.energy.name,
                   desc="primaries with energies below this threshold are discarded")
        bm.dataset("max_angle", float(loaded["max_angle"]), unit="rad",
                   desc="primaries propagating at angles larger than this are discarded")
        _write_output_config(conf, opts, units, laser_defines_z)
        _write_final_state(root, laser, out, units, focusing, decayed, dump_decayed, engine)
        hdf5.write(fname, root)
        return
    bm.dataset("offset", hdf5.Vector(np.asarray(list(desc.offset)) * L.scale), unit=L.name)
    bm.dataset("imported_from_file", False)
    bm.dataset("n_real", n * desc.weight, unit="1",
               desc="total number of real particles represented by the primary macroparticles")
    charge = {abi.ELECTRON: 1.0, abi.POSITRON: -1.0, abi.PHOTON: 0.0}[species] * n * desc.weight * -ELEMENTARY_CHARGE
    bm.dataset("charge", charge, unit="C")
    brem = desc.gamma_dstr == abi.GAMMA_BREM
    bm.dataset("gamma", float(desc.gamma_max if brem else desc.gamma_mean), unit="1")
    bm.dataset("sigma", float(desc.gamma_sigma), unit="1")
    bm.dataset("bremsstrahlung_source", bool(brem))
    if brem:
        bm.dataset("gamma_min", float(desc.gamma_min), unit="1")
    if desc.radial_dstr == abi.RADIAL_UNIFORM:
        radius, r_max = desc.r_max, desc.r_max
    elif desc.radial_dstr == abi.RADIAL_TRUNC_NORMAL:
        radius, r_max = desc.sigma_x, desc.x_max
    else:
        radius, r_max = desc.sigma_x, math.inf
    bm.dataset("radius", radius * L.scale, unit=L.name)
    bm.dataset("radius_max", r_max * L.scale, unit=L.name,
               desc="density distribution is cut off at this perpendicular distance from the beam axis")
    bm.dataset("length", desc.sigma_z * L.scale, unit=L.name)
    bm.dataset("rms_divergence", float(desc.rms_div), unit="rad")
    bm.dataset("polarization", hdf5.Vector(list(desc.pol)), unit="1",
               desc="Stokes parameters of the primary particles: I, Q, U, V", alias="polarisation")
    bm.dataset("transverse_distribution_is_normal", desc.radial_dstr != abi.RADIAL_UNIFORM)
    bm.dataset("longitudinal_distribution_is_normal", True)
    _write_output_config(conf, opts, units, laser_defines_z)
    _write_final_state(root, laser, out, units, focusing, decayed, dump_decayed, engine)
    hdf5.write(fname, root)


def _write_output_config(conf, opts, units, laser_defines_z):
    E = units.energy
    op = conf.group("output")
    op.dataset("laser_defines_positive_z", bool(laser_defines_z))
    op.dataset("beam_defines_positive_z", not laser_defines_z)
    op.dataset("discard_background_e", bool(opts.discard_bg_e))
    op.dataset("discard_background_ph", bool(opts.discard_bg_ph))
    op.dataset("min_energy", opts.min_energy * E.scale, unit=E.name)  # opts.min_energy is in MeV


def _write_intermediate_state(root, decayed, units):
    """main.rs:1633-1688: the photons that decayed into pairs, as they were
    when they decayed."""
    L, P = units.length, units.momentum
    g = root.group("intermediate-state").group("photon")
    g.dataset("weight", decayed["weight"], unit="1", desc="number of real photons each macrophoton represents")
    g.dataset("a0_at_creation", decayed["payload"], unit="1",
              desc="normalized amplitude (RMS under LMA) at point of emission", alias="xi")
    g.dataset("parent_chi", decayed["parent_chi"], unit="1",
              desc="quantum parameter (RMS under LMA) of parent at point of emission")
    g.dataset("n_pos", decayed["interaction_count"], unit="1",
              desc="total probability of pair creation for the photon")
    g.dataset("id", decayed["id"], desc="unique ID of the photon")
    g.dataset("parent_id", decayed["parent_id"],
              desc="ID of the particle that created the photon (for primary particles, parent_id = id")
    g.dataset("polarization", decayed["pol"], desc="Stokes parameters of the photon: I, Q, U, V", unit="1",
              alias="polarisation")
    g.dataset("position", decayed["r"] * L.scale, unit=L.name, desc="four-position of the photon")
    g.dataset("momentum", decayed["u"] * (ELECTRON_MASS_MEV * P.scale), unit=P.name,
              desc="four-momentum of the photon")


def chirped_energy_flux(laser, engine):
    """FastPlaneWave::integrated_intensity (field/fast_plane_wave.rs:56-85),
    the energy per unit area of a chirped plane wave: the field energy
    density at 10 (1 + 2 pi b n_cycles) points per wavelength along the
    pulse, summed with alternating 2/3, 4/3 weights and Kahan compensation.
    The fields are the device's FP64 FastPlaneWave fields."""
    ppw = int(10.0 * (1.0 + 2.0 * math.pi * laser.chirp_b * laser.n_cycles))
    nc = laser.n_cycles
    max_phase = {abi.COS2: math.pi * nc, abi.FLATTOP: math.pi * (nc + 1.0)}.get(laser.envelope, 6.0 * math.pi * nc)
    k = 2.0 * math.pi / laser.wavelength
    dphi = 2.0 * math.pi / ppw
    dz = dphi / k
    n_pts = int(max_phase / dphi)
    idx = np.arange(-n_pts, n_pts)
    r = np.zeros((len(idx), 4))
    r[:, 3] = -(idx * dphi) / k
    fpw = abi.laser_desc(abi.FAST_PLANE_WAVE, laser.a0, laser.wavelength, laser.polarization, laser.envelope,
                         n_cycles=nc, chirp_b=laser.chirp_b)
    E, B, _ = engine.fields(fpw, r)
    dens = 0.5 * VACUUM_PERMITTIVITY * (np.sum(E * E, axis=1) + SPEED_OF_LIGHT ** 2 * np.sum(B * B, axis=1))
    flux, comp = 0.0, 0.0
    for n, u in zip(idx, dens):
        w = 2.0 / 3.0 if n % 2 == 0 else 4.0 / 3.0
        y = w * float(u) * dz - comp
        t = flux + y
        comp = (t - flux) - y
        flux = t
    return flux


def _write_final_state(root, laser, out, units, focusing, decayed=None, dump_decayed=False, engine=None):
    L, E = units.length, units.energy
    P = units.momentum
    fs = root.group("final-state")

    def pick(code):
        sel = out["species"] == code
        return {k: v[sel] for k, v in out.items()}

    ph = pick(abi.PHOTON)
    g = fs.group("photon")
    g.dataset("weight", ph["weight"], unit="1", desc="number of real photons each macrophoton represents")
    g.dataset("a0_at_creation", ph["payload"], unit="1",
              desc="normalized amplitude (RMS under LMA) at point of emission", alias="xi")
    g.dataset("parent_chi", ph["parent_chi"], unit="1",
              desc="quantum parameter (RMS under LMA) of parent at point of emission")
    g.dataset("n_pos", ph["interaction_count"], unit="1", desc="total probability of pair creation for the photon")
    g.dataset("id", ph["id"], desc="unique ID of the photon")
    g.dataset("parent_id", ph["parent_id"],
              desc="ID of the particle that created the photon (for primary particles, parent_id = id")
    g.dataset("polarization", ph["pol"], unit="1", desc="Stokes parameters of the photon: I, Q, U, V",
              alias="polarisation")
    g.dataset("position", ph["r"] * L.scale, unit=L.name, desc="four-position of the photon")
    g.dataset("momentum", ph["u"] * (ELECTRON_MASS_MEV * P.scale), unit=P.name, desc="four-momentum of the photon")
    for code, name in ((abi.ELECTRON, "electron"), (abi.POSITRON, "positron")):
        q = pick(code)
        g = fs.group(name)
        g.dataset("weight", q["weight"], unit="1", desc="number of real %ss each macro%s represents" % (name, name))
        if code == abi.POSITRON:
            g.dataset("a0_at_creation", q["payload"], unit="1",
                      desc="normalized amplitude (RMS under LMA) at point of creation", alias="xi")
            g.dataset("parent_chi", q["parent_chi"], unit="1",
                      desc="quantum parameter (RMS under LMA) of parent at point of creation")
        g.dataset("n_gamma", q["interaction_count"], unit="1",
                  desc="total number of photons emitted by the %s" % name)
        g.dataset("id", q["id"], desc="unique ID of the %s" % name)
        g.dataset("parent_id", q["parent_id"],
                  desc="ID of the particle that created the %s (for primary particles, parent_id = id)" % name)
        g.dataset("absorption", q["work"] * (ELECTRON_MASS_MEV * E.scale), unit=E.name,
                  desc="energy absorbed from the laser")
        g.dataset("position", q["r"] * L.scale, unit=L.name, desc="four-position of the %s" % name)
        if code == abi.POSITRON:
            g.dataset("position_at_creation", q["r0"] * L.scale, unit=L.name,
                      desc="four-position at which the positron was created")
        g.dataset("momentum", q["u"] * (ELECTRON_MASS_MEV * P.scale), unit=P.name,
                  desc="four-momentum of the %s" % name)
    if dump_decayed and decayed is not None:
        _write_intermediate_state(root, decayed, units)
    lg = fs.group("laser")
    en = laser_energy(laser)
    if en is None and engine is not None:
        en = (chirped_energy_flux(laser, engine), "J/m^2")
    if en is not None:
        if focusing:
            lg.dataset("energy", en[0], unit=en[1], desc="total energy of the laser pulse")
        else:
            lg.dataset("energy_flux", en[0], unit=en[1], desc="total energy of the laser pulse, per unit area")
    # over every particle, the decayed photons included (main.rs:1141-1146)
    work = float(np.sum(out["weight"] * out["work"]))
    if decayed is not None and len(decayed["weight"]):
        work += float(np.sum(decayed["weight"] * decayed["work"]))
    absorption = work * ELECTRON_MASS_MEV * 1.0e6 * ELEMENTARY_CHARGE
    lg.dataset("absorption", absorption, unit="J", desc="energy absorbed from the laser")


# ------------------------------------------------------------ HDF5 load ---
_LENGTH_UNITS = {"um": 1.0e6, "micron": 1.0e6, "mm": 1.0e3, "m": 1.0}
_MOMENTUM_UNITS = {"MeV/c": 1.0, "MeV": 1.0, "GeV/c": 1.0e-3, "GeV": 1.0e-3,
                   "kg/m/s": 1.0 / (1.0e6 * ELEMENTARY_CHARGE / SPEED_OF_LIGHT)}


def _h5_get(tree, path):
    node = tree
    for part in path.split("/"):
        if node.get("kind") != "group" or part not in node["members"]:
            return None
        node = node["members"][part]
    return node


def load_beam_hdf5(fname, species, distance, collision_angle, offset, auto_timing, min_energy, max_angle,
                   initial_z):
    """BeamLoader::build (particle/loader.rs:142-284) for files this
    package's HDF5 module can read (its own final-state files, or files of
    the same structures): the species' weight, position, momentum and
    optional polarization in the file's units, rotated from the file's
    beam axis onto the collision axis, shifted by the offset, propagated
    between the interaction points (auto timing), and filtered by energy
    (MeV) and angle.  Returns primaries for Engine.collide."""
    tree = hdf5.read(fname)
    sp = _SPECIES_NAME[species]

    def need(path):
        node = _h5_get(tree, path)
        if node is None or node["kind"] != "dataset":
            raise InputError("%s has no dataset %s" % (fname, path))
        return node["value"]

    x_unit = _LENGTH_UNITS.get(need("config/unit/position"))
    p_unit = _MOMENTUM_UNITS.get(need("config/unit/momentum"))
    if x_unit is None or p_unit is None:
        raise InputError("%s: unrecognised position or momentum unit" % fname)

    def flag(path):
        node = _h5_get(tree, path)
        return node is not None and node["kind"] == "dataset" and node["value"] is True

    ca = _h5_get(tree, "config/beam/collision_angle")
    ax = _h5_get(tree, "beam_axis")
    if flag("config/output/beam_defines_positive_z"):
        beam_axis = np.array([0.0, 0.0, 1.0])
    elif flag("config/output/laser_defines_positive_z") and ca is not None:
        beam_axis = np.array([-math.sin(ca["value"]), 0.0, -math.cos(ca["value"])])
    elif ax is not None and ax["value"] in ("+x", "-x", "+z", "-z"):
        beam_axis = {"+x": (1.0, 0.0, 0.0), "-x": (-1.0, 0.0, 0.0), "+z": (0.0, 0.0, 1.0),
                     "-z": (0.0, 0.0, -1.0)}[ax["value"]]
        beam_axis = np.array(beam_axis)
    else:
        beam_axis = np.array([0.0, 0.0, 1.0])  # the reference warns and assumes this
    new_axis = np.array([-math.sin(collision_angle), 0.0, -math.cos(collision_angle)])
    cross_y = beam_axis[2] * new_axis[0] - beam_axis[0] * new_axis[2]
    theta = math.copysign(abs(math.acos(float(np.dot(new_axis, beam_axis)))), cross_y)

    w = np.asarray(need("final-state/%s/weight" % sp), dtype=np.float64)
    r = np.asarray(need("final-state/%s/position" % sp), dtype=np.float64).reshape(-1, 4) / x_unit
    p = np.asarray(need("final-state/%s/momentum" % sp), dtype=np.float64).reshape(-1, 4) / p_unit
    pol_node = _h5_get(tree, "final-state/%s/polarization" % sp)
    m = min(len(w), len(r), len(p))
    w, r, p = w[:m], r[:m], p[:m]
    pol = (np.asarray(pol_node["value"], dtype=np.float64).reshape(-1, 4)[:m] if pol_node is not None
           else np.tile([1.0, 0.0, 0.0, 0.0], (m, 1)))
    u = p / ELECTRON_MASS_MEV

    def rot_y(v):  # FourVector::rotate_around_y
        sn, cs = math.sin(theta), math.cos(theta)
        o = v.copy()
        o[:, 1] = cs * v[:, 1] + sn * v[:, 3]
        o[:, 3] = cs * v[:, 3] - sn * v[:, 1]
        return o

    u, r = rot_y(u), rot_y(r)
    sa, ca_ = math.sin(collision_angle), math.cos(collision_angle)
    ox, oy, oz = offset
    r[:, 1] += ca_ * ox + sa * oz  # ThreeVector::rotate_around_y(angle) of the offset
    r[:, 2] += oy
    r[:, 3] += ca_ * oz - sa * ox
    if auto_timing:
        beta = u / u[:, :1]
        den = (beta[:, 0] - beta[:, 3])[:, None]
        lead = np.array([-1.0, sa, 0.0, ca_])
        shift = distance * (lead[None, :] + (1.0 + ca_) * beta / den)
        shift = shift - (2.0 * initial_z + r[:, :1] - r[:, 3:4]) * beta / den
        r = r + shift
    e = ELECTRON_MASS_MEV * u[:, 0]
    n3 = u[:, 1:] / np.linalg.norm(u[:, 1:], axis=1, keepdims=True)
    keep = (e > min_energy) & (n3 @ new_axis > math.cos(max_angle))
    idx = np.nonzero(keep)[0].astype(np.uint64)
    k = len(idx)
    return {"species": np.full(k, species, dtype=np.int32), "r": np.ascontiguousarray(r[keep]),
            "u": np.ascontiguousarray(u[keep]), "pol": np.ascontiguousarray(pol[keep]),
            "weight": np.ascontiguousarray(w[keep]), "id": idx.copy(), "parent_id": idx.copy()}


def beam_from_hdf5_input(inp, laser, input_path):
    """main.rs:533-560: beam:from_hdf5 (file relative to the input file,
    distance_bt_ips, auto_timing, min_energy in J, max_angle) with
    beam:species, collision_angle and offset."""
    species = SPECIES.get(inp.str("beam:species", "electron"))
    if species is None:
        raise InputError("beam:species must be electron, positron or photon")
    fname = inp.str("beam:from_hdf5:file")
    if not os.path.isabs(fname):
        fname = os.path.join(os.path.dirname(os.path.abspath(input_path)), fname)
    distance = inp.float("beam:from_hdf5:distance_bt_ips")
    auto_timing = inp.bool("beam:from_hdf5:auto_timing", True)
    min_energy = 1.0e-6 * inp.float("beam:from_hdf5:min_energy") / ELEMENTARY_CHARGE \
        if inp.contains("beam:from_hdf5:min_energy") else 0.0
    max_angle = inp.float("beam:from_hdf5:max_angle", math.pi)
    angle = inp.float("beam:collision_angle", 0.0)
    plane_s = inp.str("beam:collision_plane", "horizontal")
    plane = {"horizontal": 0.0, "vertical": math.pi / 2}.get(plane_s)
    if plane is None:
        plane = inp.evaluate(plane_s)
    offset = inp.floats("beam:offset", [0.0, 0.0, 0.0])
    prim = load_beam_hdf5(fname, species, distance, angle, offset, auto_timing, min_energy, max_angle,
                          engine_mod.laser_initial_z(laser))
    return prim, {"species": species, "angle": angle, "plane": plane, "offset": offset, "distance": distance,
                  "min_energy": min_energy, "max_angle": max_angle}
