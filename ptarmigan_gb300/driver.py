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
stats (electron / photon / positron, and expressions) and constants.
Not supported: beam:spectrum, beam:from_hdf5, output:dump_all_particles,
intermediate-particle output, increase_pair_rate_by: auto and
stop_at_time: auto.
"""

import math
import os

import numpy as np

from . import abi, engine as engine_mod
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


def beam_from_input(inp, laser):
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
    if inp.contains("beam:spectrum"):
        raise InputError("beam:spectrum is not supported by this driver")
    brem = species == abi.PHOTON and inp.bool("beam:bremsstrahlung_source", False)
    kw = {}
    if brem:
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
    return desc, n, species, inp.float("beam:collision_angle", 0.0), plane


def options_from_input(inp, keep_decayed):
    """main.rs:339-398, 862-880 and 1106-1124."""
    classical_s = inp.str("control:classical", "false")
    classical, gaunt = {"true": (True, False), "false": (False, False),
                        "gaunt_factor_corrected": (True, True)}.get(classical_s, (None, None))
    if classical is None:
        raise InputError("control:classical must be one of 'true', 'false' or 'gaunt_factor_corrected'")
    mult = inp.int("control:select_multiplicity") if inp.contains("control:select_multiplicity") else -1
    rate = inp.float("control:increase_pair_rate_by", 1.0)
    if rate < 1.0:
        raise InputError("increase in pair creation rate must be >= 1.0")
    stop = inp.str("control:stop_at_time", "")
    if stop == "auto":
        raise InputError("control:stop_at_time: auto is not supported by this driver")
    if inp.contains("output:discard_background"):
        bg_e = bg_ph = inp.bool("output:discard_background")
    else:
        bg_e, bg_ph = inp.bool("output:discard_background_e", False), False
    return abi.collide_options(
        dt_multiplier=inp.float("control:dt_multiplier", 1.0), rate_increase=rate,
        t_stop=inp.evaluate(stop) if stop else math.inf,
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


def run(path, output_dir="", engine=None, log=print):
    """Runs the input file; returns the list of files written."""
    inp = Input.from_file(path)
    ident = inp.str("output:ident", "")
    if ident == "auto":
        ident = os.path.splitext(os.path.basename(path))[0]
    if inp.contains("output:dump_all_particles"):
        raise InputError("output:dump_all_particles is not supported by this driver")
    if inp.list("output:intermediate") or inp.list("stats:intermediate"):
        raise InputError("intermediate-particle output is not supported by this driver")
    units = UnitSystem.named(inp.str("output:units", "auto"))
    fmt = inp.str("output:file_format", "plain_text")
    fmt = {"plain_text": "plain_text", "plain-text": "plain_text", "ascii": "plain_text", "fits": "fits"}.get(fmt)
    if fmt is None:
        fmt = "plain_text"
    dstrs = {sp: [DistributionFunction.load(s) for s in inp.list("output:" + sp)] for sp in SPECIES}
    stats_specs = {sp: inp.list("stats:" + sp) for sp in SPECIES}
    exprs = inp.list("stats:expression")
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
            desc, n, species, angle, plane = beam_from_input(inp, laser)
            opts = options_from_input(inp, keep_decayed=False)
            prim = eng.build_beam(desc, n, seed=seed)
            host = {k: v.cpu().numpy() for k, v in prim.items()}
            out, st = eng.collide(laser, opts, host, seed=seed)
            log("a0 = %g: %d primaries -> %d particles (%d photons emitted, %d pairs), %.1f ms on the device"
                % (a0, n, st["n_out"], st["emissions"], st["pair_events"], st["device_ms"]))
            if beam_frame:
                to_beam_basis(out, angle, plane)
            import torch
            dev = {k: torch.from_numpy(np.ascontiguousarray(v)).to("cuda:%d" % eng.device) for k, v in out.items()}
            cur = ident if len(a0s) == 1 else "%s%sa0_%.3f" % (ident, "_" if ident else "", a0)
            base = os.path.join(output_dir, cur + ("_" if cur else "")) if output_dir else cur + ("_" if cur else "")
            for sp, code in SPECIES.items():
                for d in dstrs[sp]:
                    f = d.write(eng, dev, code, units, base + sp, fmt)
                    if f:
                        written.append(f)
            stat_objs = {}
            for sp, code in SPECIES.items():
                stat_objs[sp] = []
                for spec in stats_specs[sp]:
                    s = SummaryStatistic(spec)
                    s.evaluate(eng, dev, code, sp)
                    stat_objs[sp].append(s)
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
