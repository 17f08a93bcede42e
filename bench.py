"""Benchmark of the collision loop: collided primaries/s (showers included),
the learned proposal in the persistent queue against the reference's table
sampler, at a fixed KS distance on the photon spectrum.

Default workload, the polarisation-resolved CP shower (one "step" = one
batch of 1e7 primaries through the collision loop): electrons at 16.5 GeV,
0.1% rms energy spread, 5 x 5 x 24 um rms, 8 urad divergence, head-on with
a circularly polarised focused Gaussian laser (FocusedLaser, LMA) a0 = 5,
w0 = 3 um, 0.8 um, 30 fs FWHM; photon Stokes parameters tracked
(pol_resolved), pair creation on, all secondaries tracked.  Inputs are
seeded synthetic beams with those distributions (the reference has no
public dataset); the input and the shower store are far larger than L2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload cp_shower|lcfa_shower|plane_wave_lma|a0_scan|learned_sampler]

Prints one JSON line.  For cp_shower:
  value         the learned proposal inside the persistent single-collision
                queue kernel (CUDA graph, autotuned launch shape), primaries
                resident in HBM, seeds 1000 .. 1000+K-1;
  plain_value   the reference's table sampler through the wave kernels;
  cross_terms   learned proposal + waves and table sampler + queue, so that
                the gain splits into sampler and scheduler (all four arms
                run the same K seeds);
  e2e           the value path through ptg_collide_multi with host buffers
                (page-locked primaries in, the shower out), same K seeds;
  ks_*          photon-energy KS distance between the value path and the
                plain path (seed 1000), against its 1e-3 critical value;
  parity        the oracle (C++ FP64 restatement of the reference) against
                the GPU on the cpu_baseline sample (same primaries, seed and
                id base): particles matched by random stream, momenta within
                tolerance, KS and chi-square on the photon spectra, pair
                yield, Stokes parameters and electron energy loss;
  roofline      the value path's dominant kernel on the FP64 pipe.
--impl reference times the oracle on all host cores (the Rust reference
cannot be built: no cargo or rustc).

Other workloads (--workload), each one JSON line of the same metric:
  lcfa_shower     1e6 electrons at 10 GeV, 1% spread, 2 x 2 x 20 um, 50 urad,
                  on a linearly polarised focused Gaussian laser (LCFA,
                  FastFocusedLaser) a0 = 10, w0 = 4 um, 0.8 um, 30 fs; pairs
                  on, secondaries tracked to generation 2.  `value` runs the
                  wave kernels, `queue_value` the same batches through the
                  single-collision queue kernel.
  plane_wave_lma  1e4 electrons at 5 GeV, 0.1% spread, 1 x 1 x 10 um, on a
                  linearly polarised plane wave (LMA), a0 = 1, 0.8 um, cos^2
                  envelope of 30 fs intensity FWHM (30.9 cycles), emission
                  only.
  a0_scan         64 collisions in one persistent queue launch: a0
                  log-spaced 0.5..20, beams log-uniform 1e3..1e6 electrons
                  (seeded) at 16.5 GeV, 0.1% spread, 2 x 2 x 20 um, 8 urad, on
                  a linearly polarised focused Gaussian laser, w0 = 5 um,
                  0.8 um, 25 fs; LMA below a0 = 5, LCFA above; pairs on.
                  The autotuner picks the queue kernel's launch shape
                  (usually the lockstep multi-collision variant);
                  `plain_value` runs the same collisions one call each.
  learned_sampler the CP photon-energy sampler alone, learned proposal
                  against the table sampler on 1e7 emissions per step.
"""

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "collided primaries/s incl. showers: learned vs table sampler at fixed KS error"
UNIT = "primaries/s"
SEED0 = 1000

# Algorithmic FP64 flops per event of the collision loop: the reference's
# formulas counted by hand (+, -, * one flop each, a fused multiply-add two;
# each library call at its executed cost on this GPU, measured with
# ptg_fp64_function_kernel under ncu: exp 30, log 44, division 10, sqrt 13,
# cbrt 16, sincos 37, pow 121, atan2 57, hypot 16, log1p 37, acos 31).
# Cross-checked against ncu's executed DFMA/DMUL/DADD counts: the LMA push
# alone (ptg_push_steps) executes 204.5 flops per step against 208 counted;
# the CP lepton wave of 2e5 primaries, emissions included, executes 16.25
# GFLOP against 14.7 counted.
OPS = {
    # FocusedLaser (LMA, CP), a step in the pulse: lma_push (gradient of
    # <a^2> at the midpoint, <a^2> at the end: 105 + 3 div + 2 exp + sqrt =
    # 208), the emission step up to its FP32 bound (a^2, eta, kappa and the
    # draw: 20) and the loop's phase tests (10)
    "lma_lepton_step": 238.0,
    # outside the pulse: two half drifts (16); the phase tests run once per
    # run of field-free steps (lma_free_run), not per step
    "free_lepton_step": 16.0,
    # a photon step in the LMA field: the drift (8), the phase test (3),
    # <a^2> and its root (70), eta, the phase step and the rate prefactor
    # (33), the Stokes parameters into and out of the LMA basis (one basis,
    # 68), the rotations by the polarisation angle (16 at angle zero, where
    # sincos is exact and skipped), the probability and the Stokes update
    # (50); the Breit-Wheeler table lookup (170) where the rate is not
    # negligible: 258 without, 428 with.  The mean, 354, is the earlier
    # build's measured 480 per step less the 126 those two changes removed.
    "lma_photon_step": 354.0,
    # one emission sampled by the reference's CP sampler (table inversion,
    # the 32-point ceiling, the trials, the finish and the kinematics):
    # about 15.9 kflop per emission at a in [0.5, 5] and eta in [0.1, 0.2]
    # (the serial sampler, ncu)
    "cp_emission": 15.9e3,
    # FastFocusedLaser (LCFA, LP): the half drift (8), the fields at the
    # half step in FP64 (271: phase, envelope, the paraxial beam and its
    # complex products; the eps^2..eps^4 corrections are FP32) and the Vay
    # push (206, with three reciprocal square roots), the emission step's
    # draw (its probability is FP32): 488 (the push alone executes 439.5)
    "lcfa_lepton_step": 488.0,
    # outside the envelope: the half drifts, gamma and the phase test
    "lcfa_free_lepton_step": 40.0,
    # a photon step: the drift and the phase test in FP64 (the fields, chi
    # and the pair rate are FP32)
    "lcfa_photon_step": 12.0,
    # a drifting photon's step: the drift
    "free_photon_step": 8.0,
    # one LCFA emission sampled (lcfa_photon_sample, ncu: 2686 per call)
    "lcfa_emission": 2686.0,
}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            for k, name in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ------------------------------------------------------------- workloads --
def cp_shower_workload(n, seed):
    """The polarisation-resolved CP LMA shower (see the module docstring)."""
    from ptarmigan_gb300 import abi, beam
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6, fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(n, g, sigma=0.001 * g, radius=5e-6, length=24e-6, rms_div=8e-6, laser=laser, seed=seed)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    return laser, opts, prim


def lcfa_workload(n, seed):
    """The focused LCFA shower (see the module docstring)."""
    from ptarmigan_gb300 import abi, beam
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(n, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=seed)
    opts = abi.collide_options(max_generation=2)
    return laser, opts, prim


# the focused LCFA shower, kept under its earlier name for callers
workload = lcfa_workload


def plane_wave_lma_workload(n, seed):
    from ptarmigan_gb300 import abi, beam
    # cos^2 envelope of total duration T: intensity FWHM = 0.364 T, so
    # 30 fs FWHM is T = 82.4 fs = 30.9 cycles of 0.8 um light
    laser = abi.laser_desc(abi.PLANE_WAVE, 1.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=30.9)
    g = beam.gamma_from_energy(5.0)
    prim = beam.build(n, g, sigma=0.001 * g, radius=1e-6, length=10e-6, rms_div=0.0, laser=laser, seed=seed)
    opts = abi.collide_options(tracking_photons=0)
    return laser, opts, prim


def a0_scan_workload(seed, scale=1.0):
    """64 collisions (laser, primaries) of the a0 scan; `scale` shrinks the
    beams (for tests of the harness)."""
    from ptarmigan_gb300 import abi, beam
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(1e6), 64))
    colls, prims, first = [], [], 0
    for k, a0 in enumerate(np.geomspace(0.5, 20.0, 64)):
        model = abi.FOCUSED_LASER if a0 < 5.0 else abi.FAST_FOCUSED_LASER
        laser = abi.laser_desc(model, float(a0), 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=5e-6, fwhm_duration=25e-15)
        n = max(1, int(round(sizes[k] * scale)))
        g = beam.gamma_from_energy(16.5)
        p = beam.build(n, g, sigma=0.001 * g, radius=2e-6, length=20e-6, rms_div=8e-6, laser=laser,
                       seed=int(seed * 1000 + k))
        prims.append(p)
        colls.append({"laser": laser, "seed": seed * 100 + k, "id_base": 1 << 40 | (k << 32), "first": first,
                      "count": n})
        first += n
    prim = {key: np.concatenate([p[key] for p in prims]) for key in prims[0]}
    return colls, abi.collide_options(), prim


WORKLOADS = {
    "cp_shower": ("cp_shower: 1e7 e- 16.5 GeV 0.1%, 5x5x24 um, 8 urad; CP FocusedLaser (LMA) a0=5 w0=3 um 0.8 um "
                  "30 fs; Stokes tracked (pol_resolved), pairs on, all generations", cp_shower_workload, 10_000_000),
    "lcfa_shower": ("lcfa_shower: 1e6 e- 10 GeV 1% spread, 2x2x20 um, 50 urad; FastFocusedLaser (LCFA) a0=10 w0=4 um "
                    "0.8 um 30 fs LP; pairs on; generations<=2", lcfa_workload, 1_000_000),
}

MLP_MARGIN = 0.25  # ln of the learned envelope's safety factor
MLP_TRAIN = dict(n_samples=50_000_000, batch=16384, epochs=3, lr=2e-3, tau=0.98, seed=7)


def train_network(eng, args=None):
    cfg = dict(MLP_TRAIN)
    if args is not None and getattr(args, "train_samples", 0):
        cfg["n_samples"] = args.train_samples
    if args is not None and getattr(args, "train_epochs", 0):
        cfg["epochs"] = args.train_epochs
    eng.mlp_init(3)
    return dict(eng.mlp_train(**cfg), **cfg)


def ks_distance(a, b):
    from ptarmigan_gb300 import equivalence
    return equivalence.ks_distance(a, b)


def ks_critical(n, m, alpha=1e-3):
    from ptarmigan_gb300 import equivalence
    return equivalence.ks_critical(n, m, alpha)


def nbytes(d):
    return int(sum(v.nbytes for v in d.values()))


def step_summary(ms):
    a = np.asarray(ms, dtype=float)
    return {"ms": [round(float(x), 3) for x in a], "mean": float(a.mean()), "p50": float(np.percentile(a, 50)),
            "p90": float(np.percentile(a, 90)), "max": float(a.max()), "min": float(a.min())}


def pinned_copy(prim):
    """The primaries in page-locked host memory, as a caller streaming
    batches to the device would hold them."""
    import torch
    out = {}
    for key, v in prim.items():
        buf = torch.empty(max(1, v.nbytes), dtype=torch.uint8, pin_memory=True).numpy()
        a = buf[:v.nbytes].view(v.dtype).reshape(v.shape)
        a[...] = v
        out[key] = a
    return out


# ------------------------------------------------------------- CPU legs --
def oracle_run(laser, opts, prim, seed, threads, id_base=None):
    """The oracle (CPU restatement of the reference) on a batch, timed."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    out, st = oracle.collide(laser, opts, prim, seed=seed, id_base=id_base, threads=threads)
    return out, st, time.perf_counter() - t0


def run_reference(args, rank, world):
    """--impl reference: the oracle on all host cores, a bounded sample of
    the workload per step, seeds 1000 .. 1000+K-1."""
    if rank != 0:
        return
    threads = cpu_threads()
    desc, make, _n = WORKLOADS[args.workload if args.workload in WORKLOADS else "cp_shower"]
    per_core = args.cpu_sample_per_core or (2500 if make is cp_shower_workload else 400)
    n_sample = max(64, per_core * threads)
    laser, opts, prim = make(n_sample, 7)
    for w in range(max(1, min(args.warmup, 1))):
        small = {k: v[:min(n_sample, 16 * threads)] for k, v in prim.items()}
        oracle_run(laser, opts, small, 99, threads)
    vals, t_all = [], 0.0
    for k in range(args.steps):
        _, _, dt = oracle_run(laser, opts, prim, SEED0 + k, threads, id_base=n_sample)
        vals.append(n_sample / dt)
        t_all += dt
    value = args.steps * n_sample / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "n_primaries_per_step": n_sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d primaries per step of the same workload, oracle C++ FP64 restatement of "
                                   "src/main.rs:134-289 (the Rust reference cannot be built: no cargo/rustc)" % n_sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------- timing --
class Timer:
    """CUDA events on the engine's stream around each call and around a
    whole run of calls."""

    def __init__(self, stream):
        import torch
        self.torch = torch
        self.stream = stream

    def event(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        return e

    def run(self, fn, seeds):
        """Calls fn(seed) for each seed; returns (total ms, per-call ms,
        per-call results)."""
        torch = self.torch
        torch.cuda.synchronize()
        e_all0 = self.event()
        per, res = [], []
        for s in seeds:
            e0 = self.event()
            r = fn(s)
            e1 = self.event()
            per.append((e0, e1))
            res.append(r)
        e_all1 = self.event()
        e_all1.synchronize()
        torch.cuda.synchronize()
        return e_all0.elapsed_time(e_all1), [a.elapsed_time(b) for a, b in per], res


def roofline_fp64(stats, kern_ms, peak_tflops, kind):
    """The dominant kernel's algorithmic FP64 work per launch (OPS times the
    launch's event counts) over its duration, against the device's measured
    FP64 FMA throughput."""
    lep, pho, emis = stats["lepton_steps"], stats["photon_steps"], stats.get("emissions", 0)
    # free steps: leptons outside the pulse, and drifting photons
    drift = stats.get("drift_steps", 0)
    lfree = stats.get("free_steps", 0) - drift
    if kind == "lma":
        flops = ((lep - lfree) * OPS["lma_lepton_step"] + lfree * OPS["free_lepton_step"] +
                 (pho - drift) * OPS["lma_photon_step"] + drift * OPS["free_photon_step"] +
                 emis * OPS["cp_emission"])
        model = {k: OPS[k] for k in ("lma_lepton_step", "free_lepton_step", "lma_photon_step", "free_photon_step",
                                     "cp_emission")}
    else:
        flops = ((lep - lfree) * OPS["lcfa_lepton_step"] + lfree * OPS["lcfa_free_lepton_step"] +
                 (pho - drift) * OPS["lcfa_photon_step"] + drift * OPS["free_photon_step"] +
                 emis * OPS["lcfa_emission"])
        model = {k: OPS[k] for k in ("lcfa_lepton_step", "lcfa_free_lepton_step", "lcfa_photon_step",
                                     "free_photon_step", "lcfa_emission")}
    achieved = flops / (kern_ms / 1e3) / 1e12
    return {"bound": "fp64", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
            "frac": achieved / peak_tflops, "algorithmic_flops_per_launch": flops, "flops_per_event": model,
            "peak_source": "measured in this run: FP64 FMA throughput kernel (ptg_fp64_peak); MEASURED_PEAKS.json "
                           "has no FP64 figure"}


# ------------------------------------------------------------ cp_shower --
def run_cp_shower(args, eng, stream, sampler, dev):
    """The CP LMA shower (1e7 e- at 16.5 GeV on an a0 = 5 CP focused laser):
    the learned proposal + persistent queue (value) against
    the reference's table sampler through the wave kernels (plain_value),
    with both cross terms, all over the same seeds."""
    import torch
    from ptarmigan_gb300 import abi, equivalence
    desc, make, n_default = WORKLOADS["cp_shower"]
    n = args.n or n_default
    t_host = time.time()
    laser, opts, prim = make(n, 1)
    host_beam_ms = (time.time() - t_host) * 1e3
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    timer = Timer(stream)
    # the same beam generated on the device (ptg_build_beam), timed apart:
    # beam generation is not part of the metric
    from ptarmigan_gb300 import beam as beam_mod
    g = beam_mod.gamma_from_energy(16.5)
    bd = abi.beam_desc(gamma_mean=g, gamma_sigma=0.001 * g, sigma_x=5e-6, sigma_z=24e-6, rms_div=8e-6,
                       initial_z=beam_mod.initial_z(laser, 24e-6))
    eng.build_beam(bd, n, seed=1)
    device_beam_ms, _, _ = timer.run(lambda s: eng.build_beam(bd, n, seed=s), [2])
    t0 = time.time()
    tr = train_network(eng, args)
    tr["wall_s"] = time.time() - t0

    def coll(seed):
        return [{"laser": laser, "seed": seed, "id_base": n, "first": 0, "count": n}]

    def learned_queue(seed):
        eng.mlp_use(True, margin=MLP_MARGIN)
        return eng.collide_multi_device(coll(seed), opts, d_prim)[3]

    def table_queue(seed):
        eng.mlp_use(False)
        return eng.collide_multi_device(coll(seed), opts, d_prim)[3]

    def table_waves(seed):
        eng.mlp_use(False)
        return eng.collide_device(laser, opts, d_prim, seed=seed, id_base=n)[1]

    def learned_waves(seed):
        eng.mlp_use(True, margin=MLP_MARGIN)
        return eng.collide_device(laser, opts, d_prim, seed=seed, id_base=n)[1]

    eng.mlp_use(True, margin=MLP_MARGIN)
    t0 = time.time()
    tune, tune_ms = eng.queue_autotune(coll(100), opts, d_prim, sample_fraction=args.tune_fraction or 0.01)
    tune_wall = time.time() - t0
    seeds = [SEED0 + k for k in range(args.steps)]
    keys = ("lepton_steps", "photon_steps", "free_steps", "emissions", "pair_events", "rejections", "n_created",
            "n_out", "particle_errors", "max_steps")

    def arm(fn, warm):
        for w in range(warm):
            fn(100 + w)
        total, per, res = timer.run(fn, seeds)
        agg = {k: (max(r[k] for r in res) if k == "max_steps" else int(sum(r[k] for r in res))) for k in keys}
        return {"value": n * len(seeds) / (total / 1e3), "ms_total": total, "steps": step_summary(per),
                "events_sum": agg, "device_ms": [r["device_ms"] for r in res], "last": res[-1]}

    with sampler:
        value_arm = arm(learned_queue, args.warmup)
    plain_arm = arm(table_waves, min(args.warmup, 2))
    lw_arm = arm(learned_waves, 1)
    tq_arm = arm(table_queue, 1)

    # end to end through the host API, the value path, the same seeds
    prim_h = pinned_copy(prim)
    eng.mlp_use(True, margin=MLP_MARGIN)
    parts, _, _ = eng.collide_multi(coll(1999), opts, prim_h)  # untimed warm-up
    del parts
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d2h = 0
    out_value_seed0 = None
    for s in seeds:
        parts, _, tot = eng.collide_multi(coll(s), opts, prim_h)
        d2h = nbytes(parts[0])
        if s == SEED0:
            out_value_seed0 = parts[0]
        del parts
    e2e_s = time.perf_counter() - t0
    e2e = n * len(seeds) / e2e_s

    # the plain path's shower for seed 1000, for the spectra
    eng.mlp_use(False)
    out_plain_seed0, _ = eng.collide(laser, opts, prim, seed=SEED0, id_base=n)
    cmp_value_plain = equivalence.compare(out_value_seed0, prim, out_plain_seed0, prim)

    peak = eng.fp64_peak()
    kern_ms = float(np.mean(value_arm["device_ms"]))
    roof = roofline_fp64(value_arm["last"], kern_ms, peak, "lma")
    roof["kernel"] = "collide_queue_single<FOCUSED_LASER> (value path); graph device time per batch"
    roof["traffic"] = None
    pk, pk_kind = peaks()

    line = {
        "metric": METRIC, "value": value_arm["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": value_arm["ms_total"] / len(seeds), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "n_primaries": n, "seeds": [seeds[0], seeds[-1]],
                   "value_path": "learned proposal + persistent single-collision queue kernel (CUDA graph, autotuned)",
                   "plain_path": "reference table sampler + wave kernels",
                   "autotuned": tune, "autotune_sample_ms": tune_ms, "autotune_wall_s": tune_wall,
                   "l2": "inputs (1.2 GB) and shower store larger than L2 (no flush needed)", "margin": MLP_MARGIN},
        "step_ms": value_arm["steps"],
        "particle_errors": value_arm["events_sum"]["particle_errors"],
        "max_steps_per_particle": value_arm["events_sum"]["max_steps"],
        "events_per_step": {k: v for k, v in value_arm["last"].items() if k in keys},
        "plain_value": plain_arm["value"], "plain_step_ms": plain_arm["steps"],
        "plain_particle_errors": plain_arm["events_sum"]["particle_errors"],
        "cross_terms": {
            "learned_waves": {"value": lw_arm["value"], "step_ms": lw_arm["steps"]},
            "table_queue": {"value": tq_arm["value"], "step_ms": tq_arm["steps"]},
        },
        "attribution": {
            "sampler_gain_on_waves": lw_arm["value"] / plain_arm["value"],
            "sampler_gain_on_queue": value_arm["value"] / tq_arm["value"],
            "scheduler_gain_with_table": tq_arm["value"] / plain_arm["value"],
            "scheduler_gain_with_learned": value_arm["value"] / lw_arm["value"],
            "total": value_arm["value"] / plain_arm["value"],
        },
        "ks_photon_energy_vs_plain": cmp_value_plain["ks_photon_energy"],
        "ks_critical_1e-3": cmp_value_plain["ks_photon_energy_critical"],
        "value_vs_plain": {k: cmp_value_plain[k] for k in ("photons", "ks_photon_polar_angle", "chi2_log_energy_200",
                                                          "chi2_dof", "chi2_p", "sigma")},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes(prim), "d2h_bytes_per_step": d2h,
                "steps": len(seeds), "seeds": "same as value"},
        # value path per step: the graph's 7 kernels and 4 that put the primaries in phase order
        "gpu_launches": int(11 * len(seeds)),
        "roofline": roof,
        "peaks": {"source": pk_kind, "hbm_gbs": pk.get("hbm_gbs")},
        "beam_generation_ms": {"device_ptg_build_beam": device_beam_ms, "host_numpy": host_beam_ms},
        "training": tr,
    }
    if not args.no_cpu_baseline:
        line.update(cpu_and_parity(eng, make, laser, opts, args, per_core=2500, out_value=out_value_seed0,
                                   prim_value=prim))
    line["clocks"] = sampler.summary()
    return line


def cpu_and_parity(eng, make, laser, opts, args, per_core, out_value=None, prim_value=None):
    """The oracle on a bounded sample of the workload (the CPU baseline),
    and the GPU's table-sampler path on exactly that batch (same primaries,
    seed and id base): particles matched by stream, and the statistics of
    both; plus, when given, the value path's large output against the
    oracle's sample (independent primaries), since the value path samples
    differently."""
    from ptarmigan_gb300 import equivalence
    threads = cpu_threads()
    n_s = max(64, (args.cpu_sample_per_core or per_core) * threads)
    _l, _o, prim_s = make(n_s, 7)
    ref, rst, dt = oracle_run(laser, opts, prim_s, 7, threads, id_base=n_s)
    eng.mlp_use(False)
    out, st = eng.collide(laser, opts, prim_s, seed=7, id_base=n_s)
    tol = 5e-7 if laser.model in (0, 2) else 1e-8
    par = equivalence.match(out, ref, tol)
    cmp_same = equivalence.compare(out, prim_s, ref, prim_s)
    par.update({"sample": "%d primaries (beam seed 7), collision seed 7: the GPU's table-sampler path and the oracle"
                          % n_s,
                "ks_photon_energy": cmp_same["ks_photon_energy"],
                "ks_photon_polar_angle": cmp_same["ks_photon_polar_angle"],
                "chi2_log_energy_200": cmp_same["chi2_log_energy_200"], "chi2_dof": cmp_same["chi2_dof"],
                "gpu": cmp_same["a"], "oracle": cmp_same["b"],
                "events": {"gpu": {k: st[k] for k in ("lepton_steps", "photon_steps", "emissions", "pair_events")},
                           "oracle": {k: rst[k] for k in ("lepton_steps", "photon_steps", "emissions",
                                                          "pair_events")}}})
    if out_value is None:
        return {"cpu_baseline": {"value": n_s / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": "%d primaries of the same workload (%.1f s), oracle C++ FP64 restatement "
                                           "of the collision loop on %d host threads" % (n_s, dt, threads)},
                "parity": par}
    cmp_val = equivalence.compare(out_value, prim_value, ref, prim_s)
    par["value_path_vs_oracle"] = {
        "what": "the value path's seed-1000 batch against the oracle's sample (independent primaries)",
        "ks_photon_energy": cmp_val["ks_photon_energy"], "ks_critical_1e-3": cmp_val["ks_photon_energy_critical"],
        "ks_photon_polar_angle": cmp_val["ks_photon_polar_angle"],
        "ks_photon_polar_angle_critical": cmp_val["ks_photon_polar_angle_critical"],
        "chi2_log_energy_200": cmp_val["chi2_log_energy_200"], "chi2_dof": cmp_val["chi2_dof"],
        "chi2_p": cmp_val["chi2_p"], "sigma": cmp_val["sigma"], "passes": equivalence.passes(cmp_val)}
    return {"cpu_baseline": {"value": n_s / dt, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d primaries of the same workload (%.1f s), oracle C++ FP64 restatement of the "
                                       "collision loop on %d host threads" % (n_s, dt, threads)},
            "parity": par}


# ---------------------------------------------------------- lcfa_shower --
def run_lcfa_shower(args, eng, stream, sampler, dev, rank, world, dist_on):
    """The focused LCFA shower (1e6 e- at 10 GeV on an a0 = 10 LP focused
    laser) through the wave kernels."""
    import torch
    import torch.distributed as dist
    desc, make, n_default = WORKLOADS["lcfa_shower"]
    n = args.n or n_default
    laser, opts, prim = make(n, 1 + rank)
    id_base = n * world + rank * (1 << 40)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    timer = Timer(stream)
    seeds = [SEED0 + k for k in range(args.steps)]
    keys = ("lepton_steps", "photon_steps", "free_steps", "emissions", "pair_events", "rejections", "n_created",
            "n_out", "particle_errors", "max_steps", "waves")

    def barrier():
        if dist_on:
            dist.barrier()
        torch.cuda.synchronize()

    for w in range(args.warmup):
        eng.collide_device(laser, opts, d_prim, seed=100 + w, id_base=id_base)
    barrier()
    with sampler:
        total, per, res = timer.run(lambda s: eng.collide_device(laser, opts, d_prim, seed=s, id_base=id_base)[1],
                                    seeds)
    barrier()
    if dist_on:
        t = torch.tensor([total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    value = n * world * len(seeds) / (total / 1e3)

    # the same batches through the single-collision queue kernel (one
    # persistent launch per batch, graph replay)
    eng.queue_config(variant=2, blocks_per_sm=0, chunk=1, use_graph=1)
    coll = [{"laser": laser, "seed": 0, "id_base": id_base, "first": 0, "count": n}]

    def queue_batch(s):
        coll[0]["seed"] = s
        return eng.collide_multi_device(coll, opts, d_prim)[3]

    queue_batch(1998)
    barrier()
    q_total, q_per, _ = timer.run(queue_batch, seeds)
    barrier()
    queue_value = n * world * len(seeds) / (q_total / 1e3)
    eng.queue_config(variant=0)

    prim_h = pinned_copy(prim)
    out, _ = eng.collide(laser, opts, prim_h, seed=1999, id_base=id_base)  # untimed warm-up
    del out
    barrier()
    t0 = time.perf_counter()
    d2h = 0
    for s in seeds:
        out, _ = eng.collide(laser, opts, prim_h, seed=s, id_base=id_base)
        d2h = nbytes(out)
        del out
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist_on:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = n * world * len(seeds) / e2e_s

    peak = eng.fp64_peak()
    kern_ms = float(np.mean([r["device_ms"] for r in res]))
    roof = roofline_fp64(res[-1], kern_ms, peak, "lcfa")
    roof["kernel"] = "collide_wave<FAST_FOCUSED_LASER>: the batch's device time"
    # DRAM bytes per primary from ncu over the waves of a 1e6 batch
    roof["traffic"] = 2.5605e9 / 1e6 * n
    pk, pk_kind = peaks()
    roof["hbm_frac"] = (roof["traffic"] / (kern_ms / 1e3) / 1e9) / pk.get("hbm_gbs", 6800.0)
    agg = {k: (max(r[k] for r in res) if k == "max_steps" else int(sum(r[k] for r in res))) for k in keys}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / len(seeds), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "n_primaries_per_gpu": n, "parallelism": "replicas x%d" % world,
                   "seeds": [seeds[0], seeds[-1]], "l2": "inputs and shower store larger than L2 (no flush needed)"},
        "step_ms": step_summary(per),
        "queue_value": queue_value, "queue_step_ms": step_summary(q_per),
        "wave_ms_per_step": [[round(x, 2) for x in r["wave_ms"][:max(1, r["waves"])]] for r in res],
        "particle_errors": agg["particle_errors"], "max_steps_per_particle": agg["max_steps"],
        "events_per_step": {k: res[-1][k] for k in keys},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nbytes(prim), "d2h_bytes_per_step": d2h,
                "steps": len(seeds), "seeds": "same as value"},
        "gpu_launches": int(sum(2 + r["waves"] + 3 * r["ordered_waves"] for r in res)),
        "roofline": roof,
        "peaks": {"source": pk_kind, "hbm_gbs": pk.get("hbm_gbs")},
        "clocks": sampler.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line.update(cpu_and_parity(eng, make, laser, opts, args, per_core=400))
    return line


# ------------------------------------------------------ other workloads --
def run_learned_sampler(args, eng, sampler, line):
    n = args.n or 10_000_000
    tr = train_network(eng, args)
    for w in range(args.warmup):
        eng.sampler_bench(min(n, 1_000_000), seed=500 + w, margin=MLP_MARGIN, want_v=False)
    runs, ks = [], None
    with sampler:
        for k in range(args.steps):
            v0, v1, st = eng.sampler_bench(n, seed=SEED0 + k, margin=MLP_MARGIN, want_v=(k == 0))
            runs.append(st)
            if k == 0:
                ks = ks_distance(v0[v0 > 0], v1[v1 > 0])
    # both methods sample the same points, drawn once by the shared first
    # pass (the harmonic n by the table sampler), which both are charged
    learned_ms = float(np.mean([r["learned_ms"] + r["features_ms"] + r["infer_ms"] for r in runs]))
    plain_ms = float(np.mean([r["plain_ms"] + r["features_ms"] for r in runs]))
    last = runs[-1]
    line.update({
        "metric": "CP photon emissions sampled/s: learned proposal vs table sampler at KS <= 1e-3",
        "unit": "emissions/s", "value": n / (learned_ms / 1e3), "ms_per_step": learned_ms,
        "plain_value": n / (plain_ms / 1e3), "plain_ms": plain_ms,
        "dtype": "f64 spectrum and accept/reject; bf16 weights, f32 accumulation in the network",
        "ks_vs_plain": ks, "ks_critical_1e-3": ks_critical(n, n),
        "acceptance": last["acceptance"], "learned_evals_per_emission": last["learned_evals"],
        "plain_evals_per_emission": last["plain_evals"],
        "envelope_violations": last["fallbacks"], "trial_cap_handovers": last["exhausted"],
        "errors": last["errors_plain"] + last["errors_learned"],
        "ms_split": {"features": last["features_ms"], "inference": last["infer_ms"], "sampling": last["learned_ms"]},
        "training": tr,
        "config": {"workload": "learned_sampler: CP NLC v-sampler, a log-uniform [0.05, 20], eta log-uniform "
                               "[1e-3, 2], n from the CP harmonic table; %d emissions per step; network 6-64-64-64-16 "
                               "SiLU trained on the GPU on %.3g table-sampler draws x %d epochs"
                               % (n, tr["n_samples"], tr["epochs"]),
                   "emissions_per_step": n, "margin": MLP_MARGIN},
        # per step: features, plain sampling, packing and inference, learned sampling
        "gpu_launches": 5 * args.steps})


def run_a0_scan(args, eng, timer, sampler, line, dev):
    import torch
    colls, opts, prim = a0_scan_workload(1, scale=args.scale)
    n = int(sum(c["count"] for c in colls))
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    tune, tune_ms = eng.queue_autotune(colls, opts, d_prim, sample_fraction=args.tune_fraction or 0.02)
    for _ in range(args.warmup):
        eng.collide_multi_device(colls, opts, d_prim)
    with sampler:
        total, per, res = timer.run(lambda s: eng.collide_multi_device(colls, opts, d_prim)[3], range(args.steps))
    stats = res[-1]
    # the same collisions through the single-collision entry point
    plain_ms = 0.0
    for c in colls:
        sub = {k: v[c["first"]:c["first"] + c["count"]] for k, v in d_prim.items()}
        t, _, _ = timer.run(lambda s: eng.collide_device(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"]),
                            [0])
        plain_ms += t
    line.update({"value": n * args.steps / (total / 1e3), "ms_per_step": total / args.steps,
                 "step_ms": step_summary(per),
                 "plain_value": n / (plain_ms / 1e3), "plain_ms": plain_ms,
                 "particle_errors": int(sum(r["particle_errors"] for r in res)),
                 "max_steps_per_particle": int(max(r["max_steps"] for r in res)),
                 "config": {"workload": "a0_scan: 64 collisions, a0 0.5..20 log, beams log-uniform 1e3..1e6 "
                                        "e- x%g, 16.5 GeV, LP focused w0=5 um 25 fs, LMA a0<5 / LCFA a0>=5, "
                                        "pairs on, one persistent queue launch (graph)" % args.scale,
                            "n_primaries": n, "autotuned": tune, "autotune_sample_ms": tune_ms,
                            "events_per_step": {k: stats[k] for k in ("lepton_steps", "photon_steps", "free_steps",
                                                                      "emissions", "pair_events", "n_created",
                                                                      "n_out", "particle_errors")}},
                 # the graph's 7 kernels, plus the phase ordering before
                 # it: one kernel, and three per collision of >= 2048
                 # primaries
                 "gpu_launches": (7 + 1 + 3 * sum(1 for c in colls if c["count"] >= 2048)) * args.steps})


def run_plane_wave(args, eng, timer, sampler, line, dev):
    import torch
    from ptarmigan_gb300 import equivalence
    laser, opts, prim = plane_wave_lma_workload(args.n or 10_000, 1)
    desc = "plane_wave_lma: 1e4 e- 5 GeV 0.1%, LP PlaneWave (LMA) a0=1 cos2 30.9 cycles, emission only"
    n = len(prim["species"])
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    for w in range(args.warmup):
        eng.collide_device(laser, opts, d_prim, seed=100 + w)
    seeds = [SEED0 + k for k in range(args.steps)]
    with sampler:
        total, per, res = timer.run(lambda s: eng.collide_device(laser, opts, d_prim, seed=s)[1], seeds)
    st = res[-1]
    line.update({"value": n * len(seeds) / (total / 1e3), "ms_per_step": total / len(seeds),
                 "step_ms": step_summary(per),
                 "particle_errors": int(sum(r["particle_errors"] for r in res)),
                 "max_steps_per_particle": int(max(r["max_steps"] for r in res)),
                 "config": {"workload": desc, "n_primaries": n,
                            "events_per_step": {k: st[k] for k in ("lepton_steps", "free_steps", "photon_steps",
                                                                   "emissions", "n_out", "waves",
                                                                   "particle_errors")}},
                 "gpu_launches": int(sum(2 + r["waves"] + 3 * r["ordered_waves"] for r in res))})
    if not args.no_cpu_baseline:
        # the oracle on the same 1e4 primaries and seed (well under a second)
        threads = cpu_threads()
        ref, rst, dt = oracle_run(laser, opts, prim, SEED0, threads)
        out, _ = eng.collide(laser, opts, prim, seed=SEED0)
        par = equivalence.match(out, ref, 5e-7)
        cmp_same = equivalence.compare(out, prim, ref, prim)
        par.update({"ks_photon_energy": cmp_same["ks_photon_energy"], "gpu": cmp_same["a"],
                    "oracle": cmp_same["b"]})
        line["cpu_baseline"] = {"value": n / dt, "unit": "primaries/s", "cores": threads, "kind": "port",
                                "sample": "the same %d primaries (%.2f s), oracle C++ FP64 restatement of the "
                                          "collision loop on %d host threads" % (n, dt, threads)}
        line["parity"] = par


def run_profile_case(args, eng, dev):
    """For profilers: one batch of the workload (--n primaries, default
    2e5, seed 1000, the reference's sampler) through the wave kernels, then
    the same batch through the single-collision queue kernel (no graph, so
    its launch is visible): a short, fixed launch sequence.  Prints their
    event counts."""
    import torch
    name = args.workload if args.workload in WORKLOADS else "cp_shower"
    desc, make, _n = WORKLOADS[name]
    n = args.n or 200_000
    laser, opts, prim = make(n, 1)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    eng.mlp_use(False)
    _, st = eng.collide_device(laser, opts, d, seed=SEED0, id_base=n)
    eng.queue_config(variant=2, blocks_per_sm=0, chunk=1, use_graph=0)
    _, _, _, qt = eng.collide_multi_device([{"laser": laser, "seed": SEED0, "id_base": n, "first": 0, "count": n}],
                                           opts, d)
    keys = ("lepton_steps", "photon_steps", "free_steps", "drift_steps", "emissions", "pair_events", "n_out",
            "particle_errors", "device_ms", "wave_ms")
    print(json.dumps({"profile_case": desc, "n_primaries": n, "waves": {k: st[k] for k in keys},
                      "queue": {k: qt[k] for k in keys}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None, help="primaries (emissions for learned_sampler)")
    ap.add_argument("--cpu-sample-per-core", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="cp_shower", choices=["cp_shower", "lcfa_shower", "plane_wave_lma",
                                                                  "a0_scan", "learned_sampler"])
    ap.add_argument("--scale", type=float, default=1.0, help="a0_scan: beam-size scale")
    ap.add_argument("--tune-fraction", type=float, default=None,
                    help="autotuner sample fraction (a0_scan 0.02, cp_shower 0.01)")
    ap.add_argument("--train-samples", type=int, default=0,
                    help="learned_sampler, cp_shower: training samples (default 5e7)")
    ap.add_argument("--train-epochs", type=int, default=0, help="learned_sampler, cp_shower: epochs (default 3)")
    ap.add_argument("--profile-case", action="store_true",
                    help="one wave batch and one queue batch of --workload at --n primaries, for profilers")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    dist_on = world > 1
    if dist_on:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local_rank)
    from ptarmigan_gb300 import build, engine
    build.build()
    eng = engine.Engine(device=local_rank)
    stream = torch.cuda.ExternalStream(eng.stream_ptr, device=local_rank)
    dev = torch.device("cuda", local_rank)
    sampler = ClockSampler(local_rank)
    try:
        if args.profile_case:
            run_profile_case(args, eng, dev)
            return
        if args.workload == "lcfa_shower":
            line = run_lcfa_shower(args, eng, stream, sampler, dev, rank, world, dist_on)
        elif args.workload == "cp_shower":
            # replicas: every rank runs the whole workload on its own GPU
            line = run_cp_shower(args, eng, stream, sampler, dev)
            if dist_on:
                t = torch.tensor([line["ms_per_step"]], device=dev)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                line["ms_per_step"] = float(t.item())
                line["value"] = line["config"]["n_primaries"] * world / (line["ms_per_step"] / 1e3)
                line["n_gpus"] = world
                line["config"]["parallelism"] = "replicas x%d" % world
        else:
            line = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic"}
            timer = Timer(stream)
            if args.workload == "learned_sampler":
                run_learned_sampler(args, eng, sampler, line)
            elif args.workload == "a0_scan":
                run_a0_scan(args, eng, timer, sampler, line, dev)
            else:
                run_plane_wave(args, eng, timer, sampler, line, dev)
            line["clocks"] = sampler.summary()
        if rank == 0:
            print(json.dumps(line), flush=True)
    finally:
        eng.close()
        if dist_on:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
