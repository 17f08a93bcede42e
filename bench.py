"""Benchmark of the collision loop: collided primaries/s (showers included).

Workload (one "step" = one batch through the collision loop): the focused
LCFA shower — 1e6 electrons at 10 GeV, 1% rms energy spread, 2 x 2 x 20 um
rms, 50 urad divergence, head-on with a linearly polarised focused Gaussian
laser (FastFocusedLaser) a0 = 10, w0 = 4 um, 0.8 um, 30 fs FWHM; LCFA
emission and pair creation on, secondaries tracked to generation 2; FP64
push.  Inputs are seeded synthetic beams with those distributions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` times ptg_collide_batch_device with the
primaries resident in HBM; `e2e` times ptg_collide_batch (host buffers in
and out, host<->device copies inside the timed region).  --impl reference
times the CPU restatement of the reference's collision loop (the reference
is Rust and no Rust toolchain is available) on all host cores.

Other workloads (--workload), each one JSON line of the same metric:
  plane_wave_lma  1e4 electrons at 5 GeV, 0.1% spread, 1 x 1 x 10 um, on a
                  linearly polarised plane wave (LMA), a0 = 1, 0.8 um, cos^2
                  envelope of 30 fs intensity FWHM (30.9 cycles), emission
                  only.
  a0_scan         64 collisions in one persistent queue launch: a0
                  log-spaced 0.5..20, beams log-uniform 1e3..1e6 electrons
                  (seeded) at 16.5 GeV, 0.1% spread, 2 x 2 x 20 um, 8 urad, on
                  a circularly polarised focused Gaussian laser, w0 = 5 um,
                  0.8 um, 25 fs; LMA below a0 = 5, LCFA above; pairs on.
                  `plain_value` runs the same collisions one call each.
  cp_shower       electrons at 16.5 GeV, 0.1% spread, 5 x 5 x 24 um, 8 urad,
                  on a circularly polarised focused laser (LMA) a0 = 5, w0 =
                  3 um, 0.8 um, 30 fs; Stokes parameters tracked, pairs on,
                  all generations (--n primaries, default 1e6).  `value` is
                  the learned proposal inside the persistent queue kernel,
                  `plain_value` the reference's sampler through the wave
                  kernels, with the photon spectra of both compared by KS.
  learned_sampler the CP photon-energy sampler alone: the network is trained
                  on the GPU on 5e7 table-sampler draws (a log-uniform in
                  [0.05, 20], eta log-uniform in [1e-3, 2]), then each step
                  samples 1e7 emissions of the same (a, eta) distribution
                  with the learned proposal (`value`, inputs and inference
                  included) and with the reference's sampler
                  (`plain_value`); acceptance rate and the KS distance
                  between the two are reported.
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

METRIC = "collided primaries/s incl. showers"
UNIT = "primaries/s"
N_PRIMARIES = 1_000_000
WORKLOAD = "focused LCFA shower: 1e6 e- 10 GeV 1% spread, 2x2x20 um, 50 urad; FastFocusedLaser a0=10 w0=4 um 0.8 um 30 fs LP; pairs on; generations<=2"


# FP64 operations per step of collide_wave on this workload (2 x DFMA + DMUL
# + DADD from ncu's SASS instruction counts over a 1e4-primary batch,
# divided by that batch's step counts) and DRAM bytes per primary
# (dram__bytes_read.sum + dram__bytes_write.sum over the lepton and photon
# waves of a 1e6-primary batch: 1.460e9 + 1.100e9 bytes; the pair waves add
# nothing measurable).
FP64_PER_LEPTON_STEP = 213.8
FP64_PER_PHOTON_STEP = 29.2
DRAM_BYTES_PER_PRIMARY = 2.5605e9 / 1e6


def workload(n, seed):
    from ptarmigan_gb300 import abi, beam
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(n, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=seed)
    opts = abi.collide_options(max_generation=2)
    return laser, opts, prim


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


def fp64_peak_tflops(dev):
    """Measured FP64 peak: cuBLAS DGEMM 8192^3 (2 N^3 flops), best of 5."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_run(n_sample, seed, threads):
    """The oracle (CPU restatement of the reference) on a sample."""
    from oracle import oracle
    oracle.build()
    laser, opts, prim = workload(n_sample, seed)
    t0 = time.perf_counter()
    _, st = oracle.collide(laser, opts, prim, seed=seed, threads=threads)
    dt = time.perf_counter() - t0
    return n_sample / dt, st, dt


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = cpu_threads()
    n_sample = max(64, args.cpu_sample_per_core * threads)
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_run(min(n_sample, 16 * threads), 99, threads)
    vals = []
    t_all = 0.0
    for k in range(args.steps):
        v, st, dt = cpu_run(n_sample, 1000 + k, threads)
        vals.append(v)
        t_all += dt
    value = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_primaries_per_step": n_sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d primaries per step of the same workload, oracle C++ FP64 restatement of "
                                   "src/main.rs:134-289 (the Rust reference cannot be built: no cargo/rustc)" % n_sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
        laser = abi.laser_desc(model, float(a0), 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=5e-6, fwhm_duration=25e-15)
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


def cp_shower_workload(n, seed):
    from ptarmigan_gb300 import abi, beam
    laser = abi.laser_desc(abi.FOCUSED_LASER, 5.0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6, fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(n, g, sigma=0.001 * g, radius=5e-6, length=24e-6, rms_div=8e-6, laser=laser, seed=seed)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    return laser, opts, prim


MLP_MARGIN = 0.25  # ln of the learned envelope's safety factor
MLP_TRAIN = dict(n_samples=50_000_000, batch=16384, epochs=3, lr=2e-3, tau=0.98, seed=7)


def ks_distance(a, b):
    """Two-sample Kolmogorov-Smirnov statistic."""
    a, b = np.sort(np.asarray(a)), np.sort(np.asarray(b))
    grid = np.concatenate([a, b])
    return float(np.max(np.abs(np.searchsorted(a, grid, side="right") / len(a) -
                               np.searchsorted(b, grid, side="right") / len(b))))


def ks_critical(n, m, alpha=1e-3):
    """Two-sample KS critical value at significance alpha."""
    c = math.sqrt(-0.5 * math.log(alpha / 2.0))
    return c * math.sqrt((n + m) / (n * m))


def train_network(eng, args=None):
    cfg = dict(MLP_TRAIN)
    if args is not None and args.train_samples:
        cfg["n_samples"] = args.train_samples
    if args is not None and args.train_epochs:
        cfg["epochs"] = args.train_epochs
    eng.mlp_init(3)
    return dict(eng.mlp_train(**cfg), **cfg)


def run_learned_sampler(args, eng, sampler, line):
    n = args.n or 10_000_000
    tr = train_network(eng, args)
    for w in range(args.warmup):
        eng.sampler_bench(min(n, 1_000_000), seed=500 + w, margin=MLP_MARGIN, want_v=False)
    runs, ks = [], None
    with sampler:
        for k in range(args.steps):
            v0, v1, st = eng.sampler_bench(n, seed=1000 + k, margin=MLP_MARGIN, want_v=(k == 0))
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


def run_extra(args):
    """The non-default workloads: device time with CUDA events on the
    engine's stream, inputs resident in HBM."""
    import torch
    from ptarmigan_gb300 import build, engine
    build.build()
    eng = engine.Engine(device=0)
    stream = torch.cuda.ExternalStream(eng.stream_ptr, device=0)
    dev = torch.device("cuda", 0)
    sampler = ClockSampler(0)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
        r = fn()
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), r

    line = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic"}
    if args.workload == "learned_sampler":
        run_learned_sampler(args, eng, sampler, line)
    elif args.workload == "a0_scan":
        colls, opts, prim = a0_scan_workload(1, scale=args.scale)
        n = int(sum(c["count"] for c in colls))
        d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
        tune, tune_ms = eng.queue_autotune(colls, opts, d_prim, sample_fraction=args.tune_fraction or 0.02)
        for _ in range(args.warmup):
            eng.collide_multi_device(colls, opts, d_prim)
        ms, stats = [], None
        with sampler:
            for _ in range(args.steps):
                t, r = timed(lambda: eng.collide_multi_device(colls, opts, d_prim))
                ms.append(t)
                stats = r[3]
        # the same collisions through the single-collision entry point
        plain_ms = 0.0
        for c in colls:
            sub = {k: v[c["first"]:c["first"] + c["count"]] for k, v in d_prim.items()}
            t, _ = timed(lambda: eng.collide_device(c["laser"], opts, sub, seed=c["seed"], id_base=c["id_base"]))
            plain_ms += t
        line.update({"value": n / (np.mean(ms) / 1e3), "ms_per_step": float(np.mean(ms)),
                     "plain_value": n / (plain_ms / 1e3), "plain_ms": plain_ms,
                     "config": {"workload": "a0_scan: 64 collisions, a0 0.5..20 log, beams log-uniform 1e3..1e6 "
                                            "e- x%g, 16.5 GeV, CP focused w0=5 um 25 fs, LMA a0<5 / LCFA a0>=5, "
                                            "pairs on, one persistent queue launch (graph)" % args.scale,
                                "n_primaries": n, "autotuned": tune, "autotune_sample_ms": tune_ms,
                                "events_per_step": {k: stats[k] for k in ("lepton_steps", "photon_steps",
                                                                          "emissions", "pair_events", "n_created",
                                                                          "n_out", "particle_errors")}},
                     # the graph's 7 kernels, plus the phase ordering before
                     # it: one kernel, and three per collision of >= 2048
                     # primaries
                     "gpu_launches": (7 + 1 + 3 * sum(1 for c in colls if c["count"] >= 2048)) * args.steps})
    elif args.workload == "plane_wave_lma":
        laser, opts, prim = plane_wave_lma_workload(args.n or 10_000, 1)
        desc = "plane_wave_lma: 1e4 e- 5 GeV 0.1%, LP PlaneWave (LMA) a0=1 cos2 30.9 cycles, emission only"
        n = len(prim["species"])
        d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
        for w in range(args.warmup):
            eng.collide_device(laser, opts, d_prim, seed=100 + w)
        ms, st = [], None
        with sampler:
            for k in range(args.steps):
                t, r = timed(lambda: eng.collide_device(laser, opts, d_prim, seed=1000 + k))
                ms.append(t)
                st = r[1]
        line.update({"value": n / (np.mean(ms) / 1e3), "ms_per_step": float(np.mean(ms)),
                     "config": {"workload": desc, "n_primaries": n,
                                "events_per_step": {k: st[k] for k in ("lepton_steps", "photon_steps", "emissions",
                                                                       "n_out", "waves", "particle_errors")}},
                     "gpu_launches": int((2 + st["waves"] + 3 * st["ordered_waves"]) * args.steps)})
        if not args.no_cpu_baseline:
            # the oracle on the same 1e4 primaries (well under a second)
            from oracle import oracle
            oracle.build()
            threads = cpu_threads()
            t0 = time.perf_counter()
            oracle.collide(laser, opts, prim, seed=1000, threads=threads)
            dt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": n / dt, "unit": "primaries/s", "cores": threads, "kind": "port",
                                    "sample": "the same %d primaries (%.2f s), oracle C++ FP64 restatement of the "
                                              "collision loop on %d host threads" % (n, dt, threads)}
    else:
        run_cp_shower(args, eng, timed, sampler, line, dev)
    line["clocks"] = sampler.summary()
    print(json.dumps(line), flush=True)
    eng.close()


def run_cp_shower(args, eng, timed, sampler, line, dev):
    """The CP LMA shower: the learned proposal inside the persistent queue
    kernel (value) against the reference's sampler through the wave kernels
    (plain_value), same primaries and seeds; the photon spectra, Stokes
    parameters and pair yields of the two are compared."""
    import torch
    from ptarmigan_gb300 import abi
    t_host = time.time()
    laser, opts, prim = cp_shower_workload(args.n or 1_000_000, 1)
    host_beam_ms = (time.time() - t_host) * 1e3
    desc = ("cp_shower: e- 16.5 GeV 0.1%, 5x5x24 um, 8 urad; CP FocusedLaser (LMA) a0=5 w0=3 um 30 fs; "
            "Stokes tracked, pairs on, all generations")
    n = len(prim["species"])
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    # the same beam generated on the device (ptg_build_beam), timed apart:
    # beam generation is not part of the metric
    from ptarmigan_gb300 import beam as beam_mod
    g = beam_mod.gamma_from_energy(16.5)
    bd = abi.beam_desc(gamma_mean=g, gamma_sigma=0.001 * g, sigma_x=5e-6, sigma_z=24e-6, rms_div=8e-6,
                       initial_z=beam_mod.initial_z(laser, 24e-6))
    eng.build_beam(bd, n, seed=1)
    device_beam_ms, _ = timed(lambda: eng.build_beam(bd, n, seed=2))
    tr = train_network(eng, args)

    def plain(seed):
        eng.mlp_use(False)
        return eng.collide_device(laser, opts, d_prim, seed=seed)

    def learned(seed):
        eng.mlp_use(True, margin=MLP_MARGIN)
        return eng.collide_multi_device([{"laser": laser, "seed": seed, "id_base": n, "first": 0, "count": n}],
                                        opts, d_prim)

    coll = [{"laser": laser, "seed": 100, "id_base": n, "first": 0, "count": n}]
    eng.mlp_use(True, margin=MLP_MARGIN)
    tune, tune_ms = eng.queue_autotune(coll, opts, d_prim, sample_fraction=args.tune_fraction or 0.1)
    for w in range(args.warmup):
        plain(100 + w)
        learned(100 + w)
    ms_l, ms_p, st_l, st_p = [], [], None, None
    with sampler:
        for k in range(args.steps):
            t, r = timed(lambda: learned(1000 + k))
            ms_l.append(t)
            st_l = r[3]
            t, r = timed(lambda: plain(1000 + k))
            ms_p.append(t)
            st_p = r[1]
    # statistics of one step of each, through the host entry points (same seeds)
    eng.mlp_use(False)
    out_p, _ = eng.collide(laser, opts, prim, seed=1000)
    eng.mlp_use(True, margin=MLP_MARGIN)
    parts, _, _ = eng.collide_multi([{"laser": laser, "seed": 1000, "id_base": n, "first": 0, "count": n}],
                                    opts, prim)
    out_l = parts[0]
    eng.mlp_use(False)

    def summary(out):
        ph = out["species"] == abi.PHOTON
        return {"photons": int(ph.sum()), "positrons": int((out["species"] == abi.POSITRON).sum()),
                "stokes_mean": [float(x) for x in out["pol"][ph].mean(axis=0)],
                "mean_electron_energy_mev": float(out["u"][out["species"] == abi.ELECTRON, 0].mean() * 0.51099895)}
    e_p = out_p["u"][out_p["species"] == abi.PHOTON, 0]
    e_l = out_l["u"][out_l["species"] == abi.PHOTON, 0]
    keys = ("lepton_steps", "photon_steps", "emissions", "pair_events", "n_created", "n_out", "particle_errors")
    line.update({"value": n / (np.mean(ms_l) / 1e3), "ms_per_step": float(np.mean(ms_l)),
                 "plain_value": n / (np.mean(ms_p) / 1e3), "plain_ms": float(np.mean(ms_p)),
                 "ms_each_step": {"value_path": [float(x) for x in ms_l], "plain_path": [float(x) for x in ms_p]},
                 "ks_photon_energy_vs_plain": ks_distance(e_p, e_l),
                 "ks_critical_1e-3": ks_critical(len(e_p), len(e_l)),
                 "learned": summary(out_l), "plain": summary(out_p),
                 "beam_generation_ms": {"device_ptg_build_beam": device_beam_ms, "host_numpy": host_beam_ms},
                 "training": tr,
                 "config": {"workload": desc, "n_primaries": n, "margin": MLP_MARGIN,
                            "value_path": "learned proposal + persistent queue kernel (CUDA graph, autotuned)",
                            "autotuned": tune, "autotune_sample_ms": tune_ms,
                            "plain_path": "reference sampler + wave kernels",
                            "events_per_step_learned": {k: st_l[k] for k in keys},
                            "events_per_step_plain": {k: st_p[k] for k in keys}},
                 # value path: the graph's 7 kernels and 4 to order the primaries;
                 # plain path: loading, waves (+3 each when phase-ordered), compaction
                 "gpu_launches": int((7 + 4 + 2 + st_p["waves"] + 3 * st_p["ordered_waves"]) * args.steps)})


def nbytes(d):
    return int(sum(v.nbytes for v in d.values()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=None, help="primaries (emissions for learned_sampler)")
    ap.add_argument("--cpu-sample-per-core", type=int, default=1500)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="lcfa_shower", choices=["lcfa_shower", "plane_wave_lma", "a0_scan",
                                                                    "cp_shower", "learned_sampler"])
    ap.add_argument("--scale", type=float, default=1.0, help="a0_scan: beam-size scale")
    ap.add_argument("--tune-fraction", type=float, default=None,
                    help="autotuner sample fraction (a0_scan 0.02, cp_shower 0.1)")
    ap.add_argument("--train-samples", type=int, default=0,
                    help="learned_sampler, cp_shower: training samples (default 5e7)")
    ap.add_argument("--train-epochs", type=int, default=0, help="learned_sampler, cp_shower: epochs (default 3)")
    args = ap.parse_args()
    if args.workload != "lcfa_shower" and args.impl == "gb300":
        args.n = args.n or 0
        run_extra(args)
        return
    if args.n is None:
        args.n = N_PRIMARIES

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

    from ptarmigan_gb300 import abi, build, engine
    build.build()
    eng = engine.Engine(device=local_rank)
    stream = torch.cuda.ExternalStream(eng.stream_ptr, device=local_rank)

    # weak scaling: every rank collides its own, disjoint set of primaries
    laser, opts, prim = workload(args.n, seed=1 + rank)
    id_base = args.n * world + rank * (1 << 40)
    dev = torch.device("cuda", local_rank)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    torch.cuda.synchronize()

    def barrier():
        if dist_on:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up (also sizes the shower store)
    for w in range(args.warmup):
        _, st = eng.collide_device(laser, opts, d_prim, seed=100 + w, id_base=id_base)

    # device-resident timing: CUDA events on the engine's stream
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    stats = []
    kern_ms = []
    sampler = ClockSampler(local_rank)
    barrier()
    with sampler:
        with torch.cuda.stream(stream):
            ev0.record(stream)
        for k in range(args.steps):
            _, st = eng.collide_device(laser, opts, d_prim, seed=1000 + k, id_base=id_base)
            stats.append(st)
            kern_ms.append(st["device_ms"])
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
    barrier()
    t_ms = ev0.elapsed_time(ev1)
    if dist_on:
        t = torch.tensor([t_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
    value = args.n * world * args.steps / (t_ms / 1e3)

    # end-to-end through the host API: H2D of the primaries and D2H of the
    # shower inside the timed region
    h2d = nbytes(prim)
    # the primaries in page-locked host memory, as a caller streaming
    # batches to the device would hold them
    prim_h = {}
    for key, v in prim.items():
        buf = torch.empty(max(1, v.nbytes), dtype=torch.uint8, pin_memory=True).numpy()
        a = buf[:v.nbytes].view(v.dtype).reshape(v.shape)
        a[...] = v
        prim_h[key] = a
    out, _ = eng.collide(laser, opts, prim_h, seed=1999, id_base=id_base)  # untimed warm-up
    del out
    barrier()
    t0 = time.perf_counter()
    d2h = 0
    for k in range(max(1, min(args.steps, 2))):
        out, st_e = eng.collide(laser, opts, prim_h, seed=2000 + k, id_base=id_base)
        d2h = nbytes(out)
        del out
    e2e_steps = max(1, min(args.steps, 2))
    barrier()
    e2e_s = time.perf_counter() - t0
    if dist_on:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = args.n * world * e2e_steps / e2e_s

    # roofline of the dominant kernel (collide_wave, FP64-pipe bound): FP64
    # operations per charged and per photon step, counted by ncu on a 1e4
    # primary batch of this workload (profiles/collide_wave_fp64_counts_n1e4.md),
    # times this run's step counts, over the waves' device time; peak = the
    # device's measured FP64 FMA throughput (ptg_fp64_peak).
    pk, pk_kind = peaks()
    st0 = stats[-1]
    flops = st0["lepton_steps"] * FP64_PER_LEPTON_STEP + st0["photon_steps"] * FP64_PER_PHOTON_STEP
    kern_s = float(np.mean(kern_ms)) / 1e3
    achieved = flops / kern_s / 1e12
    peak = eng.fp64_peak()
    traffic = DRAM_BYTES_PER_PRIMARY * args.n
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "traffic": traffic,
                "peak_source": "measured in this run: FP64 FMA throughput kernel (ptg_fp64_peak); "
                               "MEASURED_PEAKS.json has no FP64 figure",
                "fp64_flops_per_step": {"lepton": FP64_PER_LEPTON_STEP, "photon": FP64_PER_PHOTON_STEP},
                "hbm_frac": (traffic / kern_s / 1e9) / pk.get("hbm_gbs", 6800.0)}

    # per batch: loading, each wave (and the three kernels that put it in
    # phase order), compaction
    launches = int(sum(2 + s["waves"] + 3 * s["ordered_waves"] for s in stats))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n_primaries_per_gpu": args.n, "parallelism": "replicas x%d" % world,
                   "l2": "inputs and shower store larger than L2 (no flush needed)",
                   "events_per_step": {k: stats[-1][k] for k in ("lepton_steps", "photon_steps", "emissions",
                                                                 "pair_events", "n_created", "n_out", "waves")}},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": sampler.summary(),
        "roofline": roofline,
        "peaks": {"source": pk_kind, "hbm_gbs": pk.get("hbm_gbs")},
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        n_sample = max(64, args.cpu_sample_per_core * threads)
        v, st_c, dt = cpu_run(n_sample, 7, threads)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d primaries of the same workload (%.1f s), oracle C++ FP64 restatement "
                                          "of the collision loop on %d host threads" % (n_sample, dt, threads)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist_on:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
