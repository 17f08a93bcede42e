"""Python binding of the C ABI (``include/ptarmigan_gb300.h``).

``Engine`` owns one device context.  ``collide()`` is the reference's
collision loop over a batch (src/main.rs:1118-1135 mapping ``collide`` over
the primaries): host arrays in, the surviving shower particles out.  There
is no CPU path: if the library is not built or no GPU is visible the
constructor raises.
"""

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import MLP_INPUTS
from .build import LIB_PATH

_lib = None

_EXPORTS = [
    "ptg_abi_version", "ptg_status_string", "ptg_last_error", "ptg_context_create", "ptg_context_destroy",
    "ptg_load_tables", "ptg_collide_batch", "ptg_collide_batch_device", "ptg_particles_free",
    "ptg_laser_timestep", "ptg_laser_initial_z", "ptg_context_stream", "ptg_context_set_limits", "ptg_pair_rate_increase", "ptg_eval_fields", "ptg_push_steps",
    "ptg_lcfa_photon_rate", "ptg_lcfa_photon_sample", "ptg_lcfa_pair_t", "ptg_double_bessel", "ptg_lp_sample", "ptg_lp_sample_warp", "ptg_cp_sample", "ptg_cp_sample_warp",
    "ptg_cp_sample_learned",
    "ptg_collide_multi", "ptg_collide_multi_device", "ptg_queue_config", "ptg_queue_autotune", "ptg_fp64_peak",
    "ptg_fp64_function_kernel", "ptg_emission_rate_bound",
    "ptg_mlp_init", "ptg_mlp_params", "ptg_mlp_train", "ptg_mlp_grad", "ptg_mlp_infer", "ptg_mlp_use",
    "ptg_mlp_min_harmonic",
    "ptg_sampler_bench", "ptg_build_beam", "ptg_histogram", "ptg_particle_sums",
]


def _hgram_info(info):
    d = info.dim
    return {"dim": d, "empty": bool(info.empty), "bins": [int(info.bins[k]) for k in range(d)],
            "min": [info.min[k] for k in range(d)], "max": [info.max[k] for k in range(d)],
            "bin_size": [info.bin_size[k] for k in range(d)], "bin_volume": info.bin_volume, "total": info.total,
            "unweighted_total": info.unweighted_total, "n_counts": int(info.n_counts)}


class PtgError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d): %s" % (load().ptg_status_string(status).decode(), status, message))
        self.status = status


def load(path=None):
    """Loads the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("ptarmigan_gb300 library not built (%s); run ptarmigan_gb300.build.build()" % path)
    L = C.CDLL(path)
    DP = C.POINTER(C.c_double)
    st = C.c_int
    ctxp = C.c_void_p
    L.ptg_abi_version.restype = C.c_int
    L.ptg_status_string.restype = C.c_char_p
    L.ptg_status_string.argtypes = [C.c_int]
    L.ptg_last_error.restype = C.c_char_p
    L.ptg_context_create.restype = st
    L.ptg_context_create.argtypes = [C.POINTER(abi.DeviceCfg), C.POINTER(C.c_void_p)]
    L.ptg_context_destroy.restype = st
    L.ptg_context_destroy.argtypes = [ctxp]
    L.ptg_load_tables.restype = st
    L.ptg_load_tables.argtypes = [ctxp, C.c_char_p]
    for name in ("ptg_collide_batch", "ptg_collide_batch_device"):
        f = getattr(L, name)
        f.restype = st
        f.argtypes = [ctxp, C.POINTER(abi.LaserDesc), C.POINTER(abi.CollideOptions), C.POINTER(abi.Particles),
                      C.c_uint64, C.c_uint64, C.POINTER(abi.Particles), C.POINTER(abi.RunStats)]
    L.ptg_particles_free.restype = None
    L.ptg_particles_free.argtypes = [C.POINTER(abi.Particles)]
    L.ptg_laser_timestep.restype = st
    L.ptg_laser_timestep.argtypes = [C.POINTER(abi.LaserDesc), DP]
    L.ptg_laser_initial_z.restype = st
    L.ptg_laser_initial_z.argtypes = [C.POINTER(abi.LaserDesc), DP]
    L.ptg_context_stream.restype = C.c_void_p
    L.ptg_context_stream.argtypes = [ctxp]
    L.ptg_pair_rate_increase.restype = st
    L.ptg_pair_rate_increase.argtypes = [ctxp, C.POINTER(abi.LaserDesc), C.c_double, C.POINTER(C.c_double)]
    L.ptg_context_set_limits.restype = st
    L.ptg_context_set_limits.argtypes = [ctxp, C.POINTER(abi.Limits), C.POINTER(abi.Limits)]
    L.ptg_eval_fields.restype = st
    L.ptg_eval_fields.argtypes = [ctxp, C.POINTER(abi.LaserDesc), C.c_size_t, DP, DP, DP, DP]
    L.ptg_push_steps.restype = st
    L.ptg_push_steps.argtypes = [ctxp, C.POINTER(abi.LaserDesc), C.c_size_t, DP, DP, C.c_double, C.c_double,
                                 C.c_int32, C.c_int32, DP]
    L.ptg_lcfa_photon_rate.restype = st
    L.ptg_lcfa_photon_rate.argtypes = [ctxp, C.c_size_t, DP, DP, DP]
    L.ptg_lcfa_photon_sample.restype = st
    L.ptg_lcfa_photon_sample.argtypes = [ctxp, C.c_size_t, DP, DP, DP, DP, DP]
    L.ptg_lcfa_pair_t.restype = st
    L.ptg_lcfa_pair_t.argtypes = [ctxp, C.c_size_t, DP, DP, DP]
    L.ptg_double_bessel.restype = st
    L.ptg_double_bessel.argtypes = [ctxp, C.c_int32, C.c_size_t, DP, DP, C.c_int32, DP]
    for name in ("ptg_lp_sample", "ptg_lp_sample_warp", "ptg_cp_sample", "ptg_cp_sample_warp"):
        getattr(L, name).restype = st
        getattr(L, name).argtypes = [ctxp, C.c_size_t, DP, DP, C.c_uint64, C.POINTER(C.c_uint64), C.c_uint32, DP,
                                     C.POINTER(C.c_int32)]
    L.ptg_cp_sample_learned.restype = st
    L.ptg_cp_sample_learned.argtypes = [ctxp, C.c_size_t, DP, DP, C.c_uint64, C.POINTER(C.c_uint64), C.c_uint32,
                                        C.c_int32, DP, C.POINTER(C.c_int32)]
    U64P = C.POINTER(C.c_uint64)
    L.ptg_collide_multi.restype = st
    L.ptg_collide_multi.argtypes = [ctxp, C.c_size_t, C.POINTER(abi.Collision), C.POINTER(abi.CollideOptions),
                                    C.POINTER(abi.Particles), C.POINTER(abi.Particles), U64P,
                                    C.POINTER(abi.RunStats), C.POINTER(abi.RunStats)]
    L.ptg_collide_multi_device.restype = st
    L.ptg_collide_multi_device.argtypes = L.ptg_collide_multi.argtypes
    L.ptg_queue_config.restype = st
    L.ptg_queue_config.argtypes = [ctxp, C.POINTER(abi.QueueCfg), C.POINTER(abi.QueueCfg)]
    L.ptg_queue_autotune.restype = st
    L.ptg_queue_autotune.argtypes = [ctxp, C.c_size_t, C.POINTER(abi.Collision), C.POINTER(abi.CollideOptions),
                                     C.POINTER(abi.Particles), C.c_double, C.POINTER(abi.QueueCfg), DP]
    L.ptg_fp64_peak.restype = st
    L.ptg_fp64_peak.argtypes = [ctxp, DP]
    L.ptg_emission_rate_bound.restype = st
    L.ptg_emission_rate_bound.argtypes = [ctxp, C.c_size_t, C.c_int32, DP, DP, DP]
    L.ptg_fp64_function_kernel.restype = st
    L.ptg_fp64_function_kernel.argtypes = [ctxp, C.c_int32, C.c_int32]
    FP = C.POINTER(C.c_float)
    L.ptg_mlp_init.restype = st
    L.ptg_mlp_init.argtypes = [ctxp, C.c_uint64]
    L.ptg_mlp_params.restype = st
    L.ptg_mlp_params.argtypes = [ctxp, FP, FP, C.POINTER(C.c_int32)]
    L.ptg_mlp_train.restype = st
    L.ptg_mlp_train.argtypes = [ctxp, C.POINTER(abi.MlpTrainCfg), C.POINTER(abi.MlpTrainStats)]
    L.ptg_mlp_grad.restype = st
    L.ptg_mlp_grad.argtypes = [ctxp, FP, C.c_size_t, C.c_float, FP, FP]
    L.ptg_mlp_infer.restype = st
    L.ptg_mlp_infer.argtypes = [ctxp, FP, C.c_size_t, FP]
    L.ptg_mlp_use.restype = st
    L.ptg_mlp_use.argtypes = [ctxp, C.c_int32, C.c_float]
    L.ptg_mlp_min_harmonic.restype = st
    L.ptg_mlp_min_harmonic.argtypes = [ctxp, C.c_int32, C.POINTER(C.c_int32)]
    L.ptg_particle_sums.restype = st
    L.ptg_particle_sums.argtypes = [ctxp, C.POINTER(abi.Particles), C.POINTER(abi.StatsSpec),
                                    C.POINTER(abi.StatsSums)]
    L.ptg_histogram.restype = st
    L.ptg_histogram.argtypes = [ctxp, C.POINTER(abi.Particles), C.POINTER(abi.HgramSpec), C.POINTER(abi.HgramInfo),
                                DP, C.c_uint64]
    L.ptg_build_beam.restype = st
    L.ptg_build_beam.argtypes = [ctxp, C.POINTER(abi.BeamDesc), C.c_uint64, C.c_uint64, C.c_uint64,
                                 C.POINTER(abi.Particles)]
    L.ptg_sampler_bench.restype = st
    L.ptg_sampler_bench.argtypes = [ctxp, C.POINTER(abi.SamplerBenchCfg), DP, DP, C.POINTER(abi.SamplerBenchDetail),
                                     C.POINTER(abi.SamplerBenchStats)]
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a, shape):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(shape))


class _HostOutput:
    """Owns a library-allocated output (ptg_particles); released with
    ptg_particles_free when the last array viewing it is gone."""

    def __init__(self, lib, out):
        self.lib, self.out = lib, out

    def __del__(self):
        try:
            self.lib.ptg_particles_free(C.byref(self.out))
        except Exception:  # interpreter shutdown
            pass


def _host_arrays(lib, out):
    """numpy views of a library output's host arrays (no copy); the block
    goes back to the library when every view has been dropped."""
    owner = _HostOutput(lib, out)
    n = out.n
    arrays = {}
    ctype_of = {np.float64: C.c_double, np.int32: C.c_int32, np.uint64: C.c_uint64}
    for name, dt, cols in abi.PARTICLE_FIELDS:
        shape = (n, cols) if cols > 1 else (n,)
        if n == 0:
            arrays[name] = np.zeros(shape, dtype=dt)
            continue
        addr = C.cast(getattr(out, name), C.c_void_p).value
        buf = (ctype_of[dt] * (n * cols)).from_address(addr)
        buf._owner = owner
        arrays[name] = np.frombuffer(buf, dtype=dt).reshape(shape)
    return arrays


class Engine:
    """One device context (stream, shower store, tables)."""

    def __init__(self, device=0, block_size=0, blocks_per_sm=0, initial_capacity=0):
        L = load()
        cfg = abi.DeviceCfg(device, block_size, blocks_per_sm, 0, initial_capacity)
        h = C.c_void_p()
        self._check(L.ptg_context_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.device = device
        self.L = L

    def _check(self, status):
        if status != abi.PTG_OK:
            raise PtgError(status, load().ptg_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            self.L.ptg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream_ptr(self):
        return self.L.ptg_context_stream(self._h)

    def set_limits(self, queue_wait_ns=0, step_cap=0, rejection_cap=0):
        """Bounds on any one queue wait, a particle's steps and a rejection
        loop's iterations (0 = the library's default); returns them."""
        new = abi.Limits(queue_wait_ns, step_cap, rejection_cap, 0)
        cur = abi.Limits()
        self._check(self.L.ptg_context_set_limits(self._h, C.byref(new), C.byref(cur)))
        return cur.as_dict()

    def pair_rate_increase(self, laser, gamma):
        """control:increase_pair_rate_by: auto for a beam of Lorentz factor
        gamma (main.rs:294-319)."""
        out = C.c_double()
        self._check(self.L.ptg_pair_rate_increase(self._h, C.byref(laser), gamma, C.byref(out)))
        return out.value

    def load_tables(self, directory=None):
        self._check(self.L.ptg_load_tables(self._h, directory.encode() if directory else None))

    # -- the collision loop ----------------------------------------------
    def collide(self, laser, options, primaries, seed, id_base=None):
        """Runs collide() over every primary (dict of numpy arrays with the
        abi.PARTICLE_FIELDS names).  Returns (arrays, stats dict)."""
        n = len(primaries["species"])
        if id_base is None:
            id_base = n
        view = abi.particles_view(primaries, n)
        out = abi.Particles()
        st = abi.RunStats()
        self._check(self.L.ptg_collide_batch(self._h, C.byref(laser), C.byref(options), C.byref(view), seed, id_base,
                                             C.byref(out), C.byref(st)))
        return _host_arrays(self.L, out), st.as_dict()

    def collide_device(self, laser, options, d_primaries, seed, id_base=None):
        """Device-resident variant: `d_primaries` maps field names to CUDA
        tensors (row-major [n][4] for four-vectors).  Returns (Particles with
        device pointers valid until the next call, stats dict)."""
        n = int(d_primaries["species"].shape[0])
        if id_base is None:
            id_base = n
        view = abi.Particles()
        view.n = n
        for name, dt, _cols in abi.PARTICLE_FIELDS:
            t = d_primaries.get(name)
            ct = {np.float64: C.POINTER(C.c_double), np.int32: C.POINTER(C.c_int32),
                  np.uint64: C.POINTER(C.c_uint64)}[dt]
            setattr(view, name, C.cast(C.c_void_p(t.data_ptr()) if t is not None else None, ct))
        out = abi.Particles()
        st = abi.RunStats()
        self._check(self.L.ptg_collide_batch_device(self._h, C.byref(laser), C.byref(options), C.byref(view), seed,
                                                    id_base, C.byref(out), C.byref(st)))
        return out, st.as_dict()

    # -- multi-collision queue ---------------------------------------------
    @staticmethod
    def _collisions(collisions):
        arr = (abi.Collision * len(collisions))()
        for k, c in enumerate(collisions):
            arr[k].laser = c["laser"]
            arr[k].seed = c["seed"]
            arr[k].id_base = c.get("id_base", 0)
            arr[k].first = c["first"]
            arr[k].count = c["count"]
        return arr

    @staticmethod
    def _device_view(d_primaries):
        view = abi.Particles()
        view.n = int(d_primaries["species"].shape[0])
        for name, dt, _cols in abi.PARTICLE_FIELDS:
            t = d_primaries.get(name)
            ct = {np.float64: C.POINTER(C.c_double), np.int32: C.POINTER(C.c_int32),
                  np.uint64: C.POINTER(C.c_uint64)}[dt]
            setattr(view, name, C.cast(C.c_void_p(t.data_ptr()) if t is not None else None, ct))
        return view

    def collide_multi(self, collisions, options, primaries):
        """Many collisions in one persistent launch.  `collisions`: dicts with
        laser, seed, id_base, first, count (rows of `primaries`).  Returns
        (list of per-collision output dicts, list of per-collision stats,
        total stats)."""
        arr = self._collisions(collisions)
        m = len(collisions)
        view = abi.particles_view(primaries, len(primaries["species"]))
        out = abi.Particles()
        offs = (C.c_uint64 * (m + 1))()
        stats = (abi.RunStats * m)()
        total = abi.RunStats()
        self._check(self.L.ptg_collide_multi(self._h, m, arr, C.byref(options), C.byref(view), C.byref(out), offs,
                                             stats, C.byref(total)))
        whole = _host_arrays(self.L, out)
        parts = [{k: v[offs[i]:offs[i + 1]] for k, v in whole.items()} for i in range(m)]
        return parts, [stats[i].as_dict() for i in range(m)], total.as_dict()

    def collide_multi_device(self, collisions, options, d_primaries):
        """Device-resident multi batch (primaries: dict of CUDA tensors).
        Returns (Particles with device pointers, offsets, per-collision
        stats, total stats)."""
        arr = self._collisions(collisions)
        m = len(collisions)
        view = self._device_view(d_primaries)
        out = abi.Particles()
        offs = (C.c_uint64 * (m + 1))()
        stats = (abi.RunStats * m)()
        total = abi.RunStats()
        self._check(self.L.ptg_collide_multi_device(self._h, m, arr, C.byref(options), C.byref(view), C.byref(out),
                                                    offs, stats, C.byref(total)))
        return out, list(offs), [stats[i].as_dict() for i in range(m)], total.as_dict()

    def queue_config(self, variant=None, blocks_per_sm=None, chunk=None, use_graph=None):
        """Reads, and optionally sets, the queue kernel's launch shape."""
        cur = abi.QueueCfg()
        self._check(self.L.ptg_queue_config(self._h, None, C.byref(cur)))
        if any(v is not None for v in (variant, blocks_per_sm, chunk, use_graph)):
            new = abi.QueueCfg(cur.variant if variant is None else variant,
                               cur.blocks_per_sm if blocks_per_sm is None else blocks_per_sm,
                               cur.chunk if chunk is None else chunk,
                               cur.use_graph if use_graph is None else int(use_graph))
            self._check(self.L.ptg_queue_config(self._h, C.byref(new), C.byref(cur)))
        return cur.as_dict()

    def queue_autotune(self, collisions, options, d_primaries, sample_fraction=0.1):
        """Runs the autotuner on a sample of a device-resident batch; the
        chosen launch shape stays set in the context."""
        arr = self._collisions(collisions)
        view = self._device_view(d_primaries)
        best = abi.QueueCfg()
        ms = C.c_double()
        self._check(self.L.ptg_queue_autotune(self._h, len(collisions), arr, C.byref(options), C.byref(view),
                                              sample_fraction, C.byref(best), C.byref(ms)))
        return best.as_dict(), ms.value

    # -- distribution output -----------------------------------------------
    def histogram(self, particles, spec):
        """Histogram of a particle set on the device (ptg_histogram).
        `particles`: a Particles struct with device pointers (as
        collide_device returns) or a dict of CUDA tensors.  Returns (info
        dict, heights array shaped [bins[1]][bins[0]] in 2d), or (info, None)
        for an empty set."""
        view = particles if isinstance(particles, abi.Particles) else self._device_view(particles)
        info = abi.HgramInfo()
        self._check(self.L.ptg_histogram(self._h, C.byref(view), C.byref(spec), C.byref(info), None, 0))
        if info.empty:
            return _hgram_info(info), None
        counts = np.zeros(info.n_counts)
        self._check(self.L.ptg_histogram(self._h, C.byref(view), C.byref(spec), C.byref(info), _dp(counts),
                                         info.n_counts))
        return _hgram_info(info), counts

    def particle_sums(self, particles, spec):
        """The sums behind a summary statistic (ptg_particle_sums)."""
        view = particles if isinstance(particles, abi.Particles) else self._device_view(particles)
        out = abi.StatsSums()
        self._check(self.L.ptg_particle_sums(self._h, C.byref(view), C.byref(spec), C.byref(out)))
        return out.as_dict()

    # -- beam builder ------------------------------------------------------
    def build_beam(self, desc, n, seed, first_id=0, device=None):
        """Generates n primaries on the device (ptg_build_beam).  Returns a
        dict of CUDA tensors (species, r, u, pol, weight, id, parent_id) that
        collide_device and collide_multi_device accept."""
        import torch
        dev = device if device is not None else torch.device("cuda", self.device)
        out = {"species": torch.empty(n, dtype=torch.int32, device=dev),
               "r": torch.empty((n, 4), dtype=torch.float64, device=dev),
               "u": torch.empty((n, 4), dtype=torch.float64, device=dev),
               "pol": torch.empty((n, 4), dtype=torch.float64, device=dev),
               "weight": torch.empty(n, dtype=torch.float64, device=dev),
               "id": torch.empty(n, dtype=torch.uint64, device=dev),
               "parent_id": torch.empty(n, dtype=torch.uint64, device=dev)}
        view = self._device_view(out)
        torch.cuda.synchronize(dev)
        self._check(self.L.ptg_build_beam(self._h, C.byref(desc), n, seed, first_id, C.byref(view)))
        return out

    # -- learned proposal --------------------------------------------------
    def mlp_init(self, seed=1):
        self._check(self.L.ptg_mlp_init(self._h, seed))

    def mlp_params(self, set_to=None):
        """Returns the FP32 parameter vector (after setting it, if given)."""
        cnt = C.c_int32()
        self._check(self.L.ptg_mlp_params(self._h, None, None, C.byref(cnt)))
        if set_to is not None:
            v = np.ascontiguousarray(set_to, dtype=np.float32)
            self._check(self.L.ptg_mlp_params(self._h, None, v.ctypes.data_as(C.POINTER(C.c_float)), None))
        out = np.zeros(cnt.value, dtype=np.float32)
        self._check(self.L.ptg_mlp_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), None, None))
        return out

    def mlp_grad(self, samples, tau):
        """Loss gradient of a batch: samples [n][MLP_INPUTS + 2] = the inputs,
        bin, target."""
        smp = np.ascontiguousarray(samples, dtype=np.float32).reshape(-1, MLP_INPUTS + 2)
        cnt = C.c_int32()
        self._check(self.L.ptg_mlp_params(self._h, None, None, C.byref(cnt)))
        g = np.zeros(cnt.value, dtype=np.float32)
        loss = C.c_float()
        FP = C.POINTER(C.c_float)
        self._check(self.L.ptg_mlp_grad(self._h, smp.ctypes.data_as(FP), len(smp), tau, g.ctypes.data_as(FP),
                                        C.byref(loss)))
        return g, loss.value

    def mlp_infer(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, MLP_INPUTS)
        out = np.zeros((len(x), 16), dtype=np.float32)
        FP = C.POINTER(C.c_float)
        self._check(self.L.ptg_mlp_infer(self._h, x.ctypes.data_as(FP), len(x), out.ctypes.data_as(FP)))
        return out

    def mlp_train(self, n_samples=2_000_000, batch=4096, epochs=1, lr=2e-3, tau=0.98, seed=7,
                  a_range=(0.05, 20.0), eta_range=(1e-3, 2.0)):
        cfg = abi.MlpTrainCfg(n_samples, batch, epochs, lr, tau, seed, a_range[0], a_range[1], eta_range[0],
                              eta_range[1])
        st = abi.MlpTrainStats()
        self._check(self.L.ptg_mlp_train(self._h, C.byref(cfg), C.byref(st)))
        return st.as_dict()

    def mlp_use(self, enabled=True, margin=0.25):
        self._check(self.L.ptg_mlp_use(self._h, int(enabled), margin))

    def mlp_min_harmonic(self, n=-1):
        """Sets the lowest harmonic at which the collision kernels use the
        network (n >= 0) and returns the previous setting."""
        prev = C.c_int32()
        self._check(self.L.ptg_mlp_min_harmonic(self._h, int(n), C.byref(prev)))
        return prev.value

    def sampler_bench(self, n, seed=3, a_range=(0.05, 20.0), eta_range=(1e-3, 2.0), margin=0.25, want_v=True,
                      detail=False):
        """Plain vs learned v sampler on the same (a, eta, n) draws.  Returns
        (v_plain, v_learned, stats[, per-emission detail dict])."""
        cfg = abi.SamplerBenchCfg(n, seed, a_range[0], a_range[1], eta_range[0], eta_range[1], margin, 0.0)
        st = abi.SamplerBenchStats()
        v0 = np.zeros(n) if want_v else None
        v1 = np.zeros(n) if want_v else None
        det = None
        dv = None
        if detail:
            det = {"x": np.zeros((n, MLP_INPUTS), np.float32), "env": np.zeros((n, 16), np.float32),
                   "status_plain": np.zeros(n, np.int32), "status_learned": np.zeros(n, np.int32),
                   "evals_plain": np.zeros(n, np.uint32), "evals_learned": np.zeros(n, np.uint32),
                   "fallback": np.zeros(n, np.uint32)}
            dv = abi.SamplerBenchDetail()
            for name, _ in abi.SamplerBenchDetail._fields_:
                setattr(dv, name, det[name].ctypes.data_as(dict(abi.SamplerBenchDetail._fields_)[name]))
        self._check(self.L.ptg_sampler_bench(self._h, C.byref(cfg), _dp(v0) if want_v else None,
                                             _dp(v1) if want_v else None, C.byref(dv) if dv is not None else None,
                                             C.byref(st)))
        if detail:
            return v0, v1, st.as_dict(), det
        return v0, v1, st.as_dict()

    def emission_rate_bound(self, a_sqd, eta, circular=True):
        """(FP32 per-step rate or NaN, FP64 rate, in-table flag) at each
        (a^2, eta): the emission step's bound against the reference's rate."""
        a_sqd, eta = _f64(a_sqd, (-1,)), _f64(eta, (-1,))
        out = np.zeros((len(a_sqd), 3))
        self._check(self.L.ptg_emission_rate_bound(self._h, len(a_sqd), int(bool(circular)), _dp(a_sqd), _dp(eta),
                                                   _dp(out)))
        return out[:, 0], out[:, 1], out[:, 2] > 0.5

    def fp64_function_kernel(self, op, iters=64):
        """One launch of k_fp64_fn<op> (abi.FP64_FUNCTIONS names the ops),
        to be profiled for the function's executed FP64 cost."""
        self._check(self.L.ptg_fp64_function_kernel(self._h, int(op), int(iters)))

    def fp64_peak(self):
        """Measured FP64 FMA throughput, TFLOP/s."""
        v = C.c_double()
        self._check(self.L.ptg_fp64_peak(self._h, C.byref(v)))
        return v.value

    # -- diagnostics -----------------------------------------------------
    def fields(self, laser, r):
        r = _f64(r, (-1, 4))
        n = len(r)
        E, B, a = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros(n)
        self._check(self.L.ptg_eval_fields(self._h, C.byref(laser), n, _dp(r), _dp(E), _dp(B), _dp(a)))
        return E, B, a

    def push_steps(self, laser, r, u, rqm, dt, nsteps, eqn=abi.LORENTZ):
        r = _f64(r, (-1, 4)).copy()
        u = _f64(u, (-1, 4)).copy()
        work = np.zeros(len(r))
        self._check(self.L.ptg_push_steps(self._h, C.byref(laser), len(r), _dp(r), _dp(u), rqm, dt, eqn, nsteps,
                                          _dp(work)))
        return r, u, work

    def lcfa_photon_rate(self, chi, gamma):
        chi, gamma = _f64(chi, (-1,)), _f64(gamma, (-1,))
        out = np.zeros(len(chi))
        self._check(self.L.ptg_lcfa_photon_rate(self._h, len(chi), _dp(chi), _dp(gamma), _dp(out)))
        return out

    def lcfa_photon_sample(self, chi, gamma, rand3):
        chi, gamma, rand3 = _f64(chi, (-1,)), _f64(gamma, (-1,)), _f64(rand3, (-1, 3))
        om, th = np.zeros(len(chi)), np.zeros(len(chi))
        self._check(self.L.ptg_lcfa_photon_sample(self._h, len(chi), _dp(chi), _dp(gamma), _dp(rand3), _dp(om),
                                                  _dp(th)))
        return om, th

    def double_bessel(self, n, x, y, mode=0):
        """J(n-2..n+2, x, y) per point, shape [m, 5]."""
        x, y = _f64(x, (-1,)), _f64(y, (-1,))
        out = np.zeros((len(x), 5))
        self._check(self.L.ptg_double_bessel(self._h, n, len(x), _dp(x), _dp(y), mode, _dp(out)))
        return out

    def lp_sample(self, a, eta, seed, streams, step, warp=False):
        """LP LMA samples: ([m, 7] = n, s, theta, 1, xi1, xi2, xi3; [m] status).
        warp=True draws them with the warp-cooperative sampler."""
        a, eta = _f64(a, (-1,)), _f64(eta, (-1,))
        streams = np.ascontiguousarray(streams, dtype=np.uint64)
        out = np.zeros((len(a), 7))
        status = np.zeros(len(a), dtype=np.int32)
        fn = self.L.ptg_lp_sample_warp if warp else self.L.ptg_lp_sample
        self._check(fn(self._h, len(a), _dp(a), _dp(eta), seed, streams.ctypes.data_as(C.POINTER(C.c_uint64)), step,
                       _dp(out), status.ctypes.data_as(C.POINTER(C.c_int32))))
        return out, status

    def cp_sample(self, a, eta, seed, streams, step, warp=False, learned=False):
        """CP LMA samples: ([m, 7] = n, s, theta, 1, xi1, xi2, xi3; [m]
        status), with the reference's sampler or (learned=True) the learned
        proposal in use (mlp_use).  warp=True draws them with the
        warp-cooperative sampler."""
        a, eta = _f64(a, (-1,)), _f64(eta, (-1,))
        streams = np.ascontiguousarray(streams, dtype=np.uint64)
        out = np.zeros((len(a), 7))
        status = np.zeros(len(a), dtype=np.int32)
        sp = streams.ctypes.data_as(C.POINTER(C.c_uint64))
        stp = status.ctypes.data_as(C.POINTER(C.c_int32))
        if learned:
            self._check(self.L.ptg_cp_sample_learned(self._h, len(a), _dp(a), _dp(eta), seed, sp, step, int(warp),
                                                     _dp(out), stp))
        else:
            fn = self.L.ptg_cp_sample_warp if warp else self.L.ptg_cp_sample
            self._check(fn(self._h, len(a), _dp(a), _dp(eta), seed, sp, step, _dp(out), stp))
        return out, status

    def lcfa_pair_t(self, chi):
        chi = _f64(chi, (-1,))
        a, b = np.zeros(len(chi)), np.zeros(len(chi))
        self._check(self.L.ptg_lcfa_pair_t(self._h, len(chi), _dp(chi), _dp(a), _dp(b)))
        return a, b


def laser_timestep(laser):
    dt = C.c_double()
    st = load().ptg_laser_timestep(C.byref(laser), C.byref(dt))
    if st != abi.PTG_OK:
        raise PtgError(st, load().ptg_last_error().decode())
    return dt.value


def laser_initial_z(laser):
    z = C.c_double()
    st = load().ptg_laser_initial_z(C.byref(laser), C.byref(z))
    if st != abi.PTG_OK:
        raise PtgError(st, load().ptg_last_error().decode())
    return z.value
