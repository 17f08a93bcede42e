"""ctypes mirror of ``include/ptarmigan_gb300.h``.

The structures here are the C ABI's, field for field; the host-side Python
API (:mod:`ptarmigan_gb300.api`) fills them from numpy arrays.
"""

import ctypes as C
import math

import numpy as np

PTG_OK = 0
PTG_ERR_INVALID_ARGUMENT = 1
PTG_ERR_OUT_OF_TABLE = 2
PTG_ERR_SANITY = 3
PTG_ERR_REJECTION_CAP = 4
PTG_ERR_QUEUE_OVERFLOW = 5
PTG_ERR_CUDA = 6
PTG_ERR_NO_DEVICE = 7
PTG_ERR_TABLES = 8
PTG_ERR_UNSUPPORTED = 9
PTG_ERR_ALLOC = 10
PTG_ERR_TIMEOUT = 11

PLANE_WAVE, FAST_PLANE_WAVE, FOCUSED_LASER, FAST_FOCUSED_LASER = 0, 1, 2, 3
LINEAR, CIRCULAR = 0, 1
COS2, FLATTOP, GAUSSIAN = 0, 1, 2
ELECTRON, POSITRON, PHOTON = 0, 1, 2

# EquationOfMotion, field/mod.rs:61-65
LORENTZ, LANDAU_LIFSHITZ, MODIFIED_LANDAU_LIFSHITZ = 0, 1, 2


class LaserDesc(C.Structure):
    _fields_ = [
        ("model", C.c_int32),
        ("polarization", C.c_int32),
        ("envelope", C.c_int32),
        ("finite_bandwidth", C.c_int32),
        ("a0", C.c_double),
        ("wavelength", C.c_double),
        ("waist", C.c_double),
        ("n_cycles", C.c_double),
        ("pol_angle", C.c_double),
        ("chirp_b", C.c_double),
    ]


class CollideOptions(C.Structure):
    _fields_ = [
        ("dt_multiplier", C.c_double),
        ("rate_increase", C.c_double),
        ("t_stop", C.c_double),
        ("min_energy", C.c_double),
        ("max_angle", C.c_double),
        ("multiplicity", C.c_int32),
        ("discard_bg_e", C.c_int32),
        ("discard_bg_ph", C.c_int32),
        ("rr", C.c_int32),
        ("tracking_photons", C.c_int32),
        ("tracking_secondaries", C.c_int32),
        ("keep_decayed_photons", C.c_int32),
        ("pol_resolved", C.c_int32),
        ("rotate_stokes_pars", C.c_int32),
        ("classical", C.c_int32),
        ("gaunt_factor", C.c_int32),
        ("max_generation", C.c_int32),
    ]


_DP = C.POINTER(C.c_double)
_I32P = C.POINTER(C.c_int32)
_U64P = C.POINTER(C.c_uint64)


class Particles(C.Structure):
    _fields_ = [
        ("n", C.c_size_t),
        ("species", _I32P),
        ("r", _DP),
        ("u", _DP),
        ("r0", _DP),
        ("u0", _DP),
        ("pol", _DP),
        ("weight", _DP),
        ("payload", _DP),
        ("parent_chi", _DP),
        ("interaction_count", _DP),
        ("work", _DP),
        ("id", _U64P),
        ("parent_id", _U64P),
        ("primary", _U64P),
        ("stream", _U64P),
        ("generation", _I32P),
        ("flags", _I32P),
        ("status", _I32P),
    ]


class RunStats(C.Structure):
    _fields_ = [
        ("n_primaries", C.c_uint64),
        ("n_out", C.c_uint64),
        ("n_created", C.c_uint64),
        ("lepton_steps", C.c_uint64),
        ("photon_steps", C.c_uint64),
        ("emissions", C.c_uint64),
        ("pair_events", C.c_uint64),
        ("rejections", C.c_uint64),
        ("particle_errors", C.c_uint64),
        ("waves", C.c_uint32),
        ("ordered_waves", C.c_uint32),
        ("absorbed_energy", C.c_double),
        ("device_ms", C.c_double),
        ("max_steps", C.c_uint64),
        ("free_steps", C.c_uint64),
        ("wave_ms", C.c_double * 8),
        ("drift_steps", C.c_uint64),
    ]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_ if name not in ("reserved", "wave_ms")}
        d["wave_ms"] = [float(x) for x in self.wave_ms]
        return d


class Collision(C.Structure):
    """ptg_collision: one collision of a multi-collision batch."""
    _fields_ = [
        ("laser", LaserDesc),
        ("seed", C.c_uint64),
        ("id_base", C.c_uint64),
        ("first", C.c_uint64),
        ("count", C.c_uint64),
    ]


class QueueCfg(C.Structure):
    """ptg_queue_cfg: launch shape of the queue kernel."""
    _fields_ = [
        ("variant", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("chunk", C.c_int32),
        ("use_graph", C.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class Limits(C.Structure):
    """ptg_limits: bounds on a particle's steps, a rejection loop and a
    queue wait (0 = the default)."""
    _fields_ = [
        ("queue_wait_ns", C.c_uint64),
        ("step_cap", C.c_uint32),
        ("rejection_cap", C.c_uint32),
        ("reserved", C.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class MlpTrainCfg(C.Structure):
    _fields_ = [
        ("n_samples", C.c_uint64),
        ("batch", C.c_int32),
        ("epochs", C.c_int32),
        ("lr", C.c_float),
        ("tau", C.c_float),
        ("seed", C.c_uint64),
        ("a_lo", C.c_double),
        ("a_hi", C.c_double),
        ("eta_lo", C.c_double),
        ("eta_hi", C.c_double),
    ]


class MlpTrainStats(C.Structure):
    _fields_ = [
        ("loss_first", C.c_float),
        ("loss_last", C.c_float),
        ("steps", C.c_int32),
        ("reserved", C.c_int32),
        ("data_ms", C.c_double),
        ("train_ms", C.c_double),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class SamplerBenchCfg(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("seed", C.c_uint64),
        ("a_lo", C.c_double),
        ("a_hi", C.c_double),
        ("eta_lo", C.c_double),
        ("eta_hi", C.c_double),
        ("margin", C.c_float),
        ("reserved", C.c_float),
    ]


BINS_AUTO, BINS_LOG, BINS_FIXED_NUMBER, BINS_FIXED_SIZE = 0, 1, 2, 3
HEIGHT_COUNT, HEIGHT_DENSITY, HEIGHT_PDF = 0, 1, 2
WEIGHT_NUMBER, WEIGHT_ENERGY, WEIGHT_POL_X, WEIGHT_POL_Y, WEIGHT_HELICITY = 0, 1, 2, 3, 4


class HgramSpec(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("species", C.c_int32),
        ("func", C.c_int32 * 2),
        ("scale", C.c_double * 2),
        ("weight", C.c_int32),
        ("bin_spec", C.c_int32),
        ("height", C.c_int32),
        ("n_bins", C.c_int32),
        ("bin_size", C.c_double),
        ("filter_func", C.c_int32),
        ("reserved", C.c_int32),
        ("filter_min", C.c_double),
        ("filter_max", C.c_double),
    ]


class HgramInfo(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("empty", C.c_int32),
        ("bins", C.c_uint64 * 2),
        ("min", C.c_double * 2),
        ("max", C.c_double * 2),
        ("bin_size", C.c_double * 2),
        ("bin_volume", C.c_double),
        ("total", C.c_double),
        ("unweighted_total", C.c_double),
        ("n_counts", C.c_uint64),
    ]


class StatsSpec(C.Structure):
    _fields_ = [
        ("species", C.c_int32),
        ("var_func", C.c_int32),
        ("weight_func", C.c_int32),
        ("filter_func", C.c_int32),
        ("min", C.c_double),
        ("max", C.c_double),
        ("shift", C.c_double),
    ]


class StatsSums(C.Structure):
    _fields_ = [(name, C.c_double) for name in ("total", "subtotal", "count", "minimum", "maximum", "sum_diffs",
                                                 "sum_sq_diffs", "sum_cos", "sum_sin")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


GAMMA_NORMAL, GAMMA_BREM, GAMMA_CUSTOM = 0, 1, 2
RADIAL_NORMAL, RADIAL_TRUNC_NORMAL, RADIAL_UNIFORM = 0, 1, 2


class BeamDesc(C.Structure):
    _fields_ = [
        ("species", C.c_int32),
        ("gamma_dstr", C.c_int32),
        ("gamma_mean", C.c_double),
        ("gamma_sigma", C.c_double),
        ("gamma_min", C.c_double),
        ("gamma_max", C.c_double),
        ("energy_chirp", C.c_double),
        ("custom_cdf", C.POINTER(C.c_double)),
        ("custom_len", C.c_int32),
        ("radial_dstr", C.c_int32),
        ("sigma_x", C.c_double),
        ("sigma_y", C.c_double),
        ("x_max", C.c_double),
        ("y_max", C.c_double),
        ("r_max", C.c_double),
        ("sigma_z", C.c_double),
        ("rms_div", C.c_double),
        ("collision_angle", C.c_double),
        ("collision_plane", C.c_double),
        ("offset", C.c_double * 3),
        ("initial_z", C.c_double),
        ("pol", C.c_double * 4),
        ("weight", C.c_double),
    ]


def beam_desc(gamma_mean=None, gamma_sigma=0.0, species=ELECTRON, gamma_dstr=GAMMA_NORMAL, gamma_min=0.0,
              gamma_max=0.0, energy_chirp=0.0, custom_cdf=None, radial_dstr=RADIAL_NORMAL, sigma_x=0.0,
              sigma_y=None, x_max=0.0, y_max=0.0, r_max=0.0, sigma_z=0.0, rms_div=0.0, collision_angle=0.0,
              collision_plane=0.0, offset=(0.0, 0.0, 0.0), initial_z=0.0, stokes=(0.0, 0.0, 0.0), weight=1.0):
    """A BeamDesc (the YAML beam section's keys).  `custom_cdf`: [len][2]
    (gamma, CDF) nodes; the array must outlive the call that uses it."""
    d = BeamDesc()
    d.species, d.gamma_dstr, d.radial_dstr = species, gamma_dstr, radial_dstr
    d.gamma_mean = gamma_mean if gamma_mean is not None else 0.0
    d.gamma_sigma, d.gamma_min, d.gamma_max, d.energy_chirp = gamma_sigma, gamma_min, gamma_max, energy_chirp
    if custom_cdf is not None:
        d.custom_cdf = custom_cdf.ctypes.data_as(C.POINTER(C.c_double))
        d.custom_len = len(custom_cdf)
    d.sigma_x = sigma_x
    d.sigma_y = sigma_x if sigma_y is None else sigma_y
    d.x_max, d.y_max, d.r_max, d.sigma_z, d.rms_div = x_max, y_max, r_max, sigma_z, rms_div
    d.collision_angle, d.collision_plane = collision_angle, collision_plane
    for k in range(3):
        d.offset[k] = offset[k]
    d.initial_z = initial_z
    d.pol[0] = 1.0
    for k in range(3):
        d.pol[k + 1] = stokes[k]
    d.weight = weight
    return d


# Inputs of the learned proposal's network (features of a, eta, n).
MLP_INPUTS = 6


class SamplerBenchDetail(C.Structure):
    _fields_ = [
        ("x", C.POINTER(C.c_float)),
        ("env", C.POINTER(C.c_float)),
        ("status_plain", C.POINTER(C.c_int32)),
        ("status_learned", C.POINTER(C.c_int32)),
        ("evals_plain", C.POINTER(C.c_uint32)),
        ("evals_learned", C.POINTER(C.c_uint32)),
        ("fallback", C.POINTER(C.c_uint32)),
    ]


class SamplerBenchStats(C.Structure):
    _fields_ = [
        ("plain_ms", C.c_double),
        ("learned_ms", C.c_double),
        ("features_ms", C.c_double),
        ("infer_ms", C.c_double),
        ("plain_evals", C.c_double),
        ("learned_evals", C.c_double),
        ("acceptance", C.c_double),
        ("fallbacks", C.c_uint64),
        ("exhausted", C.c_uint64),
        ("errors_plain", C.c_uint64),
        ("errors_learned", C.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class DeviceCfg(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("reserved", C.c_int32),
        ("initial_capacity", C.c_size_t),
    ]


# Array layout of each Particles field: (name, dtype, columns)
PARTICLE_FIELDS = [
    ("species", np.int32, 1),
    ("r", np.float64, 4),
    ("u", np.float64, 4),
    ("r0", np.float64, 4),
    ("u0", np.float64, 4),
    ("pol", np.float64, 4),
    ("weight", np.float64, 1),
    ("payload", np.float64, 1),
    ("parent_chi", np.float64, 1),
    ("interaction_count", np.float64, 1),
    ("work", np.float64, 1),
    ("id", np.uint64, 1),
    ("parent_id", np.uint64, 1),
    ("primary", np.uint64, 1),
    ("stream", np.uint64, 1),
    ("generation", np.int32, 1),
    ("flags", np.int32, 1),
    ("status", np.int32, 1),
]

_CT = {np.float64: _DP, np.int32: _I32P, np.uint64: _U64P}


def empty_arrays(n):
    """Host arrays for every Particles field, n rows."""
    out = {}
    for name, dt, cols in PARTICLE_FIELDS:
        shape = (n, cols) if cols > 1 else (n,)
        out[name] = np.zeros(shape, dtype=dt)
    return out


def particles_view(arrays, n=None):
    """A Particles struct pointing at the given numpy arrays (kept alive by
    the caller).  Missing fields are NULL."""
    p = Particles()
    first = next(iter(arrays.values()))
    p.n = len(first) if n is None else n
    for name, dt, _cols in PARTICLE_FIELDS:
        a = arrays.get(name)
        if a is None:
            setattr(p, name, C.cast(None, _CT[dt]))
            continue
        if a.dtype != dt or not a.flags["C_CONTIGUOUS"]:
            raise TypeError("field %s must be a C-contiguous %s array" % (name, np.dtype(dt).name))
        setattr(p, name, a.ctypes.data_as(_CT[dt]))
    return p


def laser_desc(model, a0, wavelength, polarization=LINEAR, envelope=None, waist=math.inf, n_cycles=None,
               fwhm_duration=None, pol_angle=0.0, chirp_b=0.0, finite_bandwidth=False):
    """Builds a LaserDesc the way main.rs:405-470 reads laser keys."""
    focusing = model in (FOCUSED_LASER, FAST_FOCUSED_LASER)
    if envelope is None:
        envelope = GAUSSIAN if focusing else COS2
    if envelope == GAUSSIAN and fwhm_duration is not None:
        n_cycles = 2.997925e8 * fwhm_duration / wavelength
    if n_cycles is None:
        raise ValueError("n_cycles (or fwhm_duration for a gaussian envelope) is required")
    if polarization == CIRCULAR:
        pol_angle = 0.0
    if focusing:
        chirp_b = 0.0
    return LaserDesc(model, polarization, envelope, int(finite_bandwidth), a0, wavelength, waist, n_cycles,
                     pol_angle, chirp_b)


def collide_options(**kw):
    """CollideOptions with the reference's defaults (main.rs:339-400, 1102-1117)."""
    o = CollideOptions()
    o.dt_multiplier = 1.0
    o.rate_increase = 1.0
    o.t_stop = math.inf
    o.min_energy = 0.0
    o.max_angle = math.pi
    o.multiplicity = -1
    o.discard_bg_e = 0
    o.discard_bg_ph = 0
    o.rr = 1
    o.tracking_photons = 1
    o.tracking_secondaries = 1
    o.keep_decayed_photons = 0
    o.pol_resolved = 0
    o.rotate_stokes_pars = 1
    o.classical = 0
    o.gaunt_factor = 0
    o.max_generation = -1
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


# ptg_fp64_function: the FP64 library functions whose executed cost
# ptg_fp64_function_kernel exposes to a profiler
FP64_FUNCTIONS = {"none": 0, "exp": 1, "log": 2, "div": 3, "sqrt": 4, "cbrt": 5, "sincos": 6, "pow": 7, "atan2": 8,
                  "hypot": 9, "log1p": 10, "acos": 11}
