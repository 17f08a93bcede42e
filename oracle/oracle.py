"""Oracle (test infrastructure only): ctypes wrapper of the FP64 CPU
restatement in this directory.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module, and only as the checker; the product library never calls
it.  ``build()`` compiles the C++ sources with the Makefile here.
"""

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from ptarmigan_gb300 import abi  # noqa: E402  (structure definitions only)

LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(quiet=True):
    jobs = str(max(1, min(8, os.cpu_count() or 1)))
    out = subprocess.run(["make", "-C", HERE, "-j", jobs], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    L = C.CDLL(LIB_PATH)
    d, i, u32, u64, vp = C.c_double, C.c_int, C.c_uint32, C.c_uint64, C.c_void_p
    DP = C.POINTER(C.c_double)
    sig = {
        "orc_lcfa_photon_rate": (d, [d, d]),
        "orc_lcfa_classical_rate": (d, [d, d]),
        "orc_lcfa_photon_sample": (None, [d, d, d, d, d, DP, DP, DP]),
        "orc_lcfa_stokes": (None, [DP, d, d, DP, DP, DP]),
        "orc_gaunt_factor": (d, [d]),
        "orc_lcfa_pair_t": (None, [d, DP, DP]),
        "orc_lcfa_pair_probability": (d, [DP, DP, d, DP, d, DP]),
        "orc_lcfa_pair_spectrum": (d, [d, d, d]),
        "orc_lcfa_pair_spectrum_ceiling": (d, [d, d]),
        "orc_lcfa_pair_angular_spectrum": (d, [d, d, d, d]),
        "orc_lcfa_pair_angular_spectrum_ceiling": (d, [d, d, d]),
        "orc_lcfa_pair_sample": (i, [DP, DP, d, DP, u64, u64, u32, DP]),
        "orc_airy_ai": (d, [d]),
        "orc_airy_ai_prime": (d, [d]),
        "orc_bessel_k13": (d, [d]),
        "orc_bessel_k23": (d, [d]),
        "orc_pwmci_evaluate": (d, [DP, i, i, d, C.POINTER(C.c_int)]),
        "orc_pwmci_invert": (d, [DP, i, i, d, C.POINTER(C.c_int)]),
        "orc_philox": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "orc_draws": (None, [u64, u64, u32, i, DP]),
        "orc_primary_stream": (u64, [u64]),
        "orc_child_stream": (u64, [u64, u32, u32]),
        "orc_max_timestep": (d, [C.POINTER(abi.LaserDesc)]),
        "orc_initial_z": (d, [C.POINTER(abi.LaserDesc)]),
        "orc_contains": (i, [C.POINTER(abi.LaserDesc), DP]),
        "orc_fields": (None, [C.POINTER(abi.LaserDesc), DP, DP, DP, DP]),
        "orc_a_sqd": (d, [C.POINTER(abi.LaserDesc), DP]),
        "orc_push": (None, [C.POINTER(abi.LaserDesc), DP, DP, d, d, i, DP, DP, DP, DP]),
        "orc_push_steps": (None, [C.POINTER(abi.LaserDesc), C.c_size_t, DP, DP, d, d, i, i, DP]),
        "orc_collide_run": (vp, [C.POINTER(abi.LaserDesc), C.POINTER(abi.CollideOptions), C.POINTER(abi.Particles),
                                 u64, u64, i]),
        "orc_result_size": (C.c_size_t, [vp]),
        "orc_result_stats": (None, [vp, C.POINTER(abi.RunStats)]),
        "orc_result_copy": (None, [vp, C.POINTER(abi.Particles)]),
        "orc_result_free": (None, [vp]),
        "orc_load_tables": (i, [C.c_char_p]),
        "orc_has_cp_cdf": (i, []),
        "orc_has_lp_mid_cdf": (i, []),
        "orc_bessel_j": (d, [d, i]),
        "orc_bessel_triple_j": (d, [i, d]),
        "orc_bessel_j_asymptotic": (d, [i, d]),
        "orc_bessel_j_pm": (None, [d, i, DP]),
        "orc_cp_diff_partial_rate": (d, [i, d, d, d]),
        "orc_cp_ceiling": (d, [i, d, d]),
        "orc_cp_partial_rate": (d, [i, d, d]),
        "orc_cp_rate": (d, [d, d]),
        "orc_cp_invert": (i, [d, d, d]),
        "orc_cp_sample": (i, [d, d, u64, u64, u32, DP]),
        "orc_nlc_generate": (i, [DP, DP, i, d, u64, u64, u32, DP]),
        "orc_nlc_probability": (d, [DP, DP, d, i]),
        "orc_cp_pair_integrate": (None, [i, d, d, DP]),
        "orc_cp_pair_by_summation": (None, [d, d, DP]),
        "orc_cp_pair_by_lookup": (i, [d, d, DP]),
        "orc_cp_pair_rates": (i, [d, d, DP]),
        "orc_bw_probability": (d, [DP, DP, DP, d, d, i, d, DP]),
        "orc_bw_generate": (i, [DP, DP, DP, d, i, d, u64, u64, u32, DP]),
        "orc_double_bessel_at": (d, [i, d, d, d, d]),
        "orc_double_bessel_evaluate": (d, [i, d, d]),
        "orc_double_bessel_spa": (d, [i, d, d]),
        "orc_lp_ceiling": (d, [i, d, d]),
        "orc_lp_partial_rate": (None, [i, d, d, DP]),
        "orc_lp_sum_limit": (i, [d, d]),
        "orc_lp_rate": (d, [d, d]),
        "orc_lp_harmonic_index": (i, [d, d, d]),
        "orc_lp_sample": (i, [d, d, u64, u64, u32, DP]),
        "orc_lp_pair_rates": (None, [d, d, DP]),
        "orc_cp_cl_integrated": (d, [i, d]),
        "orc_lp_cl_partial_rate": (d, [i, d]),
        "orc_nlc_classical_rate": (d, [d, d, i]),
        "orc_nlc_classical_sample": (i, [d, d, i, u64, u64, u32, DP]),
        "orc_lp_pair_dd_rate": (None, [i, d, d, d, d, DP]),
        "orc_lp_pair_partial_rate": (None, [i, d, d, DP]),
        "orc_lp_pair_by_summation": (None, [d, d, DP]),
        "orc_lp_pair_sample": (i, [d, d, d, d, u64, u64, u32, DP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    tables = os.path.join(ROOT, "ptarmigan_gb300", "tables", "data")
    if L.orc_load_tables(tables.encode()) != 0:
        raise RuntimeError("oracle could not load the LMA tables from " + tables)
    _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _vec(x, n):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(n))
    return a


# -- scalar physics -------------------------------------------------------
def lcfa_photon_rate(chi, gamma):
    return lib().orc_lcfa_photon_rate(chi, gamma)


def lcfa_photon_sample(chi, gamma, r1, r2, r3):
    o, t, p = C.c_double(), C.c_double(), C.c_double()
    lib().orc_lcfa_photon_sample(chi, gamma, r1, r2, r3, C.byref(o), C.byref(t), C.byref(p))
    return o.value, (None if t.value < 0 else t.value), p.value


def lcfa_stokes(k, chi, gamma, v, w):
    out = np.zeros(4)
    k, v, w = _vec(k, 4), _vec(v, 3), _vec(w, 3)
    lib().orc_lcfa_stokes(_dp(k), chi, gamma, _dp(v), _dp(w), _dp(out))
    return out


def gaunt_factor(chi):
    return lib().orc_gaunt_factor(chi)


def lcfa_pair_t(chi):
    a, b = C.c_double(), C.c_double()
    lib().orc_lcfa_pair_t(chi, C.byref(a), C.byref(b))
    return a.value, b.value


def lcfa_pair_probability(ell, sv, chi, a_perp, dt):
    ell, sv, a_perp = _vec(ell, 4), _vec(sv, 4), _vec(a_perp, 3)
    out = np.zeros(4)
    p = lib().orc_lcfa_pair_probability(_dp(ell), _dp(sv), chi, _dp(a_perp), dt, _dp(out))
    return p, out


def lcfa_pair_spectrum(s, chi, sv1):
    return lib().orc_lcfa_pair_spectrum(s, chi, sv1)


def lcfa_pair_spectrum_ceiling(chi, sv1):
    return lib().orc_lcfa_pair_spectrum_ceiling(chi, sv1)


def lcfa_pair_angular_spectrum(y, s, chi, sv1):
    return lib().orc_lcfa_pair_angular_spectrum(y, s, chi, sv1)


def lcfa_pair_angular_spectrum_ceiling(s, chi, sv1):
    return lib().orc_lcfa_pair_angular_spectrum_ceiling(s, chi, sv1)


def lcfa_pair_sample(ell, sv, chi, a_perp, seed, stream, step):
    ell, sv, a_perp = _vec(ell, 4), _vec(sv, 4), _vec(a_perp, 3)
    out = np.zeros(5)
    rc = lib().orc_lcfa_pair_sample(_dp(ell), _dp(sv), chi, _dp(a_perp), seed, stream, step, _dp(out))
    return rc, out


def airy_ai(x):
    return lib().orc_airy_ai(x)


def airy_ai_prime(x):
    return lib().orc_airy_ai_prime(x)


def bessel_k13(x):
    return lib().orc_bessel_k13(x)


def bessel_k23(x):
    return lib().orc_bessel_k23(x)


def pwmci_evaluate(table, x, extrapolate=False):
    t = np.ascontiguousarray(np.asarray(table, dtype=np.float64))
    ok = C.c_int()
    v = lib().orc_pwmci_evaluate(_dp(t), len(t), int(extrapolate), x, C.byref(ok))
    return v if ok.value else None


def pwmci_invert(table, f, extrapolate=False):
    t = np.ascontiguousarray(np.asarray(table, dtype=np.float64))
    ok = C.c_int()
    v = lib().orc_pwmci_invert(_dp(t), len(t), int(extrapolate), f, C.byref(ok))
    return v if ok.value else None


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def draws(seed, stream, step, n):
    out = np.zeros(n)
    lib().orc_draws(seed, stream, step, n, _dp(out))
    return out


def primary_stream(i):
    return lib().orc_primary_stream(i)


def child_stream(parent, step, slot):
    return lib().orc_child_stream(parent, step, slot)


# -- LMA ------------------------------------------------------------------
def bessel_j(x, n):
    return lib().orc_bessel_j(x, n)


def bessel_triple_j(n, x):
    return lib().orc_bessel_triple_j(n, x)


def bessel_j_asymptotic(n, x):
    return lib().orc_bessel_j_asymptotic(n, x)


def bessel_j_pm(x, n):
    out = np.zeros(3)
    lib().orc_bessel_j_pm(x, n, _dp(out))
    return out


def cp_diff_partial_rate(n, a, eta, v):
    return lib().orc_cp_diff_partial_rate(n, a, eta, v)


def cp_ceiling(n, a, eta):
    return lib().orc_cp_ceiling(n, a, eta)


def cp_partial_rate(n, a, eta):
    return lib().orc_cp_partial_rate(n, a, eta)


def cp_rate(a, eta):
    return lib().orc_cp_rate(a, eta)


def has_lp_mid_cdf():
    return bool(lib().orc_has_lp_mid_cdf())


def has_cp_cdf():
    return bool(lib().orc_has_cp_cdf())


def cp_invert(a, eta, frac):
    return lib().orc_cp_invert(a, eta, frac)


def cp_sample(a, eta, seed, stream, step):
    out = np.zeros(7)
    rc = lib().orc_cp_sample(a, eta, seed, stream, step, _dp(out))
    return rc, out


def nlc_generate(k, q, pol, pol_angle, seed, stream, step):
    k, q = _vec(k, 4), _vec(q, 4)
    out = np.zeros(9)
    rc = lib().orc_nlc_generate(_dp(k), _dp(q), pol, pol_angle, seed, stream, step, _dp(out))
    return rc, out


def nlc_probability(k, q, dt, pol):
    k, q = _vec(k, 4), _vec(q, 4)
    return lib().orc_nlc_probability(_dp(k), _dp(q), dt, pol)


def cp_pair_integrate(n, a, eta):
    out = np.zeros(2)
    lib().orc_cp_pair_integrate(n, a, eta, _dp(out))
    return out


def cp_pair_by_summation(a, eta):
    out = np.zeros(2)
    lib().orc_cp_pair_by_summation(a, eta, _dp(out))
    return out


def cp_pair_by_lookup(a, eta):
    out = np.zeros(2)
    rc = lib().orc_cp_pair_by_lookup(a, eta, _dp(out))
    return None if rc else out


def cp_pair_rates(a, eta):
    out = np.zeros(2)
    rc = lib().orc_cp_pair_rates(a, eta, _dp(out))
    return None if rc else out


def bw_probability(ell, sv, k, a, dt, pol, pol_angle=0.0):
    ell, sv, k = _vec(ell, 4), _vec(sv, 4), _vec(k, 4)
    out = np.zeros(4)
    p = lib().orc_bw_probability(_dp(ell), _dp(sv), _dp(k), a, dt, pol, pol_angle, _dp(out))
    return p, out


def bw_generate(ell, sv, k, a, pol, pol_angle, seed, stream, step):
    ell, sv, k = _vec(ell, 4), _vec(sv, 4), _vec(k, 4)
    out = np.zeros(5)
    rc = lib().orc_bw_generate(_dp(ell), _dp(sv), _dp(k), a, pol, pol_angle, seed, stream, step, _dp(out))
    return rc, out


def double_bessel_at(n, x_max, y_max, x, y):
    return lib().orc_double_bessel_at(n, x_max, y_max, x, y)


def double_bessel_evaluate(n, x, y):
    return lib().orc_double_bessel_evaluate(n, x, y)


def double_bessel_spa(n, x, y):
    return lib().orc_double_bessel_spa(n, x, y)


def lp_ceiling(n, a, eta):
    return lib().orc_lp_ceiling(n, a, eta)


def lp_partial_rate(n, a, eta):
    out = np.zeros(2)
    lib().orc_lp_partial_rate(n, a, eta, _dp(out))
    return out


def lp_sum_limit(a, eta):
    return lib().orc_lp_sum_limit(a, eta)


def lp_rate(a, eta):
    return lib().orc_lp_rate(a, eta)


def lp_harmonic_index(a, eta, frac):
    return lib().orc_lp_harmonic_index(a, eta, frac)


def lp_sample(a, eta, seed, stream, step):
    out = np.zeros(7)
    rc = lib().orc_lp_sample(a, eta, seed, stream, step, _dp(out))
    return rc, out


def cp_cl_integrated(n, a):
    return lib().orc_cp_cl_integrated(n, a)


def lp_cl_partial_rate(n, a):
    return lib().orc_lp_cl_partial_rate(n, a)


def nlc_classical_rate(a, eta, pol):
    return lib().orc_nlc_classical_rate(a, eta, pol)


def nlc_classical_sample(a, eta, pol, seed, stream, step):
    out = np.zeros(7)
    rc = lib().orc_nlc_classical_sample(a, eta, pol, seed, stream, step, _dp(out))
    return rc, out


def lp_pair_rates(a, eta):
    out = np.zeros(2)
    lib().orc_lp_pair_rates(a, eta, _dp(out))
    return out


def lp_pair_dd_rate(n, a, eta, s, theta):
    out = np.zeros(2)
    lib().orc_lp_pair_dd_rate(n, a, eta, s, theta, _dp(out))
    return out


def lp_pair_partial_rate(n, a, eta):
    out = np.zeros(2)
    lib().orc_lp_pair_partial_rate(n, a, eta, _dp(out))
    return out


def lp_pair_by_summation(a, eta):
    out = np.zeros(48)
    lib().orc_lp_pair_by_summation(a, eta, _dp(out))
    return out.reshape(16, 3)


def lp_pair_sample(a, eta, sv1, sv2, seed, stream, step):
    out = np.zeros(3)
    rc = lib().orc_lp_pair_sample(a, eta, sv1, sv2, seed, stream, step, _dp(out))
    return rc, out


# -- fields ---------------------------------------------------------------
def max_timestep(laser):
    return lib().orc_max_timestep(C.byref(laser))


def initial_z(laser):
    return lib().orc_initial_z(C.byref(laser))


def contains(laser, r):
    r = _vec(r, 4)
    return bool(lib().orc_contains(C.byref(laser), _dp(r)))


def fields(laser, r):
    r = _vec(r, 4)
    E, B, a = np.zeros(3), np.zeros(3), C.c_double()
    lib().orc_fields(C.byref(laser), _dp(r), _dp(E), _dp(B), C.byref(a))
    return E, B, a.value


def a_sqd(laser, r):
    r = _vec(r, 4)
    return lib().orc_a_sqd(C.byref(laser), _dp(r))


def push(laser, r, u, rqm, dt, eqn=abi.LORENTZ):
    r, u = _vec(r, 4), _vec(u, 4)
    ro, uo, dto, w = np.zeros(4), np.zeros(4), C.c_double(), C.c_double()
    lib().orc_push(C.byref(laser), _dp(r), _dp(u), rqm, dt, eqn, _dp(ro), _dp(uo), C.byref(dto), C.byref(w))
    return ro, uo, dto.value, w.value


def push_steps(laser, r, u, rqm, dt, nsteps, eqn=abi.LORENTZ):
    r = np.ascontiguousarray(np.array(r, dtype=np.float64).reshape(-1, 4))
    u = np.ascontiguousarray(np.array(u, dtype=np.float64).reshape(-1, 4))
    work = np.zeros(len(r))
    lib().orc_push_steps(C.byref(laser), len(r), _dp(r), _dp(u), rqm, dt, eqn, nsteps, _dp(work))
    return r, u, work


# -- collision loop -------------------------------------------------------
def collide(laser, options, primaries, seed, id_base=None, threads=1):
    """Runs the oracle's collide() over a batch of primaries (dict of numpy
    arrays with the abi.PARTICLE_FIELDS names).  Returns (arrays, stats)."""
    n = len(primaries["species"])
    if id_base is None:
        id_base = n
    view = abi.particles_view(primaries, n)
    h = lib().orc_collide_run(C.byref(laser), C.byref(options), C.byref(view), seed, id_base, threads)
    try:
        m = lib().orc_result_size(h)
        out = abi.empty_arrays(m)
        ov = abi.particles_view(out, m)
        lib().orc_result_copy(h, C.byref(ov))
        st = abi.RunStats()
        lib().orc_result_stats(h, C.byref(st))
        st.n_primaries = n
    finally:
        lib().orc_result_free(h)
    return out, st.as_dict()
