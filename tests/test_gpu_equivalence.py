"""Statistical equivalence with the reference at the configurations' own
sizes and rates (no rate_increase).

The oracle (the FP64 C++ restatement of src/main.rs:134-289, pinned to the
reference's known-answer tests) runs 1e5 primaries of each workload; the
GPU runs 1e6 primaries of an independent beam with the same distributions
(another beam seed).  Photon energy and polar-angle spectra are compared
by two-sample KS at the 1e-3 significance level and by a chi-square on 200
logarithmic energy bins (1 MeV to 5 GeV); the pair yield, the mean photon
Stokes parameters and the mean electron energy loss must agree within 5
combined standard errors.  The learned proposal in the persistent queue
(the CP shower's value path) is compared with the oracle directly.

A smaller batch shared by both sides (same primaries, seed and id base)
is matched particle by particle: the table sampler draws from the same
streams as the oracle, so at least 99.9 % of the oracle's particles must
be present on the GPU with momenta agreeing to the stated tolerance, and
the event counts must agree to 0.1 %.
"""

import numpy as np
import pytest

from ptarmigan_gb300 import equivalence

pytestmark = pytest.mark.gpu

N_GPU = 1_000_000
N_ORACLE = 100_000


@pytest.fixture(scope="module")
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    yield e
    e.close()


def _threads():
    import os
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _oracle(make, n, beam_seed, seed):
    from oracle import oracle
    oracle.build()
    laser, opts, prim = make(n, beam_seed)
    out, st = oracle.collide(laser, opts, prim, seed=seed, threads=_threads())
    assert st["particle_errors"] == 0
    return out, prim


def _check(cmp, label):
    assert equivalence.passes(cmp), (label, {k: cmp[k] for k in (
        "ks_photon_energy", "ks_photon_energy_critical", "ks_photon_polar_angle", "ks_photon_polar_angle_critical",
        "chi2_log_energy_200", "chi2_dof", "chi2_p", "sigma")})


def _shared_batch(eng, make, n, tol):
    from oracle import oracle
    laser, opts, prim = make(n, 11)
    ref, rst = oracle.collide(laser, opts, prim, seed=13, threads=_threads())
    eng.mlp_use(False)
    out, st = eng.collide(laser, opts, prim, seed=13)
    m = equivalence.match(out, ref, tol)
    assert m["matched_frac"] >= 0.999, m
    assert m["momentum_agree_frac"] >= 0.999, m
    # the same events: a decision differs only where a draw falls within
    # rounding of its probability
    for k in ("lepton_steps", "photon_steps", "emissions", "pair_events"):
        assert abs(st[k] - rst[k]) <= 1e-3 * rst[k] + 2, (k, st[k], rst[k])


def test_cp_shower_equivalence(eng):
    """The CP LMA shower (a0 = 5 CP focused laser) with Stokes parameters tracked, pairs
    on.  Both the reference sampler (waves) and the learned proposal
    (persistent queue) against the oracle."""
    import bench
    make = bench.cp_shower_workload
    ref, prim_r = _oracle(make, N_ORACLE, 2, 3)
    laser, opts, prim = make(N_GPU, 1)
    eng.mlp_use(False)
    out, st = eng.collide(laser, opts, prim, seed=1000)
    assert st["particle_errors"] == 0
    _check(equivalence.compare(out, prim, ref, prim_r), "table sampler, waves")
    eng.mlp_init(3)
    eng.mlp_train(n_samples=10_000_000, batch=16384, epochs=2)
    eng.mlp_use(True)
    coll = [{"laser": laser, "seed": 1000, "id_base": N_GPU, "first": 0, "count": N_GPU}]
    parts, _, total = eng.collide_multi(coll, opts, prim)
    eng.mlp_use(False)
    assert total["particle_errors"] == 0
    _check(equivalence.compare(parts[0], prim, ref, prim_r), "learned proposal, queue")
    _shared_batch(eng, make, 20_000, 5e-7)


def test_lcfa_shower_equivalence(eng):
    """The focused LCFA shower (a0 = 10 LP), pairs on, generations <= 2."""
    import bench
    make = bench.lcfa_workload
    ref, prim_r = _oracle(make, N_ORACLE, 2, 3)
    laser, opts, prim = make(N_GPU, 1)
    out, st = eng.collide(laser, opts, prim, seed=1000)
    assert st["particle_errors"] == 0
    _check(equivalence.compare(out, prim, ref, prim_r), "LCFA shower")
    _shared_batch(eng, make, 8_000, 1e-8)


def test_plane_wave_equivalence(eng):
    """The LP plane wave (a0 = 1, cos^2 envelope) in the LMA, emission only."""
    import bench
    make = bench.plane_wave_lma_workload
    ref, prim_r = _oracle(make, N_ORACLE, 2, 3)
    laser, opts, prim = make(N_GPU, 1)
    out, st = eng.collide(laser, opts, prim, seed=1000)
    assert st["particle_errors"] == 0
    _check(equivalence.compare(out, prim, ref, prim_r), "LP plane wave")
    _shared_batch(eng, make, 20_000, 5e-7)
