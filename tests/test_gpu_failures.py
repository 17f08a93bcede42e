"""The collision loop's failure exits, reached without faulting the GPU.

The reference panics where a sampler cannot proceed (out-of-table
lookups, nonlinear_compton/mod.rs:32-35 and 84-85; the failed kinematics
checks of pair_creation/cp/mod.rs:402,445) and its loops run until they
finish.  Here every loop is bounded and every failure is a per-particle
status (counted in particle_errors) or a call's status, and the context
stays usable afterwards.  The bounds are lowered through
ptg_context_set_limits so that each exit is taken on purpose:

  - a queue wait limited to nanoseconds runs out: PTG_ERR_TIMEOUT;
  - a step cap below the particles' path length: every particle still in
    the field at the cap is retired with PTG_ERR_REJECTION_CAP;
  - a rejection cap of one iteration: samples that need a second trial
    retire their particle with PTG_ERR_REJECTION_CAP;
  - LMA rate tables read outside their range (a0 above 20): the particle
    is retired with PTG_ERR_OUT_OF_TABLE;
  - missing, truncated, mislabelled or NaN-holding table files:
    PTG_ERR_TABLES, with the loaded tables left as they were.
"""

import os
import shutil

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu


@pytest.fixture()
def eng():
    from ptarmigan_gb300 import build, engine
    build.build()
    e = engine.Engine()
    yield e
    e.close()


def _lcfa(n=64, seed=3):
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(n, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=seed)
    return laser, prim


def _cp(n=400, seed=4, a0=5.0):
    laser = abi.laser_desc(abi.FOCUSED_LASER, a0, 0.8e-6, abi.CIRCULAR, abi.GAUSSIAN, waist=3e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(16.5)
    prim = beam.build(n, g, sigma=0.001 * g, radius=1e-6, length=10e-6, rms_div=8e-6, laser=laser, seed=seed)
    return laser, prim


def _status_count(out, status):
    return int(np.sum(out["status"] == status))


def test_queue_wait_runs_out(eng):
    from ptarmigan_gb300.engine import PtgError
    laser, prim = _lcfa()
    opts = abi.collide_options(max_generation=2, rate_increase=100.0)
    coll = [{"laser": laser, "seed": 5, "id_base": len(prim["species"]), "first": 0, "count": len(prim["species"])}]
    ref, ref_st = eng.collide(laser, opts, prim, seed=5)
    for variant in (0, 2):
        eng.queue_config(variant=variant, blocks_per_sm=0, chunk=1, use_graph=0)
        assert eng.set_limits(queue_wait_ns=1)["queue_wait_ns"] == 1
        with pytest.raises(PtgError) as e:
            eng.collide_multi(coll, opts, prim)
        assert e.value.status == abi.PTG_ERR_TIMEOUT
        # the context is still usable: the same batch with the default bound
        eng.set_limits()
        parts, _, total = eng.collide_multi(coll, opts, prim)
        assert total["emissions"] == ref_st["emissions"] and total["lepton_steps"] == ref_st["lepton_steps"]
        assert len(parts[0]["species"]) == len(ref["species"])


def test_step_cap_retires_particles(eng):
    laser, prim = _lcfa()
    opts = abi.collide_options(max_generation=2)
    _, free = eng.collide(laser, opts, prim, seed=7)
    assert free["particle_errors"] == 0
    cap = 300
    eng.set_limits(step_cap=cap)
    out, st = eng.collide(laser, opts, prim, seed=7)
    eng.set_limits()
    n_cap = _status_count(out, abi.PTG_ERR_REJECTION_CAP)
    # every primary needs thousands of steps through the pulse
    prim_rows = out["generation"] == 0
    assert np.all(out["status"][prim_rows] == abi.PTG_ERR_REJECTION_CAP)
    assert st["particle_errors"] == n_cap >= len(prim["species"])
    assert st["max_steps"] <= max(cap, 1 << 18)
    assert st["lepton_steps"] < free["lepton_steps"]


def test_rejection_cap_retires_particles(eng):
    laser, prim = _cp()
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    _, free = eng.collide(laser, opts, prim, seed=9)
    assert free["particle_errors"] == 0 and free["rejections"] > 0
    eng.set_limits(rejection_cap=1)
    out, st = eng.collide(laser, opts, prim, seed=9)
    eng.set_limits()
    n_cap = _status_count(out, abi.PTG_ERR_REJECTION_CAP)
    assert n_cap > 0
    assert st["particle_errors"] == n_cap
    # the same batch with the default cap again: as before
    _, again = eng.collide(laser, opts, prim, seed=9)
    assert again["particle_errors"] == 0 and again["emissions"] == free["emissions"]


def test_out_of_table_amplitude(eng):
    """a0 = 25 takes the CP rate lookup past a = 20 (cp/tables/mod.rs:11-13):
    the reference panics; here the particle is retired with
    PTG_ERR_OUT_OF_TABLE and the batch completes."""
    laser, prim = _cp(n=64, a0=25.0)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    out, st = eng.collide(laser, opts, prim, seed=11)
    n_oot = _status_count(out, abi.PTG_ERR_OUT_OF_TABLE)
    assert n_oot > 0
    assert st["particle_errors"] == n_oot + _status_count(out, abi.PTG_ERR_REJECTION_CAP) + \
        _status_count(out, abi.PTG_ERR_SANITY)


def _table_dir():
    from ptarmigan_gb300 import tables
    return os.path.join(os.path.dirname(tables.__file__), "data")


@pytest.mark.parametrize("damage", ["missing", "truncated", "magic", "nan", "shape"])
def test_bad_table_files(eng, tmp_path, damage):
    from ptarmigan_gb300.engine import PtgError
    laser, prim = _cp(n=64)
    opts = abi.collide_options(pol_resolved=1, max_generation=-1)
    _, before = eng.collide(laser, opts, prim, seed=13)  # loads the shipped tables
    d = tmp_path / "tables"
    shutil.copytree(_table_dir(), d)
    victim = d / "nlc_cp_rate.ptgt"
    raw = victim.read_bytes()
    if damage == "missing":
        victim.unlink()
    elif damage == "truncated":
        victim.write_bytes(raw[:len(raw) // 2])
    elif damage == "magic":
        victim.write_bytes(b"XXXX" + raw[4:])
    elif damage == "nan":
        b = bytearray(raw)
        b[-8:] = np.array([np.nan]).tobytes()
        victim.write_bytes(bytes(b))
    else:
        # a header that claims a different shape
        b = bytearray(raw)
        b[8:12] = np.array([69], dtype=np.uint32).tobytes()
        victim.write_bytes(bytes(b[:len(b) - 61 * 8]))
    with pytest.raises(PtgError) as e:
        eng.load_tables(str(d))
    assert e.value.status == abi.PTG_ERR_TABLES
    # the tables loaded before are still in force
    _, after = eng.collide(laser, opts, prim, seed=13)
    assert after["emissions"] == before["emissions"] and after["lepton_steps"] == before["lepton_steps"]
