"""The allocation-free entry point, ptg_collide_batch_noalloc.

It exists for callers that cannot let the library call cudaMalloc (their
device memory belongs to another runtime's pool, or an allocation's device
synchronisation would stall their other streams).  This test calls it
through the C ABI, twice in a row, and checks each result against the
allocating entry point on the same batch: the same kernels and random
streams run, so every particle (matched by its stream id) must agree
exactly.  The file name makes pytest collect it last.
"""

import ctypes as C

import numpy as np
import pytest

from ptarmigan_gb300 import abi, beam

pytestmark = pytest.mark.gpu


def _batch():
    laser = abi.laser_desc(abi.FAST_FOCUSED_LASER, 10.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=4e-6,
                           fwhm_duration=30e-15)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(96, g, sigma=0.01 * g, radius=2e-6, length=20e-6, rms_div=50e-6, laser=laser, seed=21)
    opts = abi.collide_options(max_generation=2, rate_increase=100.0)
    return laser, opts, prim


def _device_view(tensors, n):
    v = abi.Particles()
    v.n = n
    for name, dt, _cols in abi.PARTICLE_FIELDS:
        ct = {np.float64: C.POINTER(C.c_double), np.int32: C.POINTER(C.c_int32),
              np.uint64: C.POINTER(C.c_uint64)}[dt]
        t = tensors.get(name)
        setattr(v, name, C.cast(C.c_void_p(t.data_ptr()) if t is not None else None, ct))
    return v


def _lib():
    from ptarmigan_gb300 import build, engine
    build.build()
    L = engine.load()
    L.ptg_collide_batch_noalloc.restype = C.c_int
    L.ptg_collide_batch_noalloc.argtypes = [
        C.POINTER(abi.LaserDesc), C.POINTER(abi.CollideOptions), C.POINTER(abi.Particles), C.c_uint64, C.c_uint64,
        C.POINTER(abi.Particles), C.c_size_t, C.c_void_p, C.POINTER(abi.RunStats)]
    return L


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from ptarmigan_gb300 import engine
    L = _lib()

    laser, opts, prim = _batch()
    n = len(prim["species"])
    eng = engine.Engine()
    ref, ref_stats = eng.collide(laser, opts, prim, seed=9, id_base=n)
    eng.close()

    dev = torch.device("cuda", 0)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    cap = 4096
    torch_dt = {np.float64: torch.float64, np.int32: torch.int32, np.uint64: torch.int64}
    stream = torch.cuda.current_stream(dev)

    for call in range(2):
        d_out = {name: torch.zeros((cap, cols) if cols > 1 else (cap,), dtype=torch_dt[dt], device=dev)
                 for name, dt, cols in abi.PARTICLE_FIELDS}
        out_view = _device_view(d_out, cap)
        st = abi.RunStats()
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        status = L.ptg_collide_batch_noalloc(C.byref(laser), C.byref(opts), C.byref(_device_view(d_prim, n)), 9, n,
                                             C.byref(out_view), cap, C.c_void_p(stream.cuda_stream), C.byref(st))
        assert status == abi.PTG_OK, L.ptg_last_error().decode()
        torch.cuda.synchronize()
        if call == 1:
            # the second call finds every kernel loaded: nothing may be allocated
            assert torch.cuda.mem_get_info(dev)[0] == free_before
        m = out_view.n
        assert m == len(ref["species"]), (call, m, len(ref["species"]))
        got = {k: v[:m].cpu().numpy() for k, v in d_out.items()}
        got["stream"] = got["stream"].view(np.uint64)
        og = np.argsort(got["stream"])
        orf = np.argsort(ref["stream"])
        assert np.array_equal(got["stream"][og], ref["stream"][orf])
        for k in ("species", "generation", "u", "r", "r0", "pol", "weight", "work", "interaction_count", "status"):
            assert np.array_equal(got[k][og], ref[k][orf]), (call, k)
        assert st.emissions == ref_stats["emissions"] and st.lepton_steps == ref_stats["lepton_steps"]


def test_noalloc_rejects_oversized_batch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = _lib()
    laser, opts, _ = _batch()
    v = abi.Particles()
    v.n = 4097
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    for name, dt, _cols in abi.PARTICLE_FIELDS:
        ct = {np.float64: C.POINTER(C.c_double), np.int32: C.POINTER(C.c_int32),
              np.uint64: C.POINTER(C.c_uint64)}[dt]
        setattr(v, name, C.cast(C.c_void_p(dummy.data_ptr()), ct))
    out = abi.Particles()
    for name, dt, _cols in abi.PARTICLE_FIELDS:
        ct = {np.float64: C.POINTER(C.c_double), np.int32: C.POINTER(C.c_int32),
              np.uint64: C.POINTER(C.c_uint64)}[dt]
        setattr(out, name, C.cast(C.c_void_p(dummy.data_ptr()), ct))
    st = abi.RunStats()
    status = L.ptg_collide_batch_noalloc(C.byref(laser), C.byref(opts), C.byref(v), 1, 0, C.byref(out), 1, None,
                                         C.byref(st))
    assert status == abi.PTG_ERR_INVALID_ARGUMENT
    assert b"4096" in L.ptg_last_error()


def _outputs(torch, dev, cap):
    torch_dt = {np.float64: torch.float64, np.int32: torch.int32, np.uint64: torch.int64}
    d_out = {name: torch.zeros((cap, cols) if cols > 1 else (cap,), dtype=torch_dt[dt], device=dev)
             for name, dt, cols in abi.PARTICLE_FIELDS}
    return d_out, _device_view(d_out, cap)


def test_noalloc_output_capacity_too_small():
    """A result longer than out_capacity is PTG_ERR_QUEUE_OVERFLOW, and the
    needed row count comes back in stats.n_out."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from ptarmigan_gb300 import engine
    L = _lib()
    laser, opts, prim = _batch()
    n = len(prim["species"])
    eng = engine.Engine()
    ref, _ = eng.collide(laser, opts, prim, seed=9, id_base=n)
    eng.close()
    assert len(ref["species"]) > 1
    dev = torch.device("cuda", 0)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    _d_out, out_view = _outputs(torch, dev, 4096)
    st = abi.RunStats()
    status = L.ptg_collide_batch_noalloc(C.byref(laser), C.byref(opts), C.byref(_device_view(d_prim, n)), 9, n,
                                         C.byref(out_view), 1, None, C.byref(st))
    torch.cuda.synchronize()
    assert status == abi.PTG_ERR_QUEUE_OVERFLOW
    assert st.n_out == len(ref["species"])
    assert b"out_capacity" in L.ptg_last_error()


def test_noalloc_store_overflow():
    """A shower that outgrows the fixed store (32768 particles, primaries
    included) is PTG_ERR_QUEUE_OVERFLOW; the allocating path runs the same
    batch and shows that it does need more."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from ptarmigan_gb300 import engine
    L = _lib()
    # 4096 electrons through a long, strong plane wave (LCFA): more than
    # ten photons each
    laser = abi.laser_desc(abi.FAST_PLANE_WAVE, 80.0, 0.8e-6, abi.LINEAR, abi.COS2, n_cycles=60.0)
    g = beam.gamma_from_energy(10.0)
    prim = beam.build(4096, g, sigma=0.001 * g, radius=1e-6, length=10e-6, rms_div=0.0, laser=laser, seed=5)
    opts = abi.collide_options(max_generation=1)
    n = len(prim["species"])
    eng = engine.Engine()
    _, ref_stats = eng.collide(laser, opts, prim, seed=3, id_base=n)
    eng.close()
    assert ref_stats["n_created"] > 32768, ref_stats["n_created"]
    dev = torch.device("cuda", 0)
    d_prim = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in prim.items()}
    _d_out, out_view = _outputs(torch, dev, 4096)
    st = abi.RunStats()
    status = L.ptg_collide_batch_noalloc(C.byref(laser), C.byref(opts), C.byref(_device_view(d_prim, n)), 3, n,
                                         C.byref(out_view), 4096, None, C.byref(st))
    torch.cuda.synchronize()
    assert status == abi.PTG_ERR_QUEUE_OVERFLOW
    assert b"32768" in L.ptg_last_error()


def test_noalloc_empty_batch():
    """No primaries: an empty result, as the allocating entry point gives,
    even with NULL arrays."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = _lib()
    laser, opts, _ = _batch()
    v = abi.Particles()
    v.n = 0
    dev = torch.device("cuda", 0)
    _d_out, out_view = _outputs(torch, dev, 16)
    out_view.n = 123
    st = abi.RunStats()
    st.n_out = 7
    status = L.ptg_collide_batch_noalloc(C.byref(laser), C.byref(opts), C.byref(v), 1, 0, C.byref(out_view), 16, None,
                                         C.byref(st))
    assert status == abi.PTG_OK, L.ptg_last_error().decode()
    assert out_view.n == 0 and st.n_out == 0 and st.n_primaries == 0
