"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point the public header declares; host-only entry
points agree with the oracle; without a GPU the context reports
PTG_ERR_NO_DEVICE instead of falling back to anything."""

import ctypes as C
import math
import os
import re

import pytest

from ptarmigan_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    from ptarmigan_gb300 import engine
    return engine.load()


def _declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(ptg_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared_functions()
    assert {"ptg_context_create", "ptg_collide_batch", "ptg_collide_batch_device", "ptg_load_tables"} <= names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(_declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib):
    assert lib.ptg_abi_version() == 2


def test_struct_sizes_match_header():
    import ctypes as C
    assert C.sizeof(abi.LaserDesc) == 16 + 6 * 8
    assert C.sizeof(abi.CollideOptions) == 5 * 8 + 12 * 4 + 0  # 88 bytes, no tail padding
    assert C.sizeof(abi.Particles) == 8 + 18 * 8


@pytest.mark.parametrize("model,env", [(abi.PLANE_WAVE, abi.COS2), (abi.FAST_PLANE_WAVE, abi.GAUSSIAN),
                                       (abi.FOCUSED_LASER, abi.GAUSSIAN), (abi.FAST_FOCUSED_LASER, abi.GAUSSIAN),
                                       (abi.FAST_PLANE_WAVE, abi.FLATTOP), (abi.FOCUSED_LASER, abi.COS2)])
def test_timestep_and_initial_z_match_oracle(lib, orc, model, env):
    from ptarmigan_gb300 import engine
    laser = abi.laser_desc(model, 7.5, 0.8e-6, abi.LINEAR, env, waist=3e-6, n_cycles=12.0)
    assert engine.laser_timestep(laser) == pytest.approx(orc.max_timestep(laser), rel=1e-15)
    assert engine.laser_initial_z(laser) == pytest.approx(orc.initial_z(laser), rel=1e-15)


def test_invalid_laser_is_rejected(lib):
    from ptarmigan_gb300 import engine
    bad = abi.laser_desc(abi.FAST_FOCUSED_LASER, 1.0, 0.8e-6, abi.LINEAR, abi.GAUSSIAN, waist=math.inf, n_cycles=5)
    with pytest.raises(engine.PtgError) as e:
        engine.laser_timestep(bad)
    assert e.value.status == abi.PTG_ERR_INVALID_ARGUMENT


def test_no_device_is_an_error_not_a_fallback(lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    from ptarmigan_gb300 import engine
    with pytest.raises(engine.PtgError) as e:
        engine.Engine()
    assert e.value.status == abi.PTG_ERR_NO_DEVICE


# ctypes mirror -> C struct of the header
_LAYOUTS = {
    "LaserDesc": "ptg_laser_desc", "CollideOptions": "ptg_collide_options", "Particles": "ptg_particles",
    "RunStats": "ptg_run_stats", "DeviceCfg": "ptg_device_cfg", "Collision": "ptg_collision",
    "QueueCfg": "ptg_queue_cfg", "MlpTrainCfg": "ptg_mlp_train_cfg", "MlpTrainStats": "ptg_mlp_train_stats",
    "SamplerBenchCfg": "ptg_sampler_bench_cfg", "SamplerBenchStats": "ptg_sampler_bench_stats",
    "SamplerBenchDetail": "ptg_sampler_bench_detail", "BeamDesc": "ptg_beam_desc", "HgramSpec": "ptg_hgram_spec",
    "HgramInfo": "ptg_hgram_info", "StatsSpec": "ptg_stats_spec", "StatsSums": "ptg_stats_sums",
    "Limits": "ptg_limits",
}


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """Every ctypes mirror has the size and field offsets that a C compiler
    gives the header's struct."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "ptarmigan_gb300.h"', "int main(void) {"]
    for py, cname in _LAYOUTS.items():
        cls = getattr(abi, py)
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (py, cname))
        for field in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (py, field[0], cname, field[0]))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([gcc, "-std=c99", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.rsplit(" ", 1) for line in out if line)
    for py in _LAYOUTS:
        cls = getattr(abi, py)
        assert int(got["%s size" % py]) == C.sizeof(cls), py
        for field in cls._fields_:
            assert int(got["%s.%s" % (py, field[0])]) == getattr(cls, field[0]).offset, (py, field[0])
