"""The C-ABI library without a GPU: it loads, exports every function the
header declares, its structures have the header's layout, and its host-only
helpers (uniform producers, parameter presets) follow the reference."""
import ctypes as C
import math
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from meteoros_gb300 import abi

HEADER = Path(__file__).resolve().parents[1] / "include" / "meteoros.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"MT_API\s+[\w\s\*]+?\b(mt_\w+)\s*\(", text)))


def test_every_declared_function_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} is declared in meteoros.h but not exported"
        assert n in abi.SIGNATURES, f"{n} has no ctypes signature"


def test_struct_layout_matches_header(tmp_path):
    fields = {
        "mt_camera_ubo": abi.CameraUBO, "mt_time_ubo": abi.TimeUBO, "mt_params": abi.Params,
        "mt_stats": abi.Stats, "mt_view": abi.View, "mt_tuning": abi.Tuning, "mt_kernel_times": abi.KernelTimes,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for cname, py in fields.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for cname, py in fields.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(out[f"{cname}.{fname}"]) == getattr(py, fname).offset, f"{cname}.{fname}"


def test_abi_version(lib):
    assert lib.mt_abi_version() == 1


def halton_reference(index: int, base: int) -> float:
    """Scene::HaltonSequenceAt (Scene.cpp:125-138) in float32."""
    f, r = np.float32(1.0), np.float32(0.0)
    while index > 0:
        f = np.float32(f / np.float32(base))
        r = np.float32(r + np.float32(f * np.float32(index % base)))
        index = index // base
    return float(r)


def test_halton_and_time_ubo(lib):
    for i in range(1, 17):
        assert lib.mt_halton(i, 3) == halton_reference(i, 3)
    t = abi.time_init()
    seq = list(t.halton_seq1) + list(t.halton_seq2) + list(t.halton_seq3) + list(t.halton_seq4)
    assert seq == [halton_reference(i, 3) for i in range(1, 17)]
    assert t.frame_count_mod16 == 0 and t.time[0] == 0.0 and t.time[1] == 0.0
    for k in range(1, 40):
        abi.time_advance(t, 0.25)
        assert t.frame_count_mod16 == k % 16
    assert t.time[1] == pytest.approx(39 * 0.25)


def test_reference_preset_matches_shader_constants(lib):
    p = abi.params_reference()
    assert p.earth_radius == 6371000.0
    assert p.shell_inner_radius == 6371000.0 + 7500.0
    assert p.shell_outer_radius == 6371000.0 + 20000.0
    assert (p.steps_min, p.steps_max) == (35, 60)
    assert p.accum_limit == 1.0 and p.coverage == np.float32(0.6) and p.coverage_mode == 0
    assert p.noise_period == 8.0 and p.eye_sign == -1.0
    assert list(p.wind_dir) == [1.0, np.float32(0.1), 0.0] and p.wind_speed == np.float32(0.08)
    assert list(p.sky_sun_pos) == [0.0, 6371000.0 * 2.0, -6371000.0 * 10.0]
    assert (p.feedback_min, p.feedback_max) == (0.0, 0.5)
    for i in range(16):  # cloudRayMarch.comp:697-698
        assert p.slot_x[i] == int(math.floor(i // 4))
        assert p.slot_y[i] == int(math.floor(i - 4 * math.floor(i / 4)))


def test_config_preset(lib):
    p = abi.params_config()
    assert p.earth_radius == np.float32(6.36e6)
    assert p.shell_outer_radius - p.shell_inner_radius == 2500.0
    assert p.steps_min == p.steps_max == 128
    assert p.feedback_min == p.feedback_max == np.float32(0.1)
    # 4x4 Bayer order visits every slot of the block once
    slots = {(p.slot_x[i], p.slot_y[i]) for i in range(16)}
    assert len(slots) == 16
    assert (p.slot_x[0], p.slot_y[0]) == (0, 0) and (p.slot_x[1], p.slot_y[1]) == (2, 2)
    # 10 m/s in noise units: metres / (thickness * noise_period)
    assert p.wind_speed == pytest.approx(10.0 / (2500.0 * 8.0))


def test_camera_look_at(lib):
    cam = abi.camera_look_at((0.0, 0.0, 2.0), (0.0, 0.0, 1.0), 45.0, 1284 / 720, 0.1, 1000.0)
    v = np.array(cam.view[:], np.float64).reshape(4, 4)  # [col][row]
    rows = v[:3, :3].T
    assert np.allclose(rows @ rows.T, np.eye(3), atol=1e-6)
    assert np.allclose(rows[2], [0, 0, 1], atol=1e-7)  # -forward, forward = -z
    assert cam.tan_fov_by_2[1] == pytest.approx(math.tan(math.radians(22.5)), rel=1e-5)
    assert cam.proj[5] < 0  # proj[1][1] flipped (camera.cpp:35)
    assert list(cam.eye) == [0.0, 0.0, 2.0, 1.0]


def test_calls_without_a_context_fail_cleanly(lib):
    cam, tm, p = abi.CameraUBO(), abi.time_init(), abi.params_reference()
    assert lib.mt_render(None, C.byref(cam), C.byref(cam), C.byref(tm), C.byref(p), None, None, None, 4, 4, 0,
                         None) == abi.MT_ERR_INVALID_ARG
    assert lib.mt_get_stats(None, None, 0, None) == abi.MT_ERR_INVALID_ARG


def test_create_without_gpu_reports_why(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    st = lib.mt_create(C.byref(h), 0)
    assert st == abi.MT_ERR_UNSUPPORTED
    assert h.value is None
    assert lib.mt_last_error(None)


def test_oracle_uniform_producers_equal_the_library(lib, oracle):
    """The oracle's restatement of the reference's producers (used by the CPU
    legs of the benchmark, which must not load the CUDA library) gives the
    same bytes as the library's, so both arms render the same inputs."""
    from meteoros_gb300 import scenes

    def raw(s):
        return bytes(C.string_at(C.addressof(s), C.sizeof(s)))

    for i in range(0, 40):
        for b in (2, 3, 5):
            assert oracle.halton(i, b) == lib.mt_halton(i, b)
    assert raw(oracle.time_init()) == raw(abi.time_init())
    assert raw(oracle.params_reference()) == raw(abi.params_reference())
    assert raw(oracle.params_config()) == raw(abi.params_config())
    rng = np.random.default_rng(3)
    for _ in range(200):
        eye = tuple(float(x) for x in rng.uniform(-100, 100, 3))
        ref = tuple(e + float(d) for e, d in zip(eye, rng.normal(size=3)))
        fov, aspect = float(rng.uniform(20, 90)), float(rng.uniform(0.5, 3.0))
        assert raw(oracle.camera_look_at(eye, ref, fov, aspect, 0.1, 1000.0)) == \
            raw(abi.camera_look_at(eye, ref, fov, aspect, 0.1, 1000.0))
    for seed in range(5):
        a = scenes.config_sequence(seed, 1920, 1080, frames=4)
        b = scenes.config_sequence(seed, 1920, 1080, frames=4, uniforms=oracle)
        for fa, fb in zip(a, b):
            assert all(raw(x) == raw(y) for x, y in zip(fa, fb))
    a = scenes.reference_frame(64, 36, pitch_deg=10.0, frame=3, t=1.5)
    b = scenes.reference_frame(64, 36, pitch_deg=10.0, frame=3, t=1.5, uniforms=oracle)
    assert all(raw(x) == raw(y) for x, y in zip(a, b))
