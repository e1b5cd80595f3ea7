"""The C-ABI library loads (no GPU needed) and exports every entry point include/rgdn.h
declares; argument validation that needs no device."""
import ctypes as C
import os
import re

import pytest

from raytracedgl1_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "rgdn.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rgdn_[a-z0-9_]+)\s*\(", src)))


def test_header_parses_to_entry_points():
    names = declared_functions()
    assert "rgdn_denoise" in names and "rgdn_calculate_exposure" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = N.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    bound = {name for name, _, _ in N.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_status_strings_and_version():
    lib = N.load()
    assert lib.rgdn_api_version() == 1
    assert lib.rgdn_status_string(N.OUT_OF_BUDGET) == b"out of the memory budget"
    assert lib.rgdn_status_string(12345) == b"unknown status"


def test_null_handles_are_rejected_without_a_device():
    lib = N.load()
    p = N.FrameParams()
    assert lib.rgdn_denoise(None, 0, C.byref(p), None) == N.WRONG_INSTANCE
    assert lib.rgdn_calculate_exposure(None, 0, C.byref(p), None) == N.WRONG_INSTANCE
    assert lib.rgdn_stream_destroy(None) == N.WRONG_INSTANCE
    assert lib.rgdn_context_destroy(None) == N.WRONG_INSTANCE
    assert lib.rgdn_submit_batch(None, None, 0, None) == N.WRONG_INSTANCE


def test_required_bytes_and_validation():
    from raytracedgl1_gb300.denoiser import required_bytes
    b_ref = required_bytes(1920, 1080, N.STORAGE_REF)
    b_f16 = required_bytes(1920, 1080, N.STORAGE_FP16)
    b_f32 = required_bytes(1920, 1080, N.STORAGE_FP32)
    assert 200 * 1920 * 1080 < b_ref < b_f16 < b_f32
    with pytest.raises(N.RgdnError):
        required_bytes(1919, 1080, N.STORAGE_REF)   # odd width (VulkanDevice.cpp:186-188)
    with pytest.raises(N.RgdnError):
        required_bytes(64, 36, 9)


def test_bin_table_rejects_empty_range():
    lib = N.load()
    buf = (C.c_uint8 * 65536)()
    assert lib.rgdn_histogram_bin_table(C.c_float(1.0), C.c_float(1.0), buf) == N.WRONG_FUNCTION_ARGUMENT


# every ctypes mirror of a struct in include/rgdn.h, by its C name
MIRRORS = {
    "rgdn_image": N.Image, "rgdn_frame_params": N.FrameParams, "rgdn_context_create_info": N.ContextCreateInfo,
    "rgdn_stream_create_info": N.StreamCreateInfo, "rgdn_final_params": N.FinalParams, "rgdn_bloom_params": N.BloomParams,
    "rgdn_volumetric_params": N.VolumetricParams, "rgdn_sphere_light": N.SphereLight, "rgdn_occluder": N.Occluder,
    "rgdn_reshade_scene": N.ReshadeScene, "rgdn_job": N.Job, "rgdn_batch_config": N.BatchConfig,
    "rgdn_server_create_info": N.ServerCreateInfo, "rgdn_frame_request": N.FrameRequest,
    "rgdn_frame_result": N.FrameResult, "rgdn_server_stats": N.ServerStats, "rgdn_stage_timing": N.StageTiming,
}


def test_struct_layouts_match_the_header(tmp_path):
    """The size and every field offset of each struct, as a C compiler lays it out from the
    header, equal the ctypes mirror's."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rgdn.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    bad = []
    for line in filter(None, out):
        cname, field, value = line.split()
        py = MIRRORS[cname]
        got = C.sizeof(py) if field == "size" else getattr(py, field).offset
        if got != int(value):
            bad.append(f"{cname}.{field}: C {value}, ctypes {got}")
    assert not bad, bad


def test_copy_host_planes_validates_before_any_copy():
    """rgdn_copy_host_planes refuses a bad count, null arrays or pointers and an unknown copy
    mode before it touches a device."""
    lib = N.load()
    vp3 = (C.c_void_p * 3)(1, 2, 3)
    nb = (C.c_size_t * 3)(16, 16, 16)
    bad = N.WRONG_FUNCTION_ARGUMENT
    assert lib.rgdn_copy_host_planes(vp3, vp3, nb, 0, N.HOST_COPY_SM, None) == bad
    assert lib.rgdn_copy_host_planes(vp3, vp3, nb, 16, N.HOST_COPY_SM, None) == bad
    assert lib.rgdn_copy_host_planes(None, vp3, nb, 3, N.HOST_COPY_SM, None) == bad
    assert lib.rgdn_copy_host_planes(vp3, vp3, None, 3, N.HOST_COPY_SM, None) == bad
    assert lib.rgdn_copy_host_planes(vp3, vp3, nb, 3, 2, None) == bad
    holes = (C.c_void_p * 3)(1, None, 3)
    assert lib.rgdn_copy_host_planes(holes, vp3, nb, 3, N.HOST_COPY_ENGINE, None) == bad
