"""The C ABI library (no GPU): loads, exports every entry point include/bsm_pt.h
declares, rejects bad arguments with the documented status codes."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "bsm_pt.h")).read()
    return sorted(set(re.findall(r"BSM_API\s+[\w\s\*]+?\b(bsm_\w+)\s*\(", txt)))


def test_header_declares_the_pass_interface():
    names = declared()
    for n in ["bsm_create", "bsm_destroy", "bsm_scene_upload", "bsm_scene_build_bvh", "bsm_render",
              "bsm_trace_closest", "bsm_trace_any", "bsm_sync", "bsm_last_error"]:
        assert n in names


def test_library_exports_every_declared_symbol(bsm):
    path = bsm.lib()._name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (bsm_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    assert set(bsm.declared_symbols()) <= exported


def test_every_declared_symbol_is_bound_in_python(bsm):
    assert set(declared()) == set(bsm.declared_symbols())


def test_api_version(bsm):
    assert bsm.lib().bsm_api_version() == 1


def test_create_without_device_or_bad_args(bsm):
    L = bsm.lib()
    h = C.c_void_p()
    assert L.bsm_create(None, 0, 0) == -1
    st = L.bsm_create(C.byref(h), 0, 0)
    if st == bsm.BSM_OK:
        L.bsm_destroy(h)
        pytest.skip("a CUDA device is present")
    assert st == -7  # BSM_ERR_NO_DEVICE


def test_null_context_calls_fail_cleanly(bsm):
    L = bsm.lib()
    assert L.bsm_sync(None, 0) == -1
    assert L.bsm_render(None, 1, None, 0, None, None, None) == -1
    assert L.bsm_trace_closest(None, 1, None, 0, None, 0) == -1
    assert L.bsm_render_primary(None, 1, None, None, 0.0, 0.0, None) == -1
    assert L.bsm_last_error(None) == b"null context"
    L.bsm_destroy(None)


def test_scene_generate_rejects_unknown_kind(bsm):
    p = bsm.SceneGenParams(7, 1, 0, 0, 0, 0)
    d = bsm.SceneDesc()
    assert bsm.lib().bsm_scene_generate(C.byref(p), C.byref(d), None) == -1


def test_bvh_host_rejects_bad_index(bsm):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=1, spheres=1)
    sc.indices = sc.indices.copy()
    sc.indices[0, 0] = sc.positions.shape[0] + 5
    with pytest.raises(bsm.BsmError):
        bsm.bvh_build_host(sc)


def test_settings_default_mirror_reference(bsm):
    s = bsm.PtSettings()
    bsm.lib().bsm_pt_settings_default(C.byref(s))
    # BasicRenderer::PathTracingSettings defaults (basic.hpp:76-81)
    assert s.ray_length == 100.0 and s.max_bounces == 3 and s.denoise == 1 and s.accumulate == 1
    assert s.spp == 1 and s.seed == 1


def test_no_cpu_fallback_without_device(bsm):
    """The product path raises instead of computing on the CPU."""
    h = C.c_void_p()
    if bsm.lib().bsm_create(C.byref(h), 0, 0) == bsm.BSM_OK:
        bsm.lib().bsm_destroy(h)
        pytest.skip("a CUDA device is present")
    with pytest.raises(bsm.BsmError):
        bsm.Context(0)


STRUCTS = {"Material": "bsm_material", "DirLight": "bsm_dir_light", "PointLight": "bsm_point_light",
           "RectLight": "bsm_rect_light", "Sky": "bsm_sky", "SceneDesc": "bsm_scene_desc", "BvhOpts": "bsm_bvh_opts",
           "BvhStats": "bsm_bvh_stats", "Camera": "bsm_camera", "PtSettings": "bsm_pt_settings",
           "ViewOutput": "bsm_view_output", "PrimaryOutput": "bsm_primary_output", "RenderStats": "bsm_render_stats",
           "ViewDesc": "bsm_view_desc", "TuneParams": "bsm_tune_params", "TuneResult": "bsm_tune_result",
           "ServerOpts": "bsm_server_opts", "Request": "bsm_request", "RequestStatus": "bsm_request_status",
           "ServerStats": "bsm_server_stats", "CacheSettings": "bsm_cache_settings",
           "SceneGenParams": "bsm_scene_gen_params", "GeometryDesc": "bsm_geometry_desc", "Instance": "bsm_instance",
           "InstancedSceneDesc": "bsm_instanced_scene_desc", "Submesh": "bsm_submesh", "MeshData": "bsm_mesh_data",
           "ProjectInfo": "bsm_project_info"}


def test_python_structures_match_the_header(bsm, tmp_path):
    """Every ctypes mirror has the size and field offsets the C compiler gives the header's struct."""
    import shutil
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "bsm_pt.h"', "int main(void) {"]
    for py, c in STRUCTS.items():
        lines.append(f'printf("{py} size %zu\\n", sizeof({c}));')
        for fname, _ in getattr(bsm, py)._fields_:
            lines.append(f'printf("{py} {fname} %zu\\n", offsetof({c}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "sizes.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    bad = []
    for line in filter(None, out):
        py, what, val = line.split()
        cls = getattr(bsm, py)
        got = C.sizeof(cls) if what == "size" else getattr(cls, what).offset
        if got != int(val):
            bad.append((py, what, got, int(val)))
    assert not bad, bad
