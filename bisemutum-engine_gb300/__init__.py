"""Host-side Python mirror of the GB300 path-tracing pass (ctypes over libbsm_pt.so).

The product is the C ABI in ``include/bsm_pt.h``; this module binds it for
tests, the benchmark and Python callers.  ``PathTracingPass`` mirrors the
reference pass's interface (bisemutum/src/renderer/pass/path_tracing.hpp:27-35:
``update_params(lights, skybox, settings)`` then ``render(camera, ..., settings)``
returning the colour output), ``PathTracingSettings`` mirrors
``BasicRenderer::PathTracingSettings`` (bisemutum/include/bisemutum/renderer/basic.hpp:76-81).

There is no CPU fallback: if the native library is missing or no CUDA device
is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbsm_pt.so")

# ---------------------------------------------------------------- status ----
BSM_OK = 0
STATUS_NAMES = {
    0: "BSM_OK", -1: "BSM_ERR_INVALID_ARG", -2: "BSM_ERR_OUT_OF_MEMORY", -3: "BSM_ERR_CUDA", -4: "BSM_ERR_TIMEOUT",
    -5: "BSM_ERR_NOT_FOUND", -6: "BSM_ERR_BAD_STATE", -7: "BSM_ERR_NO_DEVICE", -8: "BSM_ERR_UNSUPPORTED",
    -9: "BSM_ERR_DEVICE_CHECK", -10: "BSM_ERR_ADMISSION", -11: "BSM_ERR_CANCELLED",
}
BSM_HOST, BSM_DEVICE = 0, 1
BSM_SKY_CONSTANT, BSM_SKY_EQUIRECT, BSM_SKY_CUBEMAP = 0, 1, 2
BSM_SCENE_ROOM, BSM_SCENE_TERRAIN = 0, 1
BSM_PT_JITTER, BSM_PT_NO_SUN_NEE, BSM_PT_NO_SKY_NEE, BSM_PT_STAGE_TIMING, BSM_PT_NO_GRAPH = 1, 2, 4, 8, 16
BSM_PT_COUNT_TRAVERSAL = 32
BSM_PT_DETERMINISTIC = 64
BSM_SERVER_DETERMINISTIC = 1
MISS = 0xFFFFFFFF


class BsmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# ---------------------------------------------------------- C structures ----
BSM_BLEND_OPAQUE, BSM_BLEND_ALPHA_TEST, BSM_BLEND_TRANSLUCENT = 0, 1, 2


class Material(C.Structure):
    _fields_ = [("base_color", C.c_float * 3), ("roughness", C.c_float), ("metallic", C.c_float),
                ("emission", C.c_float * 3), ("opacity", C.c_float), ("blend_mode", C.c_uint32)]


class DirLight(C.Structure):
    _fields_ = [("direction", C.c_float * 3), ("emission", C.c_float * 3)]


class Sky(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("color", C.c_float * 3), ("width", C.c_uint32), ("height", C.c_uint32),
                ("rgba16f", C.POINTER(C.c_uint16)), ("transform", C.c_float * 9)]


class PointLight(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("emission", C.c_float * 3), ("range", C.c_float),
                ("direction", C.c_float * 3), ("cos_inner", C.c_float), ("cos_outer", C.c_float)]


class RectLight(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("axis_x", C.c_float * 3), ("axis_y", C.c_float * 3),
                ("width", C.c_float), ("height", C.c_float), ("emission", C.c_float * 3),
                ("two_sided", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.POINTER(C.c_float)),
                ("num_triangles", C.c_uint32), ("indices", C.POINTER(C.c_uint32)),
                ("material_ids", C.POINTER(C.c_uint32)), ("num_materials", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_dir_lights", C.c_uint32),
                ("dir_lights", C.POINTER(DirLight)), ("sky", Sky), ("num_point_lights", C.c_uint32),
                ("point_lights", C.POINTER(PointLight)), ("num_rect_lights", C.c_uint32),
                ("rect_lights", C.POINTER(RectLight)), ("normals", C.POINTER(C.c_float))]


BSM_COLLAPSE_SAH_OPTIMAL, BSM_COLLAPSE_GREEDY = 0, 1
BSM_BUILD_DEVICE, BSM_BUILD_HOST = 0, 1


class BvhOpts(C.Structure):
    _fields_ = [("sah_bins", C.c_uint32), ("max_leaf_tris", C.c_uint32), ("num_threads", C.c_uint32),
                ("collapse", C.c_uint32), ("tri_cost", C.c_float), ("builder", C.c_uint32)]


class BvhStats(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_tris", C.c_uint32), ("max_depth", C.c_uint32),
                ("builder", C.c_uint32), ("build_ms", C.c_double), ("sah_cost", C.c_double),
                ("node_bytes", C.c_uint64), ("tri_bytes", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("front", C.c_float * 3), ("up", C.c_float * 3),
                ("yfov_deg", C.c_float), ("width", C.c_uint32), ("height", C.c_uint32)]

    def as_array(self) -> np.ndarray:
        """pos3 front3 up3 fov w h — the oracle's camera layout."""
        return np.array([*self.position, *self.front, *self.up, self.yfov_deg, self.width, self.height], np.float32)


class PtSettings(C.Structure):
    _fields_ = [("ray_length", C.c_float), ("max_bounces", C.c_uint32), ("accumulate", C.c_uint32),
                ("denoise", C.c_uint32), ("spp", C.c_uint32), ("max_segments", C.c_uint32), ("seed", C.c_uint64),
                ("sample_offset", C.c_uint32), ("flags", C.c_uint32), ("t_min", C.c_float),
                ("ray_offset", C.c_float), ("wavefront_capacity", C.c_uint32), ("block_size", C.c_uint32)]


class ViewOutput(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("row_pitch_px", C.c_uint32), ("location", C.c_uint32)]


class PrimaryOutput(C.Structure):
    _fields_ = [("depth", C.c_void_p), ("gbuffer", C.c_void_p * 4), ("hit_positions", C.c_void_p),
                ("location", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("rays_per_segment", C.c_uint64 * 16), ("chunks", C.c_uint32), ("extend_launches", C.c_uint32),
                ("ms_total", C.c_float), ("ms_camera", C.c_float), ("ms_extend", C.c_float),
                ("ms_shade", C.c_float), ("ms_shadow", C.c_float), ("ms_resolve", C.c_float),
                ("traversal_nodes", C.c_uint64), ("traversal_tris", C.c_uint64)]


class ViewDesc(C.Structure):
    _fields_ = [("camera", Camera), ("spp", C.c_uint32), ("max_segments", C.c_uint32), ("seed", C.c_uint64)]


class TuneParams(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("wavefront_capacity", C.c_uint32), ("postpone_depth", C.c_uint32),
                ("refill_lanes", C.c_uint32), ("register_cap", C.c_uint32)]


class TuneResult(C.Structure):
    _fields_ = [("best", TuneParams), ("best_ms", C.c_float), ("default_ms", C.c_float), ("tried", C.c_uint32),
                ("from_cache", C.c_uint32), ("worst_ms", C.c_float), ("reserved", C.c_uint32)]


class ServerOpts(C.Structure):
    _fields_ = [("pool_bytes", C.c_uint64), ("chunk_paths", C.c_uint32), ("lanes", C.c_uint32),
                ("max_views_per_chunk", C.c_uint32), ("flags", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene_id", C.c_uint32), ("camera", Camera), ("spp", C.c_uint32), ("max_segments", C.c_uint32),
                ("seed", C.c_uint64), ("out_rgba", C.c_void_p)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_uint32), ("cancelled", C.c_uint32), ("submit_ms", C.c_double),
                ("admit_ms", C.c_double), ("done_ms", C.c_double), ("paths", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("completed", C.c_uint64),
                ("rejected", C.c_uint64), ("extend_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("pool_bytes", C.c_uint64), ("pool_used_bytes", C.c_uint64), ("active", C.c_uint32),
                ("queued", C.c_uint32), ("elapsed_ms", C.c_double), ("cancelled", C.c_uint64)]


BSM_REQ_QUEUED, BSM_REQ_RUNNING, BSM_REQ_DONE, BSM_REQ_FAILED, BSM_REQ_CANCELLED = 0, 1, 2, 3, 4


class CacheSettings(C.Structure):
    _fields_ = [("cache_segment", C.c_uint32), ("train_paths", C.c_uint32), ("train_segments", C.c_uint32),
                ("train_batch", C.c_uint32), ("train_steps", C.c_uint32), ("lr", C.c_float),
                ("ema_decay", C.c_float), ("min_roughness", C.c_float), ("extra_segments", C.c_uint32)]


class SceneGenParams(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("seed", C.c_uint64), ("grid", C.c_uint32), ("spheres", C.c_uint32),
                ("sky_width", C.c_uint32), ("sky_height", C.c_uint32)]


# -------------------------------------------------------------- library ----
_lib = None

class GeometryDesc(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.POINTER(C.c_float)), ("num_triangles", C.c_uint32),
                ("indices", C.POINTER(C.c_uint32)), ("material_ids", C.POINTER(C.c_uint32))]


class Instance(C.Structure):
    _fields_ = [("geometry_id", C.c_uint32), ("material_id", C.c_uint32), ("transform", C.c_float * 12)]


class InstancedSceneDesc(C.Structure):
    _fields_ = [("num_instances", C.c_uint32), ("instances", C.POINTER(Instance)), ("num_materials", C.c_uint32),
                ("materials", C.POINTER(Material)), ("num_dir_lights", C.c_uint32),
                ("dir_lights", C.POINTER(DirLight)), ("sky", Sky), ("num_point_lights", C.c_uint32),
                ("point_lights", C.POINTER(PointLight)), ("num_rect_lights", C.c_uint32),
                ("rect_lights", C.POINTER(RectLight))]


class Submesh(C.Structure):
    _fields_ = [("base_vertex", C.c_uint32), ("index_offset", C.c_uint32), ("num_indices", C.c_uint32),
                ("topology", C.c_uint32)]


class MeshData(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("positions", C.POINTER(C.c_float)),
                ("num_normals", C.c_uint32), ("normals", C.POINTER(C.c_float)),
                ("num_tangents", C.c_uint32), ("tangents", C.POINTER(C.c_float)),
                ("num_colors", C.c_uint32), ("colors", C.POINTER(C.c_float)),
                ("num_texcoords", C.c_uint32), ("texcoords", C.POINTER(C.c_float)),
                ("num_texcoords2", C.c_uint32), ("texcoords2", C.POINTER(C.c_float)),
                ("num_indices", C.c_uint32), ("indices", C.POINTER(C.c_uint32)),
                ("num_submeshes", C.c_uint32), ("submeshes", C.POINTER(Submesh)),
                ("handle", C.c_void_p)]


class ProjectInfo(C.Structure):
    _fields_ = [("camera", Camera), ("near_z", C.c_float), ("far_z", C.c_float), ("has_camera", C.c_uint32),
                ("camera_orthographic", C.c_uint32), ("settings", PtSettings), ("num_objects", C.c_uint32),
                ("num_drawables", C.c_uint32), ("num_skipped_submeshes", C.c_uint32),
                ("num_materials_approximated", C.c_uint32), ("num_non_opaque_materials", C.c_uint32),
                ("num_unsupported_lights", C.c_uint32), ("has_skybox", C.c_uint32), ("error", C.c_char * 256)]


_SIGS = {
    "bsm_create": (C.c_int32, [C.POINTER(C.c_void_p), C.c_int, C.c_uint64]),
    "bsm_destroy": (None, [C.c_void_p]),
    "bsm_last_error": (C.c_char_p, [C.c_void_p]),
    "bsm_api_version": (C.c_int, []),
    "bsm_sync": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "bsm_set_stream": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bsm_get_stream": (C.c_void_p, [C.c_void_p]),
    "bsm_render_stats_read": (C.c_int32, [C.c_void_p, C.POINTER(RenderStats)]),
    "bsm_device_alloc": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "bsm_device_free": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bsm_memcpy": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int]),
    "bsm_host_alloc": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "bsm_host_free": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bsm_scene_upload": (C.c_int32, [C.c_void_p, C.POINTER(SceneDesc), C.POINTER(C.c_uint32)]),
    "bsm_scene_build_bvh": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(BvhOpts), C.POINTER(BvhStats)]),
    "bsm_scene_release": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "bsm_bvh_build_host": (C.c_int32, [C.POINTER(SceneDesc), C.POINTER(BvhOpts), C.c_void_p, C.c_uint64,
                                       C.c_void_p, C.c_uint64, C.POINTER(BvhStats)]),
    "bsm_scene_device_bytes": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)]),
    "bsm_scene_download_bvh": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "bsm_pt_settings_default": (None, [C.POINTER(PtSettings)]),
    "bsm_render": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.c_uint32, C.POINTER(PtSettings),
                               C.POINTER(ViewOutput), C.POINTER(RenderStats)]),
    "bsm_render_batch": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(ViewDesc), C.c_uint32,
                                     C.POINTER(PtSettings), C.POINTER(ViewOutput), C.POINTER(RenderStats)]),
    "bsm_autotune": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(ViewDesc), C.c_uint32, C.POINTER(PtSettings),
                                 C.c_char_p, C.POINTER(TuneResult)]),
    "bsm_set_tuning": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(TuneParams)]),
    "bsm_read_view": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(ViewOutput)]),
    "bsm_export_history": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint32), C.c_uint32]),
    "bsm_import_history": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.c_void_p, C.c_uint32,
                                       C.c_uint32]),
    "bsm_trace_closest": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "bsm_trace_any": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "bsm_trace_counts": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]),
    "bsm_render_primary": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.POINTER(PtSettings), C.c_float,
                                       C.c_float, C.POINTER(PrimaryOutput)]),
    "bsm_render_noalloc": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.POINTER(PtSettings),
                                       C.c_void_p]),
    "bsm_server_start": (C.c_int32, [C.c_void_p, C.POINTER(ServerOpts)]),
    "bsm_server_submit": (C.c_int32, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_uint64)]),
    "bsm_server_poll": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(RequestStatus)]),
    "bsm_server_wait": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(RequestStatus)]),
    "bsm_server_get_stats": (C.c_int32, [C.c_void_p, C.POINTER(ServerStats)]),
    "bsm_server_stop": (C.c_int32, [C.c_void_p]),
    "bsm_server_cancel": (C.c_int32, [C.c_void_p, C.c_uint64]),
    "bsm_cache_settings_default": (None, [C.POINTER(CacheSettings)]),
    "bsm_cache_param_count": (C.c_uint32, []),
    "bsm_cache_create": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "bsm_cache_destroy": (None, [C.c_void_p]),
    "bsm_cache_weights": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "bsm_cache_render_weights": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "bsm_cache_predict": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "bsm_cache_gradient": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_float)]),
    "bsm_cache_train": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_float,
                                    C.POINTER(C.c_float)]),
    "bsm_cache_save": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "bsm_cache_load": (C.c_int32, [C.c_void_p, C.c_char_p]),
    "bsm_render_cached": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(Camera), C.POINTER(PtSettings), C.c_void_p,
                                      C.POINTER(CacheSettings), C.POINTER(ViewOutput), C.POINTER(RenderStats),
                                      C.POINTER(C.c_float)]),
    "bsm_scene_generate": (C.c_int32, [C.POINTER(SceneGenParams), C.POINTER(SceneDesc), C.POINTER(Camera)]),
    "bsm_scene_gen_free": (None, [C.POINTER(SceneDesc)]),
    "bsm_geometry_create": (C.c_int32, [C.c_void_p, C.POINTER(GeometryDesc), C.c_void_p, C.POINTER(C.c_uint32)]),
    "bsm_geometry_release": (C.c_int32, [C.c_void_p, C.c_uint32]),
    "bsm_scene_create_instanced": (C.c_int32, [C.c_void_p, C.POINTER(InstancedSceneDesc), C.POINTER(C.c_uint32)]),
    "bsm_scene_update_instances": (C.c_int32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32]),
    "bsm_static_mesh_read": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(MeshData), C.c_char_p, C.c_uint32]),
    "bsm_static_mesh_free": (None, [C.POINTER(MeshData)]),
    "bsm_static_mesh_write": (C.c_int32, [C.POINTER(MeshData), C.c_uint32, C.c_void_p, C.c_uint64,
                                          C.POINTER(C.c_uint64)]),
    "bsm_project_load": (C.c_int32, [C.c_char_p, C.POINTER(SceneDesc), C.POINTER(ProjectInfo)]),
    "bsm_project_free": (None, [C.POINTER(SceneDesc)]),
    "bsm_toml_check": (C.c_int32, [C.c_char_p, C.c_char_p, C.c_uint32]),
}


def lib() -> C.CDLL:
    """Loads libbsm_pt.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from importlib import util
        spec = util.spec_from_file_location("_bsm_build", os.path.join(HERE, "build.py"))
        mod = util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def declared_symbols() -> list[str]:
    return list(_SIGS)


def _ptr(a: np.ndarray, ctype=C.c_float):
    return a.ctypes.data_as(C.POINTER(ctype))


# ----------------------------------------------------------- scene data ----
@dataclass
class SceneData:
    """A scene in host memory (numpy arrays) — what bsm_scene_desc points at."""
    positions: np.ndarray             # (V, 3) float32
    indices: np.ndarray | None        # (T, 3) uint32
    material_ids: np.ndarray          # (T,) uint32
    materials: np.ndarray             # (M, 5) or (M, 7) float32: base rgb, roughness, metallic[, opacity, blend mode]
    lights: np.ndarray                # (L, 6) float32: direction to light, emission
    sky_kind: int = BSM_SKY_CONSTANT
    sky_color: tuple = (0.5, 0.5, 0.5)
    sky_texels: np.ndarray | None = None  # (H, W, 4) uint16 IEEE half, or (6, S, S, 4) for a cubemap
    camera: Camera | None = None
    _keep: list = field(default_factory=list, repr=False)
    point_lights: np.ndarray | None = None  # (P, 12): position, emission, range, direction to light, cos_inner, cos_outer
    rect_lights: np.ndarray | None = None   # (R, 15): centre, axis x, axis y, width, height, emission, two_sided
    sky_transform: np.ndarray | None = None  # (9,) cubemap lookup rotation, row-major
    normals: np.ndarray | None = None  # (V, 3) float32 vertex normals (shading normals), or None

    @property
    def num_triangles(self) -> int:
        return int(self.material_ids.shape[0])

    def desc(self) -> SceneDesc:
        pos = np.ascontiguousarray(self.positions, np.float32)
        idx = None if self.indices is None else np.ascontiguousarray(self.indices, np.uint32)
        mids = np.ascontiguousarray(self.material_ids, np.uint32)
        mats = (Material * len(self.materials))()
        for i, m in enumerate(self.materials):
            mats[i].base_color[:] = [float(m[0]), float(m[1]), float(m[2])]
            mats[i].roughness = float(m[3])
            mats[i].metallic = float(m[4])
            mats[i].opacity = float(m[5]) if len(m) > 5 else 1.0
            mats[i].blend_mode = int(m[6]) if len(m) > 6 else BSM_BLEND_OPAQUE
        lights = (DirLight * max(1, len(self.lights)))()
        for i, l in enumerate(self.lights):
            lights[i].direction[:] = [float(x) for x in l[:3]]
            lights[i].emission[:] = [float(x) for x in l[3:6]]
        d = SceneDesc()
        d.num_vertices = pos.shape[0]
        d.positions = _ptr(pos)
        d.num_triangles = mids.shape[0]
        d.indices = _ptr(idx, C.c_uint32) if idx is not None else None
        d.material_ids = _ptr(mids, C.c_uint32)
        d.num_materials = len(self.materials)
        d.materials = mats
        d.num_dir_lights = len(self.lights)
        d.dir_lights = lights
        keep = [pos, idx, mids, mats, lights]
        if self.normals is not None:
            nrm = np.ascontiguousarray(self.normals, np.float32).reshape(-1, 3)
            if nrm.shape[0] != pos.shape[0]:
                raise ValueError("normals need one row per vertex")
            d.normals = _ptr(nrm)
            keep.append(nrm)
        keep += _fill_sky_and_lights(d, self)
        self._keep = keep
        return d


def _fill_sky_and_lights(d, scene) -> list:
    """Sets the sky and the point / rect lights of a scene descriptor; returns the arrays to keep alive."""
    keep = []
    d.sky.kind = scene.sky_kind
    d.sky.color[:] = list(scene.sky_color)
    if scene.sky_texels is not None:
        tex = np.ascontiguousarray(scene.sky_texels, np.uint16)
        if scene.sky_kind == BSM_SKY_CUBEMAP:
            d.sky.width, d.sky.height = tex.shape[2], tex.shape[1]
        else:
            d.sky.width, d.sky.height = tex.shape[1], tex.shape[0]
        d.sky.rgba16f = _ptr(tex, C.c_uint16)
        keep.append(tex)
    if getattr(scene, "sky_transform", None) is not None:
        d.sky.transform[:] = [float(x) for x in np.asarray(scene.sky_transform).ravel()[:9]]
    pl = getattr(scene, "point_lights", None)
    if pl is not None and len(pl):
        pl = np.asarray(pl, np.float32).reshape(-1, 12)
        arr = (PointLight * len(pl))()
        for i, r in enumerate(pl):
            arr[i].position[:] = [float(x) for x in r[0:3]]
            arr[i].emission[:] = [float(x) for x in r[3:6]]
            arr[i].range = float(r[6])
            arr[i].direction[:] = [float(x) for x in r[7:10]]
            arr[i].cos_inner, arr[i].cos_outer = float(r[10]), float(r[11])
        d.num_point_lights, d.point_lights = len(pl), arr
        keep.append(arr)
    rl = getattr(scene, "rect_lights", None)
    if rl is not None and len(rl):
        rl = np.asarray(rl, np.float32).reshape(-1, 15)
        arr = (RectLight * len(rl))()
        for i, r in enumerate(rl):
            arr[i].center[:] = [float(x) for x in r[0:3]]
            arr[i].axis_x[:] = [float(x) for x in r[3:6]]
            arr[i].axis_y[:] = [float(x) for x in r[6:9]]
            arr[i].width, arr[i].height = float(r[9]), float(r[10])
            arr[i].emission[:] = [float(x) for x in r[11:14]]
            arr[i].two_sided = int(r[14])
        d.num_rect_lights, d.rect_lights = len(rl), arr
        keep.append(arr)
    return keep


def _materials_array(materials) -> "C.Array":
    mats = (Material * len(materials))()
    for i, m in enumerate(materials):
        mats[i].base_color[:] = [float(m[0]), float(m[1]), float(m[2])]
        mats[i].roughness = float(m[3])
        mats[i].metallic = float(m[4])
        mats[i].opacity = float(m[5]) if len(m) > 5 else 1.0
        mats[i].blend_mode = int(m[6]) if len(m) > 6 else BSM_BLEND_OPAQUE
    return mats


@dataclass
class GeometryData:
    """An object-space mesh of a two-level scene (bsm_geometry_desc)."""
    positions: np.ndarray             # (V, 3) float32
    indices: np.ndarray | None        # (T, 3) uint32
    material_ids: np.ndarray | None = None

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0]) if self.indices is not None else int(self.positions.shape[0] // 3)


@dataclass
class InstancedSceneData:
    """A two-level scene: geometries and their instances (bsm_instanced_scene_desc)."""
    geometries: list
    inst_geometry: np.ndarray         # (N,) index into geometries
    inst_material: np.ndarray         # (N,) uint32 material of every triangle, or 0xffffffff
    inst_transform: np.ndarray        # (N, 12) float32 object-to-world, row-major 3x4
    materials: np.ndarray             # (M, 5) or (M, 7), as SceneData
    lights: np.ndarray                # (L, 6)
    sky_kind: int = BSM_SKY_CONSTANT
    sky_color: tuple = (0.5, 0.5, 0.5)
    sky_texels: np.ndarray | None = None
    camera: Camera | None = None
    point_lights: np.ndarray | None = None
    rect_lights: np.ndarray | None = None
    sky_transform: np.ndarray | None = None

    @property
    def num_triangles(self) -> int:
        return int(sum(self.geometries[g].num_triangles for g in self.inst_geometry))

    def flattened(self) -> SceneData:
        """The same scene as one world-space mesh (each instance's triangles transformed in float64)."""
        pos, idx, mids = [], [], []
        base = 0
        for g, m, xf in zip(self.inst_geometry, self.inst_material, self.inst_transform):
            G = self.geometries[int(g)]
            M = np.asarray(xf, np.float64).reshape(3, 4)
            p = np.asarray(G.positions, np.float64) @ M[:, :3].T + M[:, 3]
            ii = np.asarray(G.indices, np.uint32) if G.indices is not None else np.arange(len(p), dtype=np.uint32).reshape(-1, 3)
            pos.append(p.astype(np.float32))
            idx.append(ii + base)
            t = len(ii)
            if int(m) != 0xFFFFFFFF:
                mids.append(np.full(t, int(m), np.uint32))
            else:
                mids.append(np.zeros(t, np.uint32) if G.material_ids is None else np.asarray(G.material_ids, np.uint32))
            base += len(p)
        return SceneData(np.concatenate(pos), np.concatenate(idx), np.concatenate(mids), self.materials, self.lights,
                         self.sky_kind, self.sky_color, self.sky_texels, self.camera, point_lights=self.point_lights,
                         rect_lights=self.rect_lights, sky_transform=self.sky_transform)


def _uv_sphere(n_lat: int, n_lon: int):
    th = np.linspace(0, np.pi, n_lat + 1)
    ph = np.linspace(0, 2 * np.pi, n_lon, endpoint=False)
    P = np.stack(np.meshgrid(th, ph, indexing="ij"), -1).reshape(-1, 2)
    pos = np.stack([np.sin(P[:, 0]) * np.cos(P[:, 1]), np.cos(P[:, 0]), np.sin(P[:, 0]) * np.sin(P[:, 1])], 1)
    tri = []
    for i in range(n_lat):
        for j in range(n_lon):
            a, b = i * n_lon + j, i * n_lon + (j + 1) % n_lon
            c, d = a + n_lon, b + n_lon
            if i > 0:
                tri.append((a, b, c))
            if i < n_lat - 1:
                tri.append((b, d, c))
    return pos.astype(np.float32), np.array(tri, np.uint32)


def generate_instanced_scene(seed: int = 1, instances: int = 200, width: int = 256, height: int = 256,
                             sphere_res: int = 16, ground: int = 64) -> InstancedSceneData:
    """A seeded two-level scene: a ground grid, a UV sphere, a box and a tetrahedron as geometries, the objects
    instanced with random rotations, non-uniform scales and translations over the ground; a sun and a constant sky."""
    rng = np.random.default_rng(seed)
    g = np.linspace(-1.0, 1.0, ground + 1)
    X, Z = np.meshgrid(g, g, indexing="ij")
    Y = 0.05 * np.sin(3 * X) * np.cos(2 * Z)
    gp = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    gi = []
    for i in range(ground):
        for j in range(ground):
            a, b, c, d = i * (ground + 1) + j, i * (ground + 1) + j + 1, (i + 1) * (ground + 1) + j, (i + 1) * (ground + 1) + j + 1
            gi += [(a, b, d), (a, d, c)]
    sp, si = _uv_sphere(sphere_res, 2 * sphere_res)
    bp = np.array([[x, y, z] for x in (-1, 1) for y in (-1, 1) for z in (-1, 1)], np.float32)
    bi = np.array([[0, 1, 3], [0, 3, 2], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
                   [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], np.uint32)
    tp = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], np.float32)
    ti = np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], np.uint32)
    geoms = [GeometryData(gp, np.array(gi, np.uint32), np.zeros(len(gi), np.uint32)),
             GeometryData(sp, si, (np.arange(len(si)) % 2 + 1).astype(np.uint32)),
             GeometryData(bp, bi, np.full(len(bi), 3, np.uint32)),
             GeometryData(tp, ti, None)]
    n_mat = 8
    mats = np.zeros((n_mat, 7), np.float32)
    mats[:, :3] = rng.uniform(0.1, 0.9, (n_mat, 3))
    mats[:, 3] = rng.uniform(0.05, 1.0, n_mat)
    mats[:, 4] = (rng.uniform(size=n_mat) < 0.3).astype(np.float32)
    mats[:, 5] = 1.0
    inst_g = [0]
    inst_m = [0xFFFFFFFF]
    xf = [np.array([[4, 0, 0, 0], [0, 1, 0, 0], [0, 0, 4, 0]], np.float32)]
    for _ in range(instances):
        kind = int(rng.integers(1, 4))
        a, b, c = rng.uniform(0, 2 * np.pi, 3)
        Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
        Rx = np.array([[1, 0, 0], [0, np.cos(b), -np.sin(b)], [0, np.sin(b), np.cos(b)]])
        Ry = np.array([[np.cos(c), 0, np.sin(c)], [0, 1, 0], [-np.sin(c), 0, np.cos(c)]])
        S = np.diag(rng.uniform(0.05, 0.3, 3))
        L = Rz @ Rx @ Ry @ S
        t = np.array([rng.uniform(-3.5, 3.5), rng.uniform(0.1, 0.6), rng.uniform(-3.5, 3.5)])
        xf.append(np.concatenate([L, t[:, None]], 1).astype(np.float32))
        inst_g.append(kind)
        inst_m.append(0xFFFFFFFF if rng.uniform() < 0.5 else int(rng.integers(4, n_mat)))
    lights = np.array([[0.4, 0.8, 0.3, 3.0, 2.9, 2.7]], np.float32)
    cam = make_camera((0.0, 2.5, 6.0), (0.0, -0.35, -1.0), yfov_deg=50.0, width=width, height=height)
    return InstancedSceneData(geoms, np.array(inst_g, np.uint32), np.array(inst_m, np.uint32),
                              np.stack(xf).reshape(-1, 12), mats, lights, BSM_SKY_CONSTANT, (0.4, 0.5, 0.6), None, cam)


def generate_scene(kind: int, seed: int = 1, grid: int = 0, spheres: int = 0, sky_width: int = 0,
                   sky_height: int = 0, width: int = 256, height: int = 256) -> SceneData:
    """Seeded procedural scene (bsm_scene_generate), copied into numpy arrays."""
    L = lib()
    p = SceneGenParams(kind, seed, grid, spheres, sky_width, sky_height)
    d = SceneDesc()
    cam = Camera()
    st = L.bsm_scene_generate(C.byref(p), C.byref(d), C.byref(cam))
    if st != BSM_OK:
        raise BsmError(st, "bsm_scene_generate failed")
    try:
        nv, nt, nm, nl = d.num_vertices, d.num_triangles, d.num_materials, d.num_dir_lights
        pos = np.ctypeslib.as_array(d.positions, (nv, 3)).copy()
        idx = np.ctypeslib.as_array(d.indices, (nt, 3)).copy() if d.indices else None
        mids = np.ctypeslib.as_array(d.material_ids, (nt,)).copy()
        mats = np.array([[*d.materials[i].base_color, d.materials[i].roughness, d.materials[i].metallic,
                          d.materials[i].opacity, d.materials[i].blend_mode] for i in range(nm)], np.float32)
        lights = np.array([[*d.dir_lights[i].direction, *d.dir_lights[i].emission] for i in range(nl)], np.float32)
        tex = None
        if d.sky.kind == BSM_SKY_EQUIRECT:
            tex = np.ctypeslib.as_array(d.sky.rgba16f, (d.sky.height, d.sky.width, 4)).copy()
        sky_color = tuple(d.sky.color)
        sky_kind = d.sky.kind
    finally:
        L.bsm_scene_gen_free(C.byref(d))
    cam.width, cam.height = width, height
    return SceneData(pos, idx, mids, mats, lights, sky_kind, sky_color, tex, cam)


def _scene_from_desc(d: SceneDesc, cam: Camera | None) -> SceneData:
    nv, nt, nm, nl = d.num_vertices, d.num_triangles, d.num_materials, d.num_dir_lights
    pos = np.ctypeslib.as_array(d.positions, (nv, 3)).copy() if nv else np.zeros((0, 3), np.float32)
    idx = np.ctypeslib.as_array(d.indices, (nt, 3)).copy() if d.indices else None
    mids = np.ctypeslib.as_array(d.material_ids, (nt,)).copy() if nt else np.zeros(0, np.uint32)
    mats = np.array([[*d.materials[i].base_color, d.materials[i].roughness, d.materials[i].metallic,
                      d.materials[i].opacity, d.materials[i].blend_mode] for i in range(nm)], np.float32).reshape(-1, 7)
    lights = np.array([[*d.dir_lights[i].direction, *d.dir_lights[i].emission] for i in range(nl)],
                      np.float32).reshape(-1, 6)
    tex = None
    if d.sky.kind == BSM_SKY_EQUIRECT:
        tex = np.ctypeslib.as_array(d.sky.rgba16f, (d.sky.height, d.sky.width, 4)).copy()
    pts = np.array([[*p.position, *p.emission, p.range, *p.direction, p.cos_inner, p.cos_outer]
                    for p in (d.point_lights[i] for i in range(d.num_point_lights))], np.float32).reshape(-1, 12)
    rects = np.array([[*r.center, *r.axis_x, *r.axis_y, r.width, r.height, *r.emission, r.two_sided]
                      for r in (d.rect_lights[i] for i in range(d.num_rect_lights))], np.float32).reshape(-1, 15)
    nrm = np.ctypeslib.as_array(d.normals, (nv, 3)).copy() if (d.normals and nv) else None
    return SceneData(pos, idx, mids, mats, lights, d.sky.kind, tuple(d.sky.color), tex, cam, point_lights=pts,
                     rect_lights=rects, normals=nrm)


_MESH_ARRAYS = [("positions", "num_vertices", 3, np.float32), ("normals", "num_normals", 3, np.float32),
                ("tangents", "num_tangents", 4, np.float32), ("colors", "num_colors", 3, np.float32),
                ("texcoords", "num_texcoords", 2, np.float32), ("texcoords2", "num_texcoords2", 2, np.float32),
                ("indices", "num_indices", 1, np.uint32)]


def read_static_mesh(data: bytes) -> dict:
    """A .static_mesh.biasset image (bsm_static_mesh_read) as numpy arrays: positions (V, 3), normals,
    tangents (N, 4), colors, texcoords (N, 2), texcoords2, indices (I,), submeshes (S, 4) uint32
    (base_vertex, index_offset, num_indices, topology)."""
    L = lib()
    buf = C.create_string_buffer(bytes(data), len(data))
    m = MeshData()
    err = C.create_string_buffer(256)
    st = L.bsm_static_mesh_read(buf, len(data), C.byref(m), err, 256)
    if st != BSM_OK:
        raise BsmError(st, "bsm_static_mesh_read: " + err.value.decode())
    try:
        out = {}
        for name, count, comps, dt in _MESH_ARRAYS:
            n = getattr(m, count)
            ptr = getattr(m, name)
            shape = (n, comps) if comps > 1 else (n,)
            out[name] = np.ctypeslib.as_array(ptr, shape).astype(dt).copy() if n and ptr else np.zeros(shape, dt)
        sub = np.zeros((m.num_submeshes, 4), np.uint32)
        for i in range(m.num_submeshes):
            s = m.submeshes[i]
            sub[i] = (s.base_vertex, s.index_offset, s.num_indices, s.topology)
        out["submeshes"] = sub
    finally:
        L.bsm_static_mesh_free(C.byref(m))
    return out


def write_static_mesh(mesh: dict, version: int = 2) -> bytes:
    """Writes a .static_mesh.biasset image (bsm_static_mesh_write) from arrays named as read_static_mesh's."""
    L = lib()
    m = MeshData()
    keep = []
    for name, count, comps, dt in _MESH_ARRAYS:
        a = mesh.get(name)
        if a is None or len(a) == 0:
            continue
        a = np.ascontiguousarray(a, dt).reshape(-1, comps) if comps > 1 else np.ascontiguousarray(a, dt).ravel()
        keep.append(a)
        setattr(m, count, a.shape[0])
        setattr(m, name, a.ctypes.data_as(C.POINTER(C.c_float if dt == np.float32 else C.c_uint32)))
    sub = np.ascontiguousarray(mesh.get("submeshes", np.zeros((0, 4))), np.uint32).reshape(-1, 4)
    subs = (Submesh * max(1, sub.shape[0]))()
    for i, r in enumerate(sub):
        subs[i] = Submesh(*[int(x) for x in r])
    m.num_submeshes = sub.shape[0]
    m.submeshes = C.cast(subs, C.POINTER(Submesh))
    size = C.c_uint64()
    st = L.bsm_static_mesh_write(C.byref(m), version, None, 0, C.byref(size))
    if st != BSM_OK:
        raise BsmError(st, "bsm_static_mesh_write failed")
    out = C.create_string_buffer(size.value)
    st = L.bsm_static_mesh_write(C.byref(m), version, out, size.value, C.byref(size))
    if st != BSM_OK:
        raise BsmError(st, "bsm_static_mesh_write failed")
    return out.raw[:size.value]


def load_project(path: str):
    """A reference project directory (bsm_project_load) -> (SceneData, ProjectInfo)."""
    L = lib()
    d = SceneDesc()
    info = ProjectInfo()
    st = L.bsm_project_load(os.fsencode(path), C.byref(d), C.byref(info))
    if st != BSM_OK:
        raise BsmError(st, "bsm_project_load: " + info.error.decode())
    try:
        cam = Camera.from_buffer_copy(info.camera)
        scene = _scene_from_desc(d, cam if info.has_camera else None)
    finally:
        L.bsm_project_free(C.byref(d))
    return scene, info


def toml_check(text: str):
    """Parses TOML text with the library's reader; raises BsmError with the reason on a syntax error."""
    err = C.create_string_buffer(256)
    st = lib().bsm_toml_check(text.encode(), err, 256)
    if st != BSM_OK:
        raise BsmError(st, err.value.decode())


def bvh_build_host(scene: SceneData, sah_bins=0, max_leaf=0, threads=0, collapse=0):
    """Host build of the compressed 8-wide BVH: returns (nodes bytes, tris bytes, BvhStats)."""
    L = lib()
    d = scene.desc()
    o = BvhOpts(sah_bins, max_leaf, threads, collapse)
    s = BvhStats()
    st = L.bsm_bvh_build_host(C.byref(d), C.byref(o), None, 0, None, 0, C.byref(s))
    if st != BSM_OK:
        raise BsmError(st, "bsm_bvh_build_host failed")
    nodes = np.zeros(s.node_bytes, np.uint8)
    tris = np.zeros(s.tri_bytes, np.uint8)
    st = L.bsm_bvh_build_host(C.byref(d), C.byref(o), nodes.ctypes.data, nodes.size, tris.ctypes.data, tris.size,
                              C.byref(s))
    if st != BSM_OK:
        raise BsmError(st, "bsm_bvh_build_host failed")
    return nodes, tris, s


def make_camera(position, front, up=(0.0, 1.0, 0.0), yfov_deg=60.0, width=256, height=256) -> Camera:
    c = Camera()
    c.position[:] = [float(x) for x in position]
    c.front[:] = [float(x) for x in front]
    c.up[:] = [float(x) for x in up]
    c.yfov_deg = yfov_deg
    c.width, c.height = width, height
    return c


def settings(spp=1, max_segments=0, max_bounces=3, seed=1, flags=0, ray_length=100.0, accumulate=0,
             sample_offset=0, wavefront_capacity=0, block_size=0, t_min=0.0) -> PtSettings:
    s = PtSettings()
    lib().bsm_pt_settings_default(C.byref(s))
    s.spp, s.max_segments, s.max_bounces, s.seed, s.flags = spp, max_segments, max_bounces, seed, flags
    s.ray_length, s.accumulate, s.sample_offset = ray_length, accumulate, sample_offset
    s.wavefront_capacity, s.block_size, s.t_min = wavefront_capacity, block_size, t_min
    return s


# -------------------------------------------------------------- context ----
class Context:
    """One CUDA device context (bsm_context)."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        self._L = lib()
        h = C.c_void_p()
        st = self._L.bsm_create(C.byref(h), device, budget_bytes)
        if st != BSM_OK:
            raise BsmError(st, "bsm_create failed (no CUDA device?)")
        self.h = h
        self._scene_geoms = {}   # two-level scene id -> its geometry ids

    def close(self):
        if self.h:
            self._L.bsm_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, st: int):
        if st != BSM_OK:
            raise BsmError(st, self._L.bsm_last_error(self.h).decode())

    # scenes
    def upload(self, scene: SceneData) -> int:
        sid = C.c_uint32()
        self.check(self._L.bsm_scene_upload(self.h, C.byref(scene.desc()), C.byref(sid)))
        return sid.value

    def build_bvh(self, scene_id: int, sah_bins=0, max_leaf=0, threads=0, collapse=0, tri_cost=0.0,
                  builder=BSM_BUILD_DEVICE) -> BvhStats:
        """Builds the scene's BVH, on the device by default (builder=BSM_BUILD_HOST: the host builder)."""
        o = BvhOpts(sah_bins, max_leaf, threads, collapse, tri_cost, builder)
        s = BvhStats()
        self.check(self._L.bsm_scene_build_bvh(self.h, scene_id, C.byref(o), C.byref(s)))
        return s

    def load_scene(self, scene: SceneData, collapse: int = 0, builder: int = BSM_BUILD_DEVICE) -> int:
        sid = self.upload(scene)
        self.build_bvh(sid, collapse=collapse, builder=builder)
        return sid

    def release(self, scene_id: int):
        self.check(self._L.bsm_scene_release(self.h, scene_id))
        for gid in self._scene_geoms.pop(scene_id, []):
            self._L.bsm_geometry_release(self.h, gid)

    def create_geometry(self, g: GeometryData, sah_bins=0, max_leaf=0, threads=0, builder=BSM_BUILD_DEVICE) -> int:
        pos = np.ascontiguousarray(g.positions, np.float32)
        idx = None if g.indices is None else np.ascontiguousarray(g.indices, np.uint32)
        mids = None if g.material_ids is None else np.ascontiguousarray(g.material_ids, np.uint32)
        d = GeometryDesc(pos.shape[0], _ptr(pos), g.num_triangles, _ptr(idx, C.c_uint32) if idx is not None else None,
                         _ptr(mids, C.c_uint32) if mids is not None else None)
        o = BvhOpts(sah_bins, max_leaf, threads, 0, 0.0, builder)
        gid = C.c_uint32()
        self.check(self._L.bsm_geometry_create(self.h, C.byref(d), C.byref(o), C.byref(gid)))
        return gid.value

    def load_instanced(self, scene: InstancedSceneData) -> int:
        """Creates the scene's geometries and the two-level scene; returns the scene id (release() frees both)."""
        gids = [self.create_geometry(g) for g in scene.geometries]
        n = len(scene.inst_geometry)
        insts = (Instance * n)()
        xf = np.ascontiguousarray(scene.inst_transform, np.float32).reshape(n, 12)
        for i in range(n):
            insts[i].geometry_id = gids[int(scene.inst_geometry[i])]
            insts[i].material_id = int(scene.inst_material[i])
            insts[i].transform[:] = [float(x) for x in xf[i]]
        mats = _materials_array(scene.materials)
        lights = (DirLight * max(1, len(scene.lights)))()
        for i, l in enumerate(scene.lights):
            lights[i].direction[:] = [float(x) for x in l[:3]]
            lights[i].emission[:] = [float(x) for x in l[3:6]]
        d = InstancedSceneDesc()
        d.num_instances = n
        d.instances = insts
        d.num_materials = len(scene.materials)
        d.materials = mats
        d.num_dir_lights = len(scene.lights)
        d.dir_lights = lights
        keep = _fill_sky_and_lights(d, scene)
        sid = C.c_uint32()
        st = self._L.bsm_scene_create_instanced(self.h, C.byref(d), C.byref(sid))
        if st != BSM_OK:
            for gid in gids:
                self._L.bsm_geometry_release(self.h, gid)
            self.check(st)
        self._scene_geoms[sid.value] = gids
        return sid.value

    def update_instances(self, scene_id: int, transforms: np.ndarray):
        """New object-to-world transforms (N, 12); the TLAS is refitted on the GPU."""
        xf = np.ascontiguousarray(transforms, np.float32).reshape(-1, 12)
        self.check(self._L.bsm_scene_update_instances(self.h, scene_id, xf.ctypes.data, xf.shape[0]))

    def scene_bytes(self, scene_id: int) -> int:
        b = C.c_uint64()
        self.check(self._L.bsm_scene_device_bytes(self.h, scene_id, C.byref(b)))
        return b.value

    def download_bvh(self, scene_id: int, stats: BvhStats):
        nodes = np.zeros(stats.node_bytes, np.uint8)
        tris = np.zeros(stats.tri_bytes, np.uint8)
        self.check(self._L.bsm_scene_download_bvh(self.h, scene_id, nodes.ctypes.data, tris.ctypes.data))
        return nodes, tris

    # stages
    def trace_closest(self, scene_id: int, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 4), np.uint32)
        self.check(self._L.bsm_trace_closest(self.h, scene_id, rays.ctypes.data, rays.shape[0], hits.ctypes.data,
                                             BSM_HOST))
        return hits

    def trace_any(self, scene_id: int, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.zeros(rays.shape[0], np.uint8)
        self.check(self._L.bsm_trace_any(self.h, scene_id, rays.ctypes.data, rays.shape[0], occ.ctypes.data,
                                         BSM_HOST))
        return occ

    def trace_counts(self, scene_id: int, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        cnt = np.zeros((rays.shape[0], 2), np.uint32)
        self.check(self._L.bsm_trace_counts(self.h, scene_id, rays.ctypes.data, rays.shape[0], cnt.ctypes.data))
        return cnt

    def render_primary(self, scene_id: int, cam: Camera, s: PtSettings | None = None, near_z: float = 0.0,
                       far_z: float = 0.0):
        """Primary-hit outputs of one pixel-centre ray per pixel: (depth (H, W), G-buffer (4, H, W, 4) as
        base_color, normal_roughness, fresnel, material_0, hit positions (H, W, 4))."""
        h, w = cam.height, cam.width
        depth = np.zeros((h, w), np.float32)
        gb = np.zeros((4, h, w, 4), np.float32)
        hp = np.zeros((h, w, 4), np.float32)
        out = PrimaryOutput()
        out.depth = depth.ctypes.data
        for k in range(4):
            out.gbuffer[k] = gb[k].ctypes.data
        out.hit_positions = hp.ctypes.data
        out.location = BSM_HOST
        self.check(self._L.bsm_render_primary(self.h, scene_id, C.byref(cam), C.byref(s) if s is not None else None,
                                              near_z, far_z, C.byref(out)))
        return depth, gb, hp

    # render
    def render(self, scene_id: int, cameras, s: PtSettings, outputs: bool = True, stats: bool = True):
        """Renders views; returns (list of (H, W, 4) float32 images or None, RenderStats or None)."""
        if isinstance(cameras, Camera):
            cameras = [cameras]
        n = len(cameras)
        cams = (Camera * n)(*cameras)
        outs = None
        imgs = None
        if outputs:
            imgs = [np.zeros((c.height, c.width, 4), np.float32) for c in cameras]
            outs = (ViewOutput * n)()
            for i, im in enumerate(imgs):
                outs[i].rgba = im.ctypes.data
                outs[i].row_pitch_px = 0
                outs[i].location = BSM_HOST
        rs = RenderStats() if stats else None
        self.check(self._L.bsm_render(self.h, scene_id, cams, n, C.byref(s), outs,
                                      C.byref(rs) if rs is not None else None))
        return imgs, rs

    def render_batch(self, scene_id: int, views, s: PtSettings, outputs: bool = True, stats: bool = True):
        """views: list of (Camera, spp, max_segments, seed); returns (images, RenderStats)."""
        n = len(views)
        descs = (ViewDesc * n)()
        for i, (cam, spp, segs, seed) in enumerate(views):
            descs[i].camera = cam
            descs[i].spp, descs[i].max_segments, descs[i].seed = spp, segs, seed
        outs, imgs = None, None
        if outputs:
            imgs = [np.zeros((v[0].height, v[0].width, 4), np.float32) for v in views]
            outs = (ViewOutput * n)()
            for i, im in enumerate(imgs):
                outs[i].rgba = im.ctypes.data
                outs[i].location = BSM_HOST
        rs = RenderStats() if stats else None
        self.check(self._L.bsm_render_batch(self.h, scene_id, descs, n, C.byref(s), outs,
                                            C.byref(rs) if rs is not None else None))
        return imgs, rs

    def autotune(self, scene_id: int, views, s: PtSettings, cache_path: str | None = None) -> TuneResult:
        n = len(views)
        descs = (ViewDesc * n)()
        for i, (cam, spp, segs, seed) in enumerate(views):
            descs[i].camera = cam
            descs[i].spp, descs[i].max_segments, descs[i].seed = spp, segs, seed
        r = TuneResult()
        self.check(self._L.bsm_autotune(self.h, scene_id, descs, n, C.byref(s),
                                        cache_path.encode() if cache_path else None, C.byref(r)))
        return r

    def set_tuning(self, scene_id: int, params: TuneParams | None):
        self.check(self._L.bsm_set_tuning(self.h, scene_id, C.byref(params) if params is not None else None))

    # serving loop
    def server_start(self, pool_bytes=0, chunk_paths=0, lanes=0, max_views_per_chunk=0, deterministic=False):
        self._reqs = {}
        flags = BSM_SERVER_DETERMINISTIC if deterministic else 0
        self.check(self._L.bsm_server_start(self.h, C.byref(ServerOpts(pool_bytes, chunk_paths, lanes,
                                                                       max_views_per_chunk, flags))))

    def submit(self, scene_id: int, cam: Camera, spp: int, max_segments: int = 8, seed: int = 1):
        """Queues a request; returns (id, output array filled when the request is done)."""
        out = np.zeros((cam.height, cam.width, 4), np.float32)
        r = Request(scene_id, cam, spp, max_segments, seed, out.ctypes.data)
        rid = C.c_uint64()
        self.check(self._L.bsm_server_submit(self.h, C.byref(r), C.byref(rid)))
        self._reqs[rid.value] = out
        return rid.value, out

    def wait(self, rid: int, timeout_ms: int = 0) -> RequestStatus:
        st = RequestStatus()
        self.check(self._L.bsm_server_wait(self.h, rid, timeout_ms, C.byref(st)))
        return st

    def poll(self, rid: int) -> RequestStatus:
        st = RequestStatus()
        self.check(self._L.bsm_server_poll(self.h, rid, C.byref(st)))
        return st

    def cancel(self, rid: int):
        """Cancels a request (bsm_server_cancel); its output array is not written afterwards."""
        self.check(self._L.bsm_server_cancel(self.h, rid))

    def server_stats(self) -> ServerStats:
        st = ServerStats()
        self.check(self._L.bsm_server_get_stats(self.h, C.byref(st)))
        return st

    def server_stop(self):
        self.check(self._L.bsm_server_stop(self.h))
        self._reqs = {}

    def sync(self, timeout_ms: int = 0):
        self.check(self._L.bsm_sync(self.h, timeout_ms))

    def set_stream(self, stream: int | None):
        """Runs later work on a caller's cudaStream_t (an integer handle), or on the context's own stream (None)."""
        self.check(self._L.bsm_set_stream(self.h, C.c_void_p(stream) if stream else None))

    def last_stats(self) -> RenderStats:
        """Waits for the last render issued and returns its statistics (bsm_render_stats_read)."""
        rs = RenderStats()
        self.check(self._L.bsm_render_stats_read(self.h, C.byref(rs)))
        return rs


# ------------------------------------------------------- radiance cache ----
def cache_settings(**kw) -> CacheSettings:
    cs = CacheSettings()
    lib().bsm_cache_settings_default(C.byref(cs))
    for k, v in kw.items():
        setattr(cs, k, v)
    return cs


class RadianceCache:
    """The learned radiance cache (bsm_cache) of one context."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        self._L = ctx._L
        h = C.c_void_p()
        ctx.check(self._L.bsm_cache_create(ctx.h, seed, C.byref(h)))
        self.h = h
        self.nparams = self._L.bsm_cache_param_count()

    def close(self):
        if self.h:
            self._L.bsm_cache_destroy(self.h)
            self.h = None

    def _st(self, st):
        if st != BSM_OK:
            raise BsmError(st, "radiance cache call failed")

    def weights(self, set_to: np.ndarray | None = None) -> np.ndarray:
        w = np.zeros(self.nparams, np.float32)
        src = None if set_to is None else np.ascontiguousarray(set_to, np.float32)
        self._st(self._L.bsm_cache_weights(self.h, w.ctypes.data, None if src is None else src.ctypes.data))
        return w if set_to is None else src

    def render_weights(self) -> np.ndarray:
        """The weights renders use: the bias-corrected moving average (ema_decay > 0), else the master weights."""
        w = np.zeros(self.nparams, np.float32)
        self._st(self._L.bsm_cache_render_weights(self.h, w.ctypes.data))
        return w

    def predict(self, samples: np.ndarray) -> np.ndarray:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 16)
        out = np.zeros((s.shape[0], 3), np.float32)
        self._st(self._L.bsm_cache_predict(self.h, s.ctypes.data, s.shape[0], out.ctypes.data))
        return out

    def gradient(self, samples: np.ndarray):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 16)
        dW = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        self._st(self._L.bsm_cache_gradient(self.h, s.ctypes.data, s.shape[0], dW.ctypes.data, C.byref(loss)))
        return dW, loss.value

    def train(self, samples: np.ndarray, batch: int = 16384, lr: float = 1e-2) -> float:
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 16)
        loss = C.c_float()
        self._st(self._L.bsm_cache_train(self.h, s.ctypes.data, s.shape[0], batch, lr, C.byref(loss)))
        return loss.value

    def save(self, path: str):
        self._st(self._L.bsm_cache_save(self.h, path.encode()))

    def load(self, path: str):
        self._st(self._L.bsm_cache_load(self.h, path.encode()))

    def render(self, scene_id: int, cam: Camera, s: PtSettings, cs: CacheSettings | None = None, outputs=True):
        """One frame with the cache (training first when cs.train_steps > 0); returns (image, stats, loss)."""
        cs = cs or cache_settings()
        img = np.zeros((cam.height, cam.width, 4), np.float32) if outputs else None
        out = None
        if outputs:
            out = ViewOutput()
            out.rgba = img.ctypes.data
            out.location = BSM_HOST
        st = RenderStats()
        loss = C.c_float()
        self.ctx.check(self._L.bsm_render_cached(self.ctx.h, scene_id, C.byref(cam), C.byref(s), self.h, C.byref(cs),
                                                 C.byref(out) if out is not None else None, C.byref(st),
                                                 C.byref(loss)))
        return img, st, loss.value


def rel_mse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2, trim: float = 0.0) -> float:
    """Relative MSE over pixels and RGB: mean((I - R)^2 / (R^2 + eps)); `trim` drops that fraction of the
    largest per-value errors first (fireflies dominate single-frame relMSE)."""
    a = img[..., :3].astype(np.float64)
    b = ref[..., :3].astype(np.float64)
    e = ((a - b) ** 2 / (b * b + eps)).ravel()
    if trim > 0.0:
        e = np.sort(e)[: max(1, int(round(e.size * (1.0 - trim))))]
    return float(np.mean(e))


# -------------------------------------------------- reference-shaped API ----
@dataclass
class PathTracingSettings:
    """BasicRenderer::PathTracingSettings (basic.hpp:76-81) plus the explicit spp and seed."""
    ray_length: float = 100.0
    max_bounces: int = 3
    denoise: bool = True
    accumulate: bool = True
    spp: int = 1
    seed: int = 1


@dataclass
class GBufferTextures:
    """GBufferTextures (renderer/context/gbuffer.hpp): the four packed planes of gbuffer.hlsl:6-11."""
    base_color: np.ndarray
    normal_roughness: np.ndarray
    fresnel: np.ndarray
    material_0: np.ndarray


class PathTracingPass:
    """Mirror of PathTracingPass (path_tracing.hpp:13-35) on the GB300 pass.

    update_params() takes the lights and skybox the reference reads from its
    LightsContext / SkyboxContext; render() traces one camera and returns the
    pass's OutputData: the colour (running mean over the accumulated frames),
    the reverse-Z depth and the G-buffer of the primary hit, and no velocity
    (invalid in the reference too, path_tracing.cpp:553-558).

    History follows path_tracing.cpp:231-245: it continues only while the same
    camera (position, orientation, field of view) and size are rendered on
    consecutive frames.  Frames are counted by this object; a caller that skips
    frames passes `frame_index` (the engine's frame count) and a gap resets
    the history as the reference's `last_frame + 1 == frame_count` test does."""

    @dataclass
    class OutputData:
        color: np.ndarray
        depth: np.ndarray | None = None
        velocity: None = None
        gbuffer: GBufferTextures | None = None

    def __init__(self, ctx: Context, scene: SceneData):
        self.ctx = ctx
        self.scene = scene
        self.scene_id = None
        self.frame = 0
        self.last_frame = None

    def update_params(self, lights=None, skybox=None, settings_: PathTracingSettings | None = None):
        if lights is not None:
            self.scene.lights = np.asarray(lights, np.float32).reshape(-1, 6)
        if skybox is not None:
            self.scene.sky_kind, self.scene.sky_color, self.scene.sky_texels = skybox
        if self.scene_id is not None:
            self.ctx.release(self.scene_id)
        self.scene_id = self.ctx.load_scene(self.scene)

    def render(self, camera: Camera, settings_: PathTracingSettings, frame_index: int | None = None,
               near_z: float = 0.01, far_z: float = 10000.0, primary: bool = True) -> "PathTracingPass.OutputData":
        if self.scene_id is None:
            self.update_params()
        frame = self.frame + 1 if frame_index is None else int(frame_index)
        consecutive = self.last_frame is not None and self.last_frame + 1 == frame
        s = settings(spp=settings_.spp, max_bounces=settings_.max_bounces, seed=settings_.seed,
                     ray_length=settings_.ray_length, accumulate=1 if settings_.accumulate and consecutive else 0)
        imgs, _ = self.ctx.render(self.scene_id, [camera], s, outputs=True, stats=False)
        self.frame = frame
        self.last_frame = frame
        out = PathTracingPass.OutputData(color=imgs[0])
        if primary:
            depth, gb, _ = self.ctx.render_primary(self.scene_id, camera, s, near_z, far_z)
            out.depth = depth
            out.gbuffer = GBufferTextures(gb[0], gb[1], gb[2], gb[3])
        return out
