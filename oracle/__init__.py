"""CPU ORACLE of the wavefront path-tracing pass — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg load
this package.  It wraps ``oracle/_build/liboracle.so`` (pt_oracle.cpp, a
multithreaded C++ restatement of the pass; each function there cites the
reference shader it follows) and, where the reference tree was present at
build time, ``oracle/_ref/libref_bsdf.so`` (the reference's own HLSL material
math compiled through a C++ shim; used only to generate golden vectors).

Parity pins: BSDF / frame / sampler formulas and the G-buffer packing against
golden vectors produced from the reference's shader sources
(tests/golden/bsdf_golden.npz, tests/golden/gbuffer_golden.npz); PCG32
against the published pcg32 demo output.  Traversal and BVH: the reference's
are inside the graphics driver, so closest-hit parity is pinned to this
restatement of the published watertight test only.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_ref = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _b
        path = _b.build_oracle()
        L = C.CDLL(path)
        vp, u32, u64, f32, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
        L.orc_scene_create.argtypes = [vp, u32, vp, u32, vp, vp, u32, vp, u32, u32, vp, u32, u32, vp, vp, vp,
                                       C.POINTER(vp)]
        L.orc_scene_create.restype = i32
        L.orc_scene_destroy.argtypes = [vp]
        L.orc_trace.argtypes = [vp, vp, u32, vp, i32, i32, vp]
        L.orc_trace.restype = i32
        L.orc_render.argtypes = [vp, vp, u32, u32, u32, u32, u64, f32, f32, u32, u32, vp, vp, i32,
                                 C.POINTER(C.c_double)]
        L.orc_render.restype = i32
        L.orc_render_cached.argtypes = [vp, vp, u32, u32, u32, u64, f32, f32, vp, u32, f32, u32, u32, vp, vp, i32]
        L.orc_render_cached.restype = i32
        L.orc_pcg32.argtypes = [u64, u64, u32, vp]
        L.orc_sincos_turns.argtypes = [vp, u32, vp, vp]
        L.orc_atan2.argtypes = [vp, vp, u32, vp]
        L.orc_eval_lit.argtypes = [vp, u32, vp]
        L.orc_vndf.argtypes = [vp, u32, vp]
        L.orc_frame.argtypes = [vp, u32, vp]
        L.orc_mlp_forward.argtypes = [vp, vp, u32, vp, i32]
        L.orc_mlp_gradient.argtypes = [vp, vp, u32, vp, i32]
        L.orc_mlp_gradient.restype = f32
        L.orc_mlp_adam.argtypes = [vp, vp, vp, vp, f32, i32]
        L.orc_primary.argtypes = [vp, vp, f32, f32, f32, f32, u64, u32, vp, vp, vp, i32]
        L.orc_primary.restype = i32
        L.orc_gbuffer_pack.argtypes = [vp, u32, vp]
        L.orc_geometry_create.argtypes = [vp, u32, vp, u32, vp, C.POINTER(vp)]
        L.orc_geometry_create.restype = i32
        L.orc_scene_create_instanced.argtypes = [vp, u32, vp, vp, vp, u32, vp, u32, vp, u32, u32, vp, u32, u32, vp,
                                                 vp, C.POINTER(vp)]
        L.orc_scene_create_instanced.restype = i32
        L.orc_sky_sample.argtypes = [vp, vp, u32, vp]
        L.orc_scene_bvh_nodes.argtypes = [vp]
        L.orc_light_eval.argtypes = [vp, vp, vp, u32, f32, vp]
        L.orc_light_eval.restype = i32
        L.orc_cwbvh_trace.argtypes = [vp, u64, vp, u64, vp, u32, i32, vp, vp, i32]
        L.orc_cwbvh_trace.restype = i32
        L.orc_scene_bvh_nodes.restype = u32
        _lib = L
    return _lib


def ref_lib() -> C.CDLL | None:
    """The reference's shader math compiled from its sources, or None where the reference tree is absent."""
    global _ref
    if _ref is None:
        from . import build as _b
        path = _b.build_reference()
        if path is None:
            return None
        R = C.CDLL(path)
        for fn in ("ref_eval_lit", "ref_vndf", "ref_frame", "ref_aniso", "ref_samplers", "ref_gbuffer",
                   "ref_gbuffer_unpack", "ref_point_light", "ref_dir_light"):
            getattr(R, fn).argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        R.ref_inv_pi.restype = C.c_float
        _ref = R
    return _ref


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def light_rows(scene) -> np.ndarray:
    """(L, 16) float32 rows of the oracle's lights: kind, then the light's fields (pt_oracle.cpp setup_shading)."""
    rows = []
    for l in np.asarray(scene.lights, np.float32).reshape(-1, 6):
        rows.append([0, *l] + [0] * 9)
    for l in np.asarray(getattr(scene, "point_lights", None) if getattr(scene, "point_lights", None) is not None
                        else np.zeros((0, 12)), np.float32).reshape(-1, 12):
        rows.append([1, *l] + [0] * 3)
    for l in np.asarray(getattr(scene, "rect_lights", None) if getattr(scene, "rect_lights", None) is not None
                        else np.zeros((0, 15)), np.float32).reshape(-1, 15):
        rows.append([2, *l])
    return np.ascontiguousarray(np.array(rows, np.float32).reshape(-1, 16))


def sky_args(scene):
    """(texels or None, width, height, transform[9]) of a scene's sky (cubemaps: 6 faces, face size)."""
    tex = None if scene.sky_texels is None else np.ascontiguousarray(scene.sky_texels, np.uint16)
    xf = np.zeros(9, np.float32) if getattr(scene, "sky_transform", None) is None else _f32(scene.sky_transform)
    if tex is None:
        return None, 0, 0, xf
    if scene.sky_kind == 2:                  # (6, S, S, 4)
        return tex, tex.shape[2], tex.shape[1], xf
    return tex, tex.shape[1], tex.shape[0], xf


def material_rows(materials) -> np.ndarray:
    """(M, 7) float32: base rgb, roughness, metallic, opacity, blend mode; 5-column input is opaque."""
    m = np.asarray(materials, np.float32)
    m = m.reshape(m.shape[0], -1)
    if m.shape[1] == 5:
        m = np.concatenate([m, np.ones((m.shape[0], 1), np.float32), np.zeros((m.shape[0], 1), np.float32)], 1)
    return np.ascontiguousarray(m[:, :7], np.float32)


class OracleScene:
    """A scene inside the oracle (own binary SAH BVH)."""

    def __init__(self, scene):
        L = lib()
        self._L = L
        if hasattr(scene, "geometries"):   # a two-level scene
            self._init_instanced(scene)
            return
        pos = _f32(scene.positions)
        idx = None if scene.indices is None else np.ascontiguousarray(scene.indices, np.uint32)
        mids = np.ascontiguousarray(scene.material_ids, np.uint32)
        mats = material_rows(scene.materials)
        lights = light_rows(scene)
        color = _f32(scene.sky_color)
        tex, sw, sh, sxf = sky_args(scene)
        nrm = getattr(scene, "normals", None)
        nrm = None if nrm is None else _f32(nrm).reshape(-1, 3)
        h = C.c_void_p()
        st = L.orc_scene_create(pos.ctypes.data, pos.shape[0], None if idx is None else idx.ctypes.data,
                                mids.shape[0], mids.ctypes.data, mats.ctypes.data, mats.shape[0],
                                lights.ctypes.data, lights.shape[0], scene.sky_kind, color.ctypes.data,
                                sw, sh, None if tex is None else tex.ctypes.data, sxf.ctypes.data,
                                None if nrm is None else nrm.ctypes.data, C.byref(h))
        if st != 0:
            raise RuntimeError("orc_scene_create failed")
        self.h = h

    def _init_instanced(self, scene):
        L = self._L
        self._geoms = []
        for g in scene.geometries:
            pos = _f32(g.positions)
            idx = None if g.indices is None else np.ascontiguousarray(g.indices, np.uint32)
            mids = None if g.material_ids is None else np.ascontiguousarray(g.material_ids, np.uint32)
            h = C.c_void_p()
            nt = idx.shape[0] if idx is not None else pos.shape[0] // 3
            if L.orc_geometry_create(pos.ctypes.data, pos.shape[0], None if idx is None else idx.ctypes.data, nt,
                                     None if mids is None else mids.ctypes.data, C.byref(h)) != 0:
                raise RuntimeError("orc_geometry_create failed")
            self._geoms.append(h)
        garr = (C.c_void_p * len(self._geoms))(*[g.value for g in self._geoms])
        ig = np.ascontiguousarray(scene.inst_geometry, np.uint32)
        im = np.ascontiguousarray(scene.inst_material, np.uint32)
        ix = _f32(scene.inst_transform).reshape(-1, 12)
        mats = material_rows(scene.materials)
        lights = light_rows(scene)
        color = _f32(scene.sky_color)
        tex, sw, sh, sxf = sky_args(scene)
        h = C.c_void_p()
        st = L.orc_scene_create_instanced(garr, len(self._geoms), ig.ctypes.data, im.ctypes.data, ix.ctypes.data,
                                          ig.shape[0], mats.ctypes.data, mats.shape[0], lights.ctypes.data,
                                          lights.shape[0], scene.sky_kind, color.ctypes.data, sw, sh,
                                          None if tex is None else tex.ctypes.data, sxf.ctypes.data, C.byref(h))
        if st != 0:
            raise RuntimeError("orc_scene_create_instanced failed")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self._L.orc_scene_destroy(self.h)
            self.h = None
        for g in getattr(self, "_geoms", []):
            self._L.orc_scene_destroy(g)
        self._geoms = []

    def trace(self, rays: np.ndarray, any_hit: bool = False, threads: int = 0, counts: bool = False):
        rays = _f32(rays).reshape(-1, 8)
        hits = np.zeros((rays.shape[0], 4), np.uint32)
        cnt = np.zeros((rays.shape[0], 2), np.uint32) if counts else None
        self._L.orc_trace(self.h, rays.ctypes.data, rays.shape[0], hits.ctypes.data, 1 if any_hit else 0, threads,
                          None if cnt is None else cnt.ctypes.data)
        return (hits, cnt) if counts else hits

    def render(self, camera: np.ndarray, spp: int, max_segments: int, seed: int = 1, flags: int = 0,
               ray_length: float = 100.0, t_min: float = 0.0, sample_offset: int = 0, rows=None, threads: int = 0):
        """Returns (mean RGBA image of the rows, stats[32], seconds)."""
        cam = _f32(camera)
        w, h = int(cam[10]), int(cam[11])
        r0, r1 = rows if rows is not None else (0, h)
        out = np.zeros((r1 - r0, w, 4), np.float32)
        stats = np.zeros(32, np.uint64)
        sec = C.c_double()
        st = self._L.orc_render(self.h, cam.ctypes.data, spp, max_segments, sample_offset, flags, seed, ray_length,
                                t_min, r0, r1, out.ctypes.data, stats.ctypes.data, threads, C.byref(sec))
        if st != 0:
            raise RuntimeError("orc_render failed")
        return out, stats, sec.value


    def render_cached(self, camera: np.ndarray, spp: int, weights: np.ndarray, cache_segment: int,
                      extra_segments: int = 0, min_roughness: float = 0.0, seed: int = 1, flags: int = 0,
                      ray_length: float = 100.0, t_min: float = 0.0, rows=None, threads: int = 0):
        """The cached pass without its training step (bsm_render_cached with train_steps = 0): paths run
        cache_segment + 1 + extra_segments segments and end in a query of the network with `weights` at the
        first hit of segment cache_segment or later whose roughness is at least min_roughness (at the last
        segment whatever its roughness).  Returns (mean RGBA image of the rows, stats[32])."""
        cam = _f32(camera)
        w, h = int(cam[10]), int(cam[11])
        r0, r1 = rows if rows is not None else (0, h)
        W = _f32(weights)
        out = np.zeros((r1 - r0, w, 4), np.float32)
        stats = np.zeros(32, np.uint64)
        st = self._L.orc_render_cached(self.h, cam.ctypes.data, spp, cache_segment + 1 + extra_segments, flags, seed,
                                       ray_length, t_min, W.ctypes.data, cache_segment,
                                       min_roughness if extra_segments else 0.0, r0, r1, out.ctypes.data,
                                       stats.ctypes.data, threads)
        if st != 0:
            raise RuntimeError("orc_render_cached failed")
        return out, stats

    def primary(self, camera: np.ndarray, ray_length: float = 100.0, t_min: float = 0.0, near_z: float = 0.01,
                far_z: float = 10000.0, seed: int = 1, sample_offset: int = 0, threads: int = 0):
        """Primary-hit outputs of one pixel-centre ray per pixel: (depth (h, w), G-buffer (4, h, w, 4),
        hit positions (h, w, 4))."""
        cam = _f32(camera)
        w, h = int(cam[10]), int(cam[11])
        depth = np.zeros((h, w), np.float32)
        gb = np.zeros((4, h, w, 4), np.float32)
        hp = np.zeros((h, w, 4), np.float32)
        st = self._L.orc_primary(self.h, cam.ctypes.data, ray_length, t_min, near_z, far_z, seed, sample_offset,
                                 depth.ctypes.data, gb.ctypes.data, hp.ctypes.data, threads)
        if st != 0:
            raise RuntimeError("orc_primary failed")
        return depth, gb, hp


    def sky_sample(self, u: np.ndarray) -> np.ndarray:
        """(n, 3) uniforms -> (n, 5): sampled direction, its pdf, and sky_pdf of that direction."""
        u = _f32(u).reshape(-1, 3)
        out = np.zeros((u.shape[0], 5), np.float32)
        self._L.orc_sky_sample(self.h, u.ctypes.data, u.shape[0], out.ctypes.data)
        return out


def cwbvh_trace(nodes: np.ndarray, tris: np.ndarray, rays: np.ndarray, any_hit: bool = False, threads: int = 0):
    """Traverses the product's compressed BVH (raw node and triangle bytes) with
    the device kernel's arithmetic; returns (hits n x 4 u32, counts n x 2 u32:
    nodes visited, triangles tested)."""
    nodes = np.ascontiguousarray(nodes).view(np.uint8)
    tris = np.ascontiguousarray(tris).view(np.uint8)
    assert nodes.size % 80 == 0 and tris.size % 48 == 0
    rays = _f32(rays).reshape(-1, 8)
    hits = np.zeros((rays.shape[0], 4), np.uint32)
    cnt = np.zeros((rays.shape[0], 2), np.uint32)
    st = lib().orc_cwbvh_trace(nodes.ctypes.data, nodes.size // 80, tris.ctypes.data, tris.size // 48,
                               rays.ctypes.data, rays.shape[0], 1 if any_hit else 0, hits.ctypes.data,
                               cnt.ctypes.data, threads)
    if st != 0:
        raise RuntimeError("orc_cwbvh_trace failed")
    return hits, cnt


def light_eval(row, P, u=None, ray_len: float = 100.0) -> np.ndarray:
    """Next-event sample of one light (a 16-float row: kind, then its fields as light_rows() lays them out) from
    points P (n, 3): (n, 8) = arriving radiance, direction to the light, shadow-ray length, reached (0/1)."""
    row = _f32(row).reshape(16)
    P = _f32(P).reshape(-1, 3)
    uu = None if u is None else _f32(u).reshape(-1, 2)
    out = np.zeros((P.shape[0], 8), np.float32)
    if lib().orc_light_eval(row.ctypes.data, P.ctypes.data, None if uu is None else uu.ctypes.data, P.shape[0],
                            ray_len, out.ctypes.data) != 0:
        raise RuntimeError("orc_light_eval failed")
    return out


def pcg32(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_pcg32(initstate, initseq, n, out.ctypes.data)
    return out


def sincos_turns(t):
    t = _f32(t)
    s = np.zeros_like(t)
    c = np.zeros_like(t)
    lib().orc_sincos_turns(t.ctypes.data, t.size, s.ctypes.data, c.ctypes.data)
    return s, c


def atan2(y, x):
    y, x = _f32(y), _f32(x)
    o = np.zeros_like(y)
    lib().orc_atan2(y.ctypes.data, x.ctypes.data, y.size, o.ctypes.data)
    return o


def _batch(fn, a, cols_in, cols_out):
    a = _f32(a).reshape(-1, cols_in)
    o = np.zeros((a.shape[0], cols_out), np.float32)
    fn(a.ctypes.data, a.shape[0], o.ctypes.data)
    return o


def gbuffer_pack(a):
    """rows of V3 N3 T3 base3 f0_3 roughness -> the four packed G-buffer float4 (16 floats)."""
    return _batch(lib().orc_gbuffer_pack, a, 16, 16)


def eval_lit(a):
    return _batch(lib().orc_eval_lit, a, 16, 3)


def vndf(a):
    return _batch(lib().orc_vndf, a, 7, 4)


def frame(a):
    return _batch(lib().orc_frame, a, 3, 6)


# ---- radiance-cache network (see pt_oracle.cpp) ----
MLP_PARAMS = 4 * 4096 + 8 * 64


def mlp_forward(W, samples, bf16=True):
    W = _f32(W)
    S = _f32(samples).reshape(-1, 16)
    out = np.zeros((S.shape[0], 3), np.float32)
    lib().orc_mlp_forward(W.ctypes.data, S.ctypes.data, S.shape[0], out.ctypes.data, 1 if bf16 else 0)
    return out


def mlp_gradient(W, samples, bf16=True):
    W = _f32(W)
    S = _f32(samples).reshape(-1, 16)
    dW = np.zeros(MLP_PARAMS, np.float32)
    loss = lib().orc_mlp_gradient(W.ctypes.data, S.ctypes.data, S.shape[0], dW.ctypes.data, 1 if bf16 else 0)
    return dW, loss


def mlp_adam(W, dW, m, v, lr, t):
    W, m, v = _f32(W).copy(), _f32(m).copy(), _f32(v).copy()
    dW = _f32(dW)
    lib().orc_mlp_adam(W.ctypes.data, dW.ctypes.data, m.ctypes.data, v.ctypes.data, lr, t)
    return W, m, v
