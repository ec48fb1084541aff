"""Two-level scenes on the GPU: TLAS over instances of per-geometry BLASes.

* closest / any hits of random and axis-aligned rays equal the oracle's bit for
  bit (t, global primitive id), with rotated, non-uniformly scaled instances;
* renders take the oracle's paths (per-segment ray counts equal, radiance
  within 1e-4) and the primary outputs match bit for bit, also with
  non-opaque materials and per-instance material overrides;
* after bsm_scene_update_instances (GPU refit of the TLAS) the hits equal an
  oracle built with the new transforms, and equal a full TLAS rebuild;
* bad transforms and releasing an instanced geometry are refused."""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_bits_equal

from test_instancing_oracle import random_world_rays

pytestmark = pytest.mark.gpu


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


@pytest.fixture(scope="module")
def inst_scene(bsm, ctx, oracle):
    sc = bsm.generate_instanced_scene(seed=4, instances=150, width=64, height=48, sphere_res=12, ground=32)
    sid = ctx.load_instanced(sc)
    yield sc, sid, oracle.OracleScene(sc)
    ctx.release(sid)


def test_hits_equal_oracle(bsm, ctx, inst_scene):
    sc, sid, osc = inst_scene
    rays = random_world_rays(30000, 7)
    rays[:2000, 4:7] = [0.0, -1.0, 0.0]        # axis-aligned: zero direction components
    rays[2000:3000, 4:7] = [1.0, 0.0, 0.0]
    h = ctx.trace_closest(sid, rays)
    ho = osc.trace(rays)
    assert np.mean(h[:, 1] != 0xFFFFFFFF) > 0.3
    assert np.array_equal(h[:, 1], ho[:, 1])
    assert np.array_equal(h[:, 0], ho[:, 0])
    assert np.array_equal(ctx.trace_any(sid, rays) != 0, ho[:, 1] != 0xFFFFFFFF)


def test_render_and_primary_equal_oracle(bsm, ctx, inst_scene):
    sc, sid, osc = inst_scene
    for flags in (0, 1):
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=9, flags=flags))
        ref, ost, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=9, flags=flags)
        assert [int(x) for x in st.rays_per_segment[:4]] == [int(x) for x in ost[:4]]
        assert int(st.shadow_rays) == int(ost[16:32].sum())
        assert rel_err(imgs[0], ref).max() <= 1e-4
        det = flags | bsm.BSM_PT_DETERMINISTIC   # fixed-point sums on both sides: equal bit for bit
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=9, flags=det))
        ref, _, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=9, flags=det)
        assert_bits_equal(imgs[0], ref)
    d, g, h = ctx.render_primary(sid, sc.camera)
    do, go, ho = osc.primary(sc.camera.as_array())
    assert np.array_equal(h.view(np.uint32), ho.view(np.uint32))
    assert np.array_equal(d.view(np.uint32), do.view(np.uint32))
    assert np.array_equal(g.view(np.uint32), go.view(np.uint32))


def test_refit_after_moving_instances(bsm, ctx, oracle, inst_scene):
    sc, sid, _ = inst_scene
    rng = np.random.default_rng(5)
    xf = sc.inst_transform.copy().reshape(-1, 12)
    moved = xf.copy()
    moved[1:, 3] += rng.uniform(-0.8, 0.8, len(xf) - 1)        # translate x
    moved[1:, 11] += rng.uniform(-0.8, 0.8, len(xf) - 1)       # translate z
    moved[1:, :3] *= 1.5                                        # and stretch the first rows
    try:
        ctx.update_instances(sid, moved)
        sc2 = bsm.InstancedSceneData(sc.geometries, sc.inst_geometry, sc.inst_material, moved, sc.materials, sc.lights,
                                     sc.sky_kind, sc.sky_color, None, sc.camera)
        osc2 = oracle.OracleScene(sc2)
        rays = random_world_rays(30000, 8)
        h = ctx.trace_closest(sid, rays)
        ho = osc2.trace(rays)
        assert np.array_equal(h[:, 1], ho[:, 1]) and np.array_equal(h[:, 0], ho[:, 0])
        ctx.build_bvh(sid)                                       # full rebuild from the same transforms
        assert np.array_equal(ctx.trace_closest(sid, rays), h)
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=1, max_segments=3, seed=2))
        ref, ost, _ = osc2.render(sc.camera.as_array(), spp=1, max_segments=3, seed=2)
        assert rel_err(imgs[0], ref).max() <= 1e-4
    finally:
        ctx.update_instances(sid, xf)


def test_non_opaque_materials_in_two_level_scene(bsm, ctx, oracle):
    sc = bsm.generate_instanced_scene(seed=6, instances=80, width=48, height=36, sphere_res=10, ground=16)
    m = sc.materials.copy()
    m[1, 5], m[1, 6] = 0.4, bsm.BSM_BLEND_TRANSLUCENT
    m[5, 5], m[5, 6] = 0.0, bsm.BSM_BLEND_ALPHA_TEST
    sc.materials = m
    sid = ctx.load_instanced(sc)
    try:
        osc = oracle.OracleScene(sc)
        rays = random_world_rays(20000, 3)
        assert np.array_equal(ctx.trace_closest(sid, rays), osc.trace(rays))
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=1))
        ref, ost, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=1)
        assert [int(x) for x in st.rays_per_segment[:4]] == [int(x) for x in ost[:4]]
        assert rel_err(imgs[0], ref).max() <= 1e-4
        det = bsm.BSM_PT_DETERMINISTIC
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=1, flags=det))
        ref, _, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=1, flags=det)
        assert_bits_equal(imgs[0], ref)
    finally:
        ctx.release(sid)


def test_instancing_errors(bsm, ctx, inst_scene):
    sc, sid, _ = inst_scene
    bad = sc.inst_transform.copy().reshape(-1, 12)
    bad[3, :3] = 0.0                                            # singular
    with pytest.raises(bsm.BsmError):
        ctx.update_instances(sid, bad)
    with pytest.raises(bsm.BsmError):
        ctx.update_instances(sid, bad[:5])                      # wrong count
    gid = ctx._scene_geoms[sid][0]
    assert ctx._L.bsm_geometry_release(ctx.h, gid) == -6        # BSM_ERR_BAD_STATE while instanced
    assert ctx._L.bsm_geometry_release(ctx.h, 99999) == -5      # BSM_ERR_NOT_FOUND
