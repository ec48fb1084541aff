"""Point / spot / rect lights and the cubemap sky on the GPU: the same paths as
the oracle (per-segment ray counts, shadow-ray count, radiance within 1e-4),
with up to eight lights of all kinds, in one- and two-level scenes."""
import numpy as np
import pytest

from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu


def rel_err(g, c):
    g = g[..., :3].astype(np.float64)
    c = c[..., :3].astype(np.float64)
    return np.abs(g - c) / np.maximum(np.abs(c), 1e-3)


def lights_for(rng, n_point, n_rect):
    pts = []
    for i in range(n_point):
        spot = i % 2 == 1
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        pts.append([*rng.uniform(0.1, 0.9, 3), *rng.uniform(0.2, 1.5, 3), rng.uniform(0.5, 3.0), *d,
                    np.cos(0.4) if spot else 0.0, np.cos(0.9) if spot else 0.0])
    rects = []
    for i in range(n_rect):
        ax = rng.normal(size=3)
        ax /= np.linalg.norm(ax)
        ay = np.cross(ax, rng.normal(size=3))
        ay /= np.linalg.norm(ay)
        rects.append([*rng.uniform(0.2, 0.8, 3), *ax, *ay, *rng.uniform(0.05, 0.3, 2), *rng.uniform(1, 6, 3), i % 2])
    return np.array(pts, np.float32).reshape(-1, 12), np.array(rects, np.float32).reshape(-1, 15)


def cube_faces(rng, S=16):
    f = rng.uniform(0.0, 2.0, (6, S, S, 4)).astype(np.float16)
    f[..., 3] = 1
    return f.view(np.uint16)


@pytest.mark.parametrize("n_dir,n_point,n_rect,cube", [(1, 2, 1, False), (2, 3, 3, True), (0, 0, 2, True)])
def test_lights_equal_oracle(bsm, ctx, oracle, n_dir, n_point, n_rect, cube):
    rng = np.random.default_rng(n_point * 10 + n_rect)
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=21, spheres=20, width=48, height=40)
    sc.lights = sc.lights[:n_dir] if n_dir <= len(sc.lights) else np.tile(sc.lights, (n_dir, 1))
    sc.point_lights, sc.rect_lights = lights_for(rng, n_point, n_rect)
    if cube:
        sc.sky_kind, sc.sky_texels = bsm.BSM_SKY_CUBEMAP, cube_faces(rng)
        sc.sky_transform = np.array([0, 0, 1, 0, 1, 0, -1, 0, 0], np.float32)
    sid = ctx.load_scene(sc)
    try:
        osc = oracle.OracleScene(sc)
        for flags in (0, 1, 2):
            imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, flags=flags))
            ref, ost, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=5, flags=flags)
            assert [int(x) for x in st.rays_per_segment[:4]] == [int(x) for x in ost[:4]]
            assert int(st.shadow_rays) == int(ost[16:32].sum())
            assert rel_err(imgs[0], ref).max() <= 1e-4
        # fixed-point sums on both sides: equal bit for bit
        det = flags | bsm.BSM_PT_DETERMINISTIC
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=4, seed=5, flags=det))
        ref, _, _ = osc.render(sc.camera.as_array(), spp=2, max_segments=4, seed=5, flags=det)
        assert_bits_equal(imgs[0], ref)
    finally:
        ctx.release(sid)


def test_lights_in_two_level_scene(bsm, ctx, oracle):
    rng = np.random.default_rng(2)
    sc = bsm.generate_instanced_scene(seed=8, instances=60, width=48, height=36, sphere_res=10, ground=16)
    pts, rects = lights_for(rng, 2, 2)
    pts[:, 0:3] = rng.uniform(-2, 2, (2, 3))
    pts[:, 1] = 1.5
    rects[:, 0:3] = [[0, 2, 0], [1, 1.5, -1]]
    sc.point_lights, sc.rect_lights = pts, rects
    sid = ctx.load_instanced(sc)
    try:
        imgs, st = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=3, seed=3))
        ref, ost, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=2, max_segments=3, seed=3)
        assert [int(x) for x in st.rays_per_segment[:3]] == [int(x) for x in ost[:3]]
        assert rel_err(imgs[0], ref).max() <= 1e-4
        det = bsm.BSM_PT_DETERMINISTIC
        imgs, _ = ctx.render(sid, [sc.camera], bsm.settings(spp=2, max_segments=3, seed=3, flags=det))
        ref, _, _ = oracle.OracleScene(sc).render(sc.camera.as_array(), spp=2, max_segments=3, seed=3, flags=det)
        assert_bits_equal(imgs[0], ref)
    finally:
        ctx.release(sid)


def test_too_many_lights_rejected(bsm, ctx):
    sc = bsm.generate_scene(bsm.BSM_SCENE_ROOM, seed=1, spheres=4, width=8, height=8)
    sc.point_lights, sc.rect_lights = lights_for(np.random.default_rng(0), 5, 3)   # 1 dir + 8 others
    with pytest.raises(bsm.BsmError):
        ctx.load_scene(sc)
